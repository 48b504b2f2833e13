// host_io.cpp -- the reference's text file families, read and written fast.
//
// Formats (all 1-indexed ids, one record per line):
//   <prefix>-0 .. <prefix>-63 : file 0 starts with "N M"; file t holds edges
//       [t*floor(M/64), (t+1)*floor(M/64)), the last file up to M, as "u v"
//       ("u v w" when weighted).  Written by tools/csr_tiling/page_rank.cpp:570-592,
//       tools/coo_tiling/page_rank.cpp:452-485, tools/column_major_tile/kcore.cpp:419-441;
//       read by apps/bfs_simd/bfs.cpp:1024-1056 and :1076-1106.
//   <prefix>-offsets : SIDE*SIDE lines, first edge index of each tile in file order.
//   <prefix>-nneibor : N lines of out-degree.
// The parsers read whole files and convert digits by hand (the reference uses
// fscanf, which is what makes its input step slow); the writers format digits
// into large buffers and produce byte-identical output to the reference's
// fprintf("%u %u\n").
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <sys/stat.h>

#include "internal.h"

namespace bfsg {

unsigned host_threads() {
	unsigned t = std::thread::hardware_concurrency();
	if (t == 0) t = 4;
	if (t > 64) t = 64;
	return t;
}

bool file_exists(const std::string &path) {
	struct stat st;
	return ::stat(path.c_str(), &st) == 0;
}

namespace {

int slurp(const std::string &path, std::vector<char> &buf) {
	FILE *f = std::fopen(path.c_str(), "rb");
	if (!f) return BFS_EIO;
	std::fseek(f, 0, SEEK_END);
	long sz = std::ftell(f);
	std::fseek(f, 0, SEEK_SET);
	if (sz < 0) { std::fclose(f); return BFS_EIO; }
	buf.resize((size_t) sz + 1);
	size_t got = sz ? std::fread(buf.data(), 1, (size_t) sz, f) : 0;
	std::fclose(f);
	if (got != (size_t) sz) return BFS_EIO;
	buf[(size_t) sz] = '\0';
	return BFS_OK;
}

// Cursor over a NUL-terminated buffer; reads unsigned decimals separated by
// whitespace, like fscanf("%u").
struct Cursor {
	const char *p;
	bool next(uint64_t *v) {
		while (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r') ++p;
		if (*p < '0' || *p > '9') return false;
		uint64_t x = 0;
		while (*p >= '0' && *p <= '9') {
			x = x * 10 + (uint64_t) (*p - '0');
			if (x > 0xFFFFFFFFull) return false;
			++p;
		}
		*v = x;
		return true;
	}
};

inline char *put_u32(char *out, uint32_t v) {
	char tmp[12];
	int k = 0;
	do { tmp[k++] = (char) ('0' + v % 10); v /= 10; } while (v);
	while (k) *out++ = tmp[--k];
	return out;
}

} // namespace

int read_header(const std::string &path, uint32_t *n, uint64_t *m) {
	FILE *f = std::fopen(path.c_str(), "rb");
	if (!f) return BFS_EIO;
	char line[256] = {0};
	size_t got = std::fread(line, 1, sizeof(line) - 1, f);
	std::fclose(f);
	line[got] = '\0';
	Cursor c{line};
	uint64_t a, b;
	if (!c.next(&a) || !c.next(&b)) return BFS_EFORMAT;
	*n = (uint32_t) a;
	*m = b;
	return BFS_OK;
}

int read_split_family(const std::string &prefix, uint64_t m, bool weighted, uint32_t n,
		uint32_t *a, uint32_t *b) {
	std::atomic<int> status{BFS_OK};
	parallel_for(kNumSplitFiles, [&](uint64_t lo_f, uint64_t hi_f, unsigned) {
		std::vector<char> buf;
		for (uint64_t tid = lo_f; tid < hi_f; ++tid) {
			uint64_t lo, hi;
			split_range(m, (unsigned) tid, &lo, &hi);
			std::string name = prefix + "-" + std::to_string(tid);
			int st = slurp(name, buf);
			if (st) { status = st; return; }
			Cursor c{buf.data()};
			uint64_t x, y, wt;
			if (tid == 0 && (!c.next(&x) || !c.next(&y))) { status = BFS_EFORMAT; return; }
			for (uint64_t i = lo; i < hi; ++i) {
				if (!c.next(&x) || !c.next(&y) || (weighted && !c.next(&wt))) {
					status = BFS_EFORMAT;
					return;
				}
				if (x == 0 || y == 0 || x > n || y > n) { status = BFS_EFORMAT; return; }
				if (a) a[i] = (uint32_t) (x - 1);
				b[i] = (uint32_t) (y - 1);
			}
		}
	});
	return status.load();
}

int read_u32_lines(const std::string &path, uint64_t count, uint32_t *out) {
	std::vector<char> buf;
	int st = slurp(path, buf);
	if (st) return st;
	Cursor c{buf.data()};
	uint64_t x;
	for (uint64_t i = 0; i < count; ++i) {
		if (!c.next(&x)) return BFS_EFORMAT;
		out[i] = (uint32_t) x;
	}
	return BFS_OK;
}

int write_split_family(const std::string &prefix, uint32_t n, uint64_t m, const uint32_t *a,
		const uint32_t *b, const uint32_t *weights) {
	std::atomic<int> status{BFS_OK};
	parallel_for(kNumSplitFiles, [&](uint64_t lo_f, uint64_t hi_f, unsigned) {
		std::vector<char> buf(1 << 22);
		for (uint64_t tid = lo_f; tid < hi_f; ++tid) {
			uint64_t lo, hi;
			split_range(m, (unsigned) tid, &lo, &hi);
			std::string name = prefix + "-" + std::to_string(tid);
			FILE *f = std::fopen(name.c_str(), "wb");
			if (!f) { status = BFS_EIO; return; }
			char *p = buf.data();
			char *end = buf.data() + buf.size() - 64;
			if (tid == 0) {
				p = put_u32(p, n); *p++ = ' ';
				p = put_u32(p, (uint32_t) m); *p++ = '\n';
			}
			for (uint64_t i = lo; i < hi; ++i) {
				p = put_u32(p, a[i] + 1); *p++ = ' ';
				p = put_u32(p, b[i] + 1);
				if (weights) { *p++ = ' '; p = put_u32(p, weights[i]); }
				*p++ = '\n';
				if (p >= end) {
					if (std::fwrite(buf.data(), 1, (size_t) (p - buf.data()), f) != (size_t) (p - buf.data())) status = BFS_EIO;
					p = buf.data();
				}
			}
			if (p != buf.data() && std::fwrite(buf.data(), 1, (size_t) (p - buf.data()), f) != (size_t) (p - buf.data()))
				status = BFS_EIO;
			std::fclose(f);
		}
	});
	return status.load();
}

int write_u32_lines(const std::string &path, const uint32_t *v, uint64_t count) {
	FILE *f = std::fopen(path.c_str(), "wb");
	if (!f) return BFS_EIO;
	std::vector<char> buf(1 << 22);
	char *p = buf.data();
	char *end = buf.data() + buf.size() - 16;
	int st = BFS_OK;
	for (uint64_t i = 0; i < count; ++i) {
		p = put_u32(p, v[i]);
		*p++ = '\n';
		if (p >= end) {
			if (std::fwrite(buf.data(), 1, (size_t) (p - buf.data()), f) != (size_t) (p - buf.data())) st = BFS_EIO;
			p = buf.data();
		}
	}
	if (p != buf.data() && std::fwrite(buf.data(), 1, (size_t) (p - buf.data()), f) != (size_t) (p - buf.data())) st = BFS_EIO;
	std::fclose(f);
	return st;
}

} // namespace bfsg

using namespace bfsg;

namespace {

// Reads an "N M" edge list (README.md:19-24) into 0-based arrays.
int read_edge_list(const char *path, bool weighted, uint32_t *n, std::vector<uint32_t> &src,
		std::vector<uint32_t> &dst, std::vector<uint32_t> *wt) {
	std::vector<char> buf;
	int st = slurp(path, buf);
	if (st) return st;
	Cursor c{buf.data()};
	uint64_t nn, mm, x, y, w;
	if (!c.next(&nn) || !c.next(&mm)) return BFS_EFORMAT;
	*n = (uint32_t) nn;
	src.resize(mm);
	dst.resize(mm);
	if (wt) wt->resize(mm);
	for (uint64_t i = 0; i < mm; ++i) {
		if (!c.next(&x) || !c.next(&y)) return BFS_EFORMAT;
		if (weighted) {
			if (!c.next(&w)) return BFS_EFORMAT;
			if (wt) (*wt)[i] = (uint32_t) w;
		}
		if (x == 0 || y == 0 || x > nn || y > nn) return BFS_EFORMAT;
		src[i] = (uint32_t) (x - 1);
		dst[i] = (uint32_t) (y - 1);
	}
	return BFS_OK;
}

} // namespace

extern "C" {

// tools/csr_tiling/page_rank.cpp main (:607-625): input_untiled (:513-605) or
// input_weighted (:414-510).  Edges are bucketed by source keeping input order;
// nothing is deduplicated.
int bfs_tool_csr_tiling(const char *edge_list, uint32_t flags) {
	if (!edge_list) return BFS_EARG;
	bool weighted = flags & BFS_LOAD_WEIGHTED;
	uint32_t n;
	std::vector<uint32_t> src, dst, wt, cs, cd, deg;
	int st = read_edge_list(edge_list, weighted, &n, src, dst, weighted ? &wt : nullptr);
	if (st) return st;
	st = csr_from_edges(n, src.size(), src.data(), dst.data(), cs, cd, deg);
	if (st) return st;
	std::vector<uint32_t> cw;
	if (weighted) {
		// The weight travels with its edge through the same stable bucketing.
		std::vector<uint64_t> start(n + 1, 0);
		for (uint32_t v = 0; v < n; ++v) start[v + 1] = start[v] + deg[v];
		cw.resize(src.size());
		for (size_t i = 0; i < src.size(); ++i) cw[start[src[i]]++] = wt[i];
	}
	std::string prefix = std::string(edge_list) + "_untiled";
	st = write_split_family(prefix, n, src.size(), cs.data(), cd.data(), weighted ? cw.data() : nullptr);
	if (st) return st;
	return write_u32_lines(prefix + "-nneibor", deg.data(), n);
}

// tools/coo_tiling/page_rank.cpp input_data (:324-515): one file family per
// tile width, min_w..max_w doubling (:399).
int bfs_tool_coo_tiling(const char *data, uint32_t min_w, uint32_t max_w, uint32_t flags) {
	if (!data || min_w == 0 || max_w < min_w) return BFS_EARG;
	(void) flags;
	std::string prefix = std::string(data) + "_untiled";
	uint32_t n;
	uint64_t m;
	int st = read_header(prefix + "-0", &n, &m);
	if (st) return st;
	std::vector<uint32_t> s(m), d(m);
	if ((st = read_split_family(prefix, m, false, n, s.data(), d.data()))) return st;
	std::vector<uint32_t> deg(n, 0);
	for (uint64_t i = 0; i < m; ++i) deg[s[i]]++;
	for (uint64_t w = min_w; w <= max_w; w *= 2) {
		uint32_t side = side_length_of(n, (uint32_t) w);
		uint64_t num_tiles = (uint64_t) side * side;
		std::vector<uint64_t> fill(num_tiles + 1, 0);
		for (uint64_t i = 0; i < m; ++i) fill[(uint64_t) (s[i] / w) * side + d[i] / w + 1]++;
		for (uint64_t t = 0; t < num_tiles; ++t) fill[t + 1] += fill[t];
		std::vector<uint32_t> off(num_tiles), ts(m), td(m);
		for (uint64_t t = 0; t < num_tiles; ++t) off[t] = (uint32_t) fill[t];
		for (uint64_t i = 0; i < m; ++i) {
			uint64_t pos = fill[(uint64_t) (s[i] / w) * side + d[i] / w]++;
			ts[pos] = s[i];
			td[pos] = d[i];
		}
		std::string out = std::string(data) + "_coo-tiled-" + std::to_string(w);
		if ((st = write_split_family(out, n, m, ts.data(), td.data(), nullptr))) return st;
		if ((st = write_u32_lines(out + "-offsets", off.data(), num_tiles))) return st;
		if ((st = write_u32_lines(out + "-nneibor", deg.data(), n))) return st;
	}
	return BFS_OK;
}

// tools/column_major_tile/kcore.cpp input (:143-244) + convert_to_col_major
// (:360-467), for S = min_s..max_s doubling (:527-534).
int bfs_tool_column_major(const char *data, uint32_t w, uint32_t min_s, uint32_t max_s, uint32_t flags) {
	if (!data || w == 0 || min_s == 0 || max_s < min_s) return BFS_EARG;
	(void) flags;
	std::string prefix = std::string(data) + "_coo-tiled-" + std::to_string(w);
	uint32_t n;
	uint64_t m;
	int st = read_header(prefix + "-0", &n, &m);
	if (st) return st;
	uint32_t side = side_length_of(n, w);
	uint64_t num_tiles = (uint64_t) side * side;
	std::vector<uint32_t> off(num_tiles), deg(n), s(m), d(m);
	if ((st = read_u32_lines(prefix + "-offsets", num_tiles, off.data()))) return st;
	if ((st = read_u32_lines(prefix + "-nneibor", n, deg.data()))) return st;
	if ((st = read_split_family(prefix, m, false, n, s.data(), d.data()))) return st;
	for (uint64_t stripe = min_s; stripe <= max_s; stripe *= 2) {
		std::vector<uint32_t> cs(m), cd(m), noff(num_tiles);
		uint64_t e_out = 0, t_out = 0;
		auto emit_tile = [&](uint64_t tile) {
			uint64_t hi = (tile != num_tiles - 1) ? off[tile + 1] : m;
			noff[t_out++] = (uint32_t) e_out;
			for (uint64_t e = off[tile]; e < hi; ++e) {
				cs[e_out] = s[e];
				cd[e_out] = d[e];
				++e_out;
			}
		};
		uint64_t side_i;
		for (side_i = 0; side_i + stripe <= side; side_i += stripe)
			for (uint64_t col = 0; col < side; ++col)
				for (uint64_t row = side_i; row < side_i + stripe; ++row) emit_tile(row * side + col);
		if (side_i != side)
			for (uint64_t col = 0; col < side; ++col)
				for (uint64_t row = side_i; row < side; ++row) emit_tile(row * side + col);
		if (e_out != m || t_out != num_tiles) return BFS_EFORMAT;
		std::string out = std::string(data) + "_col-" + std::to_string(stripe) + "-coo-tiled-" + std::to_string(w);
		if ((st = write_split_family(out, n, m, cs.data(), cd.data(), nullptr))) return st;
		if ((st = write_u32_lines(out + "-offsets", noff.data(), num_tiles))) return st;
		if ((st = write_u32_lines(out + "-nneibor", deg.data(), n))) return st;
	}
	return BFS_OK;
}

// tools/vertex_id_remap/bfs.cpp BFSGraph (:69-247): label vertices in BFS
// discovery order from vertex 0, level by level in ascending old id
// (add_mask2map :465-479), unreached last (add_remainder2map :481-491); write
// the CSR-ordered edges relabelled as <data>_reorder (make_up_data :42-64).
int bfs_tool_vertex_remap(const char *data, uint32_t flags) {
	if (!data) return BFS_EARG;
	std::string prefix = std::string(data) + "_untiled";
	uint32_t n;
	uint64_t m;
	int st = read_header(prefix + "-0", &n, &m);
	if (st) return st;
	std::vector<uint32_t> s(m), d(m), deg(n);
	if ((st = read_split_family(prefix, m, false, n, s.data(), d.data()))) return st;
	if ((st = read_u32_lines(prefix + "-nneibor", n, deg.data()))) return st;
	std::vector<uint64_t> start(n + 1, 0);
	for (uint32_t v = 0; v < n; ++v) start[v + 1] = start[v] + deg[v];
	if (start[n] != m) return BFS_EFORMAT;
	std::vector<uint32_t> map(n, kUnvisited), frontier, next;
	if (flags & BFS_TOOL_DEVICE) {
		// the BFS on the GPU, the labels from its levels (same map)
		bfs_graph *g = nullptr;
		if ((st = bfs_graph_from_edges(n, m, s.data(), d.data(), 1024, 16, BFS_LOAD_DEVICE_BUILD, &g))) return st;
		st = bfs_graph_bfs_order(g, 0, map.data());
		bfs_graph_free(g);
		if (st) return st;
	} else {
		std::vector<uint8_t> seen(n, 0);
		uint32_t top = 0;
		if (n) {
			map[0] = top++;
			seen[0] = 1;
			frontier.push_back(0);
		}
		while (!frontier.empty()) {
			next.clear();
			for (uint32_t u : frontier)
				for (uint64_t e = start[u]; e < start[u + 1]; ++e)
					if (!seen[d[e]]) { seen[d[e]] = 1; next.push_back(d[e]); }
			std::sort(next.begin(), next.end());
			for (uint32_t v : next) map[v] = top++;
			frontier.swap(next);
		}
		for (uint32_t v = 0; v < n; ++v)
			if (map[v] == kUnvisited) map[v] = top++;
	}
	std::string out = std::string(data) + "_reorder";
	FILE *f = std::fopen(out.c_str(), "wb");
	if (!f) return BFS_EIO;
	std::vector<char> buf(1 << 22);
	char *p = buf.data(), *end = buf.data() + buf.size() - 32;
	p = put_u32(p, n); *p++ = ' '; p = put_u32(p, (uint32_t) m); *p++ = '\n';
	for (uint64_t i = 0; i < m; ++i) {
		p = put_u32(p, map[s[i]] + 1); *p++ = ' ';
		p = put_u32(p, map[d[i]] + 1); *p++ = '\n';
		if (p >= end) { std::fwrite(buf.data(), 1, (size_t) (p - buf.data()), f); p = buf.data(); }
	}
	size_t rest = (size_t) (p - buf.data());
	bool ok = std::fwrite(buf.data(), 1, rest, f) == rest;
	std::fclose(f);
	return ok ? BFS_OK : BFS_EIO;
}

// The ONEDEBUG dump of apps/bfs_simd/bfs.cpp:927-954.
int bfs_write_level_dump(const char *dir, uint32_t num_vertices, const int32_t *levels) {
	if (!dir || (!levels && num_vertices)) return BFS_EARG;
	uint32_t per = num_vertices / 64;
	std::atomic<int> status{BFS_OK};
	parallel_for(64, [&](uint64_t lo_f, uint64_t hi_f, unsigned) {
		for (uint64_t t = lo_f; t < hi_f; ++t) {
			uint32_t lo = (uint32_t) t * per;
			uint32_t hi = (t != 63) ? lo + per : num_vertices;
			std::string name = std::string(dir) + "/path" + std::to_string(t) + ".txt";
			FILE *f = std::fopen(name.c_str(), "wb");
			if (!f) { status = BFS_EIO; return; }
			std::vector<char> buf(1 << 20);
			char *p = buf.data(), *end = buf.data() + buf.size() - 40;
			for (uint32_t v = lo; v < hi; ++v) {
				p = put_u32(p, v);
				std::memcpy(p, ") cost:", 7); p += 7;
				int32_t c = levels[v];
				if (c < 0) { *p++ = '-'; p = put_u32(p, (uint32_t) (-(int64_t) c)); }
				else p = put_u32(p, (uint32_t) c);
				*p++ = '\n';
				if (p >= end) { std::fwrite(buf.data(), 1, (size_t) (p - buf.data()), f); p = buf.data(); }
			}
			size_t rest = (size_t) (p - buf.data());
			if (std::fwrite(buf.data(), 1, rest, f) != rest) status = BFS_EIO;
			std::fclose(f);
		}
	});
	return status.load();
}

} // extern "C"
