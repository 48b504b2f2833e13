// layout.cpp -- edge orders of the reference's file families, and the packed
// column-major tile stream that the bottom-up kernel streams from HBM.
//
// Orders (restated from the tools, 0-based):
//   CSR order        : stable bucketing of the input by source
//                      (tools/csr_tiling/page_rank.cpp:531-567).
//   column-major COO : tiles of W x W; stripes of S tile rows; inside a stripe
//                      tiles go column by column, rows inner
//                      (tools/column_major_tile/kcore.cpp:378-415), and inside a
//                      tile edges keep CSR order (tools/coo_tiling/page_rank.cpp:416-447).
//                      That is a stable sort of the CSR list by
//                      (stripe(u), col(v), row(u)); because CSR order is already
//                      sorted by u, a stable counting sort by the segment key
//                      (stripe(u), col(v)) alone produces it.
//
// Packed stream (this project's HBM layout, no counterpart in the reference):
//   Tile columns are cut into column groups (runs of whole columns with about
//   equal edge counts).  For stripe k and group g the edges of the group's
//   columns inside stripe k are one contiguous run of the column-major order;
//   each becomes one segment, padded with dummy words to a multiple of
//   four words so that every segment starts on a 16-byte boundary (the TMA
//   rule).  Segments are stored group-major, seg_off[g*num_stripes + k], so
//   that a group's segments of consecutive stripes are one contiguous range
//   and a single bulk copy moves several of them.
//   An edge u->v of stripe k, column c of group g is one 32-bit word:
//       bits [0, vbits)            v - c*W          (destination inside its column)
//       bits [vbits, vbits+cbits)  c - group_col[g] (column inside the group)
//       bits [vbits+cbits, 32)     u - k*S*W        (source inside the stripe)
//   vbits = ceil(log2 W), ubits = ceil(log2 (S*W)), cbits = 32 - vbits - ubits.
//   Padding words name a dummy destination just past the group's vertices
//   (see pack_tiles), which the kernel treats as already visited.
#include <algorithm>
#include <atomic>
#include <cstring>

#include "internal.h"

namespace bfsg {

int csr_from_edges(uint32_t n, uint64_t m, const uint32_t *src, const uint32_t *dst,
		std::vector<uint32_t> &csr_src, std::vector<uint32_t> &csr_dst, std::vector<uint32_t> &degrees) {
	degrees.assign(n, 0);
	for (uint64_t i = 0; i < m; ++i) {
		if (src[i] >= n || dst[i] >= n) return BFS_EFORMAT;
		degrees[src[i]]++;
	}
	std::vector<uint64_t> start(n + 1, 0);
	for (uint32_t v = 0; v < n; ++v) start[v + 1] = start[v] + degrees[v];
	csr_src.resize(m);
	csr_dst.resize(m);
	for (uint64_t i = 0; i < m; ++i) {
		uint64_t pos = start[src[i]]++;
		csr_src[pos] = src[i];
		csr_dst[pos] = dst[i];
	}
	return BFS_OK;
}

// Position of tile (row, col) in the column-major numbering of
// tools/column_major_tile/kcore.cpp:378-415, which apps/bfs_simd/bfs.cpp:262-275
// reads back as start_row*SIDE + col*step + (row - start_row).
static inline uint64_t colmajor_tile_id(uint64_t row, uint64_t col, uint32_t side, uint32_t s) {
	uint64_t start_row = row - row % s;
	uint64_t step = (start_row + s <= side) ? s : side - start_row;
	return start_row * side + col * step + (row - start_row);
}

int colmajor_from_csr(uint32_t n, uint64_t m, uint32_t w, uint32_t s, const uint32_t *csr_src,
		const uint32_t *csr_dst, std::vector<uint32_t> &heads, std::vector<uint32_t> &tails,
		std::vector<uint32_t> *tile_offsets) {
	uint32_t side = side_length_of(n, w);
	uint32_t stripes = (side + s - 1) / s;
	uint64_t nseg = (uint64_t) stripes * side;
	std::vector<uint64_t> cnt(nseg + 1, 0);
	for (uint64_t i = 0; i < m; ++i) {
		uint64_t key = (uint64_t) (csr_src[i] / w / s) * side + csr_dst[i] / w;
		cnt[key + 1]++;
	}
	for (uint64_t k = 0; k < nseg; ++k) cnt[k + 1] += cnt[k];
	heads.resize(m);
	tails.resize(m);
	for (uint64_t i = 0; i < m; ++i) {
		uint64_t key = (uint64_t) (csr_src[i] / w / s) * side + csr_dst[i] / w;
		uint64_t pos = cnt[key]++;
		heads[pos] = csr_src[i];
		tails[pos] = csr_dst[i];
	}
	if (tile_offsets) {
		uint64_t num_tiles = (uint64_t) side * side;
		std::vector<uint64_t> tc(num_tiles + 1, 0);
		for (uint64_t i = 0; i < m; ++i) tc[colmajor_tile_id(heads[i] / w, tails[i] / w, side, s) + 1]++;
		tile_offsets->resize(num_tiles);
		for (uint64_t t = 0; t < num_tiles; ++t) {
			tc[t + 1] += tc[t];
			(*tile_offsets)[t] = (uint32_t) tc[t];
		}
	}
	return BFS_OK;
}

// Checks that heads/tails are in column-major tile order and, when present,
// that tile_offsets agrees with the edges (the reference trusts its files;
// a drop-in loader reports inconsistent ones instead).
int validate_colmajor(const HostGraph &g) {
	const uint32_t side = g.side, w = g.w, s = g.s;
	const uint64_t num_tiles = (uint64_t) side * side;
	std::atomic<int> bad{0};
	parallel_for(g.m, [&](uint64_t lo, uint64_t hi, unsigned) {
		uint64_t prev = 0;
		bool first = true;
		for (uint64_t i = lo; i < hi; ++i) {
			uint32_t u = g.heads[i], v = g.tails[i];
			if (u >= g.n || v >= g.n) { bad = 1; return; }
			uint64_t t = colmajor_tile_id(u / w, v / w, side, s);
			if (!first && t < prev) { bad = 1; return; }
			prev = t;
			first = false;
		}
		if (lo > 0 && hi > lo) {
			uint32_t u0 = g.heads[lo - 1], v0 = g.tails[lo - 1];
			if (u0 < g.n && v0 < g.n &&
					colmajor_tile_id(u0 / w, v0 / w, side, s) > colmajor_tile_id(g.heads[lo] / w, g.tails[lo] / w, side, s))
				bad = 1;
		}
	});
	if (bad) return BFS_EFORMAT;
	if (!g.tile_offsets.empty()) {
		if (g.tile_offsets.size() != num_tiles) return BFS_EFORMAT;
		if (num_tiles && g.tile_offsets[0] != 0) return BFS_EFORMAT;
		for (uint64_t t = 0; t + 1 < num_tiles; ++t)
			if (g.tile_offsets[t] > g.tile_offsets[t + 1]) return BFS_EFORMAT;
		if (num_tiles && g.tile_offsets[num_tiles - 1] > g.m) return BFS_EFORMAT;
		parallel_for(num_tiles, [&](uint64_t lo, uint64_t hi, unsigned) {
			for (uint64_t t = lo; t < hi && !bad; ++t) {
				uint64_t a = g.tile_offsets[t], b = (t + 1 < num_tiles) ? g.tile_offsets[t + 1] : g.m;
				for (uint64_t i = a; i < b; ++i) {
					if (colmajor_tile_id(g.heads[i] / w, g.tails[i] / w, side, s) != t) { bad = 1; break; }
				}
			}
		});
		if (bad) return BFS_EFORMAT;
	}
	return BFS_OK;
}

// Row starts from out-degrees (apps/bfs_simd/bfs.cpp:1108-1113) and checks.
int finish_csr(HostGraph &g) {
	g.row_off.assign((size_t) g.n + 1, 0);
	uint64_t acc = 0;
	g.max_degree = 0;
	for (uint32_t v = 0; v < g.n; ++v) {
		g.row_off[v] = (uint32_t) acc;
		acc += g.degrees[v];
		g.max_degree = std::max(g.max_degree, g.degrees[v]);
	}
	if (acc != g.m || acc > 0xFFFFFFFFull) return BFS_EFORMAT;
	g.row_off[g.n] = (uint32_t) acc;
	return BFS_OK;
}

int plan_groups(uint32_t n, uint32_t w, uint32_t s, uint32_t side, const std::vector<uint64_t> &col_edges,
		uint64_t m, uint32_t target_groups, uint32_t max_group_vertices, PackedTiles &out) {
	out.vbits = ceil_log2(w);
	out.ubits = ceil_log2((uint64_t) s * w);
	if (out.vbits + out.ubits > 31) return BFS_EUNSUPPORTED;
	out.cbits = std::min<uint32_t>(32 - out.vbits - out.ubits, 16);  // keeps every shift below 32
	// A group spans at most cmask - ceil(32/W) columns so that the padding
	// word of any group can still name the group's dummy slot (below).
	const uint64_t cmask = (1ull << out.cbits) - 1;
	const uint64_t pad_cols = (32 + w - 1) / w;
	if (cmask < pad_cols + 1) return BFS_EUNSUPPORTED;
	uint64_t max_cols = cmask - pad_cols;
	if (max_cols > 0xFFFF) max_cols = 0xFFFF;
	uint64_t cols_by_smem = std::max<uint64_t>(1, max_group_vertices / w);
	if (w > max_group_vertices) return BFS_EUNSUPPORTED;
	max_cols = std::min(max_cols, cols_by_smem);

	// Greedy column groups of about m/target_groups edges.
	if (target_groups == 0) target_groups = 1;
	uint64_t target = std::max<uint64_t>(1, (m + target_groups - 1) / target_groups);
	out.group_col.clear();
	out.group_col.push_back(0);
	uint64_t acc = 0, cols = 0;
	for (uint32_t c = 0; c < side; ++c) {
		acc += col_edges[c];
		cols++;
		if (acc >= target || cols >= max_cols) {
			out.group_col.push_back(c + 1);
			acc = 0;
			cols = 0;
		}
	}
	if (out.group_col.back() != side) out.group_col.push_back(side);
	out.num_groups = (uint32_t) out.group_col.size() - 1;
	out.max_group_vertices = 0;
	for (uint32_t gi = 0; gi < out.num_groups; ++gi) {
		uint64_t v0 = (uint64_t) out.group_col[gi] * w;
		uint64_t v1 = std::min<uint64_t>((uint64_t) out.group_col[gi + 1] * w, n);
		out.max_group_vertices = std::max<uint32_t>(out.max_group_vertices, (uint32_t) (v1 - v0));
	}
	(void) s;
	return BFS_OK;
}

uint32_t group_pad_word(const PackedTiles &out, uint32_t gi, uint32_t n, uint32_t w) {
	// Padding words decode to destination 32*ceil(group_vertices/32): the slot
	// right after the group's bitmap, which the kernel keeps "visited", so a
	// padding word is skipped by the ordinary visited test.
	uint64_t v0 = (uint64_t) out.group_col[gi] * w;
	uint64_t v1 = std::min<uint64_t>((uint64_t) out.group_col[gi + 1] * w, n);
	uint64_t d = (v1 - v0 + 31) / 32 * 32;
	return (uint32_t) (d % w) | (uint32_t) ((d / w) << out.vbits);
}

int segment_offsets(const std::vector<uint64_t> &seg_count, PackedTiles &out) {
	const uint64_t nseg = seg_count.size();
	out.seg_off.assign(nseg + 1, 0);
	uint64_t words = 0;
	for (uint64_t j = 0; j < nseg; ++j) {
		out.seg_off[j] = (uint32_t) words;
		words += (seg_count[j] + 3) & ~uint64_t(3);
		if (words > 0xFFFFFFF0ull) return BFS_EUNSUPPORTED;
	}
	out.seg_off[nseg] = (uint32_t) words;
	return BFS_OK;
}

int pack_tiles(const HostGraph &g, uint32_t target_groups, uint32_t max_group_vertices, PackedTiles &out) {
	const uint32_t w = g.w, s = g.s, side = g.side, stripes = g.num_stripes;
	// In-edges per tile column and the in-degree > 0 bitmap.
	std::vector<uint64_t> col_edges(side, 0);
	out.hasin_bits.assign(((size_t) g.n + 31) / 32, 0);
	for (uint64_t i = 0; i < g.m; ++i) {
		uint32_t v = g.tails[i];
		col_edges[v / w]++;
		out.hasin_bits[v >> 5] |= 1u << (v & 31);
	}
	int st = plan_groups(g.n, w, s, side, col_edges, g.m, target_groups, max_group_vertices, out);
	if (st) return st;
	std::vector<uint32_t> group_of(side);
	for (uint32_t gi = 0; gi < out.num_groups; ++gi)
		for (uint32_t c = out.group_col[gi]; c < out.group_col[gi + 1]; ++c) group_of[c] = gi;

	// Segment sizes: heads/tails are in column-major order, so the edges of
	// (stripe, group) are contiguous; count them.
	const uint64_t nseg = (uint64_t) stripes * out.num_groups;
	std::vector<uint64_t> seg_count(nseg, 0);
	for (uint64_t i = 0; i < g.m; ++i) {
		uint32_t k = g.heads[i] / w / s;
		seg_count[(uint64_t) group_of[g.tails[i] / w] * stripes + k]++;
	}
	if ((st = segment_offsets(seg_count, out))) return st;
	out.words.assign(out.seg_off[nseg], 0);
	std::vector<uint32_t> pad_word(out.num_groups);
	for (uint32_t gi = 0; gi < out.num_groups; ++gi) pad_word[gi] = group_pad_word(out, gi, g.n, w);
	for (uint64_t j = 0; j < nseg; ++j) {
		uint32_t gi = (uint32_t) (j / stripes);
		for (uint64_t x = out.seg_off[j] + seg_count[j]; x < out.seg_off[j + 1]; ++x) out.words[x] = pad_word[gi];
	}

	// Fill in file order: each edge goes to the next slot of its segment.
	std::vector<uint64_t> fill(out.seg_off.begin(), out.seg_off.end() - 1);
	const uint32_t cshift = out.vbits, ushift = out.vbits + out.cbits;
	for (uint64_t i = 0; i < g.m; ++i) {
		uint32_t u = g.heads[i], v = g.tails[i];
		uint32_t k = u / w / s, c = v / w, gi = group_of[c];
		uint64_t j = (uint64_t) gi * stripes + k;
		uint32_t word = (v - c * w) | ((c - out.group_col[gi]) << cshift) | ((u - k * s * w) << ushift);
		out.words[fill[j]++] = word;
	}
	return BFS_OK;
}

} // namespace bfsg
