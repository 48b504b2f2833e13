// autotune.cpp -- per-graph choice of the tile shape and the traversal options
// by measurement.
//
// The reference fixes them by hand: W and S on the command line (picked with
// tools/tile-size-computer and the stripe-length sweeps of
// tools/stripe_length/process.sh) and the direction switch at T_RATIO = 20
// (apps/bfs_simd/bfs.cpp:1171).  Here:
//   - bfs_tune_options times candidate options on a resident graph (every
//     candidate runs all the given sources, timed by the kernels' CUDA events)
//     and keeps the best by coordinate descent: one option at a time over its
//     candidate values, the others fixed, two sweeps;
//   - bfs_autotune builds the graph at every tile width x stripe length,
//     tunes each and keeps the fastest, with an optional cache file keyed by
//     the graph's size and out-degree signature.
// Levels never depend on these choices (they are checked equal in the tests);
// only time does.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/bfs_gb300.h"

namespace {

struct Tuner {
	bfs_graph *g;
	const uint32_t *sources;
	uint32_t ns;
	uint32_t tile_width, stripe_length;
	uint8_t *d_levels = nullptr;  // batch output
	bfs_tune_result *res;
	uint32_t load_flags = 0;      // the layout of the graph being tuned
};

void add_trial(Tuner &t, const bfs_options &o, double gteps, uint32_t kind) {
	bfs_tune_result *r = t.res;
	if (r->num_trials >= BFS_TUNE_MAX_TRIALS) return;
	bfs_tune_trial &tr = r->trials[r->num_trials++];
	tr.tile_width = t.tile_width;
	tr.stripe_length = t.stripe_length;
	tr.options = o;
	tr.gteps = gteps;
	tr.kind = kind;
	tr.load_flags = t.load_flags;
}

// Single-source GTEPS of the sources with options o (0 on any error).
double time_single(Tuner &t, const bfs_options &o) {
	if (bfs_set_options(t.g, &o) != BFS_OK) return 0;
	double ms = 0, edges = 0;
	for (uint32_t i = 0; i < t.ns; ++i) {
		bfs_stats st;
		if (bfs_run(t.g, t.sources[i], nullptr, nullptr, &st) != BFS_OK) return 0;
		ms += st.kernel_ms;
		edges += (double) st.edges_traversed;
	}
	return ms > 0 ? edges / (ms * 1e-3) / 1e9 : 0;
}

double time_batch(Tuner &t, const bfs_options &o) {
	if (bfs_set_options(t.g, &o) != BFS_OK) return 0;
	bfs_batch_stats st;
	if (bfs_run_batch(t.g, t.sources, t.ns, t.d_levels, nullptr, &st) != BFS_OK) return 0;
	return st.device_ms > 0 ? (double) st.edges_traversed / (st.device_ms * 1e-3) / 1e9 : 0;
}

struct Axis {
	uint32_t bfs_options::*field;
	std::vector<uint32_t> values;
};

// Coordinate descent over the axes; returns the best GTEPS, leaves best in o.
template <class F> double descend(Tuner &t, bfs_options &o, const std::vector<Axis> &axes, F time_fn, uint32_t kind) {
	double best = time_fn(t, o);
	add_trial(t, o, best, kind);
	for (int sweep = 0; sweep < 2; ++sweep) {
		bool changed = false;
		for (const Axis &ax : axes) {
			const uint32_t keep = o.*(ax.field);
			uint32_t pick = keep;
			for (uint32_t v : ax.values) {
				if (v == keep) continue;
				bfs_options c = o;
				c.*(ax.field) = v;
				if (c.cta_max_degree < c.warp_max_degree) continue;
				const double x = time_fn(t, c);
				add_trial(t, c, x, kind);
				if (x > best * 1.01) {  // 1% above noise
					best = x;
					pick = v;
				}
			}
			if (pick != keep) changed = true;
			o.*(ax.field) = pick;
		}
		if (!changed) break;
	}
	return best;
}

uint64_t fnv1a(uint64_t h, const void *p, size_t n) {
	const uint8_t *b = (const uint8_t *) p;
	for (size_t i = 0; i < n; ++i) {
		h ^= b[i];
		h *= 1099511628211ull;
	}
	return h;
}

const char *kFields[] = {"mode", "to_dense_ratio", "to_sparse_ratio", "warp_max_degree", "cta_max_degree",
		"bottom_up", "batch_planes", "batch_budget_mb", "batch_single_max", "batch_push_div", "switch_rule",
		"bu_alpha", "td_beta", "ctas_per_sm"};
constexpr int kNumFields = 14;
uint32_t *field_ptr(bfs_options &o, int i) {
	uint32_t *f[] = {&o.mode, &o.to_dense_ratio, &o.to_sparse_ratio, &o.warp_max_degree, &o.cta_max_degree,
			&o.bottom_up, &o.batch_planes, &o.batch_budget_mb, &o.batch_single_max, &o.batch_push_div,
			&o.switch_rule, &o.bu_alpha, &o.td_beta, &o.ctas_per_sm};
	return f[i];
}

// Cache lines: "<key> W S single batch name=value ...".
bool cache_lookup(const char *path, const std::string &key, bfs_tune_result *r) {
	FILE *f = std::fopen(path, "r");
	if (!f) return false;
	char line[2048];
	bool found = false;
	while (std::fgets(line, sizeof line, f)) {
		char k[64];
		unsigned w = 0, s = 0;
		double sg = 0, bg = 0;
		int off = 0;
		if (std::sscanf(line, "%63s %u %u %lf %lf%n", k, &w, &s, &sg, &bg, &off) != 5 || key != k) continue;
		bfs_options o;
		bfs_options_default(&o);
		const char *p = line + off;
		char name[64];
		unsigned v = 0;
		int used = 0;
		while (std::sscanf(p, " %63[^=]=%u%n", name, &v, &used) == 2) {
			for (int i = 0; i < kNumFields; ++i)
				if (!std::strcmp(name, kFields[i])) *field_ptr(o, i) = v;
			p += used;
		}
		r->tile_width = w;
		r->stripe_length = s;
		r->options = o;
		r->single_gteps = sg;
		r->batch_gteps = bg;
		r->from_cache = 1;
		const char *lf = std::strstr(line, " layout=");
		r->load_flags = lf ? (uint32_t) std::strtoul(lf + 8, nullptr, 10) : 0u;
		found = true;  // the last matching line wins
	}
	std::fclose(f);
	return found;
}

void cache_append(const char *path, const std::string &key, const bfs_tune_result *r) {
	FILE *f = std::fopen(path, "a");
	if (!f) return;
	std::fprintf(f, "%s %u %u %.6f %.6f", key.c_str(), r->tile_width, r->stripe_length, r->single_gteps,
			r->batch_gteps);
	bfs_options o = r->options;
	for (int i = 0; i < kNumFields; ++i) std::fprintf(f, " %s=%u", kFields[i], *field_ptr(o, i));
	std::fprintf(f, " layout=%u\n", r->load_flags);
	std::fclose(f);
}

int tune(Tuner &t, uint32_t flags, bfs_options *best_out, double *single_out, double *batch_out, double *def_single,
		double *def_batch) {
	bfs_options o;
	int st = bfs_get_options(t.g, &o);
	if (st) return st;
	*single_out = *batch_out = 0;
	if (flags & BFS_TUNE_SINGLE) {
		time_single(t, o);  // warm-up
		const std::vector<Axis> axes = {
				{&bfs_options::bottom_up, {BFS_BU_PULL, BFS_BU_STREAM}},
				{&bfs_options::ctas_per_sm, {0, 1}},
				{&bfs_options::switch_rule, {BFS_SWITCH_REFERENCE, BFS_SWITCH_UNVISITED}},
				{&bfs_options::to_dense_ratio, {5, 10, 20, 40, 80, 160}},
				{&bfs_options::to_sparse_ratio, {5, 10, 20, 40, 80, 160}},
				{&bfs_options::bu_alpha, {2, 4, 8, 14, 32, 64}},
				{&bfs_options::td_beta, {8, 24, 64, 256}},
				{&bfs_options::warp_max_degree, {8, 16, 32, 64}},
				{&bfs_options::cta_max_degree, {512, 1024, 4096, 16384}},
		};
		const uint32_t first = t.res->num_trials;
		*single_out = descend(t, o, axes, time_single, BFS_TUNE_SINGLE);
		if (def_single && first < t.res->num_trials) *def_single = t.res->trials[first].gteps;
	}
	if ((flags & BFS_TUNE_BATCH) && t.ns > o.batch_single_max) {
		bfs_graph_info info;
		bfs_graph_get_info(t.g, &info);
		if (cudaMalloc(&t.d_levels, (size_t) t.ns * info.num_vertices) != cudaSuccess) {
			cudaGetLastError();
			return BFS_ENOMEM;
		}
		time_batch(t, o);  // warm-up (allocates the batch state)
		const std::vector<Axis> axes = {{&bfs_options::batch_push_div, {4, 8, 16, 32, 64, 128}},
				{&bfs_options::ctas_per_sm, {0, 1}}};
		const uint32_t first = t.res->num_trials;
		*batch_out = descend(t, o, axes, time_batch, BFS_TUNE_BATCH);
		if (def_batch && first < t.res->num_trials) *def_batch = t.res->trials[first].gteps;
		cudaFree(t.d_levels);
		t.d_levels = nullptr;
	}
	bfs_set_options(t.g, &o);
	*best_out = o;
	return BFS_OK;
}

} // namespace

extern "C" {

// tools/tile-size-computer/tile-size-computer.cpp:21-56, restated: the
// smallest power-of-two width (from 64) whose SIDE^2 tile count fits 32 bits
// and whose tiles average at least 8 edges is the minimum; the maximum is
// a quarter of the first width, doubling from there, at which SIDE <= 64.
int bfs_tile_size_range(uint32_t num_vertices, uint64_t num_edges, uint32_t *min_width, uint32_t *max_width) {
	if (!min_width || !max_width || num_vertices == 0 || num_edges > 0xFFFFFFFFull) return BFS_EARG;
	auto side = [&](uint64_t w) { return (uint64_t) num_vertices / w + (num_vertices % w ? 1 : 0); };
	auto tiles = [&](uint64_t w) { const uint64_t sl = side(w); return sl * sl; };
	uint64_t w = 64;
	while (tiles(w) > 4294967295ull) w *= 2;
	while ((uint32_t) (num_edges / tiles(w)) < 8) {
		if (w > (1ull << 40)) return BFS_EARG;  // too few edges for any width (the tool would not stop)
		w *= 2;
	}
	const uint64_t lo = w;
	while (side(w) > 64) w *= 2;
	w = std::max<uint64_t>(1, w / 2);
	if (w > 0xFFFFFFFFull || lo > 0xFFFFFFFFull) return BFS_EARG;
	*min_width = (uint32_t) lo;
	*max_width = (uint32_t) w;
	return BFS_OK;
}

int bfs_tune_options(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, uint32_t flags,
		bfs_tune_result *result) {
	if (!g || !sources || !num_sources || !result || !(flags & (BFS_TUNE_SINGLE | BFS_TUNE_BATCH))) return BFS_EARG;
	if ((flags & BFS_TUNE_BATCH) && num_sources > BFS_BATCH_MAX_SOURCES) return BFS_EARG;
	std::memset(result, 0, sizeof(*result));
	bfs_graph_info info;
	int st = bfs_graph_get_info(g, &info);
	if (st) return st;
	for (uint32_t i = 0; i < num_sources; ++i)
		if (sources[i] >= info.num_vertices) return BFS_EARG;
	Tuner t{g, sources, num_sources, info.tile_width, info.stripe_length, nullptr, result};
	result->tile_width = info.tile_width;
	result->stripe_length = info.stripe_length;
	return tune(t, flags, &result->options, &result->single_gteps, &result->batch_gteps,
			&result->default_single_gteps, &result->default_batch_gteps);
}

int bfs_autotune(uint32_t num_vertices, uint64_t num_edges, const uint32_t *src, const uint32_t *dst,
		const uint32_t *sources, uint32_t num_sources, const uint32_t *tile_widths, uint32_t num_widths,
		const uint32_t *stripe_lengths, uint32_t num_stripes, uint32_t flags, const char *cache_path,
		bfs_tune_result *result) {
	if (!result || !sources || !num_sources || !stripe_lengths || !num_stripes || (num_edges && (!src || !dst)) ||
			!(flags & (BFS_TUNE_SINGLE | BFS_TUNE_BATCH)) || (num_widths && !tile_widths))
		return BFS_EARG;
	std::memset(result, 0, sizeof(*result));
	std::vector<uint32_t> widths(tile_widths, tile_widths + num_widths);
	if (widths.empty()) {
		// the tile-size computer's range (powers of two), within what the packing holds
		uint32_t lo = 0, hi = 0;
		int st = bfs_tile_size_range(num_vertices, num_edges, &lo, &hi);
		if (st) return st;
		for (uint64_t w = lo; w <= std::max(lo, hi) && w <= 8192; w *= 2) widths.push_back((uint32_t) w);
		if (widths.empty()) widths.push_back(std::min<uint32_t>(lo, 8192));
	}
	tile_widths = widths.data();
	num_widths = (uint32_t) widths.size();
	for (uint32_t i = 0; i < num_sources; ++i)
		if (sources[i] >= num_vertices) return BFS_EARG;
	// signature: N, E, out-degrees, flags and the shapes searched
	std::vector<uint32_t> deg(num_vertices, 0);
	for (uint64_t i = 0; i < num_edges; ++i)
		if (src[i] < num_vertices) deg[src[i]]++;
	uint64_t h = 1469598103934665603ull;
	h = fnv1a(h, &num_vertices, sizeof num_vertices);
	h = fnv1a(h, &num_edges, sizeof num_edges);
	h = fnv1a(h, deg.data(), deg.size() * sizeof(uint32_t));
	h = fnv1a(h, &flags, sizeof flags);
	h = fnv1a(h, tile_widths, num_widths * sizeof(uint32_t));
	h = fnv1a(h, stripe_lengths, num_stripes * sizeof(uint32_t));
	char key[32];
	std::snprintf(key, sizeof key, "%016llx", (unsigned long long) h);
	if (cache_path && cache_lookup(cache_path, key, result)) return BFS_OK;

	const bool by_single = flags & BFS_TUNE_SINGLE;
	// layouts: the caller's ids, and (single-source tuning only) the degree order
	std::vector<uint32_t> layouts = {0u};
	if ((flags & BFS_TUNE_LAYOUTS) && !(flags & BFS_TUNE_BATCH)) layouts.push_back(BFS_LOAD_DEGREE_ORDER);
	const uint32_t build_flags = (flags & BFS_TUNE_DEVICE_BUILD) ? BFS_LOAD_DEVICE_BUILD : 0u;
	double best = -1;
	bool first = true;
	int last_err = BFS_EUNSUPPORTED;
	for (uint32_t layout : layouts)
	for (uint32_t wi = 0; wi < num_widths; ++wi) {
		for (uint32_t si = 0; si < num_stripes; ++si) {
			bfs_graph *g = nullptr;
			int st = bfs_graph_from_edges(num_vertices, num_edges, src, dst, tile_widths[wi], stripe_lengths[si],
					build_flags | layout, &g);
			if (st) {
				last_err = st;
				continue;  // a shape the packing cannot hold
			}
			Tuner t{g, sources, num_sources, tile_widths[wi], stripe_lengths[si], nullptr, result, layout};
			bfs_options o;
			double sg = 0, bg = 0, dsg = 0, dbg = 0;
			st = tune(t, flags, &o, &sg, &bg, &dsg, &dbg);
			bfs_graph_free(g);
			if (st) {
				last_err = st;
				continue;
			}
			if (first) {
				result->default_single_gteps = dsg;
				result->default_batch_gteps = dbg;
				first = false;
			}
			const double score = by_single ? sg : bg;
			if (score > best) {
				best = score;
				result->tile_width = tile_widths[wi];
				result->stripe_length = stripe_lengths[si];
				result->options = o;
				result->single_gteps = sg;
				result->batch_gteps = bg;
				result->load_flags = layout;
			}
		}
	}
	if (best < 0) return last_err;
	if (cache_path) cache_append(cache_path, key, result);
	return BFS_OK;
}

} // extern "C"
