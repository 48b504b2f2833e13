// rmat.cpp -- seeded R-MAT edge lists (the synthetic stand-ins for the
// reference's datasets; no counterpart in the reference, which downloads
// KONECT files, README.md:15-24).
//
// Each candidate edge i draws its quadrant bits from a counter-based hash
// (splitmix64 of seed and i), so the list does not depend on the thread
// count or the platform.  With d = 1-a-b-c, one level picks
//   (u,v) bits (0,0) with a, (0,1) with b, (1,0) with c, (1,1) with d.
// The scale is ceil(log2 N); ids >= N are rejected.  Self loops and duplicates
// are dropped on request (keeping the first occurrence), and candidates are
// drawn until exactly num_edges survive.  BFS_RMAT_PERMUTE relabels vertices
// with a seeded Fisher-Yates permutation.
#include <algorithm>
#include <atomic>
#include <cstring>

#include "internal.h"

namespace {

inline uint64_t splitmix64(uint64_t x) {
	x += 0x9E3779B97F4A7C15ull;
	x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
	x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
	return x ^ (x >> 31);
}

struct Thresholds {
	uint32_t ta, tab, tabc;
};

// Candidate `i`: returns false when rejected (id out of range or self loop).
inline bool candidate(uint64_t seed, uint64_t i, uint32_t scale, uint32_t n, const Thresholds &t,
		bool no_loops, uint32_t *pu, uint32_t *pv) {
	uint32_t u = 0, v = 0;
	uint64_t h = 0;
	for (uint32_t l = 0; l < scale; ++l) {
		if ((l & 1) == 0) h = splitmix64(seed ^ splitmix64(i * 64 + l));
		uint32_t r = (l & 1) ? (uint32_t) (h >> 32) : (uint32_t) h;
		uint32_t bu, bv;
		if (r < t.ta) { bu = 0; bv = 0; }
		else if (r < t.tab) { bu = 0; bv = 1; }
		else if (r < t.tabc) { bu = 1; bv = 0; }
		else { bu = 1; bv = 1; }
		u = (u << 1) | bu;
		v = (v << 1) | bv;
	}
	if (u >= n || v >= n) return false;
	if (no_loops && u == v) return false;
	*pu = u;
	*pv = v;
	return true;
}

// Drops repeated keys, keeping the first occurrence, order otherwise kept.
// Keys are hashed into buckets (each bucket keeps candidate order), buckets
// are sorted by (key, position) in parallel, and the survivors are compacted.
void dedup_stable(std::vector<uint64_t> &keys) {
	const uint64_t n = keys.size();
	if (n < 2) return;
	const unsigned nt = bfsg::host_threads();
	const unsigned kBits = 10, kBuckets = 1u << kBits;
	auto bucket_of = [&](uint64_t k) { return (unsigned) (splitmix64(k) >> (64 - kBits)); };
	std::vector<uint64_t> counts((size_t) nt * kBuckets, 0);
	std::vector<uint64_t> lo_of(nt + 1);
	for (unsigned t = 0; t <= nt; ++t) lo_of[t] = n * t / nt;
	bfsg::parallel_for(nt, [&](uint64_t a, uint64_t b, unsigned) {
		for (uint64_t t = a; t < b; ++t)
			for (uint64_t i = lo_of[t]; i < lo_of[t + 1]; ++i) counts[t * kBuckets + bucket_of(keys[i])]++;
	});
	std::vector<uint64_t> bstart(kBuckets + 1, 0);
	std::vector<uint64_t> off((size_t) nt * kBuckets);
	uint64_t acc = 0;
	for (unsigned bk = 0; bk < kBuckets; ++bk) {
		bstart[bk] = acc;
		for (unsigned t = 0; t < nt; ++t) { off[(size_t) t * kBuckets + bk] = acc; acc += counts[(size_t) t * kBuckets + bk]; }
	}
	bstart[kBuckets] = acc;
	std::vector<std::pair<uint64_t, uint64_t>> pairs(n);
	bfsg::parallel_for(nt, [&](uint64_t a, uint64_t b, unsigned) {
		for (uint64_t t = a; t < b; ++t)
			for (uint64_t i = lo_of[t]; i < lo_of[t + 1]; ++i)
				pairs[off[t * kBuckets + bucket_of(keys[i])]++] = {keys[i], i};
	});
	std::vector<uint8_t> keep(n, 0);
	bfsg::parallel_for(kBuckets, [&](uint64_t a, uint64_t b, unsigned) {
		for (uint64_t bk = a; bk < b; ++bk) {
			auto first = pairs.begin() + (long) bstart[bk], last = pairs.begin() + (long) bstart[bk + 1];
			std::sort(first, last);
			for (auto it = first; it != last; ++it)
				if (it == first || it->first != (it - 1)->first) keep[it->second] = 1;
		}
	});
	uint64_t w = 0;
	for (uint64_t i = 0; i < n; ++i)
		if (keep[i]) keys[w++] = keys[i];
	keys.resize(w);
}

inline uint32_t to_threshold(double p) {
	if (p <= 0) return 0;
	if (p >= 1) return 0xFFFFFFFFu;
	return (uint32_t) (p * 4294967296.0);
}

} // namespace

using namespace bfsg;

extern "C" int bfs_gen_rmat(const bfs_rmat_params *p, uint32_t *src, uint32_t *dst, uint64_t capacity) {
	if (!p || !src || !dst || p->num_vertices == 0 || capacity < p->num_edges) return BFS_EARG;
	if (p->a < 0 || p->b < 0 || p->c < 0 || p->a + p->b + p->c > 1.0 + 1e-12) return BFS_EARG;
	const uint32_t n = p->num_vertices;
	const uint64_t m = p->num_edges;
	const bool no_loops = p->flags & BFS_RMAT_NO_SELF_LOOPS;
	const bool dedup = p->flags & BFS_RMAT_DEDUP;
	if (n == 1 && no_loops && m > 0) return BFS_EARG;
	if (dedup) {
		uint64_t max_m = (uint64_t) n * (no_loops ? n - 1 : n);
		if (m > max_m) return BFS_EARG;
	}
	const uint32_t scale = ceil_log2(n);
	Thresholds t{to_threshold(p->a), to_threshold(p->a + p->b), to_threshold(p->a + p->b + p->c)};
	const uint64_t seed = splitmix64(p->seed ^ 0x5851F42D4C957F2Dull);
	const unsigned nt = host_threads();

	// Accepted edges as 64-bit keys (u << 32 | v) in candidate order.
	std::vector<uint64_t> keys;
	keys.reserve(m + m / 8 + 16);
	uint64_t next_candidate = 0;
	while (keys.size() < m) {
		uint64_t want = m - keys.size();
		uint64_t batch = want + want / 6 + 1024;
		// Draw `batch` candidates in parallel; concatenate per-thread runs in order.
		std::vector<std::vector<uint64_t>> part(nt);
		uint64_t base = next_candidate;
		parallel_for(batch, [&](uint64_t lo, uint64_t hi, unsigned tid) {
			auto &out = part[tid];
			out.reserve(hi - lo);
			for (uint64_t i = lo; i < hi; ++i) {
				uint32_t u, v;
				if (candidate(seed, base + i, scale, n, t, no_loops, &u, &v))
					out.push_back(((uint64_t) u << 32) | v);
			}
		});
		next_candidate += batch;
		for (auto &pv : part) keys.insert(keys.end(), pv.begin(), pv.end());
		if (dedup) dedup_stable(keys);
	}
	keys.resize(m);

	std::vector<uint32_t> perm;
	if (p->flags & BFS_RMAT_PERMUTE) {
		perm.resize(n);
		for (uint32_t v = 0; v < n; ++v) perm[v] = v;
		uint64_t st = splitmix64(seed ^ 0xD1B54A32D192ED03ull);
		for (uint32_t v = n - 1; v > 0; --v) {
			st = splitmix64(st);
			uint32_t j = (uint32_t) (((unsigned __int128) st * (uint64_t) (v + 1)) >> 64);
			std::swap(perm[v], perm[j]);
		}
	}
	parallel_for(m, [&](uint64_t lo, uint64_t hi, unsigned) {
		for (uint64_t i = lo; i < hi; ++i) {
			uint32_t u = (uint32_t) (keys[i] >> 32), v = (uint32_t) keys[i];
			if (!perm.empty()) { u = perm[u]; v = perm[v]; }
			src[i] = u;
			dst[i] = v;
		}
	});
	return BFS_OK;
}
