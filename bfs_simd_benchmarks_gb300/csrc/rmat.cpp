// rmat.cpp -- seeded R-MAT edge lists (the synthetic stand-ins for the
// reference's datasets; no counterpart in the reference, which downloads
// KONECT files, README.md:15-24).
//
// The candidate edges are defined in rmat_common.h (shared with the device
// generator, rmat_device.cu).  Self loops and duplicates are dropped on
// request (keeping the first occurrence), and candidates are drawn until
// exactly num_edges survive.  BFS_RMAT_PERMUTE relabels vertices with a
// seeded Fisher-Yates permutation.
#include <algorithm>
#include <atomic>
#include <cstring>

#include "internal.h"
#include "rmat_common.h"

namespace {

using bfsg::rmat::splitmix64;
using bfsg::rmat::Thresholds;
using bfsg::rmat::candidate;

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
	Thresholds t{bfsg::rmat::to_threshold(p->a), bfsg::rmat::to_threshold(p->a + p->b),
			bfsg::rmat::to_threshold(p->a + p->b + p->c)};
	const uint64_t seed = bfsg::rmat::mixed_seed(p->seed);
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
	if (p->flags & BFS_RMAT_PERMUTE) bfsg::rmat::permutation(seed, n, perm);
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
