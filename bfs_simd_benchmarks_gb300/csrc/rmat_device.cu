// rmat_device.cu -- the seeded R-MAT generator on the GPU, drawing exactly the
// edge list of the host generator (bfs_gen_rmat, rmat.cpp): the same
// candidates (rmat_common.h), the same first-occurrence deduplication in
// candidate order, the same truncation to num_edges and the same
// relabelling.  No counterpart in the reference (it reads downloaded files).
//
// Candidates are drawn in rounds of up to kMaxRound.  Every valid candidate
// is inserted into a device hash table of edge keys (u << 32 | v, open
// addressing) that also keeps, per key, the smallest candidate index seen
// (atomicMin); after the round, a candidate is a first occurrence exactly
// when the table's index for its key is its own.  First occurrences are
// compacted in candidate order (an exclusive scan) behind the edges kept so
// far, until num_edges are kept.  The relabelling is a sequential
// Fisher-Yates shuffle computed on the host and applied on the device.
#include <algorithm>
#include <vector>

#include "../../include/bfs_gb300.h"
#include "build_device.h"
#include "device_common.cuh"
#include "rmat_common.h"

namespace {

using namespace bfsg;

constexpr uint64_t kEmptyKey = 0xFFFFFFFFFFFFFFFFull;  // u = v = 2^32-1: not an edge (ids < N < 2^32)
constexpr uint32_t kMaxRound = 1u << 27;                // candidates per round

struct Table {
	unsigned long long *key;
	uint32_t *first;  // smallest candidate index of the key
	uint64_t mask;    // slots - 1
};

__device__ __forceinline__ uint64_t slot_of(uint64_t key, uint64_t mask) { return rmat::splitmix64(key) & mask; }

// Draws candidates [c0, c0 + count) and inserts the valid ones.  key_of[i]
// (kEmptyKey if rejected) and slot[i] record where each went.  A probe
// sequence longer than the table sets *err (never at the load factors used).
__global__ void k_rmat_draw(uint64_t seed, uint64_t c0, uint32_t count, uint32_t scale, uint32_t n,
		rmat::Thresholds t, int no_loops, int dedup, Table tb, unsigned long long *key_of, uint32_t *slot,
		int *err) {
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
		uint32_t u, v;
		uint64_t key = kEmptyKey;
		uint32_t s = 0;
		if (rmat::candidate(seed, c0 + i, scale, n, t, no_loops, &u, &v)) {
			key = ((uint64_t) u << 32) | v;
			if (dedup) {
				uint64_t h = slot_of(key, tb.mask);
				for (uint64_t probe = 0;; ++probe) {
					if (probe > tb.mask) { atomicExch(err, BFS_ENOMEM); key = kEmptyKey; break; }
					const unsigned long long old = atomicCAS(tb.key + h, kEmptyKey, (unsigned long long) key);
					if (old == kEmptyKey || old == key) {
						atomicMin(tb.first + h, (uint32_t) (c0 + i));
						s = (uint32_t) h;
						break;
					}
					h = (h + 1) & tb.mask;
				}
			}
		}
		key_of[i] = key;
		slot[i] = s;
	}
}

// keep[i] = 1 when candidate c0 + i is valid and the first of its key.
__global__ void k_rmat_first(uint64_t c0, uint32_t count, int dedup, Table tb, const unsigned long long *key_of,
		const uint32_t *slot, uint32_t *keep) {
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
		const bool valid = key_of[i] != kEmptyKey;
		keep[i] = valid && (!dedup || __ldg(tb.first + slot[i]) == (uint32_t) (c0 + i)) ? 1u : 0u;
	}
}

// Kept candidates to src/dst at kept + their rank, up to m edges in all.
__global__ void k_rmat_compact(uint32_t count, const unsigned long long *key_of, const uint32_t *keep,
		const uint32_t *rank, uint64_t kept, uint64_t m, uint32_t *src, uint32_t *dst) {
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
		if (!keep[i]) continue;
		const uint64_t pos = kept + rank[i];
		if (pos >= m) continue;
		src[pos] = (uint32_t) (key_of[i] >> 32);
		dst[pos] = (uint32_t) key_of[i];
	}
}

__global__ void k_rmat_relabel(uint64_t m, const uint32_t *perm, uint32_t *src, uint32_t *dst) {
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t) gridDim.x * blockDim.x) {
		src[i] = __ldg(perm + src[i]);
		dst[i] = __ldg(perm + dst[i]);
	}
}

__global__ void k_fill_u64(unsigned long long *p, uint64_t count, unsigned long long x) {
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (uint64_t) gridDim.x * blockDim.x)
		p[i] = x;
}

struct DevTmp {
	std::vector<void *> ptrs;
	template <class T> int alloc(T **p, size_t count) {
		void *q = nullptr;
		if (cudaMalloc(&q, std::max<size_t>(count * sizeof(T), 16)) != cudaSuccess) {
			cudaGetLastError();
			return BFS_ENOMEM;
		}
		ptrs.push_back(q);
		*p = (T *) q;
		return BFS_OK;
	}
	~DevTmp() {
		for (void *p : ptrs) cudaFree(p);
	}
};

}  // namespace

extern "C" int bfs_gen_rmat_device(const bfs_rmat_params *p, uint32_t *src, uint32_t *dst, uint64_t capacity) {
	if (!p || !src || !dst || p->num_vertices == 0 || capacity < p->num_edges) return BFS_EARG;
	if (p->a < 0 || p->b < 0 || p->c < 0 || p->a + p->b + p->c > 1.0 + 1e-12) return BFS_EARG;
	const uint32_t n = p->num_vertices;
	const uint64_t m = p->num_edges;
	const bool no_loops = p->flags & BFS_RMAT_NO_SELF_LOOPS;
	const bool dedup = p->flags & BFS_RMAT_DEDUP;
	if (n == 1 && no_loops && m > 0) return BFS_EARG;
	if (dedup && m > (uint64_t) n * (no_loops ? n - 1 : n)) return BFS_EARG;
	if (m > 0xFFFFFFFFull) return BFS_EUNSUPPORTED;  // candidate indices are kept in 32 bits
	if (m == 0) return BFS_OK;
	int dev = 0, sms = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
		return BFS_ENODEV;
	uint32_t scale = 0;
	while ((1ull << scale) < n) ++scale;
	const rmat::Thresholds t{rmat::to_threshold(p->a), rmat::to_threshold(p->a + p->b),
			rmat::to_threshold(p->a + p->b + p->c)};
	const uint64_t seed = rmat::mixed_seed(p->seed);
	DevTmp tmp;
	int st;
	// Table: at most m + m/4 + 4096 keys are ever inserted (a round draws at
	// most 5/4 of the edges still missing, + 4096); twice that many slots.
	Table tb{nullptr, nullptr, 0};
	if (dedup) {
		uint64_t slots = 1024;
		while (slots < 2 * (m + m / 4 + 4096)) slots <<= 1;
		tb.mask = slots - 1;
		if ((st = tmp.alloc(&tb.key, slots)) || (st = tmp.alloc(&tb.first, slots))) return st;
		k_fill_u64<<<sms * 8, 512>>>(tb.key, slots, kEmptyKey);
		if (cudaMemset(tb.first, 0xFF, slots * 4) != cudaSuccess) return BFS_ECUDA;
	}
	unsigned long long *key_of = nullptr;
	uint32_t *slot = nullptr, *keep = nullptr, *rank = nullptr, *scan_tmp = nullptr;
	int *d_err = nullptr;
	if ((st = tmp.alloc(&key_of, kMaxRound)) || (st = tmp.alloc(&slot, kMaxRound)) ||
			(st = tmp.alloc(&keep, kMaxRound)) || (st = tmp.alloc(&rank, (size_t) kMaxRound + 1)) ||
			(st = tmp.alloc(&scan_tmp, dbuild_scan_tmp_words(kMaxRound))) || (st = tmp.alloc(&d_err, 1)))
		return st;
	if (cudaMemset(d_err, 0, sizeof(int)) != cudaSuccess) return BFS_ECUDA;
	uint64_t kept = 0, c0 = 0;
	while (kept < m) {
		const uint64_t want = m - kept;
		const uint32_t count = (uint32_t) std::min<uint64_t>(kMaxRound, want + want / 4 + 4096);
		if (c0 + count > 0xFFFFFFFFull) return BFS_EUNSUPPORTED;
		k_rmat_draw<<<sms * 8, 256>>>(seed, c0, count, scale, n, t, no_loops, dedup, tb, key_of, slot, d_err);
		k_rmat_first<<<sms * 8, 256>>>(c0, count, dedup, tb, key_of, slot, keep);
		if ((st = dbuild_exclusive_scan(keep, count, scan_tmp, rank, nullptr))) return st;
		k_rmat_compact<<<sms * 8, 256>>>(count, key_of, keep, rank, kept, m, src, dst);
		uint32_t got = 0;
		int herr = 0;
		if (cudaMemcpy(&got, rank + count, 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
				cudaMemcpy(&herr, d_err, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
			return BFS_ECUDA;
		if (herr) return herr;
		kept += std::min<uint64_t>(got, m - kept);
		c0 += count;
	}
	if (p->flags & BFS_RMAT_PERMUTE) {
		std::vector<uint32_t> perm;
		rmat::permutation(seed, n, perm);
		uint32_t *d_perm = nullptr;
		if ((st = tmp.alloc(&d_perm, n))) return st;
		if (cudaMemcpy(d_perm, perm.data(), (size_t) n * 4, cudaMemcpyHostToDevice) != cudaSuccess) return BFS_ECUDA;
		k_rmat_relabel<<<sms * 8, 512>>>(m, d_perm, src, dst);
	}
	if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return BFS_ECUDA;
	return BFS_OK;
}
