// build_device.cu -- the graph layout built on the GPU from an edge list:
// CSR, the in-edge lists and the packed column-major segments, by histogram,
// exclusive-scan and scatter kernels.
//
// It replaces, for large in-memory graphs, the host passes of the loader (the
// bucketing that tools/csr_tiling and tools/column_major_tile do,
// tools/csr_tiling/page_rank.cpp:531-567, tools/column_major_tile/kcore.cpp:
// 378-415, and this library's packing).  The scatters use atomics, so the
// order of edges inside a CSR row, an in-edge list or a packed segment is not
// the files' order; no traversal result depends on that order (levels are
// distances; parents are checked as a BFS tree).
#include <algorithm>
#include <cstdint>

#include "../../include/bfs_gb300.h"
#include "build_device.h"
#include "device_common.cuh"

namespace bfsg {

namespace {

constexpr int kBThreads = 512;
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;  // per thread
constexpr uint32_t kScanTile = kScanThreads * kScanItems;

__global__ void k_degrees(const uint32_t *src, const uint32_t *dst, uint64_t m, uint32_t n, uint32_t *out_deg,
		uint32_t *in_deg, int *err) {
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
		const uint32_t u = src[i], v = dst[i];
		if (u >= n || v >= n) {
			atomicExch(err, BFS_EFORMAT);
			continue;
		}
		atomicAdd(out_deg + u, 1u);
		atomicAdd(in_deg + v, 1u);
	}
}

// Block-wide exclusive scan of kScanTile values, in place in shared memory
// (thread t holds items 4t..4t+3).
__device__ void block_exclusive_scan(uint32_t *vals) {
	__shared__ uint32_t warp_tot[kScanThreads / 32];
	uint32_t v[kScanItems], sum = 0;
#pragma unroll
	for (int k = 0; k < kScanItems; ++k) {
		v[k] = vals[threadIdx.x * kScanItems + k];
		sum += v[k];
	}
	const uint32_t incl = warp_incl_scan(sum);
	if (lane_id() == 31) warp_tot[warp_id()] = incl;
	__syncthreads();
	if (warp_id() == 0) {
		const uint32_t t = lane_id() < kScanThreads / 32 ? warp_tot[lane_id()] : 0u;
		const uint32_t ti = warp_incl_scan(t);
		if (lane_id() < kScanThreads / 32) warp_tot[lane_id()] = ti - t;  // exclusive
	}
	__syncthreads();
	uint32_t run = warp_tot[warp_id()] + incl - sum;
#pragma unroll
	for (int k = 0; k < kScanItems; ++k) {
		vals[threadIdx.x * kScanItems + k] = run;
		run += v[k];
	}
	__syncthreads();
}

// Phase 1: the total of each tile.
__global__ void __launch_bounds__(kScanThreads) k_tile_sums(const uint32_t *in, uint32_t n, uint32_t *sums) {
	const uint64_t base = (uint64_t) blockIdx.x * kScanTile;
	uint32_t s = 0;
	for (uint32_t k = threadIdx.x; k < kScanTile; k += kScanThreads)
		if (base + k < n) s += in[base + k];
	s = warp_sum(s);
	__shared__ uint32_t ws[kScanThreads / 32];
	if (lane_id() == 0) ws[warp_id()] = s;
	__syncthreads();
	if (threadIdx.x == 0) {
		uint32_t t = 0;
		for (int w = 0; w < kScanThreads / 32; ++w) t += ws[w];
		sums[blockIdx.x] = t;
	}
}

// Phase 2 (one CTA): exclusive scan of the tile sums, in place; total at [tiles].
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(uint32_t *sums, uint32_t tiles) {
	__shared__ uint32_t buf[kScanTile];
	uint32_t carry = 0;
	for (uint32_t base = 0; base < tiles; base += kScanTile) {
		for (uint32_t k = threadIdx.x; k < kScanTile; k += kScanThreads) buf[k] = base + k < tiles ? sums[base + k] : 0u;
		__syncthreads();
		uint32_t last = buf[kScanTile - 1];
		__syncthreads();
		block_exclusive_scan(buf);
		for (uint32_t k = threadIdx.x; k < kScanTile; k += kScanThreads)
			if (base + k < tiles) sums[base + k] = buf[k] + carry;
		const uint32_t tile_total = buf[kScanTile - 1] + last;
		__syncthreads();
		carry += tile_total;
	}
	if (threadIdx.x == 0) sums[tiles] = carry;
}

// Phase 3: each tile's exclusive scan plus its offset; out[n] = total.
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const uint32_t *in, uint32_t n, const uint32_t *sums,
		uint32_t tiles, uint32_t *out) {
	__shared__ uint32_t buf[kScanTile];
	const uint64_t base = (uint64_t) blockIdx.x * kScanTile;
	for (uint32_t k = threadIdx.x; k < kScanTile; k += kScanThreads) buf[k] = base + k < n ? in[base + k] : 0u;
	__syncthreads();
	block_exclusive_scan(buf);
	const uint32_t off = sums[blockIdx.x];
	for (uint32_t k = threadIdx.x; k < kScanTile; k += kScanThreads)
		if (base + k < n) out[base + k] = buf[k] + off;
	if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = sums[tiles];
}

// out[pos] = val[i] with pos the next free slot of key[i]'s bucket.
__global__ void k_scatter(const uint32_t *key, const uint32_t *val, uint64_t m, uint32_t *cursor, uint32_t *out) {
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride)
		out[atomicAdd(cursor + key[i], 1u)] = val[i];
}

constexpr uint32_t kColHistSmem = 12288;  // tile columns counted in shared memory

// In-edges per tile column (a per-CTA shared histogram when the columns fit:
// every edge hits one of few counters) and the has-in-edge bitmap.
__global__ void k_col_hist(const uint32_t *dst, uint64_t m, uint32_t w, uint32_t side, uint32_t *col_edges,
		uint32_t *hasin) {
	__shared__ uint32_t hist[kColHistSmem];
	const bool local = side <= kColHistSmem;
	if (local)
		for (uint32_t c = threadIdx.x; c < side; c += blockDim.x) hist[c] = 0;
	__syncthreads();
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
		const uint32_t v = dst[i];
		if (local) atomicAdd(hist + v / w, 1u);
		else atomicAdd(col_edges + v / w, 1u);
		const uint32_t bit = 1u << (v & 31);
		if (!(ld_cg(hasin + (v >> 5)) & bit)) atomicOr(hasin + (v >> 5), bit);
	}
	__syncthreads();
	if (local)
		for (uint32_t c = threadIdx.x; c < side; c += blockDim.x)
			if (hist[c]) atomicAdd(col_edges + c, hist[c]);
}

__device__ __forceinline__ uint32_t seg_of(uint32_t u, uint32_t v, const DeviceBuildShape &sh, const uint32_t *group_of) {
	return group_of[v / sh.w] * sh.stripes + u / sh.w / sh.s;
}

__global__ void k_seg_hist(const uint32_t *src, const uint32_t *dst, uint64_t m, DeviceBuildShape sh,
		const uint32_t *group_of, uint32_t *seg_count) {
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride)
		atomicAdd(seg_count + seg_of(src[i], dst[i], sh, group_of), 1u);
}

// Packs u->v into its segment (the word layout of pack_tiles).
__global__ void k_seg_fill(const uint32_t *src, const uint32_t *dst, uint64_t m, DeviceBuildShape sh,
		const uint32_t *group_of, const uint32_t *group_col, uint32_t *cursor, uint32_t *words) {
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	const uint32_t cshift = sh.vbits, ushift = sh.vbits + sh.cbits;
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
		const uint32_t u = src[i], v = dst[i];
		const uint32_t k = u / sh.w / sh.s, c = v / sh.w, gi = group_of[c];
		const uint32_t word = (v - c * sh.w) | ((c - group_col[gi]) << cshift) | ((u - k * sh.s * sh.w) << ushift);
		words[atomicAdd(cursor + gi * sh.stripes + k, 1u)] = word;
	}
}

// Padding words after every segment's edges, up to the next segment.
__global__ void k_seg_pad(const uint32_t *seg_off, const uint32_t *seg_count, uint64_t nseg, uint32_t stripes,
		const uint32_t *pad_word, uint32_t *words) {
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	for (uint64_t j = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; j < nseg; j += stride) {
		const uint32_t pw = pad_word[j / stripes];
		for (uint32_t x = seg_off[j] + seg_count[j]; x < seg_off[j + 1]; ++x) words[x] = pw;
	}
}

int grid_for(uint64_t work, int num_sms) {
	const uint64_t g = (work + kBThreads - 1) / kBThreads;
	return (int) std::max<uint64_t>(1, std::min<uint64_t>(g, (uint64_t) num_sms * 8));
}

} // namespace

int dbuild_degrees(const uint32_t *src, const uint32_t *dst, uint64_t m, uint32_t n, uint32_t *out_deg,
		uint32_t *in_deg, int *err, int num_sms, cudaStream_t st) {
	k_degrees<<<grid_for(m, num_sms), kBThreads, 0, st>>>(src, dst, m, n, out_deg, in_deg, err);
	return cudaGetLastError() == cudaSuccess ? BFS_OK : BFS_ECUDA;
}

uint32_t dbuild_scan_tmp_words(uint32_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

int dbuild_exclusive_scan(const uint32_t *in, uint32_t n, uint32_t *tmp, uint32_t *out, cudaStream_t st) {
	const uint32_t tiles = dbuild_scan_tmp_words(n) - 1;
	if (tiles == 0) return cudaMemsetAsync(out, 0, sizeof(uint32_t), st) == cudaSuccess ? BFS_OK : BFS_ECUDA;
	k_tile_sums<<<tiles, kScanThreads, 0, st>>>(in, n, tmp);
	k_scan_sums<<<1, kScanThreads, 0, st>>>(tmp, tiles);
	k_scan_tiles<<<tiles, kScanThreads, 0, st>>>(in, n, tmp, tiles, out);
	return cudaGetLastError() == cudaSuccess ? BFS_OK : BFS_ECUDA;
}

int dbuild_scatter(const uint32_t *key, const uint32_t *val, uint64_t m, uint32_t *cursor, uint32_t *out, int num_sms,
		cudaStream_t st) {
	k_scatter<<<grid_for(m, num_sms), kBThreads, 0, st>>>(key, val, m, cursor, out);
	return cudaGetLastError() == cudaSuccess ? BFS_OK : BFS_ECUDA;
}

int dbuild_col_hist(const uint32_t *dst, uint64_t m, uint32_t w, uint32_t side, uint32_t *col_edges, uint32_t *hasin,
		int num_sms, cudaStream_t st) {
	k_col_hist<<<grid_for(m, num_sms), kBThreads, 0, st>>>(dst, m, w, side, col_edges, hasin);
	return cudaGetLastError() == cudaSuccess ? BFS_OK : BFS_ECUDA;
}

int dbuild_seg_hist(const uint32_t *src, const uint32_t *dst, uint64_t m, const DeviceBuildShape &sh,
		const uint32_t *group_of, uint32_t *seg_count, int num_sms, cudaStream_t st) {
	k_seg_hist<<<grid_for(m, num_sms), kBThreads, 0, st>>>(src, dst, m, sh, group_of, seg_count);
	return cudaGetLastError() == cudaSuccess ? BFS_OK : BFS_ECUDA;
}

int dbuild_seg_fill(const uint32_t *src, const uint32_t *dst, uint64_t m, const DeviceBuildShape &sh,
		const uint32_t *group_of, const uint32_t *group_col, uint32_t *cursor, uint32_t *words, int num_sms,
		cudaStream_t st) {
	k_seg_fill<<<grid_for(m, num_sms), kBThreads, 0, st>>>(src, dst, m, sh, group_of, group_col, cursor, words);
	return cudaGetLastError() == cudaSuccess ? BFS_OK : BFS_ECUDA;
}

int dbuild_seg_pad(const uint32_t *seg_off, const uint32_t *seg_count, uint64_t nseg, uint32_t stripes,
		const uint32_t *pad_word, uint32_t *words, int num_sms, cudaStream_t st) {
	k_seg_pad<<<grid_for(nseg, num_sms), kBThreads, 0, st>>>(seg_off, seg_count, nseg, stripes, pad_word, words);
	return cudaGetLastError() == cudaSuccess ? BFS_OK : BFS_ECUDA;
}

} // namespace bfsg
