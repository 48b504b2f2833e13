// bc.cu -- betweenness-centrality dependencies of one source, on the device.
//
// The reference's BC() (apps/betweennessCentrality_simd/bc.cpp:1717-2097)
// runs a forward BFS that adds path counts along every edge into a newly
// reached vertex (BFS_kernel_sparse :572-775, bfs_kernel_dense :1083-1162),
// keeps every level's frontier, then walks the frontiers backwards adding
// 1/paths to each vertex and pushing its sum to unvisited in-neighbours over
// the reverse graph (:1987-2030), and finally turns the sums into
// dependencies (:2032-2061).
//
// Here the levels come from the single-source traversal (k_bfs_persistent),
// and one cooperative launch does the rest with pulls instead of pushes, so
// that no atomics touch the values and every sum has a fixed order:
//   1. level sort: reached vertices are ordered by (level, class), with the
//      vertices whose in- or out-degree exceeds kBcBig first in each level.
//      Each warp owns a range of 32*q vertices and counts / places them with
//      __match_any_sync, so the order is deterministic.
//   2. path counts, level by level: sigma(v) = sum of sigma(u) over in-edges
//      u -> v with level(u) = level(v) - 1 (unsigned, wraps like the
//      reference's unsigned adds).
//   3. dependency sums, deepest level first: D(v) = 1/sigma(v) + sum of D(w)
//      over out-edges v -> w with level(w) = level(v) + 1; the output is
//      (D - 1/sigma) / (1/sigma), 0 where sigma is 0 -- the reference's float
//      formulas, with its signed int -> float conversion of the counts.
// Per level, the edge lists of big vertices are cut into kBcChunk-edge chunks
// that CTAs all over the grid sum (partials added in chunk order after a grid
// barrier), medium vertices are summed by half-warps, and small ones by warps
// that take 32 vertices and walk their concatenated edge lists 32 edges at a
// time (owner by a binary search over the warp's degree prefix, segmented
// shuffle scan per 32 edges).
#include "bc.h"

#include <algorithm>
#include <type_traits>

#include "../../include/bfs_gb300.h"
#include "device_common.cuh"

namespace bfsg {
namespace {

constexpr int kBcThreads = 512;
constexpr int kBcWarps = kBcThreads / 32;
constexpr int kBcUnroll = 4;

struct BcShared {
	float f[kBcWarps];
	uint32_t u[kBcWarps];
	unsigned long long e[kBcWarps];
	uint32_t scan[kBcWarps];
	uint32_t total;
	uint32_t chunk_beg, chunk_end;
	uint32_t cpre[kBcSmemBig + 1];   // chunk prefix of the level's big vertices
};
__device__ __shared__ BcShared bsh;

template <class T> __device__ __forceinline__ T *bsh_slot();
template <> __device__ __forceinline__ float *bsh_slot<float>() { return bsh.f; }
template <> __device__ __forceinline__ uint32_t *bsh_slot<uint32_t>() { return bsh.u; }
template <> __device__ __forceinline__ unsigned long long *bsh_slot<unsigned long long>() { return bsh.e; }

// CTA-wide sum with a fixed association (all threads call; warp 0 gets it).
template <class T> __device__ __forceinline__ T block_sum(T x) {
	T *slot = bsh_slot<T>();
	x = warp_sum(x);
	if (lane_id() == 0) slot[warp_id()] = x;
	__syncthreads();
	T t = T(0);
	if (warp_id() == 0) {
		t = lane_id() < (unsigned) kBcWarps ? slot[lane_id()] : T(0);
		t = warp_sum(t);
	}
	__syncthreads();
	return t;
}

// CTA-wide exclusive scan; *total gets the CTA's sum (all threads call).
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t x, uint32_t *total) {
	const unsigned lane = lane_id(), wid = warp_id();
	const uint32_t incl = warp_incl_scan(x);
	if (lane == 31) bsh.scan[wid] = incl;
	__syncthreads();
	if (wid == 0) {
		const uint32_t w = lane < (unsigned) kBcWarps ? bsh.scan[lane] : 0u;
		const uint32_t wi = warp_incl_scan(w);
		if (lane < (unsigned) kBcWarps) bsh.scan[lane] = wi - w;
		if (lane == 31) bsh.total = wi;
	}
	__syncthreads();
	const uint32_t r = incl - x + bsh.scan[wid];
	*total = bsh.total;
	__syncthreads();
	return r;
}

// Sort key of a vertex: kBcClasses*level + class by the larger of its in- and
// out-degree d (0: d > 1024; 1..5: d in (512, 1024], (256, 512], (128, 256],
// (64, 128], (32, 64]; 6: d <= 32); -1 for unreached and out-of-range ids.
__device__ __forceinline__ int vertex_key(const BcArgs &a, uint64_t v, uint32_t depth, int *bad) {
	if (v >= a.n) return -1;
	const int lv = a.level[v];
	if (lv < 0) return -1;
	if ((uint32_t) lv > depth) { *bad = 1; return -1; }
	const uint32_t od = a.row_off[v + 1] - a.row_off[v];
	const uint32_t id = a.in_off[v + 1] - a.in_off[v];
	const uint32_t dmax = od > id ? od : id;
	int cls = (int) kBcClasses - 1;
	if (dmax > kBcBig) cls = 0;
	else if (dmax > kBcMedium) cls = 1 + (31 - __clz(kBcBig - 1)) - (31 - __clz(dmax - 1));
	return (int) kBcClasses * lv + cls;
}

template <bool kFwd> struct Dir {
	using T = typename std::conditional<kFwd, uint32_t, float>::type;
	static __device__ __forceinline__ uint32_t bits(T x);
	static __device__ __forceinline__ const uint32_t *off(const BcArgs &a) { return kFwd ? a.in_off : a.row_off; }
	static __device__ __forceinline__ const uint32_t *adj(const BcArgs &a) { return kFwd ? a.in_src : a.col; }
	static __device__ __forceinline__ T value(uint32_t bits);
};
template <> __device__ __forceinline__ uint32_t Dir<true>::value(uint32_t bits) { return bits; }
template <> __device__ __forceinline__ float Dir<false>::value(uint32_t bits) { return __uint_as_float(bits); }
template <> __device__ __forceinline__ uint32_t Dir<true>::bits(uint32_t x) { return x; }
template <> __device__ __forceinline__ uint32_t Dir<false>::bits(float x) { return __float_as_uint(x); }

// {level, value} of a neighbour in one 8-byte load (written earlier in this launch: via L2)
__device__ __forceinline__ uint2 ld_lvx(const uint2 *p) { return __ldcg(p); }

// Level tags and value bits of the neighbours nb[] (0xFFFFFFFF: none): with
// use8 the byte level first and the value only where it matches `target`,
// else {level, value} in one 8-byte load.
template <int U>
__device__ __forceinline__ void gather_tags(const BcArgs &a, const uint32_t (&nb)[U], uint2 (&lx)[U], bool use8,
		int target) {
#pragma unroll
	for (int k = 0; k < U; ++k) {
		if (nb[k] == 0xFFFFFFFFu) lx[k] = make_uint2(0xFFFFFFFEu, 0u);
		else if (use8) lx[k] = make_uint2((uint32_t) ld_cg_u8(a.lv8 + nb[k]), 0u);
		else lx[k] = ld_lvx(a.lvx + nb[k]);
	}
	if (use8) {
#pragma unroll
		for (int k = 0; k < U; ++k)
			if ((int) lx[k].x == target) lx[k].y = ld_cg(reinterpret_cast<const uint32_t *>(a.lvx + nb[k]) + 1);
	}
}

// Sum over the edges [beg, end) of one vertex by the whole CTA (result in warp 0).
template <bool kFwd>
__device__ __forceinline__ typename Dir<kFwd>::T cta_range_sum(const BcArgs &a, uint64_t beg, uint64_t end, int target,
		bool use8) {
	using T = typename Dir<kFwd>::T;
	const uint32_t *adj = Dir<kFwd>::adj(a);
	T s = T(0);
	for (uint64_t e = beg + threadIdx.x; e < end; e += (uint64_t) kBcThreads * kBcUnroll) {
		uint32_t nb[kBcUnroll];
		uint2 lx[kBcUnroll];
#pragma unroll
		for (int k = 0; k < kBcUnroll; ++k) {
			const uint64_t ee = e + (uint64_t) k * kBcThreads;
			nb[k] = ee < end ? __ldg(adj + ee) : 0xFFFFFFFFu;
		}
		gather_tags(a, nb, lx, use8, target);
#pragma unroll
		for (int k = 0; k < kBcUnroll; ++k)
			if ((int) lx[k].x == target) s += Dir<kFwd>::value(lx[k].y);
	}
	return block_sum(s);
}


// Big vertices order[bb .. bb+nbig) (nbig <= kBcSmemBig) cut into chunks of
// kBcChunk edges: every CTA builds the same chunk prefix in shared memory,
// then CTA c sums chunks c, c + grid, ... into partial[] (value bits).
template <bool kFwd>
__device__ __forceinline__ void big_chunks(const BcArgs &a, uint32_t bb, uint32_t nbig, int target, bool use8) {
	const uint32_t *off = Dir<kFwd>::off(a);
	uint32_t carry = 0;
	for (uint32_t t0 = 0; t0 < nbig; t0 += kBcThreads) {
		const uint32_t i = t0 + threadIdx.x;
		uint32_t c = 0;
		if (i < nbig) {
			const uint32_t v = ld_cg(a.order + bb + i);
			c = (off[v + 1] - off[v] + kBcChunk - 1) / kBcChunk;
		}
		uint32_t tot;
		const uint32_t ex = block_excl_scan(c, &tot);
		if (i < nbig) bsh.cpre[i] = carry + ex;
		carry += tot;
	}
	if (threadIdx.x == 0) bsh.cpre[nbig] = carry;
	__syncthreads();
	for (uint32_t j = blockIdx.x; j < carry; j += gridDim.x) {
		if (threadIdx.x == 0) {
			// the largest i with cpre[i] <= j (cpre[nbig] = carry > j)
			uint32_t lo = 0, hi = nbig;
			while (lo < hi) {
				const uint32_t mid = (lo + hi + 1) / 2;
				if (bsh.cpre[mid] <= j) lo = mid;
				else hi = mid - 1;
			}
			const uint32_t v = ld_cg(a.order + bb + lo);
			const uint32_t beg = off[v] + (j - bsh.cpre[lo]) * kBcChunk;
			const uint32_t end = off[v + 1];
			bsh.chunk_beg = beg;
			bsh.chunk_end = end - beg > kBcChunk ? beg + kBcChunk : end;
		}
		__syncthreads();
		const uint32_t beg = bsh.chunk_beg, end = bsh.chunk_end;
		const typename Dir<kFwd>::T s = cta_range_sum<kFwd>(a, beg, end, target, use8);
		if (threadIdx.x == 0) a.partial[j] = Dir<kFwd>::bits(s);
	}
}

// The same for a level with more than kBcSmemBig big vertices: the chunk
// prefix is scanned grid-wide into a.cpre (two grid barriers), then CTA c sums
// the contiguous chunk range [c*per, (c+1)*per).  Returns false when a barrier
// gave up.
template <bool kFwd>
__device__ __forceinline__ bool big_chunks_global(const BcArgs &a, uint32_t bb, uint32_t nbig, int target, bool use8) {
	const uint32_t *off = Dir<kFwd>::off(a);
	BcControl *ctl = a.ctl;
	const uint32_t L = (nbig + gridDim.x - 1) / gridDim.x;
	const uint32_t lo = blockIdx.x * L < nbig ? blockIdx.x * L : nbig;
	const uint32_t hi = lo + L < nbig ? lo + L : nbig;
	{
		uint32_t s = 0;
		for (uint32_t i = lo + threadIdx.x; i < hi; i += kBcThreads) {
			const uint32_t v = ld_cg(a.order + bb + i);
			s += (off[v + 1] - off[v] + kBcChunk - 1) / kBcChunk;
		}
		s = block_sum(s);
		if (threadIdx.x == 0) ctl->blk[blockIdx.x] = s;
	}
	if (!grid_barrier(ctl->bar, &ctl->err)) return false;
	uint32_t base = 0, total = 0;
	for (uint32_t c = threadIdx.x; c < gridDim.x; c += kBcThreads) {
		const uint32_t x = ld_cg(ctl->blk + c);
		if (c < blockIdx.x) base += x;
		total += x;
	}
	base = block_sum(base);
	total = block_sum(total);
	if (threadIdx.x == 0) {
		bsh.chunk_beg = base;
		bsh.chunk_end = total;
	}
	__syncthreads();
	base = bsh.chunk_beg;
	total = bsh.chunk_end;
	__syncthreads();
	for (uint32_t t0 = lo; t0 < hi; t0 += kBcThreads) {
		const uint32_t i = t0 + threadIdx.x;
		uint32_t c = 0;
		if (i < hi) {
			const uint32_t v = ld_cg(a.order + bb + i);
			c = (off[v + 1] - off[v] + kBcChunk - 1) / kBcChunk;
		}
		uint32_t tot;
		const uint32_t ex = block_excl_scan(c, &tot);
		if (i < hi) a.cpre[i] = base + ex;
		base += tot;
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) a.cpre[nbig] = total;
	if (!grid_barrier(ctl->bar, &ctl->err)) return false;
	const uint32_t per = (total + gridDim.x - 1) / gridDim.x;
	const uint32_t j0 = blockIdx.x * per < total ? blockIdx.x * per : total;
	const uint32_t j1 = j0 + per < total ? j0 + per : total;
	uint32_t owner = 0;
	if (j0 < j1 && threadIdx.x == 0) {
		// the largest i with cpre[i] <= j0 (cpre[nbig] = total > j0)
		uint32_t l = 0, h = nbig;
		while (l < h) {
			const uint32_t mid = (l + h + 1) / 2;
			if (ld_cg(a.cpre + mid) <= j0) l = mid;
			else h = mid - 1;
		}
		owner = l;
	}
	for (uint32_t j = j0; j < j1; ++j) {
		if (threadIdx.x == 0) {
			while (ld_cg(a.cpre + owner + 1) <= j) ++owner;
			const uint32_t v = ld_cg(a.order + bb + owner);
			const uint32_t beg = off[v] + (j - ld_cg(a.cpre + owner)) * kBcChunk;
			const uint32_t end = off[v + 1];
			bsh.chunk_beg = beg;
			bsh.chunk_end = end - beg > kBcChunk ? beg + kBcChunk : end;
		}
		__syncthreads();
		const uint32_t beg = bsh.chunk_beg, end = bsh.chunk_end;
		const typename Dir<kFwd>::T s = cta_range_sum<kFwd>(a, beg, end, target, use8);
		if (threadIdx.x == 0) a.partial[j] = Dir<kFwd>::bits(s);
	}
	return true;
}

// Sum of big vertex i's chunk partials in chunk order, by one warp (all lanes
// get it); the chunk prefix is in shared memory (global: in a.cpre).
template <bool kFwd>
__device__ __forceinline__ typename Dir<kFwd>::T big_finish_sum(const BcArgs &a, uint32_t i, bool global) {
	using T = typename Dir<kFwd>::T;
	const uint32_t c0 = global ? ld_cg(a.cpre + i) : bsh.cpre[i];
	const uint32_t c1 = global ? ld_cg(a.cpre + i + 1) : bsh.cpre[i + 1];
	T s = T(0);
	for (uint32_t j = c0 + lane_id(); j < c1; j += 32) s += Dir<kFwd>::value(ld_cg(a.partial + j));
	return warp_sum(s);
}

// Sum over the edge list of one vertex by a half-warp (16 lanes); v_ok false
// gives 0.  Both halves call it together (the reduction shuffles the warp).
template <bool kFwd>
__device__ __forceinline__ typename Dir<kFwd>::T half_vertex_sum(const BcArgs &a, uint32_t v, bool v_ok, int target,
		bool use8) {
	using T = typename Dir<kFwd>::T;
	const uint32_t *adj = Dir<kFwd>::adj(a);
	const uint32_t hl = lane_id() & 15u;
	uint32_t beg = 0, end = 0;
	if (v_ok) {
		beg = Dir<kFwd>::off(a)[v];
		end = Dir<kFwd>::off(a)[v + 1];
	}
	T s = T(0);
	for (uint32_t e = beg + hl; e < end; e += 16u * kBcUnroll) {
		uint32_t nb[kBcUnroll];
		uint2 lx[kBcUnroll];
#pragma unroll
		for (int k = 0; k < kBcUnroll; ++k) {
			const uint32_t ee = e + (uint32_t) k * 16u;
			nb[k] = ee < end ? __ldg(adj + ee) : 0xFFFFFFFFu;
		}
		gather_tags(a, nb, lx, use8, target);
#pragma unroll
		for (int k = 0; k < kBcUnroll; ++k)
			if ((int) lx[k].x == target) s += Dir<kFwd>::value(lx[k].y);
	}
#pragma unroll
	for (int d = 8; d > 0; d >>= 1) s += __shfl_xor_sync(kFull, s, d);
	return s;
}

// Sums of the edge lists of 32 vertices order[first .. min(first+32, end))
// by one warp; lane i gets vertex i's sum (0 for lanes past `end`).
template <bool kFwd>
__device__ __forceinline__ typename Dir<kFwd>::T warp_group_sum(const BcArgs &a, uint32_t v, bool valid, int target,
		bool skip, bool use8, unsigned long long *edges) {
	using T = typename Dir<kFwd>::T;
	const unsigned lane = lane_id();
	uint32_t beg = 0, deg = 0;
	if (valid) {
		beg = Dir<kFwd>::off(a)[v];
		deg = Dir<kFwd>::off(a)[v + 1] - beg;
	}
	if (skip) deg = 0;
	*edges += deg;
	const uint32_t incl = warp_incl_scan(deg);
	const uint32_t excl = incl - deg;
	const uint32_t total = __shfl_sync(kFull, incl, 31);
	const uint32_t *adj = Dir<kFwd>::adj(a);
	T acc = T(0);
	for (uint32_t f0 = 0; f0 < total; f0 += 32u * kBcUnroll) {
		uint32_t nb[kBcUnroll], own[kBcUnroll];
		uint2 lx[kBcUnroll];
		T val[kBcUnroll];
#pragma unroll
		for (int k = 0; k < kBcUnroll; ++k) {
			const uint32_t f = f0 + (uint32_t) k * 32u + lane;
			// owner = number of lanes whose inclusive prefix is <= f
			uint32_t o = 0;
#pragma unroll
			for (uint32_t step = 16; step > 0; step >>= 1) {
				const uint32_t x = __shfl_sync(kFull, incl, o + step - 1);
				if (x <= f) o += step;
			}
			const uint32_t ob = __shfl_sync(kFull, beg, o);
			const uint32_t oe = __shfl_sync(kFull, excl, o);
			const bool on = f < total;
			own[k] = on ? o : 32u;
			nb[k] = on ? __ldg(adj + ob + (f - oe)) : 0xFFFFFFFFu;
		}
		gather_tags(a, nb, lx, use8, target);
#pragma unroll
		for (int k = 0; k < kBcUnroll; ++k) val[k] = (int) lx[k].x == target ? Dir<kFwd>::value(lx[k].y) : T(0);
#pragma unroll
		for (int k = 0; k < kBcUnroll; ++k) {
			T x = val[k];
			const uint32_t o = own[k];
#pragma unroll
			for (uint32_t dd = 1; dd < 32; dd <<= 1) {
				const T y = __shfl_up_sync(kFull, x, dd);
				const uint32_t oo = __shfl_up_sync(kFull, o, dd);
				if (lane >= dd && oo == o) x += y;
			}
			// the last lane of this vertex's run in these 32 edges holds its sum
			const uint32_t base = f0 + (uint32_t) k * 32u;
			const bool mine = deg > 0 && incl > base && excl < base + 32u;
			const uint32_t src = mine ? min(incl, base + 32u) - 1u - base : 0u;
			const T got = __shfl_sync(kFull, x, src);
			if (mine) acc += got;
		}
	}
	return acc;
}

__device__ __forceinline__ void finish_dependency(const BcArgs &a, uint32_t v, float sum) {
	const uint32_t sg = ld_cg(a.sigma + v);
	const float inv = sg ? 1.0f / (float) (int) sg : 0.0f;
	const float dv = sum + inv;
	a.lvx[v].y = __float_as_uint(dv);
	const float del = inv != 0.0f ? (dv - inv) / inv : 0.0f;
	a.delta[v] = del;
	if (a.acc && v != a.source) a.acc[v] += del;
}

__global__ void __launch_bounds__(kBcThreads, 2) k_bc(BcArgs a) {
	BcControl *ctl = a.ctl;
	const unsigned lane = lane_id();
	const uint32_t gw = blockIdx.x * kBcWarps + warp_id();
	const uint32_t tw = gridDim.x * kBcWarps;
	if (blockIdx.x == 0 && threadIdx.x == 0) ctl->t[0] = global_timer_ns();
	// the traversal's outcome decides for every CTA alike
	const int bfs_st = *(const volatile int *) a.bfs_status;
	const uint32_t steps = *(const volatile uint32_t *) a.num_steps;
	if (bfs_st != 0 || steps == 0 || steps > kBcMaxLevels) {
		if (blockIdx.x == 0 && threadIdx.x == 0)
			ctl->err = bfs_st != 0 ? bfs_st : (steps == 0 ? BFS_ECUDA : BFS_EUNSUPPORTED);
		return;
	}
	const uint32_t depth = steps - 1;
	const bool use8 = a.byte_levels && depth <= 254;
	const uint32_t K = kBcClasses * steps;
	const uint64_t W32 = ((uint64_t) a.n + 31) / 32;
	uint64_t q = (K * W32 + kBcCntCap - 1) / kBcCntCap;
	if (q == 0) q = 1;
	uint64_t R = (W32 + q - 1) / q;
	while ((uint64_t) K * R > kBcCntCap) {
		++q;
		R = (W32 + q - 1) / q;
	}
	const uint64_t KR = (uint64_t) K * R;

	// ---- 1a. count (level key, range) and initialise the outputs ----------
	unsigned long long my_edges = 0;
	uint32_t my_reached = 0;
	int bad = 0;
	for (uint64_t r = gw; r < R; r += tw) {
		for (uint32_t k = lane; k < K; k += 32) a.cnt[(uint64_t) k * R + r] = 0;
		__syncwarp();
		const uint64_t v0 = r * 32 * q;
		for (uint64_t j = 0; j < q; ++j) {
			const uint64_t v = v0 + j * 32 + lane;
			const int key = vertex_key(a, v, depth, &bad);
			if (v < a.n) {
				a.sigma[v] = v == a.source ? 1u : 0u;
				a.delta[v] = 0.0f;
				const int lv = a.level[v];
				a.lvx[v] = make_uint2((uint32_t) lv, v == a.source ? 1u : 0u);
				a.lv8[v] = (uint8_t) (lv < 0 || lv > 254 ? 255 : lv);
			}
			if (key >= 0) {
				++my_reached;
				my_edges += a.row_off[v + 1] - a.row_off[v];
			}
			const unsigned mm = __match_any_sync(kFull, key);
			if (key >= 0 && lane == (unsigned) (__ffs(mm) - 1)) a.cnt[(uint64_t) key * R + r] += __popc(mm);
			__syncwarp();
		}
	}
	{
		const unsigned long long e = block_sum(my_edges);
		const uint32_t rc = block_sum(my_reached);
		const uint32_t b = block_sum((uint32_t) bad);
		if (threadIdx.x == 0) {
			if (e) atomicAdd(&ctl->edges_reached, e);
			if (rc) atomicAdd(&ctl->reached, rc);
			if (b) atomicExch(&ctl->err, BFS_ECUDA);
		}
	}
	if (!grid_barrier(ctl->bar, &ctl->err)) return;

	// ---- 1b. exclusive scan of the counters (key-major) --------------------
	const uint64_t L = (KR + gridDim.x - 1) / gridDim.x;
	const uint64_t lo = (uint64_t) blockIdx.x * L < KR ? (uint64_t) blockIdx.x * L : KR;
	const uint64_t hi = lo + L < KR ? lo + L : KR;
	{
		uint32_t s = 0;
		for (uint64_t i = lo + threadIdx.x; i < hi; i += kBcThreads) s += a.cnt[i];
		s = block_sum(s);
		if (threadIdx.x == 0) ctl->blk[blockIdx.x] = s;
	}
	if (!grid_barrier(ctl->bar, &ctl->err)) return;
	{
		uint32_t base = 0;
		for (uint32_t c = threadIdx.x; c < blockIdx.x; c += kBcThreads) base += ld_cg(ctl->blk + c);
		base = block_sum(base);
		if (warp_id() == 0 && lane == 0) bsh.u[0] = base;
		__syncthreads();
		base = bsh.u[0];
		__syncthreads();
		for (uint64_t t0 = lo; t0 < hi; t0 += kBcThreads) {
			const uint64_t i = t0 + threadIdx.x;
			const uint32_t x = i < hi ? a.cnt[i] : 0u;
			uint32_t tot;
			const uint32_t ex = block_excl_scan(x, &tot) + base;
			if (i < hi) {
				a.cnt[i] = ex;
				if (i % R == 0) a.kstart[i / R] = ex;
			}
			base += tot;
		}
		if (blockIdx.x == 0 && threadIdx.x == 0) a.kstart[K] = ld_cg(&ctl->reached);
	}
	if (!grid_barrier(ctl->bar, &ctl->err)) return;

	// ---- 1c. place the vertices ------------------------------------------
	for (uint64_t r = gw; r < R; r += tw) {
		const uint64_t v0 = r * 32 * q;
		for (uint64_t j = 0; j < q; ++j) {
			const uint64_t v = v0 + j * 32 + lane;
			int dummy = 0;
			const int key = vertex_key(a, v, depth, &dummy);
			const unsigned mm = __match_any_sync(kFull, key);
			const unsigned leader = (unsigned) (__ffs(mm) - 1);
			uint32_t base = 0;
			if (key >= 0 && lane == leader) base = ld_cg(a.cnt + (uint64_t) key * R + r);
			base = __shfl_sync(kFull, base, leader);
			if (key >= 0) {
				a.order[base + __popc(mm & lanemask_lt())] = (uint32_t) v;
				if (lane == leader) a.cnt[(uint64_t) key * R + r] = base + __popc(mm);
			}
			__syncwarp();
		}
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) ctl->t[1] = global_timer_ns();
	if (!grid_barrier(ctl->bar, &ctl->err)) return;

	// ---- 2. path counts, level by level ----------------------------------
	unsigned long long e_fwd = 0, e_rev = 0;
	for (uint32_t d = 1; d <= depth; ++d) {
		const uint32_t bb = ld_cg(a.kstart + kBcClasses * d), be = ld_cg(a.kstart + kBcClasses * d + 1);
		const uint32_t me = ld_cg(a.kstart + kBcClasses * d + kBcClasses - 1);
		const uint32_t se = ld_cg(a.kstart + kBcClasses * d + kBcClasses);
		const uint32_t nbig = be - bb;
		if (nbig > 0) {
			const bool global = nbig > kBcSmemBig;
			if (global) {
				if (!big_chunks_global<true>(a, bb, nbig, (int) d - 1, use8)) return;
			} else {
				big_chunks<true>(a, bb, nbig, (int) d - 1, use8);
			}
			if (!grid_barrier(ctl->bar, &ctl->err)) return;
			for (uint32_t i = gw; i < nbig; i += tw) {
				const uint32_t v = ld_cg(a.order + bb + i);
				const uint32_t s = big_finish_sum<true>(a, i, global);
				if (lane == 0) {
					a.sigma[v] = s;
					a.lvx[v].y = s;
					e_fwd += a.in_off[v + 1] - a.in_off[v];
				}
			}
		}
		for (uint32_t i0 = be + 2 * (tw - 1 - gw); i0 < me; i0 += 2 * tw) {
			const uint32_t i = i0 + (lane >> 4);
			const bool ok = i < me;
			const uint32_t v = ok ? ld_cg(a.order + i) : 0u;
			const uint32_t s = half_vertex_sum<true>(a, v, ok, (int) d - 1, use8);
			if (ok && (lane & 15u) == 0) {
				a.sigma[v] = s;
				a.lvx[v].y = s;
				e_fwd += a.in_off[v + 1] - a.in_off[v];
			}
		}
		const uint32_t groups = (se - me + 31) / 32;
		for (uint32_t grp = gw; grp < groups; grp += tw) {
			const uint32_t idx = me + grp * 32 + lane;
			const bool valid = idx < se;
			const uint32_t v = valid ? ld_cg(a.order + idx) : 0u;
			const uint32_t s = warp_group_sum<true>(a, v, valid, (int) d - 1, false, use8, &e_fwd);
			if (valid) {
				a.sigma[v] = s;
				a.lvx[v].y = s;
			}
		}
		if (!grid_barrier(ctl->bar, &ctl->err)) return;
		if (blockIdx.x == 0 && threadIdx.x == 0 && d < kBcTraceLevels) ctl->t_fwd[d] = global_timer_ns();
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) ctl->t[2] = global_timer_ns();

	// ---- 3. dependency sums, deepest level first ---------------------------
	for (int d = (int) depth; d >= 0; --d) {
		const bool deepest = (uint32_t) d == depth;
		const uint32_t bb = ld_cg(a.kstart + kBcClasses * d), be = ld_cg(a.kstart + kBcClasses * d + 1);
		const uint32_t me = ld_cg(a.kstart + kBcClasses * d + kBcClasses - 1);
		const uint32_t se = ld_cg(a.kstart + kBcClasses * d + kBcClasses);
		const uint32_t nbig = be - bb;
		if (deepest) {
			for (uint32_t i = gw; i < nbig; i += tw)
				if (lane == 0) finish_dependency(a, ld_cg(a.order + bb + i), 0.0f);
		} else if (nbig > 0) {
			const bool global = nbig > kBcSmemBig;
			if (global) {
				if (!big_chunks_global<false>(a, bb, nbig, d + 1, use8)) return;
			} else {
				big_chunks<false>(a, bb, nbig, d + 1, use8);
			}
			if (!grid_barrier(ctl->bar, &ctl->err)) return;
			for (uint32_t i = gw; i < nbig; i += tw) {
				const uint32_t v = ld_cg(a.order + bb + i);
				const float s = big_finish_sum<false>(a, i, global);
				if (lane == 0) {
					finish_dependency(a, v, s);
					e_rev += a.row_off[v + 1] - a.row_off[v];
				}
			}
		}
		for (uint32_t i0 = be + 2 * (tw - 1 - gw); i0 < me; i0 += 2 * tw) {
			const uint32_t i = i0 + (lane >> 4);
			const bool ok = i < me;
			const uint32_t v = ok ? ld_cg(a.order + i) : 0u;
			const float s = half_vertex_sum<false>(a, v, ok && !deepest, d + 1, use8);
			if (ok && (lane & 15u) == 0) {
				finish_dependency(a, v, s);
				if (!deepest) e_rev += a.row_off[v + 1] - a.row_off[v];
			}
		}
		const uint32_t groups = (se - me + 31) / 32;
		for (uint32_t grp = gw; grp < groups; grp += tw) {
			const uint32_t idx = me + grp * 32 + lane;
			const bool valid = idx < se;
			const uint32_t v = valid ? ld_cg(a.order + idx) : 0u;
			const float s = warp_group_sum<false>(a, v, valid, d + 1, deepest, use8, &e_rev);
			if (valid) finish_dependency(a, v, s);
		}
		if (d > 0 && !grid_barrier(ctl->bar, &ctl->err)) return;
		if (blockIdx.x == 0 && threadIdx.x == 0 && (uint32_t) d < kBcTraceLevels) {
			ctl->t_rev[d] = global_timer_ns();
			ctl->lv_vertices[d] = se - bb;
			ctl->lv_big[d] = be - bb;
			ctl->lv_medium[d] = me - be;
		}
	}
	{
		const unsigned long long ef = block_sum(e_fwd);
		const unsigned long long er = block_sum(e_rev);
		if (threadIdx.x == 0) {
			if (ef) atomicAdd(&ctl->edges_fwd, ef);
			if (er) atomicAdd(&ctl->edges_rev, er);
			ctl->depth = depth;
		}
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) ctl->t[3] = global_timer_ns();
}

} // namespace

int bc_launch(const BcArgs &a, int num_sms, cudaStream_t st, int *grid) {
	int per_sm = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bc, kBcThreads, 0) != cudaSuccess || per_sm < 1)
		return BFS_ECUDA;
	per_sm = std::min(per_sm, 2);
	const int g = std::min<int>(num_sms * per_sm, (int) kBcMaxGrid);
	if (grid) *grid = g;
	if (cudaMemsetAsync(a.ctl, 0, sizeof(BcControl), st) != cudaSuccess) return BFS_ECUDA;
	BcArgs aa = a;
	void *args[] = {&aa};
	if (cudaLaunchCooperativeKernel((const void *) k_bc, dim3(g), dim3(kBcThreads), args, 0, st) != cudaSuccess)
		return BFS_ECUDA;
	return BFS_OK;
}

} // namespace bfsg
