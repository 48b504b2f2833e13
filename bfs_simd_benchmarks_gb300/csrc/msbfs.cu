// msbfs.cu -- batched BFS: up to 4096 sources traversed together, bit-sliced.
//
// No counterpart in the reference, which runs one source per program run
// (apps/bfs_simd/bfs.cpp:1159); each source's levels equal what graph_prepare
// (apps/bfs_simd/bfs.cpp:753-963) computes for it.
//
// Layout (K = ceil(num_sources / 64) words, source i is bit i%64 of word i/64):
//   vis[v][K]          sources that have reached v
//   hist[p][v][K]      sources that reached v first at level base + p; the
//                      plane of level L is the frontier that level L expands
//   act[L&1][v]        bit k: word k of v's row in the plane of level L is
//                      non-zero (the frontier's vertex set and which rows to read)
//   queue[L&1]         the frontier's vertices: degree <= kMsBig from the
//                      front, higher degree from the back
// A level is expanded either
//   - push (top-down) while the frontier holds few edges: a warp takes a
//     frontier vertex, loads its K words once and ORs the non-zero ones into
//     every out-neighbour's next words (64-bit atomics); a high-degree vertex
//     has its edges spread over every warp of the grid; or
//   - pull (bottom-up) once it holds many: a warp owns a destination, gathers
//     the non-zero words of its frontier in-neighbours that the destination
//     still lacks and stops as soon as every source has reached it
//     (per-destination early exit); destinations with many in-edges are cut
//     into chunks that warps all over the grid gather and OR together.
// Everything -- clearing, seeding, all levels, the output and the edge count
// -- runs in one cooperative launch, levels separated by a bounded-spin grid
// barrier.  The output pass turns planes into uint8 levels [source][vertex]
// (255 = unreached) through a shared-memory transpose.  When a traversal is
// deeper than the planes allocated, the planes so far are written out, the
// current frontier plane becomes plane 0 and the traversal goes on; the later
// output passes merge into the bytes already written.
#include <algorithm>
#include <cstring>

#include "../../include/bfs_gb300.h"
#include "device_common.cuh"
#include "msbfs.h"

namespace bfsg {

constexpr int kMsThreads = 512;
constexpr int kMsWarps = kMsThreads / 32;
constexpr uint32_t kMsWq = 64;          // per-warp staged queue appends (pull)
constexpr uint32_t kMsBig = 1024;       // push: higher-degree vertices are spread over the grid
constexpr int kMsGather = 4;            // pull: frontier rows gathered per round
constexpr uint32_t kEmitWords = 8;      // output tile: 8 words (512 sources) ...
constexpr uint32_t kEmitRows = kEmitWords * 64;
constexpr uint32_t kEmitV = 64;         // ... x 64 vertices
constexpr uint32_t kEmitStride = 68;    // shared row stride in bytes (17 words: column writes spread over banks)

__device__ __forceinline__ uint64_t ld_cg64(const uint64_t *p) { return __ldcg((const unsigned long long *) p); }
__device__ __forceinline__ uint64_t shfl64(uint64_t x, int src) {
	return (uint64_t) __shfl_sync(kFull, (unsigned long long) x, src);
}
__device__ __forceinline__ uint32_t deg_of(const MsArgs &a, uint32_t v) {
	return __ldg(a.row_off + v + 1) - __ldg(a.row_off + v);
}

// Warp-aggregated append of the lanes with `small` / `big` set to the
// queue of the next level (small from the front, big from the back).
__device__ __forceinline__ void ms_append(const MsArgs &a, MsCounters *cn, uint32_t *qn, uint32_t v, bool small,
		bool big) {
	const unsigned ms = __ballot_sync(kFull, small);
	if (ms) {
		uint32_t base = 0;
		if (lane_id() == 0) base = atomicAdd(&cn->nact, (unsigned) __popc(ms));
		base = __shfl_sync(kFull, base, 0);
		if (small) qn[base + __popc(ms & lanemask_lt())] = v;
	}
	const unsigned mb = __ballot_sync(kFull, big);
	if (mb) {
		uint32_t base = 0;
		if (lane_id() == 0) base = atomicAdd(&cn->nbig, (unsigned) __popc(mb));
		base = __shfl_sync(kFull, base, 0);
		if (big) qn[a.n - 1 - (base + __popc(mb & lanemask_lt()))] = v;
	}
}

// Push: ORs u's non-zero frontier words into the next words of its out-edges
// [beg + first, end), taking 32 edges per warp step of `step`.  Warp-uniform.
__device__ __forceinline__ void ms_push_edges(const MsArgs &a, const uint64_t *cur, const uint64_t *actc,
		uint64_t *nxt, uint32_t u, uint32_t beg, uint32_t end, uint32_t first, uint32_t step) {
	const uint32_t K = a.K;
	const unsigned lane = lane_id();
	const uint64_t um = ld_cg64(actc + u);  // which of u's words are non-zero
	const uint32_t nz0 = (uint32_t) um, nz1 = (uint32_t) (um >> 32);
	const uint64_t w0 = (nz0 >> lane) & 1u ? ld_cg64(cur + (size_t) u * K + lane) : 0ull;
	const uint64_t w1 = (nz1 >> lane) & 1u ? ld_cg64(cur + (size_t) u * K + lane + 32) : 0ull;
	for (uint32_t e0 = beg + first; e0 < end; e0 += step) {
		const uint32_t e = e0 + lane;
		const bool ok = e < end;
		const uint32_t v = ok ? __ldg(a.col + e) : 0u;
		unsigned long long *dst = (unsigned long long *) (nxt + (size_t) v * K);
		for (uint32_t m = nz0; m; m &= m - 1) {
			const int k = __ffs(m) - 1;
			const uint64_t w = shfl64(w0, k);
			if (ok) atomicOr(dst + k, (unsigned long long) w);
		}
		for (uint32_t m = nz1; m; m &= m - 1) {
			const int k = __ffs(m) - 1;
			const uint64_t w = shfl64(w1, k);
			if (ok) atomicOr(dst + 32 + k, (unsigned long long) w);
		}
		if (ok && !ld_cg_u8(a.touched + v)) a.touched[v] = 1;
	}
}

__device__ void ms_push(const MsArgs &a, uint32_t lvl, const uint64_t *cur, uint64_t *nxt, uint32_t nq, uint32_t nb) {
	const uint32_t *q = a.queue[lvl & 1];
	const uint64_t *actc = a.act[lvl & 1];
	const uint32_t gwarp = blockIdx.x * kMsWarps + warp_id();
	const uint32_t nwarps = gridDim.x * kMsWarps;
	for (uint32_t i = gwarp; i < nq; i += nwarps) {
		const uint32_t u = ld_cg(q + i);
		ms_push_edges(a, cur, actc, nxt, u, __ldg(a.row_off + u), __ldg(a.row_off + u + 1), 0, 32);
	}
	for (uint32_t i = 0; i < nb; ++i) {
		const uint32_t u = ld_cg(q + a.n - 1 - i);
		ms_push_edges(a, cur, actc, nxt, u, __ldg(a.row_off + u), __ldg(a.row_off + u + 1), gwarp * 32, nwarps * 32);
	}
}

// The next-frontier mask of a row whose new words lanes hold (word l, l + 32).
__device__ __forceinline__ uint64_t row_mask(uint64_t n0, uint64_t n1) {
	return (uint64_t) __ballot_sync(kFull, n0 != 0ull) | ((uint64_t) __ballot_sync(kFull, n1 != 0ull) << 32);
}

// After a push level: the OR'ed words lose the bits already visited, the rest
// are new, go into vis and put v into the next frontier.  A warp takes 32
// vertices, then works through the touched ones together (K words each).
__device__ void ms_push_finish(const MsArgs &a, uint32_t lvl, uint64_t *nxt, unsigned long long &actdeg) {
	const uint32_t K = a.K;
	const unsigned lane = lane_id();
	uint32_t *qn = a.queue[(lvl + 1) & 1];
	uint64_t *actn = a.act[(lvl + 1) & 1];
	MsCounters *cn = &a.ctl->ctr[(lvl + 1) % 3];
	const uint32_t gwarp = blockIdx.x * kMsWarps + warp_id();
	const uint32_t nwarps = gridDim.x * kMsWarps;
	for (uint32_t vb = gwarp * 32; vb < a.n; vb += nwarps * 32) {
		const uint32_t v = vb + lane;
		const bool t = v < a.n && ld_cg_u8(a.touched + v);
		uint32_t anym = 0;
		for (uint32_t tm = __ballot_sync(kFull, t); tm; tm &= tm - 1) {
			const int j = __ffs(tm) - 1;
			const size_t row = (size_t) (vb + j) * K;
			uint64_t nw[2] = {0ull, 0ull};
#pragma unroll
			for (int h = 0; h < 2; ++h) {
				const uint32_t k = lane + 32 * h;
				if (k >= K) continue;
				const uint64_t w = ld_cg64(nxt + row + k);
				if (!w) continue;
				const uint64_t vv = ld_cg64(a.vis + row + k);
				nw[h] = w & ~vv;
				if (nw[h] != w) nxt[row + k] = nw[h];
				if (nw[h]) a.vis[row + k] = vv | nw[h];
			}
			const uint64_t mask = row_mask(nw[0], nw[1]);
			if (lane == 0) actn[vb + j] = mask;
			if (mask) anym |= 1u << j;
		}
		if (t) a.touched[v] = 0;
		else if (v < a.n) actn[v] = 0;
		const bool any = (anym >> lane) & 1u;
		const uint32_t d = any ? deg_of(a, v) : 0u;
		ms_append(a, cn, qn, v, any && d <= kMsBig, any && d > kMsBig);
		actdeg += d;
	}
}

// Pull appends: small vertices go through a per-warp shared buffer (one
// atomicAdd per kMsWq vertices), big ones straight to the queue's back.
__device__ __forceinline__ void ms_wq_flush(MsCounters *cn, uint32_t *qn, uint32_t *wbuf, uint32_t &wn) {
	__syncwarp();
	if (wn) {
		uint32_t base = 0;
		if (lane_id() == 0) base = atomicAdd(&cn->nact, wn);
		base = __shfl_sync(kFull, base, 0);
		for (uint32_t i = lane_id(); i < wn; i += 32) qn[base + i] = wbuf[i];
	}
	__syncwarp();
	wn = 0;
}

// The bits a complete word of lane's word (lane + 32 * h) holds.
struct FullMask {
	uint64_t f0, f1;
	__device__ __forceinline__ FullMask(const MsArgs &a, unsigned lane) {
		const uint64_t last = a.last_bits == 64 ? ~0ull : ((1ull << a.last_bits) - 1);
		f0 = lane < a.K ? (lane == a.K - 1 ? last : ~0ull) : 0ull;
		f1 = lane + 32 < a.K ? (lane + 32 == a.K - 1 ? last : ~0ull) : 0ull;
	}
	__device__ __forceinline__ bool complete(uint64_t x0, uint64_t x1) const {
		return __all_sync(kFull, (x0 & f0) == f0 && (x1 & f1) == f1);
	}
};

// ORs into acc the frontier words of the in-neighbours in [beg, end) until
// every source has reached the destination.  Only words that are non-zero in
// the neighbour's row and still incomplete in the destination's are read.
// Returns true when it stopped early.  Warp-uniform.
__device__ __forceinline__ bool ms_gather(const MsArgs &a, const uint64_t *cur, const uint64_t *actc, uint32_t beg,
		uint32_t end, const FullMask &fm, uint64_t vis0, uint64_t vis1, uint64_t &acc0, uint64_t &acc1,
		unsigned long long &gathered) {
	const uint32_t K = a.K;
	const unsigned lane = lane_id();
	bool done = false;
	for (uint32_t e0 = beg; e0 < end && !done; e0 += 32) {
		const uint32_t e = e0 + lane;
		const uint32_t u = e < end ? __ldg(a.in_src + e) : 0u;
		const uint64_t um = e < end ? ld_cg64(actc + u) : 0ull;
		uint32_t lm = __ballot_sync(kFull, um != 0ull);
		while (lm && !done) {
			const bool need0 = ((acc0 | vis0) & fm.f0) != fm.f0;
			const bool need1 = ((acc1 | vis1) & fm.f1) != fm.f1;
			uint64_t g0[kMsGather], g1[kMsGather];
			int cnt = 0;
#pragma unroll
			for (int t = 0; t < kMsGather; ++t) {
				uint32_t ut = 0;
				uint64_t mt = 0;
				if (lm) {
					const int src_lane = __ffs(lm) - 1;
					lm &= lm - 1;
					ut = __shfl_sync(kFull, u, src_lane);
					mt = shfl64(um, src_lane);
					++cnt;
				}
				const uint64_t *r = cur + (size_t) ut * K;
				g0[t] = (need0 && ((mt >> lane) & 1ull)) ? ld_cg64(r + lane) : 0ull;
				g1[t] = (need1 && ((mt >> (lane + 32)) & 1ull)) ? ld_cg64(r + lane + 32) : 0ull;
			}
#pragma unroll
			for (int t = 0; t < kMsGather; ++t) { acc0 |= g0[t]; acc1 |= g1[t]; }
			if (lane == 0) gathered += cnt;
			done = fm.complete(acc0 | vis0, acc1 | vis1);
		}
	}
	return done;
}

// Pull, destinations with at most kMsPullBig in-edges: a warp per
// destination, lane l owns words l and l + 32.  The rows of the others are
// cleared here and filled by ms_pull_chunks.
__device__ void ms_pull(const MsArgs &a, uint32_t lvl, const uint64_t *cur, uint64_t *nxt, unsigned long long &actdeg,
		unsigned long long &gathered, uint32_t *wq_base) {
	const uint32_t K = a.K;
	const uint64_t *actc = a.act[lvl & 1];
	uint64_t *actn = a.act[(lvl + 1) & 1];
	uint32_t *qn = a.queue[(lvl + 1) & 1];
	MsCounters *cn = &a.ctl->ctr[(lvl + 1) % 3];
	const unsigned lane = lane_id();
	const uint32_t gwarp = blockIdx.x * kMsWarps + warp_id();
	const uint32_t nwarps = gridDim.x * kMsWarps;
	const bool w0 = lane < K, w1 = lane + 32 < K;
	const FullMask fm(a, lane);
	uint32_t *wbuf = wq_base + warp_id() * kMsWq;
	uint32_t wn = 0;
	for (uint32_t v = gwarp; v < a.n; v += nwarps) {
		const size_t row = (size_t) v * K;
		const uint32_t beg = __ldg(a.in_off + v), end = __ldg(a.in_off + v + 1);
		const uint64_t vis0 = w0 ? ld_cg64(a.vis + row + lane) : 0ull;
		const uint64_t vis1 = w1 ? ld_cg64(a.vis + row + lane + 32) : 0ull;
		if (end - beg > kMsPullBig) {
			if (w0) nxt[row + lane] = 0;
			if (w1) nxt[row + lane + 32] = 0;
			continue;
		}
		uint64_t acc0 = 0, acc1 = 0;
		if (!fm.complete(vis0, vis1)) ms_gather(a, cur, actc, beg, end, fm, vis0, vis1, acc0, acc1, gathered);
		const uint64_t n0 = acc0 & ~vis0 & fm.f0, n1 = acc1 & ~vis1 & fm.f1;
		if (w0) { nxt[row + lane] = n0; if (n0) a.vis[row + lane] = vis0 | n0; }
		if (w1) { nxt[row + lane + 32] = n1; if (n1) a.vis[row + lane + 32] = vis1 | n1; }
		const uint64_t mask = row_mask(n0, n1);
		if (lane == 0) actn[v] = mask;
		if (mask) {
			const uint32_t d = deg_of(a, v);
			if (lane == 0) actdeg += d;
			if (d > kMsBig) {
				if (lane == 0) qn[a.n - 1 - atomicAdd(&cn->nbig, 1u)] = v;
			} else {
				if (lane == 0) wbuf[wn] = v;
				if (++wn == kMsWq) ms_wq_flush(cn, qn, wbuf, wn);
			}
		}
	}
	ms_wq_flush(cn, qn, wbuf, wn);
}

// Pull, destinations with many in-edges: warps take chunks of kMsChunk
// in-edges over the whole grid and OR what they gather into the row.
__device__ void ms_pull_chunks(const MsArgs &a, uint32_t lvl, const uint64_t *cur, uint64_t *nxt,
		unsigned long long &gathered) {
	const uint32_t K = a.K;
	const uint64_t *actc = a.act[lvl & 1];
	const unsigned lane = lane_id();
	const uint32_t gwarp = blockIdx.x * kMsWarps + warp_id();
	const uint32_t nwarps = gridDim.x * kMsWarps;
	const bool w0 = lane < K, w1 = lane + 32 < K;
	const FullMask fm(a, lane);
	for (uint32_t c = gwarp; c < a.nchunks; c += nwarps) {
		const uint32_t v = __ldg(a.chunk_v + c), beg = __ldg(a.chunk_beg + c);
		const uint32_t end = min(beg + kMsChunk, __ldg(a.in_off + v + 1));
		const size_t row = (size_t) v * K;
		const uint64_t vis0 = w0 ? ld_cg64(a.vis + row + lane) : 0ull;
		const uint64_t vis1 = w1 ? ld_cg64(a.vis + row + lane + 32) : 0ull;
		if (fm.complete(vis0, vis1)) continue;
		uint64_t acc0 = 0, acc1 = 0;
		ms_gather(a, cur, actc, beg, end, fm, vis0, vis1, acc0, acc1, gathered);
		const uint64_t n0 = acc0 & ~vis0 & fm.f0, n1 = acc1 & ~vis1 & fm.f1;
		if (n0) atomicOr((unsigned long long *) (nxt + row + lane), (unsigned long long) n0);
		if (n1) atomicOr((unsigned long long *) (nxt + row + lane + 32), (unsigned long long) n1);
	}
}

// After ms_pull_chunks: the many-in-edge destinations' rows hold their new
// bits; update vis, the frontier mask and the queue.
__device__ void ms_pull_chunks_finish(const MsArgs &a, uint32_t lvl, uint64_t *nxt, unsigned long long &actdeg) {
	const uint32_t K = a.K;
	uint64_t *actn = a.act[(lvl + 1) & 1];
	uint32_t *qn = a.queue[(lvl + 1) & 1];
	MsCounters *cn = &a.ctl->ctr[(lvl + 1) % 3];
	const unsigned lane = lane_id();
	const uint32_t gwarp = blockIdx.x * kMsWarps + warp_id();
	const uint32_t nwarps = gridDim.x * kMsWarps;
	const bool w0 = lane < K, w1 = lane + 32 < K;
	for (uint32_t j = gwarp; j < a.nbig_in; j += nwarps) {
		const uint32_t v = __ldg(a.in_big + j);
		const size_t row = (size_t) v * K;
		uint64_t n0 = 0, n1 = 0;
		if (w0) {
			n0 = ld_cg64(nxt + row + lane);
			if (n0) a.vis[row + lane] = ld_cg64(a.vis + row + lane) | n0;
		}
		if (w1) {
			n1 = ld_cg64(nxt + row + lane + 32);
			if (n1) a.vis[row + lane + 32] = ld_cg64(a.vis + row + lane + 32) | n1;
		}
		const uint64_t mask = row_mask(n0, n1);
		if (lane == 0) {
			actn[v] = mask;
			if (mask) {
				const uint32_t d = deg_of(a, v);
				actdeg += d;
				if (d > kMsBig) qn[a.n - 1 - atomicAdd(&cn->nbig, 1u)] = v;
				else qn[atomicAdd(&cn->nact, 1u)] = v;
			}
		}
	}
}

// Planes [first, last] (levels base + p) -> uint8 levels [source][vertex].
// A CTA takes tiles of 64 vertices x 8 words: each thread loads one word per
// plane (a warp reads 4 vertices x 64 contiguous bytes), writes the level of
// each set bit into the shared tile, then the tile leaves as 64-byte rows.
// `merge` starts each tile from the bytes already in `levels` (a later
// segment of a traversal deeper than the planes) instead of 255.
__device__ void ms_emit(const MsArgs &a, uint8_t *levels, uint32_t ns, uint32_t base, uint32_t first, uint32_t last,
		bool merge, uint8_t *lev) {
	const uint32_t K = a.K, n = a.n;
	const uint32_t vtiles = (n + kEmitV - 1) / kEmitV, wtiles = (K + kEmitWords - 1) / kEmitWords;
	const uint32_t vi = threadIdx.x / kEmitWords, wi = threadIdx.x % kEmitWords;
	for (uint32_t tile = blockIdx.x; tile < vtiles * wtiles; tile += gridDim.x) {
		const uint32_t v0 = (tile % vtiles) * kEmitV, k0 = (tile / vtiles) * kEmitWords;
		const uint32_t nv = min(kEmitV, n - v0);
		const uint32_t nrows = min(kEmitRows, ns - k0 * 64);
		const bool vec = a.vec_out && nv == kEmitV;
		// 1. start values
		for (uint32_t idx = threadIdx.x; idx < kEmitRows * (kEmitV / 4); idx += blockDim.x) {
			const uint32_t r = idx / (kEmitV / 4), c = (idx % (kEmitV / 4)) * 4;
			uint32_t val = 0xFFFFFFFFu;
			if (merge && r < nrows) {
				const uint8_t *src = levels + (size_t) (k0 * 64 + r) * n + v0 + c;
				if (vec) {
					val = __ldcg((const unsigned int *) src);
				} else {
					for (uint32_t b = 0; b < 4; ++b)
						if (c + b < nv) val = (val & ~(0xFFu << (8 * b))) | ((uint32_t) ld_cg_u8(src + b) << (8 * b));
				}
			}
			*(uint32_t *) (lev + r * kEmitStride + c) = val;
		}
		__syncthreads();
		// 2. the level of every set bit
		if (vi < nv && k0 + wi < K) {
			const uint64_t *p = a.hist + ((size_t) first * n + v0 + vi) * K + k0 + wi;
			const size_t pstride = (size_t) n * K;
			uint8_t *col = lev + wi * 64 * kEmitStride + vi;
			for (uint32_t l = first; l <= last; l += 4) {
				uint64_t w[4];
#pragma unroll
				for (int t = 0; t < 4; ++t) w[t] = l + t <= last ? ld_cg64(p + (size_t) (l - first + t) * pstride) : 0ull;
#pragma unroll
				for (int t = 0; t < 4; ++t) {
					const uint8_t val = (uint8_t) (base + l + t);
					for (uint64_t x = w[t]; x; x &= x - 1) col[(__ffsll((long long) x) - 1) * kEmitStride] = val;
				}
			}
		}
		__syncthreads();
		// 3. rows out
		for (uint32_t idx = threadIdx.x; idx < kEmitRows * (kEmitV / 16); idx += blockDim.x) {
			const uint32_t r = idx / (kEmitV / 16), c = (idx % (kEmitV / 16)) * 16;
			if (r >= nrows) continue;
			uint8_t *dst = levels + (size_t) (k0 * 64 + r) * n + v0 + c;
			const uint8_t *s = lev + r * kEmitStride + c;
			if (vec) {
				uint4 x;
				x.x = *(const uint32_t *) (s + 0);
				x.y = *(const uint32_t *) (s + 4);
				x.z = *(const uint32_t *) (s + 8);
				x.w = *(const uint32_t *) (s + 12);
				*(uint4 *) dst = x;
			} else {
				for (uint32_t b = 0; b < 16; ++b)
					if (c + b < nv) dst[b] = s[b];
			}
		}
		__syncthreads();
	}
}

__global__ void __launch_bounds__(kMsThreads, 2) k_ms_bfs(MsArgs a, const uint32_t *sources, uint32_t ns,
		uint8_t *levels) {
	__shared__ unsigned long long red[kMsWarps];
	__shared__ uint32_t wq[kMsWarps * kMsWq];
	__shared__ __align__(16) uint8_t lev[kEmitRows * kEmitStride];
	MsControl *ctl = a.ctl;
	const uint32_t stride = gridDim.x * blockDim.x;
	const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
	const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
	const size_t nK = (size_t) a.n * a.K;
	// clear (the control block was zeroed by the host)
	for (size_t i = t0; i < nK; i += stride) { a.vis[i] = 0; a.hist[i] = 0; }
	for (uint32_t i = t0; i < a.n; i += stride) {
		a.act[0][i] = 0;
		a.act[1][i] = 0;
		a.touched[i] = 0;
		a.seed_flag[i] = 0;
	}
	bool ok = grid_barrier(ctl->bar, &ctl->err);
	// plane 0: every source reaches itself
	if (ok) {
		for (uint32_t i = t0; i < ns; i += stride) {
			const uint32_t v = sources[i];
			const size_t x = (size_t) v * a.K + i / 64;
			const unsigned long long bit = 1ull << (i % 64);
			atomicOr((unsigned long long *) (a.hist + x), bit);
			atomicOr((unsigned long long *) (a.vis + x), bit);
			atomicOr((unsigned long long *) (a.act[0] + v), 1ull << (i / 64));
			if (atomicExch(a.seed_flag + v, 1u) == 0u) {
				const uint32_t d = deg_of(a, v);
				if (d > kMsBig) a.queue[0][a.n - 1 - atomicAdd(&ctl->ctr[0].nbig, 1u)] = v;
				else a.queue[0][atomicAdd(&ctl->ctr[0].nact, 1u)] = v;
				atomicAdd(&ctl->ctr[0].act_deg, (unsigned long long) d);
			}
		}
		ok = grid_barrier(ctl->bar, &ctl->err);
	}
	if (leader) ctl->stats.t_levels0 = global_timer_ns();
	unsigned long long gathered = 0;
	uint32_t base = 0, lvl = 0;
	bool complete = false;
	for (; ok; ++lvl) {
		MsCounters *cc = &ctl->ctr[lvl % 3];
		const uint32_t nq = ld_volatile(&cc->nact), nb = ld_volatile(&cc->nbig);
		const unsigned long long qdeg = ld_volatile_u64(&cc->act_deg);
		if (nq + nb == 0) { complete = true; break; }
		if (lvl >= kMsMaxLevel) {
			if (leader) atomicExch(&ctl->err, BFS_EUNSUPPORTED);
			break;
		}
		if (lvl + 1 - base >= a.planes) {
			// planes full: write them out, keep the frontier's plane as plane 0
			ms_emit(a, levels, ns, base, base == 0 ? 0 : 1, lvl - base, base != 0, lev);
			if (!(ok = grid_barrier(ctl->bar, &ctl->err))) break;
			const uint64_t *src = a.hist + (size_t) (lvl - base) * nK;
			for (size_t i = t0; i < nK; i += stride) a.hist[i] = ld_cg64(src + i);
			base = lvl;
			if (leader) ctl->stats.spills++;
			if (!(ok = grid_barrier(ctl->bar, &ctl->err))) break;
		}
		// the counters of the level after next are free again
		if (leader) {
			if (lvl < kMsTraceLevels) {
				ctl->stats.t_level[lvl] = global_timer_ns();
				ctl->stats.frontier[lvl] = nq + nb;
				ctl->stats.push[lvl] = qdeg * (unsigned long long) a.push_div < (unsigned long long) a.m;
			}
			MsCounters *c2 = &ctl->ctr[(lvl + 2) % 3];
			c2->nact = 0;
			c2->nbig = 0;
			c2->act_deg = 0;
		}
		const uint64_t *cur = a.hist + (size_t) (lvl - base) * nK;
		uint64_t *nxt = a.hist + (size_t) (lvl + 1 - base) * nK;
		unsigned long long actdeg = 0;
		const bool push = qdeg * (unsigned long long) a.push_div < (unsigned long long) a.m;
		if (push) {
			for (size_t i = t0; i < nK; i += stride) nxt[i] = 0;
			if (!(ok = grid_barrier(ctl->bar, &ctl->err))) break;
			ms_push(a, lvl, cur, nxt, nq, nb);
			if (!(ok = grid_barrier(ctl->bar, &ctl->err))) break;
			ms_push_finish(a, lvl, nxt, actdeg);
		} else {
			ms_pull(a, lvl, cur, nxt, actdeg, gathered, wq);
			if (a.nbig_in) {
				if (!(ok = grid_barrier(ctl->bar, &ctl->err))) break;
				ms_pull_chunks(a, lvl, cur, nxt, gathered);
				if (!(ok = grid_barrier(ctl->bar, &ctl->err))) break;
				ms_pull_chunks_finish(a, lvl, nxt, actdeg);
			}
		}
		// the next frontier's out-degree: per-CTA sum, one atomic per CTA
		const unsigned long long d = warp_sum(actdeg);
		if (lane_id() == 0) red[warp_id()] = d;
		__syncthreads();
		if (threadIdx.x == 0) {
			unsigned long long tsum = 0;
			for (int w = 0; w < kMsWarps; ++w) tsum += red[w];
			if (tsum) atomicAdd(&ctl->ctr[(lvl + 1) % 3].act_deg, tsum);
			if (blockIdx.x == 0) {
				ctl->stats.levels = lvl + 1;
				if (push) ctl->stats.push_levels++;
			}
		}
		__syncthreads();
		ok = grid_barrier(ctl->bar, &ctl->err);
	}
	if (leader) {
		ctl->stats.t_levels1 = global_timer_ns();
		if (lvl < kMsTraceLevels) ctl->stats.t_level[lvl] = ctl->stats.t_levels1;
	}
	if (complete) {
		// plane lvl - base is the empty frontier; a later segment's plane 0 was written already
		const uint32_t first = base == 0 ? 0 : 1;
		if (lvl - 1 >= base + first) ms_emit(a, levels, ns, base, first, lvl - 1 - base, base != 0, lev);
		// TEPS numerator: sum over (source, reached vertex) of out-degree
		unsigned long long tr = 0;
		for (uint32_t v = t0; v < a.n; v += stride) {
			uint32_t c = 0;
			for (uint32_t k = 0; k < a.K; ++k) c += __popcll(ld_cg64(a.vis + (size_t) v * a.K + k));
			tr += (unsigned long long) c * deg_of(a, v);
		}
		tr = warp_sum(tr);
		__syncthreads();
		if (lane_id() == 0) red[warp_id()] = tr;
		__syncthreads();
		if (threadIdx.x == 0) {
			unsigned long long tsum = 0;
			for (int w = 0; w < kMsWarps; ++w) tsum += red[w];
			if (tsum) atomicAdd(&ctl->stats.traversed, tsum);
		}
	}
	const unsigned long long gw = warp_sum(gathered);
	if (lane_id() == 0 && gw) atomicAdd(&ctl->stats.edges, gw);
	if (leader) ctl->stats.depth = lvl;
}

int ms_launch(const MsArgs &a, const uint32_t *d_sources, uint32_t ns, uint8_t *levels, int num_sms, cudaStream_t st,
		int *grid) {
	int per_sm = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ms_bfs, kMsThreads, 0) != cudaSuccess || per_sm < 1)
		return BFS_ECUDA;
	per_sm = std::min(per_sm, 2);
	if (grid) *grid = num_sms * per_sm;
	if (cudaMemsetAsync(a.ctl, 0, sizeof(MsControl), st) != cudaSuccess) return BFS_ECUDA;
	MsArgs aa = a;
	const uint32_t *src = d_sources;
	uint32_t nsrc = ns;
	uint8_t *out = levels;
	void *args[] = {&aa, (void *) &src, &nsrc, &out};
	if (cudaLaunchCooperativeKernel((const void *) k_ms_bfs, dim3(num_sms * per_sm), dim3(kMsThreads), args, 0, st) !=
			cudaSuccess)
		return BFS_ECUDA;
	return BFS_OK;
}

} // namespace bfsg
