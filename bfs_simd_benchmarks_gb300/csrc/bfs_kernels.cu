// bfs_kernels.cu -- the single-source hybrid BFS on one GB300.
//
// Steps follow the reference's graph_prepare loop (apps/bfs_simd/bfs.cpp:806-912):
// step 0 is top-down from the source; every later step goes bottom-up ("dense")
// when frontier + out_degree of the frontier exceeds E / T_RATIO (:832-834) and
// top-down ("sparse") otherwise, converting the frontier between queue and
// bitmap form when the direction changes (to_dense :54-88, to_sparse :400-465).
//
// GPU design (no counterpart in the reference's code, same results):
//   - top-down (BFS_kernel_sparse, :510-711): the frontier lives in three
//     queues bucketed by out-degree; small-degree vertices are expanded 32 at a
//     time by one warp (warp-wide scan of degrees, lanes take consecutive
//     edges), medium ones by one CTA each, large ones by all CTAs of the grid.
//     A vertex is claimed by atomicOr on the visited bitmap (the reference CASes
//     parents[v], :575); claimed vertices are appended to the next queues with
//     one atomicAdd per warp and bucket.
//   - bottom-up (BFS_dense -> scheduler_dense -> bfs_kernel_dense, :181-388):
//     a CTA owns a column group (whole tile columns = a destination vertex
//     range), keeps that range's visited and next-frontier bits in shared
//     memory, and streams the group's segment of every active stripe from the
//     packed column-major tile stream with 128-bit loads.  The stripe's frontier
//     slice (S*W bits) is staged in shared memory.  An edge whose destination is
//     already visited is skipped without touching the frontier (per-vertex early
//     exit), and the CTA stops streaming a group once every vertex of the group
//     that has an in-edge is visited (per-group early exit).
//   - queue<->bitmap conversions use ballot/popc and warp-aggregated atomics.
//   - BFS_MODE_PERSISTENT runs every step in one cooperative launch separated
//     by a bounded-spin grid barrier; BFS_MODE_STEPWISE launches each phase on
//     its own and decides the direction on the host.
#include <cstdio>

#include "bfs_device.cuh"
#include "device_common.cuh"
#include "kernels_api.h"

namespace bfsg {

constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;

// Per-CTA phase stamps for profiling builds (nvcc -DBFS_CTA_TIMERS): thread 0
// of every CTA records the globaltimer at fixed points of the first 16 steps.
#ifdef BFS_CTA_TIMERS
constexpr int kProfPoints = 10;
__device__ unsigned long long g_cta_prof[16][kProfPoints][kMaxGrid];
#define CTA_STAMP(step, k) \
	do { if (threadIdx.x == 0 && (step) < 16) g_cta_prof[step][k][blockIdx.x] = global_timer_ns(); } while (0)
#else
#define CTA_STAMP(step, k) do { } while (0)
#endif

struct ThreadAcc {
	unsigned long long count, degsum, td_edges, td_vertices, bu_words, bu_slices, bu_groups, bu_vertices;
};

__device__ __forceinline__ uint32_t bucket_of(uint32_t deg, const StepParams &p) {
	return deg <= p.warp_max_degree ? 0u : (deg <= p.cta_max_degree ? 1u : 2u);
}

constexpr int kTdPerLane = 4;  // candidate edges a lane handles per top-down iteration
// Medium-degree buckets up to this size join the grid-flat expansion of the
// large ones (a few chunks); larger ones are spread over CTAs in chunks.
constexpr uint32_t kFlatMediumMax = 4 * kThreads;
// Flat-expansion vertices staged per chunk (in dynamic shared memory after
// the warps' append buffers).
constexpr uint32_t kFlatChunk = 4 * kThreads;

// Next-frontier appends of one warp are staged in a shared-memory buffer per
// degree bucket and moved to the global queue in blocks, so the queue tails
// see one atomicAdd per block of up to kWqCap vertices instead of one per
// warp iteration (the three tails share a cache line that every CTA hits).
constexpr uint32_t kWqCap = 32 * kTdPerLane;

struct WarpQ {
	uint32_t *buf;           // this warp's 3 x kWqCap entries
	uint32_t n[3];           // staged entries per bucket (warp-uniform)
	uint32_t *const *qn;     // the global next-frontier queues
	unsigned *tails;
};

__device__ __forceinline__ void wq_flush(WarpQ &wq, int bk) {
	__syncwarp();
	const unsigned lane = lane_id();
	uint32_t base = 0;
	if (lane == 0) base = atomicAdd(&wq.tails[bk], wq.n[bk]);
	base = __shfl_sync(kFull, base, 0);
	for (uint32_t i = lane; i < wq.n[bk]; i += 32) wq.qn[bk][base + i] = wq.buf[bk * kWqCap + i];
	__syncwarp();
	wq.n[bk] = 0;
}

__device__ __forceinline__ void wq_flush_all(WarpQ &wq) {
#pragma unroll
	for (int bk = 0; bk < 3; ++bk)
		if (wq.n[bk]) wq_flush(wq, bk);
}

// All 32 lanes of the warp call this with up to kTdPerLane candidate edges
// u[q] -> v[q] each (has[q] false for an empty slot).  Each stage -- the
// claiming compare-and-swap, the degree load of the claimed -- is issued for
// all candidates before any result is used, so a lane waits for two round
// trips per batch of edges, not per edge.  (A visited-bitmap pre-load before
// the claim kept visited destinations off the atomic unit but cost a round
// trip per batch: measured slower on R-MAT frontiers.)
// Claimed vertices get their level and parent, their bit in the next
// frontier's bitmap `nbm` (so that a bottom-up step after this one needs no
// queue -> bitmap conversion) and are staged for the next queue bucket of
// their out-degree.
__device__ __forceinline__ void visit_and_append(const bool (&has)[kTdPerLane], const uint32_t (&u)[kTdPerLane],
		const uint32_t (&v)[kTdPerLane], int32_t next_level, const DevGraph &g, const RunCtx &r, uint32_t *nbm,
		WarpQ &wq, const StepParams &p, ThreadAcc &acc) {
	// The claim is a compare-and-swap on the destination's own level (-1 ->
	// next level): only edges to the same destination contend, not the 32
	// destinations of a bitmap word.  The visited bit follows with a
	// reduction whose result nobody waits for.
	bool claimed[kTdPerLane];
#pragma unroll
	for (int q = 0; q < kTdPerLane; ++q)
		claimed[q] = has[q] && atomicCAS((int *) r.level + v[q], -1, next_level) == -1;
	uint32_t deg[kTdPerLane];
#pragma unroll
	for (int q = 0; q < kTdPerLane; ++q) {
		if (claimed[q]) {
			atomicOr(r.vis + (v[q] >> 5), 1u << (v[q] & 31));
			atomicOr(nbm + (v[q] >> 5), 1u << (v[q] & 31));
		}
		deg[q] = claimed[q] ? __ldg(g.row_off + v[q] + 1) - __ldg(g.row_off + v[q]) : 0u;
	}
	uint32_t cnt[3] = {0, 0, 0};
#pragma unroll
	for (int q = 0; q < kTdPerLane; ++q) {
		if (!claimed[q]) continue;
		if (r.parent) r.parent[v[q]] = u[q];
		acc.count++;
		acc.degsum += deg[q];
		cnt[bucket_of(deg[q], p)]++;
	}
	if (!__ballot_sync(kFull, cnt[0] | cnt[1] | cnt[2])) return;
	uint32_t pos[3];
#pragma unroll
	for (int bk = 0; bk < 3; ++bk) {
		const uint32_t incl = warp_incl_scan(cnt[bk]);
		const uint32_t tot = __shfl_sync(kFull, incl, 31);
		if (wq.n[bk] + tot > kWqCap) wq_flush(wq, bk);
		pos[bk] = wq.n[bk] + incl - cnt[bk];
		wq.n[bk] += tot;
	}
#pragma unroll
	for (int q = 0; q < kTdPerLane; ++q) {
		if (!claimed[q]) continue;
		const uint32_t bk = bucket_of(deg[q], p);
		wq.buf[bk * kWqCap + pos[bk]++] = v[q];
	}
	__syncwarp();
}

// Vertices of a top-down chunk staged in shared memory.
struct ExpandShared {
	uint32_t u[kThreads], beg[kThreads], pre[kThreads];
	uint32_t wsum[kWarps];
};
__device__ __shared__ ExpandShared xsh;

// CTA-wide inclusive scan (all threads call).
__device__ __forceinline__ uint32_t block_incl_scan(uint32_t x) {
	const unsigned lane = lane_id(), wid = warp_id();
	uint32_t incl = warp_incl_scan(x);
	if (lane == 31) xsh.wsum[wid] = incl;
	__syncthreads();
	if (wid == 0) {
		uint32_t w = lane < kWarps ? xsh.wsum[lane] : 0u;
		uint32_t wi = warp_incl_scan(w);
		if (lane < kWarps) xsh.wsum[lane] = wi - w;
	}
	__syncthreads();
	return incl + xsh.wsum[wid];
}

// ---------------------------------------------------------------------------
// Top-down step (BFS_kernel_sparse + update_sparse, apps/bfs_simd/bfs.cpp:467-711)
// ---------------------------------------------------------------------------
// The frontier's queue sizes nS, nM, nL (small, medium, large out-degree)
// come from the caller, which loads them together with the step totals.
__device__ __forceinline__ void phase_expand(const DevGraph &g, const RunCtx &r, const StepParams &p, uint32_t step,
		uint32_t nS, uint32_t nM, uint32_t nL, uint32_t *smem, ThreadAcc &acc) {
	const uint32_t cur = step & 1, nxt = (step + 1) & 1;
	StepCounters *out = r.ctr + step % 3;
	uint32_t *nbm = r.bm[step % 3];
	const uint32_t *qS = r.q[cur][0], *qM = r.q[cur][1], *qL = r.q[cur][2];
	uint32_t *const qn[3] = {r.q[nxt][0], r.q[nxt][1], r.q[nxt][2]};
	const int32_t nl = (int32_t) step + 1;
	const unsigned lane = lane_id(), wid = warp_id();
	// warps numbered across CTAs first, so that a small amount of work is
	// spread over all SMs rather than the first CTAs' warps
	const uint64_t gwarp = (uint64_t) wid * gridDim.x + blockIdx.x;
	const uint64_t nwarps = (uint64_t) gridDim.x * kWarps;
	constexpr uint32_t kSpan = 32 * kTdPerLane;  // edges per warp iteration
	WarpQ wq{smem + (size_t) wid * 3 * kWqCap, {0, 0, 0}, qn, out->tail};
	bool has[kTdPerLane];
	uint32_t uu[kTdPerLane], vv[kTdPerLane];

	// Large out-degree vertices -- and medium ones when there are few of them
	// -- are expanded as one flat edge range that every warp of the grid
	// shares evenly.  Each CTA stages a chunk of up to kFlatChunk such
	// vertices (usually all of them: every chunk costs each warp a setup and
	// a partial edge batch) with the inclusive prefix of their degrees in
	// shared memory; a lane finds the owner of its edge by binary search.
	const bool flat_medium = nM <= kFlatMediumMax;
	const uint32_t nflat = nL + (flat_medium ? nM : 0u);
	uint32_t *fu = smem + (size_t) kWarps * 3 * kWqCap, *fbeg = fu + kFlatChunk, *fpre = fbeg + kFlatChunk;
	for (uint32_t c0 = 0; c0 < nflat; c0 += kFlatChunk) {
		const uint32_t cn = min(kFlatChunk, nflat - c0);
		constexpr int kPer = kFlatChunk / kThreads;  // entries per thread, consecutive
		uint32_t u[kPer], beg[kPer], deg[kPer];
#pragma unroll
		for (int k = 0; k < kPer; ++k) {
			const uint32_t x = threadIdx.x * kPer + k, y = c0 + x;
			u[k] = x < cn ? ld_cg(y < nL ? qL + y : qM + (y - nL)) : 0u;
		}
#pragma unroll
		for (int k = 0; k < kPer; ++k) {
			const bool in = threadIdx.x * kPer + k < cn;
			beg[k] = in ? __ldg(g.row_off + u[k]) : 0u;
			deg[k] = in ? __ldg(g.row_off + u[k] + 1) - beg[k] : 0u;
		}
		uint32_t sum = 0;
#pragma unroll
		for (int k = 0; k < kPer; ++k) sum += deg[k];
		uint32_t run = block_incl_scan(sum) - sum;
#pragma unroll
		for (int k = 0; k < kPer; ++k) {
			const uint32_t x = threadIdx.x * kPer + k;
			run += deg[k];
			fu[x] = u[k];
			fbeg[x] = beg[k];
			fpre[x] = run;
		}
		__syncthreads();
		const uint32_t total = fpre[cn - 1];
		const uint64_t per = (total + nwarps - 1) / nwarps;
		const uint64_t lo = min((uint64_t) total, gwarp * per), hi = min((uint64_t) total, lo + per);
		for (uint64_t f0 = lo; f0 < hi; f0 += kSpan) {
#pragma unroll
			for (int q = 0; q < kTdPerLane; ++q) {
				const uint64_t f = f0 + q * 32 + lane;
				has[q] = f < hi;
				uint32_t j = 0;  // owner: the number of entries whose inclusive prefix is <= f
				if (has[q]) {
#pragma unroll
					for (uint32_t sp = kFlatChunk / 2; sp >= 1; sp >>= 1)
						if (j + sp < cn && fpre[j + sp - 1] <= f) j += sp;
				}
				const uint32_t jj = min(j, cn - 1);
				const uint32_t prev = jj ? fpre[jj - 1] : 0u;
				uu[q] = fu[jj];
				vv[q] = has[q] ? __ldg(g.col + fbeg[jj] + (uint32_t) (f - prev)) : 0u;
			}
			visit_and_append(has, uu, vv, nl, g, r, nbm, wq, p, acc);
		}
		if (blockIdx.x == 0 && threadIdx.x == 0) { acc.td_edges += total; acc.td_vertices += cn; }
		__syncthreads();
	}
	CTA_STAMP(step, 6);
	// Medium out-degree, many vertices: a CTA expands a chunk of up to 32
	// vertices as one flat edge list.  Chunks (about 8 per CTA) are handed out
	// by a counter, the next one fetched while this one runs: medium degrees
	// span 33..cta_max_degree, and a fixed assignment left CTAs with the
	// heavy chunks finishing long after the rest.
	if (!flat_medium) {
		__shared__ uint32_t s_next;
		const uint32_t chunk = max(1u, min(32u, nM / (gridDim.x * 8)));
		const uint32_t nchunks = (nM + chunk - 1) / chunk;
		if (threadIdx.x == 0) s_next = atomicAdd(&out->work, 1u);
		__syncthreads();
		uint32_t pending = 0;
		for (uint32_t ci = s_next; ci < nchunks;) {
			if (threadIdx.x == 0) pending = atomicAdd(&out->work, 1u);
			const uint32_t c0 = ci * chunk, cn = min(chunk, nM - c0);
			if (wid == 0) {
				uint32_t deg = 0, u = 0, beg = 0;
				if (lane < cn) {
					u = ld_cg(qM + c0 + lane);
					beg = __ldg(g.row_off + u);
					deg = __ldg(g.row_off + u + 1) - beg;
				}
				const uint32_t incl = warp_incl_scan(deg);
				xsh.u[lane] = u;
				xsh.beg[lane] = beg;
				xsh.pre[lane] = incl;
			}
			__syncthreads();
			const uint32_t total = xsh.pre[cn - 1];
			for (uint64_t f0 = (uint64_t) wid * kSpan; f0 < total; f0 += (uint64_t) kWarps * kSpan) {
#pragma unroll
				for (int q = 0; q < kTdPerLane; ++q) {
					const uint64_t f = f0 + q * 32 + lane;
					has[q] = f < total;
					uint32_t j = 0;
					if (has[q]) {
#pragma unroll
						for (uint32_t sp = 16; sp >= 1; sp >>= 1)
							if (j + sp < cn && xsh.pre[j + sp - 1] <= f) j += sp;
					}
					const uint32_t jj = min(j, cn - 1);
					const uint32_t prev = jj ? xsh.pre[jj - 1] : 0u;
					uu[q] = xsh.u[jj];
					vv[q] = has[q] ? __ldg(g.col + xsh.beg[jj] + (uint32_t) (f - prev)) : 0u;
				}
				visit_and_append(has, uu, vv, nl, g, r, nbm, wq, p, acc);
			}
			if (threadIdx.x == 0) {
				acc.td_edges += total;
				acc.td_vertices += cn;
				s_next = pending;
			}
			__syncthreads();
			ci = s_next;
		}
	}
	CTA_STAMP(step, 7);
	// Small out-degree: one warp expands up to 32 vertices together; lanes
	// take consecutive edges of the warp's combined edge list.  A small
	// frontier is spread thinner (down to one vertex per warp), so that its
	// chain of dependent loads runs on many warps at once.
	const uint32_t vpw = nS >= nwarps * 32 ? 32u : (uint32_t) max((uint64_t) 1, (nS + nwarps - 1) / nwarps);
	for (uint64_t base = gwarp * vpw; base < nS; base += nwarps * vpw) {
		const uint64_t i = base + lane;
		const bool valid = lane < vpw && i < nS;
		const uint32_t u = valid ? ld_cg(qS + i) : 0u;
		const uint32_t beg = valid ? __ldg(g.row_off + u) : 0u;
		const uint32_t deg = valid ? __ldg(g.row_off + u + 1) - beg : 0u;
		const uint32_t incl = warp_incl_scan(deg);
		const uint32_t total = __shfl_sync(kFull, incl, 31);
		const uint32_t excl = incl - deg;
		for (uint32_t f0 = 0; f0 < total; f0 += kSpan) {
#pragma unroll
			for (int q = 0; q < kTdPerLane; ++q) {
				const uint32_t f = f0 + q * 32 + lane;
				has[q] = f < total;
				// owner = number of lanes whose inclusive degree sum is <= f
				int lo = 0;
#pragma unroll
				for (int st = 16; st >= 1; st >>= 1) {
					const uint32_t val = __shfl_sync(kFull, incl, lo + st - 1);
					if (val <= f) lo += st;
				}
				uu[q] = __shfl_sync(kFull, u, lo);
				const uint32_t ob = __shfl_sync(kFull, beg, lo);
				const uint32_t oe = __shfl_sync(kFull, excl, lo);
				vv[q] = has[q] ? __ldg(g.col + ob + (f - oe)) : 0u;
			}
			visit_and_append(has, uu, vv, nl, g, r, nbm, wq, p, acc);
		}
		const unsigned nvalid = (unsigned) __popc(__ballot_sync(kFull, valid));
		if (lane == 0) {
			acc.td_edges += total;
			acc.td_vertices += nvalid;
		}
	}
	CTA_STAMP(step, 8);
	wq_flush_all(wq);
}

// ---------------------------------------------------------------------------
// Queue -> bitmap (to_dense, apps/bfs_simd/bfs.cpp:54-88)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void phase_to_dense(const DevGraph &g, const RunCtx &r, uint32_t step, bool track_stripes) {
	const StepCounters *in = r.ctr + (step + 2) % 3;
	const uint32_t cur = step & 1;
	uint32_t n0 = ld_volatile(&in->tail[0]), n1 = ld_volatile(&in->tail[1]), n2 = ld_volatile(&in->tail[2]);
	uint32_t *bm = r.bm[(step + 2) % 3];
	uint8_t *sf = r.sf[(step + 2) % 3];
	uint64_t total = (uint64_t) n0 + n1 + n2;
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < total;
			i += (uint64_t) gridDim.x * blockDim.x) {
		uint32_t v;
		if (i < n0) v = ld_cg(r.q[cur][0] + i);
		else if (i < (uint64_t) n0 + n1) v = ld_cg(r.q[cur][1] + (i - n0));
		else v = ld_cg(r.q[cur][2] + (i - n0 - n1));
		atomicOr(bm + (v >> 5), 1u << (v & 31));
		// stripe flags feed only the streaming bottom-up step; read before
		// writing, since every CTA hits the same few cache lines
		if (track_stripes && !ld_cg_u8(sf + v / g.sw)) sf[v / g.sw] = 1;
	}
}

// ---------------------------------------------------------------------------
// Bitmap -> queue (to_sparse, apps/bfs_simd/bfs.cpp:400-465)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void phase_to_sparse(const DevGraph &g, const RunCtx &r, const StepParams &p, uint32_t step) {
	const uint32_t *bm = r.bm[(step + 2) % 3];
	const uint32_t cur = step & 1;
	StepCounters *slot = r.ctr + (step + 2) % 3;
	const unsigned lane = lane_id();
	const uint64_t gwarp = (uint64_t) blockIdx.x * kWarps + warp_id();
	const uint64_t nwarps = (uint64_t) gridDim.x * kWarps;
	for (uint64_t base = gwarp * 32; base < g.nwords; base += nwarps * 32) {
		uint64_t w = base + lane;
		uint32_t bits = (w < g.nwords) ? ld_cg(bm + w) : 0u;
		uint32_t c[3] = {0, 0, 0};
		for (uint32_t b = bits; b; b &= b - 1) {
			uint32_t v = (uint32_t) (w * 32 + (__ffs(b) - 1));
			uint32_t deg = __ldg(g.row_off + v + 1) - __ldg(g.row_off + v);
			c[bucket_of(deg, p)]++;
		}
		uint32_t off[3];
#pragma unroll
		for (int bk = 0; bk < 3; ++bk) {
			uint32_t incl = warp_incl_scan(c[bk]);
			uint32_t tot = __shfl_sync(kFull, incl, 31);
			uint32_t b0 = 0;
			if (lane == 31 && tot) b0 = atomicAdd(&slot->tail[bk], tot);
			b0 = __shfl_sync(kFull, b0, 31);
			off[bk] = b0 + incl - c[bk];
		}
		for (uint32_t b = bits; b; b &= b - 1) {
			uint32_t v = (uint32_t) (w * 32 + (__ffs(b) - 1));
			uint32_t deg = __ldg(g.row_off + v + 1) - __ldg(g.row_off + v);
			uint32_t bk = bucket_of(deg, p);
			r.q[cur][bk][off[bk]++] = v;
		}
	}
}

// ---------------------------------------------------------------------------
// Bottom-up step (BFS_dense / scheduler_dense / bfs_kernel_dense + update_dense,
// apps/bfs_simd/bfs.cpp:91-388)
// ---------------------------------------------------------------------------
struct DenseShared {
	uint32_t group, unsettled, nlist, stop;
	uint32_t wcount[kWarps], woff[kWarps];
	uint32_t prefix[kMaxSliceBatch + 1];
	uint32_t seq;  // bulk-copy batches this CTA has consumed (keeps the mbarrier parities)
	uint32_t fail; // a bulk-copy wait of this CTA ran out
};

// One bulk-copy stage: which stripes its entries belong to and where their
// vectors start (entries are packed back to back in the stage buffer).
struct TmaMeta {
	uint32_t nent;
	uint32_t kfirst;  // stripe of the first slice in the stage
	uint32_t k[kMaxSliceBatch];
	uint32_t pre[kMaxSliceBatch + 1];  // vector prefix; pre[nent] = vectors in the stage
};

struct DenseGroup {
	uint64_t v0, v1;   // destination vertex range of the group
	uint32_t gi, gw;   // group index, bitmap words
};

__device__ __shared__ DenseShared dsh;
__device__ __shared__ TmaMeta tma_meta[kTmaStages];
__device__ __shared__ alignas(8) uint64_t tma_bar[kTmaStages];    // stage filled
__device__ __shared__ alignas(8) uint64_t tma_empty[kTmaStages];  // stage released by every consumer warp

// Claims the next work item -- a column group, or with `split` > 1 one of
// `split` equal parts (in 32-vertex words) of a column group -- loads its
// visited bits into vis_s and a copy into nxt_s, and counts the vertices
// with an in-edge that are still unvisited.  Returns false when no item is
// left.  Uniform across the CTA.
__device__ __forceinline__ bool dense_group_begin(const DevGraph &g, const RunCtx &r, StepCounters *out, uint32_t *vis_s,
		uint32_t *nxt_s, DenseGroup &gr, uint32_t *hin_s = nullptr, uint32_t split = 1, bool first = false) {
	__syncthreads();
	if (threadIdx.x == 0) {
		// with `first`, a CTA's first item is its own index (no atomic: the
		// whole grid asking at once queued on one line); later items are
		// counted from gridDim.x
		dsh.group = first ? blockIdx.x : (split > 1 ? gridDim.x : 0u) + atomicAdd(&out->work, 1u);
		dsh.unsettled = 0;
		dsh.stop = 0;
	}
	__syncthreads();
	const uint32_t item = dsh.group;
	if (item >= g.num_groups * split) return false;
	gr.gi = item / split;
	const uint32_t part = item % split;
	const uint32_t c0 = __ldg(g.group_col + gr.gi), c1 = __ldg(g.group_col + gr.gi + 1);
	const uint64_t a = (uint64_t) c0 * g.w, b = min((uint64_t) c1 * g.w, (uint64_t) g.n);
	const uint64_t words = (b - a + 31) / 32;
	gr.v0 = min(b, a + 32 * (words * part / split));
	gr.v1 = min(b, a + 32 * (words * (part + 1) / split));
	gr.gw = (uint32_t) ((gr.v1 - gr.v0 + 31) / 32);
	uint32_t uns = 0;
	for (uint32_t j = threadIdx.x; j < gr.gw; j += kThreads) {
		uint32_t vb = bits_at(r.vis, gr.v0 + 32ull * j, gr.v1, kFull);
		uint32_t hb = bits_at(g.hasin, gr.v0 + 32ull * j, gr.v1, 0u);
		vis_s[j] = vb;
		nxt_s[j] = vb;  // visited bits at the start: the new frontier is vis_s & ~nxt_s
		if (hin_s) hin_s[j] = hb;
		uns += __popc(hb & ~vb);
	}
	if (threadIdx.x == 0) vis_s[gr.gw] = kFull;  // the slot padding words point at
	uns = warp_sum(uns);
	if (lane_id() == 0 && uns) atomicAdd(&dsh.unsettled, uns);
	__syncthreads();
	return true;
}

// Graph constants of the bottom-up step, held in registers.
struct DenseRegs {
	uint32_t vbits, cmask, vmask, w, ushift, dmask, sw;
	int32_t *level;
	uint32_t *parent;
};

__device__ __forceinline__ DenseRegs dense_regs(const DevGraph &g, const RunCtx &r) {
	DenseRegs d;
	d.vbits = g.vbits;
	d.cmask = g.cmask;
	d.vmask = g.vmask;
	d.w = g.w;
	d.ushift = g.ushift;
	d.dmask = (g.vbits + g.cbits >= 32) ? 0xFFFFFFFFu : ((1u << (g.vbits + g.cbits)) - 1u);
	d.sw = g.sw;
	d.level = r.level;
	d.parent = r.parent;
	return d;
}

// The bottom-up test of one vector (four packed edge words) of a stage
// (bfs_kernel_dense, apps/bfs_simd/bfs.cpp:194-217): an edge is a candidate
// when its destination is not visited yet (a visited destination's scan is
// over; padding words land on an always-visited slot) and its source is in
// the stripe's frontier slice.  Both tests are done for all four words
// without branches; only candidates, a few percent of the edges, take the
// claiming branch, and a warp with no candidate skips it as a whole.  With
// a power-of-two tile width the destination is the low bits of the word.
// A claim sets the destination's bit in vis_s (the group's new frontier is
// vis_s & ~vis0_s at publish time, where the levels are written) and stores
// its parent.  Returns the number of destinations this thread claimed.
// All 32 lanes of the warp must call it; `active` false lanes take part
// without testing anything.
template <bool kPow2W>
__device__ __forceinline__ uint32_t dense_vec(bool active, const uint4 &x4, const DenseRegs &dr, uint32_t v0,
		uint32_t *vis_s, uint32_t *nxt_s, const uint32_t *sl, uint32_t ubase, int32_t nl) {
	const uint32_t e[4] = {x4.x, x4.y, x4.z, x4.w};
	uint32_t d[4], ul[4], cand = 0;
#pragma unroll
	for (int q = 0; q < 4; ++q) {
		d[q] = kPow2W ? (e[q] & dr.dmask) : ((e[q] >> dr.vbits) & dr.cmask) * dr.w + (e[q] & dr.vmask);
		ul[q] = e[q] >> dr.ushift;
		const uint32_t vw = vis_s[d[q] >> 5];
		const uint32_t fw = sl[ul[q] >> 5];
		cand |= (((~vw >> (d[q] & 31)) & (fw >> (ul[q] & 31))) & 1u) << q;
	}
	if (!active) cand = 0;
	if (!__any_sync(kFull, cand)) return 0;
	uint32_t claims = 0;
#pragma unroll
	for (int q = 0; q < 4; ++q) {
		if ((cand >> q) & 1u) {
			const uint32_t bit = 1u << (d[q] & 31);
			if (!(atomicOr(&vis_s[d[q] >> 5], bit) & bit)) {
				if (dr.parent) dr.parent[v0 + d[q]] = ubase + ul[q];
				++claims;
			}
		}
	}
	return claims;
}

// Per-warp sum of claims, taken off the group's count of unsettled vertices.
__device__ __forceinline__ void dense_settle(uint32_t claims) {
	claims = warp_sum(claims);
	if (lane_id() == 0 && claims) atomicSub(&dsh.unsettled, claims);
}

// Publishes the group's newly found vertices: next-frontier and visited bits,
// and the "stripe has a frontier vertex" flags of the next step.  Counts them
// and sums their out-degrees (for the direction switch) with coalesced reads
// of the row offsets: a lane per vertex, four bitmap words per warp in flight.
__device__ __forceinline__ void dense_group_publish(const DevGraph &g, const RunCtx &r, const DenseGroup &gr,
		const uint32_t *vis_s, const uint32_t *vis0_s, int32_t nl, uint32_t *nxt, uint8_t *sf_nxt, ThreadAcc &acc) {
	const unsigned lane = lane_id();
	const uint32_t v0 = (uint32_t) gr.v0, sw = g.sw;
	for (uint32_t j0 = warp_id() * 4; j0 < gr.gw; j0 += kWarps * 4) {
		uint32_t bits[4], deg[4];
#pragma unroll
		for (int q = 0; q < 4; ++q) {
			const uint32_t j = j0 + q;
			bits[q] = (j < gr.gw) ? (vis_s[j] & ~vis0_s[j]) : 0u;
			deg[q] = 0;
			if ((bits[q] >> lane) & 1u) {
				const uint32_t v = v0 + 32u * j + lane;
				deg[q] = __ldg(g.row_off + v + 1) - __ldg(g.row_off + v);
				r.level[v] = nl;
			}
		}
#pragma unroll
		for (int q = 0; q < 4; ++q) {
			acc.degsum += deg[q];
			if (lane == 0 && bits[q]) {
				const uint64_t vb = gr.v0 + 32ull * (j0 + q);
				acc.count += __popc(bits[q]);
				or_bits_at(nxt, vb, bits[q]);
				or_bits_at(r.vis, vb, bits[q]);
				if (sf_nxt) {
					// the stripes of the first and last new vertex of the word
					// (a word of 32 vertices spans at most two stripes when S*W >= 32)
					const uint32_t ka = (uint32_t) ((vb + (__ffs(bits[q]) - 1)) / sw);
					const uint32_t kb = (uint32_t) ((vb + (31 - __clz(bits[q]))) / sw);
					for (uint32_t k = ka; k <= kb; ++k)
						if (!ld_cg_u8(sf_nxt + k)) sf_nxt[k] = 1;
				}
			}
		}
	}
}

// Lists the group's non-empty segments in the active stripes [kb, kb+kThreads)
// in stripe order (the reference skips tiles whose row has no frontier vertex,
// bfs.cpp:274-277; here the unit is the stripe).  Returns the count.
__device__ __forceinline__ uint32_t dense_window(const DevGraph &g, const uint8_t *sf_cur, uint32_t gi, uint32_t kb,
		uint32_t *list_k, uint32_t *list_start, uint32_t *list_nw) {
	const unsigned tid = threadIdx.x, lane = lane_id(), wid = warp_id();
	const uint32_t k = kb + tid;
	bool act = false;
	uint32_t st = 0, nw = 0;
	if (k < g.num_stripes && ld_cg_u8(sf_cur + k)) {
		uint64_t j = (uint64_t) gi * g.num_stripes + k;
		st = __ldg(g.seg_off + j);
		nw = __ldg(g.seg_off + j + 1) - st;
		act = nw > 0;
	}
	unsigned bal = __ballot_sync(kFull, act);
	if (lane == 0) dsh.wcount[wid] = __popc(bal);
	__syncthreads();
	if (wid == 0) {
		uint32_t cnt = lane < kWarps ? dsh.wcount[lane] : 0u;
		uint32_t inc = warp_incl_scan(cnt);
		if (lane < kWarps) dsh.woff[lane] = inc - cnt;
		if (lane == 31) dsh.nlist = inc;
	}
	__syncthreads();
	if (act) {
		uint32_t pos = dsh.woff[wid] + __popc(bal & lanemask_lt());
		list_k[pos] = k;
		list_start[pos] = st;
		list_nw[pos] = nw;
	}
	__syncthreads();
	return dsh.nlist;
}

// Generic bottom-up step: slices staged with plain loads (any tile width).
__device__ __forceinline__ void phase_dense_generic(const DevGraph &g, const RunCtx &r, uint32_t step, uint32_t batch,
		uint32_t *smem, ThreadAcc &acc) {
	const uint32_t *cur = r.bm[(step + 2) % 3];
	uint32_t *nxt = r.bm[step % 3];
	const uint8_t *sf_cur = r.sf[(step + 2) % 3];
	uint8_t *sf_nxt = r.sf[step % 3];
	StepCounters *out = r.ctr + step % 3;
	const int32_t nl = (int32_t) step + 1;
	const unsigned tid = threadIdx.x;
	uint32_t *vis_s = smem;
	uint32_t *nxt_s = vis_s + g.max_group_words + 1;
	uint32_t *slices = nxt_s + g.max_group_words + 1;
	const DenseRegs dr = dense_regs(g, r);
	uint32_t *list_k = slices + (size_t) batch * g.slice_words;
	uint32_t *list_start = list_k + kThreads;
	uint32_t *list_nw = list_start + kThreads;
	DenseGroup gr;
	while (dense_group_begin(g, r, out, vis_s, nxt_s, gr)) {
		if (dsh.unsettled == 0) continue;
		if (tid == 0) acc.bu_groups++;
		bool done = false;
		for (uint32_t kb = 0; kb < g.num_stripes && !done; kb += kThreads) {
			const uint32_t nlist = dense_window(g, sf_cur, gr.gi, kb, list_k, list_start, list_nw);
			for (uint32_t b0 = 0; b0 < nlist; b0 += batch) {
				const uint32_t nb = min(batch, nlist - b0);
				if (tid == 0) {
					uint32_t a = 0;
					for (uint32_t j = 0; j < nb; ++j) { dsh.prefix[j] = a; a += list_nw[b0 + j] >> 2; }
					dsh.prefix[nb] = a;
				}
				for (uint32_t x = tid; x < nb * g.slice_words; x += kThreads) {
					uint32_t j = x / g.slice_words, wd = x - j * g.slice_words;
					uint64_t sb = (uint64_t) list_k[b0 + j] * g.sw;
					uint64_t se = min(sb + g.sw, (uint64_t) g.n);
					slices[x] = bits_at(cur, sb + 32ull * wd, se, 0u);
				}
				__syncthreads();
				const uint32_t total = dsh.prefix[nb];
				uint32_t claims = 0;
				// warp-uniform trip count: lanes past the end take part inactive
				for (uint32_t i0 = tid - lane_id(); i0 < total; i0 += kThreads) {
					const uint32_t i = i0 + lane_id();
					const bool act = i < total;
					uint32_t j = 0;
					while (act && j + 1 < nb && dsh.prefix[j + 1] <= i) ++j;
					const uint32_t *sl = slices + j * g.slice_words;
					const uint32_t kk = list_k[b0 + j];
					const uint4 x4 = act ? ldg_v4(g.packed + list_start[b0 + j] + 4ull * (i - dsh.prefix[j]))
					                     : make_uint4(0, 0, 0, 0);
					claims += dense_vec<false>(act, x4, dr, (uint32_t) gr.v0, vis_s, nxt_s, sl, kk * g.sw, nl);
				}
				dense_settle(claims);
				if (tid == 0) { acc.bu_words += 4ull * total; acc.bu_slices += nb; }
				__syncthreads();
				if (dsh.unsettled == 0) { done = true; break; }
			}
		}
		dense_group_publish(g, r, gr, vis_s, nxt_s, nl, nxt, sf_nxt, acc);
	}
}

// Producer side of the bulk-copy pipeline (lane 0 of warp 0): fills stage
// `st` with the next run of the window's segments -- consecutive list
// entries whose words are contiguous (group-major layout), spanning at most
// tma_batch stripes and kTmaEdgeWords words -- with ONE bulk copy for the
// edges and ONE for the frontier slices of stripes k_first..k_last, and arms
// the stage's "full" mbarrier with the exact byte count.  A stage with
// nent == 0 marks the end of the window.
struct TmaCursor {
	uint32_t li, lo;   // list entry and word offset inside it
};

__device__ __forceinline__ bool tma_issue(const DevGraph &g, const uint32_t *cur, uint32_t *smem_stages, uint32_t st,
		const uint32_t *list_k, const uint32_t *list_start, const uint32_t *list_nw, uint32_t nlist,
		TmaCursor &c, bool stop, ThreadAcc &acc) {
	const uint32_t stage_words = kTmaEdgeWords + g.tma_batch * g.slice_words;
	uint32_t *edges = smem_stages + (size_t) st * stage_words;
	uint32_t *slices = edges + kTmaEdgeWords;
	TmaMeta &mt = tma_meta[st];
	uint32_t nent = 0, used = 0;
	uint32_t src = 0, kfirst = 0, next_word = 0;
	while (!stop && nent < kMaxSliceBatch && c.li < nlist && used < kTmaEdgeWords) {
		const uint32_t k = list_k[c.li];
		const uint32_t w0 = list_start[c.li] + c.lo;
		if (nent == 0) {
			src = w0;
			kfirst = k;
		} else if (w0 != next_word || k - kfirst >= g.tma_batch) {
			break;  // not contiguous with the run, or its slice does not fit
		}
		const uint32_t take = min(list_nw[c.li] - c.lo, kTmaEdgeWords - used);
		mt.k[nent] = k;
		mt.pre[nent] = used >> 2;
		++nent;
		used += take;
		next_word = w0 + take;
		c.lo += take;
		if (c.lo == list_nw[c.li]) { c.li++; c.lo = 0; }
	}
	mt.nent = nent;
	mt.pre[nent] = used >> 2;
	mt.kfirst = kfirst;
	const uint32_t nslices = nent ? mt.k[nent - 1] - kfirst + 1 : 0;
	acc.bu_words += used;
	acc.bu_slices += nslices;
	mbar_arrive_expect_tx(&tma_bar[st], 4u * (used + nslices * g.slice_words));
	if (nent) {
		bulk_copy_g2s(edges, g.packed + src, 4u * used, &tma_bar[st]);
		bulk_copy_g2s(slices, cur + (size_t) kfirst * g.slice_words, 4u * nslices * g.slice_words, &tma_bar[st]);
	}
	return nent != 0;
}

__device__ void dense_tma_init() {
	if (threadIdx.x == 0) {
		for (uint32_t s = 0; s < kTmaStages; ++s) {
			mbar_init(&tma_bar[s], 1);
			mbar_init(&tma_empty[s], kWarps - 1);
		}
		dsh.seq = 0;
		dsh.fail = 0;
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
	}
	__syncthreads();
}

// Bottom-up step streaming each group's segments and the stripes' frontier
// slices into a ring of shared-memory stages with 1-D bulk copies (TMA).
// Warp 0 is the producer; warps 1.. consume: they wait on a stage's "full"
// barrier, test its edges and release the stage on its "empty" barrier, so
// no CTA-wide barrier separates batches.  Needs S*W to be a multiple of 128
// so that every slice starts on a 16-byte boundary.
__device__ __forceinline__ void phase_dense_tma(const DevGraph &g, const RunCtx &r, uint32_t step, uint32_t *smem, ThreadAcc &acc) {
	const uint32_t *cur = r.bm[(step + 2) % 3];
	uint32_t *nxt = r.bm[step % 3];
	const uint8_t *sf_cur = r.sf[(step + 2) % 3];
	uint8_t *sf_nxt = r.sf[step % 3];
	StepCounters *out = r.ctr + step % 3;
	const int32_t nl = (int32_t) step + 1;
	const unsigned tid = threadIdx.x, wid = warp_id(), lane = lane_id();
	const uint32_t stage_words = kTmaEdgeWords + g.tma_batch * g.slice_words;
	uint32_t *stages = smem;
	uint32_t *vis_s = stages + (size_t) kTmaStages * stage_words;
	uint32_t *nxt_s = vis_s + g.max_group_words + 1;
	uint32_t *list_k = nxt_s + g.max_group_words + 1;
	const DenseRegs dr = dense_regs(g, r);
	const bool pow2w = (g.w & (g.w - 1)) == 0;
	const uint32_t slice_words = g.slice_words;
	uint32_t *list_start = list_k + kThreads;
	uint32_t *list_nw = list_start + kThreads;
	constexpr uint32_t kConsumers = kThreads - 32;
	// The frontier bitmap was written by other CTAs through the generic
	// proxy; order those writes before this CTA's bulk copies read it.
	if (tid == 0) fence_proxy_async_global();
	DenseGroup gr;
	unsigned long long cyc[6] = {0, 0, 0, 0, 0, 0};
	long long t0 = clock64();
	while (dense_group_begin(g, r, out, vis_s, nxt_s, gr)) {
		{ long long t1 = clock64(); cyc[0] += t1 - t0; t0 = t1; }
		const uint32_t v0 = (uint32_t) gr.v0;
		if (dsh.unsettled == 0) continue;
		if (tid == 0) acc.bu_groups++;
		for (uint32_t kb = 0; kb < g.num_stripes; kb += kThreads) {
			if (dsh.unsettled == 0 || dsh.fail) break;
			const uint32_t seq0 = dsh.seq;  // read before the barriers inside dense_window
			const uint32_t nlist = dense_window(g, sf_cur, gr.gi, kb, list_k, list_start, list_nw);
			{ long long t1 = clock64(); cyc[1] += t1 - t0; t0 = t1; }
			if (nlist == 0) continue;
			if (wid == 0) {
				if (lane == 0) {
					TmaCursor c{0, 0};
					for (uint32_t t = seq0;; ++t) {
						const uint32_t st = t % kTmaStages;
						const long long w0 = clock64();
						if (t >= kTmaStages &&
								!mbar_wait_bounded(&tma_empty[st], ((t / kTmaStages) + 1) & 1u, r.err, 4000)) {
							dsh.fail = 1;
							break;
						}
						cyc[4] += clock64() - w0;
						fence_proxy_async_shared();
						const bool stop = *(volatile uint32_t *) &dsh.unsettled == 0;
						if (!tma_issue(g, cur, stages, st, list_k, list_start, list_nw, nlist, c, stop, acc)) {
							dsh.seq = t + 1;
							break;
						}
					}
				}
			} else {
				const uint32_t ct = tid - 32;
				for (uint32_t t = seq0;; ++t) {
					const uint32_t st = t % kTmaStages;
					const long long w0 = clock64();
					if (!mbar_wait_bounded(&tma_bar[st], (t / kTmaStages) & 1u, r.err)) {
						dsh.fail = 1;
						break;
					}
					const long long w1 = clock64();
					cyc[2] += w1 - w0;
					const TmaMeta &mt = tma_meta[st];
					const uint32_t nent = mt.nent;
					uint32_t claims = 0;
					const uint4 *edges4 = (const uint4 *) (stages + (size_t) st * stage_words);
					const uint32_t *slices = stages + (size_t) st * stage_words + kTmaEdgeWords;
					// Warp cw takes chunks of 32 consecutive vectors (one per lane);
					// a lane finds its entry (stripe) with a branch-free search over
					// the stage's few entries -- the lanes of a chunk mostly read the
					// same prefix words, which shared memory broadcasts.
					const uint32_t total = mt.pre[nent];
					const uint32_t cw = wid - 1;
					for (uint32_t c0 = cw * 32; c0 < total; c0 += (kWarps - 1) * 32) {
						const uint32_t i = c0 + lane;
						const bool act = i < total;
						uint32_t j = 0;
#pragma unroll
						for (uint32_t sp = kMaxSliceBatch / 2; sp >= 1; sp >>= 1)
							j += (j + sp < nent && mt.pre[j + sp] <= i) ? sp : 0u;
						const uint32_t kk = mt.k[j];
						const uint32_t *sl = slices + (size_t) (kk - mt.kfirst) * slice_words;
						const uint4 x4 = edges4[act ? i : 0];
						if (pow2w) claims += dense_vec<true>(act, x4, dr, v0, vis_s, nxt_s, sl, kk * dr.sw, nl);
						else claims += dense_vec<false>(act, x4, dr, v0, vis_s, nxt_s, sl, kk * dr.sw, nl);
					}
					dense_settle(claims);
					__syncwarp();
					cyc[3] += clock64() - w1;
					if (lane == 0) mbar_arrive(&tma_empty[st]);
					if (nent == 0) break;
				}
			}
			__syncthreads();
			t0 = clock64();
		}
		if (dsh.fail) break;
		dense_group_publish(g, r, gr, vis_s, nxt_s, nl, nxt, sf_nxt, acc);
		{ long long t1 = clock64(); cyc[5] += t1 - t0; t0 = t1; }
	}
	// thread 0 reports setup/window/publish and producer wait, warp 1 lane 0 the consumer side
	if (tid == 0) {
		atomicAdd(&r.stats->bu_cycles[0], cyc[0]);
		atomicAdd(&r.stats->bu_cycles[1], cyc[1]);
		atomicAdd(&r.stats->bu_cycles[4], cyc[4]);
		atomicAdd(&r.stats->bu_cycles[5], cyc[5]);
	}
	if (tid == 32) {
		atomicAdd(&r.stats->bu_cycles[2], cyc[2]);
		atomicAdd(&r.stats->bu_cycles[3], cyc[3]);
	}
}

// Bottom-up step as a pull over in-edge lists (the column's tiles sorted by
// destination): a CTA owns a column group with its visited bits in shared
// memory; every unvisited destination that has in-edges scans them in order
// and stops at the first source in the frontier (Beamer's bottom-up; the
// reference's dense step tests every edge of the active rows instead,
// apps/bfs_simd/bfs.cpp:194-217, with the same levels).  Pass 1 gives each
// destination one lane and its first kPullShort in-edges; destinations not
// settled by then go to a shared-memory queue that whole warps scan 32 edges
// at a time with a ballot to stop at the first hit.
constexpr uint32_t kPullShort = 4;
// Work items of a pull step: each column group in this many parts, handed
// out dynamically (whole groups left a few CTAs with most of the work: the
// early exit makes a group's cost depend on where its frontier sources are).
constexpr uint32_t kPullSplit = 4;

__device__ __forceinline__ bool frontier_bit(const uint32_t *cur, uint32_t u) {
	return (ld_cg(cur + (u >> 5)) >> (u & 31)) & 1u;
}

__device__ __forceinline__ void phase_pull(const DevGraph &g, const RunCtx &r, uint32_t step, uint32_t *smem,
		ThreadAcc &acc) {
	const uint32_t *cur = r.bm[(step + 2) % 3];
	uint32_t *nxt = r.bm[step % 3];
	StepCounters *out = r.ctr + step % 3;
	const int32_t nl = (int32_t) step + 1;
	const unsigned wid = warp_id(), lane = lane_id();
	const uint32_t mgw = g.max_group_words + 1;
	uint32_t *vis_s = smem;
	uint32_t *vis0_s = vis_s + mgw;
	uint32_t *hin_s = vis0_s + mgw;
	uint32_t *longq = hin_s + mgw;
	const uint32_t long_cap = g.pull_long_cap;
	uint32_t *parent = r.parent;
	DenseGroup gr;
	unsigned long long cyc[4] = {0, 0, 0, 0};
	long long t0 = clock64();
	bool first = true;
	while (dense_group_begin(g, r, out, vis_s, vis0_s, gr, hin_s, kPullSplit, first)) {
		first = false;
		{ long long t1 = clock64(); cyc[0] += t1 - t0; t0 = t1; }
		if (dsh.unsettled == 0) continue;
		if (threadIdx.x == 0) { acc.bu_groups++; dsh.nlist = 0; }
		__syncthreads();
		const uint32_t v0 = (uint32_t) gr.v0;
		uint32_t edges = 0, tested = 0;
		// Pass 1: a warp takes four bitmap words (a lane per destination in
		// each); the list offsets, the first in-edge and its frontier word of
		// all four destinations are loaded stage by stage, so a lane waits for
		// three round trips per four destinations, not per destination.
		for (uint32_t j0 = wid * 4; j0 < gr.gw; j0 += kWarps * 4) {
			uint32_t todo_w[4], beg[4], end[4], u[4];
			bool found[4];
#pragma unroll
			for (int q = 0; q < 4; ++q) {
				const uint32_t j = j0 + q;
				todo_w[q] = (j < gr.gw) ? (hin_s[j] & ~vis0_s[j]) : 0u;
				found[q] = false;
				beg[q] = end[q] = 0;
				if ((todo_w[q] >> lane) & 1u) {
					const uint32_t v = v0 + 32u * j + lane;
					beg[q] = __ldg(g.in_off + v);
					end[q] = __ldg(g.in_off + v + 1);
				}
			}
#pragma unroll
			for (int q = 0; q < 4; ++q) u[q] = (beg[q] < end[q]) ? __ldg(g.in_src + beg[q]) : 0u;
#pragma unroll
			for (int q = 0; q < 4; ++q) {
				if (beg[q] < end[q]) {
					++tested;
					++edges;
					found[q] = frontier_bit(cur, u[q]);
				}
			}
#pragma unroll
			for (int q = 0; q < 4; ++q) {
				if (beg[q] < end[q] && !found[q]) {
					// the next few in-edges, then the long queue
					const uint32_t v = v0 + 32u * (j0 + q) + lane;
					const uint32_t stop = min(end[q], beg[q] + kPullShort);
					uint32_t e = beg[q] + 1;
					for (; e < stop; ++e) {
						++edges;
						u[q] = __ldg(g.in_src + e);
						if (frontier_bit(cur, u[q])) { found[q] = true; break; }
					}
					if (!found[q] && e < end[q]) {
						const uint32_t pos = atomicAdd(&dsh.nlist, 1u);
						if (pos < long_cap) {
							longq[pos] = v;
						} else {
							// queue full: finish the scan here
							for (; e < end[q]; ++e) {
								++edges;
								u[q] = __ldg(g.in_src + e);
								if (frontier_bit(cur, u[q])) { found[q] = true; break; }
							}
						}
					}
				}
				if (found[q] && parent) parent[v0 + 32u * (j0 + q) + lane] = u[q];
				const uint32_t fmask = __ballot_sync(kFull, found[q]);
				if (lane == 0 && fmask) atomicOr(&vis_s[j0 + q], fmask);
			}
		}
		__syncthreads();
		{ long long t1 = clock64(); cyc[1] += t1 - t0; t0 = t1; }
		// Pass 2: a warp per remaining destination, 32 in-edges at a time.
		const uint32_t nlong = min(dsh.nlist, long_cap);
		for (uint32_t x = wid; x < nlong; x += kWarps) {
			const uint32_t v = longq[x];
			const uint32_t end = __ldg(g.in_off + v + 1);
			for (uint32_t e0 = __ldg(g.in_off + v) + kPullShort; e0 < end; e0 += 32) {
				const uint32_t e = e0 + lane;
				uint32_t u = 0;
				const bool hit = e < end && frontier_bit(cur, u = __ldg(g.in_src + e));
				const uint32_t hm = __ballot_sync(kFull, hit);
				if (hm) {
					const int first = __ffs(hm) - 1;
					if (lane == (unsigned) first) {
						if (parent) parent[v] = u;
						const uint32_t d = v - v0;
						atomicOr(&vis_s[d >> 5], 1u << (d & 31));
					}
					if (lane == 0) edges += (uint32_t) first + 1;
					break;
				}
				if (lane == 0) edges += min(32u, end - e0);
			}
		}
		acc.bu_words += edges;
		acc.bu_vertices += tested;
		__syncthreads();
		{ long long t1 = clock64(); cyc[2] += t1 - t0; t0 = t1; }
		dense_group_publish(g, r, gr, vis_s, vis0_s, nl, nxt, nullptr, acc);  // the pull reads no stripe flags
		{ long long t1 = clock64(); cyc[3] += t1 - t0; t0 = t1; }
	}
	if (threadIdx.x == 0)
		for (int i = 0; i < 4; ++i) atomicAdd(&r.stats->bu_cycles[i], cyc[i]);
}

__device__ __forceinline__ void phase_dense(const DevGraph &g, const RunCtx &r, const StepParams &p, uint32_t step,
		uint32_t batch, uint32_t *smem, ThreadAcc &acc) {
	if (p.bottom_up == 0) phase_pull(g, r, step, smem, acc);
	else if (g.tma) phase_dense_tma(g, r, step, smem, acc);
	else phase_dense_generic(g, r, step, batch, smem, acc);
}

// ---------------------------------------------------------------------------
// Step bookkeeping
// ---------------------------------------------------------------------------
__device__ __forceinline__ void clear_slot(const DevGraph &g, const RunCtx &r, uint32_t slot) {
	uint32_t *bm = r.bm[slot];
	uint8_t *sf = r.sf[slot];
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < g.bm_words; i += stride) bm[i] = 0;
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < g.num_stripes; i += stride) sf[i] = 0;
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		StepCounters *c = r.ctr + slot;
		c->tail[0] = c->tail[1] = c->tail[2] = 0;
		c->work = 0;
	}
}

// The step totals (vertices discovered, their out-degree sum) are written as
// one partial per CTA -- plain stores, no atomics on a shared cache line --
// and every CTA sums the partials after the grid barrier.
__device__ __forceinline__ unsigned long long *part_at(const RunCtx &r, uint32_t slot, uint32_t which) {
	return r.part + ((size_t) slot * 2 + which) * kMaxGrid;
}

__device__ __forceinline__ void flush_step(ThreadAcc &acc, const RunCtx &r, uint32_t slot) {
	__shared__ unsigned long long red[2][kWarps];
	const unsigned lane = lane_id(), wid = warp_id();
	const unsigned long long c = warp_sum(acc.count), d = warp_sum(acc.degsum);
	if (lane == 0) { red[0][wid] = c; red[1][wid] = d; }
	__syncthreads();
	if (threadIdx.x < 2) {
		unsigned long long t = 0;
		for (int w = 0; w < kWarps; ++w) t += red[threadIdx.x][w];
		part_at(r, slot, threadIdx.x)[blockIdx.x] = t;
	}
	__syncthreads();
	acc.count = 0;
	acc.degsum = 0;
}

// Sums the partials of `slot` over the grid (all threads call), and loads
// the slot's three queue tails in the same round trip.
__device__ __forceinline__ void step_totals(const RunCtx &r, uint32_t slot, uint32_t *count,
		unsigned long long *degsum, uint32_t (&tails)[3]) {
	// every thread loads at most a few partials (one L2 round trip), then a
	// block reduction; three threads load the tails (every thread loading
	// them put hundreds of thousands of requests on one hot line)
	__shared__ unsigned long long red[2][kWarps];
	__shared__ uint32_t s_tails[3];
	if (threadIdx.x < 3) s_tails[threadIdx.x] = __ldcg(&r.ctr[slot].tail[threadIdx.x]);
	unsigned long long c = 0, d = 0;
	const unsigned long long *pc = part_at(r, slot, 0), *pd = part_at(r, slot, 1);
	for (uint32_t i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
		c += __ldcg(pc + i);
		d += __ldcg(pd + i);
	}
	c = warp_sum(c);
	d = warp_sum(d);
	if (lane_id() == 0) { red[0][warp_id()] = c; red[1][warp_id()] = d; }
	__syncthreads();
	unsigned long long tc = 0, td = 0;
#pragma unroll
	for (int w = 0; w < kWarps; ++w) { tc += red[0][w]; td += red[1][w]; }
	*count = (uint32_t) tc;
	*degsum = td;
	tails[0] = s_tails[0];
	tails[1] = s_tails[1];
	tails[2] = s_tails[2];
	__syncthreads();
}

// Adds the CTA's counters to the run statistics (once per launch).
__device__ __forceinline__ void flush_stats(ThreadAcc &acc, DevStats *stats) {
	__shared__ unsigned long long red[6][kWarps];
	unsigned long long v[6] = {acc.td_edges, acc.td_vertices, acc.bu_words, acc.bu_slices, acc.bu_groups,
			acc.bu_vertices};
	const unsigned lane = lane_id(), wid = warp_id();
#pragma unroll
	for (int i = 0; i < 6; ++i) {
		unsigned long long x = warp_sum(v[i]);
		if (lane == 0) red[i][wid] = x;
	}
	__syncthreads();
	if (threadIdx.x < 6) {
		unsigned long long t = 0;
		for (int w = 0; w < kWarps; ++w) t += red[threadIdx.x][w];
		if (t) {
			switch (threadIdx.x) {
			case 0: atomicAdd(&stats->td_edges, t); break;
			case 1: atomicAdd(&stats->td_vertices, t); break;
			case 2: atomicAdd(&stats->bu_words, t); break;
			case 3: atomicAdd(&stats->bu_slices, t); break;
			case 4: atomicAdd(&stats->bu_groups, t); break;
			default: atomicAdd(&stats->bu_vertices, t); break;
			}
		}
	}
	__syncthreads();
	acc.td_edges = acc.td_vertices = acc.bu_words = acc.bu_slices = acc.bu_groups = acc.bu_vertices = 0;
}

__device__ void seed_source(const DevGraph &g, const RunCtx &r, const StepParams &p) {
	const uint32_t s = p.source;
	r.level[s] = 0;
	if (r.parent) r.parent[s] = s;
	atomicOr(r.vis + (s >> 5), 1u << (s & 31));
	uint32_t deg = g.row_off[s + 1] - g.row_off[s];
	uint32_t bk = bucket_of(deg, p);
	r.q[0][bk][0] = s;
	StepCounters *c = r.ctr + 2;  // the frontier "produced by step -1"
	c->tail[bk] = 1;
	part_at(r, 2, 0)[0] = 1;
	part_at(r, 2, 1)[0] = deg;
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
// Clears the run state and, when `seed`, seeds the source in the same
// writes (the values written at the source's indices are the seeded ones),
// so the traversal needs no seeding step.  Grid-strided over the launch.
// The barrier words and the status word are not touched: the persistent
// kernel leaves them zero when it exits.
__device__ __forceinline__ void init_run(const DevGraph &g, const RunCtx &r, const StepParams &p, bool seed) {
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	const uint64_t t0 = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x;
	const uint32_t s = p.source;
	for (uint64_t i = t0; i < g.n; i += stride) {
		const bool src = seed && i == s;
		r.level[i] = src ? 0 : -1;
		if (r.parent) r.parent[i] = src ? s : kUnvisitedWord;
	}
	for (uint64_t i = t0; i < g.nwords; i += stride) r.vis[i] = (seed && i == (s >> 5)) ? 1u << (s & 31) : 0u;
	for (uint64_t i = t0; i < g.bm_words; i += stride) {
		r.bm[0][i] = 0;
		r.bm[1][i] = 0;
		r.bm[2][i] = 0;
	}
	for (uint64_t i = t0; i < g.num_stripes; i += stride) { r.sf[0][i] = 0; r.sf[1][i] = 0; r.sf[2][i] = 0; }
	// the source is the frontier "produced by step -1": the queue bucket of
	// its out-degree, counter slot 2, CTA 0's partials of slot 2
	constexpr uint64_t kCtrWords = 3 * sizeof(StepCounters) / 4;
	uint32_t deg = 0, bk = 0;
	if (seed && t0 <= kCtrWords) {
		deg = __ldg(g.row_off + s + 1) - __ldg(g.row_off + s);
		bk = bucket_of(deg, p);
	}
	if (t0 < kCtrWords) {
		const uint64_t tail_idx = (2 * sizeof(StepCounters) + bk * sizeof(unsigned)) / 4;
		((uint32_t *) r.ctr)[t0] = (seed && t0 == tail_idx) ? 1u : 0u;
	}
	if (seed && t0 == kCtrWords) r.q[0][bk][0] = s;
	for (uint64_t i = t0; i < 6ull * kMaxGrid; i += stride) {
		unsigned long long x = 0;
		if (seed && i == (2 * 2 + 0) * (uint64_t) kMaxGrid) x = 1;
		if (seed && i == (2 * 2 + 1) * (uint64_t) kMaxGrid) x = __ldg(g.row_off + s + 1) - __ldg(g.row_off + s);
		r.part[i] = x;
	}
	for (uint64_t i = t0; i < sizeof(DevStats) / 4; i += stride) ((uint32_t *) r.stats)[i] = 0;
}

// The stepwise mode's clearing launch (the host loop seeds with k_seed).
__global__ void __launch_bounds__(kThreads) k_init(DevGraph g, RunCtx r, StepParams p) {
	init_run(g, r, p, false);
	const uint64_t t0 = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x;
	if (t0 < 2) r.bar[t0] = 0;
	if (t0 == 0) *r.err = 0;
}

__global__ void k_seed(DevGraph g, RunCtx r, StepParams p) {
	if (blockIdx.x == 0 && threadIdx.x == 0) seed_source(g, r, p);
}

// All steps of one traversal in one cooperative launch, the clearing of the
// run state and the seeding of the source included (one grid barrier after
// them).  The run statistics that only CTA 0 keeps are held in its
// registers and written once at the end, so CTA 0 (which every light step
// waits for) takes no extra round trips.  The grid barrier's arrival count,
// the exit count and the status word are zero when the launch starts: the
// last CTA to exit resets them.
__global__ void __launch_bounds__(kThreads, 2) k_bfs_persistent(DevGraph g, RunCtx r, StepParams p, uint32_t batch) {
	extern __shared__ __align__(128) uint32_t smem[];
	__shared__ uint32_t s_conv_tails[3];
	ThreadAcc acc{0, 0, 0, 0, 0, 0, 0, 0};
	bool ok = true;
	dense_tma_init();
	const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
	unsigned long long st_reached = 0, st_edges = 0;
	uint32_t st_dense = 0;
	unsigned epoch = 0;  // grid barriers this CTA has passed
	unsigned long long seen = 0;  // out-edges of the vertices reached so far (frontiers included)
	bool last_dense = false;
	uint32_t step = 0;
	CTA_STAMP(15, 0);  // profiling builds: the prologue in the slot of step 15
	init_run(g, r, p, true);
	CTA_STAMP(15, 1);
	ok = grid_sync(r.bar, epoch, r.err, p.wait_limit_ns, p.hold_barrier);
	CTA_STAMP(15, 2);
	for (; ok; ++step) {
		uint32_t fsize, tails[3];
		unsigned long long dsum;
		CTA_STAMP(step, 0);
		step_totals(r, (step + 2) % 3, &fsize, &dsum, tails);
		CTA_STAMP(step, 1);
		if (leader) {
			st_reached += fsize;
			st_edges += dsum;
			if (step < 257) r.stats->t_step[step] = global_timer_ns();
		}
		if (fsize == 0) break;
		seen += dsum;
		bool dense = false;
		if (step > 0) {
			if (p.switch_rule == 0) {
				unsigned long long thr = last_dense ? p.to_sparse_threshold : p.to_dense_threshold;
				dense = (unsigned long long) fsize + dsum > thr;
			} else {
				const unsigned long long unseen = g.m > seen ? g.m - seen : 0ull;
				dense = last_dense ? (unsigned long long) fsize * p.beta >= g.n : dsum * p.alpha > unseen;
			}
		}
		clear_slot(g, r, (step + 1) % 3);
		CTA_STAMP(step, 2);
		if (dense) {
			// the top-down step that produced this frontier also set its
			// bitmap; only the streaming variant needs the stripe flags built
			if (!last_dense && p.bottom_up != 0) {
				phase_to_dense(g, r, step, true);
				if (!(ok = grid_sync(r.bar, epoch, r.err, p.wait_limit_ns, p.hold_barrier))) break;
				if (leader && step < 256) r.stats->t_conv[step] = global_timer_ns();
			}
			CTA_STAMP(step, 3);
			phase_dense(g, r, p, step, batch, smem, acc);
		} else {
			if (last_dense) {
				phase_to_sparse(g, r, p, step);
				if (!(ok = grid_sync(r.bar, epoch, r.err, p.wait_limit_ns, p.hold_barrier))) break;
				if (leader && step < 256) r.stats->t_conv[step] = global_timer_ns();
				if (threadIdx.x < 3) s_conv_tails[threadIdx.x] = __ldcg(&r.ctr[(step + 2) % 3].tail[threadIdx.x]);
				__syncthreads();
				tails[0] = s_conv_tails[0];
				tails[1] = s_conv_tails[1];
				tails[2] = s_conv_tails[2];
			}
			CTA_STAMP(step, 3);
			phase_expand(g, r, p, step, tails[0], tails[1], tails[2], smem, acc);
		}
		CTA_STAMP(step, 4);
		flush_step(acc, r, step % 3);
		CTA_STAMP(step, 5);
		if (threadIdx.x == 0 && step < 256) {
			const unsigned long long t = global_timer_ns();
			atomicMax(&r.stats->t_work_max[step], t);
			atomicMax(&r.stats->t_work_min_inv[step], ~t);
		}
		if (leader) {
			if (step < 256) r.stats->trace[step] = dense ? 1 : 0;
			st_dense += dense;
		}
		last_dense = dense;
		ok = grid_sync(r.bar, epoch, r.err, p.wait_limit_ns, p.hold_barrier);
	}
	flush_stats(acc, r.stats);
	if (leader) {
		r.stats->reached = st_reached;
		r.stats->edges_traversed = st_edges;
		r.stats->dense_steps = st_dense;
		r.stats->num_steps = step;
		r.stats->status = *(volatile int *) r.err;
	}
	// the last CTA out resets the barrier and status words for the next launch
	// (every CTA has left every barrier and read the status by then)
	__syncthreads();
	if (threadIdx.x == 0) {
		__threadfence();
		if (atomicAdd(&r.bar[1], 1u) == gridDim.x - 1) {
			atomicExch(&r.bar[0], 0u);
			atomicExch(&r.bar[1], 0u);
			atomicExch(r.err, 0);
		}
	}
}

// Stepwise kernels: one phase per launch (the host decides the direction).
__global__ void __launch_bounds__(kThreads) k_step_clear(DevGraph g, RunCtx r, uint32_t step) {
	clear_slot(g, r, (step + 1) % 3);
}
__global__ void __launch_bounds__(kThreads) k_step_to_dense(DevGraph g, RunCtx r, StepParams p, uint32_t step) {
	phase_to_dense(g, r, step, p.bottom_up != 0);
}
__global__ void __launch_bounds__(kThreads) k_step_to_sparse(DevGraph g, RunCtx r, StepParams p, uint32_t step) {
	phase_to_sparse(g, r, p, step);
}
__global__ void __launch_bounds__(kThreads) k_step_expand(DevGraph g, RunCtx r, StepParams p, uint32_t step) {
	extern __shared__ __align__(128) uint32_t smem[];
	ThreadAcc acc{0, 0, 0, 0, 0, 0, 0, 0};
	const StepCounters *in = r.ctr + (step + 2) % 3;
	phase_expand(g, r, p, step, ld_volatile(&in->tail[0]), ld_volatile(&in->tail[1]), ld_volatile(&in->tail[2]),
			smem, acc);
	flush_step(acc, r, step % 3);
	flush_stats(acc, r.stats);
}
__global__ void __launch_bounds__(kThreads, 2) k_step_dense(DevGraph g, RunCtx r, StepParams p, uint32_t step,
		uint32_t batch) {
	extern __shared__ __align__(128) uint32_t smem[];
	ThreadAcc acc{0, 0, 0, 0, 0, 0, 0, 0};
	dense_tma_init();
	phase_dense(g, r, p, step, batch, smem, acc);
	flush_step(acc, r, step % 3);
	flush_stats(acc, r.stats);
}

// ---------------------------------------------------------------------------
// Host-side launchers
// ---------------------------------------------------------------------------
size_t dense_smem_bytes(const DevGraph &g, uint32_t batch) {
	size_t words = (size_t) 2 * (g.max_group_words + 1) + 3 * kThreads;
	if (g.tma) words += (size_t) kTmaStages * (kTmaEdgeWords + (size_t) g.tma_batch * g.slice_words);
	else words += (size_t) batch * g.slice_words;
	const size_t pull = (size_t) 3 * (g.max_group_words + 1) + g.pull_long_cap;
	const size_t expand = (size_t) kWarps * 3 * kWqCap + 3 * (size_t) kFlatChunk;
	size_t need = words > pull ? words : pull;
	need = need > expand ? need : expand;
	return sizeof(uint32_t) * need;
}

int persistent_grid(const DevGraph &g, uint32_t batch, int num_sms, int *grid, size_t *smem) {
	*smem = dense_smem_bytes(g, batch);
	if (cudaFuncSetAttribute(k_bfs_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) *smem) != cudaSuccess)
		return BFS_ECUDA;
	if (cudaFuncSetAttribute(k_step_dense, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) *smem) != cudaSuccess)
		return BFS_ECUDA;
	if (cudaFuncSetAttribute(k_step_expand, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) *smem) != cudaSuccess)
		return BFS_ECUDA;
	int per_sm = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bfs_persistent, kThreads, *smem) != cudaSuccess)
		return BFS_ECUDA;
	if (per_sm < 1) return BFS_EUNSUPPORTED;
	if (per_sm > 2) per_sm = 2;
	*grid = per_sm * num_sms;
	return BFS_OK;
}

int launch_init(const DevGraph &g, const RunCtx &r, cudaStream_t st, int num_sms) {
	StepParams p{};
	k_init<<<num_sms * 4, kThreads, 0, st>>>(g, r, p);
	return cudaGetLastError() == cudaSuccess ? BFS_OK : BFS_ECUDA;
}

int launch_persistent(const DevGraph &g, const RunCtx &r, const StepParams &p, uint32_t batch, int grid,
		size_t smem, cudaStream_t st) {
	DevGraph gg = g;
	RunCtx rr = r;
	StepParams pp = p;
	uint32_t bb = batch;
	void *args[] = {&gg, &rr, &pp, &bb};
	cudaError_t e = cudaLaunchCooperativeKernel((const void *) k_bfs_persistent, dim3(grid), dim3(kThreads), args, smem, st);
	return e == cudaSuccess ? BFS_OK : BFS_ECUDA;
}

int launch_step(int kind, const DevGraph &g, const RunCtx &r, const StepParams &p, uint32_t step, uint32_t batch,
		int grid, size_t smem, cudaStream_t st) {
	switch (kind) {
	case kStepSeed: k_seed<<<1, 32, 0, st>>>(g, r, p); break;
	case kStepClear: k_step_clear<<<grid, kThreads, 0, st>>>(g, r, step); break;
	case kStepToDense: k_step_to_dense<<<grid, kThreads, 0, st>>>(g, r, p, step); break;
	case kStepToSparse: k_step_to_sparse<<<grid, kThreads, 0, st>>>(g, r, p, step); break;
	case kStepExpand: k_step_expand<<<grid, kThreads, smem, st>>>(g, r, p, step); break;
	case kStepDense: k_step_dense<<<grid, kThreads, smem, st>>>(g, r, p, step, batch); break;
	default: return BFS_EARG;
	}
	return cudaGetLastError() == cudaSuccess ? BFS_OK : BFS_ECUDA;
}

int kernel_threads() { return kThreads; }

#ifdef BFS_CTA_TIMERS
extern "C" int bfs_debug_cta_profile(unsigned long long *host) {
	return cudaMemcpyFromSymbol(host, g_cta_prof, sizeof(g_cta_prof)) == cudaSuccess ? 0 : BFS_ECUDA;
}
#endif

} // namespace bfsg
