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

struct ThreadAcc {
	unsigned long long count, degsum, td_edges, td_vertices, bu_words, bu_slices, bu_groups;
};

__device__ __forceinline__ uint32_t bucket_of(uint32_t deg, const StepParams &p) {
	return deg <= p.warp_max_degree ? 0u : (deg <= p.cta_max_degree ? 1u : 2u);
}

__device__ __forceinline__ bool try_claim(uint32_t *vis, uint32_t v) {
	uint32_t bit = 1u << (v & 31);
	uint32_t *w = vis + (v >> 5);
	if (ld_cg(w) & bit) return false;
	return !(atomicOr(w, bit) & bit);
}

// All 32 lanes of the warp call this with one candidate edge u->v each.
__device__ __forceinline__ void visit_and_append(bool has, uint32_t u, uint32_t v, int32_t next_level,
		const DevGraph &g, const RunCtx &r, uint32_t *const *qn, unsigned *tails,
		const StepParams &p, ThreadAcc &acc) {
	bool claimed = false;
	uint32_t deg = 0;
	if (has && try_claim(r.vis, v)) {
		claimed = true;
		r.level[v] = next_level;
		if (r.parent) r.parent[v] = u;
		deg = __ldg(g.row_off + v + 1) - __ldg(g.row_off + v);
		acc.count++;
		acc.degsum += deg;
	}
	if (!__ballot_sync(kFull, claimed)) return;
	const uint32_t b = bucket_of(deg, p);
#pragma unroll
	for (uint32_t bk = 0; bk < 3; ++bk) {
		unsigned mask = __ballot_sync(kFull, claimed && b == bk);
		if (!mask) continue;
		int leader = __ffs(mask) - 1;
		unsigned base = 0;
		if (lane_id() == (unsigned) leader) base = atomicAdd(&tails[bk], (unsigned) __popc(mask));
		base = __shfl_sync(kFull, base, leader);
		if (claimed && b == bk) qn[bk][base + __popc(mask & lanemask_lt())] = v;
	}
}

// ---------------------------------------------------------------------------
// Top-down step (BFS_kernel_sparse + update_sparse, apps/bfs_simd/bfs.cpp:467-711)
// ---------------------------------------------------------------------------
__device__ void phase_expand(const DevGraph &g, const RunCtx &r, const StepParams &p, uint32_t step,
		ThreadAcc &acc) {
	const uint32_t cur = step & 1, nxt = (step + 1) & 1;
	const StepCounters *in = r.ctr + (step + 2) % 3;
	StepCounters *out = r.ctr + step % 3;
	const uint32_t nS = ld_volatile(&in->tail[0]);
	const uint32_t nM = ld_volatile(&in->tail[1]);
	const uint32_t nL = ld_volatile(&in->tail[2]);
	const uint32_t *qS = r.q[cur][0], *qM = r.q[cur][1], *qL = r.q[cur][2];
	uint32_t *const qn[3] = {r.q[nxt][0], r.q[nxt][1], r.q[nxt][2]};
	unsigned *tails = out->tail;
	const int32_t nl = (int32_t) step + 1;
	const unsigned lane = lane_id(), wid = warp_id();
	const uint64_t gwarp = (uint64_t) blockIdx.x * kWarps + wid;
	const uint64_t nwarps = (uint64_t) gridDim.x * kWarps;

	// Large out-degree: every warp of the grid takes a strided share of the edges.
	for (uint32_t i = 0; i < nL; ++i) {
		uint32_t u = ld_cg(qL + i);
		uint32_t beg = __ldg(g.row_off + u), end = __ldg(g.row_off + u + 1);
		for (uint64_t e0 = beg + gwarp * 32; e0 < end; e0 += nwarps * 32) {
			uint64_t e = e0 + lane;
			bool has = e < end;
			uint32_t v = has ? __ldg(g.col + e) : 0u;
			visit_and_append(has, u, v, nl, g, r, qn, tails, p, acc);
		}
		if (blockIdx.x == 0 && threadIdx.x == 0) { acc.td_edges += end - beg; acc.td_vertices++; }
	}
	// Medium out-degree: one CTA per vertex.
	for (uint32_t i = blockIdx.x; i < nM; i += gridDim.x) {
		uint32_t u = ld_cg(qM + i);
		uint32_t beg = __ldg(g.row_off + u), end = __ldg(g.row_off + u + 1);
		for (uint64_t e0 = beg + (uint64_t) wid * 32; e0 < end; e0 += kThreads) {
			uint64_t e = e0 + lane;
			bool has = e < end;
			uint32_t v = has ? __ldg(g.col + e) : 0u;
			visit_and_append(has, u, v, nl, g, r, qn, tails, p, acc);
		}
		if (threadIdx.x == 0) { acc.td_edges += end - beg; acc.td_vertices++; }
	}
	// Small out-degree: one warp expands 32 vertices together.
	for (uint64_t base = gwarp * 32; base < nS; base += nwarps * 32) {
		uint64_t i = base + lane;
		bool valid = i < nS;
		uint32_t u = valid ? ld_cg(qS + i) : 0u;
		uint32_t beg = valid ? __ldg(g.row_off + u) : 0u;
		uint32_t deg = valid ? __ldg(g.row_off + u + 1) - beg : 0u;
		uint32_t incl = warp_incl_scan(deg);
		uint32_t total = __shfl_sync(kFull, incl, 31);
		uint32_t excl = incl - deg;
		for (uint32_t f0 = 0; f0 < total; f0 += 32) {
			uint32_t f = f0 + lane;
			bool has = f < total;
			// owner = number of lanes whose inclusive degree sum is <= f
			int lo = 0;
#pragma unroll
			for (int st = 16; st >= 1; st >>= 1) {
				uint32_t val = __shfl_sync(kFull, incl, lo + st - 1);
				if (val <= f) lo += st;
			}
			uint32_t ou = __shfl_sync(kFull, u, lo);
			uint32_t ob = __shfl_sync(kFull, beg, lo);
			uint32_t oe = __shfl_sync(kFull, excl, lo);
			uint32_t v = has ? __ldg(g.col + ob + (f - oe)) : 0u;
			visit_and_append(has, ou, v, nl, g, r, qn, tails, p, acc);
		}
		const unsigned nvalid = (unsigned) __popc(__ballot_sync(kFull, valid));
		if (lane == 0) {
			acc.td_edges += total;
			acc.td_vertices += nvalid;
		}
	}
}

// ---------------------------------------------------------------------------
// Queue -> bitmap (to_dense, apps/bfs_simd/bfs.cpp:54-88)
// ---------------------------------------------------------------------------
__device__ void phase_to_dense(const DevGraph &g, const RunCtx &r, uint32_t step) {
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
		sf[v / g.sw] = 1;
	}
}

// ---------------------------------------------------------------------------
// Bitmap -> queue (to_sparse, apps/bfs_simd/bfs.cpp:400-465)
// ---------------------------------------------------------------------------
__device__ void phase_to_sparse(const DevGraph &g, const RunCtx &r, const StepParams &p, uint32_t step) {
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
	uint32_t group, unsettled, nlist, pad;
	uint32_t wcount[kWarps], woff[kWarps];
	uint32_t prefix[kMaxSliceBatch + 1];
};

__device__ void phase_dense(const DevGraph &g, const RunCtx &r, uint32_t step, uint32_t batch,
		uint32_t *smem, ThreadAcc &acc) {
	__shared__ DenseShared sh;
	const uint32_t *cur = r.bm[(step + 2) % 3];
	uint32_t *nxt = r.bm[step % 3];
	const uint8_t *sf_cur = r.sf[(step + 2) % 3];
	uint8_t *sf_nxt = r.sf[step % 3];
	StepCounters *out = r.ctr + step % 3;
	const int32_t nl = (int32_t) step + 1;
	const unsigned tid = threadIdx.x, lane = lane_id(), wid = warp_id();

	uint32_t *vis_s = smem;
	uint32_t *nxt_s = vis_s + g.max_group_words;
	uint32_t *slices = nxt_s + g.max_group_words;
	uint32_t *list_k = slices + (size_t) batch * g.slice_words;
	uint32_t *list_start = list_k + kThreads;
	uint32_t *list_nvec = list_start + kThreads;

	const uint32_t w = g.w, vbits = g.vbits, vmask = g.vmask, cmask = g.cmask, ushift = g.ushift;

	for (;;) {
		__syncthreads();
		if (tid == 0) sh.group = atomicAdd(&out->work, 1u);
		__syncthreads();
		const uint32_t gi = sh.group;
		if (gi >= g.num_groups) break;
		const uint32_t c0 = __ldg(g.group_col + gi), c1 = __ldg(g.group_col + gi + 1);
		const uint64_t v0 = (uint64_t) c0 * w;
		const uint64_t v1 = min((uint64_t) c1 * w, (uint64_t) g.n);
		const uint32_t gw = (uint32_t) ((v1 - v0 + 31) / 32);
		if (tid == 0) sh.unsettled = 0;
		__syncthreads();
		uint32_t uns = 0;
		for (uint32_t j = tid; j < gw; j += kThreads) {
			uint32_t vb = bits_at(r.vis, v0 + 32ull * j, v1, kFull);
			uint32_t hb = bits_at(g.hasin, v0 + 32ull * j, v1, 0u);
			vis_s[j] = vb;
			nxt_s[j] = 0;
			uns += __popc(hb & ~vb);
		}
		uns = warp_sum(uns);
		if (lane == 0 && uns) atomicAdd(&sh.unsettled, uns);
		__syncthreads();
		if (sh.unsettled == 0) continue;
		if (tid == 0) acc.bu_groups++;

		bool done = false;
		for (uint32_t kb = 0; kb < g.num_stripes && !done; kb += kThreads) {
			// Active, non-empty segments of this group in stripes [kb, kb+kThreads).
			const uint32_t k = kb + tid;
			bool act = false;
			uint32_t st = 0, nvec = 0;
			if (k < g.num_stripes && ld_cg_u8(sf_cur + k)) {
				uint64_t j = (uint64_t) k * g.num_groups + gi;
				st = __ldg(g.seg_off + j);
				nvec = (__ldg(g.seg_off + j + 1) - st) >> 2;
				act = nvec > 0;
			}
			unsigned bal = __ballot_sync(kFull, act);
			if (lane == 0) sh.wcount[wid] = __popc(bal);
			__syncthreads();
			if (wid == 0) {
				uint32_t cnt = lane < kWarps ? sh.wcount[lane] : 0u;
				uint32_t inc = warp_incl_scan(cnt);
				if (lane < kWarps) sh.woff[lane] = inc - cnt;
				if (lane == 31) sh.nlist = inc;
			}
			__syncthreads();
			if (act) {
				uint32_t pos = sh.woff[wid] + __popc(bal & lanemask_lt());
				list_k[pos] = k;
				list_start[pos] = st;
				list_nvec[pos] = nvec;
			}
			__syncthreads();
			const uint32_t nlist = sh.nlist;
			for (uint32_t b0 = 0; b0 < nlist; b0 += batch) {
				const uint32_t nb = min(batch, nlist - b0);
				if (tid == 0) {
					uint32_t a = 0;
					for (uint32_t j = 0; j < nb; ++j) { sh.prefix[j] = a; a += list_nvec[b0 + j]; }
					sh.prefix[nb] = a;
				}
				// Stage the frontier slices of the nb stripes.
				for (uint32_t x = tid; x < nb * g.slice_words; x += kThreads) {
					uint32_t j = x / g.slice_words, wd = x - j * g.slice_words;
					uint64_t sb = (uint64_t) list_k[b0 + j] * g.sw;
					uint64_t se = min(sb + g.sw, (uint64_t) g.n);
					slices[x] = bits_at(cur, sb + 32ull * wd, se, 0u);
				}
				__syncthreads();
				const uint32_t total = sh.prefix[nb];
				for (uint32_t i = tid; i < total; i += kThreads) {
					uint32_t j = 0;
					while (j + 1 < nb && sh.prefix[j + 1] <= i) ++j;
					const uint32_t *sl = slices + j * g.slice_words;
					const uint32_t kk = list_k[b0 + j];
					uint4 x4 = ldg_v4(g.packed + list_start[b0 + j] + 4ull * (i - sh.prefix[j]));
					uint32_t wv[4] = {x4.x, x4.y, x4.z, x4.w};
#pragma unroll
					for (int q = 0; q < 4; ++q) {
						uint32_t e = wv[q];
						if (e == kSentinelWord) continue;
						uint32_t d = ((e >> vbits) & cmask) * w + (e & vmask);
						uint32_t bit = 1u << (d & 31);
						if (vis_s[d >> 5] & bit) continue;           // destination already found
						uint32_t ul = e >> ushift;
						if (!((sl[ul >> 5] >> (ul & 31)) & 1u)) continue; // source not in the frontier
						if (atomicOr(&vis_s[d >> 5], bit) & bit) continue;
						atomicOr(&nxt_s[d >> 5], bit);
						uint32_t v = (uint32_t) (v0 + d);
						r.level[v] = nl;
						if (r.parent) r.parent[v] = kk * g.sw + ul;
						uint32_t deg = __ldg(g.row_off + v + 1) - __ldg(g.row_off + v);
						acc.count++;
						acc.degsum += deg;
						atomicSub(&sh.unsettled, 1u);
					}
				}
				if (tid == 0) { acc.bu_words += 4ull * total; acc.bu_slices += nb; }
				__syncthreads();
				if (sh.unsettled == 0) { done = true; break; }
			}
		}
		// Publish the group's new frontier and visited bits.
		for (uint32_t j = tid; j < gw; j += kThreads) {
			uint32_t bits = nxt_s[j];
			if (!bits) continue;
			uint64_t vb = v0 + 32ull * j;
			or_bits_at(nxt, vb, bits);
			or_bits_at(r.vis, vb, bits);
			uint64_t kf = (vb + (__ffs(bits) - 1)) / g.sw, kl = (vb + (31 - __clz(bits))) / g.sw;
			for (uint64_t k = kf; k <= kl; ++k) sf_nxt[k] = 1;
		}
	}
}

// ---------------------------------------------------------------------------
// Step bookkeeping
// ---------------------------------------------------------------------------
__device__ void clear_slot(const DevGraph &g, const RunCtx &r, uint32_t slot) {
	uint32_t *bm = r.bm[slot];
	uint8_t *sf = r.sf[slot];
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < g.nwords; i += stride) bm[i] = 0;
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < g.num_stripes; i += stride) sf[i] = 0;
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		StepCounters *c = r.ctr + slot;
		c->tail[0] = c->tail[1] = c->tail[2] = 0;
		c->count = 0;
		c->degsum = 0;
		c->work = 0;
	}
}

// Adds the CTA's accumulated counts to the step slot and the run statistics.
__device__ void flush_acc(ThreadAcc &acc, StepCounters *slot, DevStats *stats) {
	__shared__ unsigned long long red[7][kWarps];
	unsigned long long v[7] = {acc.count, acc.degsum, acc.td_edges, acc.td_vertices, acc.bu_words, acc.bu_slices, acc.bu_groups};
	const unsigned lane = lane_id(), wid = warp_id();
#pragma unroll
	for (int i = 0; i < 7; ++i) {
		unsigned long long x = warp_sum(v[i]);
		if (lane == 0) red[i][wid] = x;
	}
	__syncthreads();
	if (threadIdx.x < 7) {
		unsigned long long s = 0;
		for (int wv = 0; wv < kWarps; ++wv) s += red[threadIdx.x][wv];
		if (s) {
			switch (threadIdx.x) {
			case 0: atomicAdd(&slot->count, (unsigned) s); break;
			case 1: atomicAdd(&slot->degsum, s); break;
			case 2: atomicAdd(&stats->td_edges, s); break;
			case 3: atomicAdd(&stats->td_vertices, s); break;
			case 4: atomicAdd(&stats->bu_words, s); break;
			case 5: atomicAdd(&stats->bu_slices, s); break;
			default: atomicAdd(&stats->bu_groups, s); break;
			}
		}
	}
	__syncthreads();
	acc = ThreadAcc{0, 0, 0, 0, 0, 0, 0};
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
	c->count = 1;
	c->degsum = deg;
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_init(DevGraph g, RunCtx r) {
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	const uint64_t t0 = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x;
	for (uint64_t i = t0; i < g.n; i += stride) {
		r.level[i] = -1;
		if (r.parent) r.parent[i] = kUnvisitedWord;
	}
	for (uint64_t i = t0; i < g.nwords; i += stride) {
		r.vis[i] = 0;
		r.bm[0][i] = 0;
		r.bm[1][i] = 0;
		r.bm[2][i] = 0;
	}
	for (uint64_t i = t0; i < g.num_stripes; i += stride) { r.sf[0][i] = 0; r.sf[1][i] = 0; r.sf[2][i] = 0; }
	if (t0 < 3 * sizeof(StepCounters) / 4) ((uint32_t *) r.ctr)[t0] = 0;
	if (t0 < sizeof(DevStats) / 4) ((uint32_t *) r.stats)[t0] = 0;
	if (t0 < 2) r.bar[t0] = 0;
	if (t0 == 0) *r.err = 0;
}

__global__ void k_seed(DevGraph g, RunCtx r, StepParams p) {
	if (blockIdx.x == 0 && threadIdx.x == 0) seed_source(g, r, p);
}

__global__ void __launch_bounds__(kThreads, 2) k_bfs_persistent(DevGraph g, RunCtx r, StepParams p, uint32_t batch) {
	extern __shared__ uint32_t smem[];
	ThreadAcc acc{0, 0, 0, 0, 0, 0, 0};
	bool ok = true;
	if (blockIdx.x == 0 && threadIdx.x == 0) seed_source(g, r, p);
	ok = grid_barrier(r.bar, r.err);
	bool last_dense = false;
	uint32_t step = 0;
	for (; ok; ++step) {
		const StepCounters *in = r.ctr + (step + 2) % 3;
		const uint32_t fsize = ld_volatile(&in->count);
		const unsigned long long dsum = ld_volatile_u64(&in->degsum);
		if (blockIdx.x == 0 && threadIdx.x == 0) {
			r.stats->reached += fsize;
			r.stats->edges_traversed += dsum;
		}
		if (fsize == 0) break;
		bool dense = false;
		if (step > 0) {
			unsigned long long thr = last_dense ? p.to_sparse_threshold : p.to_dense_threshold;
			dense = (unsigned long long) fsize + dsum > thr;
		}
		clear_slot(g, r, (step + 1) % 3);
		if (dense) {
			if (!last_dense) {
				phase_to_dense(g, r, step);
				if (!(ok = grid_barrier(r.bar, r.err))) break;
			}
			phase_dense(g, r, step, batch, smem, acc);
		} else {
			if (last_dense) {
				phase_to_sparse(g, r, p, step);
				if (!(ok = grid_barrier(r.bar, r.err))) break;
			}
			phase_expand(g, r, p, step, acc);
		}
		flush_acc(acc, r.ctr + step % 3, r.stats);
		if (blockIdx.x == 0 && threadIdx.x == 0) {
			if (step < 256) r.stats->trace[step] = dense ? 1 : 0;
			if (dense) r.stats->dense_steps++;
		}
		last_dense = dense;
		ok = grid_barrier(r.bar, r.err);
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		r.stats->num_steps = step;
		r.stats->status = *(volatile int *) r.err;
	}
}

// Stepwise kernels: one phase per launch (the host decides the direction).
__global__ void __launch_bounds__(kThreads) k_step_clear(DevGraph g, RunCtx r, uint32_t step) {
	clear_slot(g, r, (step + 1) % 3);
}
__global__ void __launch_bounds__(kThreads) k_step_to_dense(DevGraph g, RunCtx r, uint32_t step) {
	phase_to_dense(g, r, step);
}
__global__ void __launch_bounds__(kThreads) k_step_to_sparse(DevGraph g, RunCtx r, StepParams p, uint32_t step) {
	phase_to_sparse(g, r, p, step);
}
__global__ void __launch_bounds__(kThreads) k_step_expand(DevGraph g, RunCtx r, StepParams p, uint32_t step) {
	ThreadAcc acc{0, 0, 0, 0, 0, 0, 0};
	phase_expand(g, r, p, step, acc);
	flush_acc(acc, r.ctr + step % 3, r.stats);
}
__global__ void __launch_bounds__(kThreads, 2) k_step_dense(DevGraph g, RunCtx r, uint32_t step, uint32_t batch) {
	extern __shared__ uint32_t smem[];
	ThreadAcc acc{0, 0, 0, 0, 0, 0, 0};
	phase_dense(g, r, step, batch, smem, acc);
	flush_acc(acc, r.ctr + step % 3, r.stats);
}

// ---------------------------------------------------------------------------
// Host-side launchers
// ---------------------------------------------------------------------------
size_t dense_smem_bytes(const DevGraph &g, uint32_t batch) {
	return sizeof(uint32_t) * ((size_t) 2 * g.max_group_words + (size_t) batch * g.slice_words + 3 * kThreads);
}

int persistent_grid(const DevGraph &g, uint32_t batch, int num_sms, int *grid, size_t *smem) {
	*smem = dense_smem_bytes(g, batch);
	if (cudaFuncSetAttribute(k_bfs_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) *smem) != cudaSuccess)
		return BFS_ECUDA;
	if (cudaFuncSetAttribute(k_step_dense, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) *smem) != cudaSuccess)
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
	k_init<<<num_sms * 4, kThreads, 0, st>>>(g, r);
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
	case kStepToDense: k_step_to_dense<<<grid, kThreads, 0, st>>>(g, r, step); break;
	case kStepToSparse: k_step_to_sparse<<<grid, kThreads, 0, st>>>(g, r, p, step); break;
	case kStepExpand: k_step_expand<<<grid, kThreads, 0, st>>>(g, r, p, step); break;
	case kStepDense: k_step_dense<<<grid, kThreads, smem, st>>>(g, r, step, batch); break;
	default: return BFS_EARG;
	}
	return cudaGetLastError() == cudaSuccess ? BFS_OK : BFS_ECUDA;
}

int kernel_threads() { return kThreads; }

} // namespace bfsg
