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
//   pmask[p][v]        bit k: word k of v's row in plane p is non-zero (the
//                      frontier's vertex set, and which words to read)
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
// Clearing, seeding, all levels and the edge count run in one cooperative
// launch, levels separated by a bounded-spin grid barrier; the output pass,
// its own launch, turns planes into uint8 levels [source][vertex] (255 =
// unreached) through a shared-memory transpose.  When a traversal is
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
constexpr uint32_t kLaneMaxWords = 2;   // pull: up to this many words per vertex ...
constexpr uint32_t kLaneMaxDeg = 32;    // ... destinations of at most this in-degree go one per lane
constexpr uint32_t kGroupMaxWords = 8;  // pull: up to this many words, in-neighbour rows in lane groups
constexpr uint32_t kEmitW = 4;          // output tile: kV vertices x 4 words (256 sources), kV = threads / 4
// shared bytes of an output tile of kV vertices: rows of one source quad (kV + 4
// words, 16-byte aligned; `bufs` copies) and the nibble table
__host__ __device__ constexpr uint32_t emit_bytes(uint32_t kV, uint32_t bufs = 1) {
	return (bufs * kEmitW * 16 * (kV + 4) + 16) * 4;
}
constexpr uint32_t kEmitV = kMsThreads / kEmitW;  // the traversal kernel's tiles (its early output passes)
constexpr uint32_t kEmitBytes = emit_bytes(kEmitV);
// The output pass launch: tiles of 64 vertices (256 threads, 4 CTAs per SM)
// or 128 vertices (512 threads, 2 per SM); by default the wide tiles from
// kEmitWideMinVertices vertices (measured: 64 wins on 2^22 vertices, 128 on
// 4.2e7, where the half-line row pieces of narrow tiles cost more)
constexpr uint32_t kEmitWideMinVertices = 1u << 24;

__device__ __forceinline__ uint64_t ld_cg64(const uint64_t *p) { return __ldcg((const unsigned long long *) p); }
__device__ __forceinline__ uint64_t shfl64(uint64_t x, int src) {
	return (uint64_t) __shfl_sync(kFull, (unsigned long long) x, src);
}
__device__ __forceinline__ uint64_t shfl_xor64(uint64_t x, int mask) {
	return (uint64_t) __shfl_xor_sync(kFull, (unsigned long long) x, mask);
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

// Push level, CTA 0: cuts the high-degree frontier vertices (the queue's back)
// into kMsPushChunk-edge chunks, listed in push_u / push_beg, so that warps
// all over the grid take them like small vertices.  A block-wide scan of the
// chunk counts, 512 vertices at a time.
__device__ void ms_push_chunk_list(const MsArgs &a, uint32_t lvl, uint32_t nb, uint32_t *scan_s) {
	const uint32_t *q = a.queue[lvl & 1];
	uint32_t running = 0;
	for (uint32_t base = 0; base < nb; base += blockDim.x) {
		const uint32_t i = base + threadIdx.x;
		uint32_t u = 0, c = 0, beg = 0, end = 0;
		if (i < nb) {
			u = ld_cg(q + a.n - 1 - i);
			beg = __ldg(a.row_off + u);
			end = __ldg(a.row_off + u + 1);
			c = (end - beg + kMsPushChunk - 1) / kMsPushChunk;
		}
		const uint32_t incl = warp_incl_scan(c);
		if (lane_id() == 31) scan_s[warp_id()] = incl;
		__syncthreads();
		uint32_t before = 0, total = 0;
		for (int w = 0; w < kMsWarps; ++w) {
			const uint32_t t = scan_s[w];
			if (w < (int) warp_id()) before += t;
			total += t;
		}
		uint32_t pos = running + before + incl - c;
		for (uint32_t k = 0; k < c && pos < a.push_cap; ++k, ++pos) {
			a.push_u[pos] = u;
			a.push_beg[pos] = beg + k * kMsPushChunk;
		}
		running += total;
		__syncthreads();
	}
	if (threadIdx.x == 0) a.ctl->push_chunks = min(running, a.push_cap);
}

__device__ void ms_push(const MsArgs &a, uint32_t lvl, const uint64_t *cur, const uint64_t *actc, uint64_t *nxt, uint32_t nq,
		uint32_t nb) {
	const uint32_t *q = a.queue[lvl & 1];
	const uint32_t gwarp = blockIdx.x * kMsWarps + warp_id();
	const uint32_t nwarps = gridDim.x * kMsWarps;
	for (uint32_t i = gwarp; i < nq; i += nwarps) {
		const uint32_t u = ld_cg(q + i);
		ms_push_edges(a, cur, actc, nxt, u, __ldg(a.row_off + u), __ldg(a.row_off + u + 1), 0, 32);
	}
	if (!nb) return;
	const uint32_t nc = ld_volatile(&a.ctl->push_chunks);
	for (uint32_t c = gwarp; c < nc; c += nwarps) {
		const uint32_t u = ld_cg(a.push_u + c), beg = ld_cg(a.push_beg + c);
		const uint32_t end = min(beg + kMsPushChunk, __ldg(a.row_off + u + 1));
		ms_push_edges(a, cur, actc, nxt, u, beg, end, 0, 32);
	}
}

// The next-frontier mask of a row whose new words lanes hold (word l, l + 32).
__device__ __forceinline__ uint64_t row_mask(uint64_t n0, uint64_t n1) {
	return (uint64_t) __ballot_sync(kFull, n0 != 0ull) | ((uint64_t) __ballot_sync(kFull, n1 != 0ull) << 32);
}

// After a push level: the OR'ed words lose the bits already visited, the rest
// are new, go into vis and put v into the next frontier.  A warp takes 32
// vertices, then works through the touched ones together (K words each).
__device__ void ms_push_finish(const MsArgs &a, uint32_t lvl, uint64_t *nxt, uint64_t *actn, unsigned long long &actdeg,
		unsigned long long *s_act) {
	const uint32_t K = a.K;
	const unsigned lane = lane_id();
	uint32_t *qn = a.queue[(lvl + 1) & 1];
	MsCounters *cn = &a.ctl->ctr[(lvl + 1) % 3];
	const uint32_t gwarp = blockIdx.x * kMsWarps + warp_id();
	const uint32_t nwarps = gridDim.x * kMsWarps;
	uint64_t newacc[2] = {0ull, 0ull};
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
				newacc[h] |= nw[h];
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
	if (lane < a.K && newacc[0]) atomicOr(s_act + lane, (unsigned long long) newacc[0]);
	if (lane + 32 < a.K && newacc[1]) atomicOr(s_act + lane + 32, (unsigned long long) newacc[1]);
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
	// `act` (may be null: every source): the level's active words
	__device__ __forceinline__ FullMask(const MsArgs &a, unsigned lane, const unsigned long long *act = nullptr) {
		const uint64_t last = a.last_bits == 64 ? ~0ull : ((1ull << a.last_bits) - 1);
		f0 = lane < a.K ? (lane == a.K - 1 ? last : ~0ull) : 0ull;
		f1 = lane + 32 < a.K ? (lane + 32 == a.K - 1 ? last : ~0ull) : 0ull;
		if (act) {
			if (lane < a.K) f0 &= ld_cg64((const uint64_t *) act + lane);
			if (lane + 32 < a.K) f1 &= ld_cg64((const uint64_t *) act + lane + 32);
		}
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
	uint32_t loads = 0;
	for (uint32_t e0 = beg; e0 < end && !done; e0 += 32) {
		const uint32_t e = e0 + lane;
		const uint32_t u = e < end ? __ldg(a.in_src + e) : 0u;
		const uint64_t um = e < end ? ld_cg64(actc + u) : 0ull;
		uint32_t lm = __ballot_sync(kFull, um != 0ull);
		while (lm && !done) {
			const bool need0 = ((acc0 | vis0) & fm.f0) != fm.f0;
			const bool need1 = ((acc1 | vis1) & fm.f1) != fm.f1;
			uint64_t g0[kMsGather], g1[kMsGather];
#pragma unroll
			for (int t = 0; t < kMsGather; ++t) {
				uint32_t ut = 0;
				uint64_t mt = 0;
				if (lm) {
					const int src_lane = __ffs(lm) - 1;
					lm &= lm - 1;
					ut = __shfl_sync(kFull, u, src_lane);
					mt = shfl64(um, src_lane);
				}
				const uint64_t *r = cur + (size_t) ut * K;
				const bool l0 = need0 && ((mt >> lane) & 1ull), l1 = need1 && ((mt >> (lane + 32)) & 1ull);
				g0[t] = l0 ? ld_cg64(r + lane) : 0ull;
				g1[t] = l1 ? ld_cg64(r + lane + 32) : 0ull;
				loads += (uint32_t) l0 + (uint32_t) l1;  // words read by this lane
			}
#pragma unroll
			for (int t = 0; t < kMsGather; ++t) { acc0 |= g0[t]; acc1 |= g1[t]; }
			done = fm.complete(acc0 | vis0, acc1 | vis1);
		}
	}
	gathered += loads;
	return done;
}

// A bijection of [0, 2^bits): xor-shift, multiply by an odd constant, xor-shift.
__device__ __forceinline__ uint32_t block_perm(uint32_t x, uint32_t bits) {
	const uint32_t mask = bits >= 32 ? 0xFFFFFFFFu : (1u << bits) - 1u;
	const uint32_t h = (bits + 1) / 2;
	x ^= x >> h;
	x = (x * 0x9E3779B1u) & mask;
	x ^= x >> h;
	return x;
}

__device__ __forceinline__ uint64_t warp_or64(uint64_t x) {
#pragma unroll
	for (int d = 16; d > 0; d >>= 1) x |= shfl_xor64(x, d);
	return x;
}

// ms_gather for 2 < K <= 16 words per vertex: the warp is split into
// 32 / kp groups of kp lanes (kp = K rounded up to a power of two); a group
// reads one in-neighbour row (lane k its word k), so a round reads
// kMsGather * 32 / kp rows; the groups' words are OR-ed together after every
// round for the early exit.  `vis` and `f` are the lane's word k (the same in
// every group); acc comes back in every group.
__device__ __forceinline__ void ms_gather_grouped(const MsArgs &a, const uint64_t *cur, const uint64_t *actc,
		uint32_t beg, uint32_t end, uint32_t kp, uint64_t f, uint64_t vis, uint64_t &acc, unsigned long long &gathered) {
	const uint32_t K = a.K;
	const unsigned lane = lane_id();
	const uint32_t k = lane & (kp - 1), grp = lane / kp, ngrp = 32 / kp;
	const bool wk = k < K;
	uint32_t loads = 0;
	bool done = __all_sync(kFull, ((vis | acc) & f) == f);
	for (uint32_t e0 = beg; e0 < end && !done; e0 += 32) {
		const uint32_t e = e0 + lane;
		const uint32_t u = e < end ? __ldg(a.in_src + e) : 0u;
		const uint64_t um = e < end ? ld_cg64(actc + u) : 0ull;
		uint32_t lm = __ballot_sync(kFull, um != 0ull);
		while (lm && !done) {
			const bool need = ((vis | acc) & f) != f;
			const uint32_t nlive = __popc(lm);
			uint64_t gv[kMsGather];
#pragma unroll
			for (int t = 0; t < kMsGather; ++t) {
				const uint32_t idx = t * ngrp + grp;
				const int src = idx < nlive ? (int) __fns(lm, 0, idx + 1) : 0;
				const uint32_t ut = __shfl_sync(kFull, u, src);
				const uint64_t mt = shfl64(um, src);
				const bool ld = idx < nlive && need && wk && ((mt >> k) & 1ull);
				gv[t] = ld ? ld_cg64(cur + (size_t) ut * K + k) : 0ull;
				loads += ld;
			}
#pragma unroll
			for (int t = 0; t < kMsGather; ++t) acc |= gv[t];
			for (uint32_t d = kp; d < 32; d <<= 1) acc |= shfl_xor64(acc, d);
			const uint32_t took = min(nlive, (uint32_t) kMsGather * ngrp);
			if (took == nlive) lm = 0;
			else lm &= ~((1u << __fns(lm, 0, took + 1)) - 1u);
			done = __all_sync(kFull, ((vis | acc) & f) == f);
		}
	}
	gathered += loads;
}

// ms_gather for K <= 2 words per vertex: lanes take in-edges (32 per step)
// instead of words, read the neighbour's needed non-zero words and OR them
// across the warp.  Inputs and outputs are word 0 / word 1 in every lane.
__device__ __forceinline__ void ms_gather_edges(const MsArgs &a, const uint64_t *cur, const uint64_t *actc,
		uint32_t beg, uint32_t end, uint64_t f0, uint64_t f1, uint64_t vis0, uint64_t vis1, uint64_t &acc0,
		uint64_t &acc1, unsigned long long &gathered) {
	const uint32_t K = a.K;
	const unsigned lane = lane_id();
	for (uint32_t e0 = beg; e0 < end; e0 += 32) {
		const bool n0 = ((vis0 | acc0) & f0) != f0, n1 = ((vis1 | acc1) & f1) != f1;
		if (!n0 && !n1) break;  // uniform: every lane holds the same words
		const uint32_t e = e0 + lane;
		const uint32_t u = e < end ? __ldg(a.in_src + e) : 0u;
		const uint64_t m = e < end ? ld_cg64(actc + u) : 0ull;
		const bool l0 = n0 && (m & 1ull), l1 = n1 && (m & 2ull);
		const uint64_t g0 = l0 ? ld_cg64(cur + (size_t) u * K) : 0ull;
		const uint64_t g1 = l1 ? ld_cg64(cur + (size_t) u * K + 1) : 0ull;
		gathered += (unsigned long long) l0 + l1;
		acc0 |= warp_or64(g0);
		acc1 |= warp_or64(g1);
	}
}

// Pull of one destination by one lane (K <= kLaneMaxWords words per vertex,
// at most kLaneMaxDeg in-edges): the lane walks the in-edges four at a time,
// reads a neighbour's word only where its mask is set and the destination
// still lacks sources, and stops when every source has arrived.  Lanes with
// `mine` false only take part in the warp-wide appends.
__device__ __forceinline__ void ms_pull_lane(const MsArgs &a, const uint64_t *cur, const uint64_t *actc,
		uint64_t *nxt, uint64_t *actn, uint32_t v, uint32_t beg, uint32_t end, bool mine, unsigned long long &actdeg,
		unsigned long long &gathered, MsCounters *cn, uint32_t *qn, uint64_t act0, uint64_t act1, uint64_t &new0,
		uint64_t &new1) {
	const uint32_t K = a.K;
	const uint64_t last = a.last_bits == 64 ? ~0ull : ((1ull << a.last_bits) - 1);
	const uint64_t f0 = (K == 1 ? last : ~0ull) & act0, f1 = (K == 2 ? last : 0ull) & act1;
	uint64_t vis0 = 0, vis1 = 0, acc0 = 0, acc1 = 0;
	bool any = false;
	uint32_t d = 0;
	if (mine) {
		const size_t row = (size_t) v * K;
		vis0 = ld_cg64(a.vis + row);
		vis1 = K == 2 ? ld_cg64(a.vis + row + 1) : 0ull;
		for (uint32_t e = beg; e < end; e += 4) {
			if (((vis0 | acc0) & f0) == f0 && ((vis1 | acc1) & f1) == f1) break;
			uint32_t u[4];
			uint64_t m[4];
#pragma unroll
			for (int t = 0; t < 4; ++t) u[t] = e + t < end ? __ldg(a.in_src + e + t) : 0xFFFFFFFFu;
#pragma unroll
			for (int t = 0; t < 4; ++t) m[t] = u[t] != 0xFFFFFFFFu ? ld_cg64(actc + u[t]) : 0ull;
			const bool n0 = ((vis0 | acc0) & f0) != f0, n1 = ((vis1 | acc1) & f1) != f1;
			uint64_t g0[4], g1[4];
#pragma unroll
			for (int t = 0; t < 4; ++t) {
				const bool l0 = n0 && (m[t] & 1ull), l1 = n1 && (m[t] & 2ull);
				g0[t] = l0 ? ld_cg64(cur + (size_t) u[t] * K) : 0ull;
				g1[t] = l1 ? ld_cg64(cur + (size_t) u[t] * K + 1) : 0ull;
				gathered += (unsigned long long) l0 + l1;
			}
#pragma unroll
			for (int t = 0; t < 4; ++t) { acc0 |= g0[t]; acc1 |= g1[t]; }
		}
		const uint64_t w0 = acc0 & ~vis0 & f0, w1 = acc1 & ~vis1 & f1;
		new0 |= w0;
		new1 |= w1;
		nxt[row] = w0;
		if (w0) a.vis[row] = vis0 | w0;
		if (K == 2) {
			nxt[row + 1] = w1;
			if (w1) a.vis[row + 1] = vis1 | w1;
		}
		actn[v] = (w0 ? 1ull : 0ull) | (w1 ? 2ull : 0ull);
		if (((vis0 | w0) & f0) == f0 && ((vis1 | w1) & f1) == f1) a.done[v] = 1;
		any = (w0 | w1) != 0ull;
		if (any) {
			d = deg_of(a, v);
			actdeg += d;
		}
	}
	ms_append(a, cn, qn, v, any && d <= kMsBig, any && d > kMsBig);
}

// Pull, destinations with at most kMsPullBig in-edges.  A warp screens 32
// consecutive destinations at once (their in-edge ranges and "every source
// has arrived" flags, lane-parallel), clears the rows of those with nothing
// to do as one contiguous block, then works through the others one at a
// time: lane l owns words l and l + 32.  The rows of many-in-edge
// destinations are cleared here and filled by ms_pull_chunks.
__device__ void ms_pull(const MsArgs &a, uint32_t lvl, const uint64_t *cur, const uint64_t *actc, uint64_t *nxt,
		uint64_t *actn, unsigned long long &actdeg, unsigned long long &gathered, uint32_t *wq_base,
		const unsigned long long *act, unsigned long long *s_act) {
	const uint32_t K = a.K;
	uint32_t *qn = a.queue[(lvl + 1) & 1];
	MsCounters *cn = &a.ctl->ctr[(lvl + 1) % 3];
	const unsigned lane = lane_id();
	const uint32_t gwarp = blockIdx.x * kMsWarps + warp_id();
	const uint32_t nwarps = gridDim.x * kMsWarps;
	const bool w0 = lane < K, w1 = lane + 32 < K;
	const FullMask fm(a, lane, act);
	const uint64_t lact0 = act ? ld_cg64((const uint64_t *) act) : ~0ull;
	const uint64_t lact1 = act && K > 1 ? ld_cg64((const uint64_t *) act + 1) : ~0ull;
	uint64_t new_lane0 = 0, new_lane1 = 0;  // new words lane / lane + 32 (warp-per-destination paths)
	uint64_t new_w0 = 0, new_w1 = 0;        // new words 0 / 1 (lane-per-destination path)
	uint32_t *wbuf = wq_base + warp_id() * kMsWq;
	uint32_t wn = 0;
	// blocks of 32 destinations in a hashed order: in-degree follows the id
	// bits of R-MAT-like graphs, so a plain stride gives some warps the heavy
	// blocks every time
	const uint32_t nblk = (a.n + 31) / 32;
	const uint32_t pbits = 32 - __clz(max(nblk - 1, 1u));
	for (uint32_t i = gwarp; i < (1u << pbits); i += nwarps) {
		const uint32_t bi = block_perm(i, pbits);
		if (bi >= nblk) continue;
		const uint32_t vb = bi * 32;
		const uint32_t vl = vb + lane;
		const bool valid = vl < a.n;
		const uint32_t lbeg = valid ? __ldg(a.in_off + vl) : 0u, lend = valid ? __ldg(a.in_off + vl + 1) : 0u;
		const bool big = lend - lbeg > kMsPullBig;
		const bool needy = valid && !big && lend > lbeg && !ld_cg_u8(a.done + vl);
		const uint32_t needm = __ballot_sync(kFull, needy);
		if (valid && !needy && !big) actn[vl] = 0;
		// rows of the block with nothing to do (and of big destinations) are zero
		const uint32_t nb = min(32u, a.n - vb);
		uint64_t *blk = nxt + (size_t) vb * K;
		for (uint32_t x = lane; x < nb * K; x += 32)
			if (!((needm >> (x / K)) & 1u)) blk[x] = 0ull;
		// few words per vertex: every lane takes its own low in-degree destination
		uint32_t warpm = needm;
		if (K <= kLaneMaxWords) {
			const bool mine = needy && lend - lbeg <= kLaneMaxDeg;
			warpm &= ~__ballot_sync(kFull, mine);
			ms_pull_lane(a, cur, actc, nxt, actn, vl, lbeg, lend, mine, actdeg, gathered, cn, qn, lact0, lact1, new_w0,
					new_w1);
		}
		for (uint32_t m = warpm; m; m &= m - 1) {
			const int jj = __ffs(m) - 1;
			const uint32_t v = vb + jj;
			const uint32_t beg = __shfl_sync(kFull, lbeg, jj), end = __shfl_sync(kFull, lend, jj);
			const size_t row = (size_t) v * K;
			const uint64_t vis0 = w0 ? ld_cg64(a.vis + row + lane) : 0ull;
			const uint64_t vis1 = w1 ? ld_cg64(a.vis + row + lane + 32) : 0ull;
			uint64_t acc0 = 0, acc1 = 0;
			if (K <= kLaneMaxWords) {
				// lanes hold words lane; the edge-parallel gather wants both words everywhere
				uint64_t a0 = 0, a1 = 0;
				ms_gather_edges(a, cur, actc, beg, end, shfl64(fm.f0, 0), shfl64(fm.f0, 1), shfl64(vis0, 0),
						shfl64(vis0, 1), a0, a1, gathered);
				acc0 = lane == 0 ? a0 : (lane == 1 ? a1 : 0ull);
			} else if (K <= kGroupMaxWords) {
				const uint32_t kp = K <= 4 ? 4 : 8;
				const uint32_t kw = lane & (kp - 1);
				uint64_t ag = 0;
				ms_gather_grouped(a, cur, actc, beg, end, kp, shfl64(fm.f0, kw), shfl64(vis0, kw), ag, gathered);
				acc0 = lane < kp ? ag : 0ull;
			} else if (!fm.complete(vis0, vis1)) {
				ms_gather(a, cur, actc, beg, end, fm, vis0, vis1, acc0, acc1, gathered);
			}
			const uint64_t n0 = acc0 & ~vis0 & fm.f0, n1 = acc1 & ~vis1 & fm.f1;
			new_lane0 |= n0;
			new_lane1 |= n1;
			if (w0) { nxt[row + lane] = n0; if (n0) a.vis[row + lane] = vis0 | n0; }
			if (w1) { nxt[row + lane + 32] = n1; if (n1) a.vis[row + lane + 32] = vis1 | n1; }
			const uint64_t mask = row_mask(n0, n1);
			const bool full = fm.complete(vis0 | n0, vis1 | n1);
			if (lane == 0) {
				actn[v] = mask;
				if (full) a.done[v] = 1;
			}
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
	}
	ms_wq_flush(cn, qn, wbuf, wn);
	if (w0 && new_lane0) atomicOr(s_act + lane, (unsigned long long) new_lane0);
	if (w1 && new_lane1) atomicOr(s_act + lane + 32, (unsigned long long) new_lane1);
	if (new_w0) atomicOr(s_act, (unsigned long long) new_w0);
	if (new_w1) atomicOr(s_act + 1, (unsigned long long) new_w1);
}

// Pull, destinations with many in-edges: warps take chunks of kMsChunk
// in-edges over the whole grid and OR what they gather into the row.
__device__ void ms_pull_chunks(const MsArgs &a, const uint64_t *cur, const uint64_t *actc, uint64_t *nxt,
		unsigned long long &gathered, const unsigned long long *act) {
	const uint32_t K = a.K;
	const unsigned lane = lane_id();
	const uint32_t gwarp = blockIdx.x * kMsWarps + warp_id();
	const uint32_t nwarps = gridDim.x * kMsWarps;
	const bool w0 = lane < K, w1 = lane + 32 < K;
	const FullMask fm(a, lane, act);
	for (uint32_t c = gwarp; c < a.nchunks; c += nwarps) {
		const uint32_t v = __ldg(a.chunk_v + c), beg = __ldg(a.chunk_beg + c);
		const uint32_t end = min(beg + kMsChunk, __ldg(a.in_off + v + 1));
		const size_t row = (size_t) v * K;
		const uint64_t vis0 = w0 ? ld_cg64(a.vis + row + lane) : 0ull;
		const uint64_t vis1 = w1 ? ld_cg64(a.vis + row + lane + 32) : 0ull;
		if (fm.complete(vis0, vis1)) continue;
		uint64_t acc0 = 0, acc1 = 0;
		if (K <= kLaneMaxWords) {
			uint64_t a0 = 0, a1 = 0;
			ms_gather_edges(a, cur, actc, beg, end, shfl64(fm.f0, 0), shfl64(fm.f0, 1), shfl64(vis0, 0), shfl64(vis0, 1),
					a0, a1, gathered);
			acc0 = lane == 0 ? a0 : (lane == 1 ? a1 : 0ull);
		} else if (K <= kGroupMaxWords) {
			const uint32_t kp = K <= 4 ? 4 : 8;
			const uint32_t kw = lane & (kp - 1);
			uint64_t ag = 0;
			ms_gather_grouped(a, cur, actc, beg, end, kp, shfl64(fm.f0, kw), shfl64(vis0, kw), ag, gathered);
			acc0 = lane < kp ? ag : 0ull;
		} else {
			ms_gather(a, cur, actc, beg, end, fm, vis0, vis1, acc0, acc1, gathered);
		}
		const uint64_t n0 = acc0 & ~vis0 & fm.f0, n1 = acc1 & ~vis1 & fm.f1;
		if (n0) atomicOr((unsigned long long *) (nxt + row + lane), (unsigned long long) n0);
		if (n1) atomicOr((unsigned long long *) (nxt + row + lane + 32), (unsigned long long) n1);
	}
}

// After ms_pull_chunks: the many-in-edge destinations' rows hold their new
// bits; update vis, the frontier mask and the queue.
__device__ void ms_pull_chunks_finish(const MsArgs &a, uint32_t lvl, uint64_t *nxt, uint64_t *actn,
		unsigned long long &actdeg, unsigned long long *s_act) {
	const uint32_t K = a.K;
	uint32_t *qn = a.queue[(lvl + 1) & 1];
	MsCounters *cn = &a.ctl->ctr[(lvl + 1) % 3];
	const unsigned lane = lane_id();
	const uint32_t gwarp = blockIdx.x * kMsWarps + warp_id();
	const uint32_t nwarps = gridDim.x * kMsWarps;
	const bool w0 = lane < K, w1 = lane + 32 < K;
	uint64_t new0 = 0, new1 = 0;
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
		new0 |= n0;
		new1 |= n1;
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
	if (w0 && new0) atomicOr(s_act + lane, (unsigned long long) new0);
	if (w1 && new1) atomicOr(s_act + lane + 32, (unsigned long long) new1);
}

// Planes [first, last] (levels base + p) -> uint8 levels [source][vertex].
// A CTA of 512 threads takes tiles of 128 vertices x 4 words (256 sources).
// 1. thread (vertex, word) -- a warp holds 32 consecutive vertices of one
//    word -- builds the 64 level bytes of its word's sources in 16 registers:
//    for every plane whose word mask says the word is non-zero it loads the
//    word and, four sources at a time, looks the nibble up in a 16-entry
//    shared table of byte masks and writes the plane's level under it.  A
//    byte starts at 255 and is written at most once (a source reaches a vertex
//    at one level), so "write" is an XOR with 255 ^ level.  The 16 words go to
//    shared memory as [word][source quad][vertex].
// 2. thread (word, source quad, 16 vertices) reads its 16 words with 16-byte
//    loads, transposes them 4 x 4 bytes at a time (byte permutes) into the
//    16-byte pieces of its 4 source rows and stores those.
// `merge` combines with the bytes already in `levels` (a later segment of a
// traversal deeper than the planes) by a byte-wise minimum: every byte is
// below 255 in at most one segment.
__device__ __forceinline__ uint32_t nibble_bytes(uint32_t nib) {
	return ((nib * 0x00204081u) & 0x01010101u) * 0xFFu;  // bit i -> byte i all ones
}

// 16 level bytes (x, vertices in order) -> levels at dst, cnt <= 16 of them,
// with the widest store the address allows.
__device__ __forceinline__ void emit_piece(uint8_t *dst, const uint32_t (&x)[4], uint32_t cnt, bool merge) {
	const uintptr_t al = (uintptr_t) dst;
	if (cnt == 16 && (al & 15) == 0) {
		uint4 y = make_uint4(x[0], x[1], x[2], x[3]);
		if (merge) {
			const uint4 old = __ldcg((const uint4 *) dst);
			y.x = __vminu4(y.x, old.x);
			y.y = __vminu4(y.y, old.y);
			y.z = __vminu4(y.z, old.z);
			y.w = __vminu4(y.w, old.w);
		}
		*(uint4 *) dst = y;
	} else if (cnt == 16 && (al & 3) == 0) {
#pragma unroll
		for (int q = 0; q < 4; ++q) {
			uint32_t y = x[q];
			if (merge) y = __vminu4(y, __ldcg((const unsigned int *) dst + q));
			((uint32_t *) dst)[q] = y;
		}
	} else if (cnt == 16 && (al & 1) == 0) {
#pragma unroll
		for (int q = 0; q < 8; ++q) {
			uint32_t y = (x[q / 2] >> (16 * (q & 1))) & 0xFFFFu;
			if (merge) {
				const uint32_t old = __ldcg((const unsigned short *) dst + q);
				y = __vminu4(y | 0xFFFF0000u, old | 0xFFFF0000u) & 0xFFFFu;
			}
			((uint16_t *) dst)[q] = (uint16_t) y;
		}
	} else {
#pragma unroll
		for (uint32_t b = 0; b < 16; ++b) {
			if (b >= cnt) break;
			const uint8_t y = (uint8_t) (x[b / 4] >> (8 * (b & 3)));
			dst[b] = merge ? min(y, ld_cg_u8(dst + b)) : y;
		}
	}
}

// kCached: the planes may be read through L1 (a launch of its own after the
// traversal; the four warps of a tile read neighbouring words of the same
// sectors); inside the traversal kernel they are read around L1.
template <bool kCached>
__device__ __forceinline__ uint64_t emit_ld(const uint64_t *p) {
	return kCached ? (uint64_t) __ldg((const unsigned long long *) p) : ld_cg64(p);
}

// kCached also selects two row buffers used in turn, so that a tile needs one
// barrier (between its two phases): a buffer is written again two tiles
// later, after the barrier that every thread reaches once done reading it.
template <bool kCached, uint32_t kV>
__device__ __noinline__ void ms_emit(const MsArgs &a, uint8_t *levels, uint32_t ns, uint32_t base, uint32_t first, uint32_t last,
		bool merge, uint8_t *lev) {
	constexpr uint32_t kEmitV = kV, kEmitRow = kV + 4;
	constexpr uint32_t kBufs = kCached ? 2 : 1, kBufWords = kEmitW * 16 * kEmitRow;
	constexpr uint32_t kRows = kEmitW * 64;
	const uint32_t K = a.K, n = a.n;
	const uint32_t vtiles = (n + kEmitV - 1) / kEmitV, wtiles = (K + kEmitW - 1) / kEmitW;
	const uint32_t vi = threadIdx.x % kEmitV, wi = threadIdx.x / kEmitV;
	const size_t pstride = (size_t) n * K;
	uint32_t *const sw0 = reinterpret_cast<uint32_t *>(lev);  // [buffer][wi * 16 + quad][kEmitRow]
	uint32_t *lut = sw0 + kBufs * kBufWords;                 // nibble -> byte mask
	if (threadIdx.x < 16) lut[threadIdx.x] = nibble_bytes(threadIdx.x);
	// phase 2's item: rows of source quad rq (word rq / 16), vertices 16 cc ...
	const uint32_t rq = threadIdx.x / (kEmitV / 16), cc = threadIdx.x % (kEmitV / 16);
	__syncthreads();
	uint32_t turn = 0;
	for (uint32_t tile = blockIdx.x; tile < vtiles * wtiles; tile += gridDim.x, ++turn) {
		uint32_t *sw = sw0 + (turn % kBufs) * kBufWords;
		const uint32_t v0 = (tile % vtiles) * kEmitV, k0 = (tile / vtiles) * kEmitW;
		const uint32_t nv = min(kEmitV, n - v0);
		const uint32_t nrows = min(kRows, ns - k0 * 64);
		// 1. this thread's 64 level bytes
		if (vi < nv && k0 + wi < K) {
			const uint32_t v = v0 + vi, k = k0 + wi;
			const uint64_t *pw = a.hist + ((size_t) first * n + v) * K + k;
			const uint64_t *pm = a.pmask + (size_t) first * n + v;
			uint32_t o[16];
#pragma unroll
			for (int q = 0; q < 16; ++q) o[q] = 0xFFFFFFFFu;
			// 8 planes per round: their word masks (one round trip), then the
			// non-zero words (one more)
			for (uint32_t l = first; l <= last; l += 8) {
				uint32_t nz = 0;
#pragma unroll
				for (int t = 0; t < 8; ++t)
					if (l + t <= last)
						nz |= (uint32_t) ((emit_ld<kCached>(pm + (size_t) (l - first + t) * n) >> k) & 1ull) << t;
				uint64_t w[8];
#pragma unroll
				for (int t = 0; t < 8; ++t)
					w[t] = ((nz >> t) & 1u) ? emit_ld<kCached>(pw + (size_t) (l - first + t) * pstride) : 0ull;
#pragma unroll
				for (int t = 0; t < 8; ++t) {
					if (!w[t]) continue;
					const uint32_t inv = ~((uint32_t) (base + l + t) * 0x01010101u);
					const uint32_t lo = (uint32_t) w[t], hi = (uint32_t) (w[t] >> 32);
#pragma unroll
					for (int q = 0; q < 8; ++q) o[q] ^= lut[(lo >> (4 * q)) & 0xFu] & inv;
#pragma unroll
					for (int q = 0; q < 8; ++q) o[8 + q] ^= lut[(hi >> (4 * q)) & 0xFu] & inv;
				}
			}
			uint32_t *col = sw + wi * 16 * kEmitRow + vi;
#pragma unroll
			for (int q = 0; q < 16; ++q) col[q * kEmitRow] = o[q];
		}
		__syncthreads();
		// 2. rows out: 16 vertices x 4 source rows per thread
		const uint32_t c = cc * 16, r0 = rq * 4;
		if (k0 + rq / 16 < K && r0 < nrows && c < nv) {
			const uint4 *sp = reinterpret_cast<const uint4 *>(sw + rq * kEmitRow + c);
			uint32_t x[16];
#pragma unroll
			for (int j = 0; j < 4; ++j) {
				const uint4 u = sp[j];
				x[4 * j] = u.x;
				x[4 * j + 1] = u.y;
				x[4 * j + 2] = u.z;
				x[4 * j + 3] = u.w;
			}
			// y[b][g]: source 4 rq + b, vertices c + 4g .. c + 4g + 3
			uint32_t y[4][4];
#pragma unroll
			for (int g = 0; g < 4; ++g) {
				const uint32_t t0 = __byte_perm(x[4 * g], x[4 * g + 1], 0x5140);
				const uint32_t t1 = __byte_perm(x[4 * g + 2], x[4 * g + 3], 0x5140);
				const uint32_t t2 = __byte_perm(x[4 * g], x[4 * g + 1], 0x7362);
				const uint32_t t3 = __byte_perm(x[4 * g + 2], x[4 * g + 3], 0x7362);
				y[0][g] = __byte_perm(t0, t1, 0x5410);
				y[1][g] = __byte_perm(t0, t1, 0x7632);
				y[2][g] = __byte_perm(t2, t3, 0x5410);
				y[3][g] = __byte_perm(t2, t3, 0x7632);
			}
			const uint32_t cnt = min(16u, nv - c);
#pragma unroll
			for (int b = 0; b < 4; ++b) {
				if (r0 + b >= nrows) break;
				emit_piece(levels + (size_t) (k0 * 64 + r0 + b) * n + v0 + c, y[b], cnt, merge);
			}
		}
		if (kBufs == 1) __syncthreads();
	}
}

__global__ void __launch_bounds__(kMsThreads, 2) k_ms_bfs(MsArgs a, const uint32_t *sources, uint32_t ns,
		uint8_t *levels) {
	__shared__ unsigned long long red[kMsWarps];
	__shared__ uint32_t wq[kMsWarps * kMsWq];
	__shared__ __align__(16) uint8_t lev[kEmitBytes];
	MsControl *ctl = a.ctl;
	const uint32_t stride = gridDim.x * blockDim.x;
	const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x;
	const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
	const size_t nK = (size_t) a.n * a.K;
	unsigned epoch = 0;  // grid barriers passed (the control block, and its arrival count, start zeroed)
	if (leader) ctl->stats.t_start = global_timer_ns();
	// clear (the control block was zeroed by the host)
	for (size_t i = t0; i < nK; i += stride) { a.vis[i] = 0; a.hist[i] = 0; }
	for (uint32_t i = t0; i < a.n; i += stride) {
		a.pmask[i] = 0;
		a.done[i] = 0;
		a.touched[i] = 0;
		a.seed_flag[i] = 0;
	}
	bool ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier);
	// plane 0: every source reaches itself
	if (ok) {
		for (uint32_t i = t0; i < ns; i += stride) {
			const uint32_t v = sources[i];
			if (v >= a.n) {  // device-resident sources are checked here
				atomicExch(&ctl->err, BFS_EARG);
				continue;
			}
			const size_t x = (size_t) v * a.K + i / 64;
			const unsigned long long bit = 1ull << (i % 64);
			atomicOr((unsigned long long *) (a.hist + x), bit);
			atomicOr((unsigned long long *) (a.vis + x), bit);
			atomicOr((unsigned long long *) (a.pmask + v), 1ull << (i / 64));
			if (atomicExch(a.seed_flag + v, 1u) == 0u) {
				const uint32_t d = deg_of(a, v);
				if (d > kMsBig) a.queue[0][a.n - 1 - atomicAdd(&ctl->ctr[0].nbig, 1u)] = v;
				else a.queue[0][atomicAdd(&ctl->ctr[0].nact, 1u)] = v;
				atomicAdd(&ctl->ctr[0].act_deg, (unsigned long long) d);
			}
		}
		ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier);
	}
	if (leader) ctl->stats.t_levels0 = global_timer_ns();
	unsigned long long gathered = 0;
	uint32_t base = 0, lvl = 0;
	bool complete = false;
	__shared__ unsigned long long s_act[64];  // this CTA's OR of the next frontier's words
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
			if (!levels) {  // planes kept for a later pass (betweenness): they must hold every level
				if (leader) atomicExch(&ctl->err, BFS_EUNSUPPORTED);
				break;
			}
			// planes full: write them out, keep the frontier's plane as plane 0
			ms_emit<false, kEmitV>(a, levels, ns, base, base == 0 ? 0 : 1, lvl - base, base != 0, lev);
			if (!(ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier))) break;
			const uint64_t *src = a.hist + (size_t) (lvl - base) * nK;
			for (size_t i = t0; i < nK; i += stride) a.hist[i] = ld_cg64(src + i);
			const uint64_t *msrc = a.pmask + (size_t) (lvl - base) * a.n;
			for (uint32_t i = t0; i < a.n; i += stride) a.pmask[i] = ld_cg64(msrc + i);
			base = lvl;
			if (leader) ctl->stats.spills++;
			if (!(ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier))) break;
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
			for (uint32_t k = 0; k < a.K; ++k) ctl->active[(lvl + 2) % 3][k] = 0;
		}
		if (threadIdx.x < 64) s_act[threadIdx.x] = 0;
		__syncthreads();
		// the sources with a frontier at this level (level 0: every source)
		const unsigned long long *act = lvl == 0 ? nullptr : ctl->active[lvl % 3];
		const uint64_t *cur = a.hist + (size_t) (lvl - base) * nK;
		uint64_t *nxt = a.hist + (size_t) (lvl + 1 - base) * nK;
		const uint64_t *actc = a.pmask + (size_t) (lvl - base) * a.n;
		uint64_t *actn = a.pmask + (size_t) (lvl + 1 - base) * a.n;
		unsigned long long *tph = lvl < kMsTraceLevels ? ctl->stats.t_phase[lvl] : nullptr;
		unsigned long long actdeg = 0;
		const bool push = qdeg * (unsigned long long) a.push_div < (unsigned long long) a.m;
		if (push) {
			if (blockIdx.x == 0 && nb) ms_push_chunk_list(a, lvl, nb, wq);
			for (size_t i = t0; i < nK; i += stride) nxt[i] = 0;
			if (!(ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier))) break;
			if (leader && tph) tph[0] = global_timer_ns();
			ms_push(a, lvl, cur, actc, nxt, nq, nb);
			if (!(ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier))) break;
			if (leader && tph) tph[1] = global_timer_ns();
			ms_push_finish(a, lvl, nxt, actn, actdeg, s_act);
		} else {
			ms_pull(a, lvl, cur, actc, nxt, actn, actdeg, gathered, wq, act, s_act);
			if (a.nbig_in) {
				if (!(ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier))) break;
				if (leader && tph) tph[0] = global_timer_ns();
				ms_pull_chunks(a, cur, actc, nxt, gathered, act);
				if (!(ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier))) break;
				if (leader && tph) tph[1] = global_timer_ns();
				ms_pull_chunks_finish(a, lvl, nxt, actn, actdeg, s_act);
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
		// the next level's active sources: this CTA's share
		if (threadIdx.x < a.K && s_act[threadIdx.x])
			atomicOr(&ctl->active[(lvl + 1) % 3][threadIdx.x], s_act[threadIdx.x]);
		__syncthreads();
		ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier);
	}
	if (leader) {
		ctl->stats.t_levels1 = global_timer_ns();
		if (lvl < kMsTraceLevels) ctl->stats.t_level[lvl] = ctl->stats.t_levels1;
		ctl->stats.base = base;
		ctl->stats.complete = complete ? 1u : 0u;
	}
	if (complete) {
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

// The final output pass, its own launch after k_ms_bfs (more CTAs per SM than
// the cooperative kernel, so more plane loads in flight).  Plane depth - base
// is the empty frontier; after an early output pass, plane 0 was written too.
// A tile's plane loads and its barriers form a chain of round trips; narrow
// tiles on small CTAs keep more chains going per SM.
template <int kThreads>
__global__ void __launch_bounds__(kThreads, kThreads == 256 ? 4 : 2) k_ms_emit(MsArgs a, uint32_t ns, uint8_t *levels) {
	constexpr uint32_t kV = kThreads / kEmitW;
	__shared__ __align__(16) uint8_t lev[emit_bytes(kV, 2)];
	const MsStats &st = a.ctl->stats;
	if (!st.complete) return;
	const uint32_t base = st.base, depth = st.depth;
	const uint32_t first = base == 0 ? 0 : 1;
	if (depth < base + first + 1) return;
	ms_emit<true, kV>(a, levels, ns, base, first, depth - 1 - base, base != 0, lev);
}

int ms_launch(const MsArgs &a, const uint32_t *d_sources, uint32_t ns, uint8_t *levels, int num_sms, cudaStream_t st,
		int *grid, cudaEvent_t between, cudaEvent_t between2) {
	int per_sm = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ms_bfs, kMsThreads, 0) != cudaSuccess || per_sm < 1)
		return BFS_ECUDA;
	per_sm = std::min(per_sm, 2);
	if (a.ctas_per_sm) per_sm = std::min(per_sm, (int) a.ctas_per_sm);
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
	if (between && cudaEventRecord(between, st) != cudaSuccess) return BFS_ECUDA;
	if (between2 && cudaEventRecord(between2, st) != cudaSuccess) return BFS_ECUDA;
	if (levels) {
		const bool wide = a.out_tile ? a.out_tile == 128 : a.n >= kEmitWideMinVertices;
		const void *fn = wide ? (const void *) k_ms_emit<512> : (const void *) k_ms_emit<256>;
		const int threads = wide ? 512 : 256;
		int out_per_sm = 0;
		if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&out_per_sm, fn, threads, 0) != cudaSuccess || out_per_sm < 1)
			return BFS_ECUDA;
		if (wide) k_ms_emit<512><<<num_sms * out_per_sm, 512, 0, st>>>(a, ns, levels);
		else k_ms_emit<256><<<num_sms * out_per_sm, 256, 0, st>>>(a, ns, levels);
	}
	return cudaGetLastError() == cudaSuccess ? BFS_OK : BFS_ECUDA;
}

} // namespace bfsg
