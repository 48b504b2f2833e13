// bc_batch.cu -- betweenness dependencies of 64 sources (one word of a batched
// traversal) in one pass.
//
// No counterpart in the reference, whose BC() (apps/betweennessCentrality_simd/
// bc.cpp:1717-2097) handles one source per call; for every source the results
// are that function's: path counts summed over in-edges from the previous
// level (unsigned, wrapping), dependency sums over out-edges to the next level
// from the deepest level up, and its float formulas (inverse
// 1.0f / (float)(int) count, result (D - inverse) / inverse, 0 where the
// count is 0).
//
// The batched traversal (msbfs.cu) leaves, for every level L, the plane
// hist[L][v]: the sources that reached v first at level L (a launch takes one
// 64-bit word of it).  u -> v is a shortest-path edge of source s exactly when
// bit s is set in both hist[L-1][u] and hist[L][v], so one AND of two words
// gives all the sources an edge serves.  The state is per (vertex, source):
// sigma[v][64] and dsum[v][64], a 256-byte row each.
//
// One cooperative launch, levels separated by grid barriers:
//   forward, L = 1 .. depth-1, every v with hist[L][v] != 0:
//     sigma[v][s] = sum of sigma[u][s] over in-edges u -> v, s in hist[L][v] & hist[L-1][u];
//   reverse, L = depth-1 .. 0:
//     dsum[v][s] = (sum of dsum[w][s] over out-edges v -> w, s in hist[L][v] & hist[L+1][w])
//                  + 1 / sigma[v][s].
// The launch first lists, per level, the blocks of 32 consecutive vertices
// and the edge chunks that have a vertex at that level; a level then hands
// its list items to warps one at a time through a counter.  A warp takes a
// block and walks the concatenated edge lists of its vertices at that level,
// 32 edges per step (each edge's vertex found by a binary search over the
// warp's degree prefix); an edge's source mask is one AND.  The edges with a
// non-empty mask are then taken in edge order by half-warps, two pairs per
// round (lane 16h + i holds sources 4i .. 4i+3: one 16-byte piece of the
// neighbour's row, read where any of the 4 is served); a vertex's sum is its
// half-0 sum plus its half-1 sum.  The finish of chunked vertices keeps lane l
// on sources l and l + 32.
// Vertices with more than kBbBig edges in the sweep's direction are cut into
// kBbChunk-edge chunks, one list item each; the partial rows are added in
// chunk order after a grid barrier.  Every sum has a fixed order, so repeated
// runs give identical bits.
// The output pass (its own launch) turns the [v][64] rows into [source][v]
// rows through a shared-memory transpose, 0 for unreached pairs, and/or adds
// each vertex's dependencies into an accumulator in source order.
#include "bc_batch.h"

#include <algorithm>

#include "../../include/bfs_gb300.h"
#include "device_common.cuh"

namespace bfsg {
namespace {

constexpr int kBbThreads = 512;
constexpr int kBbWarps = kBbThreads / 32;
constexpr int kBbUnroll = 4;   // chunk partial rows added per round (finish)
constexpr int kBbPairs = 2;    // pairs of served edges per round (their rows loaded together)
constexpr uint32_t kBbOutV = 64;   // output pass: vertices per tile
constexpr int kBbOutThreads = 256;

__device__ __forceinline__ uint64_t bb_shfl64(uint64_t x, int src) {
	return (uint64_t) __shfl_sync(kFull, (unsigned long long) x, src);
}
__device__ __forceinline__ uint64_t bb_ldg64(const uint64_t *p) { return __ldg((const unsigned long long *) p); }
// Plane L of the launch's word, and vertex v's entry in it (planes hold K words per vertex).
__device__ __forceinline__ const uint64_t *bb_plane(const BbArgs &a, uint32_t L) {
	return a.hist + (size_t) L * a.n * a.K + a.word;
}
__device__ __forceinline__ uint64_t bb_word(const uint64_t *plane, const BbArgs &a, uint32_t v) {
	return bb_ldg64(plane + (size_t) v * a.K);
}

// A warp's counts over a sweep: edges read (lane 0), edges that serve a
// source (lane 0), and (edge, source) pairs summed (every lane its own edges).
struct BbCount {
	unsigned long long edges, matched, served;
};

// The two sweeps: forward reads in-edges and path counts, reverse reads
// out-edges and dependency sums.
template <bool kFwd> struct BbDir;
template <> struct BbDir<true> {
	using T = uint32_t;
	static __device__ __forceinline__ const uint32_t *off(const BbArgs &a) { return a.in_off; }
	static __device__ __forceinline__ const uint32_t *adj(const BbArgs &a) { return a.in_src; }
	static __device__ __forceinline__ const uint32_t *chunk_v(const BbArgs &a) { return a.ichunk_v; }
	static __device__ __forceinline__ const uint32_t *chunk_beg(const BbArgs &a) { return a.ichunk_beg; }
	static __device__ __forceinline__ uint32_t nchunks(const BbArgs &a) { return a.nich; }
	static __device__ __forceinline__ const T *vals(const BbArgs &a) { return a.sigma; }
	static __device__ __forceinline__ T from_bits(uint32_t b) { return b; }
	static __device__ __forceinline__ uint32_t to_bits(T x) { return x; }
	static __device__ __forceinline__ uint32_t pre(const BbArgs &, size_t, bool) { return 0u; }
	static __device__ __forceinline__ void store(const BbArgs &a, size_t i, T sum, uint32_t) { a.sigma[i] = sum; }
};
template <> struct BbDir<false> {
	using T = float;
	static __device__ __forceinline__ const uint32_t *off(const BbArgs &a) { return a.row_off; }
	static __device__ __forceinline__ const uint32_t *adj(const BbArgs &a) { return a.col; }
	static __device__ __forceinline__ const uint32_t *chunk_v(const BbArgs &a) { return a.ochunk_v; }
	static __device__ __forceinline__ const uint32_t *chunk_beg(const BbArgs &a) { return a.ochunk_beg; }
	static __device__ __forceinline__ uint32_t nchunks(const BbArgs &a) { return a.noch; }
	static __device__ __forceinline__ const T *vals(const BbArgs &a) { return a.dsum; }
	static __device__ __forceinline__ T from_bits(uint32_t b) { return __uint_as_float(b); }
	static __device__ __forceinline__ uint32_t to_bits(T x) { return __float_as_uint(x); }
	// the vertex's path count, loaded ahead of its sum's store
	static __device__ __forceinline__ uint32_t pre(const BbArgs &a, size_t i, bool mine) {
		return mine ? __ldcg(a.sigma + i) : 0u;
	}
	// the reference's inverse: signed conversion of the unsigned count
	static __device__ __forceinline__ void store(const BbArgs &a, size_t i, T sum, uint32_t sg) {
		const float inv = sg ? 1.0f / (float) (int) sg : 0.0f;
		a.dsum[i] = sum + inv;
	}
};

// The finish of chunked vertices (lane l: sources l and l + 32): what a
// vertex's finished sums need besides the sums (the reverse sweep: its path
// counts for this lane's two sources), loaded ahead.
struct BbPre {
	uint32_t p0, p1;
};
template <bool kFwd> __device__ __forceinline__ BbPre bb_pre(const BbArgs &a, uint32_t v, uint64_t hv) {
	const unsigned lane = lane_id();
	const size_t row = (size_t) v * 64;
	return {BbDir<kFwd>::pre(a, row + lane, (hv >> lane) & 1ull),
			BbDir<kFwd>::pre(a, row + lane + 32, (hv >> (lane + 32)) & 1ull)};
}

// Writes vertex v's finished sums for the sources in hv (lane: sources lane
// and lane + 32).
template <bool kFwd>
__device__ __forceinline__ void bb_flush(const BbArgs &a, uint32_t v, uint64_t hv, typename BbDir<kFwd>::T acc0,
		typename BbDir<kFwd>::T acc1, BbPre pre) {
	const unsigned lane = lane_id();
	const size_t row = (size_t) v * 64;
	if ((hv >> lane) & 1ull) BbDir<kFwd>::store(a, row + lane, acc0, pre.p0);
	if ((hv >> (lane + 32)) & 1ull) BbDir<kFwd>::store(a, row + lane + 32, acc1, pre.p1);
}

// ---- half-warp sums over the edges that serve a source -------------------
// Lane 16h + i (half h) holds sources 4i .. 4i+3 of a row: 16 bytes, one
// load.  The served edges of a step are taken two at a time in edge order,
// the first by half 0 and the second by half 1, so that one round reads two
// rows; a vertex's sum is its half-0 sum plus its half-1 sum (one xor
// shuffle), written by half 0.

template <class T> __device__ __forceinline__ T bb_as(uint32_t b);
template <> __device__ __forceinline__ uint32_t bb_as<uint32_t>(uint32_t b) { return b; }
template <> __device__ __forceinline__ float bb_as<float>(uint32_t b) { return __uint_as_float(b); }

__device__ __forceinline__ uint32_t bb_quad() { return 4u * (lane_id() & 15u); }  // this lane's first source

// The open vertex's sums for this lane's 4 sources and (reverse sweep, half 0)
// its path counts for them, loaded when it is opened.
template <bool kFwd> struct BbOpen {
	typename BbDir<kFwd>::T acc[4];
	uint32_t pre[4];
};

template <bool kFwd> __device__ __forceinline__ void bb_open(const BbArgs &a, uint32_t v, uint64_t h, BbOpen<kFwd> &o) {
#pragma unroll
	for (int i = 0; i < 4; ++i) o.acc[i] = typename BbDir<kFwd>::T(0);
	if (!kFwd && lane_id() < 16u && ((h >> bb_quad()) & 0xFull)) {
		const uint4 p = __ldcg(reinterpret_cast<const uint4 *>(a.sigma + (size_t) v * 64 + bb_quad()));
		o.pre[0] = p.x;
		o.pre[1] = p.y;
		o.pre[2] = p.z;
		o.pre[3] = p.w;
	}
}

// Adds the halves and writes the open vertex's sums for its sources h.
template <bool kFwd> __device__ __forceinline__ void bb_close(const BbArgs &a, uint32_t v, uint64_t h, BbOpen<kFwd> &o) {
#pragma unroll
	for (int i = 0; i < 4; ++i) o.acc[i] += __shfl_xor_sync(kFull, o.acc[i], 16);
	const uint32_t bits = (uint32_t) (h >> bb_quad()) & 0xFu;
	if (lane_id() < 16u && bits) {
		const size_t row = (size_t) v * 64 + bb_quad();
#pragma unroll
		for (int i = 0; i < 4; ++i)
			if ((bits >> i) & 1u) BbDir<kFwd>::store(a, row + i, o.acc[i], o.pre[i]);
	}
}

// This half's edge: the neighbour's row entries for this lane's 4 sources
// where the edge serves them (mask m), else 0.
template <bool kFwd>
__device__ __forceinline__ void bb_vals(const BbArgs &a, uint32_t u, uint64_t m, typename BbDir<kFwd>::T (&x)[4]) {
	using T = typename BbDir<kFwd>::T;
	const uint32_t sb = (uint32_t) (m >> bb_quad()) & 0xFu;
#pragma unroll
	for (int i = 0; i < 4; ++i) x[i] = T(0);
	if (sb) {
		const uint4 r = __ldcg(reinterpret_cast<const uint4 *>(BbDir<kFwd>::vals(a) + (size_t) u * 64 + bb_quad()));
		x[0] = (sb & 1u) ? bb_as<T>(r.x) : T(0);
		x[1] = (sb & 2u) ? bb_as<T>(r.y) : T(0);
		x[2] = (sb & 4u) ? bb_as<T>(r.z) : T(0);
		x[3] = (sb & 8u) ? bb_as<T>(r.w) : T(0);
	}
}

// The next one or two served edges of `bal` (warp-uniform): lane's half
// takes the first (half 0) or the second (half 1); *j0 / *j1 get their lanes
// (*j1 = *j0 when there is one).
__device__ __forceinline__ void bb_pair(uint32_t &bal, uint32_t u, uint64_t m, uint32_t *uj, uint64_t *mj, int *j0,
		int *j1) {
	*j0 = __ffs(bal) - 1;
	bal &= bal - 1u;
	const bool two = bal != 0u;
	*j1 = two ? __ffs(bal) - 1 : *j0;
	bal &= bal - 1u;
	const int jm = (lane_id() & 16u) ? *j1 : *j0;
	*uj = __shfl_sync(kFull, u, jm);
	const uint64_t mm = bb_shfl64(m, jm);
	*mj = ((lane_id() & 16u) && !two) ? 0ull : mm;
}

// Adds a pair of served edges (vertex slots oa <= ob, this half's values x)
// to the open vertex, closing it and opening the next where the slot changes.
template <bool kFwd>
__device__ __forceinline__ void bb_add_pair(const BbArgs &a, uint32_t vb, uint64_t hv, int oa, int ob,
		const typename BbDir<kFwd>::T (&x)[4], int &cur, uint64_t &hcur, BbOpen<kFwd> &op, uint32_t &flushed) {
	const bool h1 = lane_id() & 16u;
	if (oa != cur) {
		if (cur >= 0) {
			bb_close<kFwd>(a, vb + cur, hcur, op);
			flushed |= 1u << cur;
		}
		cur = oa;
		hcur = bb_shfl64(hv, cur);
		bb_open<kFwd>(a, vb + cur, hcur, op);
	}
	if (ob == oa) {
#pragma unroll
		for (int i = 0; i < 4; ++i) op.acc[i] += x[i];
		return;
	}
	// the pair straddles two vertices: half 0's edge ends the open one
	if (!h1)
#pragma unroll
		for (int i = 0; i < 4; ++i) op.acc[i] += x[i];
	bb_close<kFwd>(a, vb + cur, hcur, op);
	flushed |= 1u << cur;
	cur = ob;
	hcur = bb_shfl64(hv, cur);
	bb_open<kFwd>(a, vb + cur, hcur, op);
	if (h1)
#pragma unroll
		for (int i = 0; i < 4; ++i) op.acc[i] += x[i];
}

// Block b of 32 consecutive vertices in one level of a sweep: those with at
// most kBbBig edges in the sweep's direction.  `has_nb`: the neighbour level
// exists (the reverse sweep's deepest level has none; its vertices get
// 1/sigma alone).
template <bool kFwd>
__device__ void bb_block(const BbArgs &a, uint32_t L, bool has_nb, uint32_t b, BbCount &cnt) {
	using D = BbDir<kFwd>;
	using T = typename D::T;
	const unsigned lane = lane_id();
	const uint64_t *own = bb_plane(a, L);
	const uint64_t *nb = bb_plane(a, kFwd ? L - 1 : L + 1);
	const uint32_t *off = D::off(a), *adj = D::adj(a);
	const uint32_t vb = b * 32, v = vb + lane;
	const uint64_t hv = v < a.n ? bb_word(own, a, v) : 0ull;
	uint32_t beg = 0, end = 0;
	if (hv) {
		beg = __ldg(off + v);
		end = __ldg(off + v + 1);
	}
	const bool part = hv != 0ull && end - beg <= kBbBig;
	const uint32_t pm = __ballot_sync(kFull, part);
	if (!pm) return;
	const uint32_t d = part && has_nb ? end - beg : 0u;
	const uint32_t incl = warp_incl_scan(d);
	const uint32_t excl = incl - d;
	const uint32_t total = __shfl_sync(kFull, incl, 31);
	int cur = -1;          // the open vertex's slot (warp-uniform)
	uint64_t hcur = 0;
	BbOpen<kFwd> op;
	uint32_t flushed = 0;
	for (uint32_t e0 = 0; e0 < total; e0 += 32) {
		const uint32_t e = e0 + lane;
		// the edge's vertex slot: the first lane whose inclusive prefix exceeds e
		uint32_t o = 0;
#pragma unroll
		for (uint32_t s = 16; s; s >>= 1) {
			const uint32_t x = __shfl_sync(kFull, incl, o + s - 1);
			if (x <= e) o += s;
		}
		const uint32_t obeg = __shfl_sync(kFull, beg, o), oex = __shfl_sync(kFull, excl, o);
		const uint64_t ohv = bb_shfl64(hv, o);
		uint32_t u = 0;
		uint64_t m = 0;
		if (e < total) {
			u = __ldg(adj + obeg + (e - oex));
			m = ohv & bb_word(nb, a, u);
		}
		uint32_t bal = __ballot_sync(kFull, m != 0ull);
		if (lane == 0) {
			cnt.edges += min(32u, total - e0);
			cnt.matched += __popc(bal);
		}
		cnt.served += __popcll(m);
		while (bal) {
			// kBbPairs pairs per round: their rows' loads in flight together
			uint32_t uj[kBbPairs];
			uint64_t mj[kBbPairs];
			int oa[kBbPairs], ob[kBbPairs];
			bool has[kBbPairs];
#pragma unroll
			for (int p = 0; p < kBbPairs; ++p) {
				int j0 = 0, j1 = 0;
				uj[p] = 0;
				mj[p] = 0;
				has[p] = bal != 0u;
				if (has[p]) bb_pair(bal, u, m, &uj[p], &mj[p], &j0, &j1);
				oa[p] = __shfl_sync(kFull, (int) o, j0);
				ob[p] = __shfl_sync(kFull, (int) o, j1);
			}
			T x[kBbPairs][4];
#pragma unroll
			for (int p = 0; p < kBbPairs; ++p) bb_vals<kFwd>(a, uj[p], mj[p], x[p]);
#pragma unroll
			for (int p = 0; p < kBbPairs; ++p)
				if (has[p]) bb_add_pair<kFwd>(a, vb, hv, oa[p], ob[p], x[p], cur, hcur, op, flushed);
		}
	}
	if (cur >= 0) {
		bb_close<kFwd>(a, vb + cur, hcur, op);
		flushed |= 1u << cur;
	}
	// vertices none of whose edges serve their sources (the deepest level,
	// sinks of the reverse sweep): nothing to add; two at a time, one per half
	for (uint32_t r = pm & ~flushed; r;) {
		const int j0 = __ffs(r) - 1;
		r &= r - 1u;
		const int j1 = r ? __ffs(r) - 1 : -1;
		if (r) r &= r - 1u;
		const int jm = (lane & 16u) ? j1 : j0;
		const uint64_t hj = bb_shfl64(hv, jm < 0 ? 0 : jm);
		if (jm >= 0) {
			const uint32_t bits = (uint32_t) (hj >> bb_quad()) & 0xFu;
			if (bits) {
				const size_t row = (size_t) (vb + jm) * 64 + bb_quad();
				uint32_t pre[4] = {0u, 0u, 0u, 0u};
				if (!kFwd) {
					const uint4 p = __ldcg(reinterpret_cast<const uint4 *>(a.sigma + row));
					pre[0] = p.x;
					pre[1] = p.y;
					pre[2] = p.z;
					pre[3] = p.w;
				}
#pragma unroll
				for (int i = 0; i < 4; ++i)
					if ((bits >> i) & 1u) D::store(a, row + i, T(0), pre[i]);
			}
		}
	}
}

// Chunk c (kBbChunk edges of a vertex with more than kBbBig edges) in one
// level of a sweep: the sums of its edges into partial[c].
template <bool kFwd>
__device__ void bb_chunk(const BbArgs &a, uint32_t L, bool has_nb, uint32_t c, uint32_t v, uint64_t hv,
		BbCount &cnt) {
	using D = BbDir<kFwd>;
	using T = typename D::T;
	const unsigned lane = lane_id();
	const uint64_t *nb = bb_plane(a, kFwd ? L - 1 : L + 1);
	const uint32_t *off = D::off(a), *adj = D::adj(a), *cb = D::chunk_beg(a);
	const uint32_t beg = __ldg(cb + c), end = min(beg + kBbChunk, __ldg(off + v + 1));
	T acc[4] = {T(0), T(0), T(0), T(0)};
	for (uint32_t e0 = beg; has_nb && e0 < end; e0 += 32) {
		const uint32_t e = e0 + lane;
		uint32_t u = 0;
		uint64_t m = 0;
		if (e < end) {
			u = __ldg(adj + e);
			m = hv & bb_word(nb, a, u);
		}
		uint32_t bal = __ballot_sync(kFull, m != 0ull);
		if (lane == 0) {
			cnt.edges += min(32u, end - e0);
			cnt.matched += __popc(bal);
		}
		cnt.served += __popcll(m);
		while (bal) {
			uint32_t uj[kBbPairs];
			uint64_t mj[kBbPairs];
#pragma unroll
			for (int p = 0; p < kBbPairs; ++p) {
				int j0, j1;
				uj[p] = 0;
				mj[p] = 0;
				if (bal) bb_pair(bal, u, m, &uj[p], &mj[p], &j0, &j1);
			}
			T x[kBbPairs][4];
#pragma unroll
			for (int p = 0; p < kBbPairs; ++p) bb_vals<kFwd>(a, uj[p], mj[p], x[p]);
#pragma unroll
			for (int p = 0; p < kBbPairs; ++p)
#pragma unroll
				for (int i = 0; i < 4; ++i) acc[i] += x[p][i];
		}
	}
#pragma unroll
	for (int i = 0; i < 4; ++i) acc[i] += __shfl_xor_sync(kFull, acc[i], 16);
	const uint32_t bits = (uint32_t) (hv >> bb_quad()) & 0xFu;
	if (lane < 16u && bits) {
		const size_t row = (size_t) c * 64 + bb_quad();
#pragma unroll
		for (int i = 0; i < 4; ++i)
			if ((bits >> i) & 1u) a.partial[row + i] = D::to_bits(acc[i]);
	}
}

// After the chunk sums of a level: each chunked vertex of that level adds its
// chunks' partial rows in chunk order (by the warp that meets its first chunk
// in the level's list).
template <bool kFwd>
__device__ void bb_finish(const BbArgs &a, uint32_t L) {
	using D = BbDir<kFwd>;
	using T = typename D::T;
	const uint32_t ncl = ld_volatile(kFwd ? &a.ctl->ni_at[L] : &a.ctl->no_at[L]);
	const uint32_t *clist = (kFwd ? a.ilist : a.olist) + (size_t) L * D::nchunks(a);
	const unsigned lane = lane_id();
	const uint64_t *own = bb_plane(a, L);
	const uint32_t *off = D::off(a), *cv = D::chunk_v(a), *cb = D::chunk_beg(a);
	const uint32_t gwarp = blockIdx.x * kBbWarps + warp_id(), nwarps = gridDim.x * kBbWarps;
	for (uint32_t i = gwarp; i < ncl; i += nwarps) {
		const uint32_t c = __ldcg(clist + i);
		const uint32_t v = __ldg(cv + c);
		const uint32_t b0 = __ldg(off + v);
		if (__ldg(cb + c) != b0) continue;
		const uint64_t hv = bb_word(own, a, v);
		const uint32_t k = (__ldg(off + v + 1) - b0 + kBbChunk - 1) / kBbChunk;
		const bool w0 = (hv >> lane) & 1ull, w1 = (hv >> (lane + 32)) & 1ull;
		T acc0 = T(0), acc1 = T(0);
		for (uint32_t i2 = 0; i2 < k; i2 += kBbUnroll) {
			T x0[kBbUnroll], x1[kBbUnroll];
#pragma unroll
			for (int j = 0; j < kBbUnroll; ++j) {
				const bool in = i2 + j < k;
				const size_t row = (size_t) (c + i2 + j) * 64;
				x0[j] = in && w0 ? D::from_bits(ld_cg(a.partial + row + lane)) : T(0);
				x1[j] = in && w1 ? D::from_bits(ld_cg(a.partial + row + lane + 32)) : T(0);
			}
#pragma unroll
			for (int j = 0; j < kBbUnroll; ++j) {
				acc0 += x0[j];
				acc1 += x1[j];
			}
		}
		bb_flush<kFwd>(a, v, hv, acc0, acc1, bb_pre<kFwd>(a, v, hv));
	}
}

// Lists, per level, of the blocks of 32 vertices and of the edge chunks
// that have a vertex at that level, so that a level's work is only its own
// (the planes are final once the traversal has ended).  A warp takes 32
// consecutive blocks (lane j: block j) or 32 chunks; one atomic per warp and
// level places them.
__device__ void bb_lists(const BbArgs &a, uint32_t depth) {
	BbControl *ctl = a.ctl;
	const unsigned lane = lane_id();
	const uint32_t gwarp = blockIdx.x * kBbWarps + warp_id(), nwarps = gridDim.x * kBbWarps;
	const uint32_t nblk = (a.n + 31) / 32;
	for (uint32_t wb = gwarp; wb * 32 < nblk; wb += nwarps) {
		for (uint32_t L = 0; L < depth; ++L) {
			const uint64_t *pl = bb_plane(a, L);
			uint32_t act = 0;
#pragma unroll 8
			for (uint32_t j = 0; j < 32; ++j) {
				const uint32_t v = (wb * 32 + j) * 32 + lane;
				const uint64_t h = v < a.n ? bb_word(pl, a, v) : 0ull;
				if (__any_sync(kFull, h != 0ull)) act |= 1u << j;
			}
			if (!act) continue;
			uint32_t base = 0;
			if (lane == 0) base = atomicAdd(&ctl->nb_at[L], (unsigned) __popc(act));
			base = __shfl_sync(kFull, base, 0);
			if ((act >> lane) & 1u) a.blist[(size_t) L * nblk + base + __popc(act & lanemask_lt())] = wb * 32 + lane;
		}
	}
	for (int dir = 0; dir < 2; ++dir) {
		const uint32_t nch = dir ? a.noch : a.nich;
		const uint32_t *cv = dir ? a.ochunk_v : a.ichunk_v;
		uint32_t *list = dir ? a.olist : a.ilist;
		unsigned *cnt = dir ? ctl->no_at : ctl->ni_at;
		for (uint32_t c0 = gwarp * 32; c0 < nch; c0 += nwarps * 32) {
			const uint32_t c = c0 + lane;
			const uint32_t v = c < nch ? __ldg(cv + c) : 0u;
			for (uint32_t L = 0; L < depth; ++L) {
				const bool at = c < nch && bb_word(bb_plane(a, L), a, v) != 0ull;
				const uint32_t m = __ballot_sync(kFull, at);
				if (!m) continue;
				uint32_t base = 0;
				if (lane == 0) base = atomicAdd(cnt + L, (unsigned) __popc(m));
				base = __shfl_sync(kFull, base, 0);
				if (at) list[(size_t) L * nch + base + __popc(m & lanemask_lt())] = c;
			}
		}
	}
}

// One level of a sweep: the level's chunks, then its blocks of 32 vertices,
// from the level's lists, handed out one at a time through a counter (the
// cost of a block varies with the edges of its vertices that serve a source;
// a fixed deal left warps waiting at the level's barrier).  The next item is
// claimed while the current one runs.
template <bool kFwd>
__device__ void bb_level(const BbArgs &a, uint32_t L, bool has_nb, unsigned *counter, BbCount &cnt) {
	using D = BbDir<kFwd>;
	const uint32_t nblk = (a.n + 31) / 32;
	const uint32_t ncl = ld_volatile(kFwd ? &a.ctl->ni_at[L] : &a.ctl->no_at[L]);
	const uint32_t nbl = ld_volatile(&a.ctl->nb_at[L]);
	const uint32_t *clist = (kFwd ? a.ilist : a.olist) + (size_t) L * D::nchunks(a);
	const uint32_t *blist = a.blist + (size_t) L * nblk;
	const uint32_t items = ncl + nbl;
	const unsigned lane = lane_id();
	uint32_t item = lane == 0 ? atomicAdd(counter, 1u) : 0u;
	item = __shfl_sync(kFull, item, 0);
	while (item < items) {
		const uint32_t next = lane == 0 ? atomicAdd(counter, 1u) : 0u;
		if (item < ncl) {
			const uint32_t c = __ldcg(clist + item);
			const uint32_t v = __ldg(D::chunk_v(a) + c);
			bb_chunk<kFwd>(a, L, has_nb, c, v, bb_word(bb_plane(a, L), a, v), cnt);
		} else {
			bb_block<kFwd>(a, L, has_nb, __ldcg(blist + (item - ncl)), cnt);
		}
		item = __shfl_sync(kFull, next, 0);
	}
}

__device__ __forceinline__ void bb_add_counts(unsigned long long *dst, const BbCount &c) {
	const unsigned long long served = warp_sum(c.served);
	if (lane_id() == 0) {
		if (c.edges) atomicAdd(dst, c.edges);
		if (c.matched) atomicAdd(dst + 1, c.matched);
		if (served) atomicAdd(dst + 2, served);
	}
}

__global__ void __launch_bounds__(kBbThreads, 2) k_bc_batch(BbArgs a) {
	BbControl *ctl = a.ctl;
	const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
	if (leader) ctl->t[0] = global_timer_ns();
	// the traversal's outcome decides for every CTA alike: its planes must hold
	// every level from 0 (no early output pass)
	const MsControl *ms = a.ms;
	const int ms_err = *(const volatile int *) &ms->err;
	const uint32_t complete = *(const volatile unsigned *) &ms->stats.complete;
	const uint32_t base = *(const volatile unsigned *) &ms->stats.base;
	const uint32_t spills = *(const volatile unsigned *) &ms->stats.spills;
	const uint32_t depth = *(const volatile unsigned *) &ms->stats.depth;
	if (ms_err || !complete || base || spills || depth == 0 || depth > a.planes) {
		if (leader) ctl->err = ms_err ? ms_err : BFS_EUNSUPPORTED;
		return;
	}
	if (leader) ctl->depth = depth;
	unsigned epoch = 0;
	const uint32_t t0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
	for (uint32_t v = t0; v < a.n; v += stride) {
		uint64_t h = bb_word(bb_plane(a, 0), a, v);
		while (h) {
			a.sigma[(size_t) v * 64 + (__ffsll((long long) h) - 1)] = 1u;
			h &= h - 1ull;
		}
	}
	bb_lists(a, depth);
	bool ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier);
	if (leader) ctl->t_fwd[0] = global_timer_ns();
	BbCount cf{0, 0, 0}, cr{0, 0, 0};
	for (uint32_t L = 1; ok && L < depth; ++L) {
		bb_level<true>(a, L, true, &ctl->work[0][L], cf);
		if (ld_volatile(&ctl->ni_at[L])) {
			if (!(ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier))) break;
			bb_finish<true>(a, L);
		}
		ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier);
		if (leader && L < kBbTraceLevels) ctl->t_fwd[L] = global_timer_ns();
	}
	if (leader) ctl->t[1] = global_timer_ns();
	for (int L = (int) depth - 1; ok && L >= 0; --L) {
		const bool has_nb = (uint32_t) L + 1 < depth;
		bb_level<false>(a, (uint32_t) L, has_nb, &ctl->work[1][L], cr);
		if (ld_volatile(&ctl->no_at[L])) {
			if (!(ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier))) break;
			bb_finish<false>(a, (uint32_t) L);
		}
		if (L > 0) ok = grid_sync(ctl->bar, epoch, &ctl->err, a.wait_limit_ns, a.hold_barrier);
		if (leader && (uint32_t) L < kBbTraceLevels) ctl->t_rev[L] = global_timer_ns();
	}
	if (leader) ctl->t[2] = global_timer_ns();
	bb_add_counts(ctl->fwd, cf);
	bb_add_counts(ctl->rev, cr);
}

// Output pass: [v][64] rows -> dependencies and path counts [source][v]
// (0 for unreached pairs) and/or acc[v] += dependencies of the sources != v,
// in source order; counts the vertices each source reached.
__global__ void __launch_bounds__(kBbOutThreads) k_bc_batch_out(BbArgs a, BbOut o) {
	if (*(const volatile int *) &a.ctl->err) return;
	__shared__ float sd[kBbOutV][kBbMaxSources + 1];
	__shared__ uint32_t sp[kBbOutV][kBbMaxSources + 1];
	__shared__ uint64_t svis[kBbOutV];
	__shared__ uint32_t ssrc[kBbMaxSources];
	const uint32_t t = threadIdx.x, ns = a.ns;
	if (t < kBbMaxSources) ssrc[t] = t < ns ? o.sources[t] : 0xFFFFFFFFu;
	const uint64_t smask = ns >= 64 ? ~0ull : (1ull << ns) - 1ull;
	uint32_t reached = 0;  // threads 64..127: vertices reached from source t - 64
	for (uint32_t v0 = blockIdx.x * kBbOutV; v0 < a.n; v0 += gridDim.x * kBbOutV) {
		const uint32_t nv = min(kBbOutV, a.n - v0);
		__syncthreads();
		if (t < nv) svis[t] = bb_ldg64(a.vis + (size_t) (v0 + t) * a.K + a.word) & smask;
		__syncthreads();
		// 16-byte loads: 4 sources of a row per thread (streamed, not kept in L2)
		for (uint32_t i = t; i < nv * 16; i += blockDim.x) {
			const uint32_t j = i / 16, s0 = 4 * (i % 16);
			const uint32_t r = (uint32_t) (svis[j] >> s0) & 0xFu;
			uint4 sg4 = make_uint4(0u, 0u, 0u, 0u), dv4 = make_uint4(0u, 0u, 0u, 0u);
			if (r) {
				const size_t x = (size_t) (v0 + j) * 64 + s0;
				sg4 = __ldcs(reinterpret_cast<const uint4 *>(a.sigma + x));
				dv4 = __ldcs(reinterpret_cast<const uint4 *>(a.dsum + x));
			}
			const uint32_t sg[4] = {sg4.x, sg4.y, sg4.z, sg4.w}, dv[4] = {dv4.x, dv4.y, dv4.z, dv4.w};
#pragma unroll
			for (int k = 0; k < 4; ++k) {
				const uint32_t g = ((r >> k) & 1u) ? sg[k] : 0u;
				const float inv = g ? 1.0f / (float) (int) g : 0.0f;
				sd[j][s0 + k] = inv != 0.0f ? (__uint_as_float(dv[k]) - inv) / inv : 0.0f;
				sp[j][s0 + k] = g;
			}
		}
		__syncthreads();
		if (o.delta || o.paths)
			for (uint32_t i = t; i < ns * kBbOutV; i += blockDim.x) {
				const uint32_t s = i / kBbOutV, j = i % kBbOutV;
				if (j >= nv) continue;
				const size_t x = (size_t) s * a.n + v0 + j;
				if (o.delta) __stcs(o.delta + x, sd[j][s]);
				if (o.paths) __stcs(o.paths + x, sp[j][s]);
			}
		if (o.acc && t < nv) {
			const uint32_t v = v0 + t;
			float x = o.acc[v];
			for (uint32_t s = 0; s < ns; ++s)
				if (ssrc[s] != v) x += sd[t][s];
			o.acc[v] = x;
		}
		if (t >= 64 && t < 64 + ns)
			for (uint32_t j = 0; j < nv; ++j) reached += (uint32_t) ((svis[j] >> (t - 64)) & 1ull);
	}
	if (t >= 64 && t < 64 + ns && reached) atomicAdd(&a.ctl->reached[t - 64], reached);
}

} // namespace

int bb_launch(const BbArgs &a, const BbOut &o, int num_sms, cudaStream_t st, int *grid, cudaEvent_t between) {
	if (a.ns == 0 || a.ns > kBbMaxSources) return BFS_EARG;
	int per_sm = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bc_batch, kBbThreads, 0) != cudaSuccess || per_sm < 1)
		return BFS_ECUDA;
	per_sm = std::min(per_sm, 2);
	if (a.ctas_per_sm) per_sm = std::min(per_sm, (int) a.ctas_per_sm);
	const int g = num_sms * per_sm;
	if (grid) *grid = g;
	if (cudaMemsetAsync(a.ctl, 0, sizeof(BbControl), st) != cudaSuccess) return BFS_ECUDA;
	BbArgs aa = a;
	void *args[] = {&aa};
	if (cudaLaunchCooperativeKernel((const void *) k_bc_batch, dim3(g), dim3(kBbThreads), args, 0, st) != cudaSuccess)
		return BFS_ECUDA;
	if (between && cudaEventRecord(between, st) != cudaSuccess) return BFS_ECUDA;
	int out_per_sm = 0;
	if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&out_per_sm, k_bc_batch_out, kBbOutThreads, 0) != cudaSuccess ||
			out_per_sm < 1)
		return BFS_ECUDA;
	k_bc_batch_out<<<num_sms * out_per_sm, kBbOutThreads, 0, st>>>(a, o);
	return cudaGetLastError() == cudaSuccess ? BFS_OK : BFS_ECUDA;
}

} // namespace bfsg
