// rmat_common.h -- the definition of an R-MAT candidate edge, shared by the
// host generator (rmat.cpp) and the device generator (rmat_device.cu) so that
// both draw the same edge list.  Internal.
//
// Candidate i draws its quadrant bits from a counter-based hash (splitmix64
// of the mixed seed and i), so the list does not depend on the thread count,
// the platform or the device.  With d = 1-a-b-c, one level picks
//   (u,v) bits (0,0) with a, (0,1) with b, (1,0) with c, (1,1) with d.
// The scale is ceil(log2 N); ids >= N are rejected (and self loops, on
// request).
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define BFSG_HD __host__ __device__
#else
#define BFSG_HD
#endif

namespace bfsg {
namespace rmat {

BFSG_HD inline uint64_t splitmix64(uint64_t x) {
	x += 0x9E3779B97F4A7C15ull;
	x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
	x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
	return x ^ (x >> 31);
}

struct Thresholds {
	uint32_t ta, tab, tabc;
};

inline uint32_t to_threshold(double p) {
	if (p <= 0) return 0;
	if (p >= 1) return 0xFFFFFFFFu;
	return (uint32_t) (p * 4294967296.0);
}

// The generator's seed after mixing (the value every candidate hash uses).
inline uint64_t mixed_seed(uint64_t seed) { return splitmix64(seed ^ 0x5851F42D4C957F2Dull); }

// Candidate `i`: returns false when rejected (id out of range or self loop).
BFSG_HD inline bool candidate(uint64_t seed, uint64_t i, uint32_t scale, uint32_t n, const Thresholds &t,
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

// The relabelling of BFS_RMAT_PERMUTE: a Fisher-Yates shuffle driven by the
// mixed seed (sequential: every swap depends on the previous state).
template <class Vec> inline void permutation(uint64_t mixed, uint32_t n, Vec &perm) {
	perm.resize(n);
	for (uint32_t v = 0; v < n; ++v) perm[v] = v;
	uint64_t st = splitmix64(mixed ^ 0xD1B54A32D192ED03ull);
	for (uint32_t v = n - 1; v > 0; --v) {
		st = splitmix64(st);
		const uint32_t j = (uint32_t) (((unsigned __int128) st * (uint64_t) (v + 1)) >> 64);
		const uint32_t x = perm[v];
		perm[v] = perm[j];
		perm[j] = x;
	}
}

}  // namespace rmat
}  // namespace bfsg
