/*
 * svml_shim.h -- force-included when the reference's apps/bfs_simd/bfs.cpp is
 * compiled with g++ for the oracle (it uses two icc/SVML-only intrinsics at
 * bfs.cpp:71, :79, :214, :241).  Both are written here from their documented
 * meaning: lane-wise signed 32-bit division truncating toward zero, the masked
 * form keeping `src` in lanes whose mask bit is clear.  Checker only; never
 * part of the product.
 */
#ifndef ORACLE_SVML_SHIM_H
#define ORACLE_SVML_SHIM_H
#include <immintrin.h>

static inline __m512i oracle_lanewise_div(__m512i src, __mmask16 k, __m512i a, __m512i b)
{
	int num[16], den[16], out[16];
	_mm512_storeu_si512((void *) num, a);
	_mm512_storeu_si512((void *) den, b);
	_mm512_storeu_si512((void *) out, src);
	for (int lane = 0; lane < 16; ++lane)
		if ((k >> lane) & 1) out[lane] = num[lane] / den[lane];
	return _mm512_loadu_si512((const void *) out);
}

static inline __m512i _mm512_div_epi32(__m512i a, __m512i b)
{
	return oracle_lanewise_div(_mm512_setzero_si512(), (__mmask16) 0xFFFF, a, b);
}

static inline __m512i _mm512_mask_div_epi32(__m512i src, __mmask16 k, __m512i a, __m512i b)
{
	return oracle_lanewise_div(src, k, a, b);
}
#endif
