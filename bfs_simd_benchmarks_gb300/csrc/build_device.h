// build_device.h -- kernels that build a graph's device layout from an edge
// list (build_device.cu).  Internal.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bfsg {

struct DeviceBuildShape {
	uint32_t w, s, stripes;
	uint32_t vbits, cbits;
};

// out_deg[u]++ / in_deg[v]++ per edge (both zeroed by the caller); an id
// >= n sets *err to BFS_EFORMAT.
int dbuild_degrees(const uint32_t *src, const uint32_t *dst, uint64_t m, uint32_t n, uint32_t *out_deg,
		uint32_t *in_deg, int *err, int num_sms, cudaStream_t st);
// out[0..n] = exclusive prefix sums of in[0..n) (out[n] = total); tmp holds
// dbuild_scan_tmp_words(n) words.
uint32_t dbuild_scan_tmp_words(uint32_t n);
int dbuild_exclusive_scan(const uint32_t *in, uint32_t n, uint32_t *tmp, uint32_t *out, cudaStream_t st);
// out[cursor[key[i]]++] = val[i]
int dbuild_scatter(const uint32_t *key, const uint32_t *val, uint64_t m, uint32_t *cursor, uint32_t *out, int num_sms,
		cudaStream_t st);
// in-edges per tile column and the has-in-edge bitmap (both zeroed by the caller)
int dbuild_col_hist(const uint32_t *dst, uint64_t m, uint32_t w, uint32_t side, uint32_t *col_edges, uint32_t *hasin,
		int num_sms, cudaStream_t st);
// edges per packed segment (group(v) * stripes + stripe(u)), zeroed by the caller
int dbuild_seg_hist(const uint32_t *src, const uint32_t *dst, uint64_t m, const DeviceBuildShape &sh,
		const uint32_t *group_of, uint32_t *seg_count, int num_sms, cudaStream_t st);
// packed words into their segments (cursor = a copy of the segment offsets)
int dbuild_seg_fill(const uint32_t *src, const uint32_t *dst, uint64_t m, const DeviceBuildShape &sh,
		const uint32_t *group_of, const uint32_t *group_col, uint32_t *cursor, uint32_t *words, int num_sms,
		cudaStream_t st);
// padding words after each segment's edges
int dbuild_seg_pad(const uint32_t *seg_off, const uint32_t *seg_count, uint64_t nseg, uint32_t stripes,
		const uint32_t *pad_word, uint32_t *words, int num_sms, cudaStream_t st);

} // namespace bfsg
