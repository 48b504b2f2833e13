// msbfs.h -- batched (bit-sliced multi-source) BFS: device arguments shared by
// msbfs.cu and the C ABI in api.cu.  Internal.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bfsg {

constexpr uint32_t kMsMaxLevel = 254;  // uint8 levels; 255 = unreached

struct MsCounters {
	unsigned int nact;            // frontier vertices of degree <= kMsBig (queue front)
	unsigned int nbig;            // frontier vertices of higher degree (queue back)
	unsigned long long act_deg;   // out-degree sum of the frontier (push cost estimate)
};

struct MsStats {
	unsigned int levels;           // levels expanded
	unsigned int push_levels;      // of which top-down
	unsigned int depth;            // level whose frontier came out empty
	unsigned int spills;           // times the level planes filled up and were written out early
	unsigned long long edges;      // in-neighbour frontier rows gathered by pull levels
	unsigned long long traversed;  // sum over (source, reached vertex) of out-degree
	unsigned long long t_levels0;  // device clock (ns) when the first level starts
	unsigned long long t_levels1;  // ... and when the last one has ended
};

// Everything the launch needs zeroed; the host clears it with one memset.
struct MsControl {
	unsigned bar[2];
	int err;
	int pad;
	MsCounters ctr[3];
	MsStats stats;
};

struct MsArgs {
	uint32_t n, m;
	uint32_t K;           // 64-bit words per vertex
	uint32_t last_bits;   // sources in the last word (1..64)
	uint32_t planes;      // level planes allocated (>= 2)
	uint32_t push_div;    // a level pushes while its frontier's edges < m / push_div
	uint32_t vec_out;     // levels rows start 16-byte aligned (16-byte stores)
	const uint32_t *row_off, *col, *in_off, *in_src;
	uint64_t *vis;        // [n][K] sources that reached v
	uint64_t *hist;       // [planes][n][K] sources that reached v first at level base + plane
	uint8_t *act[2];      // [n] frontier vertex flags by level parity
	uint8_t *touched;     // [n] push: destination received a word
	uint32_t *seed_flag;  // [n]
	uint32_t *queue[2];   // [n] frontier vertices by level parity (small front, big back)
	MsControl *ctl;
};

// Enqueues the whole batched traversal (one cooperative launch) on `st`;
// *grid receives the launch's CTA count.
int ms_launch(const MsArgs &a, const uint32_t *d_sources, uint32_t ns, uint8_t *levels, int num_sms, cudaStream_t st,
		int *grid);

} // namespace bfsg
