// msbfs.h -- batched (bit-sliced multi-source) BFS: device arguments shared by
// msbfs.cu and the C ABI in api.cu.  Internal.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bfsg {

constexpr uint32_t kMsMaxLevel = 254;  // uint8 levels; 255 = unreached
constexpr uint32_t kMsTraceLevels = 64; // levels with per-level statistics
constexpr uint32_t kMsPullBig = 256;    // pull: destinations with more in-edges are split ...
constexpr uint32_t kMsChunk = 256;      // ... into chunks of this many in-edges
constexpr uint32_t kMsPushChunk = 1024; // push: high-degree vertices' edges go out in chunks of this many

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
	unsigned int base;             // level of plane 0 when the traversal ended
	unsigned int complete;         // 1: every level ran (the output pass may go)
	unsigned long long edges;      // frontier words (64-bit) read by pull levels
	unsigned long long traversed;  // sum over (source, reached vertex) of out-degree
	unsigned long long t_levels0;  // device clock (ns) when the first level starts
	unsigned long long t_levels1;  // ... and when the last one has ended
	unsigned long long t_start;    // device clock when the launch starts
	unsigned long long t_level[kMsTraceLevels + 1];  // device clock at the start of each level
	unsigned long long t_phase[kMsTraceLevels][2];   // ... after its first and second grid barrier
	unsigned int frontier[kMsTraceLevels];           // frontier vertices of each level
	unsigned char push[kMsTraceLevels];              // 1: the level was pushed
};

// Everything the launch needs zeroed; the host clears it with one memset.
struct MsControl {
	unsigned bar[2];
	int err;
	unsigned push_chunks;  // push level: 1024-edge chunks of its high-degree frontier vertices
	MsCounters ctr[3];
	MsStats stats;
	// active[l % 3][k]: OR of word k over level l's frontier rows -- the
	// sources that still have a frontier; only they can reach a vertex at
	// level l, so the pulls' completion tests ignore the others
	unsigned long long active[3][64];
};

struct MsArgs {
	uint32_t n, m;
	uint32_t K;           // 64-bit words per vertex
	uint32_t last_bits;   // sources in the last word (1..64)
	uint32_t planes;      // level planes allocated (>= 2)
	uint32_t push_div;    // a level pushes while its frontier's edges < m / push_div
	uint32_t nbig_in;     // destinations with more than kMsPullBig in-edges
	uint32_t nchunks;     // their in-edge chunks
	const uint32_t *row_off, *col, *in_off, *in_src;
	const uint32_t *in_big;              // [nbig_in] those destinations
	const uint32_t *chunk_v, *chunk_beg; // [nchunks] destination and first in-edge of each chunk
	uint32_t *push_u, *push_beg;         // [push_cap] push: vertex and first edge of each 1024-edge chunk
	uint32_t push_cap;
	uint64_t *vis;        // [n][K] sources that reached v
	uint64_t *hist;       // [planes][n][K] sources that reached v first at level base + plane
	uint64_t *pmask;      // [planes][n] bit k: word k of v's row in that plane is non-zero
	uint8_t *touched;     // [n] push: destination received a word
	uint8_t *done;        // [n] pull: every source has reached v (set by pulls; a hint)
	uint32_t *seed_flag;  // [n]
	uint32_t *queue[2];   // [n] frontier vertices by level parity (small front, big back)
	MsControl *ctl;
	unsigned long long wait_limit_ns;  // bound of every grid-barrier wait
	uint32_t hold_barrier;             // tests: CTA 0 skips its arrival at this barrier (0 = off)
	uint32_t ctas_per_sm;              // 0 = as many as fit (at most 2)
	uint32_t out_tile;                 // output pass tile width in vertices: 64, 128, or 0 = by graph size
};

// Enqueues the whole batched traversal (one cooperative launch and the
// output pass) on `st`; `between` and `between2` (either may be null) are
// recorded between the two;
// *grid receives the launch's CTA count.  levels == null: no output pass, the
// planes stay for a later pass, and a traversal deeper than the planes stops
// with BFS_EUNSUPPORTED.
int ms_launch(const MsArgs &a, const uint32_t *d_sources, uint32_t ns, uint8_t *levels, int num_sms, cudaStream_t st,
		int *grid, cudaEvent_t between, cudaEvent_t between2);

} // namespace bfsg
