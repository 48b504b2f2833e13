// bc_batch.h -- betweenness dependencies of many sources at once (64 per
// launch, up to 4 launches per call), on the bit-sliced batched traversal
// (internal).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "msbfs.h"

namespace bfsg {

constexpr uint32_t kBbMaxSources = 64;       // sources per launch: one 64-bit word of the traversal
constexpr uint32_t kBbMaxWords = 4;          // words per call (BFS_BC_BATCH_MAX_SOURCES = 256 sources)
constexpr uint32_t kBbBig = kMsPullBig;      // degree above which a vertex's edges are summed in chunks ...
constexpr uint32_t kBbChunk = kMsChunk;      // ... of this many edges (the batched pull's in-edge chunks)
constexpr uint32_t kBbTraceLevels = 64;      // per-level timers kept for the first levels

struct BbControl {
	unsigned bar[2];                 // grid barrier
	int err;                         // BFS_* status (0 ok)
	uint32_t depth;                  // levels of the traversal (deepest level + 1)
	// path-count sweeps (in-edges) / dependency sweeps (out-edges): edges read,
	// of which serving at least one source, and (edge, source) pairs summed
	unsigned long long fwd[3];
	unsigned long long rev[3];
	unsigned long long t[3];         // global timer: start, path counts done, dependencies done
	unsigned long long t_fwd[kBbTraceLevels];  // end of the path counts of level d (d = 0: the seeds)
	unsigned long long t_rev[kBbTraceLevels];  // end of the dependency sums of level d
	unsigned int reached[kBbMaxSources];  // vertices reached from each source (output pass)
	unsigned int work[2][kMsMaxLevel + 1];  // per sweep and level: next work item (chunks, then vertex blocks)
	unsigned int nb_at[kMsMaxLevel + 1];    // per level: blocks of 32 vertices with a vertex at that level
	unsigned int ni_at[kMsMaxLevel + 1];    // ... in-edge chunks whose vertex is at that level
	unsigned int no_at[kMsMaxLevel + 1];    // ... out-edge chunks
};

struct BbArgs {
	uint32_t n, ns;                    // ns: sources of this launch's word (1..64)
	uint32_t K, word;                  // the traversal's words per vertex; the word this launch takes
	const uint32_t *row_off, *col;     // CSR
	const uint32_t *in_off, *in_src;   // in-edge lists
	const uint64_t *hist;              // [planes][n][K]: sources that reached v first at level L
	const uint64_t *vis;               // [n][K] sources that reached v
	const MsControl *ms;               // the traversal's control block (depth, completion, status)
	const uint32_t *ichunk_v, *ichunk_beg;  // in-edge chunks of vertices with in-degree > kBbBig
	uint32_t nich;
	const uint32_t *ochunk_v, *ochunk_beg;  // out-edge chunks of vertices with out-degree > kBbBig
	uint32_t noch;
	uint32_t *sigma;                   // [n][64] path counts (mod 2^32)
	float *dsum;                       // [n][64] 1/sigma + the dependency sums of the next level
	uint32_t *partial;                 // [max(nich, noch)][64] chunk sums (value bits)
	// per level L < planes, built at the start of the launch (any order):
	uint32_t *blist;                   // [planes][ceil(n / 32)] blocks of 32 vertices with a vertex at level L
	uint32_t *ilist;                   // [planes][nich] in-edge chunks of vertices at level L
	uint32_t *olist;                   // [planes][noch] out-edge chunks of vertices at level L
	uint32_t planes;                   // levels the lists have room for
	BbControl *ctl;
	unsigned long long wait_limit_ns;  // bound of every grid-barrier wait
	uint32_t hold_barrier;             // tests: CTA 0 skips its arrival at this barrier (0 = off)
	uint32_t ctas_per_sm;              // 0 = as many as fit (at most 2)
};

struct BbOut {
	const uint32_t *sources;  // [ns] device
	float *delta;             // [ns][n] dependencies, or null
	uint32_t *paths;          // [ns][n] path counts, or null
	float *acc;               // [n] or null: += the dependency of each source s on v (v != s), sources in order
};

// Enqueues, after the batched traversal that filled a.hist / a.vis / a.ms,
// the cooperative path-count and dependency launch for the sources of word
// a.word and the output pass; the control block is cleared first.  `between` (may be null) is recorded
// between the two launches; *grid gets the CTA count.
int bb_launch(const BbArgs &a, const BbOut &o, int num_sms, cudaStream_t st, int *grid, cudaEvent_t between);

} // namespace bfsg
