// bfs_device.cuh -- device-side data structures of the single-source BFS.
#pragma once

#include <cstdint>

namespace bfsg {

// Upper bound of the persistent grid: per-CTA partial sums are indexed by CTA.
constexpr uint32_t kMaxGrid = 2048;

// The graph as it sits in HBM (all read-only during a traversal).
struct DevGraph {
	uint32_t n;            // vertices
	uint32_t m;            // edges (< 2^32, like the reference's NEDGES)
	uint32_t w, s;         // tile width, stripe length
	uint32_t side;         // ceil(n / w)
	uint32_t num_stripes;  // ceil(side / s)
	uint32_t sw;           // s * w : sources per stripe
	uint32_t vbits, cbits, ushift;
	uint32_t vmask, cmask;
	uint32_t num_groups;
	uint32_t max_group_words;   // 32-bit words of the largest group bitmap
	uint32_t slice_words;       // 32-bit words of one stripe's frontier slice
	uint32_t nwords;            // ceil(n / 32)
	uint32_t bm_words;          // words of a frontier bitmap, padded to whole stripe slices
	uint32_t tma;               // 1: the bottom-up step streams segments and slices with bulk copies
	uint32_t tma_batch;         // frontier slices per bulk-copy stage
	uint32_t pull_long_cap;     // shared-memory queue of destinations needing a long in-edge scan
	const uint32_t *row_off;    // [n+1] CSR row starts
	const uint32_t *col;        // [m]   CSR destinations
	const uint32_t *packed;     // packed column-major stream (16-byte aligned segments)
	const uint32_t *seg_off;    // [num_groups*num_stripes+1], group-major
	const uint32_t *group_col;  // [num_groups+1]
	const uint32_t *hasin;      // [nwords] in-degree > 0
	const uint32_t *in_off;     // [n+1] in-edge list starts (destination-sorted column tiles)
	const uint32_t *in_src;     // [m]   sources of the in-edges, ascending within a list
};

// Counters of the frontier a step produces (three slots rotate by step).
struct StepCounters {
	unsigned int tail[3];       // queue bucket tails (top-down appends, to_sparse)
	unsigned int work;          // dynamic work counter (column groups)
};

// Per-run statistics gathered on the device.
struct DevStats {
	unsigned long long td_edges;
	unsigned long long td_vertices;
	unsigned long long bu_words;
	unsigned long long bu_slices;
	unsigned long long bu_groups;
	unsigned long long bu_vertices;   // destinations tested by pull steps
	unsigned long long reached;
	unsigned long long edges_traversed;
	unsigned int num_steps;
	unsigned int dense_steps;
	int status;
	unsigned int pad;
	unsigned char trace[256];
	// globaltimer stamps taken by CTA 0 after the grid barriers: the start of
	// every step and the end of its queue<->bitmap conversion (if any)
	unsigned long long t_step[257];
	unsigned long long t_conv[256];
	// per step, over the CTAs: the latest and (bit-inverted) the earliest
	// globaltimer stamp at which a CTA had finished the step's work
	unsigned long long t_work_max[256];
	unsigned long long t_work_min_inv[256];
	// SM cycles summed over CTAs inside the bottom-up step: group setup,
	// window lists, consumer wait, consumer work, producer wait, publish
	unsigned long long bu_cycles[8];
};

// Scratch of one traversal context (owned by the graph's run context).
struct RunCtx {
	int32_t *level;        // [n] output levels
	uint32_t *parent;      // [n] output parents (may be null)
	uint32_t *vis;         // [nwords] visited bitmap
	uint32_t *bm[3];       // [nwords] rotating frontier bitmaps
	uint8_t *sf[3];        // [num_stripes] rotating "stripe has a frontier vertex" flags
	uint32_t *q[2][3];     // [2 sets][3 buckets][n] frontier queues
	StepCounters *ctr;     // [3]
	unsigned long long *part;  // [3 slots][2 (count, degsum)][kMaxGrid] per-CTA step totals
	DevStats *stats;
	unsigned *bar;         // [2] grid barrier: arrival count, exits (0 between launches)
	int *err;              // device status word
};

struct StepParams {
	uint32_t source;
	uint32_t warp_max_degree;
	uint32_t cta_max_degree;
	uint32_t bottom_up;   // 0: pull over in-edge lists, 1: stream the packed tiles
	unsigned long long to_dense_threshold;   // dense when frontier + degsum > this
	unsigned long long to_sparse_threshold;  // stay dense while frontier + degsum > this
	unsigned long long wait_limit_ns;        // bound of every grid-barrier wait
	uint32_t hold_barrier;                   // tests: CTA 0 skips its arrival at this barrier (0 = off)
	uint32_t switch_rule;                    // 0: thresholds above; 1: out-edges of the unvisited (alpha, beta)
	uint32_t alpha, beta;
};

} // namespace bfsg
