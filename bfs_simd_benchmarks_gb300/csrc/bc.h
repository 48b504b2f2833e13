// bc.h -- betweenness-centrality dependencies of one source on the device
// (internal): the reference's BC() (apps/betweennessCentrality_simd/bc.cpp:
// 1717-2097) as one cooperative launch after a single-source traversal.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bfsg {

constexpr uint32_t kBcMaxLevels = 1u << 19;   // deeper traversals are refused (BFS_EUNSUPPORTED)
constexpr uint32_t kBcCntCap = 1u << 22;      // (level key, vertex range) counters of the level sort
constexpr uint32_t kBcBig = 1024;             // in- or out-degree above which a whole CTA reduces a vertex
constexpr uint32_t kBcMedium = 32;            // above this (and up to kBcBig) one warp reduces a vertex;
                                              // at most this, a warp takes 32 vertices at once
constexpr uint32_t kBcClasses = 7;            // sort keys per level: big, five medium degree bands
                                              // (highest first, so that warps dealt medium vertices in
                                              // turn get similar work), small
constexpr uint32_t kBcMaxGrid = 1024;
constexpr uint32_t kBcTraceLevels = 64;       // per-level timers and sizes kept for the first levels
static_assert(kBcClasses * kBcMaxLevels <= kBcCntCap, "every sort key needs a counter");
constexpr uint32_t kBcByteLevelsMinVertices = 1u << 22;  // default: byte levels from here (the 8-byte
                                                         // {level, value} array outgrows L2)
constexpr uint32_t kBcChunk = 4096;           // edges of a big vertex one CTA sums as one task
constexpr uint32_t kBcSmemBig = 4096;         // big vertices of a level whose chunk list every CTA keeps in shared
                                              // memory; a level with more builds it in global memory

// Chunk partial sums a graph of n vertices and m edges can need in one level.
inline size_t bc_partial_capacity(uint64_t n, uint64_t m) { return n + kBcSmemBig + m / kBcChunk + 2; }

struct BcControl {
	unsigned bar[2];            // grid barrier
	int err;                    // BFS_* status (0 ok)
	uint32_t depth;             // deepest level
	uint32_t reached;
	uint32_t pad;
	unsigned long long edges_fwd;      // in-edges read by the path-count sweep
	unsigned long long edges_rev;      // out-edges read by the dependency sweep
	unsigned long long edges_reached;  // sum of out-degrees of reached vertices
	unsigned long long t[4];           // global timer: start, sorted, path counts done, end
	unsigned long long t_fwd[kBcTraceLevels];  // end of the path counts of level d
	unsigned long long t_rev[kBcTraceLevels];  // end of the dependency sums of level d
	uint32_t lv_vertices[kBcTraceLevels];      // vertices of level d
	uint32_t lv_big[kBcTraceLevels];           // of which reduced by a whole CTA
	uint32_t lv_medium[kBcTraceLevels];        // of which reduced by one warp
	uint32_t blk[kBcMaxGrid];          // per-CTA totals of the counter scan
};

struct BcArgs {
	uint32_t n, source;
	uint32_t byte_levels;              // 1: test lv8 first (used when the traversal is at most 254 deep)
	const uint32_t *row_off, *col;     // CSR
	const uint32_t *in_off, *in_src;   // in-edge lists (the reverse graph)
	const int32_t *level;              // levels of the traversal from `source`, -1 unreached
	const uint32_t *num_steps;         // the traversal's step count (deepest level + 1)
	const int *bfs_status;             // the traversal's status word
	uint32_t *sigma;                   // [n] shortest-path counts (mod 2^32)
	uint8_t *lv8;                      // [n] levels as bytes (255: unreached or deeper than 254), checked
	                                   // first when the traversal is at most 254 levels deep (fits in L2)
	uint2 *lvx;                        // [n] {level, value}: the path count in the forward sweep, then the
	                                   // bits of the float sum (1 + dependency) / paths in the reverse one
	float *delta;                      // [n] dependencies (output)
	float *acc;                        // [n] or null: += dependency for every vertex but the source
	uint32_t *order;                   // [n] reached vertices sorted by (level, class: big, medium, small)
	uint32_t *cnt;                     // [kBcCntCap] counters of the level sort
	uint32_t *kstart;                  // [kBcClasses * kBcMaxLevels + 1] start of every key in `order`
	uint32_t *partial;                 // [bc_partial_capacity(n, m)] chunk sums of big vertices (value bits)
	uint32_t *cpre;                    // [n + 1] chunk prefix of a level with more than kBcSmemBig big vertices
	BcControl *ctl;
};

// Enqueues the dependency computation on `st` (after the traversal that wrote
// a.level).  The control block is cleared first.  *grid gets the CTA count.
int bc_launch(const BcArgs &a, int num_sms, cudaStream_t st, int *grid);

} // namespace bfsg
