// internal.h -- host-side structures shared by the loader, the layout builder
// and the CUDA runtime of libbfs_gb300.so.  Not part of the public ABI.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/bfs_gb300.h"

namespace bfsg {

constexpr unsigned kNumSplitFiles = 64;   // the 64-way split of every text family
constexpr uint32_t kUnvisited = 0xFFFFFFFFu;
constexpr uint32_t kSentinel = 0xFFFFFFFFu; // padding word of the packed tile stream

inline uint32_t side_length_of(uint32_t n, uint32_t w) { return (n % w) ? n / w + 1 : n / w; }
inline uint32_t ceil_log2(uint64_t x) {
	uint32_t b = 0;
	while ((uint64_t(1) << b) < x) ++b;
	return b;
}
inline void split_range(uint64_t m, unsigned tid, uint64_t *lo, uint64_t *hi) {
	uint64_t bound = m / kNumSplitFiles;
	*lo = tid * bound;
	*hi = (tid != kNumSplitFiles - 1) ? *lo + bound : m;
}

// The arrays the reference's graph_input builds (apps/bfs_simd/bfs.cpp:968-1118),
// 0-based, plus what the GPU layout derives from them.
struct HostGraph {
	uint32_t n = 0;
	uint64_t m = 0;
	uint32_t w = 0, s = 0, side = 0, num_stripes = 0;
	std::vector<uint32_t> degrees;   // [n] out-degree (_untiled-nneibor)
	std::vector<uint32_t> row_off;   // [n+1] CSR row starts
	std::vector<uint32_t> csr_dst;   // [m] CSR destinations in file order
	std::vector<uint32_t> heads;     // [m] column-major COO sources
	std::vector<uint32_t> tails;     // [m] column-major COO destinations
	std::vector<uint32_t> tile_offsets; // [side*side] first edge of each tile (col-major numbering), may be empty
	uint32_t max_degree = 0;
	std::string base;
	bool used_reorder = false;
};

// The packed column-major stream the bottom-up kernel reads (see layout.cpp).
struct PackedTiles {
	uint32_t vbits = 0, cbits = 0, ubits = 0;
	uint32_t num_groups = 0;
	uint32_t max_group_vertices = 0;
	std::vector<uint32_t> group_col;  // [num_groups+1] first tile column of each group
	std::vector<uint32_t> seg_off;    // [num_stripes*num_groups+1] word offset of segment (stripe, group)
	std::vector<uint32_t> words;      // packed edges + sentinel padding
	std::vector<uint32_t> hasin_bits; // [ceil(n/32)] bit v set when v has an in-edge
};

// host_io.cpp
int read_split_family(const std::string &prefix, uint64_t m, bool weighted, uint32_t n,
		uint32_t *a, uint32_t *b);
int read_header(const std::string &path, uint32_t *n, uint64_t *m);
int read_u32_lines(const std::string &path, uint64_t count, uint32_t *out);
int write_split_family(const std::string &prefix, uint32_t n, uint64_t m, const uint32_t *a,
		const uint32_t *b, const uint32_t *weights);
int write_u32_lines(const std::string &path, const uint32_t *v, uint64_t count);
bool file_exists(const std::string &path);

// layout.cpp
int csr_from_edges(uint32_t n, uint64_t m, const uint32_t *src, const uint32_t *dst,
		std::vector<uint32_t> &csr_src, std::vector<uint32_t> &csr_dst, std::vector<uint32_t> &degrees);
int colmajor_from_csr(uint32_t n, uint64_t m, uint32_t w, uint32_t s, const uint32_t *csr_src,
		const uint32_t *csr_dst, std::vector<uint32_t> &heads, std::vector<uint32_t> &tails,
		std::vector<uint32_t> *tile_offsets);
int validate_colmajor(const HostGraph &g);
int finish_csr(HostGraph &g);
int pack_tiles(const HostGraph &g, uint32_t target_groups, uint32_t max_group_vertices, PackedTiles &out);
// the parts of pack_tiles the device build shares: column groups from the
// in-edges per tile column, a group's padding word, segment offsets (padded)
int plan_groups(uint32_t n, uint32_t w, uint32_t s, uint32_t side, const std::vector<uint64_t> &col_edges,
		uint64_t m, uint32_t target_groups, uint32_t max_group_vertices, PackedTiles &out);
uint32_t group_pad_word(const PackedTiles &out, uint32_t gi, uint32_t n, uint32_t w);
int segment_offsets(const std::vector<uint64_t> &seg_count, PackedTiles &out);

// small parallel helper
unsigned host_threads();
template <class F> void parallel_for(uint64_t n, F &&f);

} // namespace bfsg

#include <thread>
namespace bfsg {
template <class F> void parallel_for(uint64_t n, F &&f) {
	unsigned t = host_threads();
	if (n < 2 || t <= 1) {
		f(uint64_t(0), n, 0u);
		return;
	}
	if (t > n) t = (unsigned) n;
	std::vector<std::thread> th;
	th.reserve(t);
	for (unsigned i = 0; i < t; ++i) {
		uint64_t lo = n * i / t, hi = n * (i + 1) / t;
		th.emplace_back([&f, lo, hi, i]() { f(lo, hi, i); });
	}
	for (auto &x : th) x.join();
}
} // namespace bfsg
