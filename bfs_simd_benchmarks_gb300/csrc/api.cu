// api.cu -- the C ABI of libbfs_gb300.so: graph handles, loading and upload,
// single-source runs.  See include/bfs_gb300.h for the reference interface
// each entry point replaces.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "build_device.h"
#include "internal.h"
#include "kernels_api.h"
#include "bc.h"
#include "bc_batch.h"
#include "msbfs.h"

using namespace bfsg;

namespace {

constexpr uint32_t kMaxGroupVertices = 32768;  // shared-memory bitmaps of one column group
constexpr uint32_t kGroupsPerCta = 1;
constexpr uint32_t kBatchDefaultPlanes = 32; // level planes when sized from the budget

struct DevBuf {
	void *p = nullptr;
	size_t bytes = 0;
};

} // namespace

struct bfs_graph {
	// host-side description
	uint32_t n = 0;
	uint64_t m = 0;
	uint32_t w = 0, s = 0, side = 0, num_stripes = 0;
	uint32_t max_degree = 0;
	std::string base;
	bool used_reorder = false;
	bool host_only = false;
	std::vector<uint32_t> degrees;  // kept for info / tests
	// device
	int device = 0;
	int num_sms = 0;
	DevGraph dg{};
	RunCtx rc{};
	uint32_t batch = 1;
	int grid = 0;
	int grid_max = 0;  // CTAs of the cooperative grid at full occupancy (grid: as the options ask)
	size_t smem = 0;
	std::vector<DevBuf> bufs;
	size_t device_bytes = 0;
	int32_t *level_buf = nullptr;    // internal outputs for bfs_run
	uint32_t *parent_buf = nullptr;
	// BFS_LOAD_DEGREE_ORDER: the device layout uses ids ranked by out-degree;
	// callers' ids are mapped in (sources) and out (levels, parents)
	bool relabeled = false;
	std::vector<uint32_t> new_of_old;
	uint32_t *d_new_of_old = nullptr, *d_old_of_new = nullptr;
	int32_t *rl_level = nullptr;     // a run's outputs in the layout's ids
	uint32_t *rl_parent = nullptr;
	DevStats *h_stats = nullptr;     // pinned
	unsigned long long *h_part = nullptr;  // pinned (stepwise mode): one slot's per-CTA partials
	cudaEvent_t ev0 = nullptr, ev1 = nullptr, evm = nullptr;
	cudaStream_t last_stream = nullptr;
	bool stats_fresh = false;
	bool have_run = false;
	bool stepwise_last = false;
	bfs_stats host_stats{};          // stepwise-mode bookkeeping
	bfs_options opt{};
	uint32_t num_groups = 0;
	uint64_t packed_words = 0;
	// batched pull: destinations with many in-edges, cut into chunks
	const uint32_t *ms_in_big = nullptr, *ms_chunk_v = nullptr, *ms_chunk_beg = nullptr;
	uint32_t ms_nbig_in = 0, ms_nchunks = 0;
	// batched traversal state, allocated by the first bfs_run_batch
	struct Batch {
		uint32_t k_alloc = 0;        // words per vertex the buffers hold
		uint32_t planes_alloc = 0;   // level planes they hold
		MsArgs args{};
		uint32_t *d_sources = nullptr;
		MsControl *h_ctl = nullptr;  // pinned
		cudaEvent_t e0 = nullptr, e1 = nullptr, em = nullptr;
		cudaStream_t stream = nullptr;
		uint32_t num_sources = 0;
		int grid = 0;
		bool have_run = false, fresh = false;
		bool singles = false;        // the last batch ran as single-source traversals
		bool em_valid = false;       // em marks the last batch's traversal end
		size_t bytes = 0;
		std::vector<DevBuf> bufs;
	} mb;
	// betweenness state, allocated by the first bfs_bc_* call
	struct Bc {
		uint32_t *sigma = nullptr, *order = nullptr, *cnt = nullptr, *kstart = nullptr, *partial = nullptr;
		uint32_t *cpre = nullptr;
		float *delta = nullptr, *acc = nullptr;
		uint2 *lvx = nullptr;
		uint8_t *lv8 = nullptr;
		BcControl *ctl = nullptr;
		BcControl *h_ctl = nullptr;  // pinned
		cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
		cudaStream_t stream = nullptr;   // of the last enqueued run
		int grid = 0;
		size_t bytes = 0;
		std::vector<DevBuf> bufs;
	} bc;
	// batched betweenness state, allocated by the first batched bfs_bc_* call
	struct BcBatch {
		uint32_t *sigma = nullptr, *partial = nullptr, *d_sources = nullptr;
		float *dsum = nullptr;
		float *delta = nullptr;      // [64][n] staging of host outputs (allocated when first asked for)
		uint32_t *paths = nullptr;
		uint32_t *blist = nullptr, *ilist = nullptr, *olist = nullptr;  // per-level work lists
		uint32_t list_planes = 0;    // levels they have room for
		std::vector<DevBuf> lbufs;
		BbControl *ctl = nullptr;
		BbControl *h_ctl = nullptr;  // pinned
		MsControl *h_ms = nullptr;   // pinned: the traversal's control block
		cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr, e3 = nullptr;
		cudaStream_t stream = nullptr;
		uint32_t ns = 0;
		uint32_t words = 0;          // words (launches) of the last batch
		int grid = 0;
		size_t bytes = 0;
		std::vector<DevBuf> bufs;
	} bb;
	// out-edge chunks of vertices with many out-edges (batched betweenness)
	const uint32_t *bb_ochunk_v = nullptr, *bb_ochunk_beg = nullptr;
	uint32_t bb_noch = 0;
	bool bb_chunks_ready = false;
	bool bc_last_batched = false;    // bfs_bc_last_stats describes a batched run
	std::mutex mu;
};

namespace {

int cuda_ok(cudaError_t e) { return e == cudaSuccess ? BFS_OK : BFS_ECUDA; }

// Bound of the device-side waits of a run, from the options (0 = default).
uint64_t wait_limit_ns(const bfs_options &o) {
	return o.wait_limit_us ? (uint64_t) o.wait_limit_us * 1000ull : 2000000000ull;  // default 2 s
}

// The degree order of tools/vertex_id_reorder_to_degrees (bfs.cpp:50-80)
// with a deterministic tie-break: new ids by out-degree descending, equal
// degrees by ascending old id (a stable counting sort by degree).  The tool
// breaks ties with rand(); this order is the project's own.
std::vector<uint32_t> degree_order(const std::vector<uint32_t> &deg) {
	const uint32_t n = (uint32_t) deg.size();
	uint32_t maxd = 0;
	for (uint32_t d : deg) maxd = std::max(maxd, d);
	std::vector<uint64_t> start((size_t) maxd + 2, 0);
	for (uint32_t d : deg) start[maxd - d + 1]++;  // bucket maxd - d: highest degree first
	for (size_t b = 1; b < start.size(); ++b) start[b] += start[b - 1];
	std::vector<uint32_t> new_of_old(n);
	for (uint32_t v = 0; v < n; ++v) new_of_old[v] = (uint32_t) start[maxd - deg[v]]++;
	return new_of_old;
}

__global__ void k_relabel_edges(uint64_t m, const uint32_t *new_of_old, uint32_t *src, uint32_t *dst) {
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t) gridDim.x * blockDim.x) {
		src[i] = __ldg(new_of_old + src[i]);
		dst[i] = __ldg(new_of_old + dst[i]);
	}
}

// levels[v] / parents[v] in the caller's ids from a run in the layout's ids
__global__ void k_unrelabel(uint32_t n, const uint32_t *new_of_old, const uint32_t *old_of_new, const int32_t *lv_new,
		const uint32_t *pa_new, int32_t *levels, uint32_t *parents) {
	for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
		const uint32_t x = __ldg(new_of_old + v);
		levels[v] = lv_new[x];
		if (parents) {
			const uint32_t p = pa_new[x];
			parents[v] = p == 0xFFFFFFFFu ? p : __ldg(old_of_new + p);
		}
	}
}

// Device array -> host memory the device can write (pinned and mapped):
// 16-byte stores when both ends are 16-byte aligned, else 4-byte ones.
__global__ void k_to_host(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst, size_t words, bool wide) {
	const size_t t0 = (size_t) blockIdx.x * blockDim.x + threadIdx.x, stride = (size_t) gridDim.x * blockDim.x;
	if (wide) {
		const size_t q = words / 4;
		for (size_t i = t0; i < q; i += stride)
			reinterpret_cast<uint4 *>(dst)[i] = __ldcs(reinterpret_cast<const uint4 *>(src) + i);
		for (size_t i = 4 * q + t0; i < words; i += stride) dst[i] = __ldcs(src + i);
	} else {
		for (size_t i = t0; i < words; i += stride) dst[i] = __ldcs(src + i);
	}
}

// Enqueues the copy of `words` 32-bit words from device memory to a host
// buffer on `st`: pinned host memory mapped into the device's address space
// is written by a copy kernel (no copy-engine round trip), any other host
// memory goes through cudaMemcpyAsync.
int enqueue_to_host(uint32_t *dst, const uint32_t *src, size_t words, int num_sms, cudaStream_t st) {
	if (!dst || !words) return BFS_OK;
	cudaPointerAttributes at{};
	if (cudaPointerGetAttributes(&at, dst) != cudaSuccess) {
		cudaGetLastError();
		at.type = cudaMemoryTypeUnregistered;
	}
	if (at.type == cudaMemoryTypeHost && at.devicePointer) {
		uint32_t *d = (uint32_t *) at.devicePointer;
		const bool wide = ((uintptr_t) d % 16) == 0 && ((uintptr_t) src % 16) == 0;
		k_to_host<<<num_sms * 4, 256, 0, st>>>(src, d, words, wide);
		return cudaGetLastError() == cudaSuccess ? BFS_OK : BFS_ECUDA;
	}
	return cudaMemcpyAsync(dst, src, sizeof(uint32_t) * words, cudaMemcpyDeviceToHost, st) == cudaSuccess ? BFS_OK
																										: BFS_ECUDA;
}

template <class T> int dev_alloc(bfs_graph *g, T **out, size_t count) {
	size_t bytes = std::max<size_t>(sizeof(T) * count, 16);
	void *p = nullptr;
	if (cudaMalloc(&p, bytes) != cudaSuccess) {
		cudaGetLastError();
		return BFS_ENOMEM;
	}
	g->bufs.push_back({p, bytes});
	g->device_bytes += bytes;
	*out = (T *) p;
	return BFS_OK;
}

template <class T> int dev_upload(bfs_graph *g, const T **out, const std::vector<T> &v) {
	T *p = nullptr;
	int st = dev_alloc(g, &p, v.size());
	if (st) return st;
	if (!v.empty() && cudaMemcpy(p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice) != cudaSuccess)
		return BFS_ECUDA;
	*out = p;
	return BFS_OK;
}

void release_batch(bfs_graph *g) {
	for (auto &b : g->mb.bufs) cudaFree(b.p);
	g->mb.bufs.clear();
	g->mb.bytes = 0;
	g->mb.k_alloc = 0;
	g->mb.planes_alloc = 0;
}

void release_bc(bfs_graph *g) {
	auto &b = g->bc;
	for (auto &x : b.bufs) cudaFree(x.p);
	b.bufs.clear();
	if (b.h_ctl) cudaFreeHost(b.h_ctl);
	if (b.e0) cudaEventDestroy(b.e0);
	if (b.e1) cudaEventDestroy(b.e1);
	if (b.e2) cudaEventDestroy(b.e2);
	b = bfs_graph::Bc{};
}

void release_bb(bfs_graph *g) {
	auto &b = g->bb;
	for (auto &x : b.bufs) cudaFree(x.p);
	b.bufs.clear();
	for (auto &x : b.lbufs) cudaFree(x.p);
	b.lbufs.clear();
	if (b.h_ctl) cudaFreeHost(b.h_ctl);
	if (b.h_ms) cudaFreeHost(b.h_ms);
	for (cudaEvent_t e : {b.e0, b.e1, b.e2, b.e3})
		if (e) cudaEventDestroy(e);
	b = bfs_graph::BcBatch{};
}

void release(bfs_graph *g) {
	release_batch(g);
	release_bc(g);
	release_bb(g);
	if (g->mb.h_ctl) cudaFreeHost(g->mb.h_ctl);
	if (g->mb.e0) cudaEventDestroy(g->mb.e0);
	if (g->mb.e1) cudaEventDestroy(g->mb.e1);
	if (g->mb.em) cudaEventDestroy(g->mb.em);
	g->mb.h_ctl = nullptr;
	g->mb.e0 = g->mb.e1 = g->mb.em = nullptr;
	for (auto &b : g->bufs) cudaFree(b.p);
	g->bufs.clear();
	if (g->h_stats) cudaFreeHost(g->h_stats);
	if (g->h_part) cudaFreeHost(g->h_part);
	if (g->ev0) cudaEventDestroy(g->ev0);
	if (g->ev1) cudaEventDestroy(g->ev1);
	if (g->evm) cudaEventDestroy(g->evm);
	g->h_stats = nullptr;
	g->h_part = nullptr;
	g->ev0 = g->ev1 = g->evm = nullptr;
}

void default_options(bfs_options *o) {
	std::memset(o, 0, sizeof(*o));
	o->mode = BFS_MODE_PERSISTENT;
	o->to_dense_ratio = 20;   // T_RATIO, apps/bfs_simd/bfs.cpp:1171
	o->to_sparse_ratio = 20;
	o->warp_max_degree = 32;
	o->cta_max_degree = 4096;
	o->bottom_up = BFS_BU_PULL;
	o->batch_planes = 0;
	o->batch_budget_mb = 40960;
	o->batch_single_max = 4;
	o->batch_push_div = 16;
	o->switch_rule = BFS_SWITCH_REFERENCE;
	o->bu_alpha = 14;
	o->td_beta = 24;
	o->ctas_per_sm = 0;
	o->bc_batch = 1;
}

int device_setup(bfs_graph *g) {
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
		cudaGetLastError();
		return BFS_ENODEV;
	}
	if (cudaGetDevice(&g->device) != cudaSuccess) return BFS_ECUDA;
	if (cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, g->device) != cudaSuccess) return BFS_ECUDA;
	int coop = 0;
	cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, g->device);
	return coop ? BFS_OK : BFS_EUNSUPPORTED;
}

// The DevGraph fields that follow from the shape and the group plan.
void set_shape(bfs_graph *g, const PackedTiles &pk, uint64_t packed_words) {
	g->num_groups = pk.num_groups;
	g->packed_words = packed_words;
	DevGraph &d = g->dg;
	d.n = g->n;
	d.m = (uint32_t) g->m;
	d.w = g->w;
	d.s = g->s;
	d.side = g->side;
	d.num_stripes = g->num_stripes;
	d.sw = g->s * g->w;
	d.vbits = pk.vbits;
	d.cbits = pk.cbits;
	d.ushift = pk.vbits + pk.cbits;
	d.vmask = (1u << pk.vbits) - 1u;
	d.cmask = (1u << pk.cbits) - 1u;
	d.num_groups = pk.num_groups;
	d.max_group_words = (pk.max_group_vertices + 31) / 32;
	d.slice_words = (d.sw + 31) / 32;
	d.nwords = (g->n + 31) / 32;
	d.bm_words = d.num_stripes * d.slice_words;  // bulk copies read whole slices
	d.tma = (d.sw % 128 == 0) ? 1u : 0u;
	d.tma_batch = std::max<uint32_t>(1, std::min<uint32_t>(kMaxSliceBatch, kTmaSliceWords / d.slice_words));
	d.pull_long_cap = 4096;
}

// Batched pull: destinations with many in-edges and their chunks.
int upload_big_in(bfs_graph *g, const std::vector<uint32_t> &in_off) {
	std::vector<uint32_t> in_big, chunk_v, chunk_beg;
	for (uint32_t v = 0; v < g->n; ++v) {
		if (in_off[v + 1] - in_off[v] <= kMsPullBig) continue;
		in_big.push_back(v);
		for (uint32_t b = in_off[v]; b < in_off[v + 1]; b += kMsChunk) {
			chunk_v.push_back(v);
			chunk_beg.push_back(b);
		}
	}
	g->ms_nbig_in = (uint32_t) in_big.size();
	g->ms_nchunks = (uint32_t) chunk_v.size();
	int st;
	if ((st = dev_upload(g, &g->ms_in_big, in_big))) return st;
	if ((st = dev_upload(g, &g->ms_chunk_v, chunk_v))) return st;
	return dev_upload(g, &g->ms_chunk_beg, chunk_beg);
}

// Run context, events and the persistent grid.
int alloc_run(bfs_graph *g) {
	DevGraph &d = g->dg;
	RunCtx &r = g->rc;
	int st;
	if ((st = dev_alloc(g, &r.vis, d.nwords))) return st;
	for (int i = 0; i < 3; ++i) {
		if ((st = dev_alloc(g, &r.bm[i], d.bm_words))) return st;
		if ((st = dev_alloc(g, &r.sf[i], d.num_stripes))) return st;
	}
	for (int set = 0; set < 2; ++set)
		for (int b = 0; b < 3; ++b)
			if ((st = dev_alloc(g, &r.q[set][b], g->n))) return st;
	if ((st = dev_alloc(g, &r.ctr, 3))) return st;
	if ((st = dev_alloc(g, &r.part, 6 * (size_t) kMaxGrid))) return st;
	if ((st = dev_alloc(g, &r.stats, 1))) return st;
	if ((st = dev_alloc(g, &r.bar, 2))) return st;
	if ((st = dev_alloc(g, &r.err, 1))) return st;
	// the persistent kernel expects its barrier and status words zero at launch
	if (cudaMemset(r.bar, 0, 2 * sizeof(unsigned)) != cudaSuccess || cudaMemset(r.err, 0, sizeof(int)) != cudaSuccess)
		return BFS_ECUDA;
	if ((st = dev_alloc(g, &g->level_buf, g->n))) return st;
	if ((st = dev_alloc(g, &g->parent_buf, g->n))) return st;
	if (cudaMallocHost(&g->h_stats, sizeof(DevStats)) != cudaSuccess) return BFS_ENOMEM;
	if (cudaMallocHost(&g->h_part, sizeof(unsigned long long) * 2 * kMaxGrid) != cudaSuccess) return BFS_ENOMEM;
	if (cudaEventCreate(&g->ev0) != cudaSuccess || cudaEventCreate(&g->ev1) != cudaSuccess ||
			cudaEventCreate(&g->evm) != cudaSuccess)
		return BFS_ECUDA;
	g->batch = std::max<uint32_t>(1, std::min<uint32_t>(kMaxSliceBatch, kSliceBudgetWords / std::max<uint32_t>(1, d.slice_words)));
	st = persistent_grid(d, g->batch, g->num_sms, &g->grid, &g->smem);
	g->grid_max = g->grid;
	return st;
}

// Builds the device copy of a validated host graph.
int upload(bfs_graph *g, HostGraph &h) {
	g->n = h.n;
	g->m = h.m;
	g->w = h.w;
	g->s = h.s;
	g->side = h.side;
	g->num_stripes = h.num_stripes;
	g->max_degree = h.max_degree;
	g->base = h.base;
	g->used_reorder = h.used_reorder;
	g->degrees = h.degrees;
	default_options(&g->opt);
	if (g->host_only) return BFS_OK;
	int st = device_setup(g);
	if (st) return st;

	PackedTiles pk;
	st = pack_tiles(h, (uint32_t) g->num_sms * 2 * kGroupsPerCta, kMaxGroupVertices, pk);  // about one group per CTA
	if (st) return st;
	set_shape(g, pk, pk.words.size());
	DevGraph &d = g->dg;
	if ((st = dev_upload(g, &d.row_off, h.row_off))) return st;
	if ((st = dev_upload(g, &d.col, h.csr_dst))) return st;
	if ((st = dev_upload(g, &d.packed, pk.words))) return st;
	if ((st = dev_upload(g, &d.seg_off, pk.seg_off))) return st;
	if ((st = dev_upload(g, &d.group_col, pk.group_col))) return st;
	if ((st = dev_upload(g, &d.hasin, pk.hasin_bits))) return st;
	{
		// In-edge lists: the column tiles sorted by destination, sources
		// ascending within a list (a stable bucketing of the CSR order).
		std::vector<uint32_t> in_off((size_t) h.n + 1, 0), in_src(h.m);
		for (uint64_t i = 0; i < h.m; ++i) in_off[h.csr_dst[i] + 1]++;
		for (uint32_t v = 0; v < h.n; ++v) in_off[v + 1] += in_off[v];
		std::vector<uint32_t> fill(in_off.begin(), in_off.end() - 1);
		for (uint32_t u = 0; u < h.n; ++u)
			for (uint32_t e = h.row_off[u]; e < h.row_off[u + 1]; ++e) in_src[fill[h.csr_dst[e]]++] = u;
		if ((st = dev_upload(g, &d.in_off, in_off))) return st;
		if ((st = dev_upload(g, &d.in_src, in_src))) return st;
		if ((st = upload_big_in(g, in_off))) return st;
	}
	return alloc_run(g);
}

// Temporary device buffers of the device build, freed on scope exit.
struct TmpDev {
	std::vector<void *> ptrs;
	template <class T> int alloc(T **p, size_t count) {
		void *q = nullptr;
		if (cudaMalloc(&q, std::max<size_t>(count * sizeof(T), 16)) != cudaSuccess) {
			cudaGetLastError();
			return BFS_ENOMEM;
		}
		ptrs.push_back(q);
		*p = (T *) q;
		return BFS_OK;
	}
	~TmpDev() {
		for (void *p : ptrs) cudaFree(p);
	}
};

// The device layout of an edge list built on the GPU (build_device.cu): CSR
// and in-edge lists by degree histograms, scans and scatters; the packed
// column-major segments by a segment histogram, the host's group plan and
// segment offsets, and a scatter; the out-degrees and in-edge offsets come
// back for the host-side fields.
int upload_device_build(bfs_graph *g, uint32_t n, uint64_t m, const uint32_t *src, const uint32_t *dst, uint32_t w,
		uint32_t s, std::vector<uint32_t> *degree_order_out) {
	g->n = n;
	g->m = m;
	g->w = w;
	g->s = s;
	g->side = side_length_of(n, w);
	g->num_stripes = (g->side + s - 1) / s;
	default_options(&g->opt);
	int st = device_setup(g);
	if (st) return st;
	cudaStream_t cs = nullptr;
	TmpDev tmp;
	DevGraph &d = g->dg;
	uint32_t *d_src = nullptr, *d_dst = nullptr, *out_deg = nullptr, *in_deg = nullptr, *cursor = nullptr, *scan_tmp = nullptr;
	int *d_err = nullptr;
	if ((st = tmp.alloc(&d_src, m)) || (st = tmp.alloc(&d_dst, m)) || (st = tmp.alloc(&out_deg, n)) ||
			(st = tmp.alloc(&in_deg, n)) || (st = tmp.alloc(&cursor, (size_t) n + 1)) ||
			(st = tmp.alloc(&scan_tmp, dbuild_scan_tmp_words(n))) || (st = tmp.alloc(&d_err, 1)))
		return st;
	// host or device edge arrays (unified addressing tells them apart)
	if (m && (cudaMemcpy(d_src, src, m * 4, cudaMemcpyDefault) != cudaSuccess ||
			cudaMemcpy(d_dst, dst, m * 4, cudaMemcpyDefault) != cudaSuccess))
		return BFS_ECUDA;
	if (cudaMemset(out_deg, 0, (size_t) n * 4) != cudaSuccess || cudaMemset(in_deg, 0, (size_t) n * 4) != cudaSuccess ||
			cudaMemset(d_err, 0, 4) != cudaSuccess)
		return BFS_ECUDA;
	if ((st = dbuild_degrees(d_src, d_dst, m, n, out_deg, in_deg, d_err, g->num_sms, cs))) return st;
	int herr = 0;
	if (cudaMemcpy(&herr, d_err, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return BFS_ECUDA;
	if (herr) return herr;
	if (degree_order_out) {
		// relabel the edges by the degree order, then count again
		std::vector<uint32_t> deg(n);
		if (cudaMemcpy(deg.data(), out_deg, (size_t) n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return BFS_ECUDA;
		*degree_order_out = degree_order(deg);
		uint32_t *d_map = nullptr;
		if ((st = tmp.alloc(&d_map, n))) return st;
		if (cudaMemcpy(d_map, degree_order_out->data(), (size_t) n * 4, cudaMemcpyHostToDevice) != cudaSuccess)
			return BFS_ECUDA;
		k_relabel_edges<<<g->num_sms * 8, 512, 0, cs>>>(m, d_map, d_src, d_dst);
		if (cudaMemset(out_deg, 0, (size_t) n * 4) != cudaSuccess || cudaMemset(in_deg, 0, (size_t) n * 4) != cudaSuccess)
			return BFS_ECUDA;
		if ((st = dbuild_degrees(d_src, d_dst, m, n, out_deg, in_deg, d_err, g->num_sms, cs))) return st;
	}
	// CSR and in-edge lists
	uint32_t *row_off = nullptr, *col = nullptr, *in_off = nullptr, *in_src = nullptr;
	if ((st = dev_alloc(g, &row_off, (size_t) n + 1)) || (st = dev_alloc(g, &col, m)) ||
			(st = dev_alloc(g, &in_off, (size_t) n + 1)) || (st = dev_alloc(g, &in_src, m)))
		return st;
	if ((st = dbuild_exclusive_scan(out_deg, n, scan_tmp, row_off, cs))) return st;
	if (cudaMemcpy(cursor, row_off, (size_t) n * 4, cudaMemcpyDeviceToDevice) != cudaSuccess) return BFS_ECUDA;
	if ((st = dbuild_scatter(d_src, d_dst, m, cursor, col, g->num_sms, cs))) return st;
	if ((st = dbuild_exclusive_scan(in_deg, n, scan_tmp, in_off, cs))) return st;
	if (cudaMemcpy(cursor, in_off, (size_t) n * 4, cudaMemcpyDeviceToDevice) != cudaSuccess) return BFS_ECUDA;
	if ((st = dbuild_scatter(d_dst, d_src, m, cursor, in_src, g->num_sms, cs))) return st;
	d.row_off = row_off;
	d.col = col;
	d.in_off = in_off;
	d.in_src = in_src;
	// host-side fields
	g->degrees.resize(n);
	std::vector<uint32_t> h_in_off((size_t) n + 1);
	if (cudaMemcpy(g->degrees.data(), out_deg, (size_t) n * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
			cudaMemcpy(h_in_off.data(), in_off, ((size_t) n + 1) * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
		return BFS_ECUDA;
	g->max_degree = 0;
	for (uint32_t v = 0; v < n; ++v) g->max_degree = std::max(g->max_degree, g->degrees[v]);
	if ((st = upload_big_in(g, h_in_off))) return st;
	// packed column-major segments
	uint32_t *col_edges = nullptr, *hasin = nullptr;
	if ((st = tmp.alloc(&col_edges, g->side)) || (st = dev_alloc(g, &hasin, ((size_t) n + 31) / 32))) return st;
	if (cudaMemset(col_edges, 0, (size_t) g->side * 4) != cudaSuccess ||
			cudaMemset(hasin, 0, ((size_t) n + 31) / 32 * 4) != cudaSuccess)
		return BFS_ECUDA;
	if ((st = dbuild_col_hist(d_dst, m, w, g->side, col_edges, hasin, g->num_sms, cs))) return st;
	std::vector<uint32_t> h_col32(g->side);
	if (cudaMemcpy(h_col32.data(), col_edges, (size_t) g->side * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
		return BFS_ECUDA;
	std::vector<uint64_t> h_col(h_col32.begin(), h_col32.end());
	PackedTiles pk;
	if ((st = plan_groups(n, w, s, g->side, h_col, m, (uint32_t) g->num_sms * 2 * kGroupsPerCta, kMaxGroupVertices, pk)))
		return st;
	std::vector<uint32_t> group_of(g->side);
	for (uint32_t gi = 0; gi < pk.num_groups; ++gi)
		for (uint32_t c = pk.group_col[gi]; c < pk.group_col[gi + 1]; ++c) group_of[c] = gi;
	const uint64_t nseg = (uint64_t) g->num_stripes * pk.num_groups;
	uint32_t *d_group_of = nullptr, *seg_count = nullptr, *seg_cursor = nullptr, *pad = nullptr;
	if ((st = tmp.alloc(&d_group_of, g->side)) || (st = tmp.alloc(&seg_count, nseg)) || (st = tmp.alloc(&seg_cursor, nseg)) ||
			(st = tmp.alloc(&pad, pk.num_groups)))
		return st;
	const uint32_t *group_col = nullptr;
	if ((st = dev_upload(g, &group_col, pk.group_col))) return st;
	if (cudaMemcpy(d_group_of, group_of.data(), (size_t) g->side * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
			cudaMemset(seg_count, 0, nseg * 4) != cudaSuccess)
		return BFS_ECUDA;
	DeviceBuildShape sh{w, s, g->num_stripes, pk.vbits, pk.cbits};
	if ((st = dbuild_seg_hist(d_src, d_dst, m, sh, d_group_of, seg_count, g->num_sms, cs))) return st;
	std::vector<uint32_t> h_seg32(nseg);
	if (cudaMemcpy(h_seg32.data(), seg_count, nseg * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return BFS_ECUDA;
	std::vector<uint64_t> h_seg(h_seg32.begin(), h_seg32.end());
	if ((st = segment_offsets(h_seg, pk))) return st;
	const uint64_t words = pk.seg_off[nseg];
	std::vector<uint32_t> pad_word(pk.num_groups);
	for (uint32_t gi = 0; gi < pk.num_groups; ++gi) pad_word[gi] = group_pad_word(pk, gi, n, w);
	const uint32_t *seg_off = nullptr;
	uint32_t *packed = nullptr;
	if ((st = dev_upload(g, &seg_off, pk.seg_off)) || (st = dev_alloc(g, &packed, words))) return st;
	if (cudaMemcpy(seg_cursor, seg_off, nseg * 4, cudaMemcpyDeviceToDevice) != cudaSuccess ||
			cudaMemcpy(pad, pad_word.data(), pk.num_groups * 4, cudaMemcpyHostToDevice) != cudaSuccess)
		return BFS_ECUDA;
	if ((st = dbuild_seg_fill(d_src, d_dst, m, sh, d_group_of, group_col, seg_cursor, packed, g->num_sms, cs))) return st;
	if ((st = dbuild_seg_pad(seg_off, seg_count, nseg, g->num_stripes, pad, packed, g->num_sms, cs))) return st;
	if (cudaDeviceSynchronize() != cudaSuccess) return BFS_ECUDA;
	d.packed = packed;
	d.seg_off = seg_off;
	d.group_col = group_col;
	d.hasin = hasin;
	set_shape(g, pk, words);
	return alloc_run(g);
}

// Makes a graph built on relabelled edges answer in the caller's ids: the
// maps on the device, run buffers in the layout's ids, out-degrees in the
// caller's order.
int attach_relabel(bfs_graph *g, std::vector<uint32_t> &&new_of_old) {
	const uint32_t n = g->n;
	std::vector<uint32_t> old_of_new(n);
	for (uint32_t v = 0; v < n; ++v) old_of_new[new_of_old[v]] = v;
	std::vector<uint32_t> deg(n);
	for (uint32_t v = 0; v < n; ++v) deg[v] = g->degrees[new_of_old[v]];
	g->degrees.swap(deg);
	int st;
	if (g->host_only) {
		g->new_of_old = std::move(new_of_old);
		g->relabeled = true;
		return BFS_OK;
	}
	if ((st = dev_alloc(g, &g->d_new_of_old, n)) || (st = dev_alloc(g, &g->d_old_of_new, n)) ||
			(st = dev_alloc(g, &g->rl_level, n)) || (st = dev_alloc(g, &g->rl_parent, n)))
		return st;
	if (cudaMemcpy(g->d_new_of_old, new_of_old.data(), (size_t) n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
			cudaMemcpy(g->d_old_of_new, old_of_new.data(), (size_t) n * 4, cudaMemcpyHostToDevice) != cudaSuccess)
		return BFS_ECUDA;
	g->new_of_old = std::move(new_of_old);
	g->relabeled = true;
	return BFS_OK;
}

int finish_graph(HostGraph &h, uint32_t flags, bfs_graph **out) {
	bfs_graph *g = new bfs_graph();
	g->host_only = flags & BFS_LOAD_HOST_ONLY;
	int st = upload(g, h);
	if (st) {
		release(g);
		delete g;
		return st;
	}
	*out = g;
	return BFS_OK;
}

int check_shape(uint32_t n, uint64_t m, uint32_t w, uint32_t s) {
	if (n == 0 || w == 0 || s == 0) return BFS_EARG;
	if (m > 0xFFFFFFFFull) return BFS_EUNSUPPORTED;
	return BFS_OK;
}

void init_shape(HostGraph &h, uint32_t n, uint64_t m, uint32_t w, uint32_t s) {
	h.n = n;
	h.m = m;
	h.w = w;
	h.s = s;
	h.side = side_length_of(n, w);
	h.num_stripes = (h.side + s - 1) / s;
}

int resolve_base(const std::string &data, uint32_t w, uint32_t s, uint32_t flags, std::string *base, bool *reorder) {
	std::string cands[2] = {data, data + "_reorder"};
	if (flags & BFS_LOAD_PREFER_REORDER) std::swap(cands[0], cands[1]);
	for (int i = 0; i < 2; ++i) {
		std::string col = cands[i] + "_col-" + std::to_string(s) + "-coo-tiled-" + std::to_string(w) + "-0";
		std::string csr = cands[i] + "_untiled-0";
		if (file_exists(col) && file_exists(csr)) {
			*base = cands[i];
			*reorder = (cands[i] != data);
			return BFS_OK;
		}
	}
	return BFS_EIO;
}

// Host side of a traversal in stepwise mode.
int run_stepwise(bfs_graph *g, const RunCtx &r, const StepParams &p, cudaStream_t st) {
	const DevGraph &d = g->dg;
	int rc;
	if ((rc = launch_step(kStepSeed, d, r, p, 0, g->batch, g->grid, g->smem, st))) return rc;
	bfs_stats &hs = g->host_stats;
	std::memset(&hs, 0, sizeof(hs));
	bool last_dense = false;
	unsigned long long seen = 0;  // out-edges of the vertices reached so far
	uint32_t step = 0;
	for (;; ++step) {
		// the step totals: sum of the per-CTA partials of the frontier's slot
		const uint32_t slot = (step + 2) % 3;
		if (cudaMemcpyAsync(g->h_part, r.part + (size_t) slot * 2 * kMaxGrid, sizeof(unsigned long long) * 2 * kMaxGrid,
				    cudaMemcpyDeviceToHost, st) != cudaSuccess ||
				cudaStreamSynchronize(st) != cudaSuccess)
			return BFS_ECUDA;
		unsigned long long count = 0, degsum = 0;
		for (int i = 0; i < g->grid; ++i) {
			count += g->h_part[i];
			degsum += g->h_part[kMaxGrid + i];
		}
		hs.reached += (uint32_t) count;
		hs.edges_traversed += degsum;
		if (count == 0) break;
		seen += degsum;
		bool dense = false;
		if (step > 0 && p.switch_rule != 0) {
			const unsigned long long unseen = g->m > seen ? g->m - seen : 0ull;
			dense = last_dense ? count * p.beta >= g->n : degsum * p.alpha > unseen;
		} else if (step > 0) {
			unsigned long long thr = last_dense ? p.to_sparse_threshold : p.to_dense_threshold;
			dense = count + degsum > thr;
		}
		if ((rc = launch_step(kStepClear, d, r, p, step, g->batch, g->grid, g->smem, st))) return rc;
		if (dense) {
			if (!last_dense && (rc = launch_step(kStepToDense, d, r, p, step, g->batch, g->grid, g->smem, st))) return rc;
			if ((rc = launch_step(kStepDense, d, r, p, step, g->batch, g->grid, g->smem, st))) return rc;
		} else {
			if (last_dense && (rc = launch_step(kStepToSparse, d, r, p, step, g->batch, g->grid, g->smem, st))) return rc;
			if ((rc = launch_step(kStepExpand, d, r, p, step, g->batch, g->grid, g->smem, st))) return rc;
		}
		if (step < BFS_TRACE_MAX) hs.trace[step] = dense ? 1 : 0;
		hs.dense_steps += dense;
		last_dense = dense;
	}
	hs.num_steps = step;
	return BFS_OK;
}

int run_impl(bfs_graph *g, uint32_t source, int32_t *levels, uint32_t *parents, cudaStream_t st) {
	if (g->host_only) return BFS_EUNSUPPORTED;
	if (source >= g->n || !levels) return BFS_EARG;
	if (cudaSetDevice(g->device) != cudaSuccess) return BFS_ECUDA;
	RunCtx r = g->rc;
	r.level = g->relabeled ? g->rl_level : levels;
	r.parent = g->relabeled ? (parents ? g->rl_parent : nullptr) : parents;
	StepParams p{};
	p.source = g->relabeled ? g->new_of_old[source] : source;
	p.warp_max_degree = g->opt.warp_max_degree;
	p.cta_max_degree = g->opt.cta_max_degree;
	p.bottom_up = g->opt.bottom_up;
	p.to_dense_threshold = g->m / std::max<uint32_t>(1, g->opt.to_dense_ratio);
	p.to_sparse_threshold = g->m / std::max<uint32_t>(1, g->opt.to_sparse_ratio);
	p.wait_limit_ns = wait_limit_ns(g->opt);
	p.hold_barrier = g->opt.test_hold_barrier;
	p.switch_rule = g->opt.switch_rule;
	p.alpha = g->opt.bu_alpha;
	p.beta = g->opt.td_beta;
	int rc;
	g->stepwise_last = g->opt.mode == BFS_MODE_STEPWISE;
	if (cudaEventRecord(g->ev0, st) != cudaSuccess) return BFS_ECUDA;
	// the persistent kernel clears the run state and seeds the source itself;
	// the stepwise host loop clears and seeds with launches of their own
	if (g->stepwise_last && (rc = launch_init(g->dg, r, st, g->num_sms))) return rc;
	if (cudaEventRecord(g->evm, st) != cudaSuccess) return BFS_ECUDA;
	if (g->stepwise_last) {
		if ((rc = run_stepwise(g, r, p, st))) return rc;
	} else {
		if ((rc = launch_persistent(g->dg, r, p, g->batch, g->grid, g->smem, st))) return rc;
	}
	if (g->relabeled) {
		k_unrelabel<<<g->num_sms * 4, 512, 0, st>>>(g->n, g->d_new_of_old, g->d_old_of_new, r.level, r.parent, levels,
				parents);
		if (cudaGetLastError() != cudaSuccess) return BFS_ECUDA;
	}
	if (cudaEventRecord(g->ev1, st) != cudaSuccess) return BFS_ECUDA;
	g->last_stream = st;
	g->stats_fresh = false;
	g->have_run = true;
	return BFS_OK;
}

int collect_stats(bfs_graph *g, bfs_stats *out) {
	if (!g->have_run) return BFS_EARG;
	// The device statistics are copied only when asked for, so that a run
	// enqueues nothing but its kernels.
	if (!g->stats_fresh) {
		if (cudaMemcpyAsync(g->h_stats, g->rc.stats, sizeof(DevStats), cudaMemcpyDeviceToHost, g->last_stream) != cudaSuccess ||
				cudaStreamSynchronize(g->last_stream) != cudaSuccess)
			return BFS_ECUDA;
		g->stats_fresh = true;
	}
	const DevStats &d = *g->h_stats;
	bfs_stats s{};
	if (g->stepwise_last) {
		s = g->host_stats;
	} else {
		s.num_steps = d.num_steps;
		s.dense_steps = d.dense_steps;
		s.reached = (uint32_t) d.reached;
		s.edges_traversed = d.edges_traversed;
		std::memcpy(s.trace, d.trace, sizeof(s.trace));
		// Phase timers from the device timestamps.
		for (uint32_t i = 0; i < s.num_steps && i < BFS_TRACE_MAX && i + 1 < 257; ++i) {
			const unsigned long long t0 = d.t_step[i], t1 = d.t_step[i + 1];
			if (!t0 || t1 < t0) continue;
			double total = (t1 - t0) * 1e-6, conv = 0;
			if (d.t_conv[i] >= t0 && d.t_conv[i] <= t1 && d.t_conv[i]) conv = (d.t_conv[i] - t0) * 1e-6;
			s.step_ms[i] = (float) total;
			const unsigned long long wmax = d.t_work_max[i], wmin = ~d.t_work_min_inv[i];
			if (d.t_work_max[i] >= t0) s.step_work_max_ms[i] = (float) ((wmax - t0) * 1e-6);
			if (d.t_work_min_inv[i] && wmin >= t0) s.step_work_min_ms[i] = (float) ((wmin - t0) * 1e-6);
			if (s.trace[i]) { s.dense_ms += total - conv; s.to_dense_ms += conv; }
			else { s.sparse_ms += total - conv; s.to_sparse_ms += conv; }
		}
	}
	for (int i = 0; i < 8; ++i) s.bu_cycles[i] = d.bu_cycles[i];
	s.td_edges = d.td_edges;
	s.td_vertices = d.td_vertices;
	s.bu_words = d.bu_words;
	s.bu_slices = d.bu_slices;
	s.bu_groups = d.bu_groups;
	s.bu_vertices = d.bu_vertices;
	s.status = g->stepwise_last ? BFS_OK : d.status;
	s.max_level = s.num_steps ? s.num_steps - 1 : 0;
	s.grid_ctas = (uint32_t) g->grid;
	float ms = 0, kms = 0;
	cudaEventElapsedTime(&ms, g->ev0, g->ev1);
	cudaEventElapsedTime(&kms, g->evm, g->ev1);
	s.device_ms = ms;
	s.kernel_ms = kms;
	if (out) *out = s;
	return s.status;
}

template <class T> int batch_alloc(bfs_graph *g, T **out, size_t count) {
	size_t bytes = std::max<size_t>(sizeof(T) * count, 16);
	void *p = nullptr;
	if (cudaMalloc(&p, bytes) != cudaSuccess) {
		cudaGetLastError();
		return BFS_ENOMEM;
	}
	g->mb.bufs.push_back({p, bytes});
	g->mb.bytes += bytes;
	*out = (T *) p;
	return BFS_OK;
}

// Level planes a batch of K words per vertex asks for.
uint32_t batch_planes_wanted(const bfs_graph *g, uint32_t K) {
	if (g->opt.batch_planes) return g->opt.batch_planes;
	const size_t plane = (size_t) g->n * K * 8;
	const size_t budget = (size_t) g->opt.batch_budget_mb << 20;
	return (uint32_t) std::max<size_t>(2, std::min<size_t>(kBatchDefaultPlanes, budget / std::max<size_t>(plane, 1)));
}

// Makes the batch buffers hold K words per vertex and enough level planes;
// returns the planes the call will use.  Buffers that hold at least K words
// are reused; with the planes sized from the budget any plane count will do
// (a deeper traversal writes its output early), an explicit batch_planes must
// fit.
int batch_prepare(bfs_graph *g, uint32_t K, uint32_t *planes_out) {
	auto &b = g->mb;
	const size_t plane = (size_t) g->n * K * 8 + (size_t) g->n * 8;  // rows + word masks
	uint32_t planes = batch_planes_wanted(g, K);
	if (!b.h_ctl) {
		if (cudaMallocHost(&b.h_ctl, sizeof(MsControl)) != cudaSuccess) return BFS_ENOMEM;
		if (cudaEventCreate(&b.e0) != cudaSuccess || cudaEventCreate(&b.e1) != cudaSuccess ||
				cudaEventCreate(&b.em) != cudaSuccess)
			return BFS_ECUDA;
	}
	const uint32_t have = b.k_alloc >= K ? b.planes_alloc : 0;
	if (have >= 2 && (have >= planes || !g->opt.batch_planes)) {
		*planes_out = g->opt.batch_planes ? planes : have;
		return BFS_OK;
	}
	// (re)allocate: wait for earlier batches that still use the buffers
	if (b.have_run && cudaEventSynchronize(b.e1) != cudaSuccess) return BFS_ECUDA;
	release_batch(g);
	const size_t fixed = (size_t) g->n * K * 8 + (size_t) g->n * (2 + 4 + 8) + sizeof(MsControl) +
			4 * BFS_BATCH_MAX_SOURCES;
	size_t free_b = 0, total_b = 0;
	if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return BFS_ECUDA;
	const size_t usable = free_b > (size_t) 1 << 30 ? free_b - ((size_t) 1 << 30) : 0;  // leave 1 GiB
	if (usable < fixed + 2 * plane) return BFS_ENOMEM;
	if (fixed + planes * plane > usable) {
		if (g->opt.batch_planes) return BFS_ENOMEM;  // an explicit plane count that does not fit
		planes = (uint32_t) ((usable - fixed) / plane);
	}
	MsArgs &a = b.args;
	int st;
	if ((st = batch_alloc(g, &a.vis, (size_t) g->n * K))) return st;
	if ((st = batch_alloc(g, &a.hist, (size_t) planes * g->n * K))) return st;
	if ((st = batch_alloc(g, &a.pmask, (size_t) planes * g->n))) return st;
	if ((st = batch_alloc(g, &a.touched, g->n))) return st;
	if ((st = batch_alloc(g, &a.done, g->n))) return st;
	if ((st = batch_alloc(g, &a.seed_flag, g->n))) return st;
	if ((st = batch_alloc(g, &a.queue[0], g->n))) return st;
	if ((st = batch_alloc(g, &a.queue[1], g->n))) return st;
	if ((st = batch_alloc(g, &a.ctl, 1))) return st;
	if ((st = batch_alloc(g, &b.d_sources, BFS_BATCH_MAX_SOURCES))) return st;
	// push chunk list: a vertex above the grid-spread degree has > 1024 edges, so
	// its chunks number at most E / 1024 + the vertices, at most 2 E / 1024
	a.push_cap = (uint32_t) std::min<uint64_t>(0xFFFFFFFFull, 2 * g->m / kMsPushChunk + 1);
	if ((st = batch_alloc(g, &a.push_u, a.push_cap))) return st;
	if ((st = batch_alloc(g, &a.push_beg, a.push_cap))) return st;
	b.k_alloc = K;
	b.planes_alloc = planes;
	*planes_out = planes;
	return BFS_OK;
}

// One single-source traversal's int32 levels -> a uint8 row (255 = unreached);
// adds the traversal's edge count, depth and status to the batch statistics.
__global__ void __launch_bounds__(512) k_levels_u8(const int32_t *lev, uint8_t *out, uint32_t n, const DevStats *ds,
		MsControl *ctl) {
	const uint32_t stride = gridDim.x * blockDim.x;
	uint32_t mx = 0;
	bool over = false;
	for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
		const int32_t l = lev[i];
		uint8_t x = 255;
		if (l >= 0) {
			over |= l > (int32_t) kMsMaxLevel;
			x = (uint8_t) min(l, (int32_t) kMsMaxLevel);
			mx = max(mx, (uint32_t) l + 1);
		}
		out[i] = x;
	}
	for (int d = 16; d > 0; d >>= 1) mx = max(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, d));
	if ((threadIdx.x & 31) == 0 && mx) atomicMax(&ctl->stats.depth, mx);
	if (over) atomicExch(&ctl->err, BFS_EUNSUPPORTED);
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		atomicAdd(&ctl->stats.traversed, ds->edges_traversed);
		if (ds->status) atomicExch(&ctl->err, ds->status);
		ctl->stats.complete = 1;
	}
}

// The batched traversal's arguments: K words per vertex, ns sources, `planes`
// level planes (the buffers batch_prepare made).
MsArgs batch_args(const bfs_graph *g, uint32_t K, uint32_t ns, uint32_t planes) {
	MsArgs a = g->mb.args;
	a.n = g->n;
	a.m = (uint32_t) g->m;
	a.K = K;
	a.last_bits = ns - 64 * (K - 1);
	a.planes = planes;
	a.push_div = std::max<uint32_t>(1, g->opt.batch_push_div);
	a.wait_limit_ns = wait_limit_ns(g->opt);
	a.hold_barrier = g->opt.test_hold_barrier;
	a.ctas_per_sm = g->opt.ctas_per_sm;
	a.out_tile = g->opt.batch_output_tile;
	a.row_off = g->dg.row_off;
	a.col = g->dg.col;
	a.in_off = g->dg.in_off;
	a.in_src = g->dg.in_src;
	a.in_big = g->ms_in_big;
	a.chunk_v = g->ms_chunk_v;
	a.chunk_beg = g->ms_chunk_beg;
	a.nbig_in = g->ms_nbig_in;
	a.nchunks = g->ms_nchunks;
	return a;
}

bool stream_capturing(cudaStream_t st) {
	cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
	return cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
}

// `dev_sources`: `sources` is device memory (validated by the kernel).
int run_batch_impl(bfs_graph *g, const uint32_t *sources, uint32_t ns, uint8_t *levels, cudaStream_t st,
		cudaEvent_t wait_before = nullptr, cudaEvent_t between = nullptr, bool dev_sources = false) {
	if (g->host_only || g->relabeled) return BFS_EUNSUPPORTED;
	if (!sources || !levels || ns == 0 || ns > BFS_BATCH_MAX_SOURCES) return BFS_EARG;
	if (!dev_sources)
		for (uint32_t i = 0; i < ns; ++i)
			if (sources[i] >= g->n) return BFS_EARG;
	if (cudaSetDevice(g->device) != cudaSuccess) return BFS_ECUDA;
	const uint32_t K = (ns + 63) / 64;
	uint32_t planes = 0;
	int rc = batch_prepare(g, K, &planes);
	if (rc) return rc;
	auto &b = g->mb;
	MsArgs a = batch_args(g, K, ns, planes);
	const bool capturing = dev_sources && stream_capturing(st);
	if (!capturing && cudaEventRecord(b.e0, st) != cudaSuccess) return BFS_ECUDA;
	const bool singles = !dev_sources && ns <= g->opt.batch_single_max && g->opt.mode == BFS_MODE_PERSISTENT;
	if (singles) {
		// a few sources: one single-source traversal each (queue-driven, no
		// sweeps over all vertices), rows converted to uint8 on the device
		if (wait_before && cudaStreamWaitEvent(st, wait_before, 0) != cudaSuccess) return BFS_ECUDA;
		if (cudaMemsetAsync(a.ctl, 0, sizeof(MsControl), st) != cudaSuccess) return BFS_ECUDA;
		RunCtx r = g->rc;
		r.level = g->level_buf;
		r.parent = g->parent_buf;
		StepParams p{};
		p.warp_max_degree = g->opt.warp_max_degree;
		p.cta_max_degree = g->opt.cta_max_degree;
		p.bottom_up = g->opt.bottom_up;
		p.to_dense_threshold = g->m / std::max<uint32_t>(1, g->opt.to_dense_ratio);
		p.to_sparse_threshold = g->m / std::max<uint32_t>(1, g->opt.to_sparse_ratio);
		p.wait_limit_ns = wait_limit_ns(g->opt);
		p.hold_barrier = g->opt.test_hold_barrier;
		p.switch_rule = g->opt.switch_rule;
		p.alpha = g->opt.bu_alpha;
		p.beta = g->opt.td_beta;
		for (uint32_t i = 0; i < ns; ++i) {
			p.source = sources[i];
			if ((rc = launch_persistent(g->dg, r, p, g->batch, g->grid, g->smem, st))) return rc;
			k_levels_u8<<<g->num_sms * 4, 512, 0, st>>>(g->level_buf, levels + (size_t) i * g->n, g->n, r.stats, a.ctl);
		}
		if (cudaGetLastError() != cudaSuccess) return BFS_ECUDA;
		if (cudaEventRecord(b.em, st) != cudaSuccess) return BFS_ECUDA;
		if (between && cudaEventRecord(between, st) != cudaSuccess) return BFS_ECUDA;
		b.grid = g->grid;
		// the single-source statistics now describe the last of these runs
		g->have_run = false;
	} else if (dev_sources) {
		// sources already on the device (checked there); device work only, so
		// the call can be captured into a CUDA graph
		if (wait_before && cudaStreamWaitEvent(st, wait_before, 0) != cudaSuccess) return BFS_ECUDA;
		if ((rc = ms_launch(a, sources, ns, levels, g->num_sms, st, &b.grid, capturing ? nullptr : b.em, between)))
			return rc;
	} else {
		// pageable source: the copy has left `sources` when the call returns
		if (cudaMemcpyAsync(b.d_sources, sources, sizeof(uint32_t) * ns, cudaMemcpyHostToDevice, st) != cudaSuccess)
			return BFS_ECUDA;
		if (wait_before && cudaStreamWaitEvent(st, wait_before, 0) != cudaSuccess) return BFS_ECUDA;
		if ((rc = ms_launch(a, b.d_sources, ns, levels, g->num_sms, st, &b.grid, b.em, between))) return rc;
	}
	b.em_valid = !capturing;
	b.singles = singles;
	b.args.planes = planes;
	b.args.K = K;
	if (capturing) return BFS_OK;  // timing events belong to the launch of the graph
	if (cudaEventRecord(b.e1, st) != cudaSuccess) return BFS_ECUDA;
	b.num_sources = ns;
	b.stream = st;
	b.have_run = true;
	b.fresh = false;
	return BFS_OK;
}

int collect_batch_stats(bfs_graph *g, bfs_batch_stats *out) {
	auto &b = g->mb;
	if (!b.have_run) return BFS_EARG;
	if (!b.fresh) {
		if (cudaMemcpyAsync(b.h_ctl, b.args.ctl, sizeof(MsControl), cudaMemcpyDeviceToHost, b.stream) != cudaSuccess ||
				cudaStreamSynchronize(b.stream) != cudaSuccess)
			return BFS_ECUDA;
		b.fresh = true;
	}
	const MsControl &c = *b.h_ctl;
	bfs_batch_stats s{};
	s.num_sources = b.num_sources;
	s.depth = c.stats.depth;
	s.push_levels = c.stats.push_levels;
	s.status = c.err;
	s.edges_traversed = c.stats.traversed;
	s.words_gathered = c.stats.edges;
	s.planes = b.args.planes;
	s.spills = c.stats.spills;
	s.words_per_vertex = b.args.K;
	s.grid_ctas = (uint32_t) b.grid;
	float ms = 0, ems = 0;
	cudaEventElapsedTime(&ms, b.e0, b.e1);
	if (b.em_valid) cudaEventElapsedTime(&ems, b.em, b.e1);
	s.device_ms = ms;
	s.output_ms = ems;
	s.setup_ms = c.stats.t_levels0 > c.stats.t_start ? (c.stats.t_levels0 - c.stats.t_start) * 1e-6 : 0.0;
	s.levels_ms = c.stats.t_levels1 > c.stats.t_levels0 ? (c.stats.t_levels1 - c.stats.t_levels0) * 1e-6 : 0.0;
	s.device_bytes = b.bytes;
	s.single_source_runs = b.singles ? b.num_sources : 0;
	const uint32_t nl = std::min<uint32_t>(c.stats.depth, kMsTraceLevels);
	for (uint32_t l = 0; l < nl; ++l) {
		const unsigned long long t0 = c.stats.t_level[l], t1 = c.stats.t_level[l + 1];
		s.level_ms[l] = (t0 && t1 > t0) ? (float) ((t1 - t0) * 1e-6) : 0.f;
		const unsigned long long p0 = c.stats.t_phase[l][0], p1 = c.stats.t_phase[l][1];
		if (t0 && p0 >= t0 && p1 >= p0 && t1 >= p1) {
			s.level_phase_ms[l][0] = (float) ((p0 - t0) * 1e-6);
			s.level_phase_ms[l][1] = (float) ((p1 - p0) * 1e-6);
			s.level_phase_ms[l][2] = (float) ((t1 - p1) * 1e-6);
		} else if (t0 && t1 > t0) {
			s.level_phase_ms[l][0] = s.level_ms[l];
		}
		s.level_frontier[l] = c.stats.frontier[l];
		s.level_push[l] = c.stats.push[l];
	}
	if (out) *out = s;
	return s.status;
}

// ---- betweenness dependencies ----------------------------------------------
template <class T> int bc_alloc(bfs_graph *g, T **out, size_t count) {
	size_t bytes = std::max<size_t>(sizeof(T) * count, 16);
	void *p = nullptr;
	if (cudaMalloc(&p, bytes) != cudaSuccess) {
		cudaGetLastError();
		return BFS_ENOMEM;
	}
	g->bc.bufs.push_back({p, bytes});
	g->bc.bytes += bytes;
	*out = (T *) p;
	return BFS_OK;
}

int bc_prepare(bfs_graph *g) {
	auto &b = g->bc;
	if (b.ctl) return BFS_OK;
	int rc;
	if ((rc = bc_alloc(g, &b.sigma, g->n)) || (rc = bc_alloc(g, &b.order, g->n)) ||
			(rc = bc_alloc(g, &b.lvx, g->n)) || (rc = bc_alloc(g, &b.lv8, g->n)) || (rc = bc_alloc(g, &b.delta, g->n)) ||
			(rc = bc_alloc(g, &b.acc, g->n)) || (rc = bc_alloc(g, &b.cnt, kBcCntCap)) ||
			(rc = bc_alloc(g, &b.kstart, kBcClasses * (size_t) kBcMaxLevels + 1)) ||
			(rc = bc_alloc(g, &b.partial, bc_partial_capacity(g->n, g->m))) ||
			(rc = bc_alloc(g, &b.cpre, (size_t) g->n + 1)) || (rc = bc_alloc(g, &b.ctl, 1))) {
		release_bc(g);
		return rc;
	}
	if (cudaMallocHost(&b.h_ctl, sizeof(BcControl)) != cudaSuccess || cudaEventCreate(&b.e0) != cudaSuccess ||
			cudaEventCreate(&b.e1) != cudaSuccess || cudaEventCreate(&b.e2) != cudaSuccess) {
		cudaGetLastError();
		release_bc(g);
		return BFS_ENOMEM;
	}
	return BFS_OK;
}

// Enqueues a traversal from `source` (always the persistent kernel: its
// device-side step count and status feed the dependency launch) and the
// dependency launch.  sigma / delta: where the path counts and dependencies go
// (the graph's own buffers when null); acc: accumulated into when non-null.
int bc_enqueue(bfs_graph *g, uint32_t source, uint32_t *sigma, float *delta, float *acc, cudaStream_t st) {
	if (g->relabeled) return BFS_EUNSUPPORTED;
	auto &b = g->bc;
	RunCtx r = g->rc;
	r.level = g->level_buf;
	r.parent = nullptr;
	StepParams p{};
	p.source = source;
	p.warp_max_degree = g->opt.warp_max_degree;
	p.cta_max_degree = g->opt.cta_max_degree;
	p.bottom_up = g->opt.bottom_up;
	p.to_dense_threshold = g->m / std::max<uint32_t>(1, g->opt.to_dense_ratio);
	p.to_sparse_threshold = g->m / std::max<uint32_t>(1, g->opt.to_sparse_ratio);
	p.wait_limit_ns = wait_limit_ns(g->opt);
	p.hold_barrier = g->opt.test_hold_barrier;
	p.switch_rule = g->opt.switch_rule;
	p.alpha = g->opt.bu_alpha;
	p.beta = g->opt.td_beta;
	int rc;
	if (cudaEventRecord(b.e0, st) != cudaSuccess) return BFS_ECUDA;
	if ((rc = launch_persistent(g->dg, r, p, g->batch, g->grid, g->smem, st))) return rc;
	if (cudaEventRecord(b.e1, st) != cudaSuccess) return BFS_ECUDA;
	BcArgs a{};
	a.n = g->n;
	a.source = source;
	a.row_off = g->dg.row_off;
	a.col = g->dg.col;
	a.in_off = g->dg.in_off;
	a.in_src = g->dg.in_src;
	a.level = g->level_buf;
	a.num_steps = &r.stats->num_steps;
	a.bfs_status = &r.stats->status;
	a.sigma = sigma ? sigma : b.sigma;
	a.lvx = b.lvx;
	a.lv8 = b.lv8;
	a.byte_levels = g->opt.bc_level_bytes == 1 || (g->opt.bc_level_bytes == 0 && g->n >= kBcByteLevelsMinVertices);
	a.delta = delta ? delta : b.delta;
	a.acc = acc;
	a.order = b.order;
	a.cnt = b.cnt;
	a.kstart = b.kstart;
	a.partial = b.partial;
	a.cpre = b.cpre;
	a.ctl = b.ctl;
	if ((rc = bc_launch(a, g->num_sms, st, &b.grid))) return rc;
	if (cudaEventRecord(b.e2, st) != cudaSuccess) return BFS_ECUDA;
	b.stream = st;
	g->bc_last_batched = false;
	// the traversal's own statistics and events were not recorded
	g->have_run = false;
	return BFS_OK;
}

int bc_collect(bfs_graph *g, bfs_bc_stats *out) {
	auto &b = g->bc;
	cudaStream_t st = b.stream;
	if (cudaMemcpyAsync(b.h_ctl, b.ctl, sizeof(BcControl), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
			cudaStreamSynchronize(st) != cudaSuccess)
		return BFS_ECUDA;
	const BcControl &c = *b.h_ctl;
	if (out) {
		bfs_bc_stats s{};
		s.num_sources = 1;
		s.depth = c.depth;
		s.reached = c.reached;
		s.status = (uint32_t) c.err;
		s.edges_reached = c.edges_reached;
		s.edges_forward = c.edges_fwd;
		s.edges_reverse = c.edges_rev;
		float ms = 0, tms = 0;
		cudaEventElapsedTime(&ms, b.e0, b.e2);
		cudaEventElapsedTime(&tms, b.e0, b.e1);
		s.device_ms = ms;
		s.traversal_ms = tms;
		if (c.t[0] && c.t[1] >= c.t[0]) s.sort_ms = (float) ((c.t[1] - c.t[0]) * 1e-6);
		if (c.t[1] && c.t[2] >= c.t[1]) s.paths_ms = (float) ((c.t[2] - c.t[1]) * 1e-6);
		if (c.t[2] && c.t[3] >= c.t[2]) s.dependencies_ms = (float) ((c.t[3] - c.t[2]) * 1e-6);
		s.grid_ctas = (uint32_t) b.grid;
		for (uint32_t d = 0; d <= c.depth && d < BFS_BC_TRACE_LEVELS; ++d) {
			s.level_vertices[d] = c.lv_vertices[d];
			s.level_big[d] = c.lv_big[d];
			s.level_medium[d] = c.lv_medium[d];
			const unsigned long long f0 = d <= 1 ? c.t[1] : c.t_fwd[d - 1], f1 = c.t_fwd[d];
			if (d > 0 && f0 && f1 >= f0) s.level_paths_ms[d] = (float) ((f1 - f0) * 1e-6);
			// the sweep of level d starts where level d + 1 ended (the deepest
			// level starts at the end of the path counts); past the recorded
			// levels the start is unknown and the entry stays 0
			if (d != c.depth && d + 1 >= BFS_BC_TRACE_LEVELS) continue;
			const unsigned long long r0 = d == c.depth ? c.t[2] : c.t_rev[d + 1], r1 = c.t_rev[d];
			if (r0 && r1 >= r0) s.level_dependencies_ms[d] = (float) ((r1 - r0) * 1e-6);
		}
		*out = s;
	}
	return c.err;
}

// ---- batched betweenness ----------------------------------------------------
template <class T> int bb_alloc(bfs_graph *g, T **out, size_t count) {
	size_t bytes = std::max<size_t>(sizeof(T) * count, 16);
	void *p = nullptr;
	if (cudaMalloc(&p, bytes) != cudaSuccess) {
		cudaGetLastError();
		return BFS_ENOMEM;
	}
	g->bb.bufs.push_back({p, bytes});
	g->bb.bytes += bytes;
	*out = (T *) p;
	return BFS_OK;
}

static_assert(BFS_BC_BATCH_MAX_SOURCES == kBbMaxWords * kBbMaxSources, "a batch is at most kBbMaxWords launches");

// Out-edge chunks (once per graph), the per-(vertex, source) state, and
// (host_out) the [64][n] staging of host outputs.
int bb_prepare(bfs_graph *g, bool host_deps, bool host_paths) {
	int rc;
	if (!g->bb_chunks_ready) {
		std::vector<uint32_t> off((size_t) g->n + 1);
		if (cudaMemcpy(off.data(), g->dg.row_off, sizeof(uint32_t) * off.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
			return BFS_ECUDA;
		std::vector<uint32_t> cv, cb;
		for (uint32_t v = 0; v < g->n; ++v) {
			if (off[v + 1] - off[v] <= kBbBig) continue;
			for (uint32_t e = off[v]; e < off[v + 1]; e += kBbChunk) {
				cv.push_back(v);
				cb.push_back(e);
			}
		}
		g->bb_noch = (uint32_t) cv.size();
		if ((rc = dev_upload(g, &g->bb_ochunk_v, cv)) || (rc = dev_upload(g, &g->bb_ochunk_beg, cb))) return rc;
		g->bb_chunks_ready = true;
	}
	auto &b = g->bb;
	if (!b.ctl) {
		const size_t rows = (size_t) g->n * kBbMaxSources;
		const size_t part = (size_t) std::max(g->ms_nchunks, g->bb_noch) * kBbMaxSources;
		if ((rc = bb_alloc(g, &b.sigma, rows)) || (rc = bb_alloc(g, &b.dsum, rows)) ||
				(rc = bb_alloc(g, &b.partial, part)) || (rc = bb_alloc(g, &b.ctl, kBbMaxWords)) ||
				(rc = bb_alloc(g, &b.d_sources, kBbMaxWords * kBbMaxSources))) {
			release_bb(g);
			return rc;
		}
		if (cudaMallocHost(&b.h_ctl, sizeof(BbControl) * kBbMaxWords) != cudaSuccess ||
				cudaMallocHost(&b.h_ms, sizeof(MsControl)) != cudaSuccess || cudaEventCreate(&b.e0) != cudaSuccess ||
				cudaEventCreate(&b.e1) != cudaSuccess || cudaEventCreate(&b.e2) != cudaSuccess ||
				cudaEventCreate(&b.e3) != cudaSuccess) {
			cudaGetLastError();
			release_bb(g);
			return BFS_ENOMEM;
		}
	}
	const size_t stage = (size_t) g->n * kBbMaxWords * kBbMaxSources;
	if (host_deps && !b.delta && (rc = bb_alloc(g, &b.delta, stage))) return rc;
	if (host_paths && !b.paths && (rc = bb_alloc(g, &b.paths, stage))) return rc;
	return BFS_OK;
}

// Enqueues the batched traversal from `sources` (host, ns <= 64) with its
// planes kept, then the path-count / dependency launch and the output pass
// into delta / paths ([ns][n], device, either may be null) and acc.
int bb_enqueue(bfs_graph *g, const uint32_t *sources, uint32_t ns, float *delta, uint32_t *paths, float *acc,
		cudaStream_t st) {
	if (g->relabeled) return BFS_EUNSUPPORTED;
	const uint32_t K = (ns + kBbMaxSources - 1) / kBbMaxSources;
	uint32_t planes = 0;
	int rc = batch_prepare(g, K, &planes);
	if (rc) return rc;
	auto &b = g->bb;
	if (b.list_planes < planes) {
		// per-level work lists for this many levels (the old ones may still be in use)
		if (cudaStreamSynchronize(st) != cudaSuccess) return BFS_ECUDA;
		for (auto &x : b.lbufs) cudaFree(x.p);
		b.lbufs.clear();
		b.list_planes = 0;
		const size_t nblk = (g->n + 31) / 32;
		const size_t sizes[3] = {planes * nblk, (size_t) planes * g->ms_nchunks, (size_t) planes * g->bb_noch};
		uint32_t **dst[3] = {&b.blist, &b.ilist, &b.olist};
		for (int i = 0; i < 3; ++i) {
			void *p = nullptr;
			const size_t bytes = std::max<size_t>(sizeof(uint32_t) * sizes[i], 16);
			if (cudaMalloc(&p, bytes) != cudaSuccess) {
				cudaGetLastError();
				return BFS_ENOMEM;
			}
			b.lbufs.push_back({p, bytes});
			*dst[i] = (uint32_t *) p;
		}
		b.list_planes = planes;
	}
	const MsArgs a = batch_args(g, K, ns, planes);
	if (cudaEventRecord(b.e0, st) != cudaSuccess) return BFS_ECUDA;
	if (cudaMemcpyAsync(b.d_sources, sources, sizeof(uint32_t) * ns, cudaMemcpyHostToDevice, st) != cudaSuccess)
		return BFS_ECUDA;
	int ms_grid = 0;
	if ((rc = ms_launch(a, b.d_sources, ns, nullptr, g->num_sms, st, &ms_grid, nullptr, nullptr))) return rc;
	if (cudaEventRecord(b.e1, st) != cudaSuccess) return BFS_ECUDA;
	BbArgs x{};
	x.n = g->n;
	x.K = K;
	x.row_off = g->dg.row_off;
	x.col = g->dg.col;
	x.in_off = g->dg.in_off;
	x.in_src = g->dg.in_src;
	x.hist = a.hist;
	x.vis = a.vis;
	x.ms = a.ctl;
	x.ichunk_v = g->ms_chunk_v;
	x.ichunk_beg = g->ms_chunk_beg;
	x.nich = g->ms_nchunks;
	x.ochunk_v = g->bb_ochunk_v;
	x.ochunk_beg = g->bb_ochunk_beg;
	x.noch = g->bb_noch;
	x.sigma = b.sigma;
	x.dsum = b.dsum;
	x.partial = b.partial;
	x.blist = b.blist;
	x.ilist = b.ilist;
	x.olist = b.olist;
	x.planes = b.list_planes;
	x.wait_limit_ns = wait_limit_ns(g->opt);
	x.hold_barrier = g->opt.test_hold_barrier;
	x.ctas_per_sm = g->opt.ctas_per_sm;
	// one launch (and output pass) per word of 64 sources, in source order, so
	// that acc receives the sources in order
	for (uint32_t w = 0; w < K; ++w) {
		x.word = w;
		x.ns = std::min<uint32_t>(kBbMaxSources, ns - w * kBbMaxSources);
		x.ctl = b.ctl + w;
		const size_t row0 = (size_t) w * kBbMaxSources * g->n;
		BbOut o{b.d_sources + w * kBbMaxSources, delta ? delta + row0 : nullptr, paths ? paths + row0 : nullptr, acc};
		if ((rc = bb_launch(x, o, g->num_sms, st, &b.grid, w == 0 ? b.e2 : nullptr))) return rc;
	}
	if (cudaEventRecord(b.e3, st) != cudaSuccess) return BFS_ECUDA;
	b.words = K;
	b.stream = st;
	b.ns = ns;
	g->bc_last_batched = true;
	// the batch buffers now hold this traversal, not a bfs_run_batch result
	g->mb.have_run = false;
	return BFS_OK;
}

// Waits for the last batched betweenness run; its statistics into *out.
int bb_collect(bfs_graph *g, bfs_bc_stats *out) {
	auto &b = g->bb;
	cudaStream_t st = b.stream;
	const uint32_t words = std::max<uint32_t>(1, b.words);
	if (cudaMemcpyAsync(b.h_ctl, b.ctl, sizeof(BbControl) * words, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
			cudaMemcpyAsync(b.h_ms, g->mb.args.ctl, sizeof(MsControl), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
			cudaStreamSynchronize(st) != cudaSuccess)
		return BFS_ECUDA;
	// per-word launches: counters and times add up; the first status wins;
	// the per-level times are the first word's
	const BbControl &c = b.h_ctl[0];
	const MsStats &ms = b.h_ms->stats;
	int err = 0;
	for (uint32_t w = 0; w < words && !err; ++w) err = b.h_ctl[w].err;
	if (out) {
		bfs_bc_stats s{};
		s.num_sources = b.ns;
		s.batched_sources = b.ns;
		s.depth = ms.depth ? ms.depth - 1 : 0;
		s.status = (uint32_t) err;
		s.edges_reached = ms.traversed;
		for (uint32_t w = 0; w < words; ++w) {
			const BbControl &cw = b.h_ctl[w];
			s.edges_forward += cw.fwd[0];
			s.edges_reverse += cw.rev[0];
			s.edges_matched_forward += cw.fwd[1];
			s.edges_matched_reverse += cw.rev[1];
			s.pairs_forward += cw.fwd[2];
			s.pairs_reverse += cw.rev[2];
			if (cw.t[0] && cw.t[1] >= cw.t[0]) s.paths_ms += (float) ((cw.t[1] - cw.t[0]) * 1e-6);
			if (cw.t[1] && cw.t[2] >= cw.t[1]) s.dependencies_ms += (float) ((cw.t[2] - cw.t[1]) * 1e-6);
			const uint32_t nsw = std::min<uint32_t>(kBbMaxSources, b.ns - w * kBbMaxSources);
			for (uint32_t i = 0; i < nsw; ++i) s.source_reached[w * kBbMaxSources + i] = cw.reached[i];
		}
		s.reached = s.source_reached[b.ns - 1];
		float ms_all = 0, tms = 0;
		cudaEventElapsedTime(&ms_all, b.e0, b.e3);
		cudaEventElapsedTime(&tms, b.e0, b.e1);
		s.device_ms = ms_all;
		s.traversal_ms = tms;
		s.grid_ctas = (uint32_t) b.grid;
		for (uint32_t d = 0; d < ms.depth && d < BFS_BC_TRACE_LEVELS && d < kMsTraceLevels; ++d) {
			s.level_vertices[d] = ms.frontier[d];
			if (d >= kBbTraceLevels) continue;
			if (d > 0 && c.t_fwd[d - 1] && c.t_fwd[d] >= c.t_fwd[d - 1])
				s.level_paths_ms[d] = (float) ((c.t_fwd[d] - c.t_fwd[d - 1]) * 1e-6);
			// the dependency sums of level d start where level d + 1 ended (the
			// deepest level: where the path counts ended)
			const bool deepest = d + 1 == ms.depth;
			if (!deepest && d + 1 >= kBbTraceLevels) continue;
			const unsigned long long r0 = deepest ? c.t[1] : c.t_rev[d + 1], r1 = c.t_rev[d];
			if (r0 && r1 >= r0) s.level_dependencies_ms[d] = (float) ((r1 - r0) * 1e-6);
		}
		*out = s;
	}
	return err;
}

// Adds one run's statistics into a total over runs.
void bc_stats_add(bfs_bc_stats &total, const bfs_bc_stats &one) {
	total.depth = std::max(total.depth, one.depth);
	total.reached = one.reached;
	total.edges_reached += one.edges_reached;
	total.edges_forward += one.edges_forward;
	total.edges_reverse += one.edges_reverse;
	total.edges_matched_forward += one.edges_matched_forward;
	total.edges_matched_reverse += one.edges_matched_reverse;
	total.pairs_forward += one.pairs_forward;
	total.pairs_reverse += one.pairs_reverse;
	total.traversal_ms += one.traversal_ms;
	total.sort_ms += one.sort_ms;
	total.paths_ms += one.paths_ms;
	total.dependencies_ms += one.dependencies_ms;
	total.num_sources += one.num_sources;
	total.batched_sources += one.batched_sources;
	total.fallback_sources += one.fallback_sources;
	total.grid_ctas = one.grid_ctas;
	std::memcpy(total.level_paths_ms, one.level_paths_ms, sizeof(one.level_paths_ms));
	std::memcpy(total.level_dependencies_ms, one.level_dependencies_ms, sizeof(one.level_dependencies_ms));
	std::memcpy(total.level_vertices, one.level_vertices, sizeof(one.level_vertices));
	std::memcpy(total.level_big, one.level_big, sizeof(one.level_big));
	std::memcpy(total.level_medium, one.level_medium, sizeof(one.level_medium));
	std::memcpy(total.source_reached, one.source_reached, sizeof(one.source_reached));
}

// One source at a time through bfs_bc_run's kernel (the batch fallback):
// dependencies / path counts to host rows (either may be null), acc added to.
int bc_sources_one_by_one(bfs_graph *g, const uint32_t *sources, uint32_t ns, float *deps, uint32_t *paths,
		float *acc, bfs_bc_stats &total) {
	int rc = bc_prepare(g);
	if (rc) return rc;
	for (uint32_t i = 0; i < ns; ++i) {
		bfs_bc_stats one{};
		if ((rc = bc_enqueue(g, sources[i], nullptr, nullptr, acc, 0))) return rc;
		if ((rc = bc_collect(g, &one))) return rc;
		if (deps && cudaMemcpy(deps + (size_t) i * g->n, g->bc.delta, sizeof(float) * g->n, cudaMemcpyDeviceToHost) !=
				cudaSuccess)
			return BFS_ECUDA;
		if (paths && cudaMemcpy(paths + (size_t) i * g->n, g->bc.sigma, sizeof(uint32_t) * g->n,
						cudaMemcpyDeviceToHost) != cudaSuccess)
			return BFS_ECUDA;
		bc_stats_add(total, one);
	}
	return BFS_OK;
}

} // namespace

struct bfs_batch_graph {
	bfs_graph *g = nullptr;
	uint32_t num_sources = 0;
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t exec = nullptr;
};

// ---- binary graph files ------------------------------------------------------
// A header of fixed-width fields, then every array of the device layout in a
// fixed order, little-endian uint32.  The layout is this library's (CSR,
// in-edge lists, packed column-major segments), not the reference's text
// families; it reloads without parsing or rebuilding.
namespace {

constexpr uint64_t kBinMagic = 0x31304D4247534642ull;  // "BFSGBM01"

struct BinHeader {
	uint64_t magic;
	uint32_t n, w, s, side, num_stripes;
	uint32_t vbits, cbits, num_groups, max_group_vertices;
	uint32_t max_degree, nbig_in, nchunks, reserved;
	uint64_t m, packed_words;
};

constexpr size_t kBinChunk = (size_t) 64 << 20;  // words per host staging chunk

int write_dev(FILE *f, const uint32_t *d, size_t count, std::vector<uint32_t> &buf) {
	for (size_t i = 0; i < count; i += kBinChunk) {
		const size_t c = std::min(kBinChunk, count - i);
		buf.resize(c);
		if (cudaMemcpy(buf.data(), d + i, c * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return BFS_ECUDA;
		if (std::fwrite(buf.data(), 4, c, f) != c) return BFS_EIO;
	}
	return BFS_OK;
}

int read_dev(FILE *f, bfs_graph *g, const uint32_t **out, size_t count, std::vector<uint32_t> &buf) {
	uint32_t *d = nullptr;
	int st = dev_alloc(g, &d, count);
	if (st) return st;
	for (size_t i = 0; i < count; i += kBinChunk) {
		const size_t c = std::min(kBinChunk, count - i);
		buf.resize(c);
		if (std::fread(buf.data(), 4, c, f) != c) return BFS_EFORMAT;
		if (cudaMemcpy(d + i, buf.data(), c * 4, cudaMemcpyHostToDevice) != cudaSuccess) return BFS_ECUDA;
	}
	*out = d;
	return BFS_OK;
}

int save_binary(const bfs_graph *g, FILE *f) {
	const DevGraph &d = g->dg;
	BinHeader h{};
	h.magic = kBinMagic;
	h.n = g->n;
	h.w = g->w;
	h.s = g->s;
	h.side = g->side;
	h.num_stripes = g->num_stripes;
	h.vbits = d.vbits;
	h.cbits = d.cbits;
	h.num_groups = d.num_groups;
	h.max_group_vertices = d.max_group_words * 32;
	h.max_degree = g->max_degree;
	h.nbig_in = g->ms_nbig_in;
	h.nchunks = g->ms_nchunks;
	h.m = g->m;
	h.packed_words = g->packed_words;
	if (std::fwrite(&h, sizeof h, 1, f) != 1) return BFS_EIO;
	if (std::fwrite(g->degrees.data(), 4, g->n, f) != g->n) return BFS_EIO;
	std::vector<uint32_t> buf;
	const size_t nseg = (size_t) g->num_stripes * d.num_groups;
	int st;
	if ((st = write_dev(f, d.row_off, (size_t) g->n + 1, buf)) || (st = write_dev(f, d.col, g->m, buf)) ||
			(st = write_dev(f, d.in_off, (size_t) g->n + 1, buf)) || (st = write_dev(f, d.in_src, g->m, buf)) ||
			(st = write_dev(f, d.packed, g->packed_words, buf)) || (st = write_dev(f, d.seg_off, nseg + 1, buf)) ||
			(st = write_dev(f, d.group_col, (size_t) d.num_groups + 1, buf)) ||
			(st = write_dev(f, d.hasin, ((size_t) g->n + 31) / 32, buf)) ||
			(st = write_dev(f, g->ms_in_big, g->ms_nbig_in, buf)) || (st = write_dev(f, g->ms_chunk_v, g->ms_nchunks, buf)) ||
			(st = write_dev(f, g->ms_chunk_beg, g->ms_nchunks, buf)))
		return st;
	return BFS_OK;
}

int load_binary(bfs_graph *g, FILE *f, uint32_t flags) {
	BinHeader h{};
	if (std::fread(&h, sizeof h, 1, f) != 1 || h.magic != kBinMagic) return BFS_EFORMAT;
	if (h.n == 0 || h.w == 0 || h.s == 0 || h.side != side_length_of(h.n, h.w) ||
			h.num_stripes != (h.side + h.s - 1) / h.s || h.m > 0xFFFFFFFFull || h.num_groups == 0 ||
			h.num_groups > h.side || h.vbits > 31 || h.cbits > 16)
		return BFS_EFORMAT;
	g->n = h.n;
	g->m = h.m;
	g->w = h.w;
	g->s = h.s;
	g->side = h.side;
	g->num_stripes = h.num_stripes;
	g->max_degree = h.max_degree;
	g->host_only = flags & BFS_LOAD_HOST_ONLY;
	default_options(&g->opt);
	g->degrees.resize(h.n);
	if (std::fread(g->degrees.data(), 4, h.n, f) != h.n) return BFS_EFORMAT;
	uint64_t sum = 0;
	for (uint32_t x : g->degrees) sum += x;
	if (sum != h.m) return BFS_EFORMAT;
	if (g->host_only) return BFS_OK;
	int st = device_setup(g);
	if (st) return st;
	PackedTiles pk;
	pk.vbits = h.vbits;
	pk.cbits = h.cbits;
	pk.num_groups = h.num_groups;
	pk.max_group_vertices = h.max_group_vertices;
	DevGraph &d = g->dg;
	std::vector<uint32_t> buf;
	const size_t nseg = (size_t) h.num_stripes * h.num_groups;
	const uint32_t *in_big = nullptr, *chunk_v = nullptr, *chunk_beg = nullptr;
	if ((st = read_dev(f, g, &d.row_off, (size_t) h.n + 1, buf)) || (st = read_dev(f, g, &d.col, h.m, buf)) ||
			(st = read_dev(f, g, &d.in_off, (size_t) h.n + 1, buf)) || (st = read_dev(f, g, &d.in_src, h.m, buf)) ||
			(st = read_dev(f, g, &d.packed, h.packed_words, buf)) || (st = read_dev(f, g, &d.seg_off, nseg + 1, buf)) ||
			(st = read_dev(f, g, &d.group_col, (size_t) h.num_groups + 1, buf)) ||
			(st = read_dev(f, g, &d.hasin, ((size_t) h.n + 31) / 32, buf)) ||
			(st = read_dev(f, g, &in_big, h.nbig_in, buf)) || (st = read_dev(f, g, &chunk_v, h.nchunks, buf)) ||
			(st = read_dev(f, g, &chunk_beg, h.nchunks, buf)))
		return st;
	if (std::fgetc(f) != EOF) return BFS_EFORMAT;  // trailing bytes: not a file this version wrote
	g->ms_in_big = in_big;
	g->ms_chunk_v = chunk_v;
	g->ms_chunk_beg = chunk_beg;
	g->ms_nbig_in = h.nbig_in;
	g->ms_nchunks = h.nchunks;
	set_shape(g, pk, h.packed_words);
	return alloc_run(g);
}

} // namespace

// ---- hooks of the serving loop (server.cpp) ---------------------------------
namespace bfsg {

int batch_reserve(bfs_graph *g, uint32_t K, uint32_t planes, size_t *batch_bytes) {
	if (!g || g->host_only) return BFS_EUNSUPPORTED;
	if (K == 0 || K > BFS_BATCH_MAX_SOURCES / 64 || planes < 2 || planes > kMsMaxLevel + 1) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	if (cudaSetDevice(g->device) != cudaSuccess) return BFS_ECUDA;
	g->opt.batch_planes = planes;
	uint32_t p = 0;
	int st = batch_prepare(g, K, &p);
	if (batch_bytes) *batch_bytes = g->mb.bytes;
	return st;
}

int run_batch_ex(bfs_graph *g, const uint32_t *sources, uint32_t ns, uint8_t *levels, cudaStream_t st,
		cudaEvent_t wait_before, cudaEvent_t between) {
	if (!g) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	return run_batch_impl(g, sources, ns, levels, st, wait_before, between);
}

size_t graph_device_bytes(const bfs_graph *g) { return g ? g->device_bytes : 0; }
uint32_t graph_num_vertices(const bfs_graph *g) { return g ? g->n : 0; }
int graph_device(const bfs_graph *g) { return g ? g->device : -1; }
// a graph the batched kernels can serve (on the device, caller's own ids)
bool graph_on_device(const bfs_graph *g) { return g && !g->host_only && !g->relabeled; }

} // namespace bfsg

extern "C" {

const char *bfs_status_string(int status) {
	switch (status) {
	case BFS_OK: return "ok";
	case BFS_EIO: return "cannot open file";
	case BFS_EFORMAT: return "malformed or inconsistent input";
	case BFS_ENOMEM: return "out of memory";
	case BFS_EARG: return "invalid argument";
	case BFS_EBUDGET: return "over the device-memory budget";
	case BFS_ETIMEOUT: return "device wait timed out";
	case BFS_ECUDA: return "CUDA error";
	case BFS_EUNSUPPORTED: return "unsupported tile width / stripe length";
	case BFS_ENODEV: return "no CUDA device";
	default: return "unknown status";
	}
}

const char *bfs_version(void) { return "bfs_gb300 0.1 (sm_103a)"; }

int bfs_graph_load(const char *data, uint32_t tile_width, uint32_t stripe_length, uint32_t flags, bfs_graph **out) {
	if (!data || !out || tile_width == 0 || stripe_length == 0) return BFS_EARG;
	*out = nullptr;
	HostGraph h;
	int st = resolve_base(data, tile_width, stripe_length, flags, &h.base, &h.used_reorder);
	if (st) return st;
	const bool weighted = flags & BFS_LOAD_WEIGHTED;
	const std::string colp = h.base + "_col-" + std::to_string(stripe_length) + "-coo-tiled-" + std::to_string(tile_width);
	const std::string csrp = h.base + "_untiled";
	uint32_t n, n2;
	uint64_t m, m2;
	if ((st = read_header(colp + "-0", &n, &m))) return st;
	if ((st = read_header(csrp + "-0", &n2, &m2))) return st;
	if (n != n2 || m != m2) return BFS_EFORMAT;
	if ((st = check_shape(n, m, tile_width, stripe_length))) return st;
	init_shape(h, n, m, tile_width, stripe_length);
	const uint64_t num_tiles = (uint64_t) h.side * h.side;
	h.tile_offsets.resize(num_tiles);
	if ((st = read_u32_lines(colp + "-offsets", num_tiles, h.tile_offsets.data()))) return st;
	h.heads.resize(m);
	h.tails.resize(m);
	if ((st = read_split_family(colp, m, weighted, n, h.heads.data(), h.tails.data()))) return st;
	h.degrees.resize(n);
	if ((st = read_u32_lines(csrp + "-nneibor", n, h.degrees.data()))) return st;
	std::vector<uint32_t> csr_src(m);
	h.csr_dst.resize(m);
	if ((st = read_split_family(csrp, m, weighted, n, csr_src.data(), h.csr_dst.data()))) return st;
	if ((st = finish_csr(h))) return st;
	// The CSR sources must match the out-degree file.
	for (uint32_t v = 0; v < n; ++v)
		for (uint32_t e = h.row_off[v]; e < h.row_off[v + 1]; ++e)
			if (csr_src[e] != v) return BFS_EFORMAT;
	if ((st = validate_colmajor(h))) return st;
	return finish_graph(h, flags, out);
}

int bfs_graph_from_edges(uint32_t num_vertices, uint64_t num_edges, const uint32_t *src, const uint32_t *dst,
		uint32_t tile_width, uint32_t stripe_length, uint32_t flags, bfs_graph **out) {
	if (!out || (num_edges && (!src || !dst))) return BFS_EARG;
	*out = nullptr;
	int st = check_shape(num_vertices, num_edges, tile_width, stripe_length);
	if (st) return st;
	const bool degree_order_layout = flags & BFS_LOAD_DEGREE_ORDER;
	if ((flags & BFS_LOAD_DEVICE_BUILD) && !(flags & BFS_LOAD_HOST_ONLY)) {
		bfs_graph *g = new bfs_graph();
		std::vector<uint32_t> new_of_old;
		st = upload_device_build(g, num_vertices, num_edges, src, dst, tile_width, stripe_length,
				degree_order_layout ? &new_of_old : nullptr);
		if (!st && degree_order_layout) st = attach_relabel(g, std::move(new_of_old));
		if (st) {
			release(g);
			delete g;
			return st;
		}
		*out = g;
		return BFS_OK;
	}
	// the degree-ordered layout on the host: relabelled copies of the edges
	std::vector<uint32_t> rs, rd, new_of_old;
	if (degree_order_layout) {
		std::vector<uint32_t> deg(num_vertices, 0);
		for (uint64_t i = 0; i < num_edges; ++i) {
			if (src[i] >= num_vertices || dst[i] >= num_vertices) return BFS_EFORMAT;
			deg[src[i]]++;
		}
		new_of_old = degree_order(deg);
		rs.resize(num_edges);
		rd.resize(num_edges);
		parallel_for(num_edges, [&](uint64_t lo, uint64_t hi, unsigned) {
			for (uint64_t i = lo; i < hi; ++i) {
				rs[i] = new_of_old[src[i]];
				rd[i] = new_of_old[dst[i]];
			}
		});
		src = rs.data();
		dst = rd.data();
	}
	HostGraph h;
	init_shape(h, num_vertices, num_edges, tile_width, stripe_length);
	std::vector<uint32_t> cs;
	if ((st = csr_from_edges(num_vertices, num_edges, src, dst, cs, h.csr_dst, h.degrees))) return st;
	if ((st = finish_csr(h))) return st;
	if ((st = colmajor_from_csr(num_vertices, num_edges, tile_width, stripe_length, cs.data(), h.csr_dst.data(),
				 h.heads, h.tails, nullptr)))
		return st;
	if ((st = finish_graph(h, flags, out))) return st;
	if (degree_order_layout && (st = attach_relabel(*out, std::move(new_of_old)))) {
		bfs_graph_free(*out);
		*out = nullptr;
		return st;
	}
	return BFS_OK;
}

int bfs_graph_from_arrays(uint32_t num_vertices, uint64_t num_edges, const uint32_t *degrees, const uint32_t *csr_dst,
		const uint32_t *heads, const uint32_t *tails, const uint32_t *tile_offsets, uint32_t tile_width,
		uint32_t stripe_length, uint32_t flags, bfs_graph **out) {
	if (!out || !degrees || (num_edges && (!csr_dst || !heads || !tails))) return BFS_EARG;
	*out = nullptr;
	int st = check_shape(num_vertices, num_edges, tile_width, stripe_length);
	if (st) return st;
	HostGraph h;
	init_shape(h, num_vertices, num_edges, tile_width, stripe_length);
	h.degrees.assign(degrees, degrees + num_vertices);
	h.csr_dst.assign(csr_dst, csr_dst + num_edges);
	for (uint64_t i = 0; i < num_edges; ++i)
		if (h.csr_dst[i] >= num_vertices) return BFS_EFORMAT;
	if ((st = finish_csr(h))) return st;
	h.heads.assign(heads, heads + num_edges);
	h.tails.assign(tails, tails + num_edges);
	if (tile_offsets) h.tile_offsets.assign(tile_offsets, tile_offsets + (uint64_t) h.side * h.side);
	if ((st = validate_colmajor(h))) return st;
	return finish_graph(h, flags, out);
}

int bfs_graph_bfs_order(bfs_graph *g, uint32_t source, uint32_t *vertex_map) {
	if (!g || !vertex_map) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	int st = run_impl(g, source, g->level_buf, g->parent_buf, 0);
	if (st) return st;
	if ((st = collect_stats(g, nullptr))) return st;
	std::vector<int32_t> lev(g->n);
	if (cudaMemcpy(lev.data(), g->level_buf, sizeof(int32_t) * g->n, cudaMemcpyDeviceToHost) != cudaSuccess)
		return BFS_ECUDA;
	// labels by (level, old id); unreached vertices last, by old id
	int32_t maxl = -1;
	for (int32_t l : lev) maxl = std::max(maxl, l);
	std::vector<uint32_t> off((size_t) maxl + 3, 0);
	for (int32_t l : lev) off[(l < 0 ? maxl + 1 : l) + 1]++;
	for (size_t i = 1; i < off.size(); ++i) off[i] += off[i - 1];
	for (uint32_t v = 0; v < g->n; ++v) vertex_map[v] = off[lev[v] < 0 ? maxl + 1 : lev[v]]++;
	return BFS_OK;
}

int bfs_graph_save(const bfs_graph *g, const char *path) {
	if (!g || !path) return BFS_EARG;
	if (g->host_only || g->relabeled) return BFS_EUNSUPPORTED;
	if (cudaSetDevice(g->device) != cudaSuccess) return BFS_ECUDA;
	FILE *f = std::fopen(path, "wb");
	if (!f) return BFS_EIO;
	const int st = save_binary(g, f);
	const bool closed = std::fclose(f) == 0;
	return st ? st : (closed ? BFS_OK : BFS_EIO);
}

int bfs_graph_load_binary(const char *path, uint32_t flags, bfs_graph **out) {
	if (!path || !out) return BFS_EARG;
	*out = nullptr;
	FILE *f = std::fopen(path, "rb");
	if (!f) return BFS_EIO;
	bfs_graph *g = new bfs_graph();
	const int st = load_binary(g, f, flags);
	std::fclose(f);
	if (st) {
		release(g);
		delete g;
		return st;
	}
	*out = g;
	return BFS_OK;
}

int bfs_graph_free(bfs_graph *g) {
	if (!g) return BFS_EARG;
	release(g);
	delete g;
	return BFS_OK;
}

int bfs_graph_get_info(const bfs_graph *g, bfs_graph_info *info) {
	if (!g || !info) return BFS_EARG;
	std::memset(info, 0, sizeof(*info));
	info->num_vertices = g->n;
	info->num_edges = g->m;
	info->tile_width = g->w;
	info->stripe_length = g->s;
	info->side_length = g->side;
	info->num_tiles = (uint64_t) g->side * g->side;
	info->num_stripes = g->num_stripes;
	info->num_groups = g->num_groups;
	info->packed_words = g->packed_words;
	info->device_bytes = g->device_bytes;
	info->max_out_degree = g->max_degree;
	info->used_reorder = g->used_reorder ? 1u : 0u;
	std::snprintf(info->base, sizeof(info->base), "%s", g->base.c_str());
	return BFS_OK;
}

int bfs_graph_get_degrees(const bfs_graph *g, uint32_t *degrees) {
	if (!g || !degrees) return BFS_EARG;
	std::memcpy(degrees, g->degrees.data(), sizeof(uint32_t) * g->n);
	return BFS_OK;
}

int bfs_options_default(bfs_options *opt) {
	if (!opt) return BFS_EARG;
	default_options(opt);
	return BFS_OK;
}

int bfs_set_options(bfs_graph *g, const bfs_options *opt) {
	if (!g || !opt) return BFS_EARG;
	if (opt->mode > BFS_MODE_STEPWISE || opt->bottom_up > BFS_BU_STREAM || opt->to_dense_ratio == 0 || opt->to_sparse_ratio == 0 ||
			opt->warp_max_degree == 0 || opt->cta_max_degree < opt->warp_max_degree || opt->batch_planes == 1 ||
			opt->batch_planes > kMsMaxLevel + 1 || (opt->batch_planes == 0 && opt->batch_budget_mb == 0) ||
			opt->batch_push_div == 0 || opt->bc_level_bytes > 2 || opt->switch_rule > BFS_SWITCH_UNVISITED ||
			opt->bu_alpha == 0 || opt->td_beta == 0 || opt->ctas_per_sm > 2 || opt->bc_batch > 1 ||
			(opt->batch_output_tile != 0 && opt->batch_output_tile != 64 && opt->batch_output_tile != 128))
		return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	g->opt = *opt;
	// the cooperative grid: the occupancy bound found at set-up, or fewer CTAs per SM
	if (!g->host_only && g->grid_max)
		g->grid = opt->ctas_per_sm ? std::min(g->grid_max, (int) opt->ctas_per_sm * g->num_sms) : g->grid_max;
	return BFS_OK;
}

int bfs_get_options(const bfs_graph *g, bfs_options *opt) {
	if (!g || !opt) return BFS_EARG;
	*opt = g->opt;
	return BFS_OK;
}

int bfs_run(bfs_graph *g, uint32_t source, int32_t *levels, uint32_t *parents, bfs_stats *stats) {
	if (!g) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	int st = run_impl(g, source, g->level_buf, parents ? g->parent_buf : nullptr, 0);
	if (st) return st;
	// the outputs' and the statistics' copies are queued behind the
	// traversal, then one wait
	if ((st = enqueue_to_host((uint32_t *) levels, (const uint32_t *) g->level_buf, g->n, g->num_sms, 0)) ||
			(st = enqueue_to_host(parents, g->parent_buf, g->n, g->num_sms, 0)))
		return st;
	static_assert(sizeof(DevStats) % 4 == 0, "the statistics are copied as 32-bit words");
	if (stats && !g->stepwise_last) {
		if ((st = enqueue_to_host((uint32_t *) g->h_stats, (const uint32_t *) g->rc.stats, sizeof(DevStats) / 4,
					 g->num_sms, 0)))
			return st;
		if (cudaStreamSynchronize(0) != cudaSuccess) return BFS_ECUDA;
		g->stats_fresh = true;
	}
	return collect_stats(g, stats);
}

int bfs_run_device(bfs_graph *g, uint32_t source, int32_t *levels, uint32_t *parents, void *stream) {
	if (!g) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	return run_impl(g, source, levels, parents, (cudaStream_t) stream);
}

int bfs_last_stats(bfs_graph *g, bfs_stats *stats) {
	if (!g) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	return collect_stats(g, stats);
}

int bfs_run_batch(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, uint8_t *levels, void *stream,
		bfs_batch_stats *stats) {
	if (!g) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	int st = run_batch_impl(g, sources, num_sources, levels, (cudaStream_t) stream);
	if (st || !stats) return st;
	return collect_batch_stats(g, stats);
}

int bfs_run_batch_device(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, uint8_t *levels, void *stream) {
	if (!g) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	return run_batch_impl(g, sources, num_sources, levels, (cudaStream_t) stream, nullptr, nullptr, true);
}

int bfs_batch_graph_create(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, uint8_t *levels,
		bfs_batch_graph **out) {
	if (!g || !out) return BFS_EARG;
	*out = nullptr;
	std::lock_guard<std::mutex> lk(g->mu);
	if (g->host_only || g->relabeled) return BFS_EUNSUPPORTED;
	if (!sources || !levels || num_sources == 0 || num_sources > BFS_BATCH_MAX_SOURCES) return BFS_EARG;
	if (cudaSetDevice(g->device) != cudaSuccess) return BFS_ECUDA;
	// allocate the batch state before capturing (no allocation inside a capture)
	uint32_t planes = 0;
	int rc = batch_prepare(g, (num_sources + 63) / 64, &planes);
	if (rc) return rc;
	cudaStream_t cs = nullptr;
	if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return BFS_ECUDA;
	bfs_batch_graph *bg = new bfs_batch_graph();
	bg->g = g;
	bg->num_sources = num_sources;
	rc = BFS_ECUDA;
	if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
		rc = run_batch_impl(g, sources, num_sources, levels, cs, nullptr, nullptr, true);
		cudaGraph_t graph = nullptr;
		const cudaError_t e = cudaStreamEndCapture(cs, &graph);
		if (rc == BFS_OK && e == cudaSuccess && graph) {
			bg->graph = graph;
			rc = cudaGraphInstantiate(&bg->exec, graph, 0) == cudaSuccess ? BFS_OK : BFS_ECUDA;
		} else {
			if (graph) cudaGraphDestroy(graph);
			if (rc == BFS_OK) rc = BFS_ECUDA;
		}
	}
	cudaGetLastError();
	cudaStreamDestroy(cs);
	g->mb.have_run = false;
	if (rc) {
		if (bg->exec) cudaGraphExecDestroy(bg->exec);
		if (bg->graph) cudaGraphDestroy(bg->graph);
		delete bg;
		return rc;
	}
	*out = bg;
	return BFS_OK;
}

int bfs_batch_graph_launch(bfs_batch_graph *bg, void *stream) {
	if (!bg || !bg->exec) return BFS_EARG;
	bfs_graph *g = bg->g;
	std::lock_guard<std::mutex> lk(g->mu);
	auto &b = g->mb;
	cudaStream_t st = (cudaStream_t) stream;
	if (cudaEventRecord(b.e0, st) != cudaSuccess || cudaGraphLaunch(bg->exec, st) != cudaSuccess ||
			cudaEventRecord(b.e1, st) != cudaSuccess)
		return BFS_ECUDA;
	b.num_sources = bg->num_sources;
	b.args.K = (bg->num_sources + 63) / 64;
	b.stream = st;
	b.have_run = true;
	b.fresh = false;
	b.singles = false;
	b.em_valid = false;
	return BFS_OK;
}

int bfs_batch_graph_destroy(bfs_batch_graph *bg) {
	if (!bg) return BFS_EARG;
	if (bg->exec) cudaGraphExecDestroy(bg->exec);
	if (bg->graph) cudaGraphDestroy(bg->graph);
	delete bg;
	return BFS_OK;
}

int bfs_last_batch_stats(bfs_graph *g, bfs_batch_stats *stats) {
	if (!g) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	return collect_batch_stats(g, stats);
}

// ---- betweenness (apps/betweennessCentrality_simd/bc.cpp:1717) ------------

int bfs_bc_run(bfs_graph *g, uint32_t source, float *dependencies, uint32_t *num_paths, bfs_bc_stats *stats) {
	if (!g) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	if (g->host_only) return BFS_EUNSUPPORTED;
	if (source >= g->n) return BFS_EARG;
	if (cudaSetDevice(g->device) != cudaSuccess) return BFS_ECUDA;
	int rc = bc_prepare(g);
	if (rc) return rc;
	if ((rc = bc_enqueue(g, source, nullptr, nullptr, nullptr, 0))) return rc;
	if ((rc = bc_collect(g, stats))) return rc;
	if (dependencies &&
			cudaMemcpy(dependencies, g->bc.delta, sizeof(float) * g->n, cudaMemcpyDeviceToHost) != cudaSuccess)
		return BFS_ECUDA;
	if (num_paths && cudaMemcpy(num_paths, g->bc.sigma, sizeof(uint32_t) * g->n, cudaMemcpyDeviceToHost) != cudaSuccess)
		return BFS_ECUDA;
	return BFS_OK;
}

int bfs_bc_run_device(bfs_graph *g, uint32_t source, float *dependencies, uint32_t *num_paths, void *stream) {
	if (!g) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	if (g->host_only) return BFS_EUNSUPPORTED;
	if (source >= g->n) return BFS_EARG;
	if (cudaSetDevice(g->device) != cudaSuccess) return BFS_ECUDA;
	int rc = bc_prepare(g);
	if (rc) return rc;
	return bc_enqueue(g, source, num_paths, dependencies, nullptr, (cudaStream_t) stream);
}

int bfs_bc_last_stats(bfs_graph *g, bfs_bc_stats *stats) {
	if (!g || !stats) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	if (g->bc_last_batched) return bb_collect(g, stats);
	if (!g->bc.ctl) return BFS_EARG;
	return bc_collect(g, stats);
}

int bfs_bc_run_batch(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, float *dependencies,
		uint32_t *num_paths, bfs_bc_stats *stats) {
	if (!g || !sources || num_sources == 0 || num_sources > BFS_BC_BATCH_MAX_SOURCES) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	if (g->host_only) return BFS_EUNSUPPORTED;
	for (uint32_t i = 0; i < num_sources; ++i)
		if (sources[i] >= g->n) return BFS_EARG;
	if (cudaSetDevice(g->device) != cudaSuccess) return BFS_ECUDA;
	int rc = bb_prepare(g, dependencies != nullptr, num_paths != nullptr);
	if (rc) return rc;
	auto &b = g->bb;
	if ((rc = bb_enqueue(g, sources, num_sources, dependencies ? b.delta : nullptr, num_paths ? b.paths : nullptr,
				 nullptr, 0)))
		return rc;
	bfs_bc_stats s{};
	rc = bb_collect(g, &s);
	if (rc == BFS_EUNSUPPORTED) {
		// deeper than the planes: one source at a time
		bfs_bc_stats total{};
		if ((rc = bc_sources_one_by_one(g, sources, num_sources, dependencies, num_paths, nullptr, total))) return rc;
		total.fallback_sources = num_sources;
		if (stats) *stats = total;
		return BFS_OK;
	}
	if (rc) return rc;
	const size_t cells = (size_t) num_sources * g->n;
	if (dependencies && cudaMemcpy(dependencies, b.delta, sizeof(float) * cells, cudaMemcpyDeviceToHost) != cudaSuccess)
		return BFS_ECUDA;
	if (num_paths && cudaMemcpy(num_paths, b.paths, sizeof(uint32_t) * cells, cudaMemcpyDeviceToHost) != cudaSuccess)
		return BFS_ECUDA;
	if (stats) *stats = s;
	return BFS_OK;
}

int bfs_bc_run_batch_device(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, float *dependencies,
		uint32_t *num_paths, void *stream) {
	if (!g || !sources || num_sources == 0 || num_sources > BFS_BC_BATCH_MAX_SOURCES) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	if (g->host_only) return BFS_EUNSUPPORTED;
	for (uint32_t i = 0; i < num_sources; ++i)
		if (sources[i] >= g->n) return BFS_EARG;
	if (cudaSetDevice(g->device) != cudaSuccess) return BFS_ECUDA;
	int rc = bb_prepare(g, false, false);
	if (rc) return rc;
	return bb_enqueue(g, sources, num_sources, dependencies, num_paths, nullptr, (cudaStream_t) stream);
}

int bfs_bc_accumulate(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, float *centrality,
		bfs_bc_stats *stats) {
	if (!g || !sources || !num_sources || !centrality) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	if (g->host_only) return BFS_EUNSUPPORTED;
	for (uint32_t i = 0; i < num_sources; ++i)
		if (sources[i] >= g->n) return BFS_EARG;
	if (cudaSetDevice(g->device) != cudaSuccess) return BFS_ECUDA;
	int rc = bc_prepare(g);
	if (rc) return rc;
	auto &b = g->bc;
	if (g->opt.bc_batch && (rc = bb_prepare(g, false, false))) return rc;
	if (cudaMemsetAsync(b.acc, 0, sizeof(float) * g->n, 0) != cudaSuccess) return BFS_ECUDA;
	cudaEvent_t start = nullptr, end = nullptr;
	if (cudaEventCreate(&start) != cudaSuccess || cudaEventCreate(&end) != cudaSuccess ||
			cudaEventRecord(start, 0) != cudaSuccess) {
		if (start) cudaEventDestroy(start);
		if (end) cudaEventDestroy(end);
		return BFS_ECUDA;
	}
	bfs_bc_stats total{};
	if (!g->opt.bc_batch) {
		rc = bc_sources_one_by_one(g, sources, num_sources, nullptr, nullptr, b.acc, total);
	} else {
		// groups of up to 64 sources; a group deeper than the planes one source at a time
		for (uint32_t i = 0; i < num_sources && rc == BFS_OK; i += BFS_BC_BATCH_MAX_SOURCES) {
			const uint32_t k = std::min<uint32_t>(BFS_BC_BATCH_MAX_SOURCES, num_sources - i);
			bfs_bc_stats one{};
			rc = bb_enqueue(g, sources + i, k, nullptr, nullptr, b.acc, 0);
			if (rc == BFS_OK) rc = bb_collect(g, &one);
			if (rc == BFS_EUNSUPPORTED) {
				bfs_bc_stats part{};
				rc = bc_sources_one_by_one(g, sources + i, k, nullptr, nullptr, b.acc, part);
				part.fallback_sources = k;
				if (rc == BFS_OK) bc_stats_add(total, part);
			} else if (rc == BFS_OK) {
				bc_stats_add(total, one);
			}
		}
	}
	float ms = 0;
	if (rc == BFS_OK && cudaEventRecord(end, 0) == cudaSuccess && cudaEventSynchronize(end) == cudaSuccess)
		cudaEventElapsedTime(&ms, start, end);
	cudaEventDestroy(start);
	cudaEventDestroy(end);
	if (rc) return rc;
	total.device_ms = ms;
	if (stats) *stats = total;
	if (cudaMemcpy(centrality, b.acc, sizeof(float) * g->n, cudaMemcpyDeviceToHost) != cudaSuccess) return BFS_ECUDA;
	return BFS_OK;
}

int bfs_bc_accumulate_device(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, float *centrality,
		void *stream) {
	if (!g || !sources || !num_sources || !centrality) return BFS_EARG;
	std::lock_guard<std::mutex> lk(g->mu);
	if (g->host_only) return BFS_EUNSUPPORTED;
	for (uint32_t i = 0; i < num_sources; ++i)
		if (sources[i] >= g->n) return BFS_EARG;
	if (cudaSetDevice(g->device) != cudaSuccess) return BFS_ECUDA;
	int rc = bc_prepare(g);
	if (rc) return rc;
	for (uint32_t i = 0; i < num_sources; ++i)
		if ((rc = bc_enqueue(g, sources[i], nullptr, nullptr, centrality, (cudaStream_t) stream))) return rc;
	return BFS_OK;
}

} // extern "C"
