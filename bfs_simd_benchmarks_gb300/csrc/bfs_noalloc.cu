// bfs_noalloc.cu -- an allocation-free single-source BFS.
//
// Some callers cannot call cudaMalloc: a plug-in whose host framework
// reserves the device memory up front and hands none out afterwards, or a
// latency-bound request path that cannot accept the device-wide
// synchronisation and unbounded time of cudaMalloc / cudaFree.
// bfs_run_noalloc serves them: the caller passes the graph (a CSR already on
// the device) and the output buffer, and the traversal's scratch -- visited
// bitmap, two frontier queues, counters -- lives in one file-scope device
// array of fixed size, so no call allocates anything.
//
// Limits and sharing:
//   - at most BFS_NOALLOC_MAX_VERTICES vertices (larger graphs are rejected
//     with BFS_EUNSUPPORTED before anything is launched);
//   - the scratch array exists once per device that loads the library and is
//     kept until the process exits; every call on that device uses it and it
//     keeps the previous call's contents, so each call clears what must start
//     at zero;
//   - calls whose work overlaps on the GPU (different streams, or host
//     threads) race on the shared scratch: serialise them;
//   - the first call on a device does a one-time set-up (it looks up the
//     device address of the scratch array); make that first call before any
//     stream capture;
//   - the CSR is checked as it is read: a column id >= num_vertices is
//     skipped and the call's status becomes BFS_EARG (the offsets themselves
//     must be non-decreasing and end inside the column array).
//
// The kernel is a top-down-only variant of the traversal kernel: one
// cooperative launch runs every level, separated by a bounded-spin grid
// barrier; a warp expands one frontier vertex at a time and claims
// destinations with atomicOr on the visited bitmap.
#include <mutex>

#include "../../include/bfs_gb300.h"
#include "device_common.cuh"

namespace {

constexpr uint32_t kNaThreads = 256;
constexpr uint32_t kNaWarps = kNaThreads / 32;
constexpr int kNaMaxDevices = 64;

struct NoAllocScratch {
	uint32_t vis[BFS_NOALLOC_MAX_VERTICES / 32];
	uint32_t queue[2][BFS_NOALLOC_MAX_VERTICES];
	uint32_t tail[3];   // frontier sizes, rotating by level
	uint32_t bar[2];    // grid barrier
	int err;
};

// The scratch of every bfs_run_noalloc call on this device (~8.1 MB).
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

__global__ void __launch_bounds__(kNaThreads) k_noalloc_bfs(const uint32_t *__restrict__ row_off,
		const uint32_t *__restrict__ col, uint32_t n, uint32_t source, int32_t *level, int32_t *status,
		NoAllocScratch *s) {
	using namespace bfsg;
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	const uint64_t t0 = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x;
	// The previous call left its state behind: clear what must start at zero.
	// The barrier words were reset by the host before the launch.
	for (uint64_t i = t0; i < n; i += stride) level[i] = -1;
	for (uint64_t i = t0; i < (n + 31) / 32; i += stride) s->vis[i] = 0;
	if (t0 == 0) {
		s->tail[0] = s->tail[1] = s->tail[2] = 0;
		s->err = 0;
	}
	// *status was zeroed by the host before the launch; every CTA that ends
	// on an error raises it below, so no CTA's late error is lost.
	bool ok = grid_barrier(s->bar, &s->err);
	if (ok && t0 == 0) {
		level[source] = 0;
		s->vis[source >> 5] = 1u << (source & 31);
		s->queue[0][0] = source;
		s->tail[0] = 1;
	}
	if (ok) ok = grid_barrier(s->bar, &s->err);
	const unsigned lane = lane_id();
	const uint64_t gwarp = (uint64_t) blockIdx.x * kNaWarps + warp_id();
	const uint64_t nwarps = (uint64_t) gridDim.x * kNaWarps;
	for (uint32_t lvl = 0; ok; ++lvl) {
		const uint32_t nq = ld_volatile(&s->tail[lvl % 3]);
		if (nq == 0) break;
		if (t0 == 0) s->tail[(lvl + 2) % 3] = 0;  // the slot of the next level but one
		const uint32_t *q = s->queue[lvl & 1];
		uint32_t *qn = s->queue[(lvl + 1) & 1];
		uint32_t *tn = &s->tail[(lvl + 1) % 3];
		for (uint64_t i = gwarp; i < nq; i += nwarps) {
			const uint32_t u = ld_cg(q + i);
			const uint32_t beg = __ldg(row_off + u), end = __ldg(row_off + u + 1);
			for (uint32_t e0 = beg; e0 < end; e0 += 32) {
				const uint32_t e = e0 + lane;
				bool claimed = false;
				uint32_t v = 0;
				if (e < end) {
					v = __ldg(col + e);
					if (v < n) {
						const uint32_t bit = 1u << (v & 31);
						if (!(ld_cg(s->vis + (v >> 5)) & bit))
							claimed = !(atomicOr(s->vis + (v >> 5), bit) & bit);
					} else {
						atomicExch(&s->err, 4 /* BFS_EARG: a column id out of range */);
					}
				}
				const unsigned mask = __ballot_sync(kFull, claimed);
				if (!mask) continue;
				const int leader = __ffs(mask) - 1;
				uint32_t base = 0;
				if (lane == (unsigned) leader) base = atomicAdd(tn, (unsigned) __popc(mask));
				base = __shfl_sync(kFull, base, leader);
				if (claimed) {
					level[v] = (int32_t) lvl + 1;
					qn[base + __popc(mask & lanemask_lt())] = v;
				}
			}
		}
		ok = grid_barrier(s->bar, &s->err);
	}
	// Every CTA reports what it saw: a CTA whose barrier gave up after CTA 0
	// had finished still raises the status (codes are positive, BFS_OK is 0).
	if (threadIdx.x == 0 && status) {
		const int e = *(volatile int *) &s->err;
		if (e) atomicMax(status, e);
	}
}

struct DeviceSetup {
	bool done = false;
	NoAllocScratch *scratch = nullptr;  // device address of g_noalloc_scratch
	int grid = 0;
};
DeviceSetup g_setup[kNaMaxDevices];
std::mutex g_setup_mu;

} // namespace

extern "C" int bfs_run_noalloc(uint32_t num_vertices, const uint32_t *row_offsets, const uint32_t *columns,
		uint32_t source, int32_t *levels, int32_t *status, void *stream) {
	if (!row_offsets || !columns || !levels || num_vertices == 0 || source >= num_vertices) return BFS_EARG;
	if (num_vertices > BFS_NOALLOC_MAX_VERTICES) return BFS_EUNSUPPORTED;
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return BFS_ECUDA;
	DeviceSetup su;
	{
		std::lock_guard<std::mutex> lk(g_setup_mu);
		DeviceSetup &d = g_setup[dev];
		if (!d.done) {
			// One-time set-up on this device (the device is current): the host
			// name g_noalloc_scratch is not a device address; ask for it.
			void *ptr = nullptr;
			if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess) return BFS_ECUDA;
			int sms = 0, per_sm = 0, coop = 0;
			if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
					cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess ||
					cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_noalloc_bfs, kNaThreads, 0) != cudaSuccess)
				return BFS_ECUDA;
			if (!coop || per_sm < 1) return BFS_EUNSUPPORTED;
			d.scratch = (NoAllocScratch *) ptr;
			d.grid = sms * (per_sm < 4 ? per_sm : 4);
			d.done = true;
		}
		su = d;
	}
	cudaStream_t st = (cudaStream_t) stream;
	// The grid barrier's words must be zero when the launch starts, and so
	// must the status, which the kernel's CTAs only raise.
	if (cudaMemsetAsync(su.scratch->bar, 0, sizeof(su.scratch->bar), st) != cudaSuccess) return BFS_ECUDA;
	if (status && cudaMemsetAsync(status, 0, sizeof(int32_t), st) != cudaSuccess) return BFS_ECUDA;
	uint32_t n = num_vertices;
	NoAllocScratch *sp = su.scratch;
	void *args[] = {(void *) &row_offsets, (void *) &columns, &n, &source, &levels, &status, &sp};
	if (cudaLaunchCooperativeKernel((const void *) k_noalloc_bfs, dim3(su.grid), dim3(kNaThreads), args, 0, st) !=
			cudaSuccess)
		return BFS_ECUDA;
	return BFS_OK;
}
