// device_common.cuh -- device-side helpers shared by the BFS kernels:
// bit helpers, warp aggregation, bounded waits and the grid barrier.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bfsg {

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned warp_id() { return threadIdx.x >> 5; }
__device__ __forceinline__ unsigned lanemask_lt() {
	unsigned m;
	asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
	return m;
}
__device__ __forceinline__ uint64_t global_timer_ns() {
	uint64_t t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

// Loads of data that other CTAs wrote in an earlier phase of the same
// persistent launch go through L2 (.cg) so that no stale L1 line is read.
__device__ __forceinline__ uint32_t ld_cg(const uint32_t *p) { return __ldcg(p); }
__device__ __forceinline__ uint8_t ld_cg_u8(const uint8_t *p) {
	return (uint8_t) __ldcg((const unsigned char *) p);
}
__device__ __forceinline__ uint32_t ld_volatile(const uint32_t *p) { return *(const volatile uint32_t *) p; }
__device__ __forceinline__ unsigned long long ld_volatile_u64(const unsigned long long *p) {
	return *(const volatile unsigned long long *) p;
}
// Immutable graph data: read-only path.
__device__ __forceinline__ uint4 ldg_v4(const uint32_t *p) { return __ldg((const uint4 *) p); }

// 32 bits of a bitmap starting at bit `bit` (any alignment); bits at or beyond
// `limit` read as `fill` (0 or all ones).
__device__ __forceinline__ uint32_t bits_at(const uint32_t *bm, uint64_t bit, uint64_t limit, uint32_t fill) {
	uint32_t out;
	if (bit >= limit) return fill;
	uint64_t w = bit >> 5;
	unsigned sh = (unsigned) (bit & 31);
	uint64_t lim_w = (limit + 31) >> 5;
	uint32_t lo = ld_cg(bm + w);
	if (sh == 0) out = lo;
	else {
		uint32_t hi = (w + 1 < lim_w) ? ld_cg(bm + w + 1) : 0u;
		out = (lo >> sh) | (hi << (32 - sh));
	}
	uint64_t valid = limit - bit;
	if (valid < 32) {
		uint32_t keep = (1u << valid) - 1u;
		out = (out & keep) | (fill & ~keep);
	}
	return out;
}

// ORs 32 bits into a bitmap starting at bit `bit` (any alignment).
__device__ __forceinline__ void or_bits_at(uint32_t *bm, uint64_t bit, uint32_t bits) {
	if (!bits) return;
	uint64_t w = bit >> 5;
	unsigned sh = (unsigned) (bit & 31);
	if (sh == 0) {
		atomicOr(bm + w, bits);
	} else {
		uint32_t lo = bits << sh, hi = bits >> (32 - sh);
		if (lo) atomicOr(bm + w, lo);
		if (hi) atomicOr(bm + w + 1, hi);
	}
}

// Bounded spin limits: a device wait gives up after this long, records
// BFS_ETIMEOUT and lets the kernel return instead of hanging the GPU.
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s
constexpr uint32_t kWaitLimitIters = 1u << 26;

// Grid barrier for a cooperative launch (all CTAs co-resident).  bar[0] is the
// arrival count, bar[1] the generation; *err becomes non-zero when any CTA
// timed out, and every later barrier returns false at once.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, int *err) {
	__shared__ int s_ok;
	__syncthreads();
	if (threadIdx.x == 0) {
		int ok = 1;
		volatile unsigned *gen_p = bar + 1;
		unsigned gen = *gen_p;
		__threadfence();
		unsigned arrived = atomicAdd(bar, 1u);
		if (arrived == gridDim.x - 1) {
			atomicExch(bar, 0u);
			__threadfence();
			atomicAdd(bar + 1, 1u);
		} else {
			uint64_t t0 = global_timer_ns();
			uint32_t it = 0;
			while (*gen_p == gen) {
				if (*(volatile int *) err) { ok = 0; break; }
				if (++it > kWaitLimitIters || global_timer_ns() - t0 > kWaitLimitNs) {
					atomicExch(err, 6 /* BFS_ETIMEOUT */);
					ok = 0;
					break;
				}
				__nanosleep(it < 64 ? 32 : 256);
			}
		}
		__threadfence();
		if (*(volatile int *) err) ok = 0;
		s_ok = ok;
	}
	__syncthreads();
	return s_ok != 0;
}

// Grid barrier over a monotonic arrival counter (*count is 0 when the launch
// starts; `epoch` is the number of these barriers the CTA has passed, the
// same in every CTA).  Arrival is a fire-and-forget add after a fence; the
// barrier is complete when the counter reaches gridDim.x * (epoch + 1), which
// every CTA sees by polling the counter itself -- no generation word to read
// before arriving, no reset, no separate release write.  Bounded like
// grid_barrier: gives up after kWaitLimitNs, records BFS_ETIMEOUT.
// `limit_ns` bounds the wait; `hold` (tests only) = the epoch at which CTA 0
// does not arrive, so that every CTA's wait runs out (0 = never).
__device__ __forceinline__ bool grid_sync(unsigned *count, unsigned &epoch, int *err,
		uint64_t limit_ns = kWaitLimitNs, unsigned hold = 0) {
	__shared__ int s_sync_ok;
	__syncthreads();
	++epoch;
	if (threadIdx.x == 0) {
		int ok = 1;
		const unsigned target = gridDim.x * epoch;
		__threadfence();
		if (!(hold == epoch && blockIdx.x == 0)) atomicAdd(count, 1u);
		uint64_t t0 = 0;
		for (uint32_t it = 0;; ++it) {
			if (ld_volatile(count) >= target) break;
			if (*(volatile int *) err) { ok = 0; break; }
			if (it == 0) t0 = global_timer_ns();
			else if (it > kWaitLimitIters || global_timer_ns() - t0 > limit_ns) {
				atomicExch(err, 6 /* BFS_ETIMEOUT */);
				ok = 0;
				break;
			}
			if (it > 16) __nanosleep(it < 256 ? 32 : 128);
		}
		__threadfence();
		if (*(volatile int *) err) ok = 0;
		s_sync_ok = ok;
	}
	__syncthreads();
	return s_sync_ok != 0;
}

// ---- shared-memory barriers and 1-D bulk copies (TMA) ---------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
	return (uint32_t) __cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
	asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}"
			::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
	asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
			"selp.u32 %0, 1, 0, p;\n\t}"
			: "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
	return ok != 0;
}
// The same test with a suspend-time hint: the thread sleeps until the phase
// completes or `hint_ns` passes, instead of spinning and taking issue slots
// from the warps that do the work.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t *bar, uint32_t parity, uint32_t hint_ns) {
	uint32_t ok;
	asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
			"selp.u32 %0, 1, 0, p;\n\t}"
			: "=r"(ok) : "r"(smem_addr(bar)), "r"(parity), "r"(hint_ns) : "memory");
	return ok != 0;
}
// Waits for the phase with the given parity; gives up (returning false and
// recording BFS_ETIMEOUT) after the wait limit.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int *err, uint32_t hint_ns = 1000) {
	if (mbar_try_wait(bar, parity)) return true;
	uint64_t t0 = global_timer_ns();
	for (uint32_t it = 0; it < kWaitLimitIters; ++it) {
		if (mbar_try_wait_sleep(bar, parity, hint_ns)) return true;
		if (global_timer_ns() - t0 > kWaitLimitNs) break;
	}
	atomicExch(err, 6 /* BFS_ETIMEOUT */);
	return false;
}
// Global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
			::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void fence_proxy_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// Warp-wide inclusive scan of a 32-bit value.
__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x) {
	const unsigned lane = lane_id();
#pragma unroll
	for (int d = 1; d < 32; d <<= 1) {
		uint32_t y = __shfl_up_sync(kFull, x, d);
		if (lane >= (unsigned) d) x += y;
	}
	return x;
}

template <class T> __device__ __forceinline__ T warp_sum(T x) {
#pragma unroll
	for (int d = 16; d > 0; d >>= 1) x += __shfl_xor_sync(kFull, x, d);
	return x;
}

} // namespace bfsg
