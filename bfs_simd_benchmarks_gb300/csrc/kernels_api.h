// kernels_api.h -- host-side entry points of bfs_kernels.cu (internal).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/bfs_gb300.h"
#include "bfs_device.cuh"

namespace bfsg {

constexpr uint32_t kSentinelWord = 0xFFFFFFFFu;
constexpr uint32_t kUnvisitedWord = 0xFFFFFFFFu;
constexpr uint32_t kMaxSliceBatch = 16;   // frontier slices staged together by the bottom-up step
constexpr uint32_t kSliceBudgetWords = 8192;
// Bulk-copy pipeline of the bottom-up step: stages per CTA, packed words per
// stage and the shared-memory budget of the frontier slices of one stage.
constexpr uint32_t kTmaStages = 3;
constexpr uint32_t kTmaEdgeWords = 4096;
constexpr uint32_t kTmaSliceWords = 4096;

enum StepKind { kStepSeed = 0, kStepClear, kStepToDense, kStepToSparse, kStepExpand, kStepDense };

size_t dense_smem_bytes(const DevGraph &g, uint32_t batch);
int persistent_grid(const DevGraph &g, uint32_t batch, int num_sms, int *grid, size_t *smem);
// Clears the run state for the stepwise mode (the persistent kernel clears
// and seeds by itself).
int launch_init(const DevGraph &g, const RunCtx &r, cudaStream_t st, int num_sms);
int launch_persistent(const DevGraph &g, const RunCtx &r, const StepParams &p, uint32_t batch, int grid,
		size_t smem, cudaStream_t st);
int launch_step(int kind, const DevGraph &g, const RunCtx &r, const StepParams &p, uint32_t step,
		uint32_t batch, int grid, size_t smem, cudaStream_t st);
int kernel_threads();

} // namespace bfsg
