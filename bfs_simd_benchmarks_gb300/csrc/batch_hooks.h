// batch_hooks.h -- what the serving loop (server.cpp) uses of a graph handle
// beyond the public ABI.  Internal.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/bfs_gb300.h"

namespace bfsg {

// Allocates the graph's batch state for K words per vertex and `planes` level
// planes now (so that serving allocates nothing per query); *batch_bytes gets
// its size.
int batch_reserve(bfs_graph *g, uint32_t K, uint32_t planes, size_t *batch_bytes);
// bfs_run_batch with two extra events: the stream first waits for
// `wait_before`, and `between` is recorded after the traversal, before the
// output pass (either may be null).
int run_batch_ex(bfs_graph *g, const uint32_t *sources, uint32_t ns, uint8_t *levels, cudaStream_t st,
		cudaEvent_t wait_before, cudaEvent_t between);
size_t graph_device_bytes(const bfs_graph *g);
uint32_t graph_num_vertices(const bfs_graph *g);
int graph_device(const bfs_graph *g);
bool graph_on_device(const bfs_graph *g);

} // namespace bfsg
