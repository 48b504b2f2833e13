// cli_bfs.cpp -- the drop-in `bfs` program: the CLI of apps/bfs_simd/bfs.cpp
// main (:1122-1209) and apps/bfs_serial/bfs.cpp main (:1183-1275) on top of
// libbfs_gb300.so.
//
//   ./bfs <data> <tile_width> <stripe_length> [-w]
//
// Like the reference it needs at least three arguments (otherwise it prints
// the usage line to stdout and exits 1), ignores further arguments except
// "-w" (weighted "u v w" files, weights dropped), traverses from vertex 0,
// runs the traversal 10 times and prints one "<T> <seconds>" line per run and
// "Average: <T> <seconds>" after them (include/peg_util.h:51-58).  T is the
// number of CTAs of the persistent launch, the GPU counterpart of the
// reference's OpenMP thread count; seconds are the device time of the
// traversal, which covers the reference's timed region (bfs.cpp:806-913).
//
// Environment (no counterpart in the reference):
//   BFS_SOURCE=<v>      source vertex (default 0)
//   BFS_RUNS=<k>        runs per sweep (default 10, the reference's k_set)
//   BFS_PATH_DUMP=<dir> write <dir>/path<t>.txt after the last run, the
//                       reference's ONEDEBUG level dump (bfs.cpp:927-954);
//                       "1" means "path" like the reference
//   BFS_MODE=stepwise   one launch per step instead of the persistent kernel
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bfs_gb300.h"

int main(int argc, char **argv) {
	if (argc < 4) {
		std::printf("Usage: ./bfs <data> <tile_width> <stripe_length>\n");
		return 1;
	}
	const char *data = argv[1];
	uint32_t w = (uint32_t) std::strtoul(argv[2], nullptr, 0);
	uint32_t s = (uint32_t) std::strtoul(argv[3], nullptr, 0);
	uint32_t flags = 0;
	for (int i = 4; i < argc; ++i)
		if (std::strcmp(argv[i], "-w") == 0) flags |= BFS_LOAD_WEIGHTED;

	bfs_graph *g = nullptr;
	int st = bfs_graph_load(data, w, s, flags, &g);
	if (st == BFS_EIO) {
		std::fprintf(stderr, "cannot open file: %s_col-%u-coo-tiled-%u-0 (or its _untiled / _reorder files)\n", data, s, w);
		return 1;
	}
	if (st != BFS_OK) {
		std::fprintf(stderr, "Error: %s (%s, W=%u, S=%u)\n", bfs_status_string(st), data, w, s);
		return 1;
	}
	bfs_graph_info info;
	bfs_graph_get_info(g, &info);
	std::fprintf(stderr, "loaded %s: %u vertices, %llu edges%s\n", info.base, info.num_vertices,
			(unsigned long long) info.num_edges, info.used_reorder ? " (_reorder files)" : "");

	const char *env = std::getenv("BFS_SOURCE");
	uint32_t source = env ? (uint32_t) std::strtoul(env, nullptr, 0) : 0u;
	env = std::getenv("BFS_RUNS");
	int runs = env ? std::atoi(env) : 10;
	if (runs < 1) runs = 1;
	env = std::getenv("BFS_MODE");
	if (env && std::strcmp(env, "stepwise") == 0) {
		bfs_options o;
		bfs_get_options(g, &o);
		o.mode = BFS_MODE_STEPWISE;
		bfs_set_options(g, &o);
	}

	std::vector<int32_t> levels(info.num_vertices);
	double total = 0;
	unsigned label = 0;
	for (int k = 0; k < runs; ++k) {
		bfs_stats stats;
		st = bfs_run(g, source, levels.data(), nullptr, &stats);
		if (st != BFS_OK) {
			std::fprintf(stderr, "Error: %s\n", bfs_status_string(st));
			bfs_graph_free(g);
			return 1;
		}
		label = stats.grid_ctas;
		double sec = stats.device_ms / 1000.0;
		std::printf("%u %lf\n", label, sec);
		total += sec;
	}
	std::printf("Average: %u %f\n", label, total / runs);

	env = std::getenv("BFS_PATH_DUMP");
	if (env && *env) {
		std::string dir = std::strcmp(env, "1") == 0 ? "path" : env;
		st = bfs_write_level_dump(dir.c_str(), info.num_vertices, levels.data());
		if (st != BFS_OK) {
			std::fprintf(stderr, "Error: cannot open file %s/path0.txt.\n", dir.c_str());
			bfs_graph_free(g);
			return 1;
		}
	}
	bfs_graph_free(g);
	return 0;
}
