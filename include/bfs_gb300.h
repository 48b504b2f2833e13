/*
 * bfs_gb300.h -- C ABI of the GB300-native GraphPhi BFS path.
 *
 * One shared library (libbfs_gb300.so) behind plain pointers and sizes.  It
 * replaces the hot path of the reference's apps/bfs_simd/bfs.cpp (and the
 * scalar twin apps/bfs_serial/bfs.cpp): the file loader, the hybrid
 * top-down / bottom-up traversal and its level output, plus the preprocessing
 * tools that write the tiled input files.  Each entry point names the
 * reference interface it replaces.
 *
 * Conventions (all follow the reference):
 *   - vertex ids are uint32_t, 0-based in memory, 1-based in the text files;
 *   - levels are int32_t, -1 for unreached, 0 for the source (h_cost);
 *   - parents are uint32_t, 0xFFFFFFFF for unreached, the source is its own
 *     parent (h_graph_parents);
 *   - every call returns a status code (BFS_OK == 0).
 */
#ifndef BFS_GB300_H
#define BFS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
/* The reference exits with status 1 on a failed fopen
 * (apps/bfs_simd/bfs.cpp:988-992, :1032-1035); the CLI maps every non-zero
 * status below to that exit(1) with a message on stderr. */
enum bfs_status {
	BFS_OK = 0,
	BFS_EIO = 1,          /* a file is missing or cannot be read/written */
	BFS_EFORMAT = 2,      /* a file or array is truncated, garbled or inconsistent */
	BFS_ENOMEM = 3,       /* host or device allocation failed */
	BFS_EARG = 4,         /* invalid argument */
	BFS_EBUDGET = 5,      /* admission refused: over the device-memory budget */
	BFS_ETIMEOUT = 6,     /* a device-side wait hit its bound and returned */
	BFS_ECUDA = 7,        /* a CUDA runtime call failed */
	BFS_EUNSUPPORTED = 8, /* tile shape that cannot be packed; batched level above 254 */
	BFS_ENODEV = 9        /* no CUDA device is available */
};

/* Short text for a status code (static storage). */
const char *bfs_status_string(int status);

/* ---- graph handle ------------------------------------------------------ */
typedef struct bfs_graph bfs_graph;

#define BFS_LOAD_WEIGHTED 0x1u     /* files carry "u v w" lines (-w); weights are dropped */
#define BFS_LOAD_PREFER_REORDER 0x2u /* try <data>_reorder_* before <data>_* */
#define BFS_LOAD_HOST_ONLY 0x4u    /* parse and validate only; allocate nothing on the GPU */
#define BFS_LOAD_DEGREE_ORDER 0x20u /* bfs_graph_from_edges: lay the graph out on vertex ids ranked by
                                       out-degree (descending, ties by ascending id) -- the layout of
                                       tools/vertex_id_reorder_to_degrees, with this library's tie-break;
                                       every call still takes and returns the caller's ids (sources are
                                       mapped in, levels and parents gathered back on the device);
                                       single-source runs only (batches, betweenness, serving and
                                       bfs_graph_save answer BFS_EUNSUPPORTED) */
#define BFS_LOAD_DEVICE_BUILD 0x8u /* bfs_graph_from_edges: build CSR, in-edge lists and packed tiles on the
                                      GPU (edge order inside rows and tiles unspecified; results unchanged);
                                      src and dst may then be host or device memory */

/*
 * Loads a graph from the reference's tiled text files and uploads it to HBM.
 * Replaces graph_input (apps/bfs_simd/bfs.cpp:968-1118; apps/bfs_serial/bfs.cpp:762-910).
 *
 * Reads <base>_col-<S>-coo-tiled-<W>-{0..63,offsets} (column-major COO tiles,
 * tools/column_major_tile) and <base>_untiled-{0..63,nneibor} (CSR,
 * tools/csr_tiling), where <base> is `data` (the bfs_serial / README naming,
 * README.md:64-67) or, when those files are absent, `data`_reorder (the
 * bfs_simd naming, apps/bfs_simd/bfs.cpp:983).  BFS_LOAD_PREFER_REORDER
 * reverses that order.
 */
int bfs_graph_load(const char *data, uint32_t tile_width, uint32_t stripe_length,
		uint32_t flags, bfs_graph **out);

/*
 * Builds the same graph from an in-memory directed edge list (0-based, any
 * order, duplicates and self loops kept as given).  Equivalent to running
 * tools/csr_tiling, tools/coo_tiling and tools/column_major_tile on the list
 * and loading the result with bfs_graph_load.
 */
int bfs_graph_from_edges(uint32_t num_vertices, uint64_t num_edges, const uint32_t *src,
		const uint32_t *dst, uint32_t tile_width, uint32_t stripe_length, uint32_t flags,
		bfs_graph **out);

/*
 * Builds the graph from the arrays graph_input produces
 * (apps/bfs_simd/bfs.cpp:968-1118): CSR out-degrees (graph_degrees[N]) and
 * destinations (graph_edges[E]), the column-major COO edges
 * (graph_heads[E], graph_tails[E], 0-based) and tile_offsets[SIDE*SIDE].
 * tile_offsets may be NULL (derived from the edges).
 */
int bfs_graph_from_arrays(uint32_t num_vertices, uint64_t num_edges, const uint32_t *degrees,
		const uint32_t *csr_dst, const uint32_t *heads, const uint32_t *tails,
		const uint32_t *tile_offsets, uint32_t tile_width, uint32_t stripe_length,
		uint32_t flags, bfs_graph **out);

int bfs_graph_free(bfs_graph *g);

/* Binary graph files (no counterpart in the reference, whose only format is
 * text): bfs_graph_save writes the graph's device layout (CSR, in-edge lists,
 * packed column-major segments) with a versioned header; bfs_graph_load_binary
 * reads it back onto the current device without parsing or rebuilding
 * (BFS_LOAD_HOST_ONLY: header and degrees only).  A file from another version
 * or a truncated one gives BFS_EFORMAT. */
int bfs_graph_save(const bfs_graph *g, const char *path);
int bfs_graph_load_binary(const char *path, uint32_t flags, bfs_graph **out);

typedef struct bfs_graph_info {
	uint32_t num_vertices;     /* NNODES */
	uint32_t tile_width;       /* TILE_WIDTH */
	uint64_t num_edges;        /* NEDGES */
	uint32_t stripe_length;    /* ROW_STEP */
	uint32_t side_length;      /* SIDE_LENGTH = ceil(N / W) */
	uint64_t num_tiles;        /* SIDE_LENGTH^2 */
	uint32_t num_stripes;      /* ceil(SIDE / S) */
	uint32_t num_groups;       /* destination column groups of the packed tile stream */
	uint64_t packed_words;     /* 32-bit words of the packed column-major stream (edges + padding) */
	uint64_t device_bytes;     /* HBM held by the graph */
	uint32_t max_out_degree;
	uint32_t used_reorder;     /* 1 if the <data>_reorder files were loaded */
	char base[1024];           /* the file base that was loaded, "" for in-memory graphs */
} bfs_graph_info;

int bfs_graph_get_info(const bfs_graph *g, bfs_graph_info *info);

/* Out-degrees (graph_degrees) and CSR destinations copied to host memory. */
int bfs_graph_get_degrees(const bfs_graph *g, uint32_t *degrees);

/* ---- traversal options ------------------------------------------------- */
#define BFS_MODE_PERSISTENT 0u /* the whole traversal in one cooperative launch */
#define BFS_MODE_STEPWISE 1u   /* one launch per step, host-driven (profiling / plain form) */

typedef struct bfs_options {
	uint32_t mode;             /* BFS_MODE_* */
	uint32_t to_dense_ratio;   /* go dense when frontier + out_degree > E / to_dense_ratio
	                              (the reference's T_RATIO = 20, apps/bfs_simd/bfs.cpp:832,1171) */
	uint32_t to_sparse_ratio;  /* stay dense while frontier + out_degree > E / to_sparse_ratio
	                              (the reference uses the same ratio for both) */
	uint32_t warp_max_degree;  /* top-down: degree <= this -> warp-cooperative gather */
	uint32_t cta_max_degree;   /* top-down: degree <= this -> one CTA per vertex; above -> grid-strided */
	uint32_t bottom_up;        /* BFS_BU_PULL or BFS_BU_STREAM */
	uint32_t batch_planes;     /* bfs_run_batch: level planes (2..255); 0 = from batch_budget_mb, at most 32 */
	uint32_t batch_budget_mb;  /* bfs_run_batch: HBM budget of the level planes in MiB (default 40960) */
	uint32_t batch_single_max; /* bfs_run_batch: batches of at most this many sources run as back-to-back
	                              single-source traversals (default 4; 0 = always bit-sliced) */
	uint32_t batch_push_div;   /* bfs_run_batch: a level is pushed top-down while its frontier's out-edges
	                              < E / batch_push_div, pulled bottom-up after (default 16) */
	uint32_t bc_level_bytes;   /* bfs_bc_*: test neighbour levels in a byte array before fetching values
	                              (traversals of at most 254 levels): 0 = for graphs of at least 2^22
	                              vertices (default), 1 = always, 2 = never; results are identical */
	uint32_t wait_limit_us;    /* bound of every device-side wait of bfs_run / bfs_run_batch (grid barriers):
	                              past it the kernel gives up, returns and the run reports BFS_ETIMEOUT
	                              (0 = the default, 2 s) */
	uint32_t test_hold_barrier; /* TESTS ONLY: k > 0 makes CTA 0 skip its arrival at the k-th grid barrier of
	                              the next runs, so that the other CTAs' bounded waits run out (the failure
	                              path of the wait limit, exercised without a GPU fault); 0 = off */
	uint32_t switch_rule;      /* BFS_SWITCH_REFERENCE (default): the thresholds above; BFS_SWITCH_UNVISITED:
	                              go bottom-up when the frontier's out-edges * bu_alpha exceed the out-edges
	                              of the vertices not reached yet, back top-down when frontier * td_beta < N
	                              (Beamer's rule); levels are identical, only the step directions differ */
	uint32_t bu_alpha;         /* BFS_SWITCH_UNVISITED: alpha (default 14) */
	uint32_t td_beta;          /* BFS_SWITCH_UNVISITED: beta (default 24) */
	uint32_t ctas_per_sm;      /* CTAs per SM of the cooperative traversal grids: 0 = as many as fit (at most
	                              2), or 1 or 2 */
	uint32_t bc_batch;         /* bfs_bc_accumulate: 1 (default) = sources in groups of up to 256 through the
	                              batched betweenness kernel (bfs_bc_run_batch); 0 = one source at a time */
	uint32_t batch_output_tile; /* bfs_run_batch output pass: vertices per tile, 64 or 128; 0 (default) = 128
	                              from 2^24 vertices, else 64; the levels are identical */
} bfs_options;

#define BFS_SWITCH_REFERENCE 0u
#define BFS_SWITCH_UNVISITED 1u

/* Bottom-up step variants.  PULL: every unvisited destination of a column
 * group scans its in-edges (the column's tiles sorted by destination) and
 * stops at the first source in the frontier.  STREAM: the column group's
 * tiles of every active stripe are streamed into shared memory with bulk
 * copies and every edge is tested, the reference's dense step. */
#define BFS_BU_PULL 0u
#define BFS_BU_STREAM 1u

/* Fills the defaults (reference switch rule, persistent mode). */
int bfs_options_default(bfs_options *opt);
int bfs_set_options(bfs_graph *g, const bfs_options *opt);
int bfs_get_options(const bfs_graph *g, bfs_options *opt);

/* ---- single-source traversal ------------------------------------------- */
#define BFS_TRACE_MAX 256

typedef struct bfs_stats {
	uint32_t num_steps;        /* traversal steps run (the reference's loop iterations + 1) */
	uint32_t dense_steps;      /* steps run bottom-up over the column-major tiles */
	uint32_t reached;          /* vertices with level >= 0 */
	uint32_t max_level;
	uint64_t edges_traversed;  /* m(s): sum of out-degrees of reached vertices (TEPS numerator) */
	uint64_t td_edges;         /* CSR edges read by top-down steps */
	uint64_t td_vertices;      /* frontier vertices expanded top-down */
	uint64_t bu_words;         /* bottom-up: packed tile words streamed (STREAM) or in-edges read (PULL) */
	uint64_t bu_slices;        /* frontier slices staged by bottom-up steps */
	uint64_t bu_groups;        /* column groups visited by bottom-up steps */
	uint64_t bu_vertices;      /* destinations tested by PULL bottom-up steps */
	double device_ms;          /* device time of the traversal, initialisation included (CUDA events) */
	double kernel_ms;          /* device time of the traversal kernel(s) alone */
	int32_t status;            /* device-side status of the run (BFS_OK or BFS_ETIMEOUT) */
	uint32_t grid_ctas;        /* CTAs of the persistent launch */
	uint8_t trace[BFS_TRACE_MAX]; /* trace[i] = 1 if step i was dense (first BFS_TRACE_MAX steps) */
	/* Phase timers, the counterpart of the reference's dense_time, to_dense_time,
	 * sparse_time and to_sparse_time (apps/bfs_simd/bfs.cpp:733-751), taken on the
	 * device between grid barriers (persistent mode only; 0 otherwise). */
	double dense_ms, to_dense_ms, sparse_ms, to_sparse_ms;
	float step_ms[BFS_TRACE_MAX]; /* duration of each step, conversion included */
	/* from the start of each step to the first / the last CTA done with the
	 * step's work (the rest of step_ms is the grid barrier and the totals) */
	float step_work_min_ms[BFS_TRACE_MAX];
	float step_work_max_ms[BFS_TRACE_MAX];
	/* Bottom-up step profile: SM cycles summed over CTAs spent in group setup,
	 * segment lists, consumer wait, consumer work, producer wait and publish. */
	uint64_t bu_cycles[8];
} bfs_stats;

/*
 * One traversal from `source`, outputs to HOST memory (either may be NULL).
 * Replaces graph_prepare (apps/bfs_simd/bfs.cpp:753-963): the same first
 * top-down step, the same dense/sparse switch rule by default, the same
 * h_cost levels.  Synchronous.
 */
int bfs_run(bfs_graph *g, uint32_t source, int32_t *levels, uint32_t *parents, bfs_stats *stats);

/*
 * The same traversal with caller-owned DEVICE outputs (levels[N] int32,
 * parents[N] uint32 or NULL), enqueued on `stream` (a cudaStream_t, NULL for
 * the default stream).  Asynchronous: nothing is copied to the host.
 * bfs_last_stats() synchronises and returns the stats of the last run.
 */
int bfs_run_device(bfs_graph *g, uint32_t source, int32_t *levels, uint32_t *parents, void *stream);
int bfs_last_stats(bfs_graph *g, bfs_stats *stats);

/* ---- batched traversal (no counterpart in the reference) --------------- */
#define BFS_BATCH_MAX_SOURCES 4096
#define BFS_BATCH_TRACE_LEVELS 64

typedef struct bfs_batch_stats {
	uint32_t num_sources;
	uint32_t depth;            /* the deepest source's max level + 1 */
	uint32_t push_levels;      /* levels expanded top-down (the others pulled bottom-up) */
	int32_t status;            /* BFS_OK, BFS_ETIMEOUT, or BFS_EUNSUPPORTED (a level above 254) */
	uint64_t edges_traversed;  /* sum over the sources of the out-degrees of the vertices each reached */
	uint64_t words_gathered;   /* 64-bit frontier words read by the pull levels' gathers */
	uint32_t planes;           /* level planes held (levels kept before an early output pass) */
	uint32_t spills;           /* early output passes (traversal deeper than the planes) */
	uint32_t words_per_vertex; /* 64-bit words per vertex, ceil(num_sources / 64) */
	uint32_t grid_ctas;
	double device_ms;          /* the whole launch (CUDA events) */
	double levels_ms;          /* the levels alone (device clock) */
	uint64_t device_bytes;     /* HBM held by the batch state */
	float level_ms[BFS_BATCH_TRACE_LEVELS];          /* time of each of the first 64 levels */
	uint32_t level_frontier[BFS_BATCH_TRACE_LEVELS]; /* frontier vertices of each level */
	uint8_t level_push[BFS_BATCH_TRACE_LEVELS];      /* 1: the level was expanded top-down */
	float level_phase_ms[BFS_BATCH_TRACE_LEVELS][3]; /* pull: small destinations, chunks, finish;
	                                                    push: clear, expand, finish */
	double setup_ms;           /* clearing and seeding (device clock) */
	double output_ms;          /* the output pass (CUDA events) */
	uint32_t single_source_runs; /* > 0: the batch ran as that many single-source traversals
	                                (batch_single_max); the per-level fields are then empty */
	uint32_t reserved;
} bfs_batch_stats;

/*
 * Traverses from num_sources (1..BFS_BATCH_MAX_SOURCES) sources at once and
 * writes uint8 levels[num_sources][N] (caller-owned device memory, source-major,
 * 255 = unreached) on `stream`.  Row i equals bfs_run(g, sources[i])'s levels
 * (graph_prepare's h_cost, apps/bfs_simd/bfs.cpp:753-963) wherever those are
 * at most 254; a traversal with a level above 254 reports BFS_EUNSUPPORTED.
 * Sources may repeat.  `sources` is host memory.  With stats NULL the call
 * only enqueues work; bfs_last_batch_stats waits for it and reads them.  The
 * batch state -- about (planes + 1) * N * ceil(num_sources / 64) * 8 bytes,
 * planes from bfs_options.batch_planes / batch_budget_mb -- is allocated by
 * the first call that needs it and kept with the graph; calls on one graph
 * must not overlap on the GPU.
 */
int bfs_run_batch(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, uint8_t *levels, void *stream,
		bfs_batch_stats *stats);
int bfs_last_batch_stats(bfs_graph *g, bfs_batch_stats *stats);

/* bfs_run_batch with `sources` in device memory: it enqueues device work only
 * (always the bit-sliced kernel; sources are checked on the device, an
 * out-of-range one makes the batch report BFS_EARG), so once the graph's batch
 * state exists it allocates nothing and can be captured into a CUDA graph. */
int bfs_run_batch_device(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, uint8_t *levels, void *stream);

/* One batched traversal captured into an instantiated CUDA graph: the sources
 * at a fixed device address (their values are read at each launch) and the
 * levels at a fixed device address.  Launching it replaces the launch
 * sequence (control-block clear, the cooperative traversal, the output pass)
 * by one graph launch; bfs_last_batch_stats then reports it (output_ms 0). */
typedef struct bfs_batch_graph bfs_batch_graph;
int bfs_batch_graph_create(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, uint8_t *levels,
		bfs_batch_graph **out);
int bfs_batch_graph_launch(bfs_batch_graph *bg, void *stream);
int bfs_batch_graph_destroy(bfs_batch_graph *bg);

/* ---- autotuner (no counterpart in the reference; it replaces choosing W, S
 * by hand with tools/tile-size-computer and the T_RATIO constant) -------- */
#define BFS_TUNE_SINGLE 1u  /* tune the single-source options (variant, switch ratios, bucket bounds) */
#define BFS_TUNE_BATCH 2u   /* tune batch_push_div on one batch of all the sources */
#define BFS_TUNE_DEVICE_BUILD 4u  /* bfs_autotune: build each candidate layout on the GPU */
#define BFS_TUNE_LAYOUTS 8u  /* bfs_autotune (single-source): also try BFS_LOAD_DEGREE_ORDER per shape */
#define BFS_TUNE_MAX_TRIALS 256

typedef struct bfs_tune_trial {
	uint32_t tile_width, stripe_length;
	bfs_options options;
	double gteps;              /* single-source trials: sum m(s) / sum kernel time; batch trials: the batch's */
	uint32_t kind;             /* BFS_TUNE_SINGLE or BFS_TUNE_BATCH */
	uint32_t load_flags;       /* layout of the trial's graph (0 or BFS_LOAD_DEGREE_ORDER) */
} bfs_tune_trial;

typedef struct bfs_tune_result {
	uint32_t tile_width, stripe_length;   /* the best shape (bfs_autotune) */
	bfs_options options;                  /* the best options for it */
	double single_gteps;                  /* measured with them (0 if not tuned) */
	double batch_gteps;
	double default_single_gteps;          /* the defaults at the first shape tried, for comparison */
	double default_batch_gteps;
	uint32_t num_trials;
	uint32_t from_cache;                  /* 1: read from the cache file, nothing measured */
	uint32_t load_flags;                  /* the best layout (0 or BFS_LOAD_DEGREE_ORDER; bfs_autotune) */
	uint32_t reserved;
	bfs_tune_trial trials[BFS_TUNE_MAX_TRIALS];
} bfs_tune_result;

/* tools/tile-size-computer: the range of tile widths it recommends for N
 * vertices and E edges (its "min_tile_size: .., max_tile_size: .." line,
 * tools/tile-size-computer/tile-size-computer.cpp:21-56).  bfs_autotune with
 * no tile widths searches the powers of two in this range. */
int bfs_tile_size_range(uint32_t num_vertices, uint64_t num_edges, uint32_t *min_width, uint32_t *max_width);

/* Tunes the options of one resident graph on the given sources (coordinate
 * descent, every candidate timed on the device) and leaves the best set. */
int bfs_tune_options(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, uint32_t flags,
		bfs_tune_result *result);
/* Builds the graph of an edge list (bfs_graph_from_edges) at every tile width
 * x stripe length given, tunes each (bfs_tune_options) and reports the best.
 * With a cache file, a graph already tuned (same N, E and out-degree
 * signature, same flags) is answered from it, and a new result is appended. */
int bfs_autotune(uint32_t num_vertices, uint64_t num_edges, const uint32_t *src, const uint32_t *dst,
		const uint32_t *sources, uint32_t num_sources, const uint32_t *tile_widths, uint32_t num_widths,
		const uint32_t *stripe_lengths, uint32_t num_stripes, uint32_t flags, const char *cache_path,
		bfs_tune_result *result);

/* ---- serving loop (no counterpart in the reference) ---------------------
 * A server keeps several graphs resident in HBM and answers single-source
 * queries (graph, source) by coalescing the queries waiting on one graph into
 * one bfs_run_batch traversal.  Admission is by a device-memory budget: a
 * graph is admitted with its batch state (reserved up front) only if graphs +
 * batch states + result slots fit; a batch takes as many waiting queries as
 * its result slot holds.  Batches of different graphs are in flight at once
 * on their own streams (their traversals run one after another on the GPU;
 * output passes and result copies overlap the next traversal); queries that
 * arrive meanwhile join the next batch of their graph as soon as a slot is
 * free (continuous batching).  A query's levels are the same as bfs_run's for
 * that source (as uint8, 255 = unreached) whatever else is in the mix.  The
 * server starts its own threads; all entry points are thread-safe.  Graphs
 * stay owned by the caller and must outlive the server.
 */
typedef struct bfs_server bfs_server;

typedef struct bfs_server_options {
	uint64_t budget_bytes;  /* HBM admission budget: graphs + batch states + result slots (default 40 GiB) */
	uint64_t slot_bytes;    /* device result buffer of one batch (default 2 GiB): at most slot_bytes / N queries
	                           of an N-vertex graph share a traversal */
	uint32_t max_batch;     /* queries per traversal (1..BFS_BATCH_MAX_SOURCES, default 1024) */
	uint32_t num_slots;     /* batches in flight (1..16, default 3) */
	uint32_t planes;        /* level planes of each graph's batch state (2..255, default 8) */
	uint32_t max_pending;   /* waiting queries before submit answers BFS_EBUDGET (default 1 << 20) */
} bfs_server_options;

#define BFS_DST_NONE 0u   /* keep no levels (load generation) */
#define BFS_DST_HOST 1u   /* dst is host memory of N bytes */
#define BFS_DST_DEVICE 2u /* dst is device memory of N bytes */

typedef struct bfs_query_result {
	int32_t status;        /* BFS_OK or the traversal's error */
	uint32_t batch_size;   /* queries in the traversal that served this one */
	uint64_t batch_id;
	double latency_ms;     /* submit -> levels written (or the traversal done, BFS_DST_NONE) */
	double queue_ms;       /* submit -> its traversal was launched */
} bfs_query_result;

typedef struct bfs_server_stats {
	uint64_t submitted;
	uint64_t completed;
	uint64_t refused;          /* submits answered BFS_EBUDGET */
	uint64_t batches;
	uint64_t edges_traversed;  /* sum over completed queries of m(s) */
	double p50_ms, p99_ms, mean_ms, max_ms;  /* query latency since the last reset */
	double mean_batch;         /* queries per traversal */
	double device_ms;          /* sum of the traversals' device time */
	uint64_t device_bytes;     /* admitted: graphs + batch states + result slots */
	uint32_t graphs;
	uint32_t reserved;
} bfs_server_stats;

int bfs_server_options_default(bfs_server_options *opt);
int bfs_server_create(const bfs_server_options *opt, bfs_server **out);
/* Admits a resident graph (BFS_EBUDGET when it does not fit; the graph is then
 * left as it was apart from its batch options). */
int bfs_server_add_graph(bfs_server *s, bfs_graph *g, uint32_t *graph_id);
int bfs_server_submit(bfs_server *s, uint32_t graph_id, uint32_t source, void *dst, uint32_t dst_kind,
		uint64_t *ticket);
/* Waits for a query (each ticket is waited for once). */
int bfs_server_wait(bfs_server *s, uint64_t ticket, bfs_query_result *result);
/* Waits until every query submitted so far has completed. */
int bfs_server_drain(bfs_server *s);
/* Open-loop load: submits query i (graph_ids[i], sources[i], levels discarded)
 * arrival_ns[i] nanoseconds after the call starts (non-decreasing), then
 * drains.  Returns the first error, if any. */
int bfs_server_replay(bfs_server *s, uint32_t count, const uint32_t *graph_ids, const uint32_t *sources,
		const uint64_t *arrival_ns);
int bfs_server_get_stats(bfs_server *s, bfs_server_stats *stats);
int bfs_server_reset_stats(bfs_server *s);
int bfs_server_destroy(bfs_server *s);

/* ---- allocation-free traversal (no counterpart in the reference) -------- */
#define BFS_NOALLOC_MAX_VERTICES (1u << 20)

/*
 * Top-down BFS from `source` over a CSR the caller already holds in device
 * memory (row_offsets[num_vertices+1], columns[row_offsets[num_vertices]],
 * 0-based), writing int32 levels (-1 unreached) into the caller's device
 * buffer levels[num_vertices] on `stream` (a cudaStream_t, NULL for the
 * default stream).  If `status` (a device int) is not NULL it is set to
 * BFS_OK on the stream before the launch and raised to BFS_ETIMEOUT (a grid
 * barrier gave up) or BFS_EARG (a column id >= num_vertices, which is then
 * skipped) by the traversal.  The row offsets must be non-decreasing and end
 * inside the column array; they are not checked.  Asynchronous.
 *
 * This entry point allocates nothing, for callers that cannot call
 * cudaMalloc: plug-ins whose host framework reserves the device memory and
 * hands none out, or request paths that cannot take the device-wide
 * synchronisation and unbounded latency of cudaMalloc / cudaFree.  Its
 * scratch is a fixed file-scope device array of about 8.1 MB per device,
 * sized for at most BFS_NOALLOC_MAX_VERTICES vertices (more returns
 * BFS_EUNSUPPORTED), held until the process exits and shared by every call
 * on that device: calls that overlap on the GPU race, so serialise them.
 * The first call on a device does a one-time set-up (it looks up the
 * scratch array's device address); make that call before any stream capture.
 */
int bfs_run_noalloc(uint32_t num_vertices, const uint32_t *row_offsets, const uint32_t *columns,
		uint32_t source, int32_t *levels, int32_t *status, void *stream);

/* ---- level dump --------------------------------------------------------- */
/* Writes <dir>/path<t>.txt, t = 0..63, "<v>) cost:<level>\n", floor(N/64)
 * vertices per file, the last taking the rest: the ONEDEBUG dump of
 * apps/bfs_simd/bfs.cpp:927-954. */
int bfs_write_level_dump(const char *dir, uint32_t num_vertices, const int32_t *levels);

/* ---- preprocessing tools (the reference's tools/ CLIs) ------------------ */
/* tools/csr_tiling/page_rank.cpp main: <edge_list> -> <edge_list>_untiled-{0..63,nneibor}. */
int bfs_tool_csr_tiling(const char *edge_list, uint32_t flags);
/* tools/coo_tiling/page_rank.cpp main: <data>_untiled-* -> <data>_coo-tiled-<W>-*,
 * W from min_w to max_w doubling. */
int bfs_tool_coo_tiling(const char *data, uint32_t min_w, uint32_t max_w, uint32_t flags);
/* tools/column_major_tile/kcore.cpp main: <data>_coo-tiled-<W>-* ->
 * <data>_col-<S>-coo-tiled-<W>-*, S from min_s to max_s doubling. */
int bfs_tool_column_major(const char *data, uint32_t w, uint32_t min_s, uint32_t max_s,
		uint32_t flags);
/* tools/vertex_id_remap/bfs.cpp main: <data>_untiled-* -> <data>_reorder
 * (BFS-discovery relabelling from vertex 0).  flags BFS_TOOL_DEVICE: the BFS
 * runs on the GPU (bfs_graph_bfs_order); the files are the same. */
#define BFS_TOOL_DEVICE 0x10u
int bfs_tool_vertex_remap(const char *data, uint32_t flags);

/* The relabelling of tools/vertex_id_remap (bfs.cpp:465-491) from a GPU
 * traversal: vertex_map[old] = new, by BFS level from `source` and ascending
 * old id within a level, unreached vertices last in ascending old id. */
int bfs_graph_bfs_order(bfs_graph *g, uint32_t source, uint32_t *vertex_map);

/* ---- betweenness centrality --------------------------------------------- */
/* Replaces BC() of apps/betweennessCentrality_simd/bc.cpp:1717-2097 (which
 * reads a second, reverse-tiled file family; the in-edge lists of the loaded
 * graph serve as the reverse graph here).  For one source s it computes the
 * shortest-path counts num_paths[v] (unsigned 32-bit, wrapping like the
 * reference's unsigned adds) and the dependencies
 *   dependencies[v] = sigma(v) * sum over out-edges v -> w one level deeper of
 *                     (1 + dependencies[w]) / sigma(w),
 * in float through the reference's formulas: inverse = 1.0f / (float)(int)
 * num_paths (0 where num_paths is 0), sums of inverses pulled level by level
 * from the deepest, result (sum - inverse) / inverse.  Unreached vertices get
 * 0; the source gets the number of other vertices it reaches (the reference
 * computes it the same way).  Sums are taken in a fixed order: repeated runs
 * give identical bits.  Traversals deeper than 2^19 levels: BFS_EUNSUPPORTED. */
#define BFS_BC_TRACE_LEVELS 64
#define BFS_BC_BATCH_MAX_SOURCES 256 /* sources per bfs_bc_run_batch call */
typedef struct bfs_bc_stats {
	uint32_t num_sources;     /* dependency runs counted here */
	uint32_t depth;           /* deepest level (the largest over the runs) */
	uint32_t reached;         /* vertices reached from the (last) source */
	uint32_t status;          /* BFS_* status of the device run */
	uint64_t edges_reached;   /* sum of the out-degrees of reached vertices, over the runs */
	uint64_t edges_forward;   /* in-edges read by the path-count sweeps */
	uint64_t edges_reverse;   /* out-edges read by the dependency sweeps */
	float device_ms;          /* traversals + dependency launches, device events */
	float traversal_ms;       /* of which the single-source traversals */
	float sort_ms;            /* level sort, path counts, dependency sums: device timers */
	float paths_ms;
	float dependencies_ms;
	uint32_t grid_ctas;
	/* the (last) run, per level d < BFS_BC_TRACE_LEVELS: path-count and
	 * dependency times, vertices, and of those the ones whose in- or
	 * out-degree is above 1024 (reduced by whole CTAs) or above 32 (one warp
	 * each; the rest are taken 32 to a warp) */
	float level_paths_ms[BFS_BC_TRACE_LEVELS];
	float level_dependencies_ms[BFS_BC_TRACE_LEVELS];
	uint32_t level_vertices[BFS_BC_TRACE_LEVELS];
	uint32_t level_big[BFS_BC_TRACE_LEVELS];
	uint32_t level_medium[BFS_BC_TRACE_LEVELS];
	/* batched runs (bfs_bc_run_batch, bfs_bc_accumulate with bc_batch = 1) */
	uint32_t batched_sources;   /* sources run through the batched kernel */
	uint32_t fallback_sources;  /* sources run one at a time because their batch's traversal was deeper than
	                               the batch's level planes */
	uint64_t edges_matched_forward;  /* edges read by the path-count sweeps that serve at least one source */
	uint64_t edges_matched_reverse;  /* ... by the dependency sweeps */
	uint64_t pairs_forward;          /* (edge, source) pairs summed by the path-count sweeps */
	uint64_t pairs_reverse;          /* ... by the dependency sweeps */
	uint32_t source_reached[BFS_BC_BATCH_MAX_SOURCES];  /* the last batch: vertices reached from each of its
	                                                       sources */
} bfs_bc_stats;

/* dependencies[N] and num_paths[N] are HOST buffers (either may be NULL). */
int bfs_bc_run(bfs_graph *g, uint32_t source, float *dependencies, uint32_t *num_paths, bfs_bc_stats *stats);
/* The same enqueued on `stream` into DEVICE buffers (either may be NULL: the
 * graph's own buffers are used); no host synchronisation. */
int bfs_bc_run_device(bfs_graph *g, uint32_t source, float *dependencies, uint32_t *num_paths, void *stream);
/* Statistics of the last bfs_bc_* run (synchronises with it). */
int bfs_bc_last_stats(bfs_graph *g, bfs_bc_stats *stats);
/* Batched betweenness (no counterpart in the reference, whose BC() takes one
 * source per call): the dependencies and path counts of up to 256 sources from
 * one bit-sliced traversal (the bfs_run_batch kernel) and, for every 64 of
 * them, one pass over the graph per level and direction, every (vertex,
 * source) pair in 8 bytes of state.  Per source the values are bfs_bc_run's (path counts bit-exact;
 * dependencies the same formulas, float sums in another fixed order: repeated
 * calls give identical bits).  dependencies [num_sources][N] and num_paths
 * [num_sources][N] are HOST buffers (either may be NULL).  A batch whose
 * traversal is deeper than its level planes (bfs_options.batch_planes /
 * batch_budget_mb; or more than 254 levels) runs one source at a time
 * through bfs_bc_run's kernel instead (stats->fallback_sources). */
int bfs_bc_run_batch(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, float *dependencies,
		uint32_t *num_paths, bfs_bc_stats *stats);
/* The same enqueued on `stream` into DEVICE buffers [num_sources][N] (either
 * may be NULL); sources is a host array.  No fallback: a batch deeper than its
 * planes ends with status BFS_EUNSUPPORTED (bfs_bc_last_stats) and leaves the
 * buffers unwritten.  The batched betweenness state (2 x 256 bytes per vertex,
 * the level lists) and the batched traversal's state are kept with the graph:
 * calls on one graph must not overlap on the GPU. */
int bfs_bc_run_batch_device(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, float *dependencies,
		uint32_t *num_paths, void *stream);
/* Betweenness centrality over a set of sources: centrality[v] (HOST, N floats,
 * overwritten) = sum over the sources s != v of the dependencies of s on v,
 * added in source order; over all N sources it is the unnormalised directed
 * betweenness.  With bfs_options.bc_batch = 1 (default) the sources go through
 * the batched kernel 256 at a time. */
int bfs_bc_accumulate(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, float *centrality,
		bfs_bc_stats *stats);
/* The same into a DEVICE buffer that is added to (not cleared), enqueued on
 * `stream`; sources is a host array.  One source at a time (bfs_bc_run's
 * kernel), whatever bc_batch says: an enqueued call cannot fall back. */
int bfs_bc_accumulate_device(bfs_graph *g, const uint32_t *sources, uint32_t num_sources, float *centrality,
		void *stream);

/* ---- synthetic inputs (no counterpart in the reference) ------------------ */
#define BFS_RMAT_NO_SELF_LOOPS 0x1u
#define BFS_RMAT_DEDUP 0x2u
#define BFS_RMAT_PERMUTE 0x4u   /* random relabelling of the vertex ids */

typedef struct bfs_rmat_params {
	uint32_t num_vertices;   /* N, any value >= 1 (ids >= N are rejected and redrawn) */
	uint32_t flags;          /* BFS_RMAT_* */
	uint64_t num_edges;      /* exact E after the cleaning the flags ask for */
	double a, b, c;          /* quadrant probabilities, d = 1 - a - b - c */
	uint64_t seed;
} bfs_rmat_params;

/* Seeded, platform-independent R-MAT edge list into src/dst (capacity >= num_edges). */
int bfs_gen_rmat(const bfs_rmat_params *p, uint32_t *src, uint32_t *dst, uint64_t capacity);
/* The same edge list, element for element, drawn on the current CUDA device
 * into DEVICE memory src/dst (capacity >= num_edges; num_edges < 2^32).  It
 * allocates its own temporaries (with deduplication a hash table of about
 * 2 x 12 bytes per edge, rounded up to a power of two) and returns when the
 * list is written.  The bench's large synthetic graphs come from here (the
 * host generator takes over a minute for 1.47 G edges). */
int bfs_gen_rmat_device(const bfs_rmat_params *p, uint32_t *src, uint32_t *dst, uint64_t capacity);

/* Library version string. */
const char *bfs_version(void);

#ifdef __cplusplus
}
#endif
#endif /* BFS_GB300_H */
