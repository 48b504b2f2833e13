"""ctypes binding of libbfs_gb300.so (the C ABI declared in include/bfs_gb300.h).

The library is built in-tree by ``bfs_simd_benchmarks_gb300.build.build()``.
Loading fails loudly when it is missing: there is no CPU fallback for any
traversal entry point.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

BFS_OK = 0
BFS_EIO = 1
BFS_EFORMAT = 2
BFS_ENOMEM = 3
BFS_EARG = 4
BFS_EBUDGET = 5
BFS_ETIMEOUT = 6
BFS_ECUDA = 7
BFS_EUNSUPPORTED = 8
BFS_ENODEV = 9

BFS_LOAD_WEIGHTED = 0x1
BFS_LOAD_PREFER_REORDER = 0x2
BFS_LOAD_HOST_ONLY = 0x4
BFS_LOAD_DEVICE_BUILD = 0x8
BFS_LOAD_DEGREE_ORDER = 0x20
BFS_TOOL_DEVICE = 0x10

BFS_MODE_PERSISTENT = 0
BFS_MODE_STEPWISE = 1

BFS_BU_PULL = 0
BFS_BU_STREAM = 1

BFS_RMAT_NO_SELF_LOOPS = 0x1
BFS_RMAT_DEDUP = 0x2
BFS_RMAT_PERMUTE = 0x4

BFS_BATCH_TRACE_LEVELS = 64
BFS_TRACE_MAX = 256

_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)


class GraphInfo(C.Structure):
    _fields_ = [
        ("num_vertices", C.c_uint32),
        ("tile_width", C.c_uint32),
        ("num_edges", C.c_uint64),
        ("stripe_length", C.c_uint32),
        ("side_length", C.c_uint32),
        ("num_tiles", C.c_uint64),
        ("num_stripes", C.c_uint32),
        ("num_groups", C.c_uint32),
        ("packed_words", C.c_uint64),
        ("device_bytes", C.c_uint64),
        ("max_out_degree", C.c_uint32),
        ("used_reorder", C.c_uint32),
        ("base", C.c_char * 1024),
    ]


class Options(C.Structure):
    _fields_ = [
        ("mode", C.c_uint32),
        ("to_dense_ratio", C.c_uint32),
        ("to_sparse_ratio", C.c_uint32),
        ("warp_max_degree", C.c_uint32),
        ("cta_max_degree", C.c_uint32),
        ("bottom_up", C.c_uint32),
        ("batch_planes", C.c_uint32),
        ("batch_budget_mb", C.c_uint32),
        ("batch_single_max", C.c_uint32),
        ("batch_push_div", C.c_uint32),
        ("bc_level_bytes", C.c_uint32),
        ("wait_limit_us", C.c_uint32),
        ("test_hold_barrier", C.c_uint32),
        ("switch_rule", C.c_uint32),
        ("bu_alpha", C.c_uint32),
        ("td_beta", C.c_uint32),
        ("ctas_per_sm", C.c_uint32),
        ("bc_batch", C.c_uint32),
        ("batch_output_tile", C.c_uint32),
    ]


BFS_BC_TRACE_LEVELS = 64
BFS_BC_BATCH_MAX_SOURCES = 256


class BcStats(C.Structure):
    _fields_ = [
        ("num_sources", C.c_uint32),
        ("depth", C.c_uint32),
        ("reached", C.c_uint32),
        ("status", C.c_uint32),
        ("edges_reached", C.c_uint64),
        ("edges_forward", C.c_uint64),
        ("edges_reverse", C.c_uint64),
        ("device_ms", C.c_float),
        ("traversal_ms", C.c_float),
        ("sort_ms", C.c_float),
        ("paths_ms", C.c_float),
        ("dependencies_ms", C.c_float),
        ("grid_ctas", C.c_uint32),
        ("level_paths_ms", C.c_float * BFS_BC_TRACE_LEVELS),
        ("level_dependencies_ms", C.c_float * BFS_BC_TRACE_LEVELS),
        ("level_vertices", C.c_uint32 * BFS_BC_TRACE_LEVELS),
        ("level_big", C.c_uint32 * BFS_BC_TRACE_LEVELS),
        ("level_medium", C.c_uint32 * BFS_BC_TRACE_LEVELS),
        ("batched_sources", C.c_uint32),
        ("fallback_sources", C.c_uint32),
        ("edges_matched_forward", C.c_uint64),
        ("edges_matched_reverse", C.c_uint64),
        ("pairs_forward", C.c_uint64),
        ("pairs_reverse", C.c_uint64),
        ("source_reached", C.c_uint32 * BFS_BC_BATCH_MAX_SOURCES),
    ]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_
             if not k.startswith("level_") and k != "source_reached"}
        d["source_reached"] = list(self.source_reached[:min(self.num_sources, BFS_BC_BATCH_MAX_SOURCES)])
        k = min(self.depth + 1, BFS_BC_TRACE_LEVELS)
        for name in ("level_paths_ms", "level_dependencies_ms"):
            d[name] = [round(x, 4) for x in getattr(self, name)[:k]]
        d["level_vertices"] = list(self.level_vertices[:k])
        d["level_big"] = list(self.level_big[:k])
        d["level_medium"] = list(self.level_medium[:k])
        return d


class BatchStats(C.Structure):
    _fields_ = [
        ("num_sources", C.c_uint32),
        ("depth", C.c_uint32),
        ("push_levels", C.c_uint32),
        ("status", C.c_int32),
        ("edges_traversed", C.c_uint64),
        ("words_gathered", C.c_uint64),
        ("planes", C.c_uint32),
        ("spills", C.c_uint32),
        ("words_per_vertex", C.c_uint32),
        ("grid_ctas", C.c_uint32),
        ("device_ms", C.c_double),
        ("levels_ms", C.c_double),
        ("device_bytes", C.c_uint64),
        ("level_ms", C.c_float * BFS_BATCH_TRACE_LEVELS),
        ("level_frontier", C.c_uint32 * BFS_BATCH_TRACE_LEVELS),
        ("level_push", C.c_uint8 * BFS_BATCH_TRACE_LEVELS),
        ("level_phase_ms", (C.c_float * 3) * BFS_BATCH_TRACE_LEVELS),
        ("setup_ms", C.c_double),
        ("output_ms", C.c_double),
        ("single_source_runs", C.c_uint32),
        ("reserved", C.c_uint32),
    ]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith("level_") and k != "reserved"}
        k = min(self.depth, BFS_BATCH_TRACE_LEVELS)
        d["level_ms"] = [round(x, 4) for x in self.level_ms[:k]]
        d["level_frontier"] = list(self.level_frontier[:k])
        d["level_push"] = list(self.level_push[:k])
        d["level_phase_ms"] = [[round(x, 4) for x in self.level_phase_ms[i]] for i in range(k)]
        return d


class Stats(C.Structure):
    _fields_ = [
        ("num_steps", C.c_uint32),
        ("dense_steps", C.c_uint32),
        ("reached", C.c_uint32),
        ("max_level", C.c_uint32),
        ("edges_traversed", C.c_uint64),
        ("td_edges", C.c_uint64),
        ("td_vertices", C.c_uint64),
        ("bu_words", C.c_uint64),
        ("bu_slices", C.c_uint64),
        ("bu_groups", C.c_uint64),
        ("bu_vertices", C.c_uint64),
        ("device_ms", C.c_double),
        ("kernel_ms", C.c_double),
        ("status", C.c_int32),
        ("grid_ctas", C.c_uint32),
        ("trace", C.c_uint8 * BFS_TRACE_MAX),
        ("dense_ms", C.c_double),
        ("to_dense_ms", C.c_double),
        ("sparse_ms", C.c_double),
        ("to_sparse_ms", C.c_double),
        ("step_ms", C.c_float * BFS_TRACE_MAX),
        ("step_work_min_ms", C.c_float * BFS_TRACE_MAX),
        ("step_work_max_ms", C.c_float * BFS_TRACE_MAX),
        ("bu_cycles", C.c_uint64 * 8),
    ]

    def as_dict(self) -> dict:
        arrays = ("trace", "step_ms", "step_work_min_ms", "step_work_max_ms", "bu_cycles")
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in arrays}
        d["bu_cycles"] = list(self.bu_cycles[:6])
        k = min(self.num_steps, BFS_TRACE_MAX)
        d["trace"] = list(self.trace[:k])
        for name in ("step_ms", "step_work_min_ms", "step_work_max_ms"):
            d[name] = [round(x, 5) for x in getattr(self, name)[:k]]
        return d


BFS_TUNE_SINGLE, BFS_TUNE_BATCH, BFS_TUNE_MAX_TRIALS = 1, 2, 256
BFS_TUNE_DEVICE_BUILD, BFS_TUNE_LAYOUTS = 4, 8


class TuneTrial(C.Structure):
    _fields_ = [
        ("tile_width", C.c_uint32),
        ("stripe_length", C.c_uint32),
        ("options", Options),
        ("gteps", C.c_double),
        ("kind", C.c_uint32),
        ("load_flags", C.c_uint32),
    ]


class TuneResult(C.Structure):
    _fields_ = [
        ("tile_width", C.c_uint32),
        ("stripe_length", C.c_uint32),
        ("options", Options),
        ("single_gteps", C.c_double),
        ("batch_gteps", C.c_double),
        ("default_single_gteps", C.c_double),
        ("default_batch_gteps", C.c_double),
        ("num_trials", C.c_uint32),
        ("from_cache", C.c_uint32),
        ("load_flags", C.c_uint32),
        ("reserved", C.c_uint32),
        ("trials", TuneTrial * BFS_TUNE_MAX_TRIALS),
    ]

    def as_dict(self) -> dict:
        opt = lambda o: {k: getattr(o, k) for k, _ in Options._fields_}  # noqa: E731
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("options", "trials")}
        d["options"] = opt(self.options)
        d["trials"] = [{"tile_width": t.tile_width, "stripe_length": t.stripe_length, "gteps": t.gteps,
                        "kind": t.kind, "load_flags": t.load_flags, "options": opt(t.options)}
                       for t in self.trials[:self.num_trials]]
        return d


class ServerOptions(C.Structure):
    _fields_ = [
        ("budget_bytes", C.c_uint64),
        ("slot_bytes", C.c_uint64),
        ("max_batch", C.c_uint32),
        ("num_slots", C.c_uint32),
        ("planes", C.c_uint32),
        ("max_pending", C.c_uint32),
    ]


class QueryResult(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("batch_size", C.c_uint32),
        ("batch_id", C.c_uint64),
        ("latency_ms", C.c_double),
        ("queue_ms", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_uint64),
        ("completed", C.c_uint64),
        ("refused", C.c_uint64),
        ("batches", C.c_uint64),
        ("edges_traversed", C.c_uint64),
        ("p50_ms", C.c_double),
        ("p99_ms", C.c_double),
        ("mean_ms", C.c_double),
        ("max_ms", C.c_double),
        ("mean_batch", C.c_double),
        ("device_ms", C.c_double),
        ("device_bytes", C.c_uint64),
        ("graphs", C.c_uint32),
        ("reserved", C.c_uint32),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


BFS_DST_NONE, BFS_DST_HOST, BFS_DST_DEVICE = 0, 1, 2


class RmatParams(C.Structure):
    _fields_ = [
        ("num_vertices", C.c_uint32),
        ("flags", C.c_uint32),
        ("num_edges", C.c_uint64),
        ("a", C.c_double),
        ("b", C.c_double),
        ("c", C.c_double),
        ("seed", C.c_uint64),
    ]


# (name, restype, argtypes)
_SIGNATURES = [
    ("bfs_status_string", C.c_char_p, [C.c_int]),
    ("bfs_version", C.c_char_p, []),
    ("bfs_graph_load", C.c_int, [C.c_char_p, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_void_p)]),
    ("bfs_graph_from_edges", C.c_int,
     [C.c_uint32, C.c_uint64, _u32p, _u32p, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_void_p)]),
    ("bfs_graph_from_arrays", C.c_int,
     [C.c_uint32, C.c_uint64, _u32p, _u32p, _u32p, _u32p, _u32p, C.c_uint32, C.c_uint32, C.c_uint32,
      C.POINTER(C.c_void_p)]),
    ("bfs_graph_free", C.c_int, [C.c_void_p]),
    ("bfs_graph_save", C.c_int, [C.c_void_p, C.c_char_p]),
    ("bfs_graph_bfs_order", C.c_int, [C.c_void_p, C.c_uint32, _u32p]),
    ("bfs_graph_load_binary", C.c_int, [C.c_char_p, C.c_uint32, C.POINTER(C.c_void_p)]),
    ("bfs_graph_get_info", C.c_int, [C.c_void_p, C.POINTER(GraphInfo)]),
    ("bfs_graph_get_degrees", C.c_int, [C.c_void_p, _u32p]),
    ("bfs_options_default", C.c_int, [C.POINTER(Options)]),
    ("bfs_set_options", C.c_int, [C.c_void_p, C.POINTER(Options)]),
    ("bfs_get_options", C.c_int, [C.c_void_p, C.POINTER(Options)]),
    ("bfs_run", C.c_int, [C.c_void_p, C.c_uint32, _i32p, _u32p, C.POINTER(Stats)]),
    ("bfs_run_device", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("bfs_last_stats", C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    ("bfs_run_batch", C.c_int, [C.c_void_p, _u32p, C.c_uint32, C.c_void_p, C.c_void_p, C.POINTER(BatchStats)]),
    ("bfs_last_batch_stats", C.c_int, [C.c_void_p, C.POINTER(BatchStats)]),
    ("bfs_bc_run", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.POINTER(BcStats)]),
    ("bfs_bc_run_device", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("bfs_bc_last_stats", C.c_int, [C.c_void_p, C.POINTER(BcStats)]),
    ("bfs_bc_run_batch", C.c_int, [C.c_void_p, _u32p, C.c_uint32, C.c_void_p, C.c_void_p, C.POINTER(BcStats)]),
    ("bfs_bc_run_batch_device", C.c_int, [C.c_void_p, _u32p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("bfs_bc_accumulate", C.c_int, [C.c_void_p, _u32p, C.c_uint32, C.c_void_p, C.POINTER(BcStats)]),
    ("bfs_bc_accumulate_device", C.c_int, [C.c_void_p, _u32p, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("bfs_run_batch_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("bfs_batch_graph_create", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_void_p)]),
    ("bfs_batch_graph_launch", C.c_int, [C.c_void_p, C.c_void_p]),
    ("bfs_batch_graph_destroy", C.c_int, [C.c_void_p]),
    ("bfs_tile_size_range", C.c_int, [C.c_uint32, C.c_uint64, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    ("bfs_tune_options", C.c_int, [C.c_void_p, _u32p, C.c_uint32, C.c_uint32, C.POINTER(TuneResult)]),
    ("bfs_autotune", C.c_int, [C.c_uint32, C.c_uint64, _u32p, _u32p, _u32p, C.c_uint32, _u32p, C.c_uint32, _u32p,
                               C.c_uint32, C.c_uint32, C.c_char_p, C.POINTER(TuneResult)]),
    ("bfs_server_options_default", C.c_int, [C.POINTER(ServerOptions)]),
    ("bfs_server_create", C.c_int, [C.POINTER(ServerOptions), C.POINTER(C.c_void_p)]),
    ("bfs_server_add_graph", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint32)]),
    ("bfs_server_submit", C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32,
                                    C.POINTER(C.c_uint64)]),
    ("bfs_server_wait", C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(QueryResult)]),
    ("bfs_server_drain", C.c_int, [C.c_void_p]),
    ("bfs_server_replay", C.c_int, [C.c_void_p, C.c_uint32, _u32p, _u32p, C.POINTER(C.c_uint64)]),
    ("bfs_server_get_stats", C.c_int, [C.c_void_p, C.POINTER(ServerStats)]),
    ("bfs_server_reset_stats", C.c_int, [C.c_void_p]),
    ("bfs_server_destroy", C.c_int, [C.c_void_p]),
    ("bfs_run_noalloc", C.c_int, [C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("bfs_write_level_dump", C.c_int, [C.c_char_p, C.c_uint32, _i32p]),
    ("bfs_tool_csr_tiling", C.c_int, [C.c_char_p, C.c_uint32]),
    ("bfs_tool_coo_tiling", C.c_int, [C.c_char_p, C.c_uint32, C.c_uint32, C.c_uint32]),
    ("bfs_tool_column_major", C.c_int, [C.c_char_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]),
    ("bfs_tool_vertex_remap", C.c_int, [C.c_char_p, C.c_uint32]),
    ("bfs_gen_rmat", C.c_int, [C.POINTER(RmatParams), _u32p, _u32p, C.c_uint64]),
    ("bfs_gen_rmat_device", C.c_int, [C.POINTER(RmatParams), C.c_void_p, C.c_void_p, C.c_uint64]),
]

_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> C.CDLL:
    """Loads libbfs_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(
                f"libbfs_gb300.so is not built ({path}); run __graft_entry__.build() or "
                "python bfs_simd_benchmarks_gb300/build.py first")
        _build.build()
    lib = C.CDLL(path)
    for name, res, args in _SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_names() -> list[str]:
    return [name for name, _, _ in _SIGNATURES]


class BfsError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        lib = load()
        msg = lib.bfs_status_string(status).decode()
        super().__init__(f"{what}: {msg} (status {status})" if what else f"{msg} (status {status})")
        self.status = status


def check(status: int, what: str = "") -> None:
    if status != BFS_OK:
        raise BfsError(status, what)
