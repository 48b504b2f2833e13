"""Host-side mirror of the reference's BFS interface over the C ABI.

``Graph.load(data, tile_width, stripe_length)`` is graph_input
(apps/bfs_simd/bfs.cpp:968-1118); ``Graph.run(source)`` is graph_prepare
(apps/bfs_simd/bfs.cpp:753-963) returning the h_cost levels and the parents;
``write_level_dump`` is the ONEDEBUG dump (:927-954); the ``tool_*`` functions
are the CLIs of tools/csr_tiling, tools/coo_tiling, tools/column_major_tile and
tools/vertex_id_remap.  Errors raise ``BfsError`` with the library's status
code, where the reference calls exit(1).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class Graph:
    """A graph resident in HBM (CSR + packed column-major COO tiles)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle

    # ---- construction -------------------------------------------------
    @classmethod
    def load(cls, data: str, tile_width: int, stripe_length: int, weighted: bool = False,
             prefer_reorder: bool = False, host_only: bool = False) -> "Graph":
        lib = N.load()
        flags = (N.BFS_LOAD_WEIGHTED if weighted else 0) | (N.BFS_LOAD_PREFER_REORDER if prefer_reorder else 0)
        flags |= N.BFS_LOAD_HOST_ONLY if host_only else 0
        h = C.c_void_p()
        N.check(lib.bfs_graph_load(data.encode(), tile_width, stripe_length, flags, C.byref(h)),
                f"bfs_graph_load({data}, {tile_width}, {stripe_length})")
        return cls(h)

    @classmethod
    def from_edges(cls, num_vertices: int, src, dst, tile_width: int, stripe_length: int,
                   host_only: bool = False, device_build: bool = False, degree_order: bool = False) -> "Graph":
        """device_build: build the layout on the GPU (BFS_LOAD_DEVICE_BUILD);
        degree_order: lay it out on degree-ranked ids (BFS_LOAD_DEGREE_ORDER;
        every call still takes and returns the caller's ids)."""
        lib = N.load()
        s, d = _u32(src), _u32(dst)
        if s.shape != d.shape:
            raise ValueError("src and dst differ in length")
        h = C.c_void_p()
        flags = ((N.BFS_LOAD_HOST_ONLY if host_only else 0) | (N.BFS_LOAD_DEVICE_BUILD if device_build else 0)
                 | (N.BFS_LOAD_DEGREE_ORDER if degree_order else 0))
        N.check(lib.bfs_graph_from_edges(num_vertices, s.size, _ptr(s, C.c_uint32), _ptr(d, C.c_uint32),
                                         tile_width, stripe_length, flags, C.byref(h)), "bfs_graph_from_edges")
        return cls(h)

    @classmethod
    def from_device_edges(cls, num_vertices: int, src_ptr: int, dst_ptr: int, num_edges: int, tile_width: int,
                          stripe_length: int) -> "Graph":
        """A graph built on the GPU from an edge list already in device memory
        (uint32 src/dst device pointers; bfs_graph_from_edges with BFS_LOAD_DEVICE_BUILD)."""
        h = C.c_void_p()
        N.check(N.load().bfs_graph_from_edges(num_vertices, num_edges, C.cast(C.c_void_p(src_ptr), _u32p_type()),
                                              C.cast(C.c_void_p(dst_ptr), _u32p_type()), tile_width, stripe_length,
                                              N.BFS_LOAD_DEVICE_BUILD, C.byref(h)), "bfs_graph_from_edges")
        return cls(h)

    @classmethod
    def from_arrays(cls, num_vertices: int, degrees, csr_dst, heads, tails, tile_offsets,
                    tile_width: int, stripe_length: int, host_only: bool = False) -> "Graph":
        lib = N.load()
        deg, cd, hd, tl = _u32(degrees), _u32(csr_dst), _u32(heads), _u32(tails)
        off = None if tile_offsets is None else _u32(tile_offsets)
        h = C.c_void_p()
        flags = N.BFS_LOAD_HOST_ONLY if host_only else 0
        N.check(lib.bfs_graph_from_arrays(
            num_vertices, cd.size, _ptr(deg, C.c_uint32), _ptr(cd, C.c_uint32), _ptr(hd, C.c_uint32),
            _ptr(tl, C.c_uint32), None if off is None else _ptr(off, C.c_uint32), tile_width, stripe_length,
            flags, C.byref(h)), "bfs_graph_from_arrays")
        return cls(h)

    @classmethod
    def load_binary(cls, path: str, host_only: bool = False) -> "Graph":
        """A graph written by Graph.save (bfs_graph_load_binary)."""
        h = C.c_void_p()
        N.check(N.load().bfs_graph_load_binary(path.encode(), N.BFS_LOAD_HOST_ONLY if host_only else 0, C.byref(h)),
                f"bfs_graph_load_binary({path})")
        return cls(h)

    def save(self, path: str) -> None:
        N.check(N.load().bfs_graph_save(self._h, path.encode()), f"bfs_graph_save({path})")

    # ---- lifetime -----------------------------------------------------
    def close(self) -> None:
        if self._h:
            N.load().bfs_graph_free(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # ---- queries ------------------------------------------------------
    def info(self) -> dict:
        inf = N.GraphInfo()
        N.check(N.load().bfs_graph_get_info(self._h, C.byref(inf)), "bfs_graph_get_info")
        d = {k: getattr(inf, k) for k, _ in N.GraphInfo._fields_}
        d["base"] = inf.base.decode()
        return d

    @property
    def num_vertices(self) -> int:
        return self.info()["num_vertices"]

    def degrees(self) -> np.ndarray:
        n = self.num_vertices
        out = np.empty(n, dtype=np.uint32)
        N.check(N.load().bfs_graph_get_degrees(self._h, _ptr(out, C.c_uint32)), "bfs_graph_get_degrees")
        return out

    def options(self) -> dict:
        o = N.Options()
        N.check(N.load().bfs_get_options(self._h, C.byref(o)), "bfs_get_options")
        return {k: getattr(o, k) for k, _ in N.Options._fields_}

    def get_options(self) -> dict:
        o = N.Options()
        N.check(N.load().bfs_get_options(self._h, C.byref(o)), "bfs_get_options")
        return {k: getattr(o, k) for k, _ in N.Options._fields_}

    def set_options(self, **kw) -> None:
        o = N.Options()
        lib = N.load()
        N.check(lib.bfs_get_options(self._h, C.byref(o)), "bfs_get_options")
        names = {f for f, _ in N.Options._fields_}
        for k, v in kw.items():
            if k not in names:
                raise ValueError(f"unknown option {k!r}")
            if k == "mode" and isinstance(v, str):
                v = {"persistent": N.BFS_MODE_PERSISTENT, "stepwise": N.BFS_MODE_STEPWISE}[v]
            if k == "bottom_up" and isinstance(v, str):
                v = {"pull": N.BFS_BU_PULL, "stream": N.BFS_BU_STREAM}[v]
            setattr(o, k, int(v))
        N.check(lib.bfs_set_options(self._h, C.byref(o)), "bfs_set_options")

    # ---- traversal ----------------------------------------------------
    def run(self, source: int, parents: bool = True):
        """Levels (int32, -1 unreached), parents (uint32) and stats of one traversal."""
        n = self.num_vertices
        lev = np.empty(n, dtype=np.int32)
        par = np.empty(n, dtype=np.uint32) if parents else None
        st = N.Stats()
        N.check(N.load().bfs_run(self._h, int(source), _ptr(lev, C.c_int32),
                                 None if par is None else _ptr(par, C.c_uint32), C.byref(st)),
                f"bfs_run(source={source})")
        return lev, par, st.as_dict()

    def bfs_order(self, source: int = 0) -> np.ndarray:
        """tools/vertex_id_remap's relabelling from a GPU traversal: map[old] = new."""
        out = np.empty(self.num_vertices, dtype=np.uint32)
        N.check(N.load().bfs_graph_bfs_order(self._h, int(source), _ptr(out, C.c_uint32)), "bfs_graph_bfs_order")
        return out

    def run_device(self, source: int, levels_ptr: int, parents_ptr: int = 0, stream: int = 0) -> None:
        """Enqueues a traversal writing caller-owned device buffers on `stream`."""
        N.check(N.load().bfs_run_device(self._h, int(source), C.c_void_p(levels_ptr),
                                        C.c_void_p(parents_ptr) if parents_ptr else None,
                                        C.c_void_p(stream) if stream else None), "bfs_run_device")

    def last_stats(self) -> dict:
        st = N.Stats()
        N.check(N.load().bfs_last_stats(self._h, C.byref(st)), "bfs_last_stats")
        return st.as_dict()

    def run_batch_device(self, sources, levels_ptr: int, stream: int = 0, stats: bool = False):
        """Enqueues a batched traversal writing uint8 levels [len(sources)][N] at a device pointer."""
        src = _u32(sources)
        st = N.BatchStats() if stats else None
        N.check(N.load().bfs_run_batch(self._h, _ptr(src, C.c_uint32), src.size, C.c_void_p(levels_ptr),
                                       C.c_void_p(stream) if stream else None,
                                       C.byref(st) if st is not None else None), "bfs_run_batch")
        return st.as_dict() if st is not None else None

    def run_batch(self, sources):
        """Levels of every source at once: a torch uint8 CUDA tensor [len(sources), N]
        (255 = unreached) and the batch stats."""
        import torch
        src = _u32(sources)
        out = torch.empty((src.size, self.num_vertices), dtype=torch.uint8, device="cuda")
        stats = self.run_batch_device(src, out.data_ptr(), torch.cuda.current_stream().cuda_stream, stats=True)
        return out, stats

    def run_batch_sources_device(self, sources_ptr: int, num_sources: int, levels_ptr: int, stream: int = 0) -> None:
        """bfs_run_batch_device: sources already in device memory (uint32)."""
        N.check(N.load().bfs_run_batch_device(self._h, C.c_void_p(sources_ptr), num_sources, C.c_void_p(levels_ptr),
                                              C.c_void_p(stream) if stream else None), "bfs_run_batch_device")

    def batch_graph(self, sources_ptr: int, num_sources: int, levels_ptr: int) -> "BatchGraph":
        """A CUDA graph of one batched traversal over fixed device buffers."""
        h = C.c_void_p()
        N.check(N.load().bfs_batch_graph_create(self._h, C.c_void_p(sources_ptr), num_sources, C.c_void_p(levels_ptr),
                                                C.byref(h)), "bfs_batch_graph_create")
        return BatchGraph(h, self)

    def tune(self, sources, single: bool = True, batch: bool = False) -> dict:
        """bfs_tune_options: times candidate options on these sources, keeps the best."""
        src = _u32(sources)
        r = N.TuneResult()
        flags = (N.BFS_TUNE_SINGLE if single else 0) | (N.BFS_TUNE_BATCH if batch else 0)
        N.check(N.load().bfs_tune_options(self._h, _ptr(src, C.c_uint32), src.size, flags, C.byref(r)),
                "bfs_tune_options")
        return r.as_dict()

    def bc(self, source: int, paths: bool = True):
        """Betweenness dependencies of one source (bfs_bc_run): float32 [N]
        dependencies, uint32 [N] shortest-path counts (or None) and the stats."""
        n = self.num_vertices
        dep = np.empty(n, dtype=np.float32)
        sig = np.empty(n, dtype=np.uint32) if paths else None
        st = N.BcStats()
        N.check(N.load().bfs_bc_run(self._h, int(source), dep.ctypes.data_as(C.c_void_p),
                                    sig.ctypes.data_as(C.c_void_p) if paths else None, C.byref(st)), "bfs_bc_run")
        return dep, sig, st.as_dict()

    def bc_device(self, source: int, dependencies_ptr: int = 0, paths_ptr: int = 0, stream: int = 0) -> None:
        """bfs_bc_run_device: enqueued on `stream`, results into device buffers."""
        N.check(N.load().bfs_bc_run_device(self._h, int(source), C.c_void_p(dependencies_ptr) if dependencies_ptr else None,
                                           C.c_void_p(paths_ptr) if paths_ptr else None,
                                           C.c_void_p(stream) if stream else None), "bfs_bc_run_device")

    def bc_batch(self, sources, paths: bool = True):
        """Betweenness of up to 256 sources at once (bfs_bc_run_batch): float32
        [k, N] dependencies, uint32 [k, N] shortest-path counts (or None) and
        the stats."""
        src = _u32(sources)
        n = self.num_vertices
        dep = np.empty((src.size, n), dtype=np.float32)
        sig = np.empty((src.size, n), dtype=np.uint32) if paths else None
        st = N.BcStats()
        N.check(N.load().bfs_bc_run_batch(self._h, _ptr(src, C.c_uint32), src.size, dep.ctypes.data_as(C.c_void_p),
                                          sig.ctypes.data_as(C.c_void_p) if paths else None, C.byref(st)),
                "bfs_bc_run_batch")
        return dep, sig, st.as_dict()

    def bc_batch_device(self, sources, dependencies_ptr: int = 0, paths_ptr: int = 0, stream: int = 0) -> None:
        """bfs_bc_run_batch_device: enqueued on `stream`, [k, N] results into device buffers."""
        src = _u32(sources)
        N.check(N.load().bfs_bc_run_batch_device(self._h, _ptr(src, C.c_uint32), src.size,
                                                 C.c_void_p(dependencies_ptr) if dependencies_ptr else None,
                                                 C.c_void_p(paths_ptr) if paths_ptr else None,
                                                 C.c_void_p(stream) if stream else None), "bfs_bc_run_batch_device")

    def bc_stats(self) -> dict:
        st = N.BcStats()
        N.check(N.load().bfs_bc_last_stats(self._h, C.byref(st)), "bfs_bc_last_stats")
        return st.as_dict()

    def betweenness(self, sources):
        """Betweenness centrality over `sources` (bfs_bc_accumulate): float32 [N]
        sum over sources s != v of the dependencies of s on v, and the stats."""
        src = _u32(sources)
        out = np.empty(self.num_vertices, dtype=np.float32)
        st = N.BcStats()
        N.check(N.load().bfs_bc_accumulate(self._h, _ptr(src, C.c_uint32), src.size, out.ctypes.data_as(C.c_void_p),
                                           C.byref(st)), "bfs_bc_accumulate")
        return out, st.as_dict()

    def betweenness_device(self, sources, centrality_ptr: int, stream: int = 0) -> None:
        """bfs_bc_accumulate_device: adds into a device float32 [N] buffer."""
        src = _u32(sources)
        N.check(N.load().bfs_bc_accumulate_device(self._h, _ptr(src, C.c_uint32), src.size, C.c_void_p(centrality_ptr),
                                                  C.c_void_p(stream) if stream else None), "bfs_bc_accumulate_device")

    def last_batch_stats(self) -> dict:
        st = N.BatchStats()
        N.check(N.load().bfs_last_batch_stats(self._h, C.byref(st)), "bfs_last_batch_stats")
        return st.as_dict()


class BatchGraph:
    """An instantiated CUDA graph of one batched traversal (bfs_batch_graph_*)."""

    def __init__(self, handle: C.c_void_p, graph: Graph):
        self._h = handle
        self._graph = graph

    def launch(self, stream: int = 0) -> None:
        N.check(N.load().bfs_batch_graph_launch(self._h, C.c_void_p(stream) if stream else None),
                "bfs_batch_graph_launch")

    def close(self) -> None:
        if self._h:
            N.load().bfs_batch_graph_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The serving loop (bfs_server_*): resident graphs, queries coalesced per
    graph into batched traversals under a device-memory budget."""

    def __init__(self, budget_bytes: int | None = None, slot_bytes: int | None = None, max_batch: int | None = None,
                 num_slots: int | None = None, planes: int | None = None, max_pending: int | None = None):
        lib = N.load()
        o = N.ServerOptions()
        N.check(lib.bfs_server_options_default(C.byref(o)), "bfs_server_options_default")
        for k, v in dict(budget_bytes=budget_bytes, slot_bytes=slot_bytes, max_batch=max_batch,
                         num_slots=num_slots, planes=planes, max_pending=max_pending).items():
            if v is not None:
                setattr(o, k, int(v))
        h = C.c_void_p()
        N.check(lib.bfs_server_create(C.byref(o), C.byref(h)), "bfs_server_create")
        self._h = h
        self._graphs = []  # keep the graphs alive as long as the server

    def add_graph(self, g: Graph) -> int:
        gid = C.c_uint32()
        N.check(N.load().bfs_server_add_graph(self._h, g.handle, C.byref(gid)), "bfs_server_add_graph")
        self._graphs.append(g)
        return gid.value

    def submit(self, graph_id: int, source: int, dst_ptr: int = 0, kind: int = N.BFS_DST_NONE) -> int:
        t = C.c_uint64()
        N.check(N.load().bfs_server_submit(self._h, graph_id, int(source), C.c_void_p(dst_ptr) if dst_ptr else None,
                                           kind, C.byref(t)), "bfs_server_submit")
        return t.value

    def submit_host(self, graph_id: int, source: int, out: np.ndarray) -> int:
        """Queues a query whose uint8 levels land in `out` (host, N bytes; keep it alive until wait)."""
        assert out.dtype == np.uint8 and out.flags["C_CONTIGUOUS"]
        return self.submit(graph_id, source, out.ctypes.data, N.BFS_DST_HOST)

    def wait(self, ticket: int) -> dict:
        r = N.QueryResult()
        st = N.load().bfs_server_wait(self._h, ticket, C.byref(r))
        N.check(st, f"bfs_server_wait({ticket})")
        return r.as_dict()

    def drain(self) -> None:
        N.check(N.load().bfs_server_drain(self._h), "bfs_server_drain")

    def replay(self, graph_ids, sources, arrival_ns) -> None:
        g = _u32(graph_ids)
        s = _u32(sources)
        a = np.ascontiguousarray(arrival_ns, dtype=np.uint64)
        N.check(N.load().bfs_server_replay(self._h, g.size, _ptr(g, C.c_uint32), _ptr(s, C.c_uint32),
                                           a.ctypes.data_as(C.POINTER(C.c_uint64))), "bfs_server_replay")

    def stats(self) -> dict:
        st = N.ServerStats()
        N.check(N.load().bfs_server_get_stats(self._h, C.byref(st)), "bfs_server_get_stats")
        return st.as_dict()

    def reset_stats(self) -> None:
        N.check(N.load().bfs_server_reset_stats(self._h), "bfs_server_reset_stats")

    def close(self) -> None:
        if self._h:
            N.load().bfs_server_destroy(self._h)
            self._h = None
            self._graphs = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tile_size_range(num_vertices: int, num_edges: int) -> tuple[int, int]:
    """tools/tile-size-computer's (min_tile_size, max_tile_size)."""
    lo, hi = C.c_uint32(), C.c_uint32()
    N.check(N.load().bfs_tile_size_range(num_vertices, num_edges, C.byref(lo), C.byref(hi)), "bfs_tile_size_range")
    return lo.value, hi.value


def autotune(num_vertices: int, src, dst, sources, tile_widths=(512, 1024, 2048, 4096), stripe_lengths=(8, 16, 32),
             single: bool = True, batch: bool = False, cache_path: str | None = None, device_build: bool = False,
             layouts: bool = False) -> dict:
    """bfs_autotune: the best tile shape, layout and options of an edge list, by
    measurement.  tile_widths=None: the powers of two in tile_size_range(N, E);
    layouts: also try the degree-ordered layout (single-source tuning)."""
    s, d, so = _u32(src), _u32(dst), _u32(sources)
    w, sl = _u32(tile_widths if tile_widths is not None else []), _u32(stripe_lengths)
    r = N.TuneResult()
    flags = ((N.BFS_TUNE_SINGLE if single else 0) | (N.BFS_TUNE_BATCH if batch else 0)
             | (N.BFS_TUNE_DEVICE_BUILD if device_build else 0) | (N.BFS_TUNE_LAYOUTS if layouts else 0))
    N.check(N.load().bfs_autotune(num_vertices, s.size, _ptr(s, C.c_uint32), _ptr(d, C.c_uint32),
                                  _ptr(so, C.c_uint32), so.size, _ptr(w, C.c_uint32), w.size, _ptr(sl, C.c_uint32),
                                  sl.size, flags, cache_path.encode() if cache_path else None, C.byref(r)),
            "bfs_autotune")
    return r.as_dict()


# ---- tools (the reference's tools/ CLIs) ------------------------------
def tool_csr_tiling(edge_list: str, weighted: bool = False) -> None:
    N.check(N.load().bfs_tool_csr_tiling(edge_list.encode(), N.BFS_LOAD_WEIGHTED if weighted else 0),
            f"csr_tiling {edge_list}")


def tool_coo_tiling(data: str, min_w: int, max_w: int) -> None:
    N.check(N.load().bfs_tool_coo_tiling(data.encode(), min_w, max_w, 0), f"coo_tiling {data}")


def tool_column_major(data: str, w: int, min_s: int, max_s: int) -> None:
    N.check(N.load().bfs_tool_column_major(data.encode(), w, min_s, max_s, 0), f"column_major_tile {data}")


def tool_vertex_remap(data: str, device: bool = False) -> None:
    N.check(N.load().bfs_tool_vertex_remap(data.encode(), N.BFS_TOOL_DEVICE if device else 0),
            f"vertex_id_remap {data}")


def write_level_dump(directory: str, levels) -> None:
    lev = np.ascontiguousarray(levels, dtype=np.int32)
    N.check(N.load().bfs_write_level_dump(directory.encode(), lev.size, _ptr(lev, C.c_int32)),
            f"level dump {directory}")


def write_edge_list(path: str, num_vertices: int, src, dst) -> None:
    """The "N M" + 1-indexed "u v" input format of README.md:19-24."""
    s, d = _u32(src), _u32(dst)
    with open(path, "w") as f:
        f.write(f"{num_vertices} {s.size}\n")
        if s.size:
            np.savetxt(f, np.stack([s.astype(np.int64) + 1, d.astype(np.int64) + 1], axis=1), fmt="%d")


# ---- synthetic inputs ---------------------------------------------------
def gen_rmat(num_vertices: int, num_edges: int, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 1, dedup: bool = True, no_self_loops: bool = True, permute: bool = False):
    """Seeded R-MAT edge list (uint32 src, dst) with exactly num_edges edges."""
    p = N.RmatParams()
    p.num_vertices = num_vertices
    p.num_edges = num_edges
    p.a, p.b, p.c = a, b, c
    p.seed = seed
    p.flags = ((N.BFS_RMAT_DEDUP if dedup else 0) | (N.BFS_RMAT_NO_SELF_LOOPS if no_self_loops else 0)
               | (N.BFS_RMAT_PERMUTE if permute else 0))
    src = np.empty(num_edges, dtype=np.uint32)
    dst = np.empty(num_edges, dtype=np.uint32)
    N.check(N.load().bfs_gen_rmat(C.byref(p), _ptr(src, C.c_uint32), _ptr(dst, C.c_uint32), num_edges),
            "bfs_gen_rmat")
    return src, dst


def gen_rmat_device(num_vertices: int, num_edges: int, a: float = 0.57, b: float = 0.19, c: float = 0.19,
                    seed: int = 1, dedup: bool = True, no_self_loops: bool = True, permute: bool = False):
    """gen_rmat's edge list drawn on the current CUDA device: two torch uint32-
    valued int32 CUDA tensors (src, dst) holding exactly gen_rmat's arrays."""
    import torch
    p = N.RmatParams()
    p.num_vertices = num_vertices
    p.num_edges = num_edges
    p.a, p.b, p.c = a, b, c
    p.seed = seed
    p.flags = ((N.BFS_RMAT_DEDUP if dedup else 0) | (N.BFS_RMAT_NO_SELF_LOOPS if no_self_loops else 0)
               | (N.BFS_RMAT_PERMUTE if permute else 0))
    src = torch.empty(num_edges, dtype=torch.int32, device="cuda")
    dst = torch.empty(num_edges, dtype=torch.int32, device="cuda")
    N.check(N.load().bfs_gen_rmat_device(C.byref(p), C.c_void_p(src.data_ptr()), C.c_void_p(dst.data_ptr()),
                                         num_edges), "bfs_gen_rmat_device")
    return src, dst


def _u32p_type():
    return C.POINTER(C.c_uint32)


def pick_sources(degrees, count: int, seed: int) -> np.ndarray:
    """`count` seeded source vertices with out-degree > 0 (repeats allowed when few exist)."""
    deg = np.asarray(degrees)
    cand = np.flatnonzero(deg > 0)
    if cand.size == 0:
        raise ValueError("no vertex has an out-edge")
    rng = np.random.default_rng(seed)
    return cand[rng.integers(0, cand.size, size=count)].astype(np.uint32)
