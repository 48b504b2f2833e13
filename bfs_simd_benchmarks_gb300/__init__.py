"""GB300-native GraphPhi BFS: the hybrid top-down / bottom-up BFS path of
apps/bfs_simd behind a C ABI (include/bfs_gb300.h), with its tiled input
formats and tools.  The compute path is hand-written CUDA for sm_103a in
csrc/; this package holds the ctypes mirror of that ABI.
"""
from ._native import BfsError, load as load_library  # noqa: F401
from .graph import (  # noqa: F401
    Graph,
    Server,
    autotune,
    tile_size_range,
    gen_rmat,
    gen_rmat_device,
    pick_sources,
    tool_column_major,
    tool_coo_tiling,
    tool_csr_tiling,
    tool_vertex_remap,
    write_edge_list,
    write_level_dump,
)

__all__ = [
    "BfsError", "Graph", "Server", "autotune", "tile_size_range", "gen_rmat", "gen_rmat_device", "load_library", "pick_sources", "tool_column_major",
    "tool_coo_tiling", "tool_csr_tiling", "tool_vertex_remap", "write_edge_list", "write_level_dump",
]
