"""vertexsurge_gb300 — GB300 (sm_103a) implementation of VertexSurge's
variable-length graph pattern matching hot path: bit-matrix multi-source BFS
expand, vertex-id hash join and multi-way intersection, behind a C ABI
(include/vertexsurge_gb300.h).  This package is the Python view of that ABI
plus the synthetic graph generators used by tests and benchmarks."""
from ._abi import (  # noqa: F401
    BitMatrix, Captured, DeviceGraph, ExpandPlan, FlatTable, Picker, RowBlock, VsError, check, expand, hash_join, init,
    expand_layers, join_count_row_blocks, kernel_launches, release_cached, layers_to_flat, lib, matrix_column_count, matrix_filter, matrix_row_or_sum, select_ids_in_range, semi_join,
    vertex_mask_any_neighbor,
    make_params, mintersect, DIR_BACKWARD, DIR_BOTH, DIR_FORWARD, KIND_COLMAIN, KIND_VARROW,
    PATH_ANY, PATH_FIND_SHORTEST, PATH_SHORTEST, STRAT_AUTO, STRAT_PULL, STRAT_PUSH, STRAT_SPARSE,
    T_I64, T_VID,
)
from . import graphgen  # noqa: F401
