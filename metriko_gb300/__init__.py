"""metriko_gb300: GB300-native smoothest 4-RoSy field, seamless integration and Integer-Grid-Map
rounding (the numerical core of komietty/metriko), as hand-written sm_103a CUDA behind a C ABI
(include/metriko_cuda.h) and header-only C++ host code (include/metriko/...).

Python here is plumbing for tests and benchmarks: `Context`, `pipeline`, `field_smoothest`.
"""
from ._lib import (Context, MetrikoError, PREC_FP64, PREC_MIXED, field_smoothest, lib,  # noqa: F401
                   field_inputs, field_solve, injective_barrier, local_injectivity, map_deviation, mesh_geometry, pipeline, seeded_init,
                   size_field_gradient, solve_opts, spmv_bench, topology_from_field, position_gradient,
                   face_geometry_backward, CsrMatrix, csr_smallest_eig, curl_matching, mesh_field_inputs,
                   field_smoothest_mesh, seam_paths, comb_turns, num_edges)
from . import meshgen  # noqa: F401
