"""GB300-native occluder rasteriser with the API of rawrunprotected/rasterizer.

Rasterises baked 8-quad occluder batches into a hierarchical 16-bit depth
buffer and tests bounding boxes against it on one GPU (sm_103a), bit-exact
with the reference's AVX2 code.  The CUDA kernels and the C ABI live in
librasterizer_gb300.so (csrc/); this package is the Python mirror of the
reference's C++ classes over that ABI.
"""
from .api import (Context, Occluder, OccError, PreparedBatch, QuadDecomposition, Rasterizer,
                  SurfaceAreaHeuristic, bake_scene, build_coverage_table, coverage_table, execute_batch,
                  unpack_bits)

__all__ = ["Context", "Occluder", "OccError", "PreparedBatch", "QuadDecomposition", "Rasterizer",
           "SurfaceAreaHeuristic", "bake_scene", "build_coverage_table", "coverage_table", "execute_batch",
           "unpack_bits"]
