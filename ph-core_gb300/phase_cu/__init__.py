"""phase_cu -- host side of the GB300 device backend for Phase n-dimensional arrays.

`CuNArray` implements the MultiIndexable / MultiWritable surface of the
reference's NArray (in-phase/ph-core) on device memory; every bulk operation is
one call into libphcuda.so (hand-written sm_103a CUDA kernels).  There is no
CPU fallback: importing works without a GPU, but the first device operation
raises when the library or the GPU is missing.
"""
from . import _abi
from .errors import ArgumentError, DeviceError, DimensionError, DivisionByZeroError, EmptyError, ShapeError
from .narray import (Bool, CuMutableView, CuNArray, CuProcView, CuView, Float32, Float64, Int32, Int64,
                     check_errors, compile_program, config, init, result_dtype, scalar_dtype, sync)
from .region import (IndexRegion, R, canonicalize_index, canonicalize_range, compatible_shapes, get_size,
                     infer_range, shape_to_size)

__all__ = [
    "ArgumentError", "Bool", "CuMutableView", "CuNArray", "CuProcView", "CuView", "DeviceError", "DimensionError",
    "DivisionByZeroError", "EmptyError", "Float32", "Float64", "IndexRegion", "Int32", "Int64", "R", "ShapeError",
    "canonicalize_index", "canonicalize_range", "check_errors", "compatible_shapes", "compile_program", "config",
    "get_size", "infer_range", "init", "result_dtype", "scalar_dtype", "shape_to_size", "sync",
]
