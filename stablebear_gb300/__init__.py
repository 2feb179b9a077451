"""stablebear_gb300 — GB300-native pairwise integration of piecewise
constant functions (PCFs).

A drop-in for stablebear's pairwise path: ``pdist`` / ``cdist`` (Lp distance
matrices, p >= 1), ``l2_kernel`` (L2 Gram matrices) and ``lp_distance``, with
the reference's ``DistanceMatrix`` / ``SymmetricMatrix`` result types and
storage order.  Computation runs in hand-written CUDA kernels for sm_103a
behind the C ABI declared in ``include/sbgpu.h``; there is no CPU fallback.
"""
from .pcf import Pcf, PcfArray, pcf32, pcf64, pcf32i, pcf64i, float32, float64, zeros
from .matrices import DistanceMatrix, SymmetricMatrix
from .comparison import allclose
from .rectangles import Rectangle, iterate_rectangles
from .distance import (
    pdist, cdist, l2_kernel, lp_distance,
    Distance_f32_f32, Distance_f64_f64, InnerProduct_f32_f32, InnerProduct_f64_f64,
)
from .system import (
    force_cpu, set_block_size, limit_cpus, limit_gpus, set_cuda_threshold, get_cuda_threshold,
    set_device_verbose, set_min_block_side, set_tuning, set_window_cap, get_window_cap, build_type, get_ngpus,
)
from .task import StoppableTask, EmptyTask
from .io import save, load
from .norms import lp_norm, Norms_f32_f32, Norms_f64_f64
from . import persistence

__all__ = [
    "Pcf", "PcfArray", "pcf32", "pcf64", "pcf32i", "pcf64i", "float32", "float64", "zeros",
    "DistanceMatrix", "SymmetricMatrix", "allclose", "Rectangle", "iterate_rectangles",
    "pdist", "cdist", "l2_kernel", "lp_distance",
    "Distance_f32_f32", "Distance_f64_f64", "InnerProduct_f32_f32", "InnerProduct_f64_f64",
    "force_cpu", "set_block_size", "limit_cpus", "limit_gpus", "set_cuda_threshold", "get_cuda_threshold",
    "set_device_verbose", "set_min_block_side", "set_tuning", "set_window_cap", "get_window_cap", "build_type",
    "get_ngpus", "StoppableTask", "EmptyTask", "save", "load", "lp_norm", "Norms_f32_f32", "Norms_f64_f64",
    "persistence",
]

__version__ = "0.1.0"
