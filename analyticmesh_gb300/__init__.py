"""GB300-native Analytic Marching: exact meshes of ReLU-MLP level sets.

Same Python surface as the reference (backend/__init__.py:1-7):
``AnalyticMarching``, ``MLP``, ``get_boundary``, ``simplify``,
``estimate_am_time``, ``save_model`` / ``load_model`` (ONNX) and ``lib``, the
drop-in for the compiled module ``cuam``.  The marching runs in CUDA kernels
for sm_103a behind the C ABI in include/analyticmesh_gb300.h.
"""
from . import cuam as lib
from .main import AnalyticMarching, DICHOTOMY_DICT, GRADIENT_DESCENT_DICT, SPHERE_TRACING_DICT, VOXEL_DICT
from .model import MLP
from .onnx_io import load_model, save_model
from .utils import estimate_am_time, get_boundary, simplify

__all__ = ["AnalyticMarching", "MLP", "save_model", "load_model", "get_boundary", "simplify", "estimate_am_time", "lib", "DICHOTOMY_DICT",
           "GRADIENT_DESCENT_DICT", "SPHERE_TRACING_DICT", "VOXEL_DICT"]
