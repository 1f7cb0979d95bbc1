"""GB300-native geodesic tracer: the drop-in for Singularity's CUDA offline backend.

The compute path is the CUDA library ``_build/libsgx.so`` (kernels for
sm_103a behind the C ABI of include/sgx.h); this package is its Python host
mirror.  Build with ``singularity_gb300.build.build_library()``.
"""

from . import _native, workloads
from .backend import (Batch, CameraState, CudaBackend, ImageData, MetricType, RenderConfig, Renderer, Scene,
                      SceneConfig, SceneLoadResult, SceneLoadStatus, SgxError, build_orbital_camera,
                      default_opts, kerr_isco_prograde, load_scene_config_from_file,
                      load_scene_config_from_string, pack_uniforms, autotune, carter_drift)

__all__ = [
    "Batch", "autotune", "workloads", "CameraState", "CudaBackend", "ImageData", "MetricType", "RenderConfig", "Renderer", "Scene",
    "SceneConfig", "SceneLoadResult", "SceneLoadStatus", "SgxError", "build_orbital_camera", "default_opts",
    "kerr_isco_prograde", "load_scene_config_from_file", "load_scene_config_from_string", "pack_uniforms",
    "carter_drift", "_native",
]
