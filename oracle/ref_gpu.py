"""TEST INFRASTRUCTURE — the reference's own CUDA kernel on the GPU, as a checker.

`make -C oracle ref` compiles render/cuda/kernels/geodesic_kernel.cu (the
reference tree, where it is present) to PTX for compute_103a with the
reference's CUDA flags; the PTX travels with the tree to the GPU host, where
this module loads it through the CUDA driver API (the driver JIT-compiles it
for the GPU) and launches `singularity::singularity_geodesic_kernel(uint8_t*,
Uniforms)` the way CudaBackend::render_frame does (16x16 blocks, one thread
per pixel; render/cuda/cuda_backend.cu:140-152).  Only tests use it.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

HERE = Path(__file__).resolve().parent
PTX = HERE / "_ref" / "geodesic_kernel_compute103a.ptx"
# Itanium mangling of singularity::singularity_geodesic_kernel(unsigned char*, Uniforms)
KERNEL = b"_ZN11singularity27singularity_geodesic_kernelEPh8Uniforms"


def available() -> bool:
    return PTX.exists()


class RefKernel:
    """The reference kernel in the current CUDA context (initialise torch's first)."""

    def __init__(self, ptx: Path = PTX):
        self._cu = C.CDLL("libcuda.so.1")
        self._cu.cuModuleLoadData.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
        self._cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
        self._cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                            C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        self._cu.cuModuleUnload.argtypes = [C.c_void_p]
        data = Path(ptx).read_bytes() + b"\0"
        self._mod = C.c_void_p()
        self._check(self._cu.cuModuleLoadData(C.byref(self._mod), data), "cuModuleLoadData")
        self._fn = C.c_void_p()
        self._check(self._cu.cuModuleGetFunction(C.byref(self._fn), self._mod, KERNEL), "cuModuleGetFunction")

    @staticmethod
    def _check(rc: int, what: str) -> None:
        if rc != 0:
            raise RuntimeError(f"{what} failed: CUresult {rc}")

    def launch(self, d_out: int, u, stream: int = 0) -> None:
        """out: device pointer to width*height RGBA8; u: the 160-byte uniform block (ctypes)."""
        out = C.c_void_p(d_out)
        args = (C.c_void_p * 2)(C.cast(C.byref(out), C.c_void_p), C.cast(C.byref(u), C.c_void_p))
        gx, gy = (u.width + 15) // 16, (u.height + 15) // 16
        self._check(self._cu.cuLaunchKernel(self._fn, gx, gy, 1, 16, 16, 1, 0, C.c_void_p(stream), args, None),
                    "cuLaunchKernel")

    def close(self) -> None:
        if self._mod:
            self._cu.cuModuleUnload(self._mod)
            self._mod = C.c_void_p()
