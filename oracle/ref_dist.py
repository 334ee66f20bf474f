"""ORACLE — test infrastructure only: the reference's own distance kernel.

``distanceToInterface_k`` (src/fem/EuclideanDistance.cu:45-58), compiled
unchanged from the reference's source file by ``oracle/Makefile`` into
``oracle/_ref/EuclideanDistance.cubin`` (sm_103a, device code only), loaded
here with the CUDA driver API and launched the way the reference's
``EuclideanDistance::resetPhi`` launches it (EuclideanDistance.cu:90-118): one
thread per mesh node, 512 threads per block, ceil(n / 512) blocks, phi holding
the pre-reset values whose signs the kernel keeps.

Only tests/ and bench.py's baseline legs use this module, to check and to time
the library's distance reset against the reference's kernel; nothing in the
package imports it.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CUBIN = HERE / "_ref" / "EuclideanDistance.cubin"
THREADS_PER_BLOCK = 512            # EuclideanDistance.cu:9
# distanceToInterface_k(const float*, int, const float*, int, double*)
KERNEL = b"_Z21distanceToInterface_kPKfiS0_iPd"


class RefDistError(RuntimeError):
    pass


def available() -> bool:
    return CUBIN.exists()


class ReferenceDistanceKernel:
    """The reference's kernel on the current CUDA device (torch's context)."""

    def __init__(self):
        import torch
        if not CUBIN.exists():
            raise RefDistError(f"{CUBIN} is missing: build it with `make -C oracle ref` where the "
                               "reference's sources are present")
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current on this thread
        self._cu = C.CDLL("libcuda.so.1")
        self._check(self._cu.cuInit(0), "cuInit")
        self._mod = C.c_void_p()
        self._check(self._cu.cuModuleLoad(C.byref(self._mod), str(CUBIN).encode()),
                    "cuModuleLoad")
        self._fn = C.c_void_p()
        self._check(self._cu.cuModuleGetFunction(C.byref(self._fn), self._mod, KERNEL),
                    "cuModuleGetFunction")

    def _check(self, rc: int, what: str) -> None:
        if rc != 0:
            raise RefDistError(f"{what} failed with CUresult {rc}")

    def launch(self, d_meshp: int, n_meshp: int, d_ifp: int, n_ifp: int, d_phi: int,
               stream: int = 0) -> None:
        """One launch on device buffers: meshp float[3 n_meshp], ifp
        float[3 n_ifp], phi double[n_meshp] (in: pre-reset values, out: signed
        distances)."""
        if n_meshp <= 0:
            return
        grid = int(math.ceil(float(n_meshp) / THREADS_PER_BLOCK))
        args = [C.c_uint64(d_meshp), C.c_int(n_meshp), C.c_uint64(d_ifp), C.c_int(n_ifp),
                C.c_uint64(d_phi)]
        params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        self._check(self._cu.cuLaunchKernel(self._fn, grid, 1, 1, THREADS_PER_BLOCK, 1, 1, 0,
                                            C.c_void_p(stream), params, None),
                    "cuLaunchKernel")

    def reset_phi(self, meshp: np.ndarray, ifp: np.ndarray, phi_n: np.ndarray) -> np.ndarray:
        """EuclideanDistance::resetPhi with host arrays: returns the new phi."""
        import torch
        dev = torch.device("cuda")
        xyz = torch.from_numpy(np.ascontiguousarray(meshp, np.float32).reshape(-1)).to(dev)
        pts = np.ascontiguousarray(ifp, np.float32).reshape(-1)
        d_ifp = torch.from_numpy(pts if pts.size else np.zeros(3, np.float32)).to(dev)
        phi = torch.from_numpy(np.ascontiguousarray(phi_n, np.float64)).to(dev)
        n = phi.shape[0]
        torch.cuda.synchronize()
        self.launch(xyz.data_ptr(), n, d_ifp.data_ptr(), pts.size // 3, phi.data_ptr())
        torch.cuda.synchronize()
        return phi.cpu().numpy()

    def close(self) -> None:
        if getattr(self, "_mod", None):
            self._cu.cuModuleUnload(self._mod)
            self._mod = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass
