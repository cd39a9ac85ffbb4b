"""Run the reference's own CUDA kernel (test infrastructure).

TEST INFRASTRUCTURE ONLY (see oracle/sh.py).

ThreePhotons.jl's GPU path (src/cuda.jl:74-108) loads src/cuda_kernel.ptx, runs
``calculate_coefficient_matrix`` (src/cuda_kernel.cu:14-43) over the PAcombos
columns -- which scales the uploaded h_P in place into PA -- and then
cublasSgemm c3 = B * PA.  This module restates that host sequence: the unmodified
kernel, compiled to PTX by oracle/build.py, is loaded with the CUDA driver API
(cuModuleLoadData / cuLaunchKernel through ctypes, as CUDAdrv does), fed the
oracle's tables (float32 wignerlist and h_P, int32 indices and PAcombos, 1-based),
and the product runs as an FP32 matrix multiply (cuBLAS SGEMM through torch with
TF32 disabled).  Tables are checked against their bounds before the launch.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .basis import OracleBasis, combolist

HERE = os.path.dirname(os.path.abspath(__file__))
PTX = os.path.join(HERE, "_ref", "cuda_kernel.ptx")

_cuda = None


def _driver():
    global _cuda
    if _cuda is None:
        _cuda = ctypes.CDLL("libcuda.so.1")
        _cuda.cuModuleLoadData.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        _cuda.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        _cuda.cuLaunchKernel.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                         ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                         ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        _cuda.cuCtxSynchronize.argtypes = []
    return _cuda


def available() -> bool:
    return os.path.exists(PTX)


def c3_reference_cuda(b: OracleBasis, coeff: np.ndarray, B32: np.ndarray, P32: np.ndarray) -> np.ndarray:
    """c3 (2N^2 x klength, float32 as float64) from the reference's kernel + SGEMM."""
    import torch
    if not available():
        raise FileNotFoundError(f"{PTX} not built (oracle/build.py builds it where the reference sources exist)")
    torch.cuda.init()
    dev = torch.device("cuda")
    K, LMAX = b.K, b.LMAX
    numcoeff = LMAX * LMAX
    klength = b.klength
    basislen = b.basislen
    combos = combolist(b)                                                   # 9 x ncombo, 1-based
    ncombo = combos.shape[1]
    # bounds of every index the kernel will use
    assert combos[0:3].min() >= 1 and combos[0:3].max() <= K
    assert combos[3].min() >= 1 and combos[3].max() <= klength
    assert combos[7].min() >= 1 and (combos[7] + combos[8] - 1).max() <= basislen
    assert b.indices[0:3].min() >= 1 and b.indices[0:3].max() <= numcoeff
    assert P32.shape == (basislen, klength) and B32.shape == (2 * b.N * b.N, basislen)
    c = np.ascontiguousarray(np.asarray(coeff)[:K], dtype=np.complex64)     # numcoeff x K column-major
    d_coeff = torch.from_numpy(c.view(np.float32).reshape(-1)).to(dev)
    d_w = torch.from_numpy(b.wignerlist.astype(np.float32)).to(dev)
    d_idx = torch.from_numpy(np.ascontiguousarray(b.indices.T.astype(np.int32)).reshape(-1)).to(dev)
    d_comb = torch.from_numpy(np.ascontiguousarray(combos.T.astype(np.int32)).reshape(-1)).to(dev)
    d_PA = torch.from_numpy(np.asfortranarray(P32).T.copy().reshape(-1)).to(dev)  # column-major basislen x klength
    torch.cuda.synchronize()
    cu = _driver()
    mod = ctypes.c_void_p()
    ptx = open(PTX, "rb").read() + b"\0"
    r = cu.cuModuleLoadData(ctypes.byref(mod), ptx)
    if r != 0:
        raise RuntimeError(f"cuModuleLoadData failed: {r}")
    fn = ctypes.c_void_p()
    r = cu.cuModuleGetFunction(ctypes.byref(fn), mod, b"calculate_coefficient_matrix")
    if r != 0:
        raise RuntimeError(f"cuModuleGetFunction failed: {r}")
    args = [ctypes.c_void_p(d_coeff.data_ptr()), ctypes.c_int(numcoeff), ctypes.c_void_p(d_w.data_ptr()),
            ctypes.c_void_p(d_idx.data_ptr()), ctypes.c_int(basislen), ctypes.c_void_p(d_comb.data_ptr()),
            ctypes.c_int(ncombo), ctypes.c_void_p(d_PA.data_ptr()), ctypes.c_int(klength)]
    params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
    blocks = (ncombo + 1023) // 1024                                        # src/cuda.jl:82-83
    r = cu.cuLaunchKernel(fn, blocks, 1, 1, 1024, 1, 1, 0, None, params, None)
    if r != 0:
        raise RuntimeError(f"cuLaunchKernel failed: {r}")
    if cu.cuCtxSynchronize() != 0:
        raise RuntimeError("reference kernel failed")
    PA = d_PA.view(klength, basislen).t()                                   # basislen x klength
    Bm = torch.from_numpy(np.ascontiguousarray(B32)).to(dev)
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        c3 = Bm @ PA                                                        # SGEMM (src/cuda.jl:88)
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev
    return c3.double().cpu().numpy()


class RefCudaTimer:
    """The same host sequence as c3_reference_cuda with the module and the read-only
    tables (coefficient-independent: wignerlist, indices, PAcombos, B) kept on the device,
    for timing repeated calls.  Each call uploads h_P again (src/cuda.jl:80 sends it with
    every call because the kernel scales it in place into PA) or, with upload_hP=False,
    restores it from a device copy; then the kernel, the SGEMM and the D2H of c3."""

    def __init__(self, b: OracleBasis, B32: np.ndarray, P32: np.ndarray):
        import torch
        if not available():
            raise FileNotFoundError(f"{PTX} not built")
        torch.cuda.init()
        self.torch = torch
        self.dev = dev = torch.device("cuda")
        self.b = b
        K, LMAX = b.K, b.LMAX
        self.numcoeff = LMAX * LMAX
        combos = combolist(b)
        self.ncombo = combos.shape[1]
        assert combos[0:3].min() >= 1 and combos[0:3].max() <= K
        assert combos[3].min() >= 1 and combos[3].max() <= b.klength
        assert combos[7].min() >= 1 and (combos[7] + combos[8] - 1).max() <= b.basislen
        assert b.indices[0:3].min() >= 1 and b.indices[0:3].max() <= self.numcoeff
        assert P32.shape == (b.basislen, b.klength) and B32.shape == (2 * b.N * b.N, b.basislen)
        self.d_w = torch.from_numpy(b.wignerlist.astype(np.float32)).to(dev)
        self.d_idx = torch.from_numpy(np.ascontiguousarray(b.indices.T.astype(np.int32)).reshape(-1)).to(dev)
        self.d_comb = torch.from_numpy(np.ascontiguousarray(combos.T.astype(np.int32)).reshape(-1)).to(dev)
        self.h_P = np.asfortranarray(P32).T.copy().reshape(-1)               # column-major basislen x klength
        self.d_P0 = torch.from_numpy(self.h_P).to(dev)                      # pristine copy (resident variant)
        self.d_PA = torch.empty_like(self.d_P0)
        self.Bm = torch.from_numpy(np.ascontiguousarray(B32)).to(dev)
        cu = _driver()
        self.mod = ctypes.c_void_p()
        ptx = open(PTX, "rb").read() + b"\0"
        if cu.cuModuleLoadData(ctypes.byref(self.mod), ptx) != 0:
            raise RuntimeError("cuModuleLoadData failed")
        self.fn = ctypes.c_void_p()
        if cu.cuModuleGetFunction(ctypes.byref(self.fn), self.mod, b"calculate_coefficient_matrix") != 0:
            raise RuntimeError("cuModuleGetFunction failed")
        torch.cuda.synchronize()

    def c3(self, coeff: np.ndarray, upload_hP: bool = True) -> np.ndarray:
        torch, b = self.torch, self.b
        c = np.ascontiguousarray(np.asarray(coeff)[: b.K], dtype=np.complex64)
        d_coeff = torch.from_numpy(c.view(np.float32).reshape(-1)).to(self.dev)
        if upload_hP:
            self.d_PA.copy_(torch.from_numpy(self.h_P))
        else:
            self.d_PA.copy_(self.d_P0)
        torch.cuda.synchronize()
        args = [ctypes.c_void_p(d_coeff.data_ptr()), ctypes.c_int(self.numcoeff), ctypes.c_void_p(self.d_w.data_ptr()),
                ctypes.c_void_p(self.d_idx.data_ptr()), ctypes.c_int(b.basislen),
                ctypes.c_void_p(self.d_comb.data_ptr()), ctypes.c_int(self.ncombo),
                ctypes.c_void_p(self.d_PA.data_ptr()), ctypes.c_int(b.klength)]
        params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        cu = _driver()
        if cu.cuLaunchKernel(self.fn, (self.ncombo + 1023) // 1024, 1, 1, 1024, 1, 1, 0, None, params, None) != 0:
            raise RuntimeError("cuLaunchKernel failed")
        if cu.cuCtxSynchronize() != 0:
            raise RuntimeError("reference kernel failed")
        PA = self.d_PA.view(b.klength, b.basislen).t()
        prev = torch.backends.cuda.matmul.allow_tf32
        torch.backends.cuda.matmul.allow_tf32 = False
        try:
            c3 = self.Bm @ PA
        finally:
            torch.backends.cuda.matmul.allow_tf32 = prev
        return c3.cpu().numpy()
