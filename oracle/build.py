"""Build the oracle's native parts (test infrastructure).

* oracle/_build/librefcpu.so -- the C + OpenMP restatement of the reference CPU path
  (oracle/refcpu.c), compiled with gcc for the host it runs on.
* oracle/_ref/cuda_kernel.ptx -- the reference's own CUDA kernel file
  (src/cuda_kernel.cu of ThreePhotons.jl), compiled unmodified to PTX, which is
  the artefact the reference itself loads (src/cuda.jl:14).  Built only where the
  reference sources are present; the PTX is architecture-neutral text, so a copy
  built here is what the GPU machine uses.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REF_SRC = os.environ.get("TP3_REFERENCE_DIR", "/root/reference")


def _newer(dst: str, *srcs: str) -> bool:
    return os.path.exists(dst) and all(os.path.getmtime(s) <= os.path.getmtime(dst) for s in srcs)


def build_refcpu() -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "refcpu.c")
    out = os.path.join(BUILD, "librefcpu.so")
    if not _newer(out, src):
        tmp = out + ".tmp"
        subprocess.run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", src, "-o", tmp, "-lm"], check=True)
        os.replace(tmp, out)
    return out


def build_ref_ptx() -> str | None:
    src = os.path.join(REF_SRC, "src", "cuda_kernel.cu")
    out = os.path.join(REF_OUT, "cuda_kernel.ptx")
    if not os.path.exists(src):
        return out if os.path.exists(out) else None
    os.makedirs(REF_OUT, exist_ok=True)
    if not _newer(out, src):
        subprocess.run(["nvcc", "-ptx", src, "-arch=compute_103a", "-O2", "-o", out], check=True)
    return out


def build() -> None:
    build_refcpu()
    build_ref_ptx()


if __name__ == "__main__":
    build()
