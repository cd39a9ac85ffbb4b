"""Golden c3 from the reference's own CUDA kernel (needs a GPU).

    python tests/golden/make_refcuda_golden.py OUT.npz

Runs ThreePhotons.jl's src/cuda_kernel.cu (compiled unmodified to PTX) plus an FP32
SGEMM -- the reference GPU path, src/cuda.jl:74-108 -- on the committed config-1
coefficients and tables (tests/golden/config1.npz), and stores the resulting c3.  The
committed copy is tests/golden/config1_refcuda.npz.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main(out: str) -> None:
    from oracle.basis import enumerate_basis, reference_tables
    from oracle.refcuda import c3_reference_cuda
    d = np.load(os.path.join(HERE, "config1.npz"))
    p = json.loads(str(d["params"]))
    b = enumerate_basis(p["L"], p["LMAX"], p["N"], p["K"])
    B32, P32 = reference_tables(b)
    c3 = c3_reference_cuda(b, d["coeff"], B32, P32)
    np.savez_compressed(out, c3_refcuda=c3.astype(np.float32), params=json.dumps(p))
    rel = np.abs(c3 - d["c3_refform"]).sum() / np.abs(d["c3_refform"]).sum()
    print("reference CUDA kernel c3 vs oracle reference form: rel L1", rel)


if __name__ == "__main__":
    main(sys.argv[1])
