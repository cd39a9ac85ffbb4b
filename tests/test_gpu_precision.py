"""Precision of every evaluation mode against the FP64 oracle at configurations 1
(L8 K8 N16 LMAX9), 2 (L18 K26 N32 LMAX25) and 4 (L24 K38 N32 LMAX25, the largest
expansion), over 1000 random common rotations each.

A rotation applied to every shell leaves c3 unchanged, so one FP64 oracle evaluation
(exact 3j basis in the reference's order, C + OpenMP triple products, FP64 l-triple
contraction; src/correlations.jl:87-193) is the exact answer for every rotated input,
and each rotated input is an independent sample of a mode's rounding error.

Bars, per mode (plain FP32, BF16 hi/lo x3, TF32 hi/lo x3) and every rotation:
  * c3 relative L1 against the FP64 oracle <= 1e-5 (the metric of tests/test_cuda.jl:15);
  * max |c3 - c3_64| / max |c3_64| <= 1e-5 and RMS(c3 - c3_64) / RMS(c3_64) <= 1e-5;
  * relative energy error against the FP64 Bayes energy <= 1e-6.
At configuration 4 every tensor-core coupling form that fits the shape is checked too
(on a subset of the rotations).  Configurations 1 and 2 also compare the unrotated c3
with the reference-form CPU restatement (f32 tables, f64 accumulation) to 1e-5; at
configuration 4 that form needs a 24.5 GB table and is skipped.

Run with -s to see one JSON line of measured errors per configuration."""
import json
import time

import numpy as np
import pytest

import tp3

pytestmark = pytest.mark.gpu

CONFIGS = {
    1: dict(L=8, LMAX=9, K=8, N=16, KMAX=8, rmax=8.0),
    2: dict(L=18, LMAX=25, K=26, N=32, KMAX=38, rmax=38.0),
    4: dict(L=24, LMAX=25, K=38, N=32, KMAX=38, rmax=38.0),
}
ROTATIONS = 1000
FORM_ROTATIONS = 16
BAR_C3, BAR_E = 1e-5, 1e-6


def _rotated_inputs(coeff, L, LMAX, count, seed):
    from oracle.sh import seanindex, wigner_D_sampled, random_rotation3
    rng = np.random.default_rng(seed)
    idx = {l: [seanindex(l, m, LMAX) - 1 for m in range(-l, l + 1)] for l in range(0, L + 1, 2)}
    out = np.empty((count,) + coeff.shape, dtype=np.complex128)
    for r in range(count):
        R = random_rotation3(rng)
        x = coeff.copy()
        for l in range(2, L + 1, 2):
            x[:, idx[l]] = coeff[:, idx[l]] @ wigner_D_sampled(l, R)
        out[r] = x
    return out


def _errors(basis, rot, ref_dev, E64, batch=8):
    """Per-rotation errors of the basis's current mode and coupling form."""
    import torch
    dev = ref_dev.device
    cmax = float(ref_dev.abs().max())
    crms = float(ref_dev.pow(2).mean().sqrt())
    cl1 = float(ref_dev.abs().sum())
    klength, G = ref_dev.shape
    d_c3 = torch.empty((batch, klength, G), dtype=torch.float32, device=dev)
    d_E = torch.empty(batch, dtype=torch.float64, device=dev)
    mx, rms, l1, ee = [], [], [], []
    for r0 in range(0, len(rot), batch):
        m = min(batch, len(rot) - r0)
        d_in = torch.from_numpy(np.ascontiguousarray(rot[r0:r0 + m]).view(np.float64)).to(dev)
        basis.c3_batch_device(m, d_in.data_ptr(), d_c3.data_ptr())
        basis.energy_batch_device(m, d_in.data_ptr(), d_E.data_ptr())
        basis.sync()
        for i in range(m):
            d = d_c3[i].double() - ref_dev
            mx.append(float(d.abs().max()) / cmax)
            rms.append(float(d.pow(2).mean().sqrt()) / crms)
            l1.append(float(d.abs().sum()) / cl1)
        ee += [abs(float(e) - E64) / abs(E64) for e in d_E[:m].cpu().numpy()]
    return {"c3_max_err_over_max": max(mx), "c3_rms_err_over_rms_max": max(rms),
            "c3_rms_err_over_rms_mean": float(np.mean(rms)), "c3_relL1_max": max(l1),
            "energy_rel_err_max": max(ee), "energy_rel_err_rms": float(np.sqrt(np.mean(np.square(ee))))}


def _check(res, what):
    assert res["c3_relL1_max"] <= BAR_C3, (what, res)
    assert res["c3_max_err_over_max"] <= BAR_C3, (what, res)
    assert res["c3_rms_err_over_rms_max"] <= BAR_C3, (what, res)
    assert res["energy_rel_err_max"] <= BAR_E, (what, res)


@pytest.mark.parametrize("cfg_id", [1, 2, 4])
def test_precision_over_common_rotations(cfg_id):
    import torch
    from oracle.basis import enumerate_basis, lt_form_F
    from oracle.c3 import energy_bayes
    from oracle.refcpu import triple_products_fast, RefCPU
    from tp3.structure import synthetic_molecule, intensity_coefficients, poisson_histogram, loadHistograms

    c = CONFIGS[cfg_id]
    L, LMAX, K, N = c["L"], c["LMAX"], c["K"], c["N"]
    t0 = time.time()
    coeff = intensity_coefficients(synthetic_molecule(327, seed=101), LMAX, c["KMAX"], c["rmax"])[:K]
    b = enumerate_basis(L, LMAX, N, K)
    c3_64 = lt_form_F(b) @ triple_products_fast(b, coeff).T          # [G, klength]
    hist = loadHistograms(poisson_histogram(c3_64, K, N, 1e9, seed=7), K)
    E64 = energy_bayes(c3_64, hist, K, N)
    out = {"config": cfg_id, **c, "rotations": ROTATIONS, "E64": E64, "oracle_seconds": time.time() - t0}
    c3r = None
    if cfg_id in (1, 2):
        c3r = RefCPU(L, LMAX, N, K).c3(coeff)
        out["refform_vs_fp64_relL1"] = float(np.abs(c3r - c3_64).sum() / np.abs(c3_64).sum())
        assert out["refform_vs_fp64_relL1"] < 1e-7
    rot = _rotated_inputs(coeff, L, LMAX, ROTATIONS, 2024 + cfg_id)
    ref_dev = torch.from_numpy(np.ascontiguousarray(c3_64.T)).cuda()   # [klength, G]
    basis = tp3.calculate_basis(L, LMAX, N, K)
    try:
        basis.set_histogram(hist)
        out["modes"] = {}
        for name, mode in (("plain_fp32", tp3.TP3_MODE_PLAIN_FP32), ("tc_bf16x3", tp3.TP3_MODE_TC_BF16X3),
                           ("tc_tf32x3", tp3.TP3_MODE_TC_TF32X3)):
            basis.set_mode(mode)
            res = _errors(basis, rot, ref_dev, E64)
            if c3r is not None:
                c3u = basis.c3_raw(coeff).astype(np.float64)
                res["c3_relL1_vs_refform_unrotated"] = float(np.abs(c3u - c3r).sum() / np.abs(c3r).sum())
                assert res["c3_relL1_vs_refform_unrotated"] <= BAR_C3, (name, res)
            _check(res, name)
            out["modes"][name] = res
        if cfg_id == 4:
            # every coupling form that fits the largest expansion
            out["forms"] = {}
            for name, mode in (("tc_bf16x3", tp3.TP3_MODE_TC_BF16X3), ("tc_tf32x3", tp3.TP3_MODE_TC_TF32X3)):
                basis.set_mode(mode)
                for form in range(9):
                    try:
                        basis.set_coupling(form)
                    except tp3.TP3Error:
                        continue  # this form does not fit the shape
                    res = _errors(basis, rot[:FORM_ROTATIONS], ref_dev, E64)
                    _check(res, (name, form))
                    out["forms"][f"{name}/form{form}"] = res
            assert len(out["forms"]) >= 2
    finally:
        basis.close()
    out["seconds"] = time.time() - t0
    print(json.dumps(out))
