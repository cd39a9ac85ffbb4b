"""Wigner-D rotations (src/spherical_harmonics.jl:572-603): the library's host
rotationMatrix against sympy's Wigner small-d (golden file) and the oracle, the Euler
convention against the sampled action of a rotation on functions, and the device
per-shell rotation against the oracle (GPU)."""
import json
import math
import os

import numpy as np
import pytest

import tp3
from oracle import sh

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "wigner_D.json")


def Rz(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])


def Ry(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def rodrigues(v):
    a = np.linalg.norm(v)
    if a == 0.0:
        return np.eye(3)
    u = v / a
    Kx = np.array([[0, -u[2], u[1]], [u[2], 0, -u[0]], [-u[1], u[0], 0]])
    return math.cos(a) * np.eye(3) + math.sin(a) * Kx + 2.0 * math.sin(0.5 * a) ** 2 * np.outer(u, u)


def test_library_wigner_D_matches_golden():
    for case in json.load(open(GOLDEN)):
        D = tp3.rotationMatrix(case["theta"], case["phi"], case["gamma"], case["l"])
        ref = np.asarray(case["re"]) + 1j * np.asarray(case["im"])
        np.testing.assert_allclose(D, ref, atol=2e-14, rtol=0)


def test_oracle_d_work_matches_golden():
    for case in json.load(open(GOLDEN)):
        if case["l"] > 7:
            continue
        D = sh.rotation_matrix(case["theta"], case["phi"], case["gamma"], case["l"])
        ref = np.asarray(case["re"]) + 1j * np.asarray(case["im"])
        np.testing.assert_allclose(D, ref, atol=1e-15, rtol=0)


@pytest.mark.parametrize("l", [1, 4, 12])
def test_wigner_D_is_unitary_and_a_representation(l):
    rng = np.random.default_rng(l)
    a1, a2 = rng.uniform(-3, 3, 3), rng.uniform(-3, 3, 3)
    D1 = tp3.rotationMatrix(abs(a1[0]), a1[1], a1[2], l)
    np.testing.assert_allclose(D1 @ D1.conj().T, np.eye(2 * l + 1), atol=1e-13)
    # rotationMatrix(theta, phi, gamma) is the action of R = Rz(phi) Ry(-theta) Rz(gamma) on functions
    R = Rz(a1[1]) @ Ry(-abs(a1[0])) @ Rz(a1[2])
    np.testing.assert_allclose(D1, sh.wigner_D_sampled(l, R), atol=1e-12)
    # homomorphism: D(R1 R2) = D(R1) D(R2)
    R2 = Rz(a2[1]) @ Ry(-abs(a2[0])) @ Rz(a2[2])
    D2 = tp3.rotationMatrix(abs(a2[0]), a2[1], a2[2], l)
    th, ph, ga = sh.axis_angle_euler(_axis_angle(R @ R2))
    np.testing.assert_allclose(tp3.rotationMatrix(th, ph, ga, l), D1 @ D2, atol=1e-12)


def _axis_angle(R):
    ang = math.acos(max(-1.0, min(1.0, (np.trace(R) - 1) / 2)))
    w = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    return w / np.linalg.norm(w) * ang


def test_axis_angle_euler_roundtrip():
    rng = np.random.default_rng(3)
    vs = [rng.normal(size=3) * s for s in (1e-9, 1e-3, 0.5, 2.0, 3.1)] + [
        np.array([0, 0, 0.4]), np.array([0.0, 0.0, -2.5]), np.array([math.pi, 0.0, 0.0]),
        np.array([0.0, -math.pi, 0.0]), np.array([1.0, 1.0, 0.0]) / math.sqrt(2) * math.pi]
    for v in vs:
        th, ph, ga = sh.axis_angle_euler(v)
        np.testing.assert_allclose(Rz(ph) @ Ry(-th) @ Rz(ga), rodrigues(v), atol=1e-13)


def test_rotate_structure_host_matches_oracle():
    rng = np.random.default_rng(5)
    LMAX, K = 9, 3
    coeff = rng.normal(size=(K, LMAX * LMAX)) + 1j * rng.normal(size=(K, LMAX * LMAX))
    vol = tp3.SphericalHarmonicsVolume(coeff, LMAX, K, 8.0)
    out = tp3.rotateStructure(vol, 0.9, -0.3, 1.7, K, range(0, LMAX))
    ref = sh.rotate_structure(coeff, 0.9, -0.3, 1.7, K, range(0, LMAX), LMAX)
    np.testing.assert_allclose(out.coeff, ref, atol=1e-13)


def _rotate_sampled(coeff, v, LMAX):
    """Oracle per-shell rotation: order l of shell k gets D(exp([v_k]x)) (function-sampled D)."""
    out = np.array(coeff, copy=True)
    for k in range(coeff.shape[0]):
        R = rodrigues(v[k])
        for l in range(LMAX):
            idx = [sh.seanindex(l, m, LMAX) - 1 for m in range(-l, l + 1)]
            out[k, idx] = sh.wigner_D_sampled(l, R) @ coeff[k, idx]
    return out


@pytest.mark.gpu
def test_rotate_shells_device_matches_oracle():
    import torch
    L, LMAX, N, K, n = 8, 25, 16, 5, 3
    rng = np.random.default_rng(11)
    coeff = rng.normal(size=(n, K, LMAX * LMAX)) + 1j * rng.normal(size=(n, K, LMAX * LMAX))
    v = rng.normal(size=(n, K, 3)) * np.array([0.1, 1.0, 2.5])[:, None, None]
    v[0, 0] = [0.0, 0.0, 0.7]          # theta = 0 branch
    v[0, 1] = [0.0, 0.0, 0.0]          # identity
    basis = tp3.calculate_basis(L, LMAX, N, K)
    dev = torch.device("cuda")
    d_in = torch.from_numpy(coeff.view(np.float64).copy()).to(dev)
    d_v = torch.from_numpy(v.copy()).to(dev)
    d_out = torch.empty_like(d_in)
    basis.rotate_shells_device(n, d_in.data_ptr(), d_v.data_ptr(), d_out.data_ptr())
    basis.sync()
    got = d_out.cpu().numpy().view(np.complex128).reshape(n, K, LMAX * LMAX)
    for i in range(n):
        np.testing.assert_allclose(got[i], _rotate_sampled(coeff[i], v[i], LMAX), atol=1e-11)
    # in place gives the same bits
    basis.rotate_shells_device(n, d_in.data_ptr(), d_v.data_ptr(), d_in.data_ptr())
    basis.sync()
    assert torch.equal(d_in, d_out)
    basis.close()


@pytest.mark.gpu
def test_common_rotation_leaves_energy_unchanged(config1, config1_hist):
    """KAT-2 on the device: one rotation applied to every shell leaves c3 and E unchanged."""
    import torch
    p = config1["params"]
    L, LMAX, N, K = p["L"], p["LMAX"], p["N"], p["K"]
    basis = tp3.calculate_basis(L, LMAX, N, K)
    basis.set_histogram(config1_hist)
    coeff = np.ascontiguousarray(config1["coeff"][:K])
    n = 4
    rng = np.random.default_rng(2)
    v = np.repeat(rng.normal(size=(n, 1, 3)), K, axis=1)
    dev = torch.device("cuda")
    d_in = torch.from_numpy(np.repeat(coeff[None], n, axis=0).view(np.float64).copy()).to(dev)
    d_v = torch.from_numpy(np.ascontiguousarray(v)).to(dev)
    d_rot = torch.empty_like(d_in)
    basis.rotate_shells_device(n, d_in.data_ptr(), d_v.data_ptr(), d_rot.data_ptr())
    E0 = torch.empty(n, dtype=torch.float64, device=dev)
    E1 = torch.empty(n, dtype=torch.float64, device=dev)
    basis.energy_batch_device(n, d_in.data_ptr(), E0.data_ptr())
    basis.energy_batch_device(n, d_rot.data_ptr(), E1.data_ptr())
    basis.sync()
    np.testing.assert_allclose(E1.cpu().numpy(), E0.cpu().numpy(), rtol=2e-7)
    basis.close()
