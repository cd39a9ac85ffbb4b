"""Throughput benchmark: c3 + Bayes proposal evaluations per second at L=18, K=26, N=32.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--batch B] [--mode auto|tuned|plain|tc|tf32]
    python bench.py --impl reference [--steps K] [--warmup W]
    python bench.py --workload ragged      # 64 chains x 16 candidates, K in 16..26, L in 12..18, own histograms
    python bench.py --workload learned     # learned vs plain annealer: time to the plain final energy
    python bench.py --no-ragged --no-learned --no-lambda   # the proposal line without the extra legs
    python bench.py --workload chains      # 64 chains x 16 candidates per CUDA-graph replay

--mode tuned (and auto) runs the evaluation-variant autotuner first and benchmarks its
choice; plain / tc / tf32 force the plain FP32, BF16 hi/lo x3 or TF32 hi/lo x3 path.

Workload (one "step" = one batch of B proposals scored end to end):
  * a seeded 327-atom synthetic molecule (C/N/O/S 60/20/18/2 %, uniform in a 13 A
    ball, >= 1.2 A apart) expanded to intensity SH coefficients at LMAX=25,
    KMAX=38, rmax=38 (first K=26 shells used);
  * a target histogram: the model c3 at L=18, K=26, N=32 scaled to 1e9 triplets,
    Poisson-sampled and normalised like loadHistograms;
  * B proposals, each the reference's annealing move (get_MC_step): for every even
    l in 2..18 one random SO(2l+1) rotation by N(0, sigma_l), sigma_l = (pi/4)(l-1),
    applied to all shells.
Synthetic data stands in for the reference's PDB / measured histograms (none are
benchmark datasets).  The L2 cache (129 MB) is flushed by a 512 MB write between
timed steps, outside the per-step event window.

The line also carries `ragged` (64 chains of mixed L and K, one ragged launch per graph
replay, with a spot check of three chains against contexts of their own shape),
`lambda` (the same workload at lambda = 2.5 through the tensor-core and plain FP32
paths) and `learned` (the learned-proposal experiment with its network-free drift
ablation).

Rank 0 prints one JSON line.  --gpus N > 1 runs N independent replicas (one per
GPU, launched by torchrun); the path has no collective (annealing chains and
proposals are independent), so scaling is weak.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "threephotons.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

L, LMAX, N, K = 18, 25, 32, 26
KMAX, RMAX = 38, 38.0
N_ATOMS, MOL_SEED, HIST_SEED, PROP_SEED = 327, 20240601, 7, 99
TRIPLETS = 1e9
METRIC = "c3+Bayes proposal evals/s at L18 K26 N32"
UNIT = "proposals/s"
MODE_NAMES = {0: "plain_fp32", 1: "tc_bf16x3", 2: "tc_tf32x3"}
COUPLING_NAMES = {0: "fused_512", 1: "split", 2: "fused_256x2", 3: "warp_local", 4: "warp_local_256x2",
                  5: "folded_8w", 6: "folded_7w", 7: "folded_13w", 8: "folded_14w_pairs"}
ANGULAR_NAMES = {0: "tile", 1: "persistent"}
ANGULAR_CODES = {v: k for k, v in ANGULAR_NAMES.items()}
DTYPES = {0: "fp32", 1: "bf16x3 (fp32 accumulate)", 2: "tf32x3 (fp32 accumulate)"}
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of each stage's kernel, measured
# with ncu on one 32-proposal launch of this workload and written as bytes per proposal plus
# a per-launch constant (each proposal's T is written and read once; the histogram and the
# tables are read once per launch), by (mode, coupling form).
STAGE_TRAFFIC = {
    ("tc_bf16x3", "folded_7w", "tile"): {"coupling": (154.2e6 / 32, 0.0), "angular": (230.2e6 / 32, 0.0),
                                 "source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one 32-proposal "
                                           "launch, scaled in proportion to the proposals "
                                           "(profiles/traffic_L18K26N32_b32_folded7w.md)"},
    ("tc_bf16x3", "folded_13w", "persistent"): {
        "coupling": (155.9e6 / 32, 0.0), "angular": (230.8e6 / 32, 0.0),
        "source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one 32-proposal launch of each stage, "
                  "scaled in proportion to the proposals (profiles/traffic_L18K26N32_b32_folded13w.md)"},
    ("tc_bf16x3", "folded_7w", "persistent"): {
        "coupling": (154.2e6 / 32, 0.0), "angular": (231.1e6 / 32, 0.0),
        "source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one 32-proposal launch of each stage, "
                  "scaled in proportion to the proposals (profiles/traffic_L18K26N32_b32_folded7w.md, "
                  "profiles/k_angular_tp_L18K26N32_b32.md)"},
}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float) -> float:
    """Max of a float over all ranks of the default process group (identity without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world_size: int, units_per_rank_step: int, steps: int, max_ms: float) -> float:
    """Units per second of the whole job: every rank processed units_per_rank_step per step,
    and the slowest rank's time bounds the job."""
    return world_size * units_per_rank_step * steps / (max_ms / 1e3)


def molecule_coefficients():
    from tp3.structure import synthetic_molecule, intensity_coefficients
    atoms = synthetic_molecule(N_ATOMS, seed=MOL_SEED)
    return intensity_coefficients(atoms, LMAX, KMAX, RMAX)


def random_rotation(dim, rng):
    """Haar SO(dim) via QR with sign fix and det > 0 (utilities.jl:165-176)."""
    while True:
        Q, R = np.linalg.qr(rng.normal(size=(dim, dim)))
        Q = Q * np.sign(np.diag(R))
        if np.linalg.det(Q) > 0:
            return Q


def random_rotation_step(dim, beta, rng):
    """C^-1 R(beta) C with a Haar C (utilities.jl:180-190)."""
    Rm = np.eye(dim)
    Rm[0, 0] = math.cos(beta); Rm[0, 1] = -math.sin(beta)
    Rm[1, 0] = math.sin(beta); Rm[1, 1] = math.cos(beta)
    C = random_rotation(dim, rng)
    return C.T @ Rm @ C


def proposals(base, n, seed):
    """n coefficient sets, each one get_MC_step of base (determination.jl:232-241)."""
    from tp3.api import Umat
    from tp3.structure import seanindex0
    rng = np.random.default_rng(seed)
    out = np.repeat(base[None, :K], n, axis=0).astype(np.complex128)
    for i in range(n):
        for l in range(2, L + 1, 2):
            sigma = (math.pi / 4) * (l - 1)
            U = Umat(l)
            rot = U.conj().T @ random_rotation_step(2 * l + 1, rng.normal() * sigma, rng) @ U
            idx = [seanindex0(l, m, LMAX) for m in range(-l, l + 1)]
            out[i][:, idx] = (rot @ base[:K][:, idx].T).T
    return out


def sample_clocks_start(path):
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        f = open(path, "w")
        p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                             stdout=f, stderr=subprocess.DEVNULL)
        return p, f
    except Exception:
        return None, None


def sample_clocks_stop(p, f, path, gpu_index):
    if p is None:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    p.terminate()
    try:
        p.wait(timeout=5)
    except Exception:
        p.kill()
    f.close()
    sm, smax, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in open(path):
        parts = [x.strip() for x in line.split(",")]
        if len(parts) < 9:
            continue
        try:
            if int(parts[0]) != gpu_index:
                continue
            sm.append(float(parts[1]))
            smax = float(parts[2])
        except ValueError:
            continue
        for nm, v in zip(names, parts[5:9]):
            if v.lower() == "active":
                reasons.add(nm)
    return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
            "samples": len(sm)}


def cpu_baseline_sample(base, hist, n_props=3):
    """Reference-form CPU path (oracle port) on this host: bounded sample."""
    from oracle.refcpu import RefCPU, threads
    t0 = time.time()
    ref = RefCPU(L, LMAX, N, K)
    setup = time.time() - t0
    props = proposals(base, n_props, PROP_SEED + 1)
    t0 = time.perf_counter()
    for c in props:
        ref.energy(c, hist)
    dt = time.perf_counter() - t0
    return {"value": n_props / dt, "unit": UNIT, "cores": threads(), "kind": "port",
            "sample": f"{n_props} proposal(s) of the L18 K26 N32 workload through the reference-form CPU path "
                      f"(f32 B/h_P tables, f64 PA and BLAS dgemm, f64 Bayes); {dt:.1f} s timed, "
                      f"{setup:.1f} s table build untimed"}


def build_histogram(basis, base):
    from tp3.structure import poisson_histogram, loadHistograms
    basis.set_mode(-1)
    c3 = basis.c3_raw(base).astype(np.float64)
    counts = poisson_histogram(c3, K, N, TRIPLETS, seed=HIST_SEED)
    return loadHistograms(counts, K)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from tp3.structure import poisson_histogram, loadHistograms
    from oracle.refcpu import RefCPU, threads
    base = molecule_coefficients()
    ref = RefCPU(L, LMAX, N, K)
    c3 = ref.c3(base)
    hist = loadHistograms(poisson_histogram(c3, K, N, TRIPLETS, seed=HIST_SEED), K)
    props = proposals(base, args.warmup + args.steps, PROP_SEED)
    for i in range(args.warmup):
        ref.energy(props[i], hist)
    t0 = time.perf_counter()
    for i in range(args.steps):
        ref.energy(props[args.warmup + i], hist)
    dt = time.perf_counter() - t0
    v = args.steps / dt
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 (f32 tables)", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "L18 K26 N32 LMAX25: one reference-form c3 + Bayes evaluation per step",
                       "L": L, "K": K, "N": N, "LMAX": LMAX, "proposals_per_step": 1},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads(), "kind": "port",
                             "sample": f"{args.steps} timed proposals (+{args.warmup} warm-up) of the workload"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line["reference_cuda"] = reference_cuda_rate(ref, props, hist)
    print(json.dumps(line), flush=True)
    return 0


def reference_cuda_rate(ref, props, hist, calls: int = 3):
    """The reference's own GPU path for the same workload, beside its CPU path: the
    unmodified src/cuda_kernel.cu kernel (PTX built from the reference sources where they
    were present) scaling h_P into PA, FP32 SGEMM c3 = B PA, c3 to the host and the FP64
    Bayes energy there (src/cuda.jl:74-108, src/correlations.jl:201).  Timed with the
    per-call h_P upload the reference makes and with h_P kept on the device."""
    try:
        import torch
        from oracle import refcuda
        from oracle.c3 import energy_bayes
        if not torch.cuda.is_available() or not refcuda.available():
            return {"unavailable": "no GPU or the reference kernel's PTX was not built"}
        timer = refcuda.RefCudaTimer(ref.b, ref.B32, ref.hP)
        out = {"kernel": "src/cuda_kernel.cu calculate_coefficient_matrix (unmodified, PTX) + FP32 SGEMM (cuBLAS, "
                         "TF32 off) + FP64 host Bayes", "unit": UNIT, "calls": calls}
        for key, up in (("value", True), ("value_hP_resident", False)):
            energy_bayes(timer.c3(props[0], up), hist, ref.K, ref.N)  # warm-up
            t0 = time.perf_counter()
            for i in range(calls):
                energy_bayes(timer.c3(props[1 + i % (len(props) - 1)], up), hist, ref.K, ref.N)
            out[key] = calls / (time.perf_counter() - t0)
        return out
    except Exception as exc:  # the baseline is informational: report why it is missing
        return {"unavailable": f"{type(exc).__name__}: {exc}"[:200]}


def ragged_measure(reps: int, warmup: int, rank: int = 0) -> dict:
    """64 chains x 16 speculative candidates per launch; chain c has its own K (16..26), L
    (12..18), molecule (200-400 atoms) and 1e9-triplet histogram; all candidates of a
    launch go through one ragged tensor-core launch on the L18 K26 N32 shape, replayed
    from a CUDA graph.  A spot check scores three chains' current states through the
    ragged launch and through contexts of their own (L, K) and reports the largest
    relative energy difference."""
    import torch
    import tp3
    from tp3.chains import Chains
    from tp3.structure import poisson_histogram, loadHistograms, seanindex0, structure_sh, synthetic_molecule
    nch, ncand = 64, 16
    rng = np.random.default_rng(20250301 + rank)
    Ks = rng.integers(16, K + 1, nch)
    Ls = rng.choice([12, 14, 16, 18], nch)
    atoms = rng.integers(200, 401, nch)
    # every chain's molecule expanded to intensity coefficients in one device call
    # (tp3_structure_sh, intensityShell route, FP64)
    mols = [synthetic_molecule(int(a), seed=5000 + 97 * c + rank) for c, a in enumerate(atoms)]
    coeffs = np.ascontiguousarray(structure_sh(mols, LMAX, KMAX, RMAX, route="intensity")["intensity"][:, :K])
    basis = tp3.calculate_basis(L, LMAX, N, K)
    hists = []
    for c in range(nch):
        x = coeffs[c].copy()
        for l in range(Ls[c] + 1, LMAX):
            x[:, [seanindex0(l, m, LMAX) for m in range(-l, l + 1)]] = 0
        c3 = basis.c3_raw(x).astype(np.float64)
        kl = int(Ks[c] * (Ks[c] + 1) * (Ks[c] + 2) // 6)
        hists.append(loadHistograms(poisson_histogram(c3[:, :kl], int(Ks[c]), N, TRIPLETS, seed=HIST_SEED + c),
                                    int(Ks[c])))
    basis.set_histograms(hists, Ks)
    # the autotuner times full-shape proposals against the first full-K chain's histogram
    full = int(np.argmax(Ks))
    c3f = basis.c3_raw(coeffs[full]).astype(np.float64)
    basis.set_histogram(loadHistograms(poisson_histogram(c3f, K, N, TRIPLETS, seed=HIST_SEED), K))
    tuning = basis.autotune(64)
    if basis.mode == tp3.TP3_MODE_PLAIN_FP32:
        basis.set_mode(tp3.TP3_MODE_TC_BF16X3)  # ragged launches are tensor-core only
    shapes = [(int(Ls[c]), int(Ks[c]), c) for c in range(nch)]
    ch = Chains(basis, coeffs, 0.1, math.pi / 4, 1.02, 0.99998, 4242 + rank, ncand=ncand, shapes=shapes)
    for _ in range(warmup):
        ch.run(1)
    s0 = ch.state()
    stream = torch.cuda.Stream()  # a real stream: the library treats handle 0 as "its own stream"
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    basis.set_stream(stream.cuda_stream)
    ev0.record(stream)
    ch.run(reps)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    s1 = ch.state()
    basis.set_stream(None)
    final = ch.coeff()
    ch.close()
    # spot check: three chains of distinct shapes, ragged launch vs contexts of their own shape
    picks, seen = [], set()
    for c in range(nch):
        if (int(Ls[c]), int(Ks[c])) not in seen and len(picks) < 3:
            seen.add((int(Ls[c]), int(Ks[c])))
            picks.append(c)
    dev = torch.device("cuda")
    states = np.stack([final[c] for c in picks])
    d_c = torch.from_numpy(np.ascontiguousarray(states).view(np.float64).copy()).to(dev)
    d_l = torch.tensor([(int(Ls[c]), int(Ks[c]), c) for c in picks], dtype=torch.int32, device=dev)
    d_E = torch.empty(len(picks), dtype=torch.float64, device=dev)
    basis.energy_batch_ragged_device(len(picks), d_c.data_ptr(), d_l.data_ptr(), d_E.data_ptr())
    basis.sync()
    E_rag = d_E.cpu().numpy()
    rel = []
    for j, c in enumerate(picks):
        own = tp3.calculate_basis(int(Ls[c]), LMAX, N, int(Ks[c]))
        own.set_mode(basis.mode)
        own.set_histogram(hists[c])
        E_own = float(own.energy_batch(states[j][None, :int(Ks[c])])[0])
        own.close()
        rel.append(abs(E_rag[j] - E_own) / abs(E_own))
    mode = basis.mode
    basis.close()
    return {"value": nch * ncand * reps / (ms / 1e3), "unit": UNIT, "ms_per_launch": ms / reps, "launches": reps,
            "chain_steps_per_s": float((s1["steps"] - s0["steps"]).sum()) / (ms / 1e3),
            "Ks": Ks.tolist(), "Ls": Ls.tolist(), "mode": MODE_NAMES.get(mode),
            "autotune": [{"mode": MODE_NAMES.get(m), "coupling": COUPLING_NAMES.get(sp) if m else None,
                          "angular": ANGULAR_NAMES.get(a) if m else None, "ms_per_proposal": t}
                         for m, sp, a, t in tuning],
            "spot_check": {"chains": [(int(Ls[c]), int(Ks[c])) for c in picks],
                           "max_rel_energy_diff_vs_own_shape_context": float(max(rel))},
            "gpu_launches_per_replay": 7,
            "workload": "64 chains (own molecule of 200-400 atoms, own 1e9-triplet histogram, K in 16..26, "
                        "L in 12..18, N32, LMAX25) x 16 speculative candidates per CUDA-graph replay; one ragged "
                        "tensor-core launch per step on the L18 K26 shape"}


def run_ragged(args):
    """--workload ragged: the ragged measurement as its own JSON line."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    r = ragged_measure(max(3, args.steps), args.warmup, rank)
    ms = max_over_ranks(r["ms_per_launch"] * r["launches"])
    value = whole_job_rate(ws, 64 * 16, r["launches"], ms)
    line = {"metric": "ragged c3+Bayes proposal evals/s, 64 chains x 16 candidates, K 16..26, L 12..18, N32",
            "value": value, "unit": UNIT, "n_gpus": ws, "steps": r["launches"], "warmup": args.warmup,
            "ms_per_step": ms / r["launches"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": DTYPES.get(tp3_mode_id(r["mode"]), "fp32"), "data": "synthetic",
            "config": {"workload": r["workload"], "Ks": r["Ks"], "Ls": r["Ls"], "mode": r["mode"],
                       "autotune": r["autotune"]},
            "chain_steps_per_s": r["chain_steps_per_s"], "spot_check": r["spot_check"],
            "gpu_launches": r["gpu_launches_per_replay"] * r["launches"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def lambda_measure(reps: int = 10, lam: float = 2.5, dq: float = 0.15) -> dict:
    """Ewald curvature: the same L18 K26 N32 workload at lambda = 2.5, dq = 0.15 (theta_k =
    acos(k lambda dq / 4 pi); the reference's own GPU test runs at lambda = 2.5), 64
    proposals per step through the tensor-core path (coupling, H from FP32 T, persistent
    tcgen05 contraction with the cosine table on the 2 048-point grid) and through the plain
    FP32 path; CUDA-event time of `reps` steps each on the launch stream, and the largest
    relative energy difference between the two paths."""
    import torch
    import tp3
    base = molecule_coefficients()
    basis = tp3.calculate_basis(L, LMAX, N, K, lam, dq)
    basis.set_histogram(build_histogram(basis, base))
    props = proposals(base, 64, PROP_SEED)
    stream = torch.cuda.Stream()
    basis.set_stream(stream.cuda_stream)
    d_coeff = torch.from_numpy(props.view(np.float64)).cuda()
    out = {"workload": f"L{L} K{K} N{N} LMAX{LMAX}, lambda {lam}, dq {dq}, 64 proposals per step", "steps": reps}
    E = {}
    for name, mode, form in (("tc_bf16x3", tp3.TP3_MODE_TC_BF16X3, 6), ("plain_fp32", tp3.TP3_MODE_PLAIN_FP32, None)):
        basis.set_mode(mode)
        if form is not None:
            basis.set_coupling(form)
        d_E = torch.empty(64, dtype=torch.float64, device="cuda")
        with torch.cuda.stream(stream):
            n = reps if mode != tp3.TP3_MODE_PLAIN_FP32 else max(2, reps // 5)
            basis.energy_batch_device(64, d_coeff.data_ptr(), d_E.data_ptr())  # warm-up
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(n):
                basis.energy_batch_device(64, d_coeff.data_ptr(), d_E.data_ptr())
            e1.record(stream)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / n
        E[name] = d_E.cpu().numpy()
        out[name] = {"proposals_per_s": 64 / (ms / 1e3), "ms_per_step": ms, "steps": n}
    basis.set_stream(None)
    basis.close()
    out["speedup_vs_plain_fp32"] = out["tc_bf16x3"]["proposals_per_s"] / out["plain_fp32"]["proposals_per_s"]
    out["max_rel_energy_diff_tc_vs_plain"] = float(np.max(np.abs(E["tc_bf16x3"] - E["plain_fp32"]) /
                                                          np.abs(E["plain_fp32"])))
    return out


def tp3_mode_id(name):
    return {v: k for k, v in MODE_NAMES.items()}.get(name, 0)


def learned_measure(rank: int = 0, **kw) -> dict:
    """The learned-proposal experiment at L18 K26 N32 (64 chains x 16 candidates): the
    isotropic per-shell annealer logs >= 1e6 moves, the network is trained on the device,
    and the learned annealer's wall-clock to the plain annealer's final median energy is
    measured from fresh starts (each shell of the molecule turned by a Haar rotation),
    beside the network-free drift annealer (the ablation)."""
    import tp3
    from tp3.learned import learned_vs_plain
    base = molecule_coefficients()
    basis = tp3.calculate_basis(L, LMAX, N, K)
    basis.set_histogram(build_histogram(basis, base))
    basis.autotune(64)
    res = learned_vs_plain(basis, base, seed=2024 + rank, **kw)
    basis.close()
    d = res.get("drift", {})
    return {"plain_seconds": res["plain"]["seconds"], "plain_launches": res["plain"]["launches"],
            "plain_final_median_E": res["plain"]["final_median_E"],
            "learned_seconds_to_target": res["learned"]["seconds_to_target"] if res["learned"]["reached"] else None,
            "learned_launches": res["learned"]["launches"], "learned_median_E": res["learned"]["median_E"],
            "time_ratio": res["time_ratio"],
            "drift_seconds_to_target": d.get("seconds_to_target") if d.get("reached") else None,
            "drift_launches": d.get("launches"), "drift_median_E": d.get("median_E"),
            "time_ratio_drift": res.get("time_ratio_drift"),
            "accept_rate": {"plain": res["plain"]["accept_rate"], "learned": res["learned"]["accept_rate"],
                            "drift": d.get("accept_rate")},
            "collect_moves": res["collect"]["moves"],
            "train": {k: res["train"][k] for k in ("steps", "heldout_nll_before", "heldout_nll_after", "seconds")},
            "workload": "64 chains x 16 candidates, per-shell SO(3) moves, 327-atom molecule, 1e9-triplet "
                        "histogram; plain = isotropic steps, learned = 0.8 network / 0.2 isotropic mixture with "
                        "Metropolis-Hastings correction, drift = the same mixture with the drift along the newest "
                        "gradient estimate and no network"}


def run_learned(args):
    """--workload learned: the learned-proposal measurement as its own JSON line."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    r = learned_measure(rank)
    line = {"metric": "time to the plain annealer's final median energy (learned proposal), L18 K26 N32",
            "value": r["learned_seconds_to_target"], "unit": "s", "n_gpus": ws, "steps": r["plain_launches"],
            "warmup": 1, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 network, fp64 moves", "data": "synthetic",
            "config": {"workload": r["workload"], "collect_moves": r["collect_moves"]}, **r}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_chains(args):
    """--workload chains: 64 chains x 16 candidates per CUDA-graph replay on the L18 K26
    N32 workload; CUDA-event time of --steps replays on the launch stream."""
    import torch
    import tp3
    from tp3.chains import Chains
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    base = molecule_coefficients()
    basis = tp3.calculate_basis(L, LMAX, N, K)
    basis.set_histogram(build_histogram(basis, base))
    if args.mode in ("auto", "tuned"):
        basis.autotune(64)
    else:
        basis.set_mode({"plain": tp3.TP3_MODE_PLAIN_FP32, "tc": tp3.TP3_MODE_TC_BF16X3,
                        "tf32": tp3.TP3_MODE_TC_TF32X3}[args.mode])
        if args.coupling >= 0:
            basis.set_coupling(args.coupling)
        if args.mode in ("tc", "tf32"):
            basis.set_angular(ANGULAR_CODES[args.angular])
    nch, ncand = 64, 16
    ch = Chains(basis, np.repeat(base[None, :K], nch, axis=0), 5.0, math.pi / 4, 1.02, 0.99998, 12345 + rank,
                ncand=ncand)
    ch.run(max(3, args.warmup))
    stream = torch.cuda.Stream()
    basis.set_stream(stream.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    ch.run(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1))
    basis.set_stream(None)
    line = {"metric": "chain launches: proposals/s, 64 chains x 16 candidates per CUDA-graph replay, L18 K26 N32",
            "value": whole_job_rate(ws, nch * ncand, args.steps, ms), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": DTYPES.get(basis.mode, "fp32"), "data": "synthetic",
            "config": {"workload": "64 chains x 16 speculative candidates (reference move) per graph replay",
                       "mode": MODE_NAMES.get(basis.mode)}, "gpu_launches": 7 * args.steps}
    ch.close()
    basis.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--mode", default="auto", choices=["auto", "tuned", "plain", "tc", "tf32"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="proposals", choices=["proposals", "ragged", "learned", "chains"])
    ap.add_argument("--coupling", type=int, default=-1, choices=[-1, 0, 1, 2, 3, 4, 5, 6, 7, 8],
                    help="force a tensor-core coupling form (with --mode tc/tf32)")
    ap.add_argument("--angular", default="persistent", choices=["persistent", "tile"],
                    help="angular-stage schedule of the tensor-core path (with --mode tc/tf32)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-chains", action="store_true")
    ap.add_argument("--no-ragged", action="store_true", help="leave the ragged-chain key out of the line")
    ap.add_argument("--no-learned", action="store_true", help="leave the learned-proposal key out of the line")
    ap.add_argument("--no-lambda", action="store_true", help="leave the lambda != 0 key out of the line")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "ragged":
        return run_ragged(args)
    if args.workload == "learned":
        return run_learned(args)
    if args.workload == "chains":
        return run_chains(args)
    args.warmup = max(args.warmup, 3)

    import torch
    import tp3
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    mode = {"auto": None, "tuned": None, "plain": tp3.TP3_MODE_PLAIN_FP32, "tc": tp3.TP3_MODE_TC_BF16X3,
            "tf32": tp3.TP3_MODE_TC_TF32X3}[args.mode]

    base = molecule_coefficients()
    basis = tp3.calculate_basis(L, LMAX, N, K)
    hist = build_histogram(basis, base)
    basis.set_histogram(hist)
    tuning = None
    if mode is None:
        tuning = [{"mode": MODE_NAMES.get(m, str(m)), "coupling": COUPLING_NAMES.get(sp) if m else None,
                   "angular": ANGULAR_NAMES.get(a) if m else None, "ms_per_proposal": ms}
                  for m, sp, a, ms in basis.autotune(args.batch)]
    else:
        basis.set_mode(mode)
        if args.coupling >= 0:
            basis.set_coupling(args.coupling)
        if mode != tp3.TP3_MODE_PLAIN_FP32:
            basis.set_angular(ANGULAR_CODES[args.angular])
    mode_used = basis.mode
    B = args.batch
    basis.reserve(B)
    props = proposals(base, B, PROP_SEED + rank)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    basis.set_stream(stream.cuda_stream)
    d_coeff = torch.from_numpy(props.view(np.float64)).cuda()
    d_E = torch.empty(B, dtype=torch.float64, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step():
        basis.energy_batch_device(B, d_coeff.data_ptr(), d_E.data_ptr())

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    E_dev = d_E.cpu().numpy()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clk_dir = tempfile.mkdtemp(prefix="tp3_clocks_")
    clk_path = os.path.join(clk_dir, f"clocks_rank{rank}.csv")
    cp, cf = sample_clocks_start(clk_path)
    time.sleep(0.3)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    basis.profile_enable(True)
    for i in range(args.steps):
        flush.zero_()
        starts[i].record(stream)
        step()
        ends[i].record(stream)
    torch.cuda.synchronize()
    n_prof, ms_prof = basis.profile_read(0)
    n_prof_c, ms_prof_c = basis.profile_read(1)
    basis.profile_enable(False)
    if ws > 1:
        torch.distributed.barrier()
    clocks = sample_clocks_stop(cp, cf, clk_path, local)
    ms = max_over_ranks(sum(s.elapsed_time(e) for s, e in zip(starts, ends)))
    ms_per_step = ms / args.steps
    value = whole_job_rate(ws, B, args.steps, ms)

    # end to end through the public host API (H2D + compute + D2H): where the device reads
    # pageable host memory, a kernel fetches the coefficients in place, else the host packs
    # them into pinned memory and copies them
    basis.set_stream(None)
    try:
        basis.set_host_input(tp3.TP3_HOST_INPUT_DIRECT)
        route = "direct: a kernel reads the used coefficients from the host array over the host page tables"
    except tp3.TP3Error:
        route = "staged: host packing into pinned memory, one cudaMemcpyAsync"
    host_props = props.copy()
    for _ in range(2):
        basis.energy_batch(host_props)
    e2e_steps = max(3, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        E_host = basis.energy_batch(host_props)
    e2e_dt = time.perf_counter() - t0
    # the host API packs the even-l <= L block of each shell (nc complex doubles) before the copy
    e2e = {"value": ws * B * e2e_steps / e2e_dt, "unit": UNIT,
           "h2d_bytes_per_step": int(B * K * basis.nc * 16), "d2h_bytes_per_step": int(E_host.nbytes),
           "host_input": route}
    if not np.allclose(E_host, E_dev, rtol=0, atol=0):
        raise SystemExit("device-resident and host-API energies differ")

    # per-stage rooflines: the coupling (SIMT FP32, the longest-running kernel) against the
    # FP32 FMA peak measured in this run, the angular contraction + fused Bayes against the
    # BF16 tensor peak of MEASURED_PEAKS.json
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 1900.0, "fallback"
    if os.path.exists(peaks_path):
        pk = json.load(open(peaks_path))
        peak, peak_src = float(pk.get("bf16_tflops", 1900.0)), "measured"
    n_lt = basis.n_lt
    klength = basis.klength
    G = 2 * N * N
    # algorithmic angular work per proposal: the cheaper exact form (separable over (m2, m3))
    M = 2 * L + 1
    nnz = basis.nnz_pi2
    W_b = min(2.0 * G * n_lt * klength, 2.0 * nnz * klength + klength * (4 * N * M * M * 2 + 4 * N * N * M * 2))
    per_launch_ms = ms_prof / max(1, n_prof)
    achieved = W_b * B / (per_launch_ms / 1e3) / 1e12
    cform = None
    aname = args.angular
    if tuning:
        best = min((t for t in tuning if t["mode"] == MODE_NAMES.get(mode_used)), key=lambda t: t["ms_per_proposal"],
                   default=None)
        cform = best["coupling"] if best else None
        aname = (best["angular"] if best else None) or aname
    elif args.coupling >= 0:
        cform = COUPLING_NAMES.get(args.coupling)
    traffic_c = traffic_a = None
    tsrc = STAGE_TRAFFIC.get((MODE_NAMES.get(mode_used), cform, aname))
    if tsrc is not None:
        traffic_c = tsrc["coupling"][0] * B + tsrc["coupling"][1]
        traffic_a = tsrc["angular"][0] * B + tsrc["angular"][1]
    stages = None
    roofline = None
    if n_prof_c > 0:
        # W_a = 10 P2 basislen + 4 S klength (pair-factorised coupling), S = sum over the
        # l-triples (even l <= L, triangle) of 2 l3 + 1
        trip = [(a, b, c) for a in range(0, L + 1, 2) for b in range(0, L + 1, 2) for c in range(0, L + 1, 2)
                if abs(a - b) <= c <= a + b]
        if len(trip) != n_lt:
            raise SystemExit("l-triple count differs from the basis")
        S = sum(2 * c + 1 for _, _, c in trip)
        W_a = 10.0 * (K * (K + 1) / 2) * basis.basislen + 4.0 * S * klength
        ms_c = ms_prof_c / n_prof_c
        fp32_peak = basis.measure_fp32_peak()
        ach_c = W_a * B / (ms_c / 1e3) / 1e12
        stages = {"coupling": {"bound": "fp32", "kernel": f"coupling ({cform or 'default form'})",
                               "ms_per_launch": ms_c, "algorithmic_flop_per_proposal": W_a, "achieved": ach_c,
                               "peak": fp32_peak, "frac": ach_c / fp32_peak, "unit": "TFLOP/s",
                               "peak_source": "measured FFMA (tp3_measure_fp32_peak, this run)",
                               "traffic": traffic_c},
                  "angular": {"bound": "tensor",
                              "kernel": f"angular contraction + fused Bayes (tcgen05, {aname} schedule)",
                              "ms_per_launch": per_launch_ms, "algorithmic_flop_per_proposal": W_b,
                              "achieved": achieved, "peak": peak, "frac": achieved / peak, "unit": "TFLOP/s",
                              "peak_source": f"{peak_src} bf16 dense burst", "traffic": traffic_a}}
        # headline: the dominant (longest-running) kernel of the step
        dom = "coupling" if ms_c >= per_launch_ms else "angular"
        st = stages[dom]
        roofline = {"bound": st["bound"], "achieved": st["achieved"], "peak": st["peak"], "unit": "TFLOP/s",
                    "frac": st["frac"], "traffic": st["traffic"], "traffic_unit": "bytes per launch",
                    "traffic_source": tsrc["source"] if tsrc else None, "peak_source": st["peak_source"],
                    "kernel": st["kernel"], "kernel_ms_per_launch": st["ms_per_launch"],
                    "algorithmic_flop_per_proposal": st["algorithmic_flop_per_proposal"],
                    "share_of_step": st["ms_per_launch"] / ms_per_step,
                    "note": "the coupling runs on the FP32 FMA pipes (MEASURED_PEAKS.json has no FP32 figure, so "
                            "its peak is measured in this run); the tensor-core stage is stages.angular"}

    # device-resident annealing chains: 64 chains x 16 speculative candidates per graph replay
    chains_info = None
    if not args.no_chains:
        from tp3.chains import Chains
        basis.set_stream(None)
        nch, ncand = 64, 16
        T0 = np.full(nch, 0.1 * float(np.std(E_dev)))
        ch = Chains(basis, np.repeat(base[None, :K], nch, axis=0), T0, math.pi / 4, 1.02, 0.99998, 12345,
                    ncand=ncand)
        ch.run(2)
        s0 = ch.state()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        reps = max(3, args.steps // 2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ch.run(reps)
        s1 = ch.state()
        dt = time.perf_counter() - t0
        chains_info = {"chains": nch, "candidates_per_launch": ncand, "launches": reps,
                       "graph_captured": ch.graph_captured,
                       "proposals_per_s": nch * ncand * reps / dt,
                       "chain_steps_per_s": float((s1["steps"] - s0["steps"]).sum()) / dt,
                       "ms_per_launch": 1e3 * dt / reps,
                       "note": "wall clock around graph replays incl. one final synchronise; proposals include "
                               "device-side move generation and the Metropolis update"}
        ch.close()
        # the same chains on the plain FP32 path: seeded chains follow the same trajectory in
        # both modes, so the time to a given energy scales with chain steps per second
        if mode_used != tp3.TP3_MODE_PLAIN_FP32:
            basis.set_mode(tp3.TP3_MODE_PLAIN_FP32)
            chp = Chains(basis, np.repeat(base[None, :K], nch, axis=0), T0, math.pi / 4, 1.02, 0.99998, 12345,
                         ncand=ncand)
            chp.run(1)
            q0 = chp.state()
            t0 = time.perf_counter()
            chp.run(10)
            q1 = chp.state()
            dtp = time.perf_counter() - t0
            chp.close()
            basis.set_mode(mode_used)
            plain_steps = float((q1["steps"] - q0["steps"]).sum()) / dtp
            chains_info["plain_fp32_chain_steps_per_s"] = plain_steps
            chains_info["time_to_energy_speedup_vs_plain_fp32"] = chains_info["chain_steps_per_s"] / plain_steps

    kernels_per_step = 4
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPES.get(mode_used, "fp32"),
            "data": "synthetic",
            "config": {"workload": f"L18 K26 N32 LMAX25, {B} proposals per step (get_MC_step moves of a 327-atom "
                                   "synthetic molecule's intensity), 1e9-triplet Poisson histogram",
                       "L": L, "K": K, "N": N, "LMAX": LMAX, "proposals_per_step": B,
                       "mode": MODE_NAMES.get(mode_used, str(mode_used)), "autotune": tuning,
                       "l2": "flushed (512 MB write) between steps, outside the per-step events"},
            "e2e": e2e, "roofline": roofline, "stages": stages, "clocks": clocks, "chains": chains_info,
            "gpu_launches": kernels_per_step * args.steps}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(base, hist)
    basis.close()
    # the batched ragged workload (64 chains of mixed L and K) and the learned-proposal
    # experiment with its drift-only ablation, measured in the same run (rank 0)
    if rank == 0 and not args.no_ragged:
        try:
            line["ragged"] = ragged_measure(10, 2, rank)
        except Exception as exc:  # informational keys: report why they are missing
            line["ragged"] = {"error": f"{type(exc).__name__}: {exc}"[:300]}
    if rank == 0 and not args.no_lambda:
        try:
            line["lambda"] = lambda_measure()
        except Exception as exc:
            line["lambda"] = {"error": f"{type(exc).__name__}: {exc}"[:300]}
    if rank == 0 and not args.no_learned:
        try:
            line["learned"] = learned_measure(rank)
        except Exception as exc:
            line["learned"] = {"error": f"{type(exc).__name__}: {exc}"[:300]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
