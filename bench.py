"""Benchmark: Beyn contour step on the star domain (CFIE Kress), one GB300.

Workload (the headline metric's configuration): CFIE_kress on the star
r(theta) = 1 + 0.2 cos(5 theta), N = 2048 nodes, one disk k0 = 200, R = 0.5,
nq = 48 trapezoid contour nodes, L = 64 seeded complex Gaussian probes (std 1),
svd_tol = 1e-12, the reference's single r -> 2r regrowth when the rank
saturates. A step = one full Beyn disk: assembly of the 48 T(z_j), batched
LU, T^-1 V solves (+ regrowth solves), moments, host SVD/eig.

metric: eigenvalues/s of the mixed form (FP32 assembly/LU + compensated
refinement) counting eigenvalues inside the disk that agree with the plain
FP64 GPU path to <= 1e-10 relative; the plain FP64 path is timed beside it.

--workload ebim prints a second line for the EBIM eigen step on the same
geometry (k = 200, dk = 0.05, nev = 5): steps/s of device assembly + eigen
step, the same from host matrices (e2e), and the oracle's dense
solve_krylov on the same matrices as the CPU baseline.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "quantumbilliards.jl_gb300"))

N_NODES, K0, RADIUS, NQ, L_PROBES, SVD_TOL = 2048, 200.0, 0.5, 48, 64, 1e-12
TOL_EIG = 1e-10
IMAG_TOL = 1e-6
SEED = 2


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


METRIC = "eigenvalues/s at <=1e-10 rel err (mixed FP32+refinement vs plain FP64), Beyn CFIE Kress star"


def workload_config():
    return {"workload": "beyn_cfie_kress_star_N2048_k0_200_R0.5_nq48_L64", "N": N_NODES, "k0": K0, "R": RADIUS,
            "nq": NQ, "L": L_PROBES, "l2": "inputs larger than L2 (3.2 GB of T(z_j))"}


def star_workspace(qb, kind="cfie"):
    b = qb.make_star(0.2, 5)
    sol = qb.CFIE_kress(1.0, b) if kind == "cfie" else qb.DLP_kress(1.0, b)
    pts, sol = qb.points_with_n(sol, b, N_NODES, K0)
    return b, sol, pts


def select(lam, k0=K0, R=RADIUS):
    lam = np.asarray(lam)
    return np.sort_complex(lam[(np.abs(lam - k0) <= R) & (np.abs(lam.imag) < IMAG_TOL)])


def match(lam, ref):
    """Per-eigenvalue relative error against the nearest reference eigenvalue."""
    if len(ref) == 0:
        return np.full(len(lam), np.inf)
    return np.array([np.min(np.abs(ref - l)) / abs(l) for l in lam])


def run_step(qb, sol, pts, ws, mixed, rng_seed=SEED, with_geometry=False):
    t0 = time.perf_counter()
    if with_geometry:
        ws = qb.Workspace(sol, pts)
    lam, info = qb.solve(sol, pts, K0 + 0j, RADIUS, nq=NQ, r=L_PROBES, svd_tol=SVD_TOL,
                         rng=np.random.default_rng(rng_seed), mixed=mixed, ws=ws, return_info=True)
    dt = time.perf_counter() - t0
    if with_geometry:
        ws.close()
    return lam, info, dt


def init_replicas():
    """Process group for the barrier and the max-over-ranks time (gloo: host-side only,
    the data path has no collective)."""
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group("gloo")


def replica_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def replica_reduce(world, t_region, eig_count):
    """(max over ranks of the timed region, sum over ranks of the eigenvalues found)."""
    if world <= 1:
        return t_region, eig_count
    import torch
    import torch.distributed as dist
    t = torch.tensor([t_region], dtype=torch.float64)
    c = torch.tensor([eig_count], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return float(t.item()), float(c.item())


def cpu_baseline(qb, sol, pts, nsample=1):
    """Oracle (NumPy/SciPy FP64 restatement) on a bounded sample: assembly +
    LU + solves for `nsample` contour nodes, extrapolated to the 48-node disk."""
    from oracle import assembly as OA
    import scipy.linalg as sla
    zj = K0 + RADIUS * np.exp(2j * math.pi * np.arange(NQ) / NQ)
    V = qb.probe_matrix(pts[0].n, L_PROBES, np.random.default_rng(SEED))
    t0 = time.perf_counter()
    for z in zj[:nsample]:
        T = OA.cfie_matrix(pts, z)
        f = sla.lu_factor(T, check_finite=False)
        sla.lu_solve(f, V, check_finite=False)
    dt = (time.perf_counter() - t0) / nsample * NQ
    return dt


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--workload", default="beyn", choices=["beyn", "ebim"],
                    help="beyn: the headline Beyn disk (default); ebim: the EBIM eigen step at one k")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank != 0:
            return
        return reference_arm_ebim(args) if args.workload == "ebim" else reference_arm(args)
    if args.workload == "ebim":
        if rank != 0:
            return
        return ebim_workload(args)
    if world > 1:
        # one process per GPU: this rank sees only its own device
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("LOCAL_RANK", str(rank)))
        init_replicas()

    import build_qbgpu as B
    B.build()
    import qbgpu as qb
    from qbgpu import _lib

    b, sol, pts = star_workspace(qb)
    ws = qb.Workspace(sol, pts)

    # FP64 reference eigenvalues for the accuracy filter (plain GPU path, validated against the oracle in tests)
    lam64, info64, t_plain_first = run_step(qb, sol, pts, ws, mixed=False)
    ref = select(lam64)
    plain_times = []
    for _ in range(max(0, args.plain_steps)):
        _, _, dt = run_step(qb, sol, pts, ws, mixed=False)
        plain_times.append(dt)
    t_plain = float(np.median(plain_times)) if plain_times else t_plain_first

    for _ in range(args.warmup):
        run_step(qb, sol, pts, ws, mixed=True)
    _lib.load().qbg_device_sync()
    replica_barrier(world)
    clk = ClockSampler()
    clk.start()
    times, counts, errs, stats = [], [], [], []
    launches0 = qb.launch_count()
    t_region0 = time.perf_counter()
    for s in range(args.steps):
        lam, info, dt = run_step(qb, sol, pts, ws, mixed=True)
        sel = select(lam)
        e = match(sel, ref)
        counts.append(int(np.count_nonzero(e <= TOL_EIG)))
        errs.append(float(e.max()) if len(e) else float("nan"))
        times.append(dt)
        stats.append(info["stats"])
    _lib.load().qbg_device_sync()
    t_region = time.perf_counter() - t_region0
    gpu_launches = qb.launch_count() - launches0
    replica_barrier(world)
    clocks = clk.stop()
    # replicas: every rank ran the same disk on its own GPU; the job's time is the slowest rank's
    t_region_max, eig_total = replica_reduce(world, t_region, float(sum(counts)))
    # end to end through the public API including the geometry upload
    e2e_times = []
    for _ in range(max(1, min(args.steps, 3))):
        _, _, dt = run_step(qb, sol, pts, None, mixed=True, with_geometry=True)
        e2e_times.append(dt)
    # FP32 form (FP32 kernel values): reported beside, with its own accuracy
    lam32, info32, t32 = run_step(qb, sol, pts, ws, mixed="fp32")
    lam32, info32, t32 = run_step(qb, sol, pts, ws, mixed="fp32")
    e32 = match(select(lam32), ref)
    fp32_form = {"ms_per_step": t32 * 1e3, "eigenvalues_inside": int(len(e32)),
                 "eigenvalues_le_1e-10": int(np.count_nonzero(e32 <= TOL_EIG)),
                 "max_rel_err_vs_fp64": float(e32.max()) if len(e32) else None}

    t_step = t_region_max / args.steps
    n_eig = float(np.mean(counts))
    value = eig_total / t_region_max  # whole job: eigenvalues of all replicas / slowest rank's time
    plain_eigs = len(ref)
    st0 = stats[-1][0]
    r_final = info["r"]
    N = ws.dim
    h2d = 8 * 8 * N + 16 * N * (L_PROBES + (r_final if r_final != L_PROBES else 0))
    d2h = 2 * 16 * N * (L_PROBES + (r_final if r_final != L_PROBES else 0))
    hbm, bf16, peak_kind = _peaks()
    # roofline kernel: the tensor-core refinement residual R = V - (hi + lo) X over
    # all nodes (k_resid_tc). Algorithmic work per launch = one complex GEMM,
    # 8 N^2 L nq real flops; the kernel issues 28 digit-pair bf16 products of
    # that real-mapped GEMM (224 N^2 Lp nq flops, Lp = L rounded up to 32).
    res_ms, res_n = 0.0, 0
    for srun in stats:
        for s in srun:
            res_ms += s["ms_residual"]
            res_n += s["n_residual"]
    res_launch_ms = res_ms / max(res_n, 1)
    res_flops = 8.0 * N * N * L_PROBES * NQ
    lp = ((L_PROBES + 31) // 32) * 32
    res_issued = 224.0 * N * N * lp * NQ
    achieved = res_flops / (res_launch_ms * 1e-3) / 1e12
    issued_tflops = res_issued / (res_launch_ms * 1e-3) / 1e12
    # DRAM traffic per launch: ncu capture of the same kernel at nq = 8, L = 64
    # (1009.98 MB read + 16.03 MB written), scaled by the contour nodes (48 / 8);
    # the algorithmic bytes (digit planes of T and X, V, R) are 1.03 GB at nq = 8
    res_traffic = (1009.98e6 + 16.03e6) * (NQ / 8.0)
    res_alg_bytes = (7 * N * 2 * N * 2 + 7 * 2 * lp * 2 * N * 2 + 2 * 16 * N * L_PROBES) * NQ
    lu_flops = NQ * (8.0 / 3.0) * N ** 3
    ms_factor = float(np.mean([s[0]["ms_factor"] for s in stats]))
    lu_achieved = lu_flops / (ms_factor * 1e-3) / 1e12
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "eigenvalues/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_step * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c64+c128",
        "data": "synthetic",
        "config": dict(workload_config(), r_final=r_final,
                       timing="wall clock of the synchronous API calls between device synchronizations (the step "
                              "ends with the host SVD and eigvals); device phases in phases_ms are CUDA events"),
        "plain_fp64": {"value": plain_eigs / t_plain, "ms_per_step": t_plain * 1e3, "eigenvalues": plain_eigs},
        "speedup_vs_plain": ((n_eig / t_step) / (plain_eigs / t_plain)) if plain_eigs else None,
        "eigenvalues_per_step": n_eig,
        "max_rel_err_vs_fp64": float(np.max(errs)),
        "phases_ms": {"assemble": st0["ms_assemble"], "factor": st0["ms_factor"],
                      "solve_refine": sum(s["ms_solve"] for s in stats[-1])},
        "host_ms": {k: float("%.3g" % v) for k, v in info["host_ms"].items()},
        "refine_sweeps": [s["refine_sweeps"] for s in stats[-1]],
        "refine_history": [[float("%.3g" % v) for v in s["refine_history"]] for s in stats[-1]],
        "plain_phases_ms": {"assemble": info64["stats"][0]["ms_assemble"], "factor": info64["stats"][0]["ms_factor"],
                            "solve": sum(s["ms_solve"] for s in info64["stats"])},
        "fp32_form": fp32_form,
        "e2e": {"value": n_eig / float(np.mean(e2e_times)), "unit": "eigenvalues/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
                     "frac": achieved / bf16, "traffic": res_traffic, "algorithmic_bytes": res_alg_bytes,
                     "kernel": "k_resid_tc (exact 7-bit digit products on tcgen05, bf16 -> FP32 TMEM)",
                     "peak_kind": peak_kind, "launch_ms": res_launch_ms,
                     "launches_per_step": res_n / max(len(stats), 1),
                     "issued_tflops": issued_tflops, "frac_issued": issued_tflops / bf16,
                     "note": "achieved counts the complex GEMM's 8 N^2 L flops; the tensor pipe executes 28 "
                             "digit-pair products of it, whose rate is issued_tflops (frac_issued of the "
                             "measured bf16 peak)"},
        "lu_phase": {"achieved_tflops": lu_achieved, "ms": ms_factor, "flops": lu_flops,
                     "engine": "FP32 panels on CUDA cores; trailing updates and solves on tcgen05 (3xTF32)"},
        "clocks": clocks,
        "gpu_launches": gpu_launches,
        "gpu_launches_per_step": gpu_launches / max(args.steps, 1),
    }
    if world > 1:
        line["config"]["parallelism"] = f"replicas{world}"
    if not args.no_cpu_baseline and rank == 0 and world == 1:
        t_cpu = cpu_baseline(qb, sol, pts, 1)
        line["cpu_baseline"] = {"value": plain_eigs / t_cpu, "unit": "eigenvalues/s", "cores": os.cpu_count(),
                                "kind": "port",
                                "sample": "oracle assembly+LU+solve of 1 of 48 contour nodes, extrapolated x48"}
    if rank == 0:
        print(json.dumps(line))


EBIM_K, EBIM_DK, EBIM_NEV = 200.0, 0.05, 5
EBIM_METRIC = "EBIM eigen steps/s (solve_krylov!, nev = 5, dk = 0.05), CFIE Kress star N = 2048, k = 200"
EBIM_CONFIG = {"workload": "ebim_cfie_kress_star_N2048_k200_dk0.05_nev5", "N": N_NODES, "k": EBIM_K, "dk": EBIM_DK,
               "nev": EBIM_NEV, "l2": "A, A', A'' and C = A^-1 A' (67 MB each) stream from HBM"}


def ebim_workload(args):
    """--workload ebim: one step = A, A', A'' assembled at k on the device and
    the eigen step of solve_krylov! (qbg_ebim_solve); e2e = the same step from
    host matrices through qbgpu.ebim.solve_krylov (the three N x N matrices
    copied in every step). cpu_baseline: the oracle's solve_krylov on the same
    matrices (dense LAPACK eig of A^-1 A' and its adjoint)."""
    import build_qbgpu as B
    B.build()
    import qbgpu as qb
    from qbgpu import _lib
    b, sol, pts = star_workspace(qb)
    ws = qb.Workspace(sol, pts)
    for _ in range(args.warmup):
        qb.ebim.solve(ws, EBIM_K, EBIM_DK, nev=EBIM_NEV)
    _lib.load().qbg_device_sync()
    clk = ClockSampler()
    clk.start()
    launches0 = qb.launch_count()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        kc, tens = qb.ebim.solve(ws, EBIM_K, EBIM_DK, nev=EBIM_NEV)
    _lib.load().qbg_device_sync()
    t = (time.perf_counter() - t0) / args.steps
    launches = qb.launch_count() - launches0
    clocks = clk.stop()
    A, dA, ddA = qb.assemble(ws, [EBIM_K], deriv=True)
    qb.ebim.solve_krylov(None, A, dA, ddA, pts, EBIM_K, EBIM_DK, nev=EBIM_NEV)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        qb.ebim.solve_krylov(None, A, dA, ddA, pts, EBIM_K, EBIM_DK, nev=EBIM_NEV)
    te = (time.perf_counter() - t0) / args.steps
    line = {"metric": EBIM_METRIC, "value": 1.0 / t, "unit": "EBIM steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic", "config": EBIM_CONFIG,
            "roots": [round(float(x), 9) for x in kc], "tensions": [float(x) for x in tens],
            "e2e": {"value": 1.0 / te, "unit": "EBIM steps/s", "h2d_bytes_per_step": 3 * 16 * ws.dim ** 2,
                    "d2h_bytes_per_step": 24 * len(kc)},
            "gpu_launches": launches, "clocks": clocks}
    if not args.no_cpu_baseline:
        from oracle import ebim as OE
        t0 = time.perf_counter()
        ko, _ = OE.solve_krylov(A, dA, ddA, EBIM_K, EBIM_DK, nev=EBIM_NEV)
        tc = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": 1.0 / tc, "unit": "EBIM steps/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": "one solve_krylov step of the oracle (LU, dense eig of A^-1 A' and of its "
                                          "adjoint) on the same device-assembled matrices"}
        if len(ko) == len(kc):
            line["max_abs_diff_vs_oracle"] = float(np.max(np.abs(np.sort(ko) - np.sort(kc)))) if len(ko) else 0.0
    print(json.dumps(line))


def reference_arm_ebim(args):
    """--impl reference --workload ebim: the oracle's solve_krylov on its own
    FP64 assembly of the same workload, one eigen step per timed step."""
    import qbgpu.geometry as G  # host-only modules (no GPU work)
    from qbgpu import solvers as S
    from oracle import assembly as OA, ebim as OE
    b = G.make_star(0.2, 5)
    pts, sol = S.points_with_n(S.CFIE_kress(1.0, b), b, N_NODES, K0)
    A, dA, ddA = OA.cfie_matrix_derivs(pts, EBIM_K)
    for _ in range(min(args.warmup, 1)):
        OE.solve_krylov(A, dA, ddA, EBIM_K, EBIM_DK, nev=EBIM_NEV)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        OE.solve_krylov(A, dA, ddA, EBIM_K, EBIM_DK, nev=EBIM_NEV)
        times.append(time.perf_counter() - t0)
    t = float(np.mean(times))
    print(json.dumps({"impl": "reference", "metric": EBIM_METRIC, "value": 1.0 / t, "unit": "EBIM steps/s",
                      "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
                      "higher_is_better": True, "dtype": "c128", "data": "synthetic", "config": EBIM_CONFIG,
                      "cpu_baseline": {"value": 1.0 / t, "unit": "EBIM steps/s", "cores": os.cpu_count(),
                                       "kind": "port", "sample": "the full eigen step per timed step"},
                      "e2e": {"value": 1.0 / t, "unit": "EBIM steps/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}))


def reference_arm(args):
    """--impl reference: the oracle's FP64 CPU restatement on the host cores."""
    import qbgpu.geometry as G  # host-only modules (no GPU work)
    from qbgpu import solvers as S
    b = G.make_star(0.2, 5)
    pts, sol = S.points_with_n(S.CFIE_kress(1.0, b), b, N_NODES, K0)
    from oracle import assembly as OA
    import scipy.linalg as sla
    zj = K0 + RADIUS * np.exp(2j * math.pi * np.arange(NQ) / NQ)
    rng = np.random.default_rng(SEED)
    V = (rng.standard_normal((pts[0].n, L_PROBES)) + 1j * rng.standard_normal((pts[0].n, L_PROBES))) * math.sqrt(.5)
    times = []
    for s in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        z = zj[s % NQ]
        T = OA.cfie_matrix(pts, z)
        f = sla.lu_factor(T, check_finite=False)
        sla.lu_solve(f, V, check_finite=False)
        if s >= args.warmup:
            times.append((time.perf_counter() - t0) * NQ)
    t = float(np.mean(times))
    eig_per_disk = 100.0  # Weyl estimate for the disk (area*k/2pi*2R - L/4pi*2R)
    val = eig_per_disk / t
    print(json.dumps({"impl": "reference", "metric": METRIC, "value": val,
                      "unit": "eigenvalues/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": t * 1e3, "higher_is_better": True, "dtype": "c128", "data": "synthetic",
                      "config": dict(workload_config(),
                                     timing="host wall clock of one contour node's FP64 CFIE assembly, LU and "
                                            "L-column solve, times 48 nodes; eigenvalues per disk = 100, the "
                                            "Weyl estimate"),
                      "cpu_baseline": {"value": val, "unit": "eigenvalues/s", "cores": os.cpu_count(), "kind": "port",
                                       "sample": "one contour node per step, extrapolated x48"},
                      "e2e": {"value": val, "unit": "eigenvalues/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}))


if __name__ == "__main__":
    main()
