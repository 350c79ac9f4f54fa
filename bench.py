"""Benchmark: Beyn contour step on the star domain (CFIE Kress), one GB300.

Workload (the headline metric's configuration): CFIE_kress on the star
r(theta) = 1 + 0.2 cos(5 theta), N = 2048 nodes, one disk k0 = 200, R = 0.5,
nq = 48 trapezoid contour nodes, L = 64 seeded complex Gaussian probes (std 1),
svd_tol = 1e-12, the reference's single r -> 2r regrowth when the rank
saturates. Chebyshev panels are tuned once per run to 1e-13 absolute error
(the tolerance compute_spectrum_beyn gives chebyshev_params), by the library's
cost-aware tuner; the tuning time is reported as plan_s. The LU plan of the
mixed step (panel width, outer-block depth, stream parts) is then chosen by
timing whole steps of this workload (qbgpu.autotune.tune_beyn; lu_plan lists
the plans tried). A step = one full Beyn disk: assembly
of the 48 T(z_j), batched LU, T^-1 V solves (+ regrowth solves), moments,
host SVD/eig.

metric: eigenvalues/s of the mixed form (FP32 LU + FP64-accurate refinement)
counting eigenvalues inside the disk that agree with the oracle's FP64
eigenvalues (tests/golden/c2_beyn.json: direct AMOS kernel values, LAPACK,
same probes and regrowth) to <= 1e-10 relative; every eigenvalue's error against the
oracle is reported, and the plain FP64 path is timed beside it.

cpu_baseline and --impl reference: the reference's CPU algorithm restated on
the host cores (oracle/cpu.py: Chebyshev tables from AMOS, C assembly threaded
over columns, LAPACK LU and solves, the fresh 2r regrowth block), one whole
disk per timed step (at most three, after at most one untimed: a disk is ~18 s
on 16 cores); the eigenvalues are matched to the oracle fixture of the
reference's regrowth policy (tests/golden/c2_beyn_fresh.json).

other_configs (default run, after the timed region; --no-extras leaves it
out): bounded samples of the other configurations -- C1 (the sigma_min sweep
of the unit circle and refine_minima), C3 (32 batched disks of the
desymmetrised stadium) and the first 60 requests of the C4 served stream with
N capped at 2048, with p50/p99 latency.

--workload ebim prints a line for the EBIM eigen step on the same geometry
(k = 200, dk = 0.05, nev = 5): steps/s of device assembly + eigen step, the
same from host matrices (e2e), and the oracle's dense solve_krylov on the
same matrices as the CPU baseline. --workload c1 / c3 / serve print one line
for that configuration (serve: the full C4 stream, 2000 requests at 20 req/s,
N in [1024, 8192], unless --requests / --rate / --nmin / --nmax / --nk say
otherwise).
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
CHEB_TOL = 1e-13
GOLDEN = ROOT / "tests" / "golden" / "c2_beyn.json"
GOLDEN_FRESH = ROOT / "tests" / "golden" / "c2_beyn_fresh.json"


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


METRIC = "eigenvalues/s at <=1e-10 rel err vs the FP64 oracle (mixed FP32 LU + FP64-accurate refinement), Beyn CFIE Kress star"


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


def oracle_eigenvalues(regrow="extend"):
    """All eigenvalues of B from the oracle's FP64 disk with the same probes and
    regrowth policy ("extend": the library's; "fresh": the reference's)."""
    g = json.loads((GOLDEN if regrow == "extend" else GOLDEN_FRESH).read_text())
    return np.array([complex(*x) for x in g["eigenvalues"]])


def accuracy(lam, oracle_all):
    """Errors of the selected eigenvalues against the oracle's, and the oracle's
    selected eigenvalues that found no partner within TOL_EIG."""
    sel = select(lam)
    e = match(sel, oracle_all)
    ref = select(oracle_all)
    missing = int(sum(1 for x in ref if len(sel) == 0 or np.min(np.abs(sel - x)) / abs(x) > TOL_EIG))
    return sel, e, missing


def run_step(qb, sol, pts, ws, mixed, rng_seed=SEED, with_geometry=False, cheb=None, nb=0):
    t0 = time.perf_counter()
    if with_geometry:
        ws = qb.Workspace(sol, pts)
    lam, info = qb.solve(sol, pts, K0 + 0j, RADIUS, nq=NQ, r=L_PROBES, svd_tol=SVD_TOL,
                         rng=np.random.default_rng(rng_seed), mixed=mixed, ws=ws, return_info=True, cheb=cheb, nb=nb)
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


def cpu_disk(steps, warmup, threads=None):
    """The reference's CPU Beyn path restated on the host cores (oracle/cpu.py):
    the panels tuned once (chebyshev_params rule, tol 1e-13; plan_s, not
    timed), `warmup` untimed whole disks, then `steps` timed whole disks, each
    the 48 contour nodes (table fit, assembly, LAPACK LU, solves of the r and
    the fresh 2r probe blocks) and the disk's moments, SVD, B and eig(B). The
    eigenvalue count is that of the last disk: eigenvalues inside the disk
    within TOL_EIG of the oracle fixture of the reference's regrowth policy."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import beyn as OB, cpu as OCPU, geometry as OG
    threads = threads or os.cpu_count()
    OCPU.build()
    pts, _ = OG.points_with_n("cfie_kress", OG.star(0.2, 5), N_NODES, K0)
    g = OCPU.Geometry(pts)
    zj, _ = OB.contour(K0 + 0j, RADIUS, NQ)
    with ThreadPoolExecutor(threads) as pool:
        t0 = time.perf_counter()
        prm = OCPU.chebyshev_params(g, zj, tol=CHEB_TOL, pool=pool)
        plan_s = time.perf_counter() - t0
    times, node_s, finish_s = [], [], []
    lam, rk, r_used = None, 0, 0
    for s in range(warmup + steps):
        cb = OCPU.BeynCPU(pts, K0, RADIUS, NQ, L_PROBES, SVD_TOL, SEED, prm[:4], threads)
        try:
            t0 = time.perf_counter()
            for j in range(NQ):
                cb.node(j)
            t1 = time.perf_counter()
            lam, rk, r_used = cb.finish()
            t2 = time.perf_counter()
        finally:
            cb.close()
        if s >= warmup:
            times.append(t2 - t0)
            node_s.append((t1 - t0) / NQ)
            finish_s.append(t2 - t1)
    sel, e, missing = accuracy(lam, oracle_eigenvalues("fresh"))
    n_eig = int(np.count_nonzero(e <= TOL_EIG))
    t_disk = float(np.mean(times))
    return dict(value=n_eig / t_disk, n_eig=n_eig, t_disk=t_disk, t_node=float(np.mean(node_s)),
                finish_s=float(np.mean(finish_s)), plan_s=plan_s, cheb=[int(x) for x in prm[:4]], cores=threads, rk=rk,
                r=r_used, max_rel_err_vs_oracle=float(e.max()) if len(e) else None, missing=missing, steps=steps,
                warmup=warmup, region_s=float(np.sum(times)))


def cpu_sample_text(c):
    return (f"{c['steps']} whole disk(s) timed after {c['warmup']} untimed ({c['region_s']:.1f} s): per disk "
            f"{NQ} contour nodes (Chebyshev tables {c['cheb']} fitted to AMOS values, C assembly on {c['cores']} "
            f"threads, LAPACK LU and solves of {L_PROBES} + {2 * L_PROBES} probes; {c['t_node']:.2f} s per node) and "
            f"the moments/SVD/B/eig ({c['finish_s']:.2f} s); {c['n_eig']} eigenvalues within 1e-10 of the oracle; "
            f"panel tuning {c['plan_s']:.1f} s not counted")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serial", action="store_true",
                    help="time the disks one solve() call after another instead of through solve_pipelined "
                         "(host SVD / eig of a disk overlapped with the device work of the next)")
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--cpu-steps", type=int, default=1, help="timed whole disks of the cpu_baseline leg")
    ap.add_argument("--workload", default="beyn", choices=["beyn", "ebim", "c1", "c3", "serve"],
                    help="beyn: the headline Beyn disk (default); ebim: the EBIM eigen step at one k; c1: the "
                         "sigma_min sweep of the unit circle and refine_minima; c3: 32 batched disks of the "
                         "desymmetrised stadium; serve: the served mixed request stream")
    ap.add_argument("--no-extras", action="store_true",
                    help="beyn: leave out the bounded samples of the other configurations (other_configs)")
    ap.add_argument("--requests", type=int, default=2000, help="serve: requests of the stream")
    ap.add_argument("--rate", type=float, default=20.0, help="serve: Poisson arrival rate (requests/s)")
    ap.add_argument("--nmin", type=int, default=1024, help="serve: smallest N")
    ap.add_argument("--nmax", type=int, default=8192, help="serve: largest N")
    ap.add_argument("--nk", type=int, default=64, help="serve: wavenumbers of a sweep request")
    ap.add_argument("--max-sweeps", type=int, default=1, help="serve: sweeps running at once")
    ap.add_argument("--mix", default="0.6,0.3,0.1", help="serve: fractions of Beyn, EBIM and sweep requests")
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
    if args.workload in ("c1", "c3", "serve"):
        if rank != 0:
            return
        return other_workload(args)
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
    oracle_all = oracle_eigenvalues()
    oracle_sel = select(oracle_all)

    # panels tuned once to CHEB_TOL on the device: of the degrees 5..15, the panel layout of the lowest
    # table-plus-series cost whose H0, H1, J0, J1 all stay within CHEB_TOL (the reference's tuner grows
    # its default layout to the same tolerance; both reproduce the oracle's eigenvalues to ~2e-13)
    zref = K0 + RADIUS * np.exp(2j * math.pi * np.arange(NQ) / NQ)
    t0 = time.perf_counter()
    cheb = tuple(int(x) for x in qb.chebyshev_params_min_cost(sol, pts, zref, ws=ws, tol=CHEB_TOL)[:4])
    plan_s = time.perf_counter() - t0
    # LU plan of the mixed step (panel width, outer-block depth, stream parts) chosen by timing this workload
    # on the path the region times: the pipelined driver (4 disks per trial), or serial solve() calls
    tuned = qb.autotune.tune_beyn(sol, pts, ws, K0 + 0j, RADIUS, NQ, L_PROBES, mixed=True, cheb=cheb,
                                  svd_tol=SVD_TOL, seed=SEED, pipelined=0 if args.serial else 4)
    nb = tuned["nb"]

    # plain FP64 form (the drop-in), timed beside the mixed one
    lam64, info64, _ = run_step(qb, sol, pts, ws, mixed=False, cheb=cheb)
    plain_times = []
    for _ in range(max(1, args.plain_steps)):
        lam64, info64, dt = run_step(qb, sol, pts, ws, mixed=False, cheb=cheb)
        plain_times.append(dt)
    t_plain = float(np.median(plain_times))
    _, e64, miss64 = accuracy(lam64, oracle_all)
    plain_ok = int(np.count_nonzero(e64 <= TOL_EIG))

    for _ in range(args.warmup):
        run_step(qb, sol, pts, ws, mixed=True, cheb=cheb, nb=nb)
    _lib.load().qbg_device_sync()
    replica_barrier(world)
    clk = ClockSampler()
    clk.start()
    times, counts, errs, stats, missing = [], [], [], [], []
    launches0 = qb.launch_count()
    t_region0 = time.perf_counter()
    if args.serial:
        for s in range(args.steps):
            lam, info, dt = run_step(qb, sol, pts, ws, mixed=True, cheb=cheb, nb=nb)
            sel, e, miss = accuracy(lam, oracle_all)
            counts.append(int(np.count_nonzero(e <= TOL_EIG)))
            errs.append(e)
            missing.append(miss)
            times.append(dt)
            stats.append(info["stats"])
    else:
        # the same disk every step, each with the probes of run_step (a fresh generator seeded SEED)
        lams, pinfo = qb.solve_pipelined(sol, pts, [K0 + 0j] * args.steps, RADIUS, nq=NQ, r=L_PROBES,
                                         svd_tol=SVD_TOL, rngs=[np.random.default_rng(SEED)
                                                                for _ in range(args.steps)],
                                         mixed=True, ws=ws, return_info=True, cheb=cheb, nb=nb)
        for lam, st in zip(lams, pinfo["stats"]):
            sel, e, miss = accuracy(lam, oracle_all)
            counts.append(int(np.count_nonzero(e <= TOL_EIG)))
            errs.append(e)
            missing.append(miss)
            stats.append([st])
        info = {"r": pinfo["r"][-1], "host_ms": {"finish_per_disk": float(np.mean(pinfo["host_ms"])),
                                                 "device_calls_per_disk": float(np.mean(pinfo["device_call_ms"])),
                                                 **pinfo["call_split_ms"]}}
    _lib.load().qbg_device_sync()
    t_region = time.perf_counter() - t_region0
    if not args.serial:
        times = [t_region / args.steps] * args.steps
    gpu_launches = qb.launch_count() - launches0
    replica_barrier(world)
    clocks = clk.stop()
    # replicas: every rank ran the same disk on its own GPU; the job's time is the slowest rank's
    t_region_max, eig_total = replica_reduce(world, t_region, float(sum(counts)))
    # end to end through the public API including the geometry upload
    e2e_times, e2e_counts = [], []
    if args.serial:
        for _ in range(max(1, min(args.steps, 3))):
            lam_e, _, dt = run_step(qb, sol, pts, None, mixed=True, with_geometry=True, cheb=cheb, nb=nb)
            e2e_times.append(dt)
            e2e_counts.append(int(np.count_nonzero(accuracy(lam_e, oracle_all)[1] <= TOL_EIG)))
    else:
        t_e = time.perf_counter()
        ws_e = qb.Workspace(sol, pts)
        lams_e = qb.solve_pipelined(sol, pts, [K0 + 0j] * args.steps, RADIUS, nq=NQ, r=L_PROBES, svd_tol=SVD_TOL,
                                    rngs=[np.random.default_rng(SEED) for _ in range(args.steps)], mixed=True,
                                    ws=ws_e, cheb=cheb, nb=nb)
        ws_e.close()
        dt = (time.perf_counter() - t_e) / args.steps
        for lam_e in lams_e:
            e2e_times.append(dt)
            e2e_counts.append(int(np.count_nonzero(accuracy(lam_e, oracle_all)[1] <= TOL_EIG)))
    # the same disks one synchronous solve() after another, for comparison
    # device phases of a disk with the GPU to itself (the pipelined disks share it): the roofline's
    # factor time and phases_ms come from these serial steps
    serial_times, serial_stats = [], []
    if not args.serial:
        for _ in range(max(1, min(args.steps, 3))):
            _, sinfo, sdt = run_step(qb, sol, pts, ws, mixed=True, cheb=cheb, nb=nb)
            serial_times.append(sdt)
            serial_stats.append(sinfo["stats"])
    # FP32 form (FP32 kernel values): reported beside, with its own accuracy
    run_step(qb, sol, pts, ws, mixed="fp32", cheb=cheb)
    lam32, info32, t32 = run_step(qb, sol, pts, ws, mixed="fp32", cheb=cheb)
    _, e32, _ = accuracy(lam32, oracle_all)
    fp32_form = {"ms_per_step": t32 * 1e3, "eigenvalues_inside": int(len(e32)),
                 "eigenvalues_le_1e-10": int(np.count_nonzero(e32 <= TOL_EIG)),
                 "max_rel_err_vs_oracle": float(e32.max()) if len(e32) else None}

    t_step = t_region_max / args.steps
    n_eig = float(np.mean(counts))
    value = eig_total / t_region_max  # whole job: eigenvalues of all replicas / slowest rank's time
    r_final = info["r"]
    N = ws.dim
    h2d = 8 * 8 * N + 16 * N * (L_PROBES + (r_final if r_final != L_PROBES else 0))
    d2h = 2 * 16 * N * (L_PROBES + (r_final if r_final != L_PROBES else 0))
    hbm, bf16, peak_kind = _peaks()
    pstats = serial_stats if serial_stats else stats  # phases of a disk alone on the device
    st_last = pstats[-1]
    ms_factor = float(np.mean([s[0]["ms_factor"] for s in pstats]))
    ms_assemble = float(np.mean([s[0]["ms_assemble"] for s in pstats]))
    # dominant work of the step: the FP32 LU of the 48 operators (panels on CUDA cores,
    # trailing updates on tcgen05 with 3xTF32), timed by CUDA events around the factor phase
    lu_flops = NQ * (8.0 / 3.0) * N ** 3
    lu_achieved = lu_flops / (ms_factor * 1e-3) / 1e12
    # tensor-core residual: HBM-bound (digit planes of T and X, V, R per launch)
    res_ms = sum(s["ms_residual"] for run in pstats for s in run)
    res_n = sum(s["n_residual"] for run in pstats for s in run)
    res_launch_ms = res_ms / max(res_n, 1)
    lp = ((L_PROBES + 31) // 32) * 32
    res_alg_bytes = (7 * N * 2 * N * 2 + 7 * 2 * lp * 2 * N * 2 + 2 * 16 * N * L_PROBES) * NQ
    # assembly: HBM floor of the written operators (complex64 hi + lo = 16 B per entry)
    asm_bytes = 16.0 * N * N * NQ
    e_last = errs[-1]
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
        "config": dict(workload_config(), r_final=r_final, cheb_panels=list(cheb), cheb_tol=CHEB_TOL,
                       timing=("wall clock of the synchronous API calls between device synchronizations (the step "
                               "ends with the host SVD and eigvals)" if args.serial else
                               "wall clock of one solve_pipelined call over `steps` disks (two disks in flight on "
                               "the device; each disk's host QR, SVDs and eigvals beside the next disk's device "
                               "work; the last disk's are inside the region)") +
                              "; device phases in phases_ms are CUDA events of a disk alone on the device"),
        "serial_ms_per_step": (float(np.median(serial_times)) * 1e3 if serial_times else None),
        "plan_s": plan_s,
        "lu_plan": {"nb": nb, "outer": tuned["outer"], "parts": tuned["parts"], "cluster": tuned["cluster"],
                    "tune_s": tuned["tune_s"],
                    "tried": [[t["nb"], t["outer"], t["parts"], t["cluster"], round(t["ms"], 1)]
                              for t in tuned["table"]]},
        "eigenvalues_per_step": n_eig,
        "oracle_eigenvalues_in_disk": int(len(oracle_sel)),
        "oracle_eigenvalues_missed": int(max(missing)),
        "max_rel_err_vs_oracle": float(max(float(e.max()) for e in errs)),
        "eig_rel_err_vs_oracle": [float("%.3g" % x) for x in e_last],
        "plain_fp64": {"value": plain_ok / t_plain, "ms_per_step": t_plain * 1e3, "eigenvalues_le_1e-10": plain_ok,
                       "eigenvalues_le_1e-12": int(np.count_nonzero(e64 <= 1e-12)),
                       "max_rel_err_vs_oracle": float(e64.max()) if len(e64) else None,
                       "oracle_eigenvalues_missed": miss64},
        "speedup_vs_plain": (n_eig / t_step) / (plain_ok / t_plain) if plain_ok else None,
        "phases_ms_pipelined": ({"assemble": float(np.mean([s[0]["ms_assemble"] for s in stats])),
                                 "factor": float(np.mean([s[0]["ms_factor"] for s in stats])),
                                 "solve_refine": float(np.mean([sum(x["ms_solve"] for x in s) for s in stats]))}
                                if serial_stats else None),
        "phases_ms": {"assemble": ms_assemble, "factor": ms_factor,
                      "solve_refine": sum(s["ms_solve"] for s in st_last)},
        "host_ms": {k: float("%.3g" % v) for k, v in info["host_ms"].items()},
        "refine_sweeps": [s["refine_sweeps"] for s in st_last],
        "refine_history": [[float("%.3g" % v) for v in s["refine_history"]] for s in st_last],
        "plain_phases_ms": {"assemble": info64["stats"][0]["ms_assemble"], "factor": info64["stats"][0]["ms_factor"],
                            "solve": sum(s["ms_solve"] for s in info64["stats"])},
        "fp32_form": fp32_form,
        "e2e": {"value": float(np.mean(e2e_counts)) / float(np.mean(e2e_times)), "unit": "eigenvalues/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "tensor", "achieved": lu_achieved, "peak": bf16, "unit": "TFLOP/s",
                     "frac": lu_achieved / bf16, "traffic": None,
                     "kernel": "LU factor phase of the 48 operators, one disk alone on the device: "
                               "k_getrf_panel_smem (FP32 panels, CUDA cores) + k_tc_cgemm_pkw trailing updates and "
                               "k_tc_cgemm in-block products (tcgen05, 3xTF32)",
                     "peak_kind": peak_kind + " bf16 dense (the TF32 tensor rate is half of it and 3xTF32 issues three "
                                              "MMAs per product)",
                     "algorithmic_flops": lu_flops, "ms": ms_factor},
        "phase_rooflines": {
            "assembly": {"bound": "fp32 alu / hbm", "ms": ms_assemble, "bytes_written": asm_bytes,
                         "achieved_gbs": asm_bytes / (ms_assemble * 1e-3) / 1e9, "peak_gbs": hbm,
                         "frac_hbm": asm_bytes / (ms_assemble * 1e-3) / 1e9 / hbm},
            "k_resid_tc": {"bound": "hbm", "launch_ms": res_launch_ms, "launches_per_step": res_n / max(len(pstats), 1),
                           "algorithmic_bytes": res_alg_bytes,
                           "achieved_gbs": res_alg_bytes / (res_launch_ms * 1e-3) / 1e9 if res_n else None,
                           "peak_gbs": hbm,
                           "frac": res_alg_bytes / (res_launch_ms * 1e-3) / 1e9 / hbm if res_n else None}},
        "clocks": clocks,
        "gpu_launches": gpu_launches,
        "gpu_launches_per_step": gpu_launches / max(args.steps, 1),
    }
    if world > 1:
        line["config"]["parallelism"] = f"replicas{world}"
    if not args.no_extras and rank == 0 and world == 1:
        ws.close()
        qb.autotune.set_lu_plan(cluster=-1)  # the panel form tuned for C2's batch back to automatic
        line["other_configs"] = {
            "c1": c1_sweep(qb),
            "c3": c3_disks(qb, repeat=2),
            "c4_sample": serve_stream(qb, requests=60, rate=20.0, nmin=1024, nmax=2048, nk=16, max_sweeps=1),
            "note": "bounded samples run after the timed region: C1 and C3 at their full configurations, C4 as the "
                    "first 60 requests of its seeded stream with N capped at 2048 and 16-k sweeps (FP64 sweeps at "
                    "N = 8192 take minutes per request on this part); bench.py --workload serve runs the full "
                    "stream"}
    if not args.no_cpu_baseline and rank == 0 and world == 1:
        c = cpu_disk(max(1, args.cpu_steps), 0)
        line["cpu_baseline"] = {"value": c["value"], "unit": "eigenvalues/s", "cores": c["cores"], "kind": "port",
                                "sample": cpu_sample_text(c), "max_rel_err_vs_oracle": c["max_rel_err_vs_oracle"]}
    if rank == 0:
        print(json.dumps(line))


# ---------------------------------------------------------------------------
# the other configurations: C1 (sweep), C3 (batched disks), C4 (served stream)
# ---------------------------------------------------------------------------
GOLDEN_C1 = ROOT / "tests" / "golden" / "c1_sweep.json"
CIRCLE_EIGS = ROOT / "tests" / "golden" / "circle_eigs.json"


def c1_sweep(qb):
    """C1: the unit circle, DLP Kress with N = 512 at k = 42 (pts_scaling_factor
    of the golden fixture), sigma_min(A(k)) at 200 k in [40, 42], then
    refine_minima (three discretisation levels, Newton on lambda_min(A^H A)).
    Errors: sigma_min against the oracle's LAPACK values (c1_sweep.json), the
    refined roots against the J_m zeros (circle_eigs.json)."""
    g = json.loads(GOLDEN_C1.read_text())
    ks, so = np.array(g["ks"]), np.array(g["sigma"])
    b = qb.make_circle(1.0)
    sol = qb.DLP_kress(g["pts_scaling_factor"], b)
    qb.k_sweep(sol, b, ks[:4])  # warm-up (workspace and kernels)
    t0 = time.perf_counter()
    sig = qb.k_sweep(sol, b, ks)
    t1 = time.perf_counter()
    kr, tr, _ = qb.refine_minima(sol, b, ks, sig)
    t2 = time.perf_counter()
    zeros = np.array([r["k"] for r in json.loads(CIRCLE_EIGS.read_text())["ranges"]["40_42"]])
    root_err = [float(np.min(np.abs(zeros - k))) for k in kr]
    return {"workload": "c1_dlp_kress_circle_N512_200k_40_42", "sweep_s": t1 - t0, "refine_s": t2 - t1,
            "k_per_s": len(ks) / (t1 - t0), "minima": len(kr),
            "sigma_max_rel_err_vs_oracle": float(np.max(np.abs(sig - so) / so)),
            "root_max_abs_err_vs_jm_zeros": max(root_err) if root_err else None}


def c3_disks(qb, repeat=2, n=4096, ndisk=32, nq=48, L=96):
    """C3: DLP Kress on the full stadium (radius 1, straight length 2)
    desymmetrised by XYReflection(-1, -1): N = 4096 full nodes (m = 1024), 32
    disks of radius 0.5 centred at 300.5 ... 331.5, 48 nodes each, L = 96
    seeded probes, Chebyshev panels at tol 1e-12 (the library's cost-aware
    tuner), mixed form; all 1536 operators assembled in one launch and
    factored as one batch. The first batch allocates (cold), the later ones
    reuse the library's cached blocks (warm). Eigenvalues: inside each disk
    with |Im| < 1e-3."""
    b = qb.make_full_stadium(1.0, 1.0)
    sol = qb.DLP_kress_global_corners(1.0, b, symmetry=qb.XYReflection(-1, -1))
    k0s = 300.5 + np.arange(ndisk)
    pts, sol = qb.points_with_n(sol, b, n, float(k0s[-1] + 0.5))
    ws = qb.Workspace(sol, pts)
    t0 = time.perf_counter()
    zref = k0s[-1] + 0.5 * np.exp(2j * math.pi * np.arange(nq) / nq)
    cheb = qb.chebyshev_params_min_cost(sol, pts, zref, ws=ws, tol=1e-12, entries=float(ws.dim) ** 2 * ndisk * nq,
                                        terms_per_entry=4.0, tables_per_call=ndisk * nq)[:4]
    plan_s = time.perf_counter() - t0
    times, info, lams = [], None, None
    for _ in range(max(1, repeat)):
        ts = time.perf_counter()
        lams, info = qb.solve_disks(sol, pts, k0s, 0.5, nq=nq, r=L, svd_tol=1e-10, rng=np.random.default_rng(3),
                                    mixed=True, ws=ws, return_info=True, cheb=cheb)
        times.append(time.perf_counter() - ts)
    m = int(ws.dim)
    ws.close()
    n_in = sum(int(np.count_nonzero((np.abs(l - k) < 0.5) & (np.abs(l.imag) < 1e-3))) for l, k in zip(lams, k0s))
    st = info["stats"]
    warm = min(times[1:]) if len(times) > 1 else times[0]
    return {"workload": "c3_dlp_kress_quarter_stadium_N4096_32disks_nq48_L96", "m": m, "operators": ndisk * nq,
            "plan_s": plan_s, "batch_s_cold": times[0], "batch_s_warm": warm, "eigenvalues": n_in,
            "eigenvalues_per_s_warm": n_in / warm, "ms_assemble": st[0]["ms_assemble"],
            "ms_factor": st[0]["ms_factor"], "ms_solve": [s["ms_solve"] for s in st],
            "host_ms": {k: float("%.3g" % v) for k, v in info.get("host_ms", {}).items()}}


def make_stream(qb, requests, rate, nmin, nmax, kmin, kmax, L, nk, seed, mix):
    """The seeded request stream of C4: Poisson arrivals; geometry uniform over
    {unit circle with an off-centre hole of radius 0.2 (CFIE Kress), full
    stadium (DLP, smooth composite), half-ellipse-cap mushroom (DLP,
    corner-graded, kressq = 4), star r = 1 + 0.2 cos 5 theta (CFIE Kress)}; N
    log-uniform in [nmin, nmax] (rounded by the node-count rule); k uniform in
    [kmin, kmax]; request kinds by `mix` (Beyn disk of radius 0.5 with 32..64
    contour nodes and L probes; EBIM at one k; sigma_min sweep of nk
    wavenumbers). Discretisations are built and uploaded before the clock."""
    rng = np.random.default_rng(seed)
    geoms = [("hole", qb.make_circle_with_hole(1.0, (0.3, 0.1, 0.2)), qb.CFIE_kress),
             ("stadium", qb.make_full_stadium(1.0, 1.0), qb.DLP_kress_global_corners),
             ("mushroom", qb.make_full_ellipse_mushroom(), qb.DLP_kress_global_corners),
             ("star", qb.make_star(0.2, 5), qb.CFIE_kress)]
    reqs = []
    t = 0.0
    for _ in range(requests):
        t += rng.exponential(1.0 / rate)
        gname, bil, cls = geoms[int(rng.integers(0, len(geoms)))]
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        k = float(rng.uniform(kmin, kmax))
        u = rng.uniform()
        kind = "beyn" if u < mix[0] else ("ebim" if u < mix[0] + mix[1] else "sweep")
        sol = cls(1.0, bil)
        pts, sol = qb.points_with_n(sol, bil, n, k)
        ws = qb.Workspace(sol, pts)
        r = dict(t=t, kind=kind, geom=gname, n=ws.dim, k=k, ws=ws)
        if kind == "beyn":
            r["nq"] = int(rng.integers(32, 65))
            r["V"] = qb.probe_matrix(ws.dim, L, rng)
        elif kind == "sweep":
            r["ks"] = k + 0.01 * np.arange(nk)
        reqs.append(r)
    return reqs


def serve_stream(qb, requests=2000, rate=20.0, nmin=1024, nmax=8192, kmin=50.0, kmax=800.0, L=32, nk=64,
                 budget_gb=150.0, workers=4, max_batch=8, max_sweeps=1, seed=4, mix=(0.6, 0.3, 0.1)):
    """C4 through the request server (qbgpu.Server: device-resident state,
    HBM-budget admission, Beyn requests on the same geometry merged into one
    batch, priority streams): requests are submitted at their arrival times
    and latency = arrival -> result on the host (submission, queue, device
    work, copies back and the host part of a Beyn request). Reports p50/p99
    overall and per kind, with the queue / run / host split."""
    import threading
    from concurrent.futures import ThreadPoolExecutor
    reqs = make_stream(qb, requests, rate, nmin, nmax, kmin, kmax, L, nk, seed, mix)
    lat, info = {}, {}
    lock = threading.Lock()
    with qb.Server(hbm_budget=int(budget_gb * 2 ** 30), workers=workers, max_batch=max_batch,
                   max_sweeps=max_sweeps) as srv, ThreadPoolExecutor(max_workers=64) as pool:
        t0 = time.perf_counter()

        def finish(i, h, t_arr):
            res = srv.wait(h)
            done = time.perf_counter()
            nl = 0
            if reqs[i]["kind"] == "beyn":
                lam = res["lam"]
                nl = int(np.count_nonzero((np.abs(lam - reqs[i]["k"]) < 0.5) & (np.abs(lam.imag) < 1e-3)))
            with lock:
                lat[i] = (done - t_arr) * 1e3
                info[i] = dict(batched=res["batched"], queue_ms=res["queue_ms"], run_ms=res["run_ms"], eig=nl,
                               lag_ms=(h.t_submit - t_arr) * 1e3, wait_ms=(done - h.t_submit) * 1e3)

        futs = []
        for i, r in enumerate(reqs):
            now = time.perf_counter() - t0
            if r["t"] > now:
                time.sleep(r["t"] - now)
            t_arr = t0 + r["t"]
            if r["kind"] == "beyn":
                h = srv.submit_beyn(r["ws"], r["k"], 0.5, r["nq"], r["V"], mixed=True)
            elif r["kind"] == "ebim":
                h = srv.submit_ebim(r["ws"], r["k"])
            else:
                h = srv.submit_sweep(r["ws"], r["ks"])
            futs.append(pool.submit(finish, i, h, t_arr))
        for f in futs:
            f.result()
        wall = time.perf_counter() - t0
    for r in reqs:
        r["ws"].close()
    Lm = np.array([lat[i] for i in range(len(reqs))])
    per = {}
    for kind in ("beyn", "ebim", "sweep"):
        idx = [i for i in range(len(reqs)) if reqs[i]["kind"] == kind]
        if not idx:
            continue
        v = np.array([lat[i] for i in idx])
        qv = np.array([info[i]["queue_ms"] for i in idx])
        rv = np.array([info[i]["run_ms"] for i in idx])
        hv = np.array([info[i]["wait_ms"] - info[i]["queue_ms"] - info[i]["run_ms"] for i in idx])
        per[kind] = dict(count=len(idx), p50_ms=float(np.percentile(v, 50)), p99_ms=float(np.percentile(v, 99)),
                         queue_p50_ms=float(np.percentile(qv, 50)), run_p50_ms=float(np.percentile(rv, 50)),
                         host_p50_ms=float(np.percentile(hv, 50)),
                         n_range=[int(min(reqs[i]["n"] for i in idx)), int(max(reqs[i]["n"] for i in idx))])
    eig = sum(info[i]["eig"] for i in info)
    return {"workload": "c4_served_stream", "requests": len(reqs), "rate_per_s": rate, "wall_s": wall,
            "p50_ms": float(np.percentile(Lm, 50)), "p99_ms": float(np.percentile(Lm, 99)),
            "throughput_req_per_s": len(reqs) / wall, "eigenvalues": eig, "eigenvalues_per_s": eig / wall,
            "per_kind": per, "beyn_batched_max": max([info[i]["batched"] for i in info] + [1]),
            "config": dict(nmin=nmin, nmax=nmax, kmin=kmin, kmax=kmax, L=L, nk=nk, budget_gb=budget_gb,
                           workers=workers, max_batch=max_batch, max_sweeps=max_sweeps, seed=seed, mix=list(mix))}


def other_workload(args):
    """--workload c1 | c3 | serve: one configuration in its own JSON line."""
    import build_qbgpu as B
    B.build()
    import qbgpu as qb
    clk = ClockSampler()
    clk.start()
    launches0 = qb.launch_count()
    if args.workload == "c1":
        r = c1_sweep(qb)
        metric, value, unit = "sigma_min evaluations/s, C1 sweep (DLP Kress circle, N = 512, 200 k)", r["k_per_s"], "k/s"
        ms = r["sweep_s"] * 1e3
    elif args.workload == "c3":
        r = c3_disks(qb, repeat=max(2, args.steps))
        metric, value, unit = "eigenvalues/s, C3 batched disks (warm batch)", r["eigenvalues_per_s_warm"], "eigenvalues/s"
        ms = r["batch_s_warm"] * 1e3
    else:
        r = serve_stream(qb, requests=args.requests, rate=args.rate, nmin=args.nmin, nmax=args.nmax, nk=args.nk,
                         max_sweeps=args.max_sweeps, mix=tuple(float(x) for x in args.mix.split(",")))
        metric, value, unit = "served requests/s (p50/p99 latency beside), C4 stream", r["throughput_req_per_s"], "req/s"
        ms = r["wall_s"] * 1e3
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64+c128",
            "data": "synthetic", "config": {"workload": r["workload"]}, "result": r,
            "gpu_launches": qb.launch_count() - launches0, "clocks": clk.stop()}
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
    from oracle import assembly as OA, ebim as OE, geometry as OG
    pts, _ = OG.points_with_n("cfie_kress", OG.star(0.2, 5), N_NODES, K0)
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
    """--impl reference: the reference's CPU Beyn path restated on the host
    cores (oracle/cpu.py, see cpu_disk), one whole disk per timed step. A disk
    takes ~18 s on the 16 host cores, so at most 3 timed disks after at most
    one untimed one are run, whatever --steps / --warmup ask (steps and
    warmup in the line are the numbers run)."""
    steps, warmup = max(1, min(args.steps, 3)), min(args.warmup, 1)
    c = cpu_disk(steps, warmup)
    print(json.dumps({"impl": "reference", "metric": METRIC, "value": c["value"], "unit": "eigenvalues/s",
                      "n_gpus": 1, "steps": steps, "warmup": warmup, "steps_requested": args.steps,
                      "warmup_requested": args.warmup, "ms_per_step": c["t_disk"] * 1e3,
                      "higher_is_better": True, "dtype": "c128", "data": "synthetic",
                      "config": dict(workload_config(), cheb_panels=c["cheb"], cheb_tol=CHEB_TOL,
                                     timing="host wall clock of each whole disk (48 node steps, moments, SVD, B, "
                                            "eig); value = eigenvalues per disk / mean disk time"),
                      "disk_s": c["t_disk"], "plan_s": c["plan_s"],
                      "eigenvalues_per_disk": c["n_eig"], "max_rel_err_vs_oracle": c["max_rel_err_vs_oracle"],
                      "rk": c["rk"], "r_final": c["r"],
                      "cpu_baseline": {"value": c["value"], "unit": "eigenvalues/s", "cores": c["cores"], "kind": "port",
                                       "sample": cpu_sample_text(c)},
                      "e2e": {"value": c["value"], "unit": "eigenvalues/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}))


if __name__ == "__main__":
    main()
