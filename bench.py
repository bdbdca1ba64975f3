"""Benchmark of the Moebius domain-wall Dslash hot path on GB300.

Workload (default): Moebius DWF, 16^4 x Ls=16, b=1.5, c=0.5, M5=1.8, mf=0.01, gauge
U = exp(i 0.5 H) (seeded), antiperiodic time, FP32.  One step = DhopEO + DhopOE on
Gaussian spinors.  The timed loop rotates over 4 independent (in, out) sets
(4 x 4 half fields x 50 MB + links, larger than the 129 MB L2), so every kernel reads
inputs that are not L2-resident.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  `value` = algorithmic GB/s of the step (228 B per output 5D site
per Dhop in FP32: 96 in + 96 out + 8 links x 72 B / Ls), inputs resident in HBM;
`e2e` = the same metric through the C ABI with pinned host buffers, the host<->device
copies of each step's input and output inside the timed region: FP32 canonical host fields
through the transfer queue (copies of consecutive steps overlap), and beside it the
blocking FP64 import / Dhop / export path.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

DIMS = (16, 16, 16, 16)
LS = 16
MF, M5, B, C, EPS = 0.01, 1.8, 1.5, 0.5, 0.5
METRIC = "DWF Dhop GB/s vs HBM peak"
UNIT = "GB/s"


def bytes_per_site(prec: int, Ls: int) -> float:
    spin = 96 if prec == 1 else 192
    link = 72 if prec == 1 else 144
    return 2 * spin + 8 * link / Ls


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(name: str):
    """dram bytes per launch from the committed ncu summary (line `traffic_bytes_per_launch: N`)."""
    f = ROOT / "profiles" / name
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                parts = [x.strip() for x in out.stdout.strip().split(",")]
                if len(parts) >= 6:
                    self.samples.append(parts)
            except Exception:
                pass
            self._stop.wait(0.05)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[2 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist


def dist_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def dist_barrier(dist):
    if dist is not None:
        dist.barrier()


# ---------------------------------------------------------------------------------------
ANTIPERIODIC_T = [1.0, 0.0, 1.0, 0.0, 1.0, 0.0, -1.0, 0.0]
CPU_KERNEL = ("Grid's CPU hopping-term algorithm (half-spinor projection, SU(3) x two-spinor, "
              "reconstruction; OpenMP over 4D sites, Ls vectorised), FP32, oracle/cpu_dhop.cpp")


def cpu_dhop_steps(budget_s: float, max_steps: int, seed_gauge=1234):
    """DhopEO + DhopOE steps of the full 16^4 x 16 workload on the host cores with the
    oracle's half-spinor CPU Dhop, inputs from the oracle's restatement of the seeded
    generator (the CUDA library is not loaded): as many steps as fit in budget_s, at most
    max_steps.  Returns (GB/s on the workload's algorithmic bytes, steps, seconds, threads)."""
    from oracle import oracle as o
    threads = o.max_threads()
    U = o.random_gauge(DIMS, EPS, seed_gauge)
    nh = int(np.prod(DIMS)) // 2 * LS
    h = o.HalfSpinorDhop(DIMS, LS, U, ANTIPERIODIC_T)
    h.set(1, o.random_gaussian(nh * 12, 1))
    h.set(0, o.random_gaussian(nh * 12, 2))
    h.dhop(0)  # warm
    h.dhop(1)
    n, t0 = 0, time.perf_counter()
    while n < max_steps:
        h.dhop(0)
        h.dhop(1)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return 2 * n * nh * bytes_per_site(1, LS) / dt / 1e9, n, dt, threads


def cpu_baseline_oracle(budget_s=12.0):
    gbs, n, dt, threads = cpu_dhop_steps(budget_s, 1 << 30)
    return {"value": gbs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} DhopEO+DhopOE pairs of the full 16^4x16 FP32 workload in {dt:.1f} s: {CPU_KERNEL}"}


def run_reference(args, ws, rank):
    """--impl reference: Grid's CPU algorithm for the path (the oracle's half-spinor Dhop;
    Grid itself cannot be built here) on the same config and metric.  Imports only oracle/."""
    if rank != 0:
        return
    # a bounded sample: at most ~60 s of timed CPU work whatever --steps asks for
    gbs, n, dt, threads = cpu_dhop_steps(60.0, max(1, args.steps))
    line = {"metric": METRIC, "value": gbs, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / n * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "mobius_dwf_16^4xLs16_dhop_eo_oe_fp32", "dims": list(DIMS), "Ls": LS,
                       "b": B, "c": C, "M5": M5, "mf": MF, "eps": EPS},
            "cpu_baseline": {"value": gbs, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{n} of {args.steps} DhopEO+DhopOE steps of the full workload timed "
                                       f"(at most ~60 s of CPU work): {CPU_KERNEL}"},
            "e2e": {"value": gbs, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args, ws, rank, local, dist):
    import grid_gb300 as g
    g.set_device(local)
    U = g.random_gauge(DIMS, EPS, 1234)
    op = g.MobiusFermion(U, DIMS, LS, MF, M5, B, C, precision=g.F32)
    nh = op.half_sites4 * LS
    NSET = 4
    # full fields: one Dhop launch computes DhopEO (odd -> even) and DhopOE (even -> odd)
    sets = []
    for k in range(NSET):
        x = op.FermionField().import_(g.random_gaussian(2 * nh * 12, 10 + k))
        sets.append((x, op.FermionField()))
    halves = []
    for k in range(NSET):
        xo = op.FermionRedBlackField(g.ODD).import_(g.random_gaussian(nh * 12, 30 + k))
        xe = op.FermionRedBlackField(g.EVEN).import_(g.random_gaussian(nh * 12, 40 + k))
        halves.append((xo, op.FermionRedBlackField(g.EVEN), xe, op.FermionRedBlackField(g.ODD)))

    def step(k):
        x, y = sets[k % NSET]
        op.Dhop(x, y, 0)

    for k in range(max(3, args.warmup)):
        step(k)
    op.sync()
    bpsite = bytes_per_site(1, LS)
    with ClockSampler(local) as clk:
        dist_barrier(dist)
        op.sync()
        op.event(0)
        for k in range(args.steps):
            step(k)
        op.event(1)
        op.sync()
        dt_ms = op.elapsed_ms(0, 1)
        # average launch time of the dominant kernel (the one-launch Dhop), same rotation,
        # and of the single-checkerboard launches
        reps = max(20, args.steps)
        full_ms = op.bench_kernel(6, [s[0] for s in sets], [s[1] for s in sets], reps)
        eo_ms = op.bench_kernel(0, [h[0] for h in halves], [h[1] for h in halves], reps)
        oe_ms = op.bench_kernel(1, [h[2] for h in halves], [h[3] for h in halves], reps)
    dt_ms = dist_max(dist, dt_ms)
    step_bytes = 2 * nh * bpsite
    value = dist_sum(dist, step_bytes * args.steps) / (dt_ms / 1e3) / 1e9 if dist else step_bytes * args.steps / (dt_ms / 1e3) / 1e9

    # ---- extra kernels of the config (Mooee, MooeeInv) ----
    m_ms = op.bench_kernel(2, [h[1] for h in halves], [h[0] for h in halves], 40)
    mi_ms = op.bench_kernel(3, [h[1] for h in halves], [h[0] for h in halves], 40)

    # ---- e2e through the C ABI with page-locked host buffers.  Headline: FP32 canonical
    # full fields (Grid's LatticeFermionF host data) through the transfer queue, so the
    # copy-in of step i+1 overlaps the copy-out of step i and the Dhop; every step still
    # moves its whole input in and its whole result out.  Beside it, the synchronous FP64
    # path (gb_field_import + gb_Dhop + gb_field_export, one blocking call each). ----
    import ctypes as Cc
    fin, fout = op.FermionField(), op.FermionField()
    q = g.TransferQueue(op)
    h32_in = [g.PinnedArray(2 * nh * 12, np.complex64) for _ in range(2)]
    h32_out = [g.PinnedArray(2 * nh * 12, np.complex64) for _ in range(2)]
    for k in range(2):
        h32_in[k].array[:] = g.random_gaussian(2 * nh * 12, 99 + k).astype(np.complex64)

    def e2e_pipelined(steps):
        for i in range(steps):
            q.import_(fin, h32_in[i % 2].array)
            assert g.lib.gb_Dhop(op.h, fin.h, fout.h, 0) == 0
            q.export(fout, h32_out[i % 2].array)
        q.wait()

    e2e_pipelined(3)
    e2e_steps = max(10, min(args.steps, 50))
    t0 = time.perf_counter()
    e2e_pipelined(e2e_steps)
    e2e_dt = dist_max(dist, (time.perf_counter() - t0) / e2e_steps)
    e2e_value = step_bytes / e2e_dt / 1e9 * (ws if dist else 1)

    host_in = g.PinnedArray(2 * nh * 12)
    host_out = g.PinnedArray(2 * nh * 12)
    host_in.array[:] = g.random_gaussian(2 * nh * 12, 99)
    pin = host_in.array.ctypes.data_as(Cc.POINTER(Cc.c_double))
    pout = host_out.array.ctypes.data_as(Cc.POINTER(Cc.c_double))
    for _ in range(2):
        g.lib.gb_field_import(fin.h, pin)
        g.lib.gb_Dhop(op.h, fin.h, fout.h, 0)
        g.lib.gb_field_export(fout.h, pout)
    sync_steps = max(3, min(args.steps, 20))
    t0 = time.perf_counter()
    for _ in range(sync_steps):
        assert g.lib.gb_field_import(fin.h, pin) == 0
        assert g.lib.gb_Dhop(op.h, fin.h, fout.h, 0) == 0
        assert g.lib.gb_field_export(fout.h, pout) == 0
    sync_dt = dist_max(dist, (time.perf_counter() - t0) / sync_steps)
    e2e_sync_value = step_bytes / sync_dt / 1e9 * (ws if dist else 1)

    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    achieved = step_bytes / (full_ms / 1e3) / 1e9
    traffic = profile_traffic("dhop_full_dwf16_fp32.txt")
    cpu = cpu_baseline_oracle() if ws == 1 else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic: seeded exp(i*0.5*H) gauge field, Gaussian spinors",
        "config": {"workload": "mobius_dwf_16^4xLs16_dhop_eo_oe_fp32", "dims": list(DIMS), "Ls": LS, "b": B, "c": C,
                   "M5": M5, "mf": MF, "eps": EPS, "boundary": "antiperiodic t",
                   "step": "DhopEO + DhopOE as one full-lattice Dhop launch",
                   "l2": "4 rotating input/output full-field sets, 800 MB total (> 129 MB L2)",
                   "parallelism": f"replicas{ws}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": "dhop_pair_kernel<float> (full Dhop, both checkerboards)",
                     "peak_source": peak_kind, "bytes_per_site": bpsite, "sites_per_launch": 2 * nh},
        "kernels_ms": {"Dhop": full_ms, "DhopEO": eo_ms, "DhopOE": oe_ms, "Mooee": m_ms, "MooeeInv": mi_ms},
        "kernels_gbs": {"Dhop": achieved, "DhopEO": nh * bpsite / (eo_ms / 1e3) / 1e9,
                        "DhopOE": nh * bpsite / (oe_ms / 1e3) / 1e9,
                        "Mooee": nh * 192 / (m_ms / 1e3) / 1e9, "MooeeInv": nh * 192 / (mi_ms / 1e3) / 1e9},
        "gflops_dhop": 1320.0 * 2 * nh / (full_ms / 1e3) / 1e9,
        "clocks": clk.summary(),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * nh * 12 * 8,
                "d2h_bytes_per_step": 2 * nh * 12 * 8, "ms_per_step": e2e_dt * 1e3,
                "path": "gb_xfer_import (H2D, canonical FP32 full field) + gb_Dhop + gb_xfer_export (D2H); "
                        "copies of consecutive steps overlap, gb_xfer_wait inside the timed region",
                "sync_fp64": {"value": e2e_sync_value, "unit": UNIT, "ms_per_step": sync_dt * 1e3,
                              "h2d_bytes_per_step": 2 * nh * 12 * 16, "d2h_bytes_per_step": 2 * nh * 12 * 16,
                              "path": "gb_field_import (canonical FP64) + gb_Dhop + gb_field_export, blocking"}},
        "gpu_launches": args.steps,
        "cpu_baseline": cpu,
    }
    if ws == 1 and not args.no_extras:
        extras = {}
        for name, fn in (("cpu_kernels_16^4xLs16", extra_cpu_kernels),
                         ("wilson_8^4_cg", lambda: extra_wilson_cg(g)),
                         ("cg_schur_24^4xLs12", lambda: extra_cg_schur(g)),
                         ("multi_rhs_wilson_32^3x64", lambda: extra_multi_rhs(g)),
                         ("serving", lambda: extra_serving(g, max_requests=args.serve_requests,
                                                           seconds=args.serve_seconds, drain=args.serve_drain))):
            t0 = time.perf_counter()
            try:
                extras[name] = fn()
            except Exception as e:  # a failed extra is reported, the headline line still prints
                extras[name] = {"error": f"{type(e).__name__}: {e}"}
            extras[name]["bench_wall_s"] = time.perf_counter() - t0
        line["extra"] = extras
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------------
# the other workloads of the path, reported beside the headline (N = 1 only)
# ---------------------------------------------------------------------------------------
def extra_cpu_kernels(budget_s=3.0):
    """The CPU side of the kernel table: the oracle's FP32 Mooee and MooeeInv (one
    checkerboard of the 16^4 x 16 workload, OpenMP over the host cores) beside the GPU
    kernels_ms, each repeated for about budget_s; GB/s on the 192 B/site algorithmic bytes."""
    from oracle import oracle as o
    threads = o.max_threads()
    o.set_threads(threads)
    ref = o.OracleOp(1, 1, DIMS, LS, [MF, M5, B, C], o.random_gauge(DIMS, EPS, 1234), ANTIPERIODIC_T)
    nh = int(np.prod(DIMS)) // 2 * LS
    x = o.random_gaussian(nh * 12, 3)
    out = {"cores": threads, "sample": "oracle/oracle.hpp FP32 (complex128 in and out), one checkerboard"}
    for name, code in (("Mooee", o.OP_MOOEE), ("MooeeInv", o.OP_MOOEE_INV)):
        ref.apply(code, x, 1)
        n, t0 = 0, time.perf_counter()
        while n < 1 or time.perf_counter() - t0 < budget_s:
            ref.apply(code, x, 1)
            n += 1
        dt = (time.perf_counter() - t0) / n
        out[name] = {"ms": dt * 1e3, "gbs": nh * 192 / dt / 1e9, "reps": n}
    return out


def extra_cg_schur(g, fp64_maxit=20000):
    """Mixed-precision SchurRedBlack CG on Moebius DWF 24^4 x Ls=12, mf=0.005, gauge eps=0.6,
    to a true residual of 1e-10: FP32 inner, FP16-stored inner (FP32 norms/arithmetic), a
    4-RHS batched mixed solve, and the plain FP64 CG; the FP32 mixed solve and the FP64 CG
    again with the FP64 hopping term in double-float arithmetic (GB_FLAG_DF64).  Reliable updates every 100
    iterations or when |r|^2 drops by 1e-6 (|r| by 1e-3).  Every solve captures its
    iteration chunks as CUDA graphs (use_graphs=1)."""
    dims, Ls, mf = (24, 24, 24, 24), 12, 0.005
    U = g.random_gauge(dims, 0.6, 3003)
    vol = int(np.prod(dims))
    out = {"workload": "mobius_dwf_24^4xLs12_mf0.005_schur_cg_1e-10"}

    def solve(inner, nrhs, seed, graphs=1, outer_flags=0):
        od = g.MobiusFermion(U, dims, Ls, mf, M5, B, C, precision=g.F64, nrhs=nrhs, flags=outer_flags)
        src = g.random_gaussian(vol * Ls * 12 * nrhs, seed)
        fs = od.FermionField().import_(src)
        fx = od.FermionField().zero()
        if inner is None:
            cg = g.ConjugateGradient(1e-10, fp64_maxit, err_on_no_conv=False, check_every=20, use_graphs=graphs)
            solver = g.SchurRedBlackDiagMooeeSolve(cg)
            keep = None
        else:
            of = g.MobiusFermion(U, dims, Ls, mf, M5, B, C, precision=inner, nrhs=nrhs)
            cg = g.ConjugateGradientReliableUpdate(1e-10, 30000, 1e-6, g.SchurDiagMooeeOperator(of),
                                                   g.SchurDiagMooeeOperator(od), relup_every=100,
                                                   err_on_no_conv=False, check_every=20, use_graphs=graphs)
            solver = g.SchurRedBlackDiagMooeeSolve(cg)
            keep = of
        od.sync()
        t0 = time.perf_counter()
        r = solver(od, fs, fx)
        od.sync()
        dt = time.perf_counter() - t0
        x = fx.export()
        del keep
        return {"seconds": dt, "solves_per_s": nrhs / dt, "iterations": int(r.iterations),
                "reliable_updates": int(r.reliable_updates), "cleanup_iterations": int(r.cleanup_iterations),
                "true_residual": float(r.true_residual), "unprec_residual": float(max(solver.unprec_residual)),
                "converged": int(r.converged), "nrhs": nrhs}, x

    def solve_restart(seed):
        """MixedPrecisionConjugateGradient: restarted FP32 inner CGs, FP64 patch-up."""
        od = g.MobiusFermion(U, dims, Ls, mf, M5, B, C, precision=g.F64)
        of = g.MobiusFermion(U, dims, Ls, mf, M5, B, C, precision=g.F32)
        src = g.random_gaussian(vol * Ls * 12, seed)
        fs = od.FermionField().import_(src)
        fx = od.FermionField().zero()
        se, so = od.FermionRedBlackField(g.EVEN), od.FermionRedBlackField(g.ODD)
        # the Schur source of SchurRedBlackDiagMooeeSolve, then the mixed solve on the odd sites
        g.pickCheckerboard(g.EVEN, se, fs)
        g.pickCheckerboard(g.ODD, so, fs)
        t_e, t_o, src_o = od.FermionRedBlackField(g.EVEN), od.FermionRedBlackField(g.ODD), od.FermionRedBlackField(g.ODD)
        od.MooeeInv(se, t_e)
        od.Meooe(t_e, t_o)
        g.axpby(t_o, 1.0, -1.0, so, t_o)
        od.MpcDag(t_o, src_o)
        x_o = od.FermionRedBlackField(g.ODD).zero()
        cg = g.MixedPrecisionConjugateGradient(1e-10, 30000, 100, None, g.SchurDiagMooeeOperator(of),
                                               g.SchurDiagMooeeOperator(od), check_every=20, use_graphs=1)
        od.sync()
        t0 = time.perf_counter()
        cg(src_o, x_o)
        od.sync()
        dt = time.perf_counter() - t0
        return {"seconds": dt, "solves_per_s": 1.0 / dt, "inner_iterations": int(cg.TotalInnerIterations),
                "restarts": int(cg.TotalOuterIterations), "patchup_iterations": int(cg.TotalFinalStepIterations),
                "true_residual": float(cg.TrueResidual),
                "note": "the odd-checkerboard Schur system (MpcDagMpc) only; the red-black source and solution steps are not timed"}

    m32, x32 = solve(g.F32, 1, 77)
    m32_loop, _ = solve(g.F32, 1, 77, graphs=2)  # the CG loop on the device (conditional graph node)
    # the FP64 operator with its hopping term in double-float arithmetic (GB_FLAG_DF64):
    # as the outer operator of the mixed solve, and for the whole FP64 CG
    try:
        m32_df, x32_df = solve(g.F32, 1, 77, outer_flags=g.DF64)
        f64_df, x64_df = solve(None, 1, 77, outer_flags=g.DF64)
    except Exception as e:  # reported, the other solves still run
        m32_df = f64_df = {"error": f"{type(e).__name__}: {e}"}
        x32_df = x64_df = None
    m16, x16 = solve(g.F16, 1, 77)
    mb, _ = solve(g.F32, 4, 78)
    f64, x64 = solve(None, 1, 77)
    from oracle import oracle as o
    m32["solution_rel_err_vs_fp64"] = o.rel_l2(x32, x64)
    m16["solution_rel_err_vs_fp64"] = o.rel_l2(x16, x64)
    if x32_df is not None:
        m32_df["solution_rel_err_vs_fp64"] = o.rel_l2(x32_df, x64)
        f64_df["solution_rel_err_vs_fp64"] = o.rel_l2(x64_df, x64)
    # bounded CPU baseline: one FP64 MpcDagMpc of the oracle on the host cores, times the
    # FP64 iteration count
    ref = o.OracleOp(1, 0, dims, Ls, [mf, M5, B, C], U, g.antiperiodic_t())
    o.set_threads(os.cpu_count() or 1)
    xh = g.random_gaussian(vol // 2 * Ls * 12, 79)
    t0 = time.perf_counter()
    ref.apply(o.OP_MPCDAGMPC, xh, 1)
    per_it = time.perf_counter() - t0
    out["cpu_oracle"] = {"seconds_per_iteration": per_it, "cores": os.cpu_count(),
                         "solve_estimate_seconds": per_it * f64["iterations"],
                         "sample": "one FP64 MpcDagMpc of the 24^4 x 12 operator, scaled by the FP64 CG iterations"}
    out["mixed_fp32_restarted"] = solve_restart(77)
    out.update({"mixed_fp32": m32, "mixed_fp32_device_loop": m32_loop, "mixed_fp16": m16, "mixed_fp32_batched4": mb, "fp64": f64,
                "mixed_fp32_df64_outer": m32_df, "fp64_df64": f64_df,
                "speedup_mixed_vs_fp64": m32["solves_per_s"] / f64["solves_per_s"],
                "speedup_mixed_batched_vs_fp64": mb["solves_per_s"] / f64["solves_per_s"]})
    return out


def extra_wilson_cg(g):
    """Wilson 8^4 (antiperiodic t), FP64, m = 0.1, gauge eps = 0.3: one full Dhop and an
    unpreconditioned CG on MdagM to 1e-8 -- on the GPU and, for the same field and source,
    on the host cores with the oracle (the reference's CPU-runnable configuration)."""
    from oracle import oracle as o
    dims, mass = (8, 8, 8, 8), 0.1
    vol = int(np.prod(dims))
    U = g.random_gauge(dims, 0.3, 1001)
    src = g.random_gaussian(vol * 12, 1002)
    op = g.WilsonFermion(U, dims, mass, precision=g.F64)
    fin, fout = op.FermionField().import_(src), op.FermionField()
    for _ in range(20):
        op.Dhop(fin, fout, 0)
    reps = 500
    op.sync()
    t0 = time.perf_counter()
    for _ in range(reps):
        op.Dhop(fin, fout, 0)
    op.sync()
    gpu_dhop = (time.perf_counter() - t0) / reps
    fx = op.FermionField()

    def gpu_solve(graphs):
        fx.zero()
        cg = g.ConjugateGradient(1e-8, 10000, use_graphs=graphs)
        op.sync()
        t0 = time.perf_counter()
        r = cg(g.MdagMLinearOperator(op), fin, fx)
        op.sync()
        return time.perf_counter() - t0, r

    gpu_solve(0)  # the operator's first solve allocates its workspace fields
    gpu_solve(1)
    gpu_cg_plain, _ = gpu_solve(0)
    gpu_cg, r = gpu_solve(1)
    ref = o.OracleOp(0, 0, dims, 1, [mass], U, g.antiperiodic_t())
    o.set_threads(os.cpu_count() or 1)
    t0 = time.perf_counter()
    for _ in range(20):
        ref.apply(o.OP_DHOP, src)
    cpu_dhop = (time.perf_counter() - t0) / 20
    t0 = time.perf_counter()
    psi, cpu_it, cpu_res = ref.cg(0, src, 1e-8, 10000)
    cpu_cg = time.perf_counter() - t0
    return {"workload": "wilson_8^4_m0.1_fp64_dhop_and_unprec_cg_1e-8",
            "gpu": {"dhop_us": gpu_dhop * 1e6, "cg_seconds": gpu_cg, "iterations": int(r.iterations),
                    "true_residual": float(r.true_residual), "cg_seconds_without_graphs": gpu_cg_plain,
                    "note": "warm operator; iteration chunks captured as CUDA graphs (use_graphs=1)"},
            "cpu_oracle": {"dhop_us": cpu_dhop * 1e6, "cg_seconds": cpu_cg, "iterations": int(cpu_it),
                           "true_residual": float(cpu_res), "cores": os.cpu_count()},
            "solution_rel_diff_gpu_vs_cpu": float(o.rel_l2(fx.export(), psi)),
            "cg_speedup_gpu_vs_cpu": cpu_cg / gpu_cg,
            "note": "8^4 is 4096 sites: launch- and latency-bound on the GPU"}


def extra_multi_rhs(g):
    """Wilson 32^3 x 64, m = 0.02, gauge eps = 0.5, 12 point sources (spin x colour at the
    origin) + 4 Z2-noise sources: the FP32 16-RHS DhopEO (links read once for all 16) and
    the batched Schur CG to 1e-10 with FP64 reliable updates."""
    dims, nrhs, mass = (32, 32, 32, 64), 16, 0.02
    vol = int(np.prod(dims))
    U = g.random_gauge(dims, 0.5, 4004)
    srcs = []
    for sc in range(12):  # point sources psi[site 0][spin][colour]
        a = np.zeros(vol * 12, dtype=np.complex128)
        a[sc] = 1.0
        srcs.append(a)
    for k in range(4):
        srcs.append(g.random_z2(vol * 12, 500 + k))
    src = np.concatenate(srcs)
    out = {"workload": "wilson_32^3x64_m0.02_16rhs"}
    of = g.WilsonFermion(U, dims, mass, precision=g.F32, nrhs=nrhs)
    ins = [of.FermionRedBlackField(g.ODD).import_(g.random_gaussian(of.half_sites4 * 12 * nrhs, 90 + k)) for k in range(2)]
    outs = [of.FermionRedBlackField(g.EVEN) for _ in range(2)]
    ms = of.bench_kernel(0, ins, outs, 20)
    sites = of.half_sites4 * nrhs
    out["dhop_eo_16rhs_ms"] = ms
    out["dhop_eo_16rhs_gbs"] = sites * (192 + 576 / nrhs) / (ms / 1e3) / 1e9
    out["dhop_eo_16rhs_bytes_per_site_rhs"] = 192 + 576 / nrhs
    del ins, outs
    od = g.WilsonFermion(U, dims, mass, precision=g.F64, nrhs=nrhs)
    fs = od.FermionField().import_(src)
    fx = od.FermionField().zero()
    cg = g.ConjugateGradientReliableUpdate(1e-10, 20000, 1e-6, g.SchurDiagMooeeOperator(of),
                                           g.SchurDiagMooeeOperator(od), relup_every=100, err_on_no_conv=False)
    solver = g.SchurRedBlackDiagMooeeSolve(cg)
    od.sync()
    t0 = time.perf_counter()
    r = solver(od, fs, fx)
    od.sync()
    dt = time.perf_counter() - t0
    out.update({"batched_solve_seconds": dt, "solves_per_s": nrhs / dt, "iterations": int(r.iterations),
                "reliable_updates": int(r.reliable_updates), "true_residual": float(r.true_residual),
                "unprec_residual": float(max(solver.unprec_residual)), "converged": int(r.converged)})
    del od, of, fs, fx
    # the same solver on one right-hand side at a time (a point source and a Z2 source),
    # for the batch's solves/s against single solves
    of1 = g.WilsonFermion(U, dims, mass, precision=g.F32)
    od1 = g.WilsonFermion(U, dims, mass, precision=g.F64)
    single = []
    for k in (0, 12):
        fs1 = od1.FermionField().import_(srcs[k])
        fx1 = od1.FermionField().zero()
        cg1 = g.ConjugateGradientReliableUpdate(1e-10, 20000, 1e-6, g.SchurDiagMooeeOperator(of1),
                                                g.SchurDiagMooeeOperator(od1), relup_every=100, err_on_no_conv=False)
        s1 = g.SchurRedBlackDiagMooeeSolve(cg1)
        od1.sync()
        t0 = time.perf_counter()
        r1 = s1(od1, fs1, fx1)
        od1.sync()
        single.append({"source": "point (spin 0, colour 0)" if k == 0 else "Z2 noise", "seconds": time.perf_counter() - t0,
                       "iterations": int(r1.iterations), "true_residual": float(r1.true_residual)})
    t1 = sum(x["seconds"] for x in single) / len(single)
    out["single_rhs"] = single
    out["single_rhs_solves_per_s"] = 1.0 / t1
    out["batch_vs_single_solves_per_s"] = (nrhs / dt) * t1
    return out


def serving_stream(seconds, rate=20.0, seed=5005):
    """The seeded request stream: Poisson arrivals, Moebius DWF volume from {8^4, 12^4,
    16^4, 24^4, 16^3x32}, Ls from {8, 12, 16}, mf log-uniform in [1e-3, 1e-1], gauge eps
    uniform in [0.3, 0.7], 1-12 Gaussian sources."""
    rng = np.random.default_rng(seed)
    vols = [(8, 8, 8, 8), (12, 12, 12, 12), (16, 16, 16, 16), (24, 24, 24, 24), (16, 16, 16, 32)]
    t, reqs = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            break
        reqs.append(dict(t=t, dims=vols[rng.integers(len(vols))], Ls=int(rng.choice([8, 12, 16])),
                         mf=float(np.exp(rng.uniform(np.log(1e-3), np.log(1e-1)))), eps=float(rng.uniform(0.3, 0.7)),
                         gauge_seed=int(rng.integers(1 << 62)), nsrc=int(rng.integers(1, 13)),
                         src_seed=int(rng.integers(1 << 62))))
    return reqs


def extra_serving(g, max_requests=None, seconds=60.0, drain=30.0, slots=6, budget_gb=150.0, inner=None,
                  age_limit=10.0):
    """Replays the seeded stream (Poisson 20/s over `seconds`: ~1200 requests) at its
    arrival times into the service: HBM budget 150 GB, mixed-precision CG to 1e-10 (FP32
    inner, or FP16 storage with `inner=g.F16`), admission of the first queued request
    that fits with an age bound.  Arrivals stop at `seconds`; at `seconds + drain` every
    request still queued is shed and those running complete.  Reports completed solves/s
    over the wall time, p50/p99 latency of the completed requests, the queue depth over
    time, shed and rejected counts, and the concurrency of the requests' device work on
    the GPU's clock."""
    inner = g.F32 if inner is None else inner
    reqs = serving_stream(seconds)
    if max_requests:
        reqs = reqs[:max_requests]
    srv = g.Server(int(budget_gb * (1 << 30)), slots=slots, flags=g.Server.GRAPHS)
    srv.set_age_limit(age_limit)
    t0 = time.perf_counter()
    for q in reqs:
        delay = q["t"] - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        srv.submit(g.make_request(q["dims"], q["Ls"], q["mf"], q["eps"], q["gauge_seed"], q["nsrc"], q["src_seed"],
                                  inner=inner))
    t_arrivals = time.perf_counter() - t0
    while time.perf_counter() - t0 < seconds + drain and srv.stats().finished < len(reqs):
        time.sleep(0.25)
    shed = srv.cancel_queued()
    t_shed = time.perf_counter() - t0
    all_done = srv.wait(len(reqs), 1800)
    wall = time.perf_counter() - t0
    res = srv.results(len(reqs) + 8)
    st = srv.stats()
    tr_t, tr_q, tr_r = srv.trace()
    srv.close()
    good = [r for r in res if r.status == 0]
    lat = np.array([r.t_end - r.t_submit for r in good])
    nsol = sum(r.nsrc for r in good)
    # time-weighted queue depth and device concurrency
    qd = {}
    if len(tr_t) > 1:
        dt = np.diff(tr_t)
        qd = {"max": int(tr_q.max()), "mean_time_weighted": float((tr_q[:-1] * dt).sum() / max(dt.sum(), 1e-9)),
              "at_10s": [int(tr_q[max(0, np.searchsorted(tr_t, x) - 1)]) for x in np.arange(10.0, tr_t[-1], 10.0)]}
    ev = sorted([(r.dev_start, 1) for r in good if r.dev_start >= 0] + [(r.dev_end, -1) for r in good if r.dev_start >= 0])
    conc, busy, multi, peak = 0, 0.0, 0.0, 0
    for k in range(len(ev) - 1):
        conc += ev[k][1]
        peak = max(peak, conc)
        span = ev[k + 1][0] - ev[k][0]
        if conc >= 1:
            busy += span
        if conc >= 2:
            multi += span
    return {"workload": f"serving: the seeded Poisson(20/s) stream over {seconds:.0f} s, {len(reqs)} requests, "
                        f"drain limit {drain:.0f} s after the last arrival window",
            "arrivals": len(reqs), "completed": len(good), "shed": int(shed), "rejected": int(st.rejected),
            "failed": len(res) - len(good) - int(shed) - int(st.rejected), "all_done": bool(all_done),
            "wall_s": wall, "arrival_window_s": t_arrivals, "shed_at_s": t_shed,
            "solves_per_s": nsol / wall, "requests_per_s": len(good) / wall,
            "completed_solves": nsol,
            "latency_p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "latency_p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "max_true_residual": float(max((r.true_residual for r in good), default=0.0)),
            "max_running": int(st.max_running), "peak_hbm_gb": st.peak_used_bytes / (1 << 30), "slots": slots,
            "budget_gb": budget_gb, "inner_precision": "fp16" if inner == g.F16 else "fp32",
            "admission": f"first queued request that fits, in arrival order; none may pass a request older than {age_limit:.0f} s",
            "queue_depth": qd,
            "device_concurrency": {"max_requests_in_flight": int(peak), "busy_s": busy,
                                   "fraction_of_busy_time_with_2_or_more": multi / busy if busy > 0 else 0.0,
                                   "source": "CUDA events bracketing each request's device work on its slot's stream"}}


def cg_profile(g, iters):
    """For a profiler's launch list, not a measurement: the mixed FP32 Schur CG of the
    24^4 x Ls12 workload stopped after `iters` inner iterations (one reliable update at
    iteration 100 when iters > 100, no final cleanup)."""
    dims, Ls, mf = (24, 24, 24, 24), 12, 0.005
    U = g.random_gauge(dims, 0.6, 3003)
    vol = int(np.prod(dims))
    od = g.MobiusFermion(U, dims, Ls, mf, M5, B, C, precision=g.F64)
    of = g.MobiusFermion(U, dims, Ls, mf, M5, B, C, precision=g.F32)
    fs = od.FermionField().import_(g.random_gaussian(vol * Ls * 12, 77))
    fx = od.FermionField().zero()
    cg = g.ConjugateGradientReliableUpdate(1e-10, iters, 1e-6, g.SchurDiagMooeeOperator(of),
                                           g.SchurDiagMooeeOperator(od), relup_every=100, err_on_no_conv=False,
                                           final_cleanup=False, check_every=20)
    r = g.SchurRedBlackDiagMooeeSolve(cg)(od, fs, fx)
    od.sync()
    print(json.dumps({"cg_profile": "mobius_dwf_24^4xLs12_mixed_fp32", "iterations": int(r.iterations)}))


DHOP_PROFILE_CASES = {
    # name: (kind, dims, Ls, nrhs, precision); every input half field is above the 129 MB L2
    "wilson16rhs_fp32": ("wilson", (24, 24, 24, 32), 1, 16, "F32"),
    "dwf_fp16": ("mobius", (32, 32, 32, 32), 12, 1, "F16"),
    "dwf_fp64": ("mobius", (16, 16, 16, 16), 16, 2, "F64"),
    "dwf_df64": ("mobius", (16, 16, 16, 16), 16, 2, "DF64"),  # FP64 fields, double-float arithmetic
    "dwf_fp32": ("mobius", (16, 16, 16, 16), 16, 1, "F32"),
    "dwf24_ls12_fp32": ("mobius", (24, 24, 24, 24), 12, 1, "F32"),
}


def dhop_profile(g, case, launches=3):
    """For a profiler's capture, not a measurement: `launches` DhopEO launches of a small
    case of each Dhop kernel (DHOP_PROFILE_CASES)."""
    kind, dims, Ls, nrhs, prec = DHOP_PROFILE_CASES[case]
    flags = g.DF64 if prec == "DF64" else 0
    prec = g.F64 if prec == "DF64" else getattr(g, prec)
    U = g.random_gauge(dims, EPS, 1234)
    if kind == "wilson":
        op = g.WilsonFermion(U, dims, 0.02, precision=prec, nrhs=nrhs, flags=flags)
    else:
        op = g.MobiusFermion(U, dims, Ls, MF, M5, B, C, precision=prec, nrhs=nrhs, flags=flags)
    n = op.half_sites4 * Ls * nrhs * 12
    fin = op.FermionRedBlackField(g.ODD).import_(g.random_gaussian(n, 7))
    fout = op.FermionRedBlackField(g.EVEN)
    for _ in range(launches):
        op.DhopEO(fin, fout, 0)
    op.sync()
    print(json.dumps({"dhop_profile": case, "dims": list(dims), "Ls": Ls, "nrhs": nrhs, "launches": launches}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-extras", action="store_true", help="only the headline DhopEO/DhopOE measurement")
    ap.add_argument("--serve-requests", type=int, default=0, help="replay only the first N requests of the stream (0: all)")
    ap.add_argument("--serve-drain", type=float, default=30.0,
                    help="seconds after the arrival window at which still-queued requests are shed")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="length of the seeded arrival stream")
    ap.add_argument("--cg-profile", type=int, default=0, metavar="ITERS",
                    help="run only ITERS iterations of the 24^4 x 12 mixed CG (for a profiler's launch list)")
    ap.add_argument("--dhop-profile", choices=sorted(DHOP_PROFILE_CASES), default=None,
                    help="run three DhopEO launches of a small case of one Dhop kernel (for a profiler's capture)")
    args = ap.parse_args()
    if args.dhop_profile:
        import grid_gb300 as g
        dhop_profile(g, args.dhop_profile)
        return
    if args.cg_profile:
        import grid_gb300 as g
        cg_profile(g, args.cg_profile)
        return
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    dist = dist_init(ws)
    run_gpu(args, ws, rank, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
