#!/usr/bin/env python
"""Benchmark of the svMultiPhysics fluid Newton-step hot path on one GB300.

Workload: the 8M-tet pipe (2.0e7 CSR blocks, 1.37M nodes; seeded 8-mode wall
perturbation), incompressible VMS P1-P1 Navier-Stokes, pulsatile inflow (10 cm/s mean
plus a 5 cm/s sine at 1 Hz), generalised-alpha rho_inf = 0.5, dt = 1e-3.  A "step" is
one time step: 3 Newton iterations, each an assembly of the residual and tangent and a
GMRES(50) + diagonal-preconditioner solve to a relative residual of 1e-6.

Our arm (default) times K steps after W warm-up steps:
  value  -- device-resident state (An/Yn/Dn stay in HBM), CUDA events on the stream the
            library launches on;
  e2e    -- the same steps through the public C ABI with host arrays (Ao/Yo/Do copied in,
            An/Yn/Dn copied out every step);
  roofline -- the block SpMV, timed with CUDA events on the library's stream after the
            timed region, against the measured HBM copy bandwidth;
  cpu_baseline -- the C oracle (a restatement of the reference's own FSILS/assembly
            code, one core) on a bounded sample of the same system.

--impl reference times the reference's CPU path (the oracle port: the reference's
sources only compile where its tree is present) on a bounded sample per step and
reports the same metric.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "s/time step + Krylov iters, learned-precond vs plain GPU, 1 GB300, res<=1e-6"
WORKLOAD = "pipe8m"
NEWTON_ITERS = 3
REL_TOL = 1e-6
KRYLOV_DIM = 50
MAX_RESTARTS = 400
U_MEAN, U_AMP, U_FREQ = 10.0, 5.0, 1.0


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([s.strip() for s in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        smax = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(self.samples)}


def spmv_bytes(nnz, nNo, val_bytes=8):
    """Algorithmic bytes of one 4x4 block SpMV: Val + colPtr once, rowPtr, x once, y once."""
    return nnz * (16 * val_bytes + 4) + (nNo + 1) * 4 + nNo * 4 * 8 + nNo * 4 * 8


def cpu_sample(mesh, rowPtr, colPtr, krylov_its_per_newton, newton_iters, frac_elems=0.02):
    """Time the oracle (the reference's FP64 algorithm restated in C, one core) on a
    bounded sample of the same system and scale it to one time step:
      * the assembly (construct_fluid + do_assem) of a slice of the elements, scaled to all;
      * one block SpMV (spar_mul) and one dot + one axpy (dot_v / omp_sum_v) on the full
        system; a GMRES(sD) iteration i costs one SpMV, i+2 dots and i+1 axpys
        (gmres.cpp:537-569), so a restart cycle averages SpMV + (sD+1)/2+1 dots + (sD+1)/2 axpys
        per iteration;
      * per step = Newton iterations x (assembly + Krylov iterations per solve x that cost)."""
    from oracle import pyoracle as po
    P = po.fluid_params()
    rng = np.random.default_rng(0)
    nNo = mesh.nNo
    Ag = np.ascontiguousarray(rng.standard_normal((nNo, 4)) * 0.1)
    Yg = np.ascontiguousarray(rng.standard_normal((nNo, 4)))
    ne = max(1, int(mesh.nEl * frac_elems))
    ien_s = np.ascontiguousarray(mesh.ien[:ne])
    R = np.zeros((nNo, 4))
    Val = np.zeros((colPtr.size, 16))
    t0 = time.perf_counter()
    po.construct_fluid(P, mesh.x, ien_s, Ag, Yg, rowPtr, colPtr, R, Val)
    t_asm = (time.perf_counter() - t0) * mesh.nEl / ne
    Val[:] = 1.0
    U = np.ascontiguousarray(rng.standard_normal((nNo, 4)))
    t0 = time.perf_counter()
    po.spar_mul(rowPtr, colPtr, Val, U)
    t_spmv = time.perf_counter() - t0
    V = np.ascontiguousarray(rng.standard_normal((nNo, 4)))
    t0 = time.perf_counter()
    po.dot(U, V)
    t_dot = time.perf_counter() - t0
    t0 = time.perf_counter()
    po.axpy(0.5, U, V)
    t_axpy = time.perf_counter() - t0
    half = (KRYLOV_DIM + 1) / 2.0
    t_it = t_spmv + (half + 1) * t_dot + half * t_axpy
    per_step = newton_iters * (t_asm + krylov_its_per_newton * t_it)
    return {"value": per_step, "unit": "s/time step", "cores": 1, "kind": "port",
            "sample": f"oracle assembly of {ne} of {mesh.nEl} tets scaled to all ({t_asm:.2f} s), one SpMV "
                      f"({t_spmv:.3f} s), one dot ({t_dot:.4f} s) and one axpy ({t_axpy:.4f} s) on the full "
                      f"{colPtr.size}-block system; per step = {newton_iters} x (assembly + "
                      f"{krylov_its_per_newton:.0f} GMRES({KRYLOV_DIM}) iterations at {t_it:.3f} s)",
            "assembly_s": t_asm, "krylov_iter_s": t_it}


def run_ours(args):
    import torch
    from svfsiplus_gb300 import api
    from svfsiplus_gb300.mesh import named_pipe

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    t0 = time.time()
    mesh = named_pipe(args.workload)
    rowPtr, colPtr = api.csr_pattern(mesh.nNo, mesh.ien)
    precision = api.SVGPU_FP64 if args.path == "plain" else api.SVGPU_MIXED
    s = api.PipeFluidSolver(mesh, device=local, sD=KRYLOV_DIM, mItr=MAX_RESTARTS, relTol=REL_TOL, absTol=1e-17,
                            newton_min=NEWTON_ITERS, newton_max=NEWTON_ITERS, newton_tol=1e-11,
                            precision=precision, rowPtr=rowPtr, colPtr=colPtr)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    api.lib().svgpu_set_stream(s.ctx._h, api.C.c_void_p(stream.cuda_stream))
    setup_s = time.time() - t0
    nNo = mesh.nNo
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    dAo, dYo, dDo = dev(s.Ao), dev(s.Yo), dev(s.Do)
    dAn, dYn, dDn = torch.empty_like(dAo), torch.empty_like(dYo), torch.empty_like(dDo)

    def dev_step():
        s.time += s.props.dt
        dirY, dirA = api.inflow(s.dir_prof, s.time, U_MEAN, U_AMP, U_FREQ)
        st = s.ctx.fluid_step(s.props, s.opts, dev(dirY), dev(dirA), dAo, dYo, dDo, dAn, dYn, dDn, s.norms)
        dAo.copy_(dAn)
        dYo.copy_(dYn)
        return st

    for _ in range(args.warmup):
        dev_step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches0 = s.ctx.kernel_launches
    stats = []
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            stats.append(dev_step())
        ev1.record(stream)
        torch.cuda.synchronize()
    dev_ms = ev0.elapsed_time(ev1)
    launches = s.ctx.kernel_launches - launches0
    if world > 1:
        t = torch.tensor([dev_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        dev_ms = float(t.item())

    # e2e: the same steps through the C ABI with host arrays
    s.Ao[:] = dAo.cpu().numpy()
    s.Yo[:] = dYo.cpu().numpy()
    torch.cuda.synchronize()
    e2e_stats = []
    t1 = time.perf_counter()
    for _ in range(args.steps):
        e2e_stats.append(s.step(U_MEAN, U_AMP, U_FREQ))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t1
    h2d = 3 * nNo * 4 * 8 + 2 * s.dir_nodes.size * 3 * 8
    d2h = 3 * nNo * 4 * 8

    # roofline of the block SpMV on the assembled system (FP64 Val, resident)
    Val = torch.empty((colPtr.size, 16), dtype=torch.float64, device="cuda")
    Val.normal_()
    x = torch.randn((nNo, 4), dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    for _ in range(3):
        s.ctx.spar_mul(4, Val, x, y)
    reps = 20
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        s.ctx.spar_mul(4, Val, x, y)
    e1.record(stream)
    torch.cuda.synchronize()
    spmv_ms = e0.elapsed_time(e1) / reps
    bytes_ = spmv_bytes(colPtr.size, nNo)
    peak, kind = peaks()
    achieved = bytes_ / (spmv_ms * 1e-3) / 1e9

    its = [x["itr"] for st in stats for x in st]
    per_newton = float(np.mean(its)) if its else 0.0
    rec = {
        "metric": METRIC, "value": dev_ms / 1e3 / args.steps, "unit": "s/time step", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.path == "plain" else "f32+f64",
        "data": "synthetic: procedural 8M-tet pipe, seeded wall perturbation (numpy seed 20261203)",
        "config": {"workload": f"{args.workload}: {mesh.nEl} tets, {nNo} nodes, {colPtr.size} blocks; VMS P1-P1 fluid, "
                               f"{NEWTON_ITERS} Newton its/step, GMRES({KRYLOV_DIM}) + diagonal preconditioner to "
                               f"rel {REL_TOL:g}", "path": args.path,
                   "l2": "inputs larger than L2 (Val is 2.6 GB)", "parallelism": "replicas" if world > 1 else "1 GPU"},
        "krylov_iters_per_newton": per_newton, "krylov_iters": its,
        "newton": [[{"iNorm": x["iNorm"], "fNorm": x["fNorm"], "itr": x["itr"], "suc": x["suc"]} for x in st] for st in stats],
        "e2e": {"value": e2e_s / args.steps, "unit": "s/time step", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "krylov_iters": [x["itr"] for st in e2e_stats for x in st]},
        "gpu_launches": launches,
        "roofline": {"kernel": "spmv4_f64 (block SpMV)", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": kind, "traffic": None,
                     "launch_ms": spmv_ms, "algorithmic_bytes": bytes_},
        "clocks": clk.summary(),
        "setup_s": setup_s,
    }
    if rank == 0 and not args.no_cpu:
        rec["cpu_baseline"] = cpu_sample(mesh, rowPtr, colPtr, per_newton, NEWTON_ITERS)
    if rank == 0:
        print(json.dumps(rec), flush=True)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    from svfsiplus_gb300.api import csr_pattern
    from svfsiplus_gb300.mesh import named_pipe
    mesh = named_pipe(args.workload)
    rowPtr, colPtr = csr_pattern(mesh.nNo, mesh.ien)
    # Krylov iterations per Newton solve of this workload with the reference algorithm
    # (GMRES(50) + diagonal preconditioner, rel 1e-6), as measured by the FP64 GPU path,
    # which runs the same algorithm.
    its = KRYLOV_ITS_PIPE8M
    samples = []
    t_total = time.perf_counter()
    for k in range(args.warmup + args.steps):
        r = cpu_sample(mesh, rowPtr, colPtr, its, NEWTON_ITERS)
        if k >= args.warmup:
            samples.append(r)
    v = float(np.mean([r["value"] for r in samples]))
    rec = {"metric": METRIC, "value": v, "unit": "s/time step", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic: procedural 8M-tet pipe",
           "config": {"workload": args.workload, "path": "reference CPU FSILS GMRES + diagonal preconditioner"},
           "impl": "reference",
           "cpu_baseline": {"value": v, "unit": "s/time step", "cores": 1, "kind": "port",
                            "sample": samples[-1]["sample"]},
           "e2e": {"value": v, "unit": "s/time step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "wall_s": time.perf_counter() - t_total}
    print(json.dumps(rec), flush=True)


# Krylov iterations per Newton solve on the 8M-tet pipe, measured with the FP64 GPU
# path (bench.py --path plain); used to scale the reference's per-iteration CPU time.
KRYLOV_ITS_PIPE8M = 1500.0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="svgpu", choices=["svgpu", "reference"])
    ap.add_argument("--path", default="plain", choices=["plain", "mixed", "learned"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
