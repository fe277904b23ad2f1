"""Benchmark: FP64 cell-updates/s of the explicit residual-and-update path on one GB300.

Workload (default): the 3D Euler Taylor-Green vortex on the periodic [0,2 pi]^3 box, 64^3
hexahedra split into 5 tetrahedra = 1,310,720 cells (2,646,016 faces), nodes jittered by
+-5% of h (seed 1234); least-squares gradients, MUSCL-UNS with the Barth post-limiter, Roe
flux, SSP-RK3 at CFL 0.8, global stability time step computed on the device each step.
A "step" is one full SSP-RK3 step (3 residual evaluations) of every cell; one
cell-update = one cell advanced by one step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload tgv3d|vortex2d|ffbox3d-implicit|kdif3d|adjoint3d] [--n 64] [--mode fast|exact]

--workload ffbox3d-implicit: time to a 1e-10 relative residual of the implicit solvers (FP64
flexible GMRES, mixed FP32/FP64, FP64 Jacobian-free) on a steady 3D far-field box, with a
per-kernel profile of one more step of each; --imp-steps K times K flexible-GMRES steps per
precision instead (a short launch sequence for ncu).
--workload kdif3d: 50 implicit heat-conduction steps, FP64 CG vs FP32 CG with FP64 refinement.
--workload adjoint3d: unsteady adjoint gradient, its cost against the primal, FD checks.

--impl reference times the CPU restatement of Typhon's solver (oracle/, OpenMP on all
host cores) on the same configuration: Typhon itself is Fortran and cannot be built here.
N > 1 runs independent replicas (the path is not sharded), one per GPU.
Prints one JSON line (rank 0).
"""
import argparse
import json
from pathlib import Path
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-updates/s FP64"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="tgv3d", choices=["tgv3d", "vortex2d", "ffbox3d-implicit", "kdif3d", "adjoint3d",
                                                             "flatplate-implicit"])
    ap.add_argument("--cell-order", default="given", choices=["given", "shuffled", "shuffled-rcm"],
                    help="tgv3d / vortex2d: the generator's cell numbering, a random one, or a random one "
                         "renumbered in reverse Cuthill-McKee order")
    ap.add_argument("--fp-nx", type=int, default=None, help="flatplate-implicit: streamwise quads (default 200)")
    ap.add_argument("--fp-nz", type=int, default=None, help="flatplate-implicit: spanwise quads (default 20)")
    ap.add_argument("--imp-time-limit", type=float, default=900.0,
                    help="flatplate-implicit: seconds per solver before the run stops short of the target")
    ap.add_argument("--fp-cfl-max", type=float, default=None, help="flatplate-implicit: CFL cap (default 500)")
    ap.add_argument("--fp-nkrylov", type=int, default=None, help="flatplate-implicit: FGMRES restart length (15)")
    ap.add_argument("--fp-max-it", type=int, default=None, help="flatplate-implicit: FGMRES cycles per step (40)")
    ap.add_argument("--fp-inv-res", type=float, default=None, help="flatplate-implicit: INV_RES (0.05)")
    ap.add_argument("--fp-scaling", default="state", choices=["state", "none"],
                    help="flatplate-implicit: row scaling of the Krylov system")
    ap.add_argument("--fp-precisions", default="fp64,mixed-fp64ortho",
                    help="flatplate-implicit: comma-separated FGMRES precisions to run")
    ap.add_argument("--n", type=int, default=None, help="cells per direction (default: the workload's)")
    ap.add_argument("--mode", default="fast", choices=["fast", "exact"])
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--cpu-sample-steps", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--imp-steps", type=int, default=0,
                    help="ffbox3d-implicit: time this many implicit steps per precision at the starting CFL "
                         "instead of the runs to 1e-10 (a short sequence of launches for ncu)")
    ap.add_argument("--kdif-inner-tol", type=float, default=1e-3, help="kdif3d: FP32 inner CG tolerance")
    ap.add_argument("--kdif-inner-max", type=int, default=300, help="kdif3d: FP32 inner CG iterations at most")
    ap.add_argument("--kdif-refine", action="store_true", help="kdif3d: also run FP32 CG inside FP64 refinement")
    ap.add_argument("--adj-cs-n", type=int, default=8, help="adjoint3d: mesh size of the complex-step check")
    ap.add_argument("--adj-cs-steps", type=int, default=0, help="adjoint3d: steps of the complex-step check "
                    "(default: the configuration's)")
    ap.add_argument("--adj-cs-directions", type=int, default=0, help="adjoint3d: directions of the complex-step "
                    "check (default: the configuration's)")
    ap.add_argument("--adj-steps", type=int, default=0, help="adjoint3d: RK steps (default: the configuration's)")
    ap.add_argument("--adj-fd-directions", type=int, default=0,
                    help="adjoint3d: directions of the central-difference check (default: the configuration's)")
    ap.add_argument("--adj-no-checks", action="store_true",
                    help="adjoint3d: skip binomial checkpointing and the derivative checks (a short launch "
                         "sequence for ncu)")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the short implicit, KDIF and adjoint runs of the default line")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, device):
    """The largest x over the ranks of the process group (the job's time is its slowest
    rank's); x itself for one rank."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world, seconds):
    """Whole-job rate of N replicas that each process units_per_rank in `seconds` (the
    max-over-ranks time): every rank's units over the slowest rank's time."""
    return units_per_rank * world / seconds


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every `interval_ms` while running.  Entering
    waits (up to 5 s) for the first sample, so that sampling is under way when the measured work
    starts; mark() / mark(end=True) bracket the timed region, and summary() then covers the
    samples taken inside it (at least the one nearest to it)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index, interval_ms=100):
        self.index = index
        self.interval_ms = interval_ms
        self.lines = []
        self.proc = None
        self.i0 = self.i1 = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", str(self.interval_ms)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.005)
        except FileNotFoundError:
            self.proc = None
        return self

    def mark(self, end=False):
        if end:
            self.i1 = len(self.lines)
        else:
            self.i0 = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if self.i0 is not None:
            i1 = self.i1 if self.i1 is not None else len(lines)
            # the samples inside the timed region, and the next one (taken as it ended)
            lines = lines[max(self.i0 - 1, 0) if i1 <= self.i0 else self.i0:i1 + 1]
        for ln in lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def fp64_peak():
    """Measured DFMA rate of this GPU (the probe fp64_peak.cu, built to _build/fp64_peak),
    FLOP/s, or None."""
    from typhon_gb300 import build as tybuild
    try:
        probe = tybuild.build_fp64_probe()
    except (OSError, RuntimeError):
        return None
    try:
        r = subprocess.run([str(probe)], capture_output=True, text=True, timeout=60)
    except (OSError, subprocess.TimeoutExpired):
        return None
    for ln in r.stdout.splitlines():
        if ln.startswith("DFMA:"):
            return float(ln.split("=")[1].split()[0]) * 1e12
    return None


def kernel_bytes(md, nslot_avg, mtab=False):
    """Compulsory (algorithmic) DRAM bytes per launch of each kernel: every array element
    the kernel needs is counted once (cells and faces of the whole mesh).  FP64 = 8 B,
    index = 4 B.  nci interior cells, nf faces, ng ghost cells, f = faces per cell."""
    nci, nf, ng = md.ncell_int, md.nface, md.ncell - md.ncell_int
    nc = md.ncell
    cf = 4 * nslot_avg * nci                                # gather list entries
    return {
        "ghost_prim": ng * (8 + 40 + 40),                   # gsrc/gface, read prim, write prim
        "grad": cf + nf * (8 + 48) + nc * 40 + nci * 120,    # list, fc1/fc2 + weights, prim, write grad
        "ghost_grad": ng * (8 + 120 + 120),
        "face_states": nf * (8 + 24 + 8 + 24 + 24 + 80) + nc * (40 + 120),  # fc, uLR, dLR, LF, RF, write cl/cr
        "barth": cf + nf * (8 + 80) + nc * 40 + nci * 24,    # list, fc, cl/cr, prim, write ratio
        "face_flux_lim": nf * (8 + 4 + 4 + 80 + 24 + 8 + 40) + nc * (40 + 24),
        "face_flux": nf * (8 + 4 + 4 + 24 + 8 + 40 + 64) + nc * (40 + 120),
        "rk_update": cf + nf * 40 + nci * (8 + 40 + 40 + 40 + 40 + 40 + 40),  # vol, flux, u0, acc r/w, cur, prim
        "gather": cf + nf * 40 + nci * (8 + 40),
        "timestep": nci * (8 + 8 + 40),
        "prim": nci * 80,
        # fused fast-mode kernels
        # lists, A^-1 d, reconstruction weights, write cl/cr; prim; write grad + ratio; or, with the
        # per-cell increment matrices (MUSCL/-UNS without limiter), lists, the matrix (nslot^2 per
        # cell), write cl/cr; prim; write ratio
        "cell_fast": (8 * nslot_avg * nci + 8 * nslot_avg ** 2 * nci + nf * 80 + nc * 40 + nci * 24) if mtab else
                     (8 * nslot_avg * nci + nf * (48 + 64 + 80) + nc * 40 + nci * (120 + 24)),
        "face_flux_fast": nf * (80 + 8 + 24 + 8 + 40),     # cl/cr, bc/partner, normal, surface, write flux
    }


def run_ours(args, rank, world, local):
    import torch
    import typhon_gb300 as ty
    from typhon_gb300 import _capi, cases
    from typhon_gb300 import build as tybuild

    tybuild.build()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w = cases.WORKLOADS[args.workload]
    n = args.n or w["n"]
    t0 = time.time()
    md = cases.make_mesh(args.workload, n, args.cell_order)
    t_mesh = time.time() - t0
    prim = cases.initial_prim(args.workload, md.cell_centre)
    g = ty.Grid(md, device=local)
    g.set_spat(w["scheme"], w["highres"], w["limiter"], w["postlim"], mode=args.mode)
    g.set_prim(prim)
    stream = torch.cuda.Stream(device=local)
    _capi.check(g.lib.ty_set_stream(g.h, stream.cuda_stream), "ty_set_stream")
    nci = md.ncell_int
    info = g.info()
    nslot_avg = (2 * md.nface_int + (md.nface - md.nface_int)) / nci
    # clocks sampled every 20 ms from before the warm-up (the timed region can be ~0.1 s)
    clk = ClockSampler(local, interval_ms=20).__enter__()
    # warmup
    g.run_steps(w["rk"], w["cfl"], args.warmup)
    torch.cuda.synchronize(local)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    _capi.check(g.lib.ty_profile_enable(g.h, 1), "ty_profile_enable")
    barrier()
    torch.cuda.synchronize(local)
    clk.mark()
    with torch.cuda.stream(stream):
        e0.record(stream)
        g.run_steps(w["rk"], w["cfl"], args.steps)
        e1.record(stream)
    torch.cuda.synchronize(local)
    clk.mark(end=True)
    time.sleep(0.03)   # the sample taken as the region ended
    clk.__exit__(None, None, None)
    barrier()
    ms = e0.elapsed_time(e1)
    nk = len(_capi.KERNEL_NAMES)
    kms = np.zeros(nk)
    kl = np.zeros(nk, np.int32)
    _capi.check(g.lib.ty_profile_read(g.h, nk, kms.ctypes.data, kl.ctypes.data), "ty_profile_read")
    _capi.check(g.lib.ty_profile_enable(g.h, 0), "ty_profile_enable")
    ms = max_over_ranks(ms, world, "cuda")
    value = job_throughput(nci * args.steps, world, ms * 1e-3)
    # per-kernel roofline
    peak, peak_kind = measured_peaks()
    mtab = (args.mode == "fast" and w["highres"] in ("MUSCL", "MUSCL-UNS") and w["limiter"] == "NONE"
            and info["max_faces_per_cell"] <= 4)
    kb = kernel_bytes(md, nslot_avg, mtab)
    per = {}
    for i, name in enumerate(_capi.KERNEL_NAMES):
        if kl[i] > 0:
            avg_ms = kms[i] / kl[i]
            per[name] = {"launches": int(kl[i]), "total_ms": round(float(kms[i]), 4),
                         "avg_ms": round(float(avg_ms), 5), "share": round(float(kms[i] / kms.sum()), 4),
                         "achieved_gbs": round(kb[name] / (avg_ms * 1e-3) / 1e9, 1)}
    dom = max(per, key=lambda k: per[k]["total_ms"])
    ach = per[dom]["achieved_gbs"]
    # DRAM traffic and FP64 instructions per unit, from one ncu capture of the same kernels on
    # the 40^3x5 mesh (320,000 cells, 649,600 faces), scaled by the units of this mesh
    per_unit = {"cell_fast": (nci, (65.42e6 + 11.33e6) / 320000, 198) if mtab else
                (nci, (96.07e6 + 53.98e6) / 320000, 261),
                "face_flux_fast": (md.nface, (72.21e6 + 4.60e6) / 649600, 127)}
    traffic = None
    fp64_roof = None
    if dom in per_unit and args.mode == "fast":
        units, bpu, ipu = per_unit[dom]
        traffic = int(bpu * units)
        peak64 = fp64_peak()
        if peak64:
            inst = ipu * units / (per[dom]["avg_ms"] * 1e-3) / 1e12
            fp64_roof = {"instr_per_unit": ipu, "units": int(units), "achieved_tinstr_s": round(inst, 4),
                    "peak_tinstr_s": round(peak64 / 2e12, 4), "frac": round(inst / (peak64 / 2e12), 4),
                    "note": "FP64 instructions (DFMA/DADD/DMUL, one each) per unit counted by ncu; peak = the "
                            "DFMA instruction rate measured on this GPU by fp64_peak.cu"}
    roofline = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": round(ach / peak, 4), "peak_source": peak_kind, "traffic": traffic,
                "traffic_source": "ncu, 40^3x5 mesh, scaled by units" if traffic else None,
                "algorithmic_bytes_per_launch": int(kb[dom]), "fp64_pipe": fp64_roof}
    # end to end through the public API with host buffers, per step: H2D of the state from
    # pinned host memory (Typhon's layout: rho, rhoE, rhou AoS), one step, D2H of the state
    e2e_steps = args.e2e_steps or max(3, min(args.steps, 10))
    pin = lambda shape: torch.empty(shape, dtype=torch.float64).pin_memory().numpy()
    rho_h, rhoE_h, rhou_h = pin((nci,)), pin((nci,)), pin((nci, 3))
    g.download_typhon(rho_h, rhoE_h, rhou_h)
    torch.cuda.synchronize(local)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        g.upload_typhon(rho_h, rhoE_h, rhou_h)
        g.run_steps(w["rk"], w["cfl"], 1)
        g.download_typhon(rho_h, rhoE_h, rhou_h)
    torch.cuda.synchronize(local)
    t_e2e = time.perf_counter() - t0
    barrier()
    t_e2e = max_over_ranks(t_e2e, world, "cuda")
    e2e = {"value": job_throughput(nci * e2e_steps, world, t_e2e), "unit": "cell-updates/s",
           "h2d_bytes_per_step": 40 * nci, "d2h_bytes_per_step": 40 * nci, "steps": e2e_steps}
    # the exact mode (bit-identical to the oracle) on the same grid and state, device time
    exact = None
    if args.mode == "fast":
        g.set_spat(w["scheme"], w["highres"], w["limiter"], w["postlim"], mode="exact")
        g.run_steps(w["rk"], w["cfl"], 2)
        ke = max(5, min(args.steps, 20))
        torch.cuda.synchronize(local)
        with torch.cuda.stream(stream):
            e0.record(stream)
            g.run_steps(w["rk"], w["cfl"], ke)
            e1.record(stream)
        torch.cuda.synchronize(local)
        mse = e0.elapsed_time(e1)
        exact = {"value": nci * ke / (mse * 1e-3), "unit": "cell-updates/s", "steps": ke,
                 "ms_per_step": round(mse / ke, 4),
                 "parity": "bit-identical to the oracle over 20 steps at this size (the fast mode agrees to 1e-12 "
                           "for 5 steps and stays within the oracle's own one-ulp sensitivity over 20)"}
        g.set_spat(w["scheme"], w["highres"], w["limiter"], w["postlim"], mode=args.mode)
    clocks = clk.summary()
    fp64 = fp64_peak()
    out = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, nci, md.nface, world),
        "e2e": e2e, "roofline": roofline, "kernels": per,
        "gpu_launches": int(kl.sum()), "clocks": clocks, "mesh_build_s": round(t_mesh, 2), "exact_mode": exact,
        "fp64_peak_tflops": round(fp64 / 1e12, 3) if fp64 else None,
    }
    g.close()
    return out


def workload_config(args, cells, faces, world):
    """The `config` object of both arms' JSON lines (the same workload and setup)."""
    from typhon_gb300 import cases
    w = cases.WORKLOADS[args.workload]
    n = args.n or w["n"]
    name = {"tgv3d": f"tgv3d {n}^3x5 tets", "vortex2d": f"vortex2d {n}x{n}x2 tris"}[args.workload]
    out = {"workload": name, "cells": int(cells), "faces": int(faces), "scheme": w["scheme"],
           "highres": w["highres"], "limiter": w["limiter"], "postlim": w["postlim"], "rk": w["rk"],
           "cfl": w["cfl"], "mode": args.mode, "parallelism": f"replicas{world}",
           "l2": "working set larger than L2 (no flush needed)"}
    if args.cell_order != "given":
        out["cell_order"] = args.cell_order
    return out


def cpu_sample(args, n_steps, warmup=1, with_mesh=False):
    """The CPU restatement (oracle, OpenMP) on the same mesh and setup: warmup untimed steps,
    then n_steps timed steps."""
    sys.path.insert(0, str(ROOT / "tests"))
    import oracle_py as op
    from typhon_gb300 import cases
    w = cases.WORKLOADS[args.workload]
    n = args.n or w["n"]
    raw = cases.make_raw(args.workload, n, args.cell_order)
    from typhon_gb300 import umesh
    om = op.Mesh.from_raw(raw).build(w["dim"], umesh.periodic_box_bcs((w["length"],) * w["dim"]))
    sch = {"HLLC": op.SCH_HLLC, "RUSANOV": op.SCH_RUSANOV, "ROE": op.SCH_ROE}[w["scheme"]]
    hres = {"NONE": op.HRES_NONE, "MUSCL": op.HRES_MUSCL, "MUSCL-FAST": op.HRES_MUSCLFAST,
            "MUSCL-UNS": op.HRES_MUSCLUNS}[w["highres"]]
    lim = {"NONE": op.LIM_NONE, "ALBADA": op.LIM_ALBADA}[w["limiter"]]
    post = {"NONE": op.POSTLIM_NONE, "BARTH": op.POSTLIM_BARTH}[w["postlim"]]
    s = op.Solver(om, sch, hres, lim, post, op.GRAD_LSQ, rk=w["rk"], cfl=w["cfl"])
    d = om.export()
    s.set_prim(cases.initial_prim(args.workload, d["ccentre"]))
    s.run_steps(max(1, warmup))  # warm (first-touch, LSQ factors)
    t0 = time.perf_counter()
    s.run_steps(n_steps)
    dt = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count()))
    out = {"value": om.ncell_int * n_steps / dt, "unit": "cell-updates/s", "cores": cores, "kind": "port",
           "sample": f"{n_steps} {w['rk']} step(s) of the full {om.ncell_int}-cell mesh, OpenMP on {cores} "
                     f"threads ({dt:.1f} s)"}
    if with_mesh:
        return out, om.ncell_int, om.nface
    return out


def run_implicit(args):
    """Steady implicit solve of the far-field box to a 1e-10 relative residual with three
    solvers: FP64 flexible GMRES (assembled BDLU, block Jacobi), the mixed form (FP32 BDLU
    mat-vec and block Jacobi, FP64 residual / CGS2 / update) and FP64 Jacobian-free
    Newton-Krylov.  Times to the target (wall clock, synchronised) and the mixed and JFNK
    converged states against the FP64 assembled one."""
    import torch
    import typhon_gb300 as ty
    from typhon_gb300 import _capi, build, cases
    build.build()
    torch.cuda.set_device(0)
    w = cases.FFBOX
    md = cases.make_ffbox(args.n)
    nci = md.ncell_int
    ff = w["freestream"]
    L = w["length"]
    prim0 = cases.perturbed_freestream(md.cell_centre, ff, (L / 2, L / 2, L / 2))
    scale = np.array([ff[0], ff[1] / 0.4, 0.3, 0.3, 0.3])
    if args.imp_steps:
        # a fixed number of FGMRES steps (FP64, then mixed) at the starting CFL, after one warm-up
        res = {}
        for prec in ("fp64", "mixed-fp64ortho", "mixed"):
            g = ty.Grid(md)
            g.set_spat(w["scheme"], w["highres"], w["limiter"], w["postlim"], mode="fast", farfield=ff)
            g.set_prim(prim0)
            kw = dict(nkrylov=w["nkrylov"], max_it=w["max_it"], inv_res=w["inv_res"], local_dt=True, precision=prec)
            g.implicit_step(w["cfl0"], "FGMRES", **kw)
            g.synchronize()
            t0 = time.perf_counter()
            for _ in range(args.imp_steps):
                st = g.implicit_step(w["cfl0"], "FGMRES", **kw)
            g.synchronize()
            res[prec] = {"ms_per_step": round((time.perf_counter() - t0) / args.imp_steps * 1e3, 3),
                         "matvecs_per_step": st["matvecs"]}
            g.close()
        print(json.dumps({"workload": f"ffbox3d {args.n or w['n']}^3x5 FGMRES steps", "cells": nci,
                          "steps": args.imp_steps, "variants": res}))
        return
    variants = {}
    states = {}
    with ClockSampler(0) as clk:
        for name, inv, prec in (("fgmres_fp64", "FGMRES", "fp64"), ("fgmres_mixed", "FGMRES", "mixed-fp64ortho"),
                                ("fgmres_mixed_f32basis", "FGMRES", "mixed"), ("jfnk_fp64", "JFNK", "fp64")):
            g = ty.Grid(md)
            g.set_spat(w["scheme"], w["highres"], w["limiter"], w["postlim"], mode="fast", farfield=ff)
            g.set_prim(prim0)
            g.implicit_step(1e-3, inv, nkrylov=w["nkrylov"], max_it=1, inv_res=0.5, local_dt=True, precision=prec)
            g.set_prim(prim0)                     # warm-up step above allocates the workspace
            g.synchronize()
            cfl, r0, steps, matvecs, rel = w["cfl0"], None, 0, 0, 1.0
            t0 = time.perf_counter()
            while steps < w["max_steps"]:
                st = g.implicit_step(cfl, inv, nkrylov=w["nkrylov"], max_it=w["max_it"], inv_res=w["inv_res"],
                                     local_dt=True, precision=prec)
                steps += 1
                matvecs += st["matvecs"]
                r = float(np.sqrt(np.sum((st["res_l2"] / scale) ** 2)))
                r0 = r0 or r
                rel = r / r0
                if rel < w["target"]:
                    break
                cfl = min(max(w["cfl0"] * r0 / r, w["cfl0"]), w["cfl_max"])
            g.synchronize()
            t = time.perf_counter() - t0
            # per-kernel device time of one more step at the final CFL (CUDA events per launch)
            nk = len(_capi.KERNEL_NAMES)
            kms, kl = np.zeros(nk), np.zeros(nk, np.int32)
            _capi.check(g.lib.ty_profile_enable(g.h, 1), "ty_profile_enable")
            t1 = time.perf_counter()
            g.implicit_step(cfl, inv, nkrylov=w["nkrylov"], max_it=w["max_it"], inv_res=w["inv_res"], local_dt=True,
                            precision=prec)
            g.synchronize()
            wall = time.perf_counter() - t1
            _capi.check(g.lib.ty_profile_read(g.h, nk, kms.ctypes.data, kl.ctypes.data), "ty_profile_read")
            _capi.check(g.lib.ty_profile_enable(g.h, 0), "ty_profile_enable")
            prof = {n: {"launches": int(kl[i]), "ms": round(float(kms[i]), 4)}
                    for i, n in enumerate(_capi.KERNEL_NAMES) if kl[i] > 0}
            states[name] = g.get_cons()
            variants[name] = {"seconds": round(t, 3), "steps": steps, "matvecs": matvecs, "final_rel_residual": rel,
                              "reached": bool(rel < w["target"]),
                              "profiled_step": {"wall_ms": round(wall * 1e3, 3), "kernels": prof}}
            g.close()
    ref = states["fgmres_fp64"]
    for name in ("fgmres_mixed", "fgmres_mixed_f32basis", "jfnk_fp64"):
        d = states[name] - ref
        variants[name]["state_vs_fp64"] = [float(np.linalg.norm(d[0]) / np.linalg.norm(ref[0])),
                                           float(np.linalg.norm(d[1]) / np.linalg.norm(ref[1])),
                                           float(np.linalg.norm(d[2:5]) / np.linalg.norm(ref[2:5]))]
    out = {"metric": "seconds to a 1e-10 relative residual, mixed implicit (FP32 Jv and block Jacobi, FP64 "
                     "Krylov basis, orthogonalisation, residual and update)", "unit": "s",
           "value": variants["fgmres_mixed"]["seconds"], "higher_is_better": False, "n_gpus": 1,
           "steps": variants["fgmres_mixed"]["steps"], "warmup": 1, "dtype": "f64+f32", "data": "synthetic",
           "scaling": "weak", "vs_baseline": None,
           "config": {"workload": f"ffbox3d {args.n or w['n']}^3x5 tets far field, Rusanov, backward Euler",
                      "cells": nci, "cfl": f"{w['cfl0']} -> {w['cfl_max']} (SER)",
                      "krylov": f"FGMRES({w['nkrylov']}) x {w['max_it']}, INV_RES {w['inv_res']}"},
           "variants": variants,
           "speedup_mixed_vs_fp64": round(variants["fgmres_fp64"]["seconds"] / variants["fgmres_mixed"]["seconds"], 3),
           "clocks": clk.summary()}
    print(json.dumps(out))


def run_flatplate(args):
    """Config 3, the laminar flat plate (cases.FLATPLATE): steady implicit solve toward a 1e-10
    relative residual with FP64 flexible GMRES and the mixed form with an FP64 Krylov basis
    (FP32 BDLU mat-vec and block Jacobi), each stopped at the target or after
    --imp-time-limit seconds.  Reports the time each solver takes to reach every residual
    decade both reach, and the residual each reached."""
    import torch
    import typhon_gb300 as ty
    from typhon_gb300 import _capi, build, cases
    build.build()
    torch.cuda.set_device(0)
    w = dict(cases.FLATPLATE)
    for key, val in (("cfl_max", args.fp_cfl_max), ("nkrylov", args.fp_nkrylov), ("max_it", args.fp_max_it),
                     ("inv_res", args.fp_inv_res)):
        if val is not None:
            w[key] = val
    names = {"fp64": "fgmres_fp64", "mixed-fp64ortho": "fgmres_mixed", "mixed": "fgmres_mixed_f32basis"}
    runs = [(names[p], p) for p in args.fp_precisions.split(",")]
    t0 = time.time()
    md = cases.make_flatplate(args.fp_nx, args.fp_nz)
    t_mesh = time.time() - t0
    nci = md.ncell_int
    ff = w["freestream"]
    scale = np.array([ff[0], ff[1] / 0.4, ff[0] * ff[2], ff[0] * ff[2], ff[0] * ff[2]])
    variants, states = {}, {}
    with ClockSampler(0) as clk:
        for name, prec in runs:
            g = ty.Grid(md)
            g.set_spat(w["scheme"], "NONE", "NONE", mode="fast", dissipative_flux="CELL-AVERAGE",
                       viscosity="SUTHERLAND", rgas=w["rgas"], prandtl=w["prandtl"], farfield=ff)
            prim0 = np.tile(np.array(ff)[:, None], (1, md.ncell))
            g.set_prim(prim0)
            kw = dict(nkrylov=w["nkrylov"], max_it=w["max_it"], inv_res=w["inv_res"], local_dt=True, precision=prec,
                      scaling=args.fp_scaling)
            g.implicit_step(1e-3, "FGMRES", **kw)   # allocates the workspace
            g.set_prim(prim0)
            g.synchronize()
            cfl, rmax, steps, matvecs, rel = w["cfl0"], None, 0, 0, 1.0
            decades, mid = {}, None
            t0 = time.perf_counter()
            while steps < w["max_steps"]:
                if steps == 40:                       # the state profiled below (one host copy)
                    mid = (g.get_cons(), cfl)
                st = g.implicit_step(cfl, "FGMRES", **kw)
                steps += 1
                matvecs += st["matvecs"]
                r = np.asarray(st["res_l2"]) / scale
                rmax = r if rmax is None else np.maximum(rmax, r)
                rel = float(np.sqrt(np.sum((r / rmax) ** 2) / 5))
                if not np.isfinite(rel):
                    break
                k = int(np.floor(-np.log10(max(rel, 1e-300))))
                for dlev in range(1, k + 1):
                    decades.setdefault(dlev, (round(time.perf_counter() - t0, 3), steps))
                if rel < w["target"] or time.perf_counter() - t0 > args.imp_time_limit:
                    break
                cfl = min(cfl * 1.5, w["cfl_max"])
            g.synchronize()
            seconds = time.perf_counter() - t0
            states[name] = g.get_cons()
            variants[name] = {"seconds": round(seconds, 3), "steps": steps, "matvecs": matvecs,
                              "final_rel_residual": rel, "reached": bool(rel < w["target"]),
                              "decades": {f"1e-{k}": v for k, v in sorted(decades.items())}}
            if mid is not None:                       # per-kernel device time of step 41 (CUDA events)
                g.set_cons(mid[0])
                nk = len(_capi.KERNEL_NAMES)
                kms, kl = np.zeros(nk), np.zeros(nk, np.int32)
                _capi.check(g.lib.ty_profile_enable(g.h, 1), "ty_profile_enable")
                t1 = time.perf_counter()
                st = g.implicit_step(mid[1], "FGMRES", **kw)
                g.synchronize()
                wall = time.perf_counter() - t1
                _capi.check(g.lib.ty_profile_read(g.h, nk, kms.ctypes.data, kl.ctypes.data), "ty_profile_read")
                _capi.check(g.lib.ty_profile_enable(g.h, 0), "ty_profile_enable")
                variants[name]["profiled_step"] = {
                    "step": 41, "cfl": mid[1], "matvecs": st["matvecs"], "wall_ms": round(wall * 1e3, 3),
                    "kernels": {n: {"launches": int(kl[i]), "ms": round(float(kms[i]), 4)}
                                for i, n in enumerate(_capi.KERNEL_NAMES) if kl[i] > 0}}
            g.close()
    both = "fgmres_fp64" in variants and "fgmres_mixed" in variants
    if both:
        d = states["fgmres_mixed"] - states["fgmres_fp64"]
        ref = states["fgmres_fp64"]
        state_diff = [float(np.linalg.norm(d[0]) / np.linalg.norm(ref[0])),
                      float(np.linalg.norm(d[1]) / np.linalg.norm(ref[1])),
                      float(np.linalg.norm(d[2:5]) / np.linalg.norm(ref[2:5]))]
    else:
        state_diff = None
    common = sorted(set.intersection(*(set(v["decades"]) for v in variants.values())),
                    key=lambda s: int(s.split("-")[1]))
    deepest = common[-1] if common else None
    head = variants["fgmres_mixed"] if "fgmres_mixed" in variants else next(iter(variants.values()))
    out = {"metric": "seconds to each residual decade, mixed implicit (FP32 Jv and block Jacobi, FP64 Krylov basis, "
                     "residual and update) vs FP64, laminar flat plate", "unit": "s",
           "value": head["decades"][deepest][0] if deepest else None,
           "higher_is_better": False, "n_gpus": 1, "dtype": "f64+f32", "data": "synthetic", "scaling": "weak",
           "vs_baseline": None,
           "config": {"workload": f"flat plate {nci} cells (prisms + tets), M 0.3, Re_L 1e4, Rusanov first order, "
                                  "cell-average viscous flux, Sutherland, adiabatic no-slip wall, far field",
                      "cells": nci, "cfl": f"{w['cfl0']} -> {w['cfl_max']} (x1.5 per step)",
                      "krylov": f"FGMRES({w['nkrylov']}) x {w['max_it']}, block Jacobi, INV_RES {w['inv_res']}, "
                                f"rows scaled: {args.fp_scaling}",
                      "time_limit_s": args.imp_time_limit, "mesh_build_s": round(t_mesh, 2)},
           "deepest_common_decade": deepest,
           "speedup_mixed_vs_fp64_at_deepest": (round(variants["fgmres_fp64"]["decades"][deepest][0] /
                                                      variants["fgmres_mixed"]["decades"][deepest][0], 3)
                                                if deepest and both else None),
           "variants": variants,
           "state_mixed_vs_fp64": state_diff,
           "clocks": clk.summary()}
    print(json.dumps(out))


def run_kdif(args):
    """Heat conduction: 50 backward-Euler steps of the KDIF config to a 1e-12 relative
    residual per step with FP64 conjugate gradients + Jacobi (fused single-reduction
    iteration) and with the mixed form (the same iteration on FP32 face conductances to 1e-6,
    then the FP64 matrix); --kdif-refine adds FP32 CG inside FP64 iterative refinement.
    Wall-clock time of the steps (synchronised), iterations, the mixed final temperature
    against the FP64 one, and the FP64 iteration's device time against the HBM roofline."""
    import torch
    import typhon_gb300 as ty
    from typhon_gb300 import build, cases
    build.build()
    torch.cuda.set_device(0)
    w = cases.KDIF3D
    md, kc, kind, val = cases.make_kdif3d(args.n)
    nci = md.ncell_int
    variants, temps = {}, {}
    runs = [("cg_fp64", "CG"), ("cg_mixed", "CG-MIXED")] + ([("cg32_refined", "CG32")] if args.kdif_refine else [])
    with ClockSampler(0) as clk:
        for name, solver in runs:
            g = ty.Grid(md)
            g.set_spat("HLLC", mode="fast")
            g.kdif_setup(kc, kind, val, flux="FULL", heat_capacity=w["heat_capacity"])
            g.kdif_set_temperature(np.zeros(md.ncell))
            g.kdif_implicit_step(w["dt"], solver, tol=1e-3)          # warm-up (workspace, clocks)
            g.kdif_set_temperature(np.zeros(md.ncell))
            g.synchronize()
            its, worst, switched = 0, 0.0, 0
            t0 = time.perf_counter()
            for _ in range(w["steps"]):
                if solver == "CG32":
                    st = g.kdif_implicit_step(w["dt"], solver, tol=w["tol"], max_it=args.kdif_inner_max,
                                              inner_tol=args.kdif_inner_tol)
                else:
                    st = g.kdif_implicit_step(w["dt"], solver, tol=w["tol"])
                its += st["iterations"]
                worst = max(worst, st["rel_res"])
                switched += st["refinements"]
            g.synchronize()
            t = time.perf_counter() - t0
            temps[name] = g.kdif_temperature()
            variants[name] = {"seconds": round(t, 3), "iterations": its, "worst_rel_res": worst,
                              "ms_per_step": round(1e3 * t / w["steps"], 3)}
            if solver == "CG-MIXED":
                variants[name]["steps_switched_to_fp64"] = switched
            if solver in ("CG", "CG-MIXED"):
                # device time of one conjugate-gradient iteration: a fixed 400 iterations
                # (tolerance out of reach), CUDA events on the handle's stream
                stream = torch.cuda.Stream()
                from typhon_gb300 import _capi
                _capi.check(g.lib.ty_set_stream(g.h, stream.cuda_stream), "ty_set_stream")
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                with torch.cuda.stream(stream):
                    e0.record(stream)
                    st = g.kdif_implicit_step(w["dt"], "CG", tol=1e-300, max_it=400)
                    e1.record(stream)
                torch.cuda.synchronize()
                _capi.check(g.lib.ty_set_stream(g.h, None), "ty_set_stream")
                ms = e0.elapsed_time(e1) / st["iterations"]
                ns = g.info()["max_faces_per_cell"]
                # algorithmic bytes per cell and iteration: A reads p, s, x, r, 1/diag and writes
                # x, r, u (64 B); B reads u, m, the conductances (8 B) and neighbour indices (4 B)
                # of every slot, p, s and writes p, s (48 + 12 ns B)
                bpc = 64 + 48 + 12 * ns
                if name == "cg_fp64":
                    peak, kind_ = measured_peaks()
                    ach = bpc * nci / (ms * 1e-3) / 1e9
                    variants[name]["iteration"] = {
                        "ms": round(ms, 5), "bytes_per_cell": bpc, "achieved_gbs": round(ach, 1), "peak_gbs": peak,
                        "frac": round(ach / peak, 4), "peak_source": kind_,
                        "note": "400 iterations timed with CUDA events, including the residual-norm read every "
                                "10 iterations and the step's residual and assembly"}
            g.close()
    d = temps["cg_mixed"] - temps["cg_fp64"]
    variants["cg_mixed"]["T_vs_fp64"] = float(np.linalg.norm(d) / np.linalg.norm(temps["cg_fp64"]))
    if "cg32_refined" in temps:
        d = temps["cg32_refined"] - temps["cg_fp64"]
        variants["cg32_refined"]["T_vs_fp64"] = float(np.linalg.norm(d) / np.linalg.norm(temps["cg_fp64"]))
    out = {"metric": "seconds for 50 implicit KDIF steps to 1e-12, mixed CG (FP32 conductances, then FP64)",
           "unit": "s", "value": variants["cg_mixed"]["seconds"], "higher_is_better": False, "n_gpus": 1,
           "steps": w["steps"], "warmup": 1, "dtype": "f64+f32", "data": "synthetic", "scaling": "weak",
           "vs_baseline": None,
           "config": {"workload": f"kdif3d {args.n or w['n']}^3x6 tets, lognormal k with 8 inclusions x100",
                      "cells": nci, "dt": w["dt"], "flux": "FULL"},
           "variants": variants,
           "speedup_mixed_vs_fp64": round(variants["cg_fp64"]["seconds"] / variants["cg_mixed"]["seconds"], 3),
           "clocks": clk.summary()}
    print(json.dumps(out))


def _cs_worker_init(tests_dir):
    sys.path.insert(0, tests_dir)


def _cs_direction(job):
    import residual_cs as cs
    md, U0, d, dts, table, box, scheme, highres, limiter = job
    return cs.box_functional_derivative(md, U0, d, dts, table, box, scheme, highres=highres, limiter=limiter)


def complex_step_sample(w, n=8, steps=None, directions=None):
    """The adjoint configuration on a small sample (TGV n^3 x 5, the configuration's steps and
    seeded directions): GPU adjoint directional derivatives against the complex step of the
    numpy restatement of the same residual (tests/residual_cs.py, the checker; never the
    measured path), one direction per process of a spawned pool."""
    import multiprocessing as mp
    import torch
    import typhon_gb300 as ty
    from typhon_gb300 import adjoint, cases
    steps = steps or w["steps"]
    directions = directions or w["directions"]
    md = cases.make_mesh("tgv3d", n)
    nci = md.ncell_int
    g = ty.Grid(md)
    g.set_spat(w["scheme"], w["highres"], w["limiter"], mode="fast")
    prim = cases.taylor_green(md.cell_centre)
    g.set_prim(prim)
    dts = [g.calc_zonetimestep(w["cfl"])] * steps
    U0 = ty.prim_to_cons(prim[:, :nci])
    cc = md.cell_centre[:nci]
    L = 2 * np.pi
    box = np.all(np.abs(cc - L / 2) < L / 4, axis=1).astype(float) * md.cell_volume[:nci]
    Ut = torch.tensor(U0, device="cuda", requires_grad=True)
    J = (adjoint.rk_solve(Ut, g, w["rk"], dts)[0] ** 2 * torch.tensor(box, device="cuda")).sum()
    J.backward()
    grad = Ut.grad.cpu().numpy()
    g.close()
    rng = np.random.default_rng(w["seed"])
    ds = [rng.standard_normal(U0.shape) * np.abs(U0).mean(axis=1, keepdims=True) for _ in range(directions)]
    jobs = [(md, U0, d, dts, adjoint.RK_TABLES[w["rk"]], box, w["scheme"], w["highres"], w["limiter"]) for d in ds]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(min(directions, os.cpu_count() or 1), initializer=_cs_worker_init,
                                       initargs=(str(ROOT / "tests"),)) as pool:
        ref = pool.map(_cs_direction, jobs)
    errs = [abs(float(np.sum(grad * d)) - r) / max(abs(r), 1e-300) for d, r in zip(ds, ref)]
    return {"sample": f"TGV {n}^3x5 tets ({nci} cells), {steps} {w['rk']} steps", "directions": directions,
            "max_rel_err": max(errs), "median_rel_err": float(np.median(errs)),
            "checker_s": round(time.perf_counter() - t0, 1)}


def run_adjoint(args):
    """Unsteady adjoint: primal run (library RK steps and the same steps composed through the
    device residual), the gradient of J by a reverse sweep over stored stage states (the
    device's storage policy for this size) and by binomial checkpointing, their cost against
    the primal, and seeded directional derivatives against central finite differences."""
    import torch
    import typhon_gb300 as ty
    from typhon_gb300 import adjoint, build, cases
    build.build()
    torch.cuda.set_device(0)
    w = cases.ADJOINT3D
    n = args.n or w["n"]
    md = cases.make_mesh("tgv3d", n)
    nci = md.ncell_int
    prim = cases.taylor_green(md.cell_centre)
    g = ty.Grid(md)
    g.set_spat(w["scheme"], w["highres"], w["limiter"], mode="fast")
    g.set_prim(prim)
    dt = g.calc_zonetimestep(w["cfl"])
    nsteps = args.adj_steps or w["steps"]
    dts = [dt] * nsteps
    U0 = torch.tensor(ty.prim_to_cons(prim[:, :nci]), device="cuda")
    cc = md.cell_centre[:nci]
    L = 2 * np.pi
    box = np.all(np.abs(cc - L / 2) < L / 4, axis=1).astype(float) * md.cell_volume[:nci]
    wbox = torch.tensor(box, device="cuda")
    st = adjoint.Stepper(g, w["rk"])

    def per_call_ms(fn, reps=20):
        """device time of one call, CUDA events on the library's stream (torch's current)"""
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def J_of(U):
        return float((U[0] ** 2 * wbox).sum())

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    with ClockSampler(0) as clk:
        adjoint.forward_steps(st, U0, dts[:2])                            # warm-up
        Uf, t_primal = timed(lambda: adjoint.forward_steps(st, U0, dts))
        # the library's own fused RK steps on the same fixed dt (the optimised primal)
        g.set_cons_device(U0.data_ptr())
        g.synchronize()
        t0 = time.perf_counter()
        for d in dts:
            g.treelevel_rungekutta(w["rk"], d)
        g.synchronize()
        t_lib = time.perf_counter() - t0
        lam = (2.0 * Uf[0] * wbox).unsqueeze(0) * torch.tensor([1.0, 0, 0, 0, 0], device="cuda").unsqueeze(1)
        lam = lam.contiguous()
        # one residual and one VJP at the final state (state upload included in both), for this
        # configuration and for the explicit benchmark's scheme and first order on the same mesh
        lam_r = torch.randn_like(U0)
        t_res_ms = per_call_ms(lambda: st.residual(Uf, dt))
        t_vjp_ms = per_call_ms(lambda: st.vjp(Uf, dt, lam_r))
        other = {}
        for label, spat in (("ROE MUSCL-UNS NONE BARTH (frozen)", ("ROE", "MUSCL-UNS", "NONE", "BARTH")),
                            ("HLLC first order", ("HLLC", "NONE", "NONE", "NONE"))):
            g2 = ty.Grid(md)
            g2.set_spat(*spat, mode="fast")
            g2.set_prim(prim)
            st2 = adjoint.Stepper(g2, w["rk"])
            r_ms = per_call_ms(lambda: st2.residual(Uf, dt))
            v_ms = per_call_ms(lambda: st2.vjp(Uf, dt, lam_r))
            other[label] = {"residual_ms": round(r_ms, 4), "vjp_ms": round(v_ms, 4), "ratio": round(v_ms / r_ms, 3)}
            g2.close()
        st = adjoint.Stepper(g, w["rk"])   # the handle's stream again for the runs below
        # the storage policy of the device: every stage state kept when it fits (it does here)
        policy = adjoint.plan_storage(nci, st.n, len(dts))
        (Uf_s, tape), t_fwd_store = timed(lambda: adjoint.forward_steps_stored(st, U0, dts))
        grad, t_rev = timed(lambda: adjoint.adjoint_steps_stored(st, dts, lam, tape))
        tape_bytes = sum(u.numel() * u.element_size() for us in tape for u in us)
        del tape
        same_primal = bool(torch.equal(Uf_s, Uf))
        # binomial checkpointing with a fixed number of stored states (memory-limited runs)
        if args.adj_no_checks:
            t_adj, binomial_diff = float("nan"), None
        else:
            grad_b, t_adj = timed(lambda: adjoint.adjoint_steps(st, U0, dts, lam, w["snaps"]))
            binomial_diff = float((grad_b - grad).abs().max())
    rng = np.random.default_rng(w["seed"])
    errs = []
    J0 = J_of(Uf)
    fd_dirs = 0 if args.adj_no_checks else (args.adj_fd_directions or w["directions"])
    for _ in range(fd_dirs):
        d = torch.tensor(rng.standard_normal((5, nci)), device="cuda") * U0.abs().mean(dim=1, keepdim=True)
        eps = 1e-6
        Jp = J_of(adjoint.forward_steps(st, U0 + eps * d, dts))
        Jm = J_of(adjoint.forward_steps(st, U0 - eps * d, dts))
        fd = (Jp - Jm) / (2 * eps)
        ad = float((grad * d).sum())
        errs.append(abs(ad - fd) / max(abs(fd), 1e-300))
    cs_check = None if args.adj_no_checks else complex_step_sample(
        w, n=args.adj_cs_n, steps=args.adj_cs_steps or w["steps"], directions=args.adj_cs_directions or w["directions"])
    out = {"metric": "adjoint gradient / primal time, unsteady gradient of int rho^2 (forward pass storing the "
                     "stage states plus the reverse sweep)", "unit": "ratio",
           "value": round((t_fwd_store + t_rev) / t_primal, 3), "higher_is_better": False, "n_gpus": 1, "steps": nsteps,
           "warmup": 2, "dtype": "f64", "data": "synthetic", "scaling": "weak", "vs_baseline": None,
           "config": {"workload": f"adjoint3d TGV {n}^3x5 tets, {w['scheme']} + {w['highres']} {w['limiter']} "
                                  f"(least-squares gradients), {w['rk']}",
                      "cells": nci, "dt": dt, "storage_policy": policy, "J": J0},
           "primal_s": round(t_primal, 4), "primal_library_rk_s": round(t_lib, 4),
           "primal_storing_stages_s": round(t_fwd_store, 4), "stage_storage_bytes": tape_bytes,
           "reverse_sweep_s": round(t_rev, 4), "reverse_sweep_vs_primal": round(t_rev / t_primal, 3),
           "gradient_total_vs_primal": round((t_fwd_store + t_rev) / t_primal, 3),
           "gradient_total_vs_library_primal": round((t_fwd_store + t_rev) / t_lib, 3),
           "vjp_vs_residual": {"residual_ms": round(t_res_ms, 4), "vjp_ms": round(t_vjp_ms, 4),
                               "ratio": round(t_vjp_ms / t_res_ms, 3), "other_residuals": other},
           "binomial": {"snapshots": w["snaps"], "adjoint_s": round(t_adj, 4),
                        "adjoint_vs_primal": round(t_adj / t_primal, 3),
                        "recomputed_steps": adjoint.checkpoint_cost(nsteps, w["snaps"]),
                        "max_abs_diff_vs_stored": binomial_diff},
           "stored_primal_bitwise_equal": same_primal,
           "fd_check": None if not errs else {"directions": fd_dirs, "eps": 1e-6, "max_rel_err": max(errs),
                        "median_rel_err": float(np.median(errs)),
                        "note": "van Albada's limiter has a kink where the two slopes change sign (local extrema): "
                                "central differences of random per-cell perturbations cross kinks over 200 steps, "
                                "so their agreement is limited there; complex_step_check is the branch-exact check"},
           "complex_step_check": cs_check,
           "clocks": clk.summary()}
    print(json.dumps(out))


def secondary_runs():
    """Short but complete runs of the other measurements, each in its own process,
    summarised for the default line: time to a 1e-10 residual of FP64 vs mixed implicit solves
    (the laminar flat plate at 40,000 cells, and ffbox3d at 24^3x5) and 50 KDIF steps of FP64 vs mixed conjugate gradients at reduced sizes (the full-size runs
    are the --workload options), and the unsteady adjoint's cost against its primal run at the
    configuration's size with fewer derivative checks."""
    runs = {"implicit": ["--workload", "flatplate-implicit", "--fp-nx", "40", "--fp-nz", "4", "--imp-time-limit", "120"],
            "implicit_ffbox3d": ["--workload", "ffbox3d-implicit", "--n", "24"],
            "kdif": ["--workload", "kdif3d", "--n", "35"],
            "adjoint": ["--workload", "adjoint3d", "--adj-fd-directions", "2", "--adj-cs-n", "6",
                        "--adj-cs-steps", "20", "--adj-cs-directions", "4"]}
    out = {}
    for name, extra in runs.items():
        try:
            r = subprocess.run([sys.executable, str(ROOT / "bench.py"), *extra], capture_output=True, text=True,
                               timeout=600)
            line = [ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1]
            d = json.loads(line)
        except (subprocess.TimeoutExpired, IndexError, ValueError) as e:
            out[name] = {"error": f"{type(e).__name__}"}
            continue
        v = d["variants"] if "variants" in d else {}
        if name == "implicit":
            out[name] = {"workload": d["config"]["workload"], "cells": d["config"]["cells"],
                         "steps": v["fgmres_mixed"]["steps"], "deepest_common_decade": d["deepest_common_decade"],
                         "seconds_fp64": v["fgmres_fp64"]["seconds"], "seconds_mixed": v["fgmres_mixed"]["seconds"],
                         "speedup_mixed_vs_fp64": d["speedup_mixed_vs_fp64_at_deepest"],
                         "mixed_state_vs_fp64": max(d["state_mixed_vs_fp64"]),
                         "reached_1e-10": all(x["reached"] for x in v.values())}
        elif name == "implicit_ffbox3d":
            out[name] = {"workload": d["config"]["workload"], "cells": d["config"]["cells"], "steps": d["steps"],
                         "seconds_fp64": v["fgmres_fp64"]["seconds"], "seconds_mixed": v["fgmres_mixed"]["seconds"],
                         "seconds_mixed_f32basis": v["fgmres_mixed_f32basis"]["seconds"],
                         "speedup_mixed_vs_fp64": d["speedup_mixed_vs_fp64"],
                         "mixed_state_vs_fp64": max(v["fgmres_mixed"]["state_vs_fp64"]),
                         "reached_1e-10": all(x["reached"] for x in v.values())}
        elif name == "kdif":
            out[name] = {"workload": d["config"]["workload"], "cells": d["config"]["cells"],
                         "seconds_cg_fp64": v["cg_fp64"]["seconds"], "seconds_cg_mixed": v["cg_mixed"]["seconds"],
                         "speedup_mixed_vs_fp64": d["speedup_mixed_vs_fp64"],
                         "cg_iteration_hbm_frac": v["cg_fp64"]["iteration"]["frac"]}
        else:
            out[name] = {"workload": d["config"]["workload"], "cells": d["config"]["cells"], "steps": d["steps"],
                         "gradient_vs_primal": d["value"],
                         "gradient_vs_library_primal": d["gradient_total_vs_library_primal"],
                         "reverse_sweep_vs_primal": d["reverse_sweep_vs_primal"],
                         "vjp_vs_residual": d["vjp_vs_residual"]["ratio"],
                         "binomial_vs_primal": d["binomial"]["adjoint_vs_primal"],
                         "complex_step_max_rel_err": d["complex_step_check"]["max_rel_err"],
                         "complex_step_sample": d["complex_step_check"]["sample"]}
    return out


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.workload == "adjoint3d":
        if rank == 0 and args.impl == "ours":
            run_adjoint(args)
        elif rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "Typhon has no adjoint"}))
        return
    if args.workload == "kdif3d":
        if rank == 0 and args.impl == "ours":
            run_kdif(args)
        elif rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the KDIF comparison has no CPU arm"}))
        return
    if args.workload == "flatplate-implicit":
        if rank == 0 and args.impl == "ours":
            run_flatplate(args)
        elif rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the implicit comparison has no CPU arm"}))
        return
    if args.workload == "ffbox3d-implicit":
        if rank == 0 and args.impl == "ours":
            run_implicit(args)
        elif rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the implicit comparison has no CPU arm"}))
        return
    if args.impl == "reference":
        if rank != 0:
            return
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
        cb, cells, faces = cpu_sample(args, args.steps, args.warmup, with_mesh=True)
        out = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": cb["unit"], "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "ms_per_step": cells / cb["value"] * 1e3,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
               "config": workload_config(args, cells, faces, world),
               "implementation": "the CPU restatement of Typhon's solver (oracle/, OpenMP on all host cores); Typhon "
                                 "itself is Fortran and no Fortran compiler exists in the image or on the GPU box",
               "cpu_baseline": cb,
               "e2e": {"value": cb["value"], "unit": cb["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return
    out = run_ours(args, rank, world, local)
    if rank == 0:
        if not args.no_cpu_baseline:
            os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
            out["cpu_baseline"] = cpu_sample(args, args.cpu_sample_steps)
        if world == 1 and not args.no_secondary and args.workload == "tgv3d" and args.n is None:
            out["secondary"] = secondary_runs()
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
