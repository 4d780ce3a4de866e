"""Benchmark: Galerkin COO triplets/s of the GB300 assembly path (+ solve DOFs/s).

Workload (one "step"): AssembleMatrixLocally with the reaction-diffusion
provider over the whole large hybrid mesh of the precision configuration:
2048 x 2048 squares on [0,1]^2, each a quadrilateral or two triangles (p=1/2,
seeded), interior nodes jittered by +-0.2h, FeSpaceLagrangeO2 (16.8M dofs),
alpha per-cell LogNormal(0,1), gamma = 0, default degree-4 rules:
~321M triplets (5.1 GB) per step.  Inputs and outputs are larger than L2
(129 MB), so every step streams from/to HBM.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--size 2048] [--solve-size 512] [--no-cpu-baseline]

--impl reference times the CPU restatement of the reference's assembly
(oracle/, C++) on the host cores, all threads, on the same workload.
Multi-GPU: replicas only (each rank assembles its own copy; no collective on
the data path); value = total triplets of all ranks / max time over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Galerkin COO triplets/s; DOFs/s solved to 1e-8 err; mixed vs FP64 on 1 GB300"
UNIT = "triplets/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=2048)
    ap.add_argument("--solve-size", type=int, default=512)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def algorithmic_bytes(space, mesh, kind):
    """Bytes one launch of the element kernel must move for its cells:
    16 n^2 triplet bytes written + vertex ids (4/vertex) + vertex coordinates
    (16/vertex) + alpha (8) + the cell's dof indices (4 n) read."""
    if kind == "tria":
        n, nv, cells = space.n_tria, 3, mesh.num_trias
    else:
        n, nv, cells = space.n_quad, 4, mesh.num_quads
    per_cell = 16 * n * n + 4 * nv + 16 * nv + 8 + 4 * n
    return per_cell * cells, per_cell


def fp64_flops(space, mesh, kind):
    """FP64 operations the kernels issue per cell (counted from the source):
    triangles (folded rule): metric ~14 + 3 FMA per upper-triangle entry;
    quadrilaterals: per point ~22 (metric) + 3 FMA per upper-triangle entry."""
    if kind == "tria":
        n = space.n_tria
        e = n * (n + 1) // 2
        return (2 * (14 + 3 * e)) * mesh.num_trias
    n = space.n_quad
    e = n * (n + 1) // 2
    nq = 9
    return (2 * nq * (22 + 3 * e)) * mesh.num_quads


def run_cpu_baseline(wl, max_seconds=20.0, threads=1):
    """The oracle (C++ restatement of the reference path), timed on host cores
    over a bounded prefix of the same cells."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle as O
    from parity import oracle_coeff
    t0 = time.perf_counter()
    m = O.Mesh(wl["mesh"]["xy"], wl["mesh"]["cells"])
    s = O.Space(m, wl["degree"])
    setup = time.perf_counter() - t0
    a, g = oracle_coeff(wl["alpha"]), oracle_coeff(wl["gamma"])
    # calibrate on a small prefix, then size the sample to ~max_seconds
    cal = min(m.num_cells, 20000)
    t0 = time.perf_counter()
    A = O.assemble_rd(s, a, g, wl["qr_tria"], wl["qr_quad"], (0, cal))
    dt = time.perf_counter() - t0
    rate_cells = cal / max(dt, 1e-9)
    ncell = int(min(m.num_cells, max(cal, rate_cells * max_seconds * threads)))
    del A
    if threads == 1:
        t0 = time.perf_counter()
        A = O.assemble_rd(s, a, g, wl["qr_tria"], wl["qr_quad"], (0, ncell))
        dt = time.perf_counter() - t0
        ntrip = len(A)
    else:
        dt, ntrip = O.assemble_rd_parallel(s, a, g, wl["qr_tria"], wl["qr_quad"], (0, ncell), threads)
    return {"value": ntrip / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "first %d of %d cells (%d triplets) of the same workload; oracle mesh+dof setup %.1f s "
                      "not timed" % (ncell, m.num_cells, ntrip, setup)}


def solve_leg(L, W, ctx, n):
    """DOFs/s of assemble + fix + COO->CSR + PCG on the config-2 generator at
    size n, FP64 PCG vs mixed precision, error vs the FP64 PCG at 1e-12."""
    wl = W.config2(n)
    keep = []
    mesh = W.build_mesh(ctx, wl["mesh"])
    space = L.Space.lagrange(mesh, 2)
    prov = L.rd_provider(W.to_coeff(ctx, wl["alpha"], keep), W.to_coeff(ctx, wl["gamma"], keep))
    lprov = L.load_provider(W.to_coeff(ctx, wl["f"], keep))
    flags = space.boundary_dof_flags()
    zeros = ctx.zeros(space.num_dofs)
    out = {"workload": "hybrid %dx%d O2 (%d dofs)" % (n, n, space.num_dofs)}
    xs = {}
    for name, prec in (("fp64", L.SOLVE_FP64), ("mixed", L.SOLVE_MIXED)):
        ctx.synchronize()
        t0 = time.perf_counter()
        coo = L.COOMatrix(ctx, space.num_dofs, space.num_dofs, space.num_triplets + space.num_dofs)
        L.assemble_matrix_rd(space, prov, coo)
        b = ctx.zeros(space.num_dofs)
        L.assemble_vector_load(space, lprov, b)
        coo.fix_flagged_solution_components(flags, zeros, b)
        A = coo.make_sparse()
        x = ctx.zeros(space.num_dofs)
        st = A.solve_pcg(b, x, precision=prec, rtol=1e-10, raise_on_failure=False)
        ctx.synchronize()
        dt = time.perf_counter() - t0
        xs[name] = x.download()
        out[name] = {"dofs_per_s": space.num_dofs / dt, "seconds": dt, "iterations": st["iterations"],
                     "refinements": st["refinements"], "rel_residual": st["rel_residual"],
                     "converged": st["converged"]}
        del coo, A
    ref = ctx.zeros(space.num_dofs)
    coo = L.COOMatrix(ctx, space.num_dofs, space.num_dofs, space.num_triplets + space.num_dofs)
    L.assemble_matrix_rd(space, prov, coo)
    b = ctx.zeros(space.num_dofs)
    L.assemble_vector_load(space, lprov, b)
    coo.fix_flagged_solution_components(flags, zeros, b)
    coo.make_sparse().solve_pcg(b, ref, precision=L.SOLVE_FP64, rtol=1e-13, raise_on_failure=False)
    r = ref.download()
    for name in xs:
        out[name]["rel_err_vs_fp64_1e-13"] = float(np.linalg.norm(xs[name] - r) / np.linalg.norm(r))
    out["mixed_vs_fp64"] = out["mixed"]["dofs_per_s"] / out["fp64"]["dofs_per_s"]
    return out


def run_ours(args):
    rank, world, local = dist_env()
    import lehrfempp_gb300 as L
    from lehrfempp_gb300 import workloads as W
    L.load()
    ctx = L.Context(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    wl = W.config2(args.size)
    keep = []
    mesh = W.build_mesh(ctx, wl["mesh"])
    space = L.Space.lagrange(mesh, wl["degree"])
    alpha_h = np.ascontiguousarray(wl["alpha"][1])
    alpha_d = ctx.to_device(alpha_h)
    prov = L.rd_provider(L.coeff(L.PER_CELL, data=alpha_d), W.to_coeff(ctx, wl["gamma"], keep))
    coo = L.COOMatrix(ctx, space.num_dofs, space.num_dofs, space.num_triplets)
    ntrip = space.num_triplets

    def step():
        coo.set_zero()
        L.assemble_matrix_rd(space, prov, coo)

    for _ in range(args.warmup):
        step()
    ctx.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = ctx.launches()
    ctx.timer_begin()
    for _ in range(args.steps):
        step()
    ms_total = ctx.timer_end()
    launches = ctx.launches() - l0
    clk = clocks.stop()
    ms = ms_total / args.steps
    if dist:
        import torch
        t = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    value = world * ntrip / (ms * 1e-3)

    # per-kernel attribution (CUDA events around each launch, separate pass)
    ctx.profile(True)
    ctx.profile_reset()
    for _ in range(max(3, args.steps // 4)):
        step()
    fam = {}
    for f in ("rd_tria_df", "rd_quad_df", "rd_general_tria", "rd_general_quad"):
        t, n = ctx.profile_read(f)
        if n:
            fam[f] = (t / n, n)
    ctx.profile(False)
    dom = max(fam, key=lambda k: fam[k][0])
    kind = "quad" if dom.endswith("quad") else "tria"
    alg_bytes, per_cell = algorithmic_bytes(space, mesh, kind)
    hbm_peak = 6777.6
    peaks_src = "MEASURED_PEAKS.json hbm_gbs (burst), of measured"
    try:
        hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, KeyError, ValueError):
        peaks_src = "fallback 6800 GB/s"
        hbm_peak = 6800.0
    achieved = alg_bytes / (fam[dom][0] * 1e-3) / 1e9
    fp64_peak = ctx.fp64_peak_tflops()
    fl = fp64_flops(space, mesh, kind)
    fp64_ach = fl / (fam[dom][0] * 1e-3) / 1e12
    whole_bytes = sum(algorithmic_bytes(space, mesh, k)[0] for k in ("tria", "quad"))

    # load vector (AssembleVectorLocally) time, informational
    b = ctx.zeros(space.num_dofs)
    lprov = L.load_provider(W.to_coeff(ctx, wl["f"], keep))
    L.assemble_vector_load(space, lprov, b)
    ctx.timer_begin()
    for _ in range(5):
        L.assemble_vector_load(space, lprov, b)
    vec_ms = ctx.timer_end() / 5

    # end to end through the C-ABI with host buffers
    e2e = None
    if not args.no_e2e:
        a_pin = ctx.pinned(alpha_h.shape, np.float64)
        a_pin.array[:] = alpha_h
        t_pin = ctx.pinned((ntrip,), L.TRIPLET_DTYPE)
        e2e_steps = max(2, min(args.steps, 5))
        for it in range(e2e_steps + 1):
            if it == 1:
                t0 = time.perf_counter()
            alpha_d.upload_async(a_pin)
            step()
            coo.download_into(t_pin)  # synchronizes
        e2e_s = (time.perf_counter() - t0) / e2e_steps
        e2e = {"value": world * ntrip / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(alpha_h.nbytes),
               "d2h_bytes_per_step": int(ntrip * 16), "ms_per_step": e2e_s * 1e3}
        del t_pin
    solve = None
    if args.solve_size > 0:
        solve = solve_leg(L, W, ctx, args.solve_size)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = run_cpu_baseline(wl, max_seconds=15.0, threads=1)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": "hybrid %dx%d squares (quad or 2 trias, p=0.5), jitter 0.2h, O2, alpha "
                                   "per-cell LogNormal(0,1), gamma 0, default rules" % (args.size, args.size),
                       "cells": mesh.num_cells, "trias": mesh.num_trias, "quads": mesh.num_quads,
                       "dofs": space.num_dofs, "triplets_per_step": ntrip,
                       "l2": "inputs+outputs %.1f GB per step >> 129 MB L2" % (whole_bytes / 1e9),
                       "parallelism": "replicas" if world > 1 else "single"},
            "clocks": clk, "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": None, "kernel": dom,
                         "algorithmic_bytes_per_launch": alg_bytes, "bytes_per_cell": per_cell,
                         "avg_launch_ms": fam[dom][0], "peak_source": peaks_src,
                         "fp64": {"achieved_tflops": fp64_ach, "peak_tflops_measured": fp64_peak,
                                  "frac": fp64_ach / fp64_peak}},
            "kernels_ms": {k: v[0] for k, v in fam.items()},
            "fp64_route_cells": int(ctx.profile_read("fp64_fallback_cells")[1]),
            "whole_step_hbm_gbs": whole_bytes / (ms * 1e-3) / 1e9,
            "load_vector_ms": vec_ms,
            "e2e": e2e, "cpu_baseline": cpu, "solve": solve,
        }
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from lehrfempp_gb300 import workloads as W
    wl = W.config2(args.size)
    threads = os.cpu_count() or 1
    rates = []
    info = None
    for it in range(args.warmup + args.steps):
        info = run_cpu_baseline(wl, max_seconds=4.0, threads=threads)
        if it >= args.warmup:
            rates.append(info["value"])
    value = statistics.median(rates)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded generator, no dataset)", "impl": "reference",
            "config": {"workload": "hybrid %dx%d squares, O2, alpha per-cell LogNormal(0,1), gamma 0" %
                                   (args.size, args.size)},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": info["sample"] + "; reference not buildable here (needs Eigen/Boost), "
                                                        "C++ restatement in oracle/ timed instead"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
