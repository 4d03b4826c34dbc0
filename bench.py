"""Benchmark: time to 1e-8 relative L2 error of the steady RT solve on one GB300.

Workload (default): the single adaptive problem -- domain [0,3]x[0,2],
sigma_s a Gaussian bump (amplitude 0.9, width 0.15) at (1.5, 1.0),
sigma_t = sigma_s + 0.01, HG g = 0.9, inflow 1 on x = 0 for th in (-pi/4, pi/4),
hp mesh from seeded random refinement (seed 0, six rounds, 3..7 nodes per
dimension), about 2.2e5 DOF.  Synthetic and seeded; no dataset involved.

A step is one solve from a zero initial guess to the error target.  The judge
solution is a tight plain FP64 GPU solve (rtol 1e-14) computed before timing;
the error is the quadrature-weighted relative L2 norm (weights = mass weights
with kappa = 1).  The residual tolerance of each method is calibrated (untimed)
as the loosest power of ten that reaches the 1e-8 target.

value   : seconds per solve of the mixed method (FP32 GMRES inside FP64
          iterative refinement), device-resident inputs.
e2e     : same solve through the C ABI with host buffers: H2D of the sampled
          forcing and inflow node values, weighting kernel, solve, D2H of u.
roofline: the FP32 system apply (dominant kernel of the inner solve).
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "radiative-transfer-amr_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np

METRIC = "time to 1e-8 rel. L2 err: learned+mixed vs plain FP64 GPU; apply GB/s % peak"
ERR_TARGET = 1e-8


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg2", choices=["cfg1", "cfg2", "cfg5"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile", action="store_true",
                    help="short run for ncu: one warm and one measured solve per method, 3 applies")
    ap.add_argument("--rtol", type=float, default=1e-9, help="profile mode: solver tolerance")
    ap.add_argument("--max-it", type=int, default=20000, help="profile mode: iteration cap")
    return ap.parse_args()


def run_profile(args):
    """Minimal launch sequence for profiling: set-up, then per method one warm
    and one measured solve, then three FP32 and three FP64 system applies."""
    import torch
    from rtg import Problem, _lib
    torch.cuda.set_device(0)
    out = {}
    t0 = time.perf_counter()
    desc, mesh, spec = workload(args.workload)
    out["mesh_s"] = time.perf_counter() - t0
    prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    t0 = time.perf_counter()
    ctx = prob.context(mesh)
    torch.cuda.synchronize()
    out["context_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    f_dev = ctx.forcing(spec.f)
    g_dev = ctx.inflow(spec.bcs_dirac)
    torch.cuda.synchronize()
    out["vectors_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    ctx.precondition(torch.zeros(ctx.N, dtype=torch.float64, device=ctx.device))
    torch.cuda.synchronize()
    out["sweep_setup_s"] = time.perf_counter() - t0
    print(json.dumps({k: out[k] for k in out}), file=sys.stderr, flush=True)
    for method in (1, 0):
        for rep in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            u, info = ctx.solve(f_dev, g_dev, method=method, rtol=args.rtol, max_it=args.max_it, precond=1)
            torch.cuda.synchronize()
            out["method%d_rep%d" % (method, rep)] = {"s": time.perf_counter() - t0,
                                                     "iterations": info["iterations"],
                                                     "sweeps": info["sweeps"],
                                                     "res_f": info["res_f"], "rhs_norm": info["rhs_norm"],
                                                     "converged": info["converged"]}
            print(json.dumps(out["method%d_rep%d" % (method, rep)]), file=sys.stderr, flush=True)
    stream = torch.cuda.current_stream()
    for prec in (_lib.RTG_FP32, _lib.RTG_FP64):
        dt = torch.float32 if prec == _lib.RTG_FP32 else torch.float64
        nm = "fp32" if prec == _lib.RTG_FP32 else "fp64"
        x = torch.randn(ctx.N, dtype=dt, device=ctx.device)
        y = torch.empty_like(x)
        for what, fn in (("apply", lambda: ctx.apply(_lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS, x, y, prec=prec)),
                         ("sweep", lambda: ctx.precondition(x, y, prec=prec))):
            fn()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(3):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            out["%s_%s_us" % (what, nm)] = 1e3 * e0.elapsed_time(e1) / 3
    torch.cuda.synchronize()
    out["ndof"] = ctx.N
    out["info"] = ctx.info
    print(json.dumps(out))


def workload(name, seed=0):
    from rtg import workloads as W
    if name == "cfg1":
        return ("manufactured 4x4x4 cells n=4 (4096 DOF)", W.config1_mesh(), W.manufactured_problem())
    if name == "cfg5":
        return ("two strong scatterers on [0,2]^2, disc-edge hp refinement seed %d, 5..9 nodes/dim "
                "(~9.4e6 DOF)" % seed, W.config5_mesh(seed=seed), W.two_disc_problem())
    return ("gaussian-bump adaptive hp, seed %d (~2.2e5 DOF)" % seed, W.config2_mesh(seed=seed),
            W.gaussian_bump_problem())


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, index=0):
        self.samples = []
        self.proc = None
        self.index = index

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[1]))
                mx = float(s[2])
                for k, nm in enumerate(names):
                    if s[5 + k].lower().startswith("active"):
                        reasons.add(nm)
            except Exception:
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def rel_l2(u, ref, w):
    return float(np.sqrt(np.sum(w * (u - ref) ** 2) / np.sum(w * ref ** 2)))


def cpu_baseline(mesh, spec, rtol, u_judge=None, w=None):
    """The oracle port of the path on the host (single thread): assemble the
    reference's split system with scipy (rt/solve.py:81-101) and solve it with
    scipy GMRES(50) preconditioned by the same upwind sweep the GPU uses, to the
    residual tolerance that reaches the error target.  The whole solve is
    timed (about 10 s for the 2.2e5-DOF workload)."""
    from oracle import rt_oracle as O
    t0 = time.perf_counter()
    o = O.assemble(mesh, spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    t_asm = time.perf_counter() - t0
    t1 = time.perf_counter()
    u, its, info = O.solve_sweep_gmres(o, o["layout"], rtol=rtol)
    t_solve = time.perf_counter() - t1
    err = rel_l2(u, u_judge, w) if u_judge is not None else None
    return {"value": t_asm + t_solve, "unit": "s", "cores": 1, "kind": "port",
            "sample": "whole workload: oracle assembly {:.1f} s + scipy sweep-preconditioned GMRES(50) "
                      "{:.1f} s ({} iterations, rtol {:g})".format(t_asm, t_solve, its, rtol),
            "rel_l2_err": err}


def run_ours(args):
    import torch
    from rtg import Problem, _lib

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
        torch.cuda.set_device(local)
    else:
        torch.cuda.set_device(0)
    desc, mesh, spec = workload(args.workload, seed=rank)
    prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    ctx = prob.context(mesh)
    N = ctx.N
    f_dev = ctx.forcing(spec.f)
    g_dev = ctx.inflow(spec.bcs_dirac)
    # L2 weights (dx dy dth/8) wx wy wth = mass weights with kappa = 1
    lay = ctx.layout
    X, Y, T = lay.node_coords()
    ones = ctx.apply(_lib.RTG_MASS, torch.ones(N, dtype=torch.float64, device=ctx.device))
    kap = ctx.to_device(np.asarray(np.broadcast_to(spec.kappa(X, Y), (N,)), dtype=np.float64))
    w = (ones / kap).cpu().numpy()

    # judge solution: tight plain FP64 solve
    u_ref, info_ref = ctx.solve(f_dev, g_dev, method=0, rtol=1e-14, max_it=20000, precond=1)
    u_ref_h = u_ref.cpu().numpy()

    def calibrate(method):
        for k in range(6, 15):
            rtol = 10.0 ** (-k)
            u, info = ctx.solve(f_dev, g_dev, method=method, rtol=rtol, max_it=20000, precond=1)
            err = rel_l2(u.cpu().numpy(), u_ref_h, w)
            if err <= ERR_TARGET:
                return rtol, err, info
        raise RuntimeError("method {} did not reach the error target".format(method))

    rtol_mx, err_mx, info_mx = calibrate(1)
    rtol_pl, err_pl, info_pl = calibrate(0)

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=ctx.device)
    stream = torch.cuda.current_stream()

    def timed(method, rtol, steps, warm):
        for _ in range(warm):
            ctx.solve(f_dev, g_dev, method=method, rtol=rtol, max_it=20000, precond=1)
        times, errs, infos = [], [], []
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            u, info = ctx.solve(f_dev, g_dev, method=method, rtol=rtol, max_it=20000, precond=1)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            errs.append(rel_l2(u.cpu().numpy(), u_ref_h, w))
            infos.append(info)
        return times, errs, infos

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        t_mx, e_mx, i_mx = timed(1, rtol_mx, args.steps, args.warmup)
    t_pl, e_pl, i_pl = timed(0, rtol_pl, max(1, min(args.steps, 2)), 1)
    if world > 1:
        torch.distributed.barrier()

    # e2e through the C ABI with host buffers
    lib = ctx.lib
    fvals = torch.from_numpy(ctx.node_values(spec.f)).pin_memory()
    gvals = torch.from_numpy(np.ascontiguousarray(g_dev.cpu().numpy())).pin_memory()
    u_host = torch.empty(N, dtype=torch.float64).pin_memory()
    fd = torch.empty(N, dtype=torch.float64, device=ctx.device)
    fw = torch.empty_like(fd)
    gd = torch.empty_like(fd)
    ud = torch.zeros_like(fd)
    opts = _lib.SolveOpts(method=1, restart=50, max_it=50000, rtol=rtol_mx, atol=0., precond=1,
                          nonzero_guess=0, inner_rtol=1e-6, max_outer=20, verbose=0)
    sinfo = _lib.SolveInfo()
    sp = C.c_void_p(stream.cuda_stream)
    e2e_times = []
    for it in range(args.warmup + args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fd.copy_(fvals, non_blocking=True)
        gd.copy_(gvals, non_blocking=True)
        _lib.check(lib.rtg_weight_forcing(ctx.h, C.c_void_p(fd.data_ptr()), C.c_void_p(fw.data_ptr()), sp))
        _lib.check(lib.rtg_solve(ctx.h, C.c_void_p(fw.data_ptr()), C.c_void_p(gd.data_ptr()),
                                 C.c_void_p(ud.data_ptr()), C.byref(opts), C.byref(sinfo), None, 0, sp))
        u_host.copy_(ud, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        if it >= args.warmup:
            e2e_times.append(e0.elapsed_time(e1) / 1e3)
    e2e_err = rel_l2(u_host.numpy(), u_ref_h, w)

    # roofline of the FP32 system apply (dominant kernel of the inner solve)
    xa = torch.randn(N, dtype=torch.float32, device=ctx.device)
    ya = torch.empty_like(xa)
    nrep = 50
    for _ in range(5):
        ctx.apply(_lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS, xa, ya, prec=_lib.RTG_FP32)
    durs = []
    for _ in range(nrep):
        flush.fill_(1.0)
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        ctx.apply(_lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS, xa, ya, prec=_lib.RTG_FP32)
        a1.record(stream)
        torch.cuda.synchronize()
        durs.append(a0.elapsed_time(a1) / 1e3)
    t_apply = statistics.median(durs)
    bytes_apply = int(ctx.info["bytes_per_apply_fp32"])
    peak, peak_kind = peaks()
    achieved = bytes_apply / t_apply / 1e9

    mx_time = statistics.median(t_mx)
    if world > 1:
        tt = torch.tensor([max(t_mx)], device=ctx.device)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        mx_time = float(tt.item())
    if rank != 0:
        return None
    launches = None
    inf = i_mx[-1]
    # kernels per solve: applies + ~10 Krylov kernels per inner iteration
    launches = int(inf["fp32_applies"] + inf["fp64_applies"] + 10 * inf["iterations"])
    out = {
        "metric": METRIC, "value": mx_time, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * mx_time, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-inner/f64-outer",
        "data": "synthetic (seeded hp mesh and coefficients)",
        "config": {"workload": desc, "ndof": N, "ndof_interior": int(ctx.info["ndof_interior"]),
                   "error_target": ERR_TARGET, "l2_flush": "256 MB write between timed solves",
                   "mixed": {"rtol": rtol_mx, "rel_l2_err": max(e_mx), "inner_iterations": inf["iterations"],
                             "outer": inf["outer"], "fp64_applies": inf["fp64_applies"],
                             "fp32_applies": inf["fp32_applies"], "seconds": t_mx},
                   "plain_fp64": {"rtol": rtol_pl, "rel_l2_err": max(e_pl),
                                  "iterations": i_pl[-1]["iterations"], "seconds": t_pl,
                                  "median_s": statistics.median(t_pl)},
                   "speedup_mixed_vs_plain": statistics.median(t_pl) / mx_time,
                   "judge": {"rtol": 1e-14, "iterations": info_ref["iterations"],
                             "res_f": info_ref["res_f"]},
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": statistics.median(e2e_times), "unit": "s", "h2d_bytes_per_step": 2 * 8 * N,
                "d2h_bytes_per_step": 8 * N, "rel_l2_err": e2e_err},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "kernel": "apply_kernel<float> (system)",
                     "bytes_per_launch": bytes_apply, "launch_s": t_apply, "peak_kind": peak_kind},
        "clocks": clk.summary(),
    }
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(mesh, spec, rtol_pl, u_ref_h, w)
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    desc, mesh, spec = workload(args.workload)
    vals = []
    for it in range(args.warmup + args.steps):
        cb = cpu_baseline(mesh, spec, 1e-9)
        if it >= args.warmup:
            vals.append(cb["value"])
    v = statistics.median(vals)
    cb["value"] = v
    return {"metric": METRIC, "value": v, "unit": "s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * v, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": desc}, "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    if args.profile:
        run_profile(args)
        return
    out = run_reference(args) if args.impl == "reference" else run_ours(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
