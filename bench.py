"""Benchmark: time to 1e-8 relative L2 error of the steady RT solve on one GB300.

Workload (default, --workload cfg2): the single adaptive problem -- domain
[0,3]x[0,2], sigma_s a Gaussian bump (amplitude 0.9, width 0.15) at (1.5, 1.0),
sigma_t = sigma_s + 0.01, HG g = 0.9, inflow 1 on x = 0 for th in
(-pi/4, pi/4), hp mesh from seeded random refinement (seed 0, six rounds, 3..7
nodes per dimension), about 2.2e5 DOF.  Synthetic and seeded; no dataset.

A step is one solve from a zero initial guess to the error target.  The
reference solution is a tight plain FP64 GPU solve (rtol 1e-14) computed before timing;
the error is the quadrature-weighted relative L2 norm (weights = mass weights
with kappa = 1).  Each method's residual tolerance is calibrated (untimed) as
the loosest power of ten that reaches the 1e-8 target.  Three methods:
  plain    FP64 GMRES, sweep preconditioner (the reference-matching method)
  mixed    FP32 GMRES inside FP64 iterative refinement, sweep preconditioner
  learned  as mixed, flexible GMRES with the sweep plus the learned correction
           (network rtg/nets/sweep_correction.npz, trained by rtg.train)

value   : seconds per learned+mixed solve, device-resident inputs.
e2e     : the same solve through the C ABI with host buffers: H2D of the
          sampled forcing and inflow node values, weighting kernel, solve, D2H
          of u.
roofline: the persistent sweep kernel (FP32), the kernel that dominates the
          solve; apply_roofline: the FP32 system apply.

--workload cfg3: 256 independent instances in one batched solve vs the same
instances solved one by one.  --workload cfg5: the ~9.4e6-DOF two-scatterer
problem: apply and sweep throughput and a bounded solve.
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
    ap.add_argument("--workload", default="cfg2", choices=["cfg1", "cfg2", "cfg3", "cfg5"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile", action="store_true",
                    help="short run for ncu: two solves per method (learned+mixed, mixed, plain), "
                         "then 3 FP32 and 3 FP64 applies and sweeps")
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
    from rtg import learned as LN
    LN.set_params(ctx, LN.load(LN.DEFAULT_NET)[0])
    # learned+mixed (the headline method), mixed, plain FP64
    for name, method, pc in (("learned_mixed", 1, 3), ("mixed", 1, 1), ("plain_fp64", 0, 1)):
        for rep in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            u, info = ctx.solve(f_dev, g_dev, method=method, rtol=args.rtol, max_it=args.max_it, precond=pc,
                                restart=30, inner_rtol=1e-5)
            torch.cuda.synchronize()
            out["%s_rep%d" % (name, rep)] = {"s": time.perf_counter() - t0,
                                             "iterations": info["iterations"],
                                             "sweeps": info["sweeps"],
                                             "res_f": info["res_f"], "rhs_norm": info["rhs_norm"],
                                             "converged": info["converged"]}
            print(json.dumps(out["%s_rep%d" % (name, rep)]), file=sys.stderr, flush=True)
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


def cpu_baseline(mesh, spec, rtol, u_ref=None, w=None):
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
    err = rel_l2(u, u_ref, w) if u_ref is not None else None
    return {"value": t_asm + t_solve, "unit": "s", "cores": 1, "kind": "port",
            "sample": "whole workload: oracle assembly {:.1f} s + scipy sweep-preconditioned GMRES(50) "
                      "{:.1f} s ({} iterations, rtol {:g})".format(t_asm, t_solve, its, rtol),
            "rel_l2_err": err}


def _batch_instance_cpu(job):
    """One instance of the batched workload through the oracle port (worker of
    cpu_baseline_batch): rebuilt from its seed, assembled, solved with the
    sweep-preconditioned GMRES(50) to rtol."""
    seed, rtol = job
    from rtg import workloads as W
    from oracle import rt_oracle as O
    mesh, spec = W.batch_instance(seed)
    o = O.assemble(mesh, spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    _, its, info = O.solve_sweep_gmres(o, o["layout"], rtol=rtol)
    return its, info


def cpu_baseline_batch(seeds, rtol, n_total, workers=None):
    """The batched workload's CPU baseline on all host cores: a bounded sample
    of its instances (seeds) through the oracle port in a spawn process pool,
    wall time scaled to n_total instances."""
    import multiprocessing as mp
    workers = workers or max(1, min(len(seeds), os.cpu_count() or 1))
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(workers) as pool:
        res = pool.map(_batch_instance_cpu, [(s, rtol) for s in seeds])
    wall = time.perf_counter() - t0
    return {"value": wall * n_total / len(seeds), "unit": "s", "cores": workers, "kind": "port",
            "sample": "{} of {} instances (seeds {}..{}), oracle assembly + scipy sweep-preconditioned GMRES(50) "
                      "to rtol {:g} in a {}-process pool, wall {:.1f} s (pool start-up included) scaled by {:.0f}"
                      .format(len(seeds), n_total, seeds[0], seeds[-1], rtol, workers, wall, n_total / len(seeds)),
            "iterations_max": max(r[0] for r in res), "all_converged": all(r[1] == 0 for r in res)}


def _events(stream):
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def kernel_time(fn, stream, flush, reps=20):
    """Median CUDA-event duration of fn() on the stream, L2 flushed before each."""
    import torch
    for _ in range(3):
        fn()
    durs = []
    for _ in range(reps):
        flush.fill_(1.0)
        e0, e1 = _events(stream)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        durs.append(e0.elapsed_time(e1) / 1e3)
    return statistics.median(durs)


def amr_indicators(ctx, mesh, u_host, stream, flush, with_cpu):
    """The AMR step after the solve on the solution: the librtg indicator
    kernels (CUDA events, L2 flushed), the whole rtg.ErrorIndicator methods
    (host flags included, wall clock), and the CPU restatement's time (oracle
    port, one core) on the same mesh and vector."""
    import torch
    from rtg import ErrorIndicator, Projection, _lib
    N = ctx.N
    lay = ctx.layout
    ud = ctx.to_device(u_host)
    ce = torch.empty(lay.nelem, dtype=torch.float64, device=ctx.device)
    cc = torch.empty(lay.ncols, dtype=torch.float64, device=ctx.device)
    cl = torch.empty(lay.ncols, dtype=torch.float64, device=ctx.device)
    el = torch.empty(lay.nelem, dtype=torch.float64, device=ctx.device)
    lib, h, sp = ctx.lib, ctx.h, C.c_void_p(stream.cuda_stream)
    p = lambda t: C.c_void_p(t.data_ptr())
    t0 = time.perf_counter()
    _lib.check(lib.rtg_error_spatial_jump(h, p(ud), p(cc), sp))   # first call builds the pair tables
    torch.cuda.synchronize()
    setup = time.perf_counter() - t0
    t_ang = kernel_time(lambda: _lib.check(lib.rtg_error_angular_jump(h, p(ud), p(ce), p(cc), sp)), stream, flush)
    t_spt = kernel_time(lambda: _lib.check(lib.rtg_error_spatial_jump(h, p(ud), p(cc), sp)), stream, flush)
    t_hp = kernel_time(lambda: _lib.check(lib.rtg_hp_steer(h, p(ud), p(cl), p(el), sp)), stream, flush)
    proj = Projection(mesh)
    proj.from_vector(u_host)
    walls = {}
    for kind in ("angular", "spatial"):
        ts = []
        for _ in range(4):
            ind = ErrorIndicator(proj, "all", "hp", (0.5, 0.5), ctx=ctx)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            (ind.error_angular_jump if kind == "angular" else ind.error_spatial_jump)()
            ts.append(time.perf_counter() - t0)
        walls[kind] = statistics.median(ts[1:])
    out = {"workload": "indicators on the solution of the same problem", "ndof": N,
           "setup_s": setup,
           "angular_jump_us": 1e6 * t_ang, "spatial_jump_us": 1e6 * t_spt, "hp_steer_us": 1e6 * t_hp,
           "error_angular_jump_method_s": walls["angular"], "error_spatial_jump_method_s": walls["spatial"],
           "dof_per_s_spatial_jump": N / t_spt}
    if with_cpu:
        from oracle import amr_oracle as AO
        t0 = time.perf_counter()
        AO.indicator(mesh, u_host, "ang", "all", "hp", (0.5, 0.5))
        t1 = time.perf_counter()
        AO.indicator(mesh, u_host, "spt", "all", "hp", (0.5, 0.5))
        t2 = time.perf_counter()
        out["cpu_baseline"] = {"kind": "port", "cores": 1, "angular_s": t1 - t0, "spatial_s": t2 - t1,
                               "sample": "whole mesh: oracle restatement (numpy) of error_angular_jump and "
                                         "error_spatial_jump with the flags and hp steering they trigger"}
    return out


def profiled_traffic(name):
    """DRAM bytes per launch recorded from an ncu capture in profiles/<name>.md
    (line "traffic_bytes_per_launch: N"), or None."""
    try:
        with open(os.path.join(REPO, "profiles", name + ".md")) as fh:
            for line in fh:
                if line.startswith("traffic_bytes_per_launch:"):
                    return int(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def sweep_bytes(ctx, prec_bytes):
    """Algorithmic bytes of one sweep kernel: read r, write z, read the element
    block inverses, the upwind maps of the one-phase elements and their upwind
    value indices (8 bytes each); upwind face values re-read through L2 count 0."""
    from rtg import _lib
    lev, lag, inv = C.c_int(), C.c_int(), C.c_int64()
    _lib.check(ctx.lib.rtg_sweep_info(ctx.h, C.byref(lev), C.byref(lag), C.byref(inv), None))
    one, gm, up = C.c_int(), C.c_int64(), C.c_int64()
    prec = _lib.RTG_FP32 if prec_bytes == 4 else _lib.RTG_FP64
    _lib.check(ctx.lib.rtg_sweep_maps(ctx.h, prec, C.byref(one), C.byref(gm), C.byref(up), None))
    total = 2 * prec_bytes * ctx.N + prec_bytes * (inv.value + gm.value) + 8 * up.value
    return int(total), int(lev.value), int(lag.value)


def run_ours(args):
    if args.workload == "cfg3":
        return run_batched(args)
    if args.workload == "cfg5":
        return run_large(args)
    import torch
    from rtg import Problem, _lib, learned as LN

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
    params, net_meta = LN.load(LN.DEFAULT_NET)
    LN.set_params(ctx, params)
    # L2 weights (dx dy dth/8) wx wy wth = mass weights with kappa = 1
    lay = ctx.layout
    X, Y, T = lay.node_coords()
    ones = ctx.apply(_lib.RTG_MASS, torch.ones(N, dtype=torch.float64, device=ctx.device))
    kap = ctx.to_device(np.asarray(np.broadcast_to(spec.kappa(X, Y), (N,)), dtype=np.float64))
    w = (ones / kap).cpu().numpy()

    # reference solution: tight plain FP64 solve
    u_ref, info_ref = ctx.solve(f_dev, g_dev, method=0, rtol=1e-14, max_it=20000, precond=1)
    u_ref_h = u_ref.cpu().numpy()
    arms = {"plain_fp64": (0, 1), "mixed": (1, 1), "learned_mixed": (1, 3)}

    def solve(arm, rtol):
        method, pc = arms[arm]
        return ctx.solve(f_dev, g_dev, method=method, rtol=rtol, max_it=20000, precond=pc, restart=30,
                         inner_rtol=1e-5)

    def calibrate(arm):
        for k in range(6, 15):
            rtol = 10.0 ** (-k)
            u, info = solve(arm, rtol)
            err = rel_l2(u.cpu().numpy(), u_ref_h, w)
            if err <= ERR_TARGET:
                return rtol
        raise RuntimeError("{} did not reach the error target".format(arm))

    rtols = {arm: calibrate(arm) for arm in arms}
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=ctx.device)
    stream = torch.cuda.current_stream()

    launch_count = ctx.lib.rtg_launch_count
    launched = {}

    def timed(arm, steps, warm):
        for _ in range(warm):
            solve(arm, rtols[arm])
        times, errs, infos = [], [], []
        launched[arm] = 0
        for _ in range(steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0, e1 = _events(stream)
            n0 = launch_count()
            e0.record(stream)
            u, info = solve(arm, rtols[arm])
            e1.record(stream)
            launched[arm] += launch_count() - n0
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            errs.append(rel_l2(u.cpu().numpy(), u_ref_h, w))
            infos.append(info)
        return times, errs, infos

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        res = {"learned_mixed": timed("learned_mixed", args.steps, args.warmup)}
    res["mixed"] = timed("mixed", max(1, min(args.steps, 3)), 1)
    res["plain_fp64"] = timed("plain_fp64", max(1, min(args.steps, 3)), 1)
    if world > 1:
        torch.distributed.barrier()

    # e2e through the C ABI with host buffers (learned+mixed)
    lib = ctx.lib
    fvals = torch.from_numpy(ctx.node_values(spec.f)).pin_memory()
    gvals = torch.from_numpy(np.ascontiguousarray(g_dev.cpu().numpy())).pin_memory()
    u_host = torch.empty(N, dtype=torch.float64).pin_memory()
    fd = torch.empty(N, dtype=torch.float64, device=ctx.device)
    fw = torch.empty_like(fd)
    gd = torch.empty_like(fd)
    ud = torch.zeros_like(fd)
    opts = _lib.SolveOpts(method=1, restart=30, max_it=20000, rtol=rtols["learned_mixed"], atol=0., precond=3,
                          nonzero_guess=0, inner_rtol=1e-5, max_outer=20, verbose=0)
    sinfo = _lib.SolveInfo()
    sp = C.c_void_p(stream.cuda_stream)
    e2e_times = []
    for it in range(args.warmup + args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0, e1 = _events(stream)
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

    # rooflines: the FP32 sweep (dominant kernel of the solve) and the FP32 apply
    peak, peak_kind = peaks()
    r32 = torch.randn(N, dtype=torch.float32, device=ctx.device)
    z32 = torch.empty_like(r32)
    t_sweep = kernel_time(lambda: ctx.precondition(r32, z32, prec=_lib.RTG_FP32), stream, flush)
    sb, nlev, nlag = sweep_bytes(ctx, 4)
    t_apply = kernel_time(lambda: ctx.apply(_lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS, r32, z32, prec=_lib.RTG_FP32),
                          stream, flush)
    bytes_apply = int(ctx.info["bytes_per_apply_fp32"])
    x64 = torch.randn(N, dtype=torch.float64, device=ctx.device)
    y64 = torch.empty_like(x64)
    t_apply64 = kernel_time(lambda: ctx.apply(_lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS, x64, y64, prec=_lib.RTG_FP64),
                            stream, flush)
    t_sweep64 = kernel_time(lambda: ctx.precondition(x64, y64, prec=_lib.RTG_FP64), stream, flush)

    t_l, e_l, i_l = res["learned_mixed"]
    value = statistics.median(t_l)
    if world > 1:
        tt = torch.tensor([max(t_l)], device=ctx.device)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        value = float(tt.item())
    if rank != 0:
        return None
    inf = i_l[-1]
    # librtg kernels launched inside the timed solves (the library's own count)
    launches = int(launched["learned_mixed"])

    def arm_summary(arm):
        t, e, i = res[arm]
        return {"rtol": rtols[arm], "rel_l2_err": max(e), "median_s": statistics.median(t), "seconds": t,
                "iterations": i[-1]["iterations"], "outer": i[-1]["outer"], "fp64_applies": i[-1]["fp64_applies"],
                "fp32_applies": i[-1]["fp32_applies"], "learned": i[-1]["learned"],
                "fallbacks": i[-1]["fallbacks"]}

    t_plain = statistics.median(res["plain_fp64"][0])
    out = {
        "metric": METRIC, "value": value, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * value, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-inner/f64-outer",
        "data": "synthetic (seeded hp mesh and coefficients)",
        "config": {"workload": desc, "ndof": N, "ndof_interior": int(ctx.info["ndof_interior"]),
                   "error_target": ERR_TARGET, "l2_flush": "256 MB write before every timed solve and kernel",
                   "learned_mixed": arm_summary("learned_mixed"), "mixed": arm_summary("mixed"),
                   "plain_fp64": arm_summary("plain_fp64"),
                   "speedup_learned_mixed_vs_plain_fp64": t_plain / value,
                   "speedup_mixed_vs_plain_fp64": t_plain / statistics.median(res["mixed"][0]),
                   "network": {"file": "rtg/nets/sweep_correction.npz", **net_meta},
                   "reference_solution": {"rtol": 1e-14, "iterations": info_ref["iterations"], "res_f": info_ref["res_f"]},
                   "kernels_us": {"sweep_fp32": 1e6 * t_sweep, "sweep_fp64": 1e6 * t_sweep64,
                                  "apply_fp32": 1e6 * t_apply, "apply_fp64": 1e6 * t_apply64},
                   "sweep": {"levels": nlev, "lagged_couplings": nlag},
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": statistics.median(e2e_times), "unit": "s", "h2d_bytes_per_step": 2 * 8 * N,
                "d2h_bytes_per_step": 8 * N, "rel_l2_err": e2e_err},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": sb / t_sweep / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": sb / t_sweep / 1e9 / peak,
                     "traffic": profiled_traffic("sweep_persistent_kernel_fp32_cfg2") if args.workload == "cfg2"
                     else None,
                     "kernel": "sweep_persistent_kernel<float>", "bytes_per_launch": sb, "launch_s": t_sweep,
                     "peak_kind": peak_kind,
                     "note": "latency bound: {} wavefront levels, {:.2f} us per level".format(
                         nlev, 1e6 * t_sweep / max(nlev, 1))},
        "apply_roofline": {"bound": "hbm", "achieved": bytes_apply / t_apply / 1e9, "peak": peak, "unit": "GB/s",
                           "frac": bytes_apply / t_apply / 1e9 / peak, "kernel": "apply_tiled_kernel (FP32 system)",
                           "bytes_per_launch": bytes_apply, "launch_s": t_apply, "peak_kind": peak_kind,
                           "dof_applies_per_s": N / t_apply},
        "clocks": clk.summary(),
    }
    out["amr_indicators"] = amr_indicators(ctx, mesh, u_ref_h, stream, flush, not args.no_cpu)
    if not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(mesh, spec, rtols["plain_fp64"], u_ref_h, w)
    return out


def run_batched(args):
    """cfg3: 256 independent instances (seeded degree, size, sigma_t, albedo,
    g) in one batched solve (method 1, one handle, graph-captured restart
    cycle), against solving the same instances one by one through rt.Problem-
    style contexts.  Each instance's error is measured against its own tight
    FP64 solve."""
    import torch
    from rtg import DeviceContext, _lib, workloads as W
    from rtg.batch import BatchContext
    rank = int(os.environ.get("RANK", "0"))
    torch.cuda.set_device(0)
    nb = 256
    inst = [W.batch_instance(1000 + k) for k in range(nb)]
    bc = BatchContext(inst)
    f = bc.forcing()
    g = bc.inflow()
    stream = torch.cuda.current_stream()
    # reference solutions: tight individual FP64 solves
    ctxs = [DeviceContext(m, p.kappa, p.sigma, p.Phi) for m, p in inst]
    fs = [c.forcing(p.f) for c, (m, p) in zip(ctxs, inst)]
    gs = [c.inflow(p.bcs_dirac) for c, (m, p) in zip(ctxs, inst)]
    refs = [c.solve(fi, gi, method=0, precond=1, rtol=1e-13, max_it=20000)[0] for c, fi, gi in zip(ctxs, fs, gs)]

    def errors(parts):
        return [float(torch.linalg.norm(a - r) / torch.linalg.norm(r)) for a, r in zip(parts, refs)]

    rtol = None
    for k in range(6, 14):
        u, infos = bc.solve(f, g, rtol=10.0 ** (-k), inner_rtol=1e-5)
        if max(errors(bc.split(u))) <= ERR_TARGET:
            rtol = 10.0 ** (-k)
            break
    if rtol is None:
        raise RuntimeError("batched solve did not reach the error target")
    for _ in range(args.warmup):
        bc.solve(f, g, rtol=rtol, inner_rtol=1e-5)
    times = []
    launch_count = _lib.load().rtg_launch_count
    n_launch = 0
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            e0, e1 = _events(stream)
            n0 = launch_count()
            e0.record(stream)
            u, infos = bc.solve(f, g, rtol=rtol, inner_rtol=1e-5)
            e1.record(stream)
            n_launch += launch_count() - n0
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    errs = errors(bc.split(u))
    seq = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for c, fi, gi in zip(ctxs, fs, gs):
            c.solve(fi, gi, method=1, precond=1, rtol=rtol, inner_rtol=1e-5, restart=30)
        torch.cuda.synchronize()
        seq.append(time.perf_counter() - t0)
    if rank != 0:
        return None
    value = statistics.median(times)
    ndof = int(bc.N)
    out = {"metric": METRIC, "value": value, "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * value, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32-inner/f64-outer", "data": "synthetic (256 seeded instances)",
            "config": {"workload": "256 independent instances (batch_instance seeds 1000..1255)", "ndof": ndof,
                       "rtol": rtol, "max_rel_err": max(errs), "error_target": ERR_TARGET,
                       "sequential_one_by_one_s": min(seq), "speedup_batched_vs_sequential": min(seq) / value,
                       "iterations_max": max(i["iterations"] for i in infos)},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                    "note": "inputs resident; the batched entry point takes device vectors"},
            "gpu_launches": int(n_launch),
            "clocks": clk.summary()}
    if not args.no_cpu:
        # all host cores, a bounded sample of 32 of the 256 instances
        out["cpu_baseline"] = cpu_baseline_batch(list(range(1000, 1032)), rtol, nb)
    return out


def run_large(args):
    """cfg5 (~9.4e6 DOF): apply and sweep throughput in FP32 and FP64, and a
    bounded learned+mixed solve (the strongly forward-peaked thick discs make
    sweep-preconditioned GMRES stagnate; the residual reached is reported)."""
    import torch
    from rtg import Problem, _lib, learned as LN
    torch.cuda.set_device(0)
    desc, mesh, spec = workload("cfg5")
    prob = Problem(spec.kappa, spec.sigma, spec.Phi, spec.f, spec.bcs_dirac)
    ctx = prob.context(mesh)
    N = ctx.N
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=ctx.device)
    peak, peak_kind = peaks()
    out = {}
    for nm, dt, prec, key in (("fp32", torch.float32, _lib.RTG_FP32, "bytes_per_apply_fp32"),
                              ("fp64", torch.float64, _lib.RTG_FP64, "bytes_per_apply_fp64")):
        x = torch.randn(N, dtype=dt, device=ctx.device)
        y = torch.empty_like(x)
        ta = kernel_time(lambda: ctx.apply(_lib.RTG_SYSTEM | _lib.RTG_MASK_ROWS, x, y, prec=prec), stream, flush, 10)
        ts = kernel_time(lambda: ctx.precondition(x, y, prec=prec), stream, flush, 5)
        out[nm] = {"apply_s": ta, "apply_gbs": ctx.info[key] / ta / 1e9, "apply_frac": ctx.info[key] / ta / 1e9 / peak,
                   "dof_applies_per_s": N / ta, "apply_tflops": ctx.info["flops_per_apply"] / ta / 1e12,
                   "sweep_s": ts}
    params, _ = LN.load(LN.DEFAULT_NET)
    LN.set_params(ctx, params)
    f_dev = ctx.forcing(spec.f)
    g_dev = ctx.inflow(spec.bcs_dirac)
    with ClockSampler(0) as clk:
        torch.cuda.synchronize()
        e0, e1 = _events(stream)
        n0 = ctx.lib.rtg_launch_count()
        e0.record(stream)
        u, info = ctx.solve(f_dev, g_dev, method=1, precond=3, rtol=1e-8, max_it=300, restart=30, inner_rtol=1e-5)
        e1.record(stream)
        n_launch = ctx.lib.rtg_launch_count() - n0
        torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    return {"metric": METRIC, "value": t, "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 0,
            "ms_per_step": 1e3 * t, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32-inner/f64-outer", "data": "synthetic (seeded disc-edge hp mesh)",
            "config": {"workload": desc, "ndof": N, "bounded_solve": {
                "max_it": 300, "iterations": info["iterations"], "converged": info["converged"],
                "rel_residual": info["res_f"] / max(info["rhs_norm"], 1e-300), "fallbacks": info["fallbacks"]},
                "kernels": out},
            "e2e": {"value": t, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "roofline": {"bound": "hbm", "achieved": out["fp32"]["apply_gbs"], "peak": peak, "unit": "GB/s",
                         "frac": out["fp32"]["apply_frac"], "traffic": None, "kernel": "apply_tiled_kernel (FP32)",
                         "peak_kind": peak_kind},
            "gpu_launches": int(n_launch), "clocks": clk.summary()}


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
