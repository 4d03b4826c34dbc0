"""Train the learned sweep correction on the GPU and save it.

    python -m rtg.train [--problems 16] [--pairs 16] [--steps 3000] [--out PATH]

Training problems (--family): "cfg4", the config-4 family
(rtg.workloads.config4_instance, seeds 0..problems-1): Gaussian-bump
scatterers of seeded amplitude, width, centre and anisotropy on seeded hp
meshes; "disc", the two-scatterer family (rtg.workloads.disc_family_instance):
thick, strongly forward-scattering discs on the resolved-angle recipe; "mix",
--problems of each.  For each problem the method's own
sweep-GMRES produces residual -> error pairs (Arnoldi vectors with their exact
errors); every feature, forward and backward pass and Adam step runs in
librtg's kernels.  The saved file holds the FP32 parameters and the training
record (final training loss relative to the sweep alone, and the held-out
ratio on seeds 100..103)."""
import argparse
import os
import sys
import time


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--problems", type=int, default=16)
    ap.add_argument("--pairs", type=int, default=16)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--rounds", type=int, default=3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--family", default="mix", choices=["cfg4", "disc", "mix"])
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    import torch
    from . import DeviceContext, learned as LN, workloads as W
    torch.cuda.set_device(0)
    t0 = time.time()
    fams = ["cfg4", "disc"] if a.family == "mix" else [a.family]

    def instance(fam, s):
        return W.config4_instance(s, rounds=a.rounds) if fam == "cfg4" else W.disc_family_instance(s)

    data = []
    for fam in fams:
        for s in range(a.problems):
            mesh, spec = instance(fam, s)
            ctx = DeviceContext(mesh, spec.kappa, spec.sigma, spec.Phi)
            data += LN.collect_pairs(ctx, ctx.forcing(spec.f), ctx.inflow(spec.bcs_dirac), n_pairs=a.pairs)
            ctx.close()
    F, M, S = LN.stack(data)
    t_data = time.time() - t0
    t1 = time.time()
    P, hist = LN.train(F, M, S, steps=a.steps, batch=32768, lr=2e-3, seed=a.seed, log_every=max(1, a.steps // 10),
                       log=lambda m: print(m, file=sys.stderr, flush=True))
    torch.cuda.synchronize()
    t_train = time.time() - t1
    held = []
    for fam, s in [(f, q) for f in fams for q in (100, 101, 102, 103)]:
        mesh, spec = instance(fam, s)
        ctx = DeviceContext(mesh, spec.kappa, spec.sigma, spec.Phi)
        held.append(LN.evaluate(P, *LN.stack(LN.collect_pairs(ctx, ctx.forcing(spec.f), ctx.inflow(spec.bcs_dirac),
                                                                 n_pairs=8))))
        ctx.close()
    meta = {"family": a.family, "problems": a.problems, "pairs": a.pairs, "steps": a.steps, "rounds": a.rounds,
            "seed": a.seed, "rows": int(F.shape[0]), "train_loss_ratio": hist[-1][1], "held_out_loss_ratio": held,
            "data_seconds": t_data, "train_seconds": t_train}
    out = a.out or LN.DEFAULT_NET
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    LN.save(out, P, meta)
    print(meta)


if __name__ == "__main__":
    main()
