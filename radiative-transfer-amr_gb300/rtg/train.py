"""Train the learned sweep correction on the GPU and save it.

    python -m rtg.train [--problems 16] [--pairs 16] [--steps 3000] [--out PATH]

Training problems are the config-4 family (rtg.workloads.config4_instance,
seeds 0..problems-1): Gaussian-bump scatterers of seeded amplitude, width,
centre and anisotropy on seeded hp meshes.  For each problem the method's own
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
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    import torch
    from . import DeviceContext, learned as LN, workloads as W
    torch.cuda.set_device(0)
    t0 = time.time()
    data = []
    for s in range(a.problems):
        mesh, spec = W.config4_instance(s, rounds=a.rounds)
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
    for s in (100, 101, 102, 103):
        mesh, spec = W.config4_instance(s, rounds=a.rounds)
        ctx = DeviceContext(mesh, spec.kappa, spec.sigma, spec.Phi)
        held.append(LN.evaluate(P, *LN.stack(LN.collect_pairs(ctx, ctx.forcing(spec.f), ctx.inflow(spec.bcs_dirac),
                                                                 n_pairs=8))))
        ctx.close()
    meta = {"problems": a.problems, "pairs": a.pairs, "steps": a.steps, "rounds": a.rounds, "seed": a.seed,
            "rows": int(F.shape[0]), "train_loss_ratio": hist[-1][1], "held_out_loss_ratio": held,
            "data_seconds": t_data, "train_seconds": t_train}
    out = a.out or LN.DEFAULT_NET
    os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
    LN.save(out, P, meta)
    print(meta)


if __name__ == "__main__":
    main()
