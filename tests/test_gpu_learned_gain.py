"""What the trained network gains over the method without it, on held-out
problems of the config-4 family (Gaussian-bump scatterers of seeded amplitude,
width, centre and anisotropy on seeded hp meshes).

The network is trained on the GPU (library kernels) on residual -> error pairs
from sweep-GMRES on eight training problems and evaluated on two unseen
optically thick ones.  Two numbers are measured per problem:
  * the error the preconditioner leaves, ||(e - z) - L z||^2 / ||e - z||^2 over
    Arnoldi vectors of the problem (1.0 = the sweep alone); the network must
    remove part of the sweep's error (ratio below 1) on problems it has not
    seen;
  * flexible-GMRES iterations to 1e-10 with the correction vs the sweep alone,
    reported (printed) as measured; the solve must converge to the same
    solution.  The first solve with the correction runs the trial that decides
    whether it stays (two timed 8-step cycles); later solves on the handle
    reuse the verdict, and where the trial dropped the correction they take
    exactly the sweep alone's iterations.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_trained_network_on_held_out_problems(capsys):
    import torch
    from rtg import DeviceContext, learned as LN, workloads as W
    data = []
    for seed in range(8):
        mesh, spec = W.config4_instance(seed, rounds=3)
        ctx = DeviceContext(mesh, spec.kappa, spec.sigma, spec.Phi)
        data += LN.collect_pairs(ctx, ctx.forcing(spec.f), ctx.inflow(spec.bcs_dirac), n_pairs=16)
        ctx.close()
    F, M, S = LN.stack(data)
    P, hist = LN.train(F, M, S, steps=1500, batch=32768, lr=2e-3, seed=0, log_every=250)
    assert hist[-1][1] < hist[0][1]
    lines = []
    for seed in (101, 104):
        mesh, spec = W.config4_instance(seed, rounds=3)
        ctx = DeviceContext(mesh, spec.kappa, spec.sigma, spec.Phi)
        f = ctx.forcing(spec.f)
        g = ctx.inflow(spec.bcs_dirac)
        ratio = LN.evaluate(P, *LN.stack(LN.collect_pairs(ctx, f, g, n_pairs=8)))
        LN.set_params(ctx, P)
        u1, i1 = ctx.solve(f, g, method=1, precond=1, rtol=1e-10, restart=30, inner_rtol=1e-5)
        u3, i3 = ctx.solve(f, g, method=1, precond=3, rtol=1e-10, restart=30, inner_rtol=1e-5)
        u4, i4 = ctx.solve(f, g, method=1, precond=3, rtol=1e-10, restart=30, inner_rtol=1e-5)
        assert i1["converged"] and i3["converged"] and i4["converged"]
        assert float(torch.linalg.norm(u3 - u1) / torch.linalg.norm(u1)) < 1e-8
        assert float(torch.linalg.norm(u4 - u1) / torch.linalg.norm(u1)) < 1e-8
        assert ratio < 1.0, (seed, ratio)
        assert i3["trial_its"] > 0 and i4["trial_its"] == 0
        assert i3["learned_kept"] == i4["learned_kept"]
        if not i4["learned_kept"]:
            assert i4["iterations"] == i1["iterations"] and i4["learned"] == 0
        lines.append("held-out seed {} (amp {:.1f}): error left {:.3f} of the sweep's; iterations sweep {} "
                     "learned {} (trial kept the correction: {}, fallbacks {})".format(
                         seed, spec.meta["amp"], ratio, i1["iterations"], i4["iterations"], i4["learned_kept"],
                         i4["fallbacks"]))
        ctx.close()
    with capsys.disabled():
        print("\n" + "\n".join(lines))
