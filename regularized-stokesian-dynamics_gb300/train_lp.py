"""Training of the learned preconditioner of the RPP solve (run on a GPU).

    python regularized-stokesian-dynamics_gb300/train_lp.py [--systems 2000] [--out lp_params.npy]

Data: the learned-preconditioner workload -- N = 1000 spheres of radius 1 at
volume fraction 0.5, a quarter of them in near-contact pairs with surface
gaps log-uniform in [1e-4, 1e-1] (configs.packing, near_contact=True) --
generated by the method itself: each trajectory starts from a seeded packing
sheared to its own Lees-Edwards strain (configs.sheared_series) and is
advanced by the mixed-precision step (rsd_stepper_stokesian_dev, dt 5e-4,
shear rate 1); every `stride` steps the resistance matrix RPP of the current
configuration (FP32, from the mixed form's factors: rsd_resistance_pp_dev)
is one training sample.  Each sample makes one supervised step (Adam, the
learning rate warmed up linearly over the first samples): the network
emits the directions W_ab = Z_aa^-1 Z_ab of the pair blocks, the loss is
their mean squared difference from those of that matrix's exact FSAI, and
Adam updates the weights (kernels in csrc/learned.cu).  Two guards keep one
outlier sample from wrecking the weights: the gradient is clipped to three
times the running mean of its norm, and a sample whose loss exceeds fifty
times the running mean of the loss makes no update.  The parameters are
kept every `snapshot` samples; the snapshot with the fewest PCG iterations
on a validation system (its own seed and strain) is written out.  Then one
held-out system in FP64 gives the PCG iteration counts of every
preconditioner.  Prints one JSON line and writes the FP32 parameters to
--out.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--systems", type=int, default=2000)
    ap.add_argument("--trajectories", type=int, default=10)
    ap.add_argument("--stride", type=int, default=2)
    ap.add_argument("--N", type=int, default=1000)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--warmup", type=int, default=50, help="samples of linear learning-rate warm-up")
    ap.add_argument("--sweeps", type=int, default=100)
    ap.add_argument("--snapshot", type=int, default=200, help="samples between kept parameter snapshots")
    ap.add_argument("--clip", type=float, default=3.0, help="gradient clip, in running means of the gradient norm")
    ap.add_argument("--spike", type=float, default=50.0, help="loss guard, in running means of the loss")
    ap.add_argument("--out", default=os.path.join(HERE, "lp_params.npy"))
    ap.add_argument("--seed", type=int, default=20264000)
    args = ap.parse_args()
    import torch

    import __graft_entry__ as ge
    rsd = ge.load_package()
    dev = torch.device("cuda", 0)
    ctx = rsd.Context(0)
    tab = rsd.LubTab(rsd.lubdat_dir())
    mu = rsd.mu_f_dimensionless(1.0)
    net = rsd.LearnedPreconditioner(0, seed=args.seed)
    N, dt = args.N, 5e-4
    per_traj = (args.systems + args.trajectories - 1) // args.trajectories
    log, done, t0 = [], 0, time.time()
    U_t = torch.empty(6 * N, dtype=torch.float64, device=dev)
    S_t = torch.empty(5 * N, dtype=torch.float64, device=dev)
    ema_loss = ema_g = None
    snapshots = []
    k = 0
    while done < args.systems and k < 3 * args.trajectories:  # more trajectories if one stops early
        strain = (k % args.trajectories) / args.trajectories
        series, radii, L = rsd.configs.sheared_series(N, 0.5, 1e-4, args.seed + k, [strain], sweeps=args.sweeps,
                                                      near_contact=True)
        conf_t = torch.tensor(series[0], dtype=torch.float64, device=dev)
        radii_t = torch.tensor(radii, dtype=torch.float64, device=dev)
        T = strain
        for s in range(per_traj):
            if done >= args.systems:
                break
            try:
                rpp, lat = rsd.resistance_pp_dev(ctx, tab, conf_t, radii_t, T, [L, L, L], 1.0, mu, 1e-10,
                                                 precision=rsd.PREC_MIXED)
            except rsd.RSDError as e:  # e.g. a factor that is not positive: next trajectory
                print("trajectory %d stops at strain %.3f: %s" % (k, T, e), flush=True)
                break
            frac = done / args.systems
            # linear warm-up (the heads start at zero, Z = I: full-size first
            # Adam steps overshoot), then steps down at 50 % and 80 %
            lr = args.lr * min(1.0, (done + 1) / args.warmup) * (1.0 if frac < 0.5 else (0.25 if frac < 0.8 else 0.05))
            if done >= 20:  # the guards, once the running means settle
                net.set_training(args.clip * ema_g, args.spike * ema_loss)
            try:
                loss = net.train_step(ctx, conf_t, radii_t, lat, rpp, lr)
            except rsd.RSDError as e:  # a local block not positive definite in FP32: skip the sample
                print("sample skipped at strain %.3f: %s" % (T, e), flush=True)
                loss = None
            if loss is None:
                T += dt
                continue
            gnorm, skipped, _ = net.training_stats()
            if done < 20 or loss <= args.spike * ema_loss:
                ema_loss = loss if ema_loss is None else 0.95 * ema_loss + 0.05 * loss
                ema_g = gnorm if ema_g is None else 0.95 * ema_g + 0.05 * gnorm
            done += 1
            if done % 50 == 0 or done == 1:
                log.append((done, loss))
                print("sample %d traj %d strain %.3f loss %.4e |g| %.3e skipped %d (%.0f s)"
                      % (done, k, T, loss, gnorm, skipped, time.time() - t0), flush=True)
            if done % args.snapshot == 0:
                snapshots.append((done, net.params()))
            try:
                for _ in range(args.stride):
                    rsd.stepper_stokesian_dev(ctx, tab, conf_t, radii_t, T, dt, [L, L, L], 1.0, mu, 1e-10, U_t, S_t,
                                              precision=rsd.PREC_MIXED)
                    T += dt
            except rsd.RSDError as e:
                print("trajectory %d stops at strain %.3f: %s" % (k, T, e), flush=True)
                break
        k += 1
    net_skipped = net.training_stats()[1]
    if not snapshots or snapshots[-1][0] != done:
        snapshots.append((done, net.params()))
    # model selection: PCG iterations on a validation system (FP64)
    series, radii, L = rsd.configs.sheared_series(N, 0.5, 1e-4, args.seed + 777, [0.25], sweeps=args.sweeps,
                                                  near_contact=True)
    conf_t = torch.tensor(series[0], dtype=torch.float64, device=dev)
    radii_t = torch.tensor(radii, dtype=torch.float64, device=dev)
    rpp, lat = rsd.resistance_pp_dev(ctx, tab, conf_t, radii_t, 0.25, [L, L, L], 1.0, mu, 1e-10)
    b = torch.tensor(np.random.default_rng(2).normal(size=6 * N), device=dev)
    val = []
    for at, p in snapshots:
        cand = rsd.LearnedPreconditioner(0, p)
        _, it, _ = rsd.pcg_dev(ctx, cand, rsd.PC_LEARNED, conf_t, radii_t, lat, rpp, b, tol=1e-12, maxit=3000)
        cand.close()
        val.append((at, it))
        print("snapshot at %d samples: %d validation iterations" % (at, it), flush=True)
    best = min(range(len(val)), key=lambda i: (val[i][1], -val[i][0]))
    params = snapshots[best][1]
    np.save(args.out, params)
    net.close()
    net = rsd.LearnedPreconditioner(0, params)
    # held-out evaluation in FP64
    series, radii, L = rsd.configs.sheared_series(N, 0.5, 1e-4, args.seed + 999, [0.5], sweeps=args.sweeps,
                                                  near_contact=True)
    conf_t = torch.tensor(series[0], dtype=torch.float64, device=dev)
    radii_t = torch.tensor(radii, dtype=torch.float64, device=dev)
    rpp, lat = rsd.resistance_pp_dev(ctx, tab, conf_t, radii_t, 0.5, [L, L, L], 1.0, mu, 1e-10)
    b = torch.tensor(np.random.default_rng(1).normal(size=6 * N), device=dev)
    evals = {}
    for name, mode in (("none", rsd.PC_NONE), ("jacobi", rsd.PC_JACOBI), ("block_jacobi", rsd.PC_BLOCK_JACOBI),
                       ("fsai", rsd.PC_FSAI), ("learned", rsd.PC_LEARNED)):
        x, it, res = rsd.pcg_dev(ctx, net, mode, conf_t, radii_t, lat, rpp, b, tol=1e-12, maxit=20000)
        evals[name] = {"iterations": it, "residual": res}
    print(json.dumps({"trained_on": done, "N": N, "loss_log": log, "final_loss": log[-1][1] if log else None,
                      "skipped": net_skipped, "validation": val, "chosen": val[best][0],
                      "seconds": time.time() - t0, "heldout_pcg": evals, "out": args.out}), flush=True)


if __name__ == "__main__":
    main()
