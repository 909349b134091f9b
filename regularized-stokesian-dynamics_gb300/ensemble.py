"""Ensembles of independent replicas of the periodic FTS suspension, each of
its own size, volume fraction and shear rate, stepped by the fused
STEPPER_Stokesian (the reference runs one system per process,
main.f90:172-229).

Scheduling.  The replicas are spread over W workers, each a host thread
with its own context (one CUDA stream, its own device buffers); a worker
steps its replicas in turn, and the workers run concurrently, so the GPU
holds the kernels of W replicas at once.  Replicas are assigned largest
first to the least-loaded worker (LPT), with a replica's cost taken as
(11 N)^3, the order of its factorisations.

Tuning.  autotune() times one step of a representative replica of every
size class (N in [32, 64), [64, 128), [128, 192), [192, 256]) under each
candidate setting of the kernels -- the FP32 factorisations on tcgen05 or on
the FP32 SIMT pipe (rsd_ctx_set_tensor_cores), with the look-ahead or the
in-order schedule (rsd_ctx_set_factor_schedule), and the number of passes
over the near real-space images (rsd_ctx_set_mixed_real_passes) -- and keeps the
fastest per class in a table (JSON), which the workers apply per replica.

The replicas are device-resident (positions, radii, velocities and
stresslets in HBM); only the lattice scalars cross to the host each step.
"""
from __future__ import annotations

import json
import math
import threading
import time

import numpy as np

SIZE_CLASSES = [(32, 64), (64, 128), (128, 192), (192, 257)]
# the factor schedule matters only on the tensor-core path (its two-level
# Cholesky); a small replica is launch-bound, where the in-order schedule's
# fewer launches can win
CANDIDATES = [dict(tensor_cores=1, real_passes=1, factor_schedule=1), dict(tensor_cores=1, real_passes=1, factor_schedule=0),
              dict(tensor_cores=0, real_passes=1, factor_schedule=1),
              dict(tensor_cores=1, real_passes=2, factor_schedule=1), dict(tensor_cores=1, real_passes=2, factor_schedule=0),
              dict(tensor_cores=0, real_passes=2, factor_schedule=1)]


def size_class(N):
    for k, (lo, hi) in enumerate(SIZE_CLASSES):
        if lo <= N < hi:
            return k
    return len(SIZE_CLASSES) - 1


def replica_specs(nrep, seed, n_range=(32, 256), phi_range=(0.10, 0.50), gamma_range=(0.1, 10.0)):
    """The ensemble workload's draws: N uniform in n_range (inclusive), phi
    uniform in phi_range, shear rate log-uniform in gamma_range; one seed per
    replica."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for r in range(nrep):
        N = int(rng.integers(n_range[0], n_range[1] + 1))
        phi = float(rng.uniform(*phi_range))
        gamma = float(math.exp(rng.uniform(math.log(gamma_range[0]), math.log(gamma_range[1]))))
        out.append(dict(N=N, phi=phi, gamma=gamma, seed=seed + 1 + r))
    return out


def lpt_assign(costs, workers):
    """Largest-first assignment to the least-loaded worker."""
    load = [0.0] * workers
    groups = [[] for _ in range(workers)]
    for i in sorted(range(len(costs)), key=lambda i: -costs[i]):
        w = min(range(workers), key=lambda k: load[k])
        groups[w].append(i)
        load[w] += costs[i]
    return groups


class Ensemble:
    """Replicas given by `specs` (replica_specs) and their packings; mixed
    precision; dt and Ewald tolerance common to all."""

    def __init__(self, rsd, specs, packings, dt=1e-3, ews=1e-10, workers=16, device=0, table=None):
        import torch
        self.rsd, self.specs, self.dt, self.ews = rsd, specs, dt, ews
        self.device = device
        self.dev = torch.device("cuda", device)
        self.mu = rsd.mu_f_dimensionless(1.0)
        self.table = table or {}
        self.conf, self.radii, self.L, self.T = [], [], [], []
        for pos, radii, L in packings:
            self.conf.append(torch.tensor(pos, dtype=torch.float64, device=self.dev))
            self.radii.append(torch.tensor(radii, dtype=torch.float64, device=self.dev))
            self.L.append(L)
            self.T.append(0.0)
        self.U = [torch.empty(6 * s["N"], dtype=torch.float64, device=self.dev) for s in specs]
        self.S = [torch.empty(5 * s["N"], dtype=torch.float64, device=self.dev) for s in specs]
        self.yeta = [None] * len(specs)
        self.info = [None] * len(specs)
        torch.cuda.synchronize(self.dev)
        self.workers = max(1, min(workers, len(specs)))
        self.groups = lpt_assign([(11.0 * s["N"]) ** 3 for s in specs], self.workers)
        self.ctx = [rsd.Context(device) for _ in range(self.workers)]
        self.tab = [rsd.LubTab(rsd.lubdat_dir()) for _ in range(self.workers)]

    def _settings(self, ctx, N):
        s = self.table.get(str(size_class(N)))
        if s:
            ctx.set_tensor_cores(s["tensor_cores"])
            ctx.set_mixed_real_passes(s["real_passes"])
            ctx.set_factor_schedule(s.get("factor_schedule", 1))

    def _step_replica(self, w, r):
        rsd, s = self.rsd, self.specs[r]
        ctx = self.ctx[w]
        self._settings(ctx, s["N"])
        L = self.L[r]
        y, info = rsd.stepper_stokesian_dev(ctx, self.tab[w], self.conf[r], self.radii[r], self.T[r], self.dt,
                                            [L, L, L], s["gamma"], self.mu, self.ews, self.U[r], self.S[r],
                                            precision=rsd.PREC_MIXED)
        self.T[r] += self.dt
        self.yeta[r] = y.copy()
        self.info[r] = (info.NR, info.NI, info.iterations, info.residual)

    def run(self, steps):
        """Advances every replica by `steps` steps; returns the wall time."""
        errors = []

        def work(w):
            try:
                for _ in range(steps):
                    for r in self.groups[w]:
                        self._step_replica(w, r)
            except Exception as e:  # reported after the join
                errors.append((w, e))

        threads = [threading.Thread(target=work, args=(w,)) for w in range(self.workers)]
        t0 = time.perf_counter()
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for c in self.ctx:
            self.rsd._sync_ctx(c)
        wall = time.perf_counter() - t0
        if errors:
            raise errors[0][1]
        return wall

    def autotune(self, path=None, reps=2):
        """Per size class, the fastest candidate setting for one step of the
        class's largest replica; stores the table (and writes it to path)."""
        import torch
        table = {}
        ctx, tab = self.ctx[0], self.tab[0]
        for k in range(len(SIZE_CLASSES)):
            members = [r for r, s in enumerate(self.specs) if size_class(s["N"]) == k]
            if not members:
                continue
            r = max(members, key=lambda i: self.specs[i]["N"])
            s, L = self.specs[r], self.L[r]
            conf0 = self.conf[r].clone()
            best = None
            for cand in CANDIDATES:
                ctx.set_tensor_cores(cand["tensor_cores"])
                ctx.set_mixed_real_passes(cand["real_passes"])
                ctx.set_factor_schedule(cand["factor_schedule"])
                times = []
                for it in range(reps + 1):
                    c = conf0.clone()
                    if self.dev.type == "cuda":
                        torch.cuda.synchronize(self.dev)
                    t0 = time.perf_counter()
                    self.rsd.stepper_stokesian_dev(ctx, tab, c, self.radii[r], self.T[r], self.dt, [L, L, L],
                                                   s["gamma"], self.mu, self.ews, self.U[r], self.S[r],
                                                   precision=self.rsd.PREC_MIXED)
                    self.rsd._sync_ctx(ctx)
                    if it:  # the first run grows the buffers
                        times.append(time.perf_counter() - t0)
                ms = 1e3 * min(times)
                if best is None or ms < best[1]:
                    best = (cand, ms)
            table[str(k)] = dict(best[0], ms=best[1], N=s["N"])
        ctx.set_tensor_cores(1)
        ctx.set_mixed_real_passes(1)
        ctx.set_factor_schedule(1)
        self.table = table
        if path:
            with open(path, "w") as fp:
                json.dump(table, fp, indent=1, sort_keys=True)
        return table
