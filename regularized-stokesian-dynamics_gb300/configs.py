"""Seeded synthetic sphere packings for the step's workloads.

No public dataset stands behind these runs: every configuration is generated
here from a seed.  Monodisperse spheres of radius a = 1 in a cubic periodic
box of edge L = (N 4/3 pi / phi)^(1/3).
  phi <= 0.35  random sequential addition, uniform in [0, L)^3, rejecting any
               periodic surface gap below g_min;
  phi >  0.35  start from a lattice (simple cubic when its spacing clears
               2a + g_min, else face-centred cubic), drop surplus sites at
               random, then Metropolis hard-sphere sweeps with hard core
               2a + g_min and a step tuned towards 40 % acceptance.
Near-contact pairs (the learned-preconditioner workload): after the sweeps,
N/4 disjoint nearest-neighbour pairs are brought to a surface gap drawn
log-uniform in [1e-4, 1e-1] a, accepting a move only if every other gap
stays >= 1e-4 a.
Gaps are measured with the minimum image of the unsheared cubic lattice; a
step at strain gamma T shifts images by L gamma T along x, so runs start at
T = 0 like the reference's shear start-up.
"""
from __future__ import annotations

import math

import numpy as np

SEED_BASE = 20260000


def box_edge(N, phi, a=1.0):
    return (N * 4.0 / 3.0 * math.pi * a ** 3 / phi) ** (1.0 / 3.0)


def _min_image(d, L):
    return d - L * np.round(d / L)


def _gap_ok(pos, i, p, L, hard):
    d = _min_image(pos - p, L)
    r2 = np.einsum("ij,ij->i", d, d)
    r2[i] = np.inf
    return bool(np.all(r2 >= hard * hard))


def _rsa(N, L, hard, rng, max_tries=2_000_000):
    pos = np.empty((N, 3))
    n = 0
    tries = 0
    while n < N:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("random sequential addition did not reach N=%d" % N)
        p = rng.uniform(0.0, L, 3)
        if n:
            d = _min_image(pos[:n] - p, L)
            if np.min(np.einsum("ij,ij->i", d, d)) < hard * hard:
                continue
        pos[n] = p
        n += 1
    return pos


def _lattice_start(N, L, hard, rng):
    """Sites of the simple-cubic, body-centred or face-centred cubic lattice
    (the smallest cell count holding N sites) with the widest
    nearest-neighbour spacing; surplus sites are dropped at random."""
    options = []
    for name, per, basis, nn_frac in (("sc", 1, [[0, 0, 0]], 1.0),
                                      ("bcc", 2, [[0, 0, 0], [0.5, 0.5, 0.5]], math.sqrt(3.0) / 2.0),
                                      ("fcc", 4, [[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]],
                                       1.0 / math.sqrt(2.0))):
        m = int(math.ceil((N / per) ** (1.0 / 3.0) - 1e-9))
        spacing = L / m * nn_frac
        if spacing >= hard:
            options.append((spacing, m, np.array(basis, dtype=float)))
    if not options:
        raise RuntimeError("volume fraction too high for a lattice start")
    _, m, basis = max(options, key=lambda t: t[0])
    c = L / m
    g = np.arange(m)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    sites = ((cells[:, None, :] + basis[None] + 0.25) * c).reshape(-1, 3)
    keep = rng.permutation(len(sites))[:N]
    return sites[np.sort(keep)].copy()


def _mc_sweeps(pos, L, hard, rng, sweeps):
    N = len(pos)
    step = 0.1 * hard
    for _ in range(sweeps):
        acc = 0
        for i in rng.permutation(N):
            p = pos[i] + rng.uniform(-step, step, 3)
            p %= L
            if _gap_ok(pos, i, p, L, hard):
                pos[i] = p
                acc += 1
        rate = acc / N
        step *= 1.2 if rate > 0.45 else (0.8 if rate < 0.35 else 1.0)
        step = min(step, 0.5 * L)
    return pos


def _near_contact_pairs(pos, L, rng, a=1.0, lo=1e-4, hi=1e-1):
    N = len(pos)
    used = np.zeros(N, bool)
    order = rng.permutation(N)
    made = 0
    for i in order:
        if made >= N // 4 or used[i]:
            continue
        d = _min_image(pos - pos[i], L)
        r = np.sqrt(np.einsum("ij,ij->i", d, d))
        r[i] = np.inf
        r[used] = np.inf
        j = int(np.argmin(r))
        if not np.isfinite(r[j]):
            continue
        gap = math.exp(rng.uniform(math.log(lo), math.log(hi))) * a
        u = d[j] / r[j]
        new = (pos[i] + u * (2 * a + gap)) % L
        others = np.ones(N, bool)
        others[[i, j]] = False
        dd = _min_image(pos[others] - new, L)
        if np.min(np.sqrt(np.einsum("ij,ij->i", dd, dd))) - 2 * a < lo * a:
            continue
        pos[j] = new
        used[i] = used[j] = True
        made += 1
    return pos


def packing(N, phi, g_min, seed, sweeps=200, near_contact=False, a=1.0):
    """Positions (N, 3) and radii (N,) of a seeded packing, and the box edge."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = box_edge(N, phi, a)
    hard = 2 * a + g_min * a
    if phi <= 0.35:
        pos = _rsa(N, L, hard, rng)
    else:
        pos = _lattice_start(N, L, hard, rng)
        pos = _mc_sweeps(pos, L, hard, rng, sweeps)
    if near_contact:
        pos = _near_contact_pairs(pos, L, rng, a)
    return pos, np.full(N, a), L


def min_gap(pos, L, a=1.0):
    """Smallest periodic surface gap (cubic minimum image)."""
    best = np.inf
    for i in range(len(pos) - 1):
        d = _min_image(pos[i + 1:] - pos[i], L)
        best = min(best, float(np.sqrt(np.min(np.einsum("ij,ij->i", d, d)))) - 2 * a)
    return best


# Workloads by number: the configurations the step is measured and checked on.
WORKLOADS = {
    1: dict(N=64, phi=0.30, g_min=0.01, gamma=1.0, dt=1e-3, steps=100),
    2: dict(N=512, phi=0.45, g_min=1e-3, gamma=1.0, dt=1e-3, steps=200),
    4: dict(N=1000, phi=0.50, g_min=1e-4, gamma=1.0, dt=5e-4, steps=1, near_contact=True),
    5: dict(N=2048, phi=0.50, g_min=1e-4, gamma=1.0, dt=5e-4, steps=10000),
}


def workload(num, replica=0, sweeps=None):
    w = dict(WORKLOADS[num])
    seed = SEED_BASE + num * 1000 + replica
    pos, radii, L = packing(w["N"], w["phi"], w["g_min"], seed, sweeps=200 if sweeps is None else sweeps,
                            near_contact=w.get("near_contact", False))
    w.update(pos=pos, radii=radii, L=L, seed=seed)
    return w
