"""Seeded synthetic sphere packings for the step's workloads.

No public dataset stands behind these runs: every configuration is generated
here from a seed.  Monodisperse spheres of radius a = 1 in a cubic periodic
box of edge L = (N 4/3 pi / phi)^(1/3).
  phi <= 0.35  random sequential addition, uniform in [0, L)^3, rejecting any
               periodic surface gap below g_min;
  phi >  0.35  start from a lattice (simple cubic when its spacing clears
               2a + g_min, else face-centred cubic), drop surplus sites at
               random, then Metropolis hard-sphere sweeps with hard core
               2a + g_min and a step tuned towards 40 % acceptance.  Where
               no cubic lattice of the box holds N sites that far apart (a
               few small N just above a lattice's site count), the start is
               instead random sequential addition at phi = 0.3 in a larger
               box, compressed to the target box in small affine steps with
               the overlaps of each step pushed apart.
Near-contact pairs (the learned-preconditioner workload): after the sweeps,
N/4 disjoint nearest-neighbour pairs are brought to a surface gap drawn
log-uniform in [1e-4, 1e-1] a, accepting a move only if every other gap
stays >= 1e-4 a.
Gaps are measured with the minimum image of the unsheared cubic lattice; a
step at strain gamma T shifts images by L gamma T along x, so runs start at
T = 0 like the reference's shear start-up.

sheared_packing() gives a configuration for a run that is already at strain
s (the Lees-Edwards lattice with LR(1,3) = s L, csd_post.f90:105-136): the
packing above is sheared affinely, x += ds z, in increments of the lattice's
skew (the images follow the same affine map, so every pair, across the
boundary too, moves continuously), and after each increment overlapping
pairs (gap below g_min in the sheared minimum image) are pushed apart along
their centre line until none is left.
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


def _compressed_start(N, L, hard, rng, phi0=0.3, steps=200):
    """Random sequential addition in the box of volume fraction phi0, then
    affine compression to edge L in `steps` steps, each followed by pushing
    overlapping pairs (minimum image) apart along their centre lines."""
    L0 = max(box_edge(N, phi0, hard / 2.0), L)
    pos = _rsa(N, L0, hard, rng)
    push = hard + 0.01
    for k in range(1, steps + 1):
        Lk = L0 + (L - L0) * k / steps
        pos = pos * (Lk / (L0 + (L - L0) * (k - 1) / steps))
        for _ in range(5000):
            d = pos[None, :, :] - pos[:, None, :]
            d = _min_image(d, Lk)
            r = np.sqrt(np.einsum("ijk,ijk->ij", d, d))
            np.fill_diagonal(r, np.inf)
            i, j = np.nonzero(np.triu(r < hard, 1))
            if len(i) == 0:
                break
            u = d[i, j] / r[i, j, None] * (0.5 * (push - r[i, j]))[:, None]
            np.add.at(pos, i, -u)
            np.add.at(pos, j, u)
            pos %= Lk
        else:
            raise RuntimeError("compression did not clear the overlaps")
    return pos % L


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
        try:
            pos = _lattice_start(N, L, hard, rng)
        except RuntimeError:
            pos = _compressed_start(N, L, hard, rng)
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


def _sheared_lattice(L, skew):
    LR = np.diag([L, L, L]).astype(float)
    LR[0, 2] = skew * L
    return LR, np.linalg.inv(LR)


_SHIFTS = np.array([[i, j, k] for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)], dtype=float)


def sheared_min_image(d, LR, LI):
    """Minimum images of separations d (..., 3) in the lattice LR (skew in
    [0, 1]): the nearest of the 27 cells around the rounded fractional
    coordinates."""
    u = d @ LI.T
    u -= np.round(u)
    c = (u[..., None, :] + _SHIFTS) @ LR.T
    k = np.argmin(np.einsum("...ij,...ij->...i", c, c), axis=-1)
    return np.take_along_axis(c, k[..., None, None], axis=-2)[..., 0, :]


def _pairs_within(pos, L, skew, cut, chunk=512):
    """Pairs i < j whose minimum image is closer than cut (< L/2), with the
    integer lattice shift n of that image: d_ij = pos[j] - pos[i] + LR n.
    For such a pair the shift along z (and y) is the one that brings that
    coordinate within L/2, and then the one along x the same for x
    (LR = [[L, 0, skew L], [0, L, 0], [0, 0, L]])."""
    N = len(pos)
    ii, jj, nn = [], [], []
    for a in range(0, N, chunk):
        d = pos[None, :, :] - pos[a:a + chunk, None, :]
        n3 = -np.round(d[..., 2] / L)
        n2 = -np.round(d[..., 1] / L)
        x = d[..., 0] + skew * L * n3
        n1 = -np.round(x / L)
        r2 = (x + L * n1) ** 2 + (d[..., 1] + L * n2) ** 2 + (d[..., 2] + L * n3) ** 2
        i, j = np.nonzero(r2 < cut * cut)
        keep = j > i + a
        i, j = i[keep], j[keep]
        ii.append(i + a)
        jj.append(j)
        nn.append(np.stack([n1[i, j], n2[i, j], n3[i, j]], -1))
    return np.concatenate(ii), np.concatenate(jj), np.concatenate(nn)


def sheared_min_gap(pos, L, skew, a=1.0):
    """Smallest surface gap in the lattice of skew `skew` (0 <= skew <= 1)."""
    LR, LI = _sheared_lattice(L, skew)
    i, j, n = _pairs_within(pos, L, skew, 2 * a + 1.0)
    if len(i) == 0:
        return np.inf
    d = pos[j] - pos[i] + n @ LR.T
    return float(np.sqrt(np.einsum("ij,ij->i", d, d)).min()) - 2 * a


def sheared_series(N, phi, g_min, seed, strains, sweeps=200, near_contact=False, a=1.0, dskew=0.005):
    """Configurations valid at each Lees-Edwards skew mod(strain, 1) of
    `strains` (each in [0, 1), ascending), from one packing sheared
    incrementally: every surface gap in the sheared minimum image is at least
    g_min (near_contact pairs keep at least 1e-4 a).  Returns the list of
    positions (wrapped into each sheared cell), the radii and the box edge."""
    pos, radii, L = packing(N, phi, g_min, seed, sweeps=sweeps, near_contact=near_contact, a=a)
    hard = 2 * a + (1e-4 * a if near_contact else g_min * a)
    push = hard + 0.01 * a
    skew, nlist_at = 0.0, -1.0
    out = []
    for target in [float(x) % 1.0 for x in strains]:
        if target < skew:
            raise ValueError("strains must be ascending within [0, 1)")
        while skew < target:
            ds = min(dskew, target - skew)
            pos[:, 0] += ds * pos[:, 2]  # affine shear of the positions with the lattice
            skew += ds
            LR, LI = _sheared_lattice(L, skew)
            if skew - nlist_at > 0.05:
                i, j, n = _pairs_within(pos, L, skew, 2 * a + 1.0)
                nlist_at = skew
            for _ in range(2000):
                d = pos[j] - pos[i] + n @ LR.T
                r = np.sqrt(np.einsum("ij,ij->i", d, d))
                bad = r < hard
                if not bad.any():
                    break
                u = d[bad] / r[bad, None] * (0.5 * (push - r[bad]))[:, None]
                np.add.at(pos, i[bad], -u)
                np.add.at(pos, j[bad], u)
            else:
                raise RuntimeError("sheared packing: overlaps remain at skew %.3f" % skew)
        LR, LI = _sheared_lattice(L, target)
        u = pos @ LI.T
        out.append((u - np.floor(u)) @ LR.T)
    return out, radii, L


def sheared_packing(N, phi, g_min, seed, strain, sweeps=200, near_contact=False, a=1.0, dskew=0.005):
    """A packing valid at Lees-Edwards skew mod(strain, 1): every surface gap
    in the sheared minimum image is at least g_min (near_contact pairs keep
    at least 1e-4 a).  Positions are wrapped into the sheared cell."""
    out, radii, L = sheared_series(N, phi, g_min, seed, [strain], sweeps, near_contact, a, dskew)
    return out[0], radii, L


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
