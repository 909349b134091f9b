"""The learned preconditioner of the resistance solve (csrc/learned.cu)
through the C-ABI.

  - Each BF16 kernel of the network (encoders, message and update layers,
    aggregation, heads; their backward passes; the Adam step) against an FP32
    PyTorch restatement of the same network on a random graph.  The kernels
    keep weights and activations in BF16 (8 significant bits) and accumulate
    in FP32, so outputs are compared to 3e-2 and gradients to 6e-2 of their
    largest entry; the Adam step, done in FP32 on both sides, to 1e-6.
  - The exact FSAI blocks against a NumPy restatement on the same matrix and
    graph (1e-9 of the largest block entry).
  - PCG on RPP with every preconditioner: the solution against a dense
    solve (1e-9), the iteration counts ordered as a preconditioner should
    make them.
  - The plain FP64 step with the PCG solve of RPP (FSAI and learned) against
    the oracle's STEPPER_Stokesian: 1e-10 (PCG to 1e-13 on cond(RPP) ~ 1e3).
"""
import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as o

pytestmark = pytest.mark.gpu

MU = o.mu_f_dimensionless(1.0)
H = 64


@pytest.fixture(scope="module")
def rsd():
    ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="module")
def ctx(rsd):
    return rsd.Context(0)


def bf16(t):
    import torch
    return t.to(torch.bfloat16).to(torch.float32)


def unpack(p):
    """The parameter layout of learned.cu (weights row-major [out][in])."""
    import torch
    shapes = [("enc_n_w", (H, 36)), ("enc_n_b", (H,)), ("enc_e_w", (H, 40)), ("enc_e_b", (H,))]
    for l in range(3):
        shapes += [("msg_w%d" % l, (H, 3 * H)), ("msg_b%d" % l, (H,)), ("upd_w%d" % l, (H, 2 * H)),
                   ("upd_b%d" % l, (H,))]
    shapes += [("head_n_w", (36, H)), ("head_n_b", (36,)), ("head_e_w", (36, 3 * H)), ("head_e_b", (36,))]
    out, o_ = {}, 0
    for name, shp in shapes:
        n = int(np.prod(shp))
        out[name] = p[o_:o_ + n].reshape(shp)
        o_ += n
    assert o_ == p.numel()
    return out


def reference_forward(W, off, src, dst, xn, xe):
    """FP32 restatement with the kernels' BF16 roundings of weights, inputs
    and stored activations."""
    import torch
    relu = torch.relu
    Wb = {k: (bf16(v) if k.endswith("_w") or "_w" in k else v) for k, v in W.items()}
    h = bf16(relu(bf16(xn) @ Wb["enc_n_w"].T + W["enc_n_b"]))
    m = bf16(relu(bf16(xe) @ Wb["enc_e_w"].T + W["enc_e_b"]))
    for l in range(3):
        msg = bf16(relu(torch.cat([h[dst], h[src], m], 1) @ Wb["msg_w%d" % l].T + W["msg_b%d" % l]))
        m = bf16(m + msg)
        agg = bf16(torch.zeros_like(h).index_add_(0, dst, msg))
        u = bf16(relu(torch.cat([h, agg], 1) @ Wb["upd_w%d" % l].T + W["upd_b%d" % l]))
        h = bf16(h + u)
    zd = h @ Wb["head_n_w"].T + W["head_n_b"] + torch.eye(6, device=h.device).reshape(36)
    ze = torch.cat([m, h[dst], h[src]], 1) @ Wb["head_e_w"].T + W["head_e_b"]
    return zd, ze


def random_graph(N, seed, torch):
    rng = np.random.default_rng(seed)
    pairs = set()
    for a in range(N):
        for b in rng.choice(N, size=6, replace=False):
            if b != a:
                pairs.add((min(a, b), max(a, b)))
    e = sorted([(a, b) for a, b in pairs] + [(b, a) for a, b in pairs])  # (dst, src), sorted
    dst = np.array([x[0] for x in e], dtype=np.int32)
    src = np.array([x[1] for x in e], dtype=np.int32)
    off = np.zeros(N + 1, dtype=np.int32)
    np.add.at(off, dst + 1, 1)
    off = np.cumsum(off).astype(np.int32)
    t = lambda a: torch.tensor(a, device="cuda")
    return t(off), t(src), t(dst)


def test_network_kernels_against_fp32_reference(rsd, ctx):
    import torch
    N = 50
    off, src, dst = random_graph(N, 3, torch)
    ne = src.shape[0]
    g = torch.Generator(device="cpu").manual_seed(7)
    net = rsd.LearnedPreconditioner(0, seed=11)
    p0 = net.params()
    # non-zero heads and biases so that every path carries signal
    p0 = p0 + 0.05 * torch.randn(p0.size, generator=g).numpy().astype(np.float32)
    net = rsd.LearnedPreconditioner(0, params=p0)
    xn = torch.randn(N, 36, generator=g).cuda()
    xe = torch.randn(ne, 40, generator=g).cuda()
    dzd = torch.randn(N, 36, generator=g).cuda()
    dze = torch.randn(ne, 36, generator=g).cuda()
    lower = (src < dst)
    dze_masked = dze * lower[:, None]
    zd, ze = net.forward(ctx, off, src, dst, xn, xe, dzd, dze)
    W = {k: v.cuda().requires_grad_(True) for k, v in unpack(torch.tensor(p0)).items()}
    rzd, rze = reference_forward(W, off.long(), src.long(), dst.long(), xn, xe)
    assert (zd - rzd).abs().max() <= 3e-2 * rzd.abs().max()
    assert (ze - rze).abs().max() <= 3e-2 * rze.abs().max()
    # backward: the kernels' gradient of sum(zd * dzd) + sum over lower edges of ze * dze
    loss = (rzd * dzd).sum() + (rze * dze_masked).sum()
    loss.backward()
    got = unpack(torch.tensor(net.grad()))
    for k, v in W.items():
        ref = v.grad.cpu()
        assert (got[k] - ref).abs().max() <= 6e-2 * max(ref.abs().max(), 1e-6), k
    # Adam: one step from zero moments moves each weight by lr * g / (|g| + eps)
    lr = 1e-3
    g_all = net.grad().astype(np.float64)
    net.adam_step(lr)
    expect = p0.astype(np.float64) - lr * g_all / (np.abs(g_all) + 1e-8)
    assert np.abs(net.params() - expect).max() <= 1e-6


def system(rsd, ctx, tab, N, phi, gmin, seed, T=0.0, near_contact=False):
    import torch
    pos, radii, L = rsd.configs.sheared_packing(N, phi, gmin, seed, T, sweeps=30, near_contact=near_contact)
    pos_t = torch.tensor(pos, dtype=torch.float64, device="cuda")
    radii_t = torch.tensor(radii, dtype=torch.float64, device="cuda")
    rpp, lat = rsd.resistance_pp_dev(ctx, tab, pos_t, radii_t, T, [L, L, L], 1.0, MU, 1e-10)
    return pos, radii, L, pos_t, radii_t, rpp, lat


def numpy_fsai(R, N, off, src, gap, kmax=16):
    """Block FSAI restated: particle-block layout, Jacobi scaling, per
    particle the nearest (by gap) kmax lower neighbours and itself; Z_a =
    L^-1 Y^T with Y = B^-1 E_a and Y_aa = L L^T (Cholesky)."""
    p = np.array([[3 * a, 3 * a + 1, 3 * a + 2, 3 * N + 3 * a, 3 * N + 3 * a + 1, 3 * N + 3 * a + 2]
                  for a in range(N)]).ravel()
    A = R[np.ix_(p, p)]
    d = 1.0 / np.sqrt(np.diag(A))
    A = A * d[:, None] * d[None, :]
    zd = np.zeros((N, 6, 6))
    ze = {}
    for a in range(N):
        es = [e for e in range(off[a], off[a + 1]) if src[e] < a]
        es = sorted(es, key=lambda e: gap[e])[:kmax]
        nb = [src[e] for e in es] + [a]
        J = np.concatenate([np.arange(6 * b, 6 * b + 6) for b in nb])
        E = np.zeros((len(J), 6))
        E[-6:] = np.eye(6)
        Y = np.linalg.solve(A[np.ix_(J, J)], E)
        S = np.linalg.inv(np.linalg.cholesky(0.5 * (Y[-6:] + Y[-6:].T)))
        Z = S @ Y.T
        zd[a] = Z[:, -6:]
        for q, e in enumerate(es):
            ze[e] = Z[:, 6 * q:6 * q + 6]
    return zd, ze


def test_exact_fsai_against_numpy(rsd, ctx):
    tab = rsd.LubTab(rsd.lubdat_dir())
    pos, radii, L, pos_t, radii_t, rpp, lat = system(rsd, ctx, tab, 64, 0.45, 1e-3, 20262200, T=0.6)
    R = rpp.cpu().numpy()
    assert np.abs(R - R.T).max() <= 1e-12 * np.abs(R).max()
    zd, ze, off, src = rsd.lp_blocks_dev(ctx, None, rsd.PC_FSAI, pos_t, radii_t, lat, rpp)
    _, gap = rsd.lp_graph_dev(ctx, pos_t, radii_t, lat)[1:]
    rzd, rze = numpy_fsai(R, 64, off, src, gap)
    scale = np.abs(rzd).max()
    assert np.abs(zd - rzd).max() <= 1e-5 * scale  # blocks are stored in FP32
    for e, blk in rze.items():
        assert np.abs(ze[e] - blk).max() <= 1e-5 * scale
    # the graph: pairs closer than 3 a, both directions, sources ascending
    assert all(np.all(np.diff(src[off[a]:off[a + 1]]) > 0) for a in range(64))
    assert len(src) % 2 == 0


def test_learned_blocks_are_normalised(rsd, ctx):
    """Whatever the network emits (here an untrained one), each row block of
    the learned Z satisfies (Z A^ Z^T)_aa = I on the Jacobi-scaled RPP, so
    that G = Z^T Z is SPD (FP32 storage of the blocks: 1e-4)."""
    tab = rsd.LubTab(rsd.lubdat_dir())
    pos, radii, L, pos_t, radii_t, rpp, lat = system(rsd, ctx, tab, 64, 0.45, 1e-3, 20262204, T=0.3)
    net = rsd.LearnedPreconditioner(0, seed=9)
    p0 = net.params()
    p0 += 0.05 * np.random.default_rng(9).normal(size=p0.size).astype(np.float32)  # non-zero heads
    net = rsd.LearnedPreconditioner(0, params=p0)
    zd, ze, off, src = rsd.lp_blocks_dev(ctx, net, rsd.PC_LEARNED, pos_t, radii_t, lat, rpp)
    N = 64
    R = rpp.cpu().numpy()
    p = np.array([[3 * a, 3 * a + 1, 3 * a + 2, 3 * N + 3 * a, 3 * N + 3 * a + 1, 3 * N + 3 * a + 2]
                  for a in range(N)]).ravel()
    A = R[np.ix_(p, p)]
    d = 1.0 / np.sqrt(np.diag(A))
    A = A * d[:, None] * d[None, :]
    Z = np.zeros((6 * N, 6 * N))
    for a in range(N):
        Z[6 * a:6 * a + 6, 6 * a:6 * a + 6] = zd[a]
        for e in range(off[a], off[a + 1]):
            if src[e] < a:
                Z[6 * a:6 * a + 6, 6 * src[e]:6 * src[e] + 6] = ze[e]
    C = Z @ A @ Z.T
    for a in range(N):
        assert np.abs(C[6 * a:6 * a + 6, 6 * a:6 * a + 6] - np.eye(6)).max() <= 1e-4
    ev = np.linalg.eigvalsh(0.5 * (C + C.T))
    # Z A Z^T is positive definite in exact arithmetic; in FP64 its smallest
    # eigenvalue may round to a few ulps of the largest below zero
    assert ev.min() > -1e-12 * ev.max()


def test_pcg_every_preconditioner(rsd, ctx):
    """Every preconditioner's PCG solve of an FP64 RPP (N = 128, phi = 0.5,
    near-contact pairs) against numpy's solve; the analytic preconditioners
    in their expected order.  (This packing is relaxed less than the
    trajectories the network was trained on; there the learned blocks take
    about as many iterations as no preconditioner, so their count is only
    reported.)"""
    import torch
    tab = rsd.LubTab(rsd.lubdat_dir())
    pos, radii, L, pos_t, radii_t, rpp, lat = system(rsd, ctx, tab, 128, 0.5, 1e-4, 20262201, near_contact=True)
    R = rpp.cpu().numpy()
    b = np.random.default_rng(5).normal(size=(2, R.shape[0]))
    x_ref = np.linalg.solve(R, b.T).T
    net = rsd.LearnedPreconditioner.trained(0)
    its = {}
    for mode in (rsd.PC_NONE, rsd.PC_JACOBI, rsd.PC_BLOCK_JACOBI, rsd.PC_FSAI, rsd.PC_LEARNED):
        x, it, res = rsd.pcg_dev(ctx, net, mode, pos_t, radii_t, lat, rpp,
                                 torch.tensor(b, device="cuda"), tol=1e-13, maxit=5000)
        assert res <= 1e-13, (mode, it, res)
        assert np.abs(x.cpu().numpy() - x_ref).max() <= 1e-9 * np.abs(x_ref).max(), mode
        its[mode] = it
    print("PCG iterations by preconditioner:", its)
    assert its[rsd.PC_FSAI] < its[rsd.PC_BLOCK_JACOBI] <= its[rsd.PC_NONE]


def test_learned_preconditioner_on_the_workload(rsd, ctx):
    """The trained network on a held-out system of its workload (N = 1000,
    phi = 0.5, near-contact pairs, sheared and relaxed like the training
    trajectories, FP64 RPP): fewer PCG iterations than block Jacobi and than
    no preconditioner, the same solution."""
    import torch
    tab = rsd.LubTab(rsd.lubdat_dir())
    N = 1000
    series, radii, L = rsd.configs.sheared_series(N, 0.5, 1e-4, 20262210, [0.4], sweeps=100, near_contact=True)
    pos_t = torch.tensor(series[0], dtype=torch.float64, device="cuda")
    radii_t = torch.tensor(radii, dtype=torch.float64, device="cuda")
    rpp, lat = rsd.resistance_pp_dev(ctx, tab, pos_t, radii_t, 0.4, [L, L, L], 1.0, MU, 1e-10)
    b = torch.tensor(np.random.default_rng(6).normal(size=6 * N), device="cuda")
    net = rsd.LearnedPreconditioner.trained(0)
    its, xs = {}, {}
    for mode in (rsd.PC_NONE, rsd.PC_BLOCK_JACOBI, rsd.PC_FSAI, rsd.PC_LEARNED):
        x, it, res = rsd.pcg_dev(ctx, net, mode, pos_t, radii_t, lat, rpp, b, tol=1e-12, maxit=5000)
        assert res <= 1e-12, (mode, it, res)
        its[mode], xs[mode] = it, x.cpu().numpy()
    print("PCG iterations by preconditioner (N = 1000):", its)
    assert its[rsd.PC_LEARNED] < its[rsd.PC_BLOCK_JACOBI] < its[rsd.PC_NONE]
    ref = xs[rsd.PC_FSAI]
    # each solve to 1e-12 relative residual: the solutions differ by at most
    # about cond(RPP) * 1e-12 (cond up to ~1e5 with gaps of 1e-4)
    assert np.abs(xs[rsd.PC_LEARNED] - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize("mode", ["fsai", "learned"])
def test_plain_step_with_pcg_solve(rsd, mode):
    """The plain FP64 step with RPP solved by PCG against the oracle."""
    tabs = rsd.LubTab(rsd.lubdat_dir()), o.LubTab(rsd.lubdat_dir())
    N = 64
    pos, radii, L = rsd.configs.sheared_packing(N, 0.45, 1e-3, 20262202, 0.3, sweeps=30)
    ctx = rsd.Context(0)
    net = rsd.LearnedPreconditioner.trained(0) if mode == "learned" else None
    ctx.set_rpp_solver(rsd.PC_LEARNED if mode == "learned" else rsd.PC_FSAI, net, tol=1e-13, maxit=3000)
    g = rsd.STEPPER_Stokesian(ctx, tabs[0], pos, radii, 0.3, 1e-3, [L, L, L], 1.0, MU, 1e-10)
    r = o.stepper_stokesian(pos, radii, [L, L, L], 0.3, 1e-3, 1.0, MU, 1e-10, tabs[1])
    assert g["info"].rpp_iterations > 0  # converged by PCG, no fallback
    rel = lambda a, b: np.abs(a - b).max() / np.abs(b).max()
    assert rel(g["U_pos"], r["U_pos"]) <= 1e-10
    assert rel(g["SijN"], r["SijN_hyd"]) <= 1e-10


def test_training_step_reduces_the_loss(rsd, ctx):
    """Supervised steps on one FP32 resistance matrix of the mixed form
    lower the block error against its exact FSAI blocks."""
    import torch
    tab = rsd.LubTab(rsd.lubdat_dir())
    pos, radii, L = rsd.configs.packing(64, 0.45, 1e-3, 20262203, sweeps=30)
    pos_t = torch.tensor(pos, dtype=torch.float64, device="cuda")
    radii_t = torch.tensor(radii, dtype=torch.float64, device="cuda")
    rpp32, lat = rsd.resistance_pp_dev(ctx, tab, pos_t, radii_t, 0.0, [L, L, L], 1.0, MU, 1e-10,
                                       precision=rsd.PREC_MIXED)
    rpp64, _ = rsd.resistance_pp_dev(ctx, tab, pos_t, radii_t, 0.0, [L, L, L], 1.0, MU, 1e-10)
    assert (rpp32.double() - rpp64).abs().max() <= 1e-3 * rpp64.abs().max()
    net = rsd.LearnedPreconditioner(0, seed=5)
    # Z starts at I (zero heads), already close to the targets after the
    # Jacobi scaling: a learning rate warmed up over 20 steps keeps the first
    # Adam steps from overshooting
    losses = [net.train_step(ctx, pos_t, radii_t, lat, rpp32, 1e-3 * min(1.0, (k + 1) / 20.0)) for k in range(200)]
    assert np.isfinite(losses).all()
    assert np.mean(losses[-10:]) < 0.8 * losses[0], losses[::20]


def test_training_guards(rsd, ctx):
    """A step whose loss is above the loss guard makes no update; the
    gradient clip bounds the first Adam step whatever the gradient's size."""
    import torch
    tab = rsd.LubTab(rsd.lubdat_dir())
    pos, radii, L = rsd.configs.packing(64, 0.45, 1e-3, 20262204, sweeps=30)
    pos_t = torch.tensor(pos, dtype=torch.float64, device="cuda")
    radii_t = torch.tensor(radii, dtype=torch.float64, device="cuda")
    rpp32, lat = rsd.resistance_pp_dev(ctx, tab, pos_t, radii_t, 0.0, [L, L, L], 1.0, MU, 1e-10,
                                       precision=rsd.PREC_MIXED)
    net = rsd.LearnedPreconditioner(0, seed=6)
    w0 = net.params()
    net.set_training(0.0, 1e-30)  # every loss is above the guard
    l0 = net.train_step(ctx, pos_t, radii_t, lat, rpp32, 1e-3)
    assert l0 > 1e-30
    assert np.array_equal(net.params(), w0)
    g0, skipped, steps = net.training_stats()
    assert (skipped, steps) == (1, 0) and g0 == 0.0
    gn = np.linalg.norm(net.grad().astype(np.float64))  # the skipped step's gradient is kept
    assert gn > 1e-4
    net.set_training(0.1 * gn, 0.0)  # a clip at a tenth of the norm
    l1 = net.train_step(ctx, pos_t, radii_t, lat, rpp32, 1e-3)
    assert abs(l1 - l0) <= 1e-6 * l0  # same weights, same sample (up to the order of atomic sums)
    g1, skipped, steps = net.training_stats()
    assert (skipped, steps) == (1, 1)
    assert abs(g1 - gn) <= 1e-4 * gn  # the norm before the clip
    w1 = net.params()
    # Adam's first step moves each weight by lr * sign(g) whatever the scale
    # of g (to within eps / |g|), so the clip leaves its size unchanged
    d = np.abs(w1 - w0)
    assert d.max() <= 1e-3 * 1.001 and d.max() >= 0.5e-3
