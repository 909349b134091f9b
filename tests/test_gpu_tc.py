"""The FP32 building blocks of the mixed-precision form, tensor-core (tcgen05
TF32 and 3xTF32) and SIMT, against FP64 numpy references of the same
operations.

Tolerances (prec 0 = FP32 SIMT, 1 = TF32, 3 = 3xTF32):
  SYRK: |err| <= tol * (|P|^T |P|) + 1e-5 |C| elementwise, tol = 1e-5 (SIMT),
  3e-3 (TF32 keeps 10 mantissa bits: 2^-11 relative per operand, two operands
  per product) and 2e-5 (3xTF32: about 2^-21 per product);
  factor: ||U^T U - A|| / ||A|| <= 1e-5, 2e-3, 2e-5;
  inverse: ||X A - I|| / sqrt(n) <= 1e-5, 1e-2, 6e-5 on a matrix with
  condition number below 10."""
import numpy as np
import pytest

import __graft_entry__ as ge

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def rsd():
    ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="module")
def ctx(rsd):
    return rsd.Context(0)


def colmajor(a):
    """Device FP32 column-major copy of a 2-D numpy array, as the transpose
    view of a contiguous tensor."""
    return torch.from_numpy(np.ascontiguousarray(a.T, dtype=np.float32)).cuda().t()


def upper_tile_mask(n, t=128):
    bi = np.arange(n) // t
    return bi[:, None] <= bi[None, :]


SYRK_TOL = {0: 1e-5, 1: 3e-3, 3: 2e-5}
FACTOR_TOL = {0: 1e-5, 1: 2e-3, 3: 2e-5}
INV_TOL = {0: 1e-5, 1: 1e-2, 3: 6e-5}


@pytest.mark.parametrize("n,k", [(128, 128), (1000, 128), (700, 96), (300, 64)])
@pytest.mark.parametrize("prec", [0, 1, 3])
def test_syrk_f32(rsd, ctx, n, k, prec):
    rng = np.random.default_rng(20261203 + n + k)
    P = rng.standard_normal((k, n)).astype(np.float32)
    C = rng.standard_normal((n, n)).astype(np.float32)
    dP, dC = colmajor(P), colmajor(C)
    before = rsd.library().rsd_launch_count()
    rsd.syrk_f32_dev(ctx, dP, dC, prec)
    assert rsd.library().rsd_launch_count() - before == 1
    got = dC.cpu().numpy()
    P64 = P.astype(np.float64)
    want = C.astype(np.float64) - P64.T @ P64
    scale = np.abs(P64).T @ np.abs(P64)
    mask = upper_tile_mask(n)
    err = np.abs(got - want)
    bound = SYRK_TOL[prec] * scale + 1e-5 * np.abs(C)
    assert np.all(err[mask] <= bound[mask]), float((err / bound)[mask].max())
    # tiles strictly below the diagonal are not touched
    assert np.array_equal(got[~mask], C[~mask])
    if prec == 1:
        # TF32 products differ from FP32 ones: the tensor-core path ran
        assert err[mask].max() > 1e-6 * scale[mask].max()
    if prec == 3:
        dC2 = colmajor(C)
        rsd.syrk_f32_dev(ctx, dP, dC2, 0)
        assert not np.array_equal(dC2.cpu().numpy()[mask], got[mask])


def spd(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, n))
    return X @ X.T / n + np.eye(n)


@pytest.mark.parametrize("n", [128, 640, 1100, 1001])
@pytest.mark.parametrize("prec", [0, 1, 3])
def test_potrf_f32(rsd, ctx, n, prec):
    A = spd(n, 20261204 + n)
    dA = colmajor(A)
    info = rsd.potrf_f32_dev(ctx, dA, prec)
    assert info == 0
    U = np.triu(dA.cpu().numpy().astype(np.float64))
    res = np.linalg.norm(U.T @ U - A) / np.linalg.norm(A)
    assert res <= FACTOR_TOL[prec], res


@pytest.mark.parametrize("n", [256, 640, 1100, 1001])
@pytest.mark.parametrize("prec", [0, 1, 3])
def test_potri_f32(rsd, ctx, n, prec):
    A = spd(n, 20261205 + n)
    dA = colmajor(A)
    assert rsd.potrf_f32_dev(ctx, dA, 0) == 0
    rsd.potri_f32_dev(ctx, dA, prec)
    X = np.triu(dA.cpu().numpy().astype(np.float64))
    X = X + np.triu(X, 1).T
    res = np.linalg.norm(X @ A - np.eye(n)) / np.sqrt(n)
    assert res <= INV_TOL[prec], res


@pytest.mark.parametrize("n", [640, 1001, 1100, 1664, 2560])
@pytest.mark.parametrize("prec", [1, 3])
def test_potrf_f32_schedules_agree(rsd, ctx, n, prec):
    """The look-ahead schedule of the two-level factorisation (the default)
    and the in-order one give the same factor: every output tile is the same
    product over the same K range, only split into other launches."""
    A = spd(n, 20261206 + n)
    out = {}
    for sched in (0, 1):
        dA = colmajor(A)
        ctx.set_factor_schedule(sched)
        try:
            assert rsd.potrf_f32_dev(ctx, dA, prec) == 0
        finally:
            ctx.set_factor_schedule(1)
        out[sched] = np.triu(dA.cpu().numpy().astype(np.float64))
        res = np.linalg.norm(out[sched].T @ out[sched] - A) / np.linalg.norm(A)
        assert res <= FACTOR_TOL[prec], (sched, res)
    d = np.abs(out[0] - out[1]).max() / np.abs(out[0]).max()
    print("schedules 0 and 1: max difference %.3e (identical: %s)" % (d, d == 0.0))
    assert d <= 1e-5


def test_tensor_cores_off_matches_simt(rsd, ctx):
    """With the context switch off, prec 1 takes the SIMT path."""
    A = spd(640, 11)
    d1, d2 = colmajor(A), colmajor(A)
    ctx.set_tensor_cores(False)
    try:
        rsd.potrf_f32_dev(ctx, d1, 1)
    finally:
        ctx.set_tensor_cores(True)
    rsd.potrf_f32_dev(ctx, d2, 0)
    assert np.array_equal(np.triu(d1.cpu().numpy()), np.triu(d2.cpu().numpy()))


def test_potrf_f32_not_spd(rsd, ctx):
    n = 512
    A = spd(n, 7)
    A[300, 300] = -5.0
    info = rsd.potrf_f32_dev(ctx, colmajor(A), 1)
    assert info > 0


def test_prec_argument_checked(rsd, ctx):
    A = spd(64, 3)
    with pytest.raises(rsd.RSDError):
        rsd.potrf_f32_dev(ctx, colmajor(A), 2)
