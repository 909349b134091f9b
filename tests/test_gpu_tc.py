"""The FP32 building blocks of the mixed-precision form, tensor-core (tcgen05
TF32) and SIMT, against FP64 numpy references of the same operations.

Tolerances:
  SIMT FP32 SYRK: |err| <= 1e-5 * (|P|^T |P| + |C|) elementwise;
  TF32 SYRK: |err| <= 3e-3 * (|P|^T |P|) + 1e-5 |C| elementwise (TF32 keeps
  10 mantissa bits: 2^-11 relative per operand, two operands per product);
  factorisations: ||U^T U - A|| / ||A|| <= 1e-5 (SIMT) and 2e-3 (TF32)."""
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
    c = rsd.Context(0)
    yield c
    c.set_tensor_cores(True)


def colmajor(a):
    """Device FP32 column-major copy of a 2-D numpy array, as the transpose
    view of a contiguous tensor."""
    return torch.from_numpy(np.ascontiguousarray(a.T, dtype=np.float32)).cuda().t()


def upper_tile_mask(n, t=128):
    bi = np.arange(n) // t
    return bi[:, None] <= bi[None, :]


@pytest.mark.parametrize("n,k", [(128, 128), (1000, 128), (700, 96), (300, 64)])
@pytest.mark.parametrize("tc", [True, False])
def test_syrk_f32(rsd, ctx, n, k, tc):
    rng = np.random.default_rng(20261203 + n + k)
    P = rng.standard_normal((k, n)).astype(np.float32)
    C = rng.standard_normal((n, n)).astype(np.float32)
    ctx.set_tensor_cores(tc)
    dP, dC = colmajor(P), colmajor(C)
    before = launches = rsd.library().rsd_launch_count()
    rsd.syrk_f32_dev(ctx, dP, dC)
    launches = rsd.library().rsd_launch_count() - before
    assert launches == 1
    got = dC.cpu().numpy()
    P64 = P.astype(np.float64)
    want = C.astype(np.float64) - P64.T @ P64
    scale = np.abs(P64).T @ np.abs(P64)
    mask = upper_tile_mask(n)
    err = np.abs(got - want)
    if tc:
        bound = 3e-3 * scale + 1e-5 * np.abs(C)
    else:
        bound = 1e-5 * (scale + np.abs(C))
    assert np.all(err[mask] <= bound[mask]), float((err / bound)[mask].max())
    # tiles strictly below the diagonal are not touched
    assert np.array_equal(got[~mask], C[~mask])
    if tc:
        # TF32 products differ from FP32 ones: the tensor-core path ran
        assert err[mask].max() > 1e-6 * scale[mask].max()


def spd(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, n))
    return X @ X.T / n + np.eye(n)


@pytest.mark.parametrize("n", [128, 640, 1100, 1001])
@pytest.mark.parametrize("tc", [True, False])
def test_potrf_f32(rsd, ctx, n, tc):
    A = spd(n, 20261204 + n)
    ctx.set_tensor_cores(tc)
    dA = colmajor(A)
    info = rsd.potrf_f32_dev(ctx, dA)
    assert info == 0
    U = np.triu(dA.cpu().numpy().astype(np.float64))
    res = np.linalg.norm(U.T @ U - A) / np.linalg.norm(A)
    assert res <= (2e-3 if tc else 1e-5), res


def test_potrf_f32_not_spd(rsd, ctx):
    n = 512
    A = spd(n, 7)
    A[300, 300] = -5.0
    ctx.set_tensor_cores(True)
    info = rsd.potrf_f32_dev(ctx, colmajor(A))
    assert info > 0
