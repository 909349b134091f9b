"""CPU oracle for the hydrodynamic step -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``
import this module; the product path never does.  It wraps the C
restatement in ``rsd_oracle.c`` (assembly, lubrication, lattice) and states
the solve chain with LAPACK DPOTRF/DPOTRI exactly as the reference calls
them (through scipy's bundled LAPACK).

Reference routines restated here (paths inside the reference project):
  src/matrices.f90      MATREV 4-34, arrangResist 218-228, averageU 230-253,
                        MobToResist_FTS 393-416, arrangement 432-445
  src/stepper.f90       STEPPER_Stokesian 33-156 (with its BROWN block
                        72-86), STEPPER_conf 160-227, STEPPER_NOGmres
                        348-410, Rheology 412-447, hydro_SD_FTS 476-546,
                        DMDX_CAL 664-688
  src/tools/gmres_mod.f90, gmres_mod_gmres.f90, algebra_lin.f90
                        gmres 48-201, simplegmres 23-61, invtrisup 72-100
  src/matrices.f90      M_Tr_front 166-190, Part_to_Whole 193-203
  src/csd_post.f90      yetamu_solve 313-367, INIT_u_bg 442-479,
                        calc_uo_bg 497-522
  src/tensors.f90       EI_transY2 / EIN_transY2 890-919
  src/mymodules.f90     dimensionless viscosity mu_f 816,846
(the overlap corrections are restated in rsd_oracle.c).

Parity status: the free-space pair tensors, the Y2 projection and MATREV are
pinned against the reference's tablefar.txt (see tests/test_oracle_pins.py);
the overlap blocks for equal spheres against the published
Rotne-Prager-Yamakawa forms (tests/test_overlap.py); the periodic Ewald sum,
the lubrication assembly and the solve chain are restated from source with
no reference outputs to pin them (parity unpinned for those parts).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "rsd_oracle.c")
LIBDIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "librsd_oracle.so")

PAI = 3.141592653589793238462643383279502884


def build(force: bool = False) -> str:
    """Compile the C restatement (plain gcc, FP contraction off so that x86
    and Arm give the same bits, like gfortran at the reference's -O0)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                           "-o", tmp, SRC, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        L.rsdo_per_grpery_inv_fri.restype = ctypes.c_int
        L.rsdo_overlap_correction_ij.restype = ctypes.c_int
        L.rsdo_lubmxcalc.restype = ctypes.c_int
        L.rsdo_lubtab_load.restype = ctypes.c_int
        L.rsdo_lubtab_sizeof.restype = ctypes.c_int
        L.rsdo_lattice_sizeof.restype = ctypes.c_int
        _ = dp
        _lib = L
    return _lib


class Lattice(ctypes.Structure):
    """LATTICE_BASE module state (src/mymodules.f90:33-42)."""
    _fields_ = [("LR", ctypes.c_double * 9), ("LI", ctypes.c_double * 9), ("LV", ctypes.c_double),
                ("lammda", ctypes.c_double), ("sig", ctypes.c_double), ("logerr", ctypes.c_double),
                ("phi", ctypes.c_double), ("NR", ctypes.c_int), ("NI", ctypes.c_int)]

    @property
    def lr(self):
        return np.array(self.LR[:]).reshape(3, 3, order="F")

    @property
    def li(self):
        return np.array(self.LI[:]).reshape(3, 3, order="F")


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def mu_f_dimensionless(mu_f_in: float = 1.0) -> float:
    """mu_f after dimentionless_calc/translate (src/mymodules.f90:816,846)."""
    lam_visc = 1.0 / PAI / mu_f_in
    return mu_f_in * lam_visc


def set_lattice_skew(T, LB, gamma, oscillation=False, gamma_alpha=0.0, frequency=0.0) -> Lattice:
    lat = Lattice()
    LB = np.ascontiguousarray(LB, dtype=np.float64)
    LV = ctypes.c_double()
    lib().rsdo_set_lattice_skew(ctypes.c_double(T), _p(LB), ctypes.c_double(gamma), ctypes.c_int(int(oscillation)),
                                ctypes.c_double(gamma_alpha), ctypes.c_double(frequency),
                                lat.LR, lat.LI, ctypes.byref(LV))
    lat.LV = LV.value
    return lat


def calc_lattice_inverse(lat: Lattice, ews_err: float, radii) -> Lattice:
    radii = np.ascontiguousarray(radii, dtype=np.float64)
    lib().rsdo_calc_lattice_inverse(ctypes.byref(lat), ctypes.c_double(ews_err), ctypes.c_int(len(radii)), _p(radii))
    return lat


def per_skew_correction(lat: Lattice, R):
    R = np.array(R, dtype=np.float64)
    d = ctypes.c_double()
    lib().rsdo_per_skew_correction(lat.LR, lat.LI, _p(R), ctypes.byref(d))
    return R, d.value


def period_correction(R, LB, T, gamma):
    R = np.array(R, dtype=np.float64)
    LB = np.ascontiguousarray(LB, dtype=np.float64)
    lib().rsdo_period_correction(_p(R), _p(LB), ctypes.c_double(T), ctypes.c_double(gamma), ctypes.c_int(0),
                                 ctypes.c_double(0.0), ctypes.c_double(0.0))
    return R


def per_rotne_prager_self(lat: Lattice, a: float):
    TTS, RRS, QQS = np.zeros(9), np.zeros(9), np.zeros(25)
    lib().rsdo_per_rotne_prager_self(ctypes.byref(lat), ctypes.c_double(a), _p(TTS), _p(RRS), _p(QQS))
    return TTS.reshape(3, 3, order="F"), RRS.reshape(3, 3, order="F"), QQS.reshape(5, 5, order="F")


def per_rotne_prager_ij(lat: Lattice, R, aI: float, aJ: float, include_k: bool = True):
    R = np.ascontiguousarray(R, dtype=np.float64)
    TT, RR, TR, QQ, G, H = (np.zeros(9), np.zeros(9), np.zeros(9), np.zeros(25), np.zeros(15), np.zeros(15))
    lib().rsdo_per_rotne_prager_ij(ctypes.byref(lat), _p(R), ctypes.c_double(aI), ctypes.c_double(aJ),
                                   ctypes.c_int(int(include_k)), _p(TT), _p(RR), _p(TR), _p(QQ), _p(G), _p(H))
    f = lambda x, s: x.reshape(s, order="F")
    return f(TT, (3, 3)), f(RR, (3, 3)), f(TR, (3, 3)), f(QQ, (5, 5)), f(G, (3, 5)), f(H, (3, 5))


def _pair_blocks(fn, *args):
    TT, RR, TR, QQ, G, H = (np.zeros(9), np.zeros(9), np.zeros(9), np.zeros(25), np.zeros(15), np.zeros(15))
    rc = fn(*args, _p(TT), _p(RR), _p(TR), _p(QQ), _p(G), _p(H))
    f = lambda x, s: x.reshape(s, order="F")
    return rc, (f(TT, (3, 3)), f(RR, (3, 3)), f(TR, (3, 3)), f(QQ, (5, 5)), f(G, (3, 5)), f(H, (3, 5)))


def yamakawa_ij(R, aI: float, aJ: float):
    """YAMAKAWA_IJ (src/GRPY_YZD.f90:768-786): the overlapping-sphere pair
    blocks TT, RR, TR (3,3), QQ_TR (5,5), GPQ_TR, HPQ_TR (3,5)."""
    R = np.ascontiguousarray(R, dtype=np.float64)
    return _pair_blocks(lib().rsdo_yamakawa_ij, _p(R), ctypes.c_double(aI), ctypes.c_double(aJ))[1]


def rotne_prager_ij_fts(R, aI: float, aJ: float):
    """ROTNE_PRAGER_IJ_FTS (src/stokesian_Green.f90:11-109): the free-space
    pair with that file's derivative chain."""
    R = np.ascontiguousarray(R, dtype=np.float64)
    return _pair_blocks(lib().rsdo_rotne_prager_ij_fts, _p(R), ctypes.c_double(aI), ctypes.c_double(aJ))[1]


def regular_rotne_prager_ij(R, aI: float, aJ: float):
    """Regular_ROTNE_PRAGER_IJ (src/Regularization.f90:18-162): the
    regularized pair blocks."""
    R = np.ascontiguousarray(R, dtype=np.float64)
    return _pair_blocks(lib().rsdo_regular_rotne_prager_ij, _p(R), ctypes.c_double(aI), ctypes.c_double(aJ))[1]


def overlap_correction_ij(method: int, R, aI: float, aJ: float):
    """overlap_*_CORRECTION_IJ (src/GRPY_YZD.f90:789-836); None for a method
    the oracle does not restate."""
    R = np.ascontiguousarray(R, dtype=np.float64)
    rc, blocks = _pair_blocks(lib().rsdo_overlap_correction_ij, ctypes.c_int(method), _p(R), ctypes.c_double(aI),
                              ctypes.c_double(aJ))
    return blocks if rc == 0 else None


def per_grpery_inv_fri(pos, radii, lat: Lattice, ews_err: float, mu_f: float, correction_method: int = 0):
    """PER_GRPERY_INV_FRI: returns (grmobmx (11N,11N) Fortran-ordered,
    n_overlap).  APP/APQ/AQQ are grmobmx[:6N,:6N], [:6N,6N:], [6N:,6N:].
    correction_method 1 (Yamakawa) or 2 (regularized) adds its correction to
    overlapping pairs; n_overlap counts the overlapping pairs of another
    nonzero method."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    radii = np.ascontiguousarray(radii, dtype=np.float64)
    N = len(radii)
    G = np.zeros((11 * N, 11 * N), order="F")
    nov = lib().rsdo_per_grpery_inv_fri(ctypes.c_int(N), _p(pos), _p(radii), ctypes.byref(lat),
                                        ctypes.c_double(ews_err), ctypes.c_double(mu_f),
                                        ctypes.c_int(correction_method), _p(G))
    return G, nov


def split_mobility(G, N):
    return G[:6 * N, :6 * N], G[:6 * N, 6 * N:], G[6 * N:, 6 * N:]


class LubTab:
    """The three lubrication tables (src/hydro_lub.f90:400-596)."""

    def __init__(self, directory: str):
        self.buf = ctypes.create_string_buffer(lib().rsdo_lubtab_sizeof())
        rc = lib().rsdo_lubtab_load(self.buf, directory.encode())
        if rc != 0:
            raise OSError("cannot read lubrication tables from %s" % directory)

    def lubcalc(self, s: float):
        o = np.zeros(19)
        lib().rsdo_lubcalc(self.buf, ctypes.c_double(s), _p(o))
        return o


def lubmxcalc(pos, radii, lat: Lattice, mu_f: float, tab: LubTab, nb: int = 0, is_period: bool = True):
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    radii = np.ascontiguousarray(radii, dtype=np.float64)
    N = len(radii)
    rfu = np.zeros((6 * N, 6 * N), order="F")
    rfe = np.zeros((6 * N, 5 * N), order="F")
    rse = np.zeros((5 * N, 5 * N), order="F")
    nc = lib().rsdo_lubmxcalc(ctypes.c_int(N), ctypes.c_int(nb), ctypes.c_int(int(is_period)), _p(pos), _p(radii),
                              lat.LR, lat.LI, ctypes.c_double(mu_f), tab.buf, _p(rfu), _p(rfe), _p(rse))
    return rfu, rfe, rse, nc


# --------------------------------------------------------------- solve chain
def matrev(A):
    """MATREV (src/matrices.f90:4-34): DPOTRF('U'), DPOTRI('U'), mirror the
    upper triangle into the lower.  Returns (inverse, info); like the
    reference, a positive DPOTRF info is reported and the chain continues."""
    from scipy.linalg import lapack
    A = np.asfortranarray(A, dtype=np.float64).copy(order="F")
    c, info = lapack.dpotrf(A, lower=0, clean=0, overwrite_a=1)
    inv, info2 = lapack.dpotri(c, lower=0, overwrite_c=1)
    iu = np.triu_indices(inv.shape[0], 1)
    inv[(iu[1], iu[0])] = inv[iu]
    return inv, int(info)


def mob_to_resist_fts(G):
    """MobToResist_FTS (src/matrices.f90:393-416) on the assembled 11N x 11N
    mobility: the full grand resistance R_inf = M^-1."""
    return matrev(G)


def ein_trans_y2(Eij, N):
    """EIN_transY2 (src/tensors.f90:905-919) with EI_transY2 890-903."""
    Y2 = np.zeros(45)
    lib().rsdo_tensor_Y2(_p(Y2))
    Y2 = Y2.reshape(5, 3, 3, order="F")
    EI = np.zeros(5)
    for m in range(5):
        a = 0.0
        for i in range(3):
            for j in range(3):
                a = a + Eij[i, j] * Y2[m, i, j]
        EI[m] = a
    return np.tile(EI, N)


def init_u_bg(gamma):
    """INIT_u_bg (src/csd_post.f90:442-479) with EI_bg = 0 on input."""
    EI_bg = np.zeros(6)
    EI_bg[4] = gamma * 0.5
    Eij = np.zeros((3, 3))
    Eij[0, 0], Eij[1, 1], Eij[2, 2] = EI_bg[0], EI_bg[1], EI_bg[2]
    Eij[0, 1] = Eij[1, 0] = EI_bg[3]
    Eij[0, 2] = Eij[2, 0] = EI_bg[4]
    Eij[1, 2] = Eij[2, 1] = EI_bg[5]
    omega_bg = np.array([0.0, gamma * 0.5, 0.0])
    eps = np.zeros((3, 3, 3))
    eps[0, 1, 2] = eps[1, 2, 0] = eps[2, 0, 1] = 1.0
    eps[0, 2, 1] = eps[2, 1, 0] = eps[1, 0, 2] = -1.0
    omegaT = np.zeros((3, 3))
    for I in range(3):
        for J in range(3):
            omegaT[I, J] = eps[J, I, 0] * omega_bg[0] + eps[J, I, 1] * omega_bg[1] + eps[J, I, 2] * omega_bg[2]
    return Eij, omega_bg, omegaT


def calc_uo_bg(pos, Eij, omega_bg, omegaT, u_bg=(0.0, 0.0, 0.0)):
    """calc_uo_bg (src/csd_post.f90:497-522)."""
    N = pos.shape[0]
    UOE = omegaT + Eij
    uo = np.zeros(6 * N)
    for i in range(N):
        uo[3 * i:3 * i + 3] = np.asarray(u_bg) + UOE @ pos[i]
        uo[3 * N + 3 * i:3 * N + 3 * i + 3] = omega_bg
    return uo


def stepper_nogmres(G, rfu, rfe, rse, Fe, EIN, Fe_inter, conf, u_brown=None):
    """STEPPER_NOGmres (src/stepper.f90:348-410) for the FTS periodic path,
    with arrangement (src/matrices.f90:432-445) and Rheology
    (src/stepper.f90:412-447).  Returns U_par, SijN_hyd, SijN_FP, SijN_B and
    RPP as the caller sees it afterwards (overwritten by its inverse inside
    Rheology), plus the MATREV infos."""
    N = conf.shape[0]
    R0, info_m = mob_to_resist_fts(G)
    RPP = R0[:6 * N, :6 * N] + rfu
    RPQ = R0[:6 * N, 6 * N:] + rfe
    RQQ = R0[6 * N:, 6 * N:] + rse
    UB = np.zeros(6 * N)
    if u_brown is not None:
        UB[:3 * N] = u_brown
    APPR, info_r = matrev(RPP)
    U_par = APPR @ (Fe + RPQ @ EIN)
    RPPINV, _ = matrev(RPP)
    mu = (RPQ.T @ RPPINV) @ RPQ - RQQ
    SijN_hyd = mu @ EIN
    RPP_inv, _ = matrev(RPP)
    SijN_FP = (RPQ.T @ RPP_inv) @ Fe_inter
    Y2 = np.zeros(45)
    lib().rsdo_tensor_Y2(_p(Y2))
    Y2 = Y2.reshape(5, 3, 3, order="F")
    for kk in range(N):
        Sij = np.zeros((3, 3))
        for i in range(3):
            for j in range(3):
                Sij[i, j] = 0.5 * (conf[kk, i] * Fe_inter[3 * kk + j] + conf[kk, j] * Fe_inter[3 * kk + i])
        part = np.array([sum(Sij[a, b] * Y2[m, a, b] for a in range(3) for b in range(3)) for m in range(5)])
        SijN_FP[5 * kk:5 * kk + 5] += part
    SijN_B = RPQ.T @ UB
    return dict(U_par=U_par, SijN_hyd=SijN_hyd, SijN_FP=SijN_FP, SijN_B=SijN_B, RPP=RPP_inv,
                info_m=info_m, info_r=info_r, RPQ=RPQ, RQQ=RQQ)


# deta of DMDX_CAL: PARAMETER(deta=0.001) gives the REAL*8 the value of the
# default-real (single precision) literal
DMDX_DETA = float(np.float32(0.001))


def dmdx_cal(conf, radii, lattice_fn, ews_err, mu_f, Z, correction_method=0):
    """DMDX_CAL (src/stepper.f90:664-688): DMDX = (A1 - A2) Z / deta with A1,
    A2 the translational blocks APP(1:3N,1:3N) of PER_GRPERY_INV_FRI at
    CONF +- deta Z / 2.  lattice_fn() returns a fresh lattice (the routine
    fills it)."""
    conf = np.asarray(conf, dtype=np.float64)
    Z = np.asarray(Z, dtype=np.float64)
    N = conf.shape[0]
    Zc = Z.reshape(N, 3)
    G1, _ = per_grpery_inv_fri(conf + 0.5 * DMDX_DETA * Zc, radii, lattice_fn(), ews_err, mu_f, correction_method)
    G2, _ = per_grpery_inv_fri(conf - 0.5 * DMDX_DETA * Zc, radii, lattice_fn(), ews_err, mu_f, correction_method)
    A1, A2 = G1[:3 * N, :3 * N], G2[:3 * N, :3 * N]
    return ((A1 - A2) @ Z) / DMDX_DETA


def brownian_velocity(APP, conf, radii, lattice_fn, ews_err, mu_f, Z, kBT, dt, correction_method=0):
    """u_brown of STEPPER_Stokesian with BROWN (src/stepper.f90:72-86):
    CHOLESKY (DPOTRF 'L', src/matrices.f90:126-157) of APP(1:3N,1:3N),
    VB = sqrt(2 kBT) L Z / DT, u_brown = VB + kBT DMDX_CAL."""
    from scipy.linalg import lapack
    N = np.asarray(conf).shape[0]
    A = np.asfortranarray(APP[:3 * N, :3 * N], dtype=np.float64).copy(order="F")
    L, info = lapack.dpotrf(A, lower=1, clean=1)
    if info:
        return None, int(info)
    VB = np.sqrt(2.0 * kBT) * (L @ Z) / dt
    return VB + kBT * dmdx_cal(conf, radii, lattice_fn, ews_err, mu_f, Z, correction_method), 0


def _grotmat(a, b, real_tol=1e-14):
    """grotmat (src/tools/gmres_mod.f90:178-201): Givens rotation."""
    if abs(b) < real_tol:
        return 1.0, 0.0
    if abs(b) > abs(a):
        t = a / b
        sn = 1.0 / np.sqrt(1.0 + t * t)
        return t * sn, sn
    t = b / a
    cs = 1.0 / np.sqrt(1.0 + t * t)
    return cs, t * cs


def _invtrisup(M, vec):
    """invtrisup (src/tools/algebra_lin.f90:72-100): upper triangular solve."""
    n = len(vec)
    res = np.zeros(n)
    res[n - 1] = vec[n - 1] / M[n - 1, n - 1]
    for ii in range(n - 2, -1, -1):
        res[ii] = vec[ii]
        for ji in range(ii + 1, n):
            res[ii] = res[ii] - M[ii, ji] * res[ji]
        res[ii] = res[ii] / M[ii, ii]
    return res


def gmres(x, b, A, tol, itmax, rst):
    """gmres (src/tools/gmres_mod.f90:48-175): restarted GMRES(rst) with
    Givens rotations, relative residual tol; returns (x, iter, res) with
    iter = -1 when not converged.  A is a dense matrix (matVecProd)."""
    x = np.array(x, dtype=np.float64)
    n = len(x)
    nb2 = np.sqrt(b @ b)
    if nb2 / n < 1e-8:
        nb2 = np.sqrt(n)
    nb2 = 1.0 / nb2
    r = b - A @ x
    nr2 = np.sqrt(r @ r)
    res = nr2 * nb2
    if res < tol:
        return x, 0, res
    V = np.zeros((rst + 1, n))
    H = np.zeros((rst + 1, rst))
    cs, sn = np.zeros(rst), np.zeros(rst)
    for it in range(1, itmax + 1):
        s = np.zeros(rst + 1)
        s[0] = nr2
        V[0] = r / nr2
        for ii in range(rst):
            w = A @ V[ii]
            for kk in range(ii + 1):
                H[kk, ii] = w @ V[kk]
                w = w - H[kk, ii] * V[kk]
            H[ii + 1, ii] = np.sqrt(w @ w)
            with np.errstate(divide="ignore", invalid="ignore"):  # as the Fortran: no breakdown test
                V[ii + 1] = w / H[ii + 1, ii]
            for kk in range(ii):
                t = cs[kk] * H[kk, ii] + sn[kk] * H[kk + 1, ii]
                H[kk + 1, ii] = -sn[kk] * H[kk, ii] + cs[kk] * H[kk + 1, ii]
                H[kk, ii] = t
            cs[ii], sn[ii] = _grotmat(H[ii, ii], H[ii + 1, ii])
            t = cs[ii] * s[ii]
            s[ii + 1] = -sn[ii] * s[ii]
            s[ii] = t
            H[ii, ii] = cs[ii] * H[ii, ii] + sn[ii] * H[ii + 1, ii]
            H[ii + 1, ii] = 0.0
            res = abs(s[ii + 1]) * nb2
            if res < tol:
                y = _invtrisup(H[:ii + 1, :ii + 1], s[:ii + 1])
                for kk in range(ii + 1):
                    x = x + V[kk] * y[kk]
                return x, it, res
        y = _invtrisup(H[:rst, :rst], s[:rst])
        for kk in range(rst):
            x = x + V[kk] * y[kk]
        r = b - A @ x
        nr2 = np.sqrt(r @ r)
        res = nr2 * nb2
        if res < tol:
            return x, it, res
    return x, -1, res


def _m_tr_front(APP, APQ, AQQ):
    """M_Tr_front (src/matrices.f90:166-190): (A_Tr_front, A_Tr_back)."""
    n6, n5 = APP.shape[0], AQQ.shape[0]
    F = np.zeros((n6 + n5, n6 + n5))
    B = np.zeros((n6 + n5, n6 + n5))
    F[:n6, :n6] = np.eye(n6)
    F[:n6, n6:] = -APQ
    F[n6:, n6:] = -AQQ
    B[n6:, n6:] = -np.eye(n5)
    B[:n6, :n6] = APP
    B[n6:, :n6] = APQ.T
    return F, B


def _part_to_whole(APP, APQ, AQQ):
    """Part_to_Whole (src/matrices.f90:193-203)."""
    return np.block([[APP, APQ], [APQ.T, AQQ]])


def hydro_sd_fts(APP, APQ, AQQ, rfu, rfe, rse, Fe, EIN, linerr=1e-10, trace=None):
    """hydro_SD_FTS (src/stepper.f90:476-546) with simplegmres
    (src/tools/gmres_mod_gmres.f90:23-61: GMRES(2), tol = 100 REAL_TOL =
    1e-12, 200 cycles): up to 50 alternations of a mobility solve and a
    lubrication solve until the FTS residual norm is below linerr 1e-2.
    Returns U_Par and SijN as the reference leaves them (SijN None when the
    loop ends unconverged: the reference does not assign it), the outer
    iteration count (-1 unconverged) and the last residual norm; trace, if
    a list, receives every residual norm."""
    n6 = APP.shape[0]
    n = n6 + AQQ.shape[0]
    A = _part_to_whole(APP, APQ, AQQ)
    gL, gR = _m_tr_front(APP, APQ, AQQ)
    RlubM = _part_to_whole(rfu, rfe, rse) @ A + np.eye(n)
    # Whole_to_Part keeps the upper-right block; M_Tr_front uses its transpose
    RL, RR = _m_tr_front(RlubM[:n6, :n6], RlubM[:n6, n6:], RlubM[n6:, n6:])
    Fff = np.array(Fe, dtype=np.float64)
    F1 = np.zeros(n)
    F2 = np.zeros(n)
    F1[n6:] = -EIN
    F2[:n6] = Fe
    err = np.inf
    U_Par = None
    for i in range(1, 51):
        F1[:n6] = Fff
        U1, _, _ = gmres(np.zeros(n), gR @ F1, gL, 1e-12, 200, 2)
        F2[n6:] = U1[n6:]
        U2, _, _ = gmres(U1.copy(), RL @ F2, RR, 1e-12, 200, 2)
        Fff = U2[:n6]
        U_Par = U1[:n6]
        Sff = U1[n6:]
        ev = np.concatenate([Fff + rfu @ U_Par + rfe @ (-EIN), APQ.T @ Fff + AQQ @ Sff])
        err = np.linalg.norm(np.concatenate([Fe, -EIN]) - ev)
        if trace is not None:
            trace.append(err)
        if err < linerr * 1e-2:
            return dict(U_Par=APP @ Fff + APQ @ (-EIN), SijN=U2[n6:], iters=i, err=err)
    return dict(U_Par=U_Par, SijN=None, iters=-1, err=err)


def average_u(APP, N, mu_f, radii_test=1.0):
    """averageU (src/matrices.f90:230-253)."""
    F = np.zeros(6 * N)
    F[0:3 * N:3] = 1.0 * (6.0 * PAI * mu_f * radii_test)
    UU = APP @ F
    return UU[0:3 * N:3].sum() / N


def yetamu_solve(APP, SijN_hyd, SijN_FP, SijN_B, EIN, LV, mu_f, phi, N):
    """yetamu_solve (src/csd_post.f90:313-367), non-GMRES build."""
    y = np.zeros(5)
    d = -2.0 * EIN[3::5]
    y[0] = ((SijN_FP[3::5] + SijN_hyd[3::5] + SijN_B[3::5]) / d).sum() / LV / mu_f
    y[1] = phi
    y[2] = 1.0 / average_u(APP, N, mu_f)
    y[3] = (SijN_B[3::5] / d).sum() / LV / mu_f
    y[4] = (SijN_FP[3::5] / d).sum() / LV / mu_f
    return y


def stepper_stokesian(conf, radii, LB, T, dt, gamma, mu_f, ews_err, tab: LubTab, Fe=None, Fe_inter=None,
                      correction_method=0):
    """One STEPPER_Stokesian step (src/stepper.f90:33-156) on the plain
    LAPACK FTS periodic path with lubrication (no Brownian motion, no DEM
    sub-stepping, no rigid bodies), with the module's correction_method
    passed to PER_GRPERY_INV_FRI.  Returns the updated configuration and
    everything the reference computes on the way."""
    conf = np.array(conf, dtype=np.float64)
    N = conf.shape[0]
    Eij, omega_bg, omegaT = init_u_bg(gamma)
    EIN = ein_trans_y2(Eij, N)
    lat = set_lattice_skew(T, LB, gamma)
    G, _ = per_grpery_inv_fri(conf, radii, lat, ews_err, mu_f, correction_method)
    Fe = np.zeros(6 * N) if Fe is None else np.asarray(Fe, dtype=np.float64)
    Fe_inter = np.zeros(6 * N) if Fe_inter is None else np.asarray(Fe_inter, dtype=np.float64)
    rfu, rfe, rse, ncontact = lubmxcalc(conf, radii, lat, mu_f, tab)
    out = stepper_nogmres(G, rfu, rfe, rse, Fe + Fe_inter, EIN, Fe_inter, conf)
    U_rel = out["U_par"]
    # STEPPER_conf (src/stepper.f90:160-227)
    uo = calc_uo_bg(conf, Eij, omega_bg, omegaT)
    U_pos = U_rel + uo
    new = conf + dt * U_pos[:3 * N].reshape(N, 3)
    for i in range(N):
        new[i] = period_correction(new[i], LB, T, gamma)
    uo = calc_uo_bg(new, Eij, omega_bg, omegaT)
    U_pos = U_rel + uo
    APP = G[:6 * N, :6 * N]
    yeta = yetamu_solve(APP, out["SijN_hyd"], out["SijN_FP"], out["SijN_B"], EIN, lat.LV, mu_f, lat.phi, N)
    out.update(conf=new, U_pos=U_pos, yeta_mu=yeta, EIN=EIN, lattice=lat, G=G, rfu=rfu, rfe=rfe, rse=rse,
               ncontact=ncontact)
    return out


def box_length(N, phi, a=1.0):
    """Cubic box edge for N spheres of radius a at volume fraction phi."""
    return (N * 4.0 / 3.0 * math.pi * a ** 3 / phi) ** (1.0 / 3.0)
