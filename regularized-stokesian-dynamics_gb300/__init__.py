"""GB300 (sm_103a) hydrodynamic step of regularized Stokesian dynamics.

Host-side mirror of the Fortran reference's interface for the hot path
(sherlockyzd/Regularized-Stokesian-Dynamics): the same subroutine names,
argument meanings and error behaviour, over the C-ABI in include/rsd_capi.h.
Arrays follow the Fortran layout: positions are (N, 3) C-ordered (= p_pos(3,N)
column-major), matrices are returned Fortran-ordered.

Everything computes on the GPU through librsd_gb300.so; importing this
package without the built library raises ImportError (there is no CPU path).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "librsd_gb300.so")

RSD_OK, RSD_EARG, RSD_ECUDA, RSD_ENAN, RSD_ETIMEOUT, RSD_ENOMEM, RSD_EIO, RSD_EUNSUP = 0, -1, -2, -3, -4, -5, -6, -7
RSD_ELIMIT = -8
RSD_ENOCONV = -9
PREC_FP64, PREC_MIXED = 0, 1
PC_NONE, PC_JACOBI, PC_BLOCK_JACOBI, PC_FSAI, PC_LEARNED = 0, 1, 2, 3, 4
PAI = 3.141592653589793238462643383279502884

if not os.path.exists(LIBPATH):
    raise ImportError("librsd_gb300.so is not built (run regularized-stokesian-dynamics_gb300/build.py); "
                      "this package has no CPU fallback")

_lib = ctypes.CDLL(LIBPATH)
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_vp = ctypes.c_void_p


class Lattice(ctypes.Structure):
    """rsd_lattice: module LATTICE_BASE (src/mymodules.f90:33-42)."""
    _fields_ = [("LR", ctypes.c_double * 9), ("LI", ctypes.c_double * 9), ("LV", ctypes.c_double),
                ("lammda", ctypes.c_double), ("sig", ctypes.c_double), ("logerr", ctypes.c_double),
                ("phi", ctypes.c_double), ("NR", ctypes.c_int32), ("NI", ctypes.c_int32)]


class StepParams(ctypes.Structure):
    _fields_ = [("nn", ctypes.c_int32), ("nb", ctypes.c_int32), ("LB", ctypes.c_double * 3), ("T", ctypes.c_double),
                ("dt", ctypes.c_double), ("gamma", ctypes.c_double), ("mu_f", ctypes.c_double),
                ("ews_err", ctypes.c_double), ("use_lub", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("tol", ctypes.c_double), ("max_iter", ctypes.c_int32)]


class StepInfo(ctypes.Structure):
    _fields_ = [("info", ctypes.c_int32), ("n_contact", ctypes.c_int32), ("NR", ctypes.c_int32),
                ("NI", ctypes.c_int32), ("iterations", ctypes.c_int32), ("residual", ctypes.c_double),
                ("phi", ctypes.c_double), ("LV", ctypes.c_double), ("rpp_iterations", ctypes.c_int32),
                ("fallback", ctypes.c_int32)]


def _sig(name, res, args):
    f = getattr(_lib, name)
    f.restype = res
    f.argtypes = args
    return f


_i = ctypes.c_int
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_d = ctypes.c_double
_LP = ctypes.POINTER(Lattice)
_sig("rsd_ctx_create", _i, [ctypes.POINTER(_vp), _i])
_sig("rsd_ctx_destroy", _i, [_vp])
_sig("rsd_ctx_last_error", ctypes.c_char_p, [_vp])
_sig("rsd_ctx_stream", _vp, [_vp])
_sig("rsd_ctx_phase_ms", _i, [_vp, _dp])
_sig("rsd_launch_count", ctypes.c_longlong, [])
_sig("rsd_set_lattice_skew", _i, [_d, _dp, _d, _i32, _d, _d, _LP])
_sig("rsd_calc_lattice_inverse", _i, [_LP, _d, _i32, _dp])
_sig("rsd_per_grpery_inv_fri", _i, [_vp, _i32, _dp, _dp, _LP, _d, _d, _i32, _dp, _dp, _dp])
_sig("rsd_per_grpery_inv_fri_dev", _i, [_vp, _i32, _vp, _vp, _LP, _d, _d, _i32, _vp, _i64])
_sig("rsd_per_grpery_inv_fri_static", _i, [_i32, _vp, _vp, _LP, _d, _d, _vp, _i64, _vp])
_sig("rsd_lubtab_load", _i, [ctypes.POINTER(_vp), ctypes.c_char_p])
_sig("rsd_lubtab_create", _i, [ctypes.POINTER(_vp), _i32, _dp, _i32, _dp, _i32, _dp])
_sig("rsd_lubtab_destroy", _i, [_vp])
_sig("rsd_lubmxcalc", _i, [_vp, _vp, _i32, _i32, _i32, _dp, _dp, _LP, _d, _dp, _dp, _dp, _ip])
_sig("rsd_lubmxcalc_dev", _i, [_vp, _vp, _i32, _i32, _i32, _vp, _vp, _LP, _d, _vp, _i64, _i32, _ip])
_sig("rsd_matrev", _i, [_vp, _i32, _dp, _ip])
_sig("rsd_matrev_dev", _i, [_vp, _i32, _vp, _i64, _ip])
_sig("rsd_cholesky", _i, [_vp, _i32, _dp, _ip])
_sig("rsd_mob_to_resist_fts", _i, [_vp, _i32, _dp, _dp, _dp, _dp, _dp, _dp, _ip])
_sig("rsd_arrangement", _i, [_vp, _i32, _dp, _dp, _dp, _dp, _ip])
_sig("rsd_stepper_nogmres", _i, [_vp, _i32] + [_dp] * 11 + [_dp] * 5 + [_ip])
_sig("rsd_hydro_sd_fts", _i, [_vp, _i32] + [_dp] * 8 + [_dp] * 2 + [_ip])
_sig("rsd_dmdx_cal", _i, [_vp, _i32, _dp, _dp, _vp, _d, _d, _i32, _dp, _dp])
_sig("rsd_brownian_velocity", _i, [_vp, _i32, _dp, _dp, _dp, _vp, _d, _d, _i32, _dp, _d, _d, _dp, _ip])
_sig("rsd_stepper_stokesian", _i, [_vp, _vp, ctypes.POINTER(StepParams), _dp, _dp, _dp, _dp, _dp, _dp,
                                   ctypes.POINTER(StepInfo)])
_sig("rsd_stepper_stokesian_dev", _i, [_vp, _vp, ctypes.POINTER(StepParams), _vp, _vp, _vp, _vp, _vp, _dp,
                                       ctypes.POINTER(StepInfo)])
_sig("rsd_ctx_set_tensor_cores", _i, [_vp, _i])
_sig("rsd_ctx_set_mixed_split", _i, [_vp, _d, _i32])
_sig("rsd_ctx_set_mixed_truncation", _i, [_vp, _d, _d])
_sig("rsd_ctx_set_mixed_lambda_scale", _i, [_vp, _d])
_sig("rsd_ctx_set_mixed_real_passes", _i, [_vp, _i32])
_sig("rsd_ctx_set_correction_method", _i, [_vp, _i32])
_sig("rsd_ctx_set_wait_limits", _i, [_vp, _i64, _i64])
_sig("rsd_ctx_set_factor_schedule", _i, [_vp, _i32])
_sig("rsd_ctx_set_refinement", _i, [_vp, _i32, _i32])
_sig("rsd_ctx_set_rpp_solver", _i, [_vp, _i32, _vp, _d, _i32])
_sig("rsd_lp_param_count", ctypes.c_int64, [])
_sig("rsd_lp_create", _i, [ctypes.POINTER(_vp), _i, _vp, ctypes.c_uint64])
_sig("rsd_lp_destroy", _i, [_vp])
_sig("rsd_lp_get_params", _i, [_vp, _vp, _vp])
_sig("rsd_lp_graph_dev", _i, [_vp, _i32, _vp, _vp, _LP, ctypes.POINTER(_i32), _vp, _vp, _vp])
_sig("rsd_lp_forward_dev", _i, [_vp, _vp, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp])
_sig("rsd_lp_adam_step", _i, [_vp, ctypes.c_float])
_sig("rsd_lp_set_training", _i, [_vp, ctypes.c_float, ctypes.c_double])
_sig("rsd_lp_training_stats", _i, [_vp, _dp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)])
_sig("rsd_lp_train_step", _i, [_vp, _vp, _i32, _vp, _vp, _LP, _i32, _vp, _i64, ctypes.c_float, _dp])
_sig("rsd_lp_blocks_dev", _i, [_vp, _vp, _i32, _i32, _vp, _vp, _LP, _i32, _vp, _i64, _vp, _vp,
                               ctypes.POINTER(_i32)])
_sig("rsd_lp_pcg_dev", _i, [_vp, _vp, _i32, _i32, _vp, _vp, _LP, _vp, _i64, _i32, _vp, _vp, _d, _i32,
                            ctypes.POINTER(_i32), _dp])
_sig("rsd_resistance_pp_dev", _i, [_vp, _vp, ctypes.POINTER(StepParams), _vp, _vp, _vp, _i64, _LP])
_sig("rsd_syrk_f32_dev", _i, [_vp, _i32, _i32, _vp, _i64, _vp, _i64, _i32])
_sig("rsd_potrf_f32_dev", _i, [_vp, _i32, _vp, _i64, _i32, _ip])
_sig("rsd_potri_f32_dev", _i, [_vp, _i32, _vp, _i64, _i32])

EXPORTED = [n for n in dir(_lib) if n.startswith("rsd_")]


def library():
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def _f64(a, shape=None, order="C"):
    a = np.require(np.asarray(a, dtype=np.float64), requirements=[order, "A", "W", "O"])
    if shape is not None and a.shape != shape:
        a = a.reshape(shape, order=order)
    return a


class RSDError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("rsd error %d: %s" % (code, msg))
        self.code = code


class Context:
    """rsd_ctx on one CUDA device: one stream, grow-only device buffers."""

    def __init__(self, device: int = 0):
        self.h = _vp()
        rc = _lib.rsd_ctx_create(ctypes.byref(self.h), device)
        if rc != 0:
            raise RSDError(rc, "cannot create a context on CUDA device %d" % device)
        self.device = device

    def check(self, rc):
        if rc < 0:
            raise RSDError(rc, (_lib.rsd_ctx_last_error(self.h) or b"").decode())
        return rc

    def phase_ms(self):
        ms = np.zeros(4)
        _lib.rsd_ctx_phase_ms(self.h, _p(ms))
        return ms

    @property
    def stream(self):
        return _lib.rsd_ctx_stream(self.h)

    def set_mixed_split(self, lam_r_cut=4.5, kshell=1):
        """FP64/FP32 split of the mixed-precision Ewald assembly."""
        self.check(_lib.rsd_ctx_set_mixed_split(self.h, float(lam_r_cut), int(kshell)))

    def set_mixed_truncation(self, lam_r_max=6.0, k2_over_4lam2_max=10.0 * np.pi):
        """Truncation of the mixed-precision Ewald sums."""
        self.check(_lib.rsd_ctx_set_mixed_truncation(self.h, float(lam_r_max), float(k2_over_4lam2_max)))

    def set_mixed_lambda_scale(self, scale=1.75):
        """Ewald splitting parameter of the mixed assembly relative to the
        reference's."""
        self.check(_lib.rsd_ctx_set_mixed_lambda_scale(self.h, float(scale)))

    def set_mixed_real_passes(self, passes=1):
        """Passes over the near images of the equal-radius mixed assembly."""
        self.check(_lib.rsd_ctx_set_mixed_real_passes(self.h, int(passes)))

    def set_correction_method(self, method=0):
        """Overlap corrections in the fused step (correction_method of
        per_GRPY_YZD.f90:98-116: 0 none, 1 Yamakawa, 2 regularized)."""
        self.check(_lib.rsd_ctx_set_correction_method(self.h, int(method)))

    def set_wait_limits(self, tc_wait_ns=0, tri_spin_polls=0):
        """Bounds of the mixed form's device-side waits (0: the defaults,
        0.5 s and 2^21 polls); a wait that gives up makes the call return
        RSD_ETIMEOUT."""
        self.check(_lib.rsd_ctx_set_wait_limits(self.h, int(tc_wait_ns), int(tri_spin_polls)))

    def set_factor_schedule(self, schedule=1):
        """Mixed form's FP32 Cholesky schedule: 1 look-ahead on the chain of
        diagonal blocks (default), 0 in-order panel steps."""
        self.check(_lib.rsd_ctx_set_factor_schedule(self.h, int(schedule)))

    def set_refinement(self, mode=0, restart=30):
        """Mixed form's refinement: 0 the stationary iteration (default), 1
        flexible GMRES."""
        self.check(_lib.rsd_ctx_set_refinement(self.h, int(mode), int(restart)))

    def set_rpp_solver(self, mode=0, net=None, tol=0.0, maxit=0):
        """RPP solve of the plain FP64 step: PC_NONE keeps the Cholesky
        factorisation; PC_JACOBI, PC_BLOCK_JACOBI, PC_FSAI or PC_LEARNED
        (with a LearnedPreconditioner) use PCG, the factorisation its
        fallback."""
        self._rpp_net = net  # keep the network alive while the context uses it
        self.check(_lib.rsd_ctx_set_rpp_solver(self.h, int(mode), net.h if net is not None else None, float(tol),
                                               int(maxit)))

    def set_tensor_cores(self, mode=1):
        """FP32 factorisations of the mixed form: 1 (or True, the default)
        tcgen05 TF32/3xTF32 per factor, 3 all 3xTF32, 0 (or False) SIMT."""
        mode = int(mode)
        self.check(_lib.rsd_ctx_set_tensor_cores(self.h, mode))

    def close(self):
        if self.h:
            _lib.rsd_ctx_destroy(self.h)
            self.h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LubTab:
    """The three lubrication tables (hydro_lub.f90:529-596), read from a
    directory holding r2babc.dat, r2bgh.dat and r2bm.dat."""

    def __init__(self, directory: str):
        self.h = _vp()
        rc = _lib.rsd_lubtab_load(ctypes.byref(self.h), directory.encode())
        if rc != 0:
            raise RSDError(rc, "cannot read lubrication tables from %s" % directory)

    def __del__(self):
        if getattr(self, "h", None):
            _lib.rsd_lubtab_destroy(self.h)
            self.h = _vp()


# ------------------------------------------------------------------ lattice
def SET_LATTICE_SKEW(T, LB, gamma, oscillation=False, gamma_alpha=0.0, frequency=0.0) -> Lattice:
    """SET_LATTICE_SKEW (src/csd_post.f90:105-136)."""
    lat = Lattice()
    LB = _f64(LB)
    rc = _lib.rsd_set_lattice_skew(T, _p(LB), gamma, int(oscillation), gamma_alpha, frequency, ctypes.byref(lat))
    if rc:
        raise RSDError(rc, "SET_LATTICE_SKEW")
    return lat


def CALC_LATTICE_INVERSE(lat: Lattice, ews_err, radii) -> Lattice:
    """CALC_LATTICE_INVERSE (src/csd_post.f90:158-183)."""
    r = _f64(radii)
    rc = _lib.rsd_calc_lattice_inverse(ctypes.byref(lat), ews_err, len(r), _p(r))
    if rc:
        raise RSDError(rc, "CALC_LATTICE_INVERSE")
    return lat


# ------------------------------------------------------------------ kernel 1
def PER_GRPERY_INV_FRI(ctx: Context, p_pos, radii, lattice: Lattice, ews_err, mu_f, correction_method=0):
    """PER_GRPERY_INV_FRI (src/per_GRPY_YZD.f90:13-200): APP, APQ, AQQ."""
    pos = _f64(p_pos)
    r = _f64(radii)
    N = len(r)
    APP = np.empty((6 * N, 6 * N), order="F")
    APQ = np.empty((6 * N, 5 * N), order="F")
    AQQ = np.empty((5 * N, 5 * N), order="F")
    ctx.check(_lib.rsd_per_grpery_inv_fri(ctx.h, N, _p(pos), _p(r), ctypes.byref(lattice), ews_err, mu_f,
                                          correction_method, _p(APP), _p(APQ), _p(AQQ)))
    return APP, APQ, AQQ


def per_grpery_inv_fri_dev(ctx: Context, pos, radii, lattice: Lattice, ews_err, mu_f, out=None, correction_method=0):
    """Device variant on torch CUDA tensors; returns the whole grmobmx as an
    (11N, 11N) tensor whose memory is column-major (returned as a transpose
    view, so indexing [i, j] is the Fortran element (i, j))."""
    import torch
    N = radii.shape[0]
    n = 11 * N
    buf = out if out is not None else torch.empty((n, n), dtype=torch.float64, device=pos.device)
    torch.cuda.synchronize(pos.device)
    ctx.check(_lib.rsd_per_grpery_inv_fri_dev(ctx.h, N, pos.data_ptr(), radii.data_ptr(), ctypes.byref(lattice),
                                              ews_err, mu_f, correction_method, buf.data_ptr(), n))
    _sync_ctx(ctx)
    return buf.t()


def syrk_f32_dev(ctx: Context, P, C, prec=1):
    """C -= P^T P on the 128 x 128 tiles on and above the diagonal.  P (k, n)
    and C (n, n) are column-major FP32 device matrices passed as the
    transpose views of contiguous torch tensors (P.t() of an (n, k) tensor).
    prec: 0 FP32 SIMT, 1 TF32 tensor cores, 3 3xTF32 tensor cores."""
    import torch
    k, n = P.shape
    assert C.shape == (n, n) and P.stride(0) == 1 and C.stride(0) == 1
    torch.cuda.synchronize(P.device)
    ctx.check(_lib.rsd_syrk_f32_dev(ctx.h, n, k, P.data_ptr(), P.stride(1), C.data_ptr(), C.stride(1), prec))
    return C


def potrf_f32_dev(ctx: Context, A, prec=1):
    """Upper Cholesky factor in place of a column-major FP32 device matrix
    (a transpose view, as syrk_f32_dev); returns info."""
    import torch
    n = A.shape[0]
    assert A.shape == (n, n) and A.stride(0) == 1
    info = ctypes.c_int32(0)
    torch.cuda.synchronize(A.device)
    ctx.check(_lib.rsd_potrf_f32_dev(ctx.h, n, A.data_ptr(), A.stride(1), prec, ctypes.byref(info)))
    return info.value


def potri_f32_dev(ctx: Context, A, prec=3):
    """A <- A^-1 (upper triangle) from the upper factor in A (DPOTRI)."""
    import torch
    n = A.shape[0]
    assert A.shape == (n, n) and A.stride(0) == 1
    torch.cuda.synchronize(A.device)
    ctx.check(_lib.rsd_potri_f32_dev(ctx.h, n, A.data_ptr(), A.stride(1), prec))
    return A


def _sync_ctx(ctx):
    import torch
    s = torch.cuda.ExternalStream(ctx.stream) if hasattr(torch.cuda, "ExternalStream") else None
    if s is not None:
        s.synchronize()
    else:
        torch.cuda.synchronize()


# ------------------------------------------------------------------ kernel 2
def lubmxcalc(ctx: Context, tab: LubTab, p_pos, radii, lattice: Lattice, mu_f, nb=0, is_period=True):
    """lubmxcalc (src/hydro_lub.f90:22-308): rfu, rfe, rse and the number
    of pairs found at s <= 2 (mirrored, like the reference)."""
    pos = _f64(p_pos)
    r = _f64(radii)
    N = len(r)
    rfu = np.empty((6 * N, 6 * N), order="F")
    rfe = np.empty((6 * N, 5 * N), order="F")
    rse = np.empty((5 * N, 5 * N), order="F")
    nc = ctypes.c_int32(0)
    ctx.check(_lib.rsd_lubmxcalc(ctx.h, tab.h, N, nb, int(is_period), _p(pos), _p(r),
                                 ctypes.byref(lattice) if lattice is not None else None, mu_f, _p(rfu), _p(rfe),
                                 _p(rse), ctypes.byref(nc)))
    return rfu, rfe, rse, nc.value


# ------------------------------------------------------------------ kernel 3
def MATREV(ctx: Context, A):
    """MATREV (src/matrices.f90:4-34): SPD inverse; returns (A^-1, info)."""
    A = np.array(A, dtype=np.float64, order="F", copy=True)
    info = ctypes.c_int32(0)
    ctx.check(_lib.rsd_matrev(ctx.h, A.shape[0], _p(A), ctypes.byref(info)))
    return A, info.value


def CHOLESKY(ctx: Context, B):
    """CHOLESKY (src/matrices.f90:126-157): lower factor, strict upper zero.
    Raises when B is not positive definite (the reference STOPs)."""
    B = np.array(B, dtype=np.float64, order="F", copy=True)
    info = ctypes.c_int32(0)
    rc = ctx.check(_lib.rsd_cholesky(ctx.h, B.shape[0], _p(B), ctypes.byref(info)))
    if rc > 0:
        raise RSDError(rc, "CHOLESKY: leading minor %d is not positive definite" % rc)
    return B


def MobToResist_FTS(ctx: Context, APP, APQ, AQQ):
    """MobToResist_FTS (src/matrices.f90:393-416)."""
    N = APP.shape[0] // 6
    APP, APQ, AQQ = (np.asfortranarray(x, dtype=np.float64) for x in (APP, APQ, AQQ))
    RPP = np.empty((6 * N, 6 * N), order="F")
    RPQ = np.empty((6 * N, 5 * N), order="F")
    RQQ = np.empty((5 * N, 5 * N), order="F")
    info = ctypes.c_int32(0)
    ctx.check(_lib.rsd_mob_to_resist_fts(ctx.h, N, _p(APP), _p(APQ), _p(AQQ), _p(RPP), _p(RPQ), _p(RQQ),
                                         ctypes.byref(info)))
    return RPP, RPQ, RQQ, info.value


def arrangement(ctx: Context, RPP, RPQ, RQQ):
    """arrangement (src/matrices.f90:432-445): mu = RPQ^T RPP^-1 RPQ - RQQ."""
    N = RPP.shape[0] // 6
    RPP, RPQ, RQQ = (np.asfortranarray(x, dtype=np.float64) for x in (RPP, RPQ, RQQ))
    mu = np.empty((5 * N, 5 * N), order="F")
    info = ctypes.c_int32(0)
    ctx.check(_lib.rsd_arrangement(ctx.h, N, _p(RPP), _p(RPQ), _p(RQQ), _p(mu), ctypes.byref(info)))
    return mu, info.value


def STEPPER_NOGmres(ctx: Context, APP, APQ, AQQ, rfu, rfe, rse, Fe, EIN, Fe_inter, conf, u_brown=None):
    """STEPPER_NOGmres (src/stepper.f90:348-410), FTS path."""
    N = APP.shape[0] // 6
    mats = [np.asfortranarray(x, dtype=np.float64) for x in (APP, APQ, AQQ, rfu, rfe, rse)]
    Fe, EIN, Fe_inter = _f64(Fe), _f64(EIN), _f64(Fe_inter)
    conf = _f64(conf)
    ub = _f64(u_brown) if u_brown is not None else None
    U_par = np.empty(6 * N)
    Sh, Sfp, Sb = np.empty(5 * N), np.empty(5 * N), np.empty(5 * N)
    RPP = np.empty((6 * N, 6 * N), order="F")
    info = ctypes.c_int32(0)
    ctx.check(_lib.rsd_stepper_nogmres(ctx.h, N, *[_p(m) for m in mats], _p(Fe), _p(EIN), _p(Fe_inter), _p(conf),
                                       _p(ub) if ub is not None else None, _p(U_par), _p(Sh), _p(Sfp), _p(Sb),
                                       _p(RPP), ctypes.byref(info)))
    return dict(U_par=U_par, SijN_hyd=Sh, SijN_FP=Sfp, SijN_B=Sb, RPP=RPP, info=info.value)


def hydro_SD_FTS(ctx: Context, APP, APQ, AQQ, rfu, rfe, rse, Fe, EIN):
    """hydro_SD_FTS (src/stepper.f90:476-546), the FTS solve of the GMRES
    variant (useGMRESmethod): U_par and SijN of the resistance problem that
    its splitting iteration approaches, solved directly."""
    N = APP.shape[0] // 6
    mats = [np.asfortranarray(x, dtype=np.float64) for x in (APP, APQ, AQQ, rfu, rfe, rse)]
    Fe, EIN = _f64(Fe), _f64(EIN)
    U_par, SijN = np.empty(6 * N), np.empty(5 * N)
    info = ctypes.c_int32(0)
    ctx.check(_lib.rsd_hydro_sd_fts(ctx.h, N, *[_p(m) for m in mats], _p(Fe), _p(EIN), _p(U_par), _p(SijN),
                                    ctypes.byref(info)))
    return dict(U_par=U_par, SijN=SijN, info=info.value)


def DMDX_CAL(ctx: Context, conf, radii, lattice: Lattice, ews_err, mu_f, Z, correction_method=0):
    """DMDX_CAL (src/stepper.f90:664-688): (A1 - A2) Z / deta from the
    translational mobility blocks at conf +- deta Z / 2."""
    conf, r, Z = _f64(conf), _f64(radii), _f64(Z)
    out = np.empty(3 * len(r))
    ctx.check(_lib.rsd_dmdx_cal(ctx.h, len(r), _p(conf), _p(r), ctypes.byref(lattice), ews_err, mu_f,
                                correction_method, _p(Z), _p(out)))
    return out


def brownian_velocity(ctx: Context, APP, conf, radii, lattice: Lattice, ews_err, mu_f, Z, kBT, dt,
                      correction_method=0):
    """u_brown of STEPPER_Stokesian with BROWN (src/stepper.f90:72-86) for
    the caller's standard normal numbers Z (3N)."""
    APP = np.asfortranarray(APP, dtype=np.float64)
    conf, r, Z = _f64(conf), _f64(radii), _f64(Z)
    out = np.empty(3 * len(r))
    info = ctypes.c_int32(0)
    ctx.check(_lib.rsd_brownian_velocity(ctx.h, len(r), _p(APP), _p(conf), _p(r), ctypes.byref(lattice), ews_err,
                                         mu_f, correction_method, _p(Z), kBT, dt, _p(out), ctypes.byref(info)))
    return out


# ------------------------------------------------------------------ fused step
def step_params(N, LB, T, dt, gamma, mu_f, ews_err, nb=0, use_lub=True, precision=PREC_FP64, tol=0.0, max_iter=0):
    p = StepParams()
    p.nn, p.nb = N, nb
    for i in range(3):
        p.LB[i] = LB[i]
    p.T, p.dt, p.gamma, p.mu_f, p.ews_err = T, dt, gamma, mu_f, ews_err
    p.use_lub, p.precision, p.tol, p.max_iter = int(use_lub), precision, tol, max_iter
    return p


def STEPPER_Stokesian(ctx: Context, tab: LubTab, conf, radii, T, dt, LB, gamma, mu_f, ews_err, Fe=None,
                      precision=PREC_FP64, nb=0, use_lub=True, tol=0.0, max_iter=0):
    """One STEPPER_Stokesian step (src/stepper.f90:33-156) on the periodic FTS
    path with lubrication.  Returns the advanced configuration, U_pos, the
    hydrodynamic stresslets SijN_hyd, yeta_mu and the step info."""
    conf = np.array(conf, dtype=np.float64, order="C", copy=True)
    r = _f64(radii)
    N = len(r)
    p = step_params(N, LB, T, dt, gamma, mu_f, ews_err, nb, use_lub, precision, tol, max_iter)
    U_pos = np.empty(6 * N)
    S = np.empty(5 * N)
    y = np.zeros(5)
    info = StepInfo()
    fe = _f64(Fe) if Fe is not None else None
    rc = _lib.rsd_stepper_stokesian(ctx.h, tab.h if tab is not None else None, ctypes.byref(p), _p(conf), _p(r),
                                    _p(fe) if fe is not None else None, _p(U_pos), _p(S), _p(y), ctypes.byref(info))
    ctx.check(rc)
    return dict(conf=conf, U_pos=U_pos, SijN=S, yeta_mu=y, info=info, rc=rc)


def stepper_stokesian_dev(ctx: Context, tab: LubTab, conf_t, radii_t, T, dt, LB, gamma, mu_f, ews_err, U_pos_t, S_t,
                          Fe_t=None, precision=PREC_FP64, nb=0, use_lub=True, tol=0.0, max_iter=0):
    """Device-resident step on torch CUDA tensors (conf_t advanced in place)."""
    N = radii_t.shape[0]
    p = step_params(N, LB, T, dt, gamma, mu_f, ews_err, nb, use_lub, precision, tol, max_iter)
    y = np.zeros(5)
    info = StepInfo()
    rc = _lib.rsd_stepper_stokesian_dev(ctx.h, tab.h if tab is not None else None, ctypes.byref(p),
                                        conf_t.data_ptr(), radii_t.data_ptr(),
                                        Fe_t.data_ptr() if Fe_t is not None else None, U_pos_t.data_ptr(),
                                        S_t.data_ptr(), _p(y), ctypes.byref(info))
    ctx.check(rc)
    return y, info


# ------------------------------------------------------- learned preconditioner
LP_PARAMS_FILE = os.path.join(HERE, "lp_params.npy")


class LearnedPreconditioner:
    """The message-passing network that emits the block-sparse approximate
    inverse of RPP (include/rsd_capi.h, rsd_lp_*).  params: FP32 array of
    rsd_lp_param_count() values, or None for a seeded initialisation."""

    def __init__(self, device=0, params=None, seed=20260400):
        self.h = _vp()
        self.n = int(_lib.rsd_lp_param_count())
        buf = None
        if params is not None:
            buf = np.ascontiguousarray(params, dtype=np.float32)
            if buf.size != self.n:
                raise ValueError("expected %d parameters, got %d" % (self.n, buf.size))
        rc = _lib.rsd_lp_create(ctypes.byref(self.h), device, buf.ctypes.data if buf is not None else None,
                                ctypes.c_uint64(seed))
        if rc != 0:
            raise RSDError(rc, "cannot create the learned preconditioner on CUDA device %d" % device)

    @classmethod
    def trained(cls, device=0, path=None):
        """The network with the committed trained parameters."""
        return cls(device, np.load(path or LP_PARAMS_FILE))

    def params(self):
        out = np.empty(self.n, dtype=np.float32)
        rc = _lib.rsd_lp_get_params(self.h, out.ctypes.data, None)
        if rc:
            raise RSDError(rc, "rsd_lp_get_params")
        return out

    def grad(self):
        out = np.empty(self.n, dtype=np.float32)
        rc = _lib.rsd_lp_get_params(self.h, None, out.ctypes.data)
        if rc:
            raise RSDError(rc, "rsd_lp_get_params")
        return out

    def forward(self, ctx, off, src, dst, xn, xe, dzd=None, dze=None):
        """The network on a given graph and FP32 inputs (torch CUDA tensors);
        returns (zd, ze); with dzd and dze also the parameter gradient."""
        import torch
        nn, ne = xn.shape[0], xe.shape[0]
        zd = torch.empty((nn, 36), dtype=torch.float32, device=xn.device)
        ze = torch.empty((max(ne, 1), 36), dtype=torch.float32, device=xn.device)
        torch.cuda.synchronize(xn.device)
        ctx.check(_lib.rsd_lp_forward_dev(ctx.h, self.h, nn, ne, off.data_ptr(), src.data_ptr(), dst.data_ptr(),
                                          xn.data_ptr(), xe.data_ptr(),
                                          dzd.data_ptr() if dzd is not None else None,
                                          dze.data_ptr() if dze is not None else None, zd.data_ptr(), ze.data_ptr()))
        return zd, ze[:ne]

    def adam_step(self, lr):
        rc = _lib.rsd_lp_adam_step(self.h, ctypes.c_float(lr))
        if rc:
            raise RSDError(rc, "rsd_lp_adam_step")

    def set_training(self, clip_norm=0.0, max_loss=0.0):
        """Guards of train_step: clip the gradient to global norm clip_norm;
        make no update on a step whose loss exceeds max_loss (0: off)."""
        rc = _lib.rsd_lp_set_training(self.h, ctypes.c_float(clip_norm), ctypes.c_double(max_loss))
        if rc:
            raise RSDError(rc, "rsd_lp_set_training")

    def training_stats(self):
        """(norm of the last gradient, steps that made no update, Adam steps)."""
        g, sk, st = ctypes.c_double(0.0), ctypes.c_int64(0), ctypes.c_int64(0)
        rc = _lib.rsd_lp_training_stats(self.h, ctypes.byref(g), ctypes.byref(sk), ctypes.byref(st))
        if rc:
            raise RSDError(rc, "rsd_lp_training_stats")
        return g.value, sk.value, st.value

    def train_step(self, ctx, pos_t, radii_t, lattice, rpp_t, lr):
        """One supervised step on one resistance matrix (torch CUDA tensor,
        FP32 or FP64, the transpose view of a column-major 6N x 6N array, as
        resistance_pp_dev returns it); returns the loss."""
        import torch
        loss = ctypes.c_double(0.0)
        torch.cuda.synchronize(pos_t.device)
        ctx.check(_lib.rsd_lp_train_step(ctx.h, self.h, radii_t.shape[0], pos_t.data_ptr(), radii_t.data_ptr(),
                                         ctypes.byref(lattice), int(rpp_t.dtype == torch.float32),
                                         rpp_t.data_ptr(), rpp_t.stride(1), ctypes.c_float(lr), ctypes.byref(loss)))
        return loss.value

    def close(self):
        if getattr(self, "h", None):
            _lib.rsd_lp_destroy(self.h)
            self.h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def resistance_pp_dev(ctx, tab, conf_t, radii_t, T, LB, gamma, mu_f, ews_err, precision=PREC_FP64, use_lub=True):
    """RPP = (M^-1)_PP + rfu of a configuration on the GPU (FP64 from the
    plain path, FP32 from the mixed form's factors), as a (6N, 6N) tensor
    whose memory is column-major (returned as a transpose view), and the
    lattice."""
    import torch
    N = radii_t.shape[0]
    P = 6 * N
    dt = torch.float64 if precision == PREC_FP64 else torch.float32
    buf = torch.empty((P, P), dtype=dt, device=conf_t.device)
    p = step_params(N, LB, T, 0.0, gamma, mu_f, ews_err, use_lub=use_lub, precision=precision)
    lat = Lattice()
    torch.cuda.synchronize(conf_t.device)
    ctx.check(_lib.rsd_resistance_pp_dev(ctx.h, tab.h if tab is not None else None, ctypes.byref(p),
                                         conf_t.data_ptr(), radii_t.data_ptr(), buf.data_ptr(), P,
                                         ctypes.byref(lat)))
    return buf.t(), lat


def lp_graph_dev(ctx, pos_t, radii_t, lattice):
    """The preconditioner's near-neighbour graph: (off, src, gap) arrays."""
    N = radii_t.shape[0]
    ne = ctypes.c_int32(0)
    ctx.check(_lib.rsd_lp_graph_dev(ctx.h, N, pos_t.data_ptr(), radii_t.data_ptr(), ctypes.byref(lattice),
                                    ctypes.byref(ne), None, None, None))
    off = np.empty(N + 1, dtype=np.int32)
    src = np.empty(max(ne.value, 1), dtype=np.int32)
    gap = np.empty(max(ne.value, 1), dtype=np.float32)
    ctx.check(_lib.rsd_lp_graph_dev(ctx.h, N, pos_t.data_ptr(), radii_t.data_ptr(), ctypes.byref(lattice),
                                    ctypes.byref(ne), off.ctypes.data, src.ctypes.data, gap.ctypes.data))
    return off, src[:ne.value], gap[:ne.value]


def lp_blocks_dev(ctx, net, mode, pos_t, radii_t, lattice, rpp_t):
    """The blocks of Z (zd: N x 6 x 6, ze: edges x 6 x 6) for a mode."""
    import torch
    N = radii_t.shape[0]
    ne = ctypes.c_int32(0)
    off, src, gap = lp_graph_dev(ctx, pos_t, radii_t, lattice)
    zd = np.empty((N, 36), dtype=np.float32)
    ze = np.empty((max(len(src), 1), 36), dtype=np.float32)
    torch.cuda.synchronize(pos_t.device)
    ctx.check(_lib.rsd_lp_blocks_dev(ctx.h, net.h if net is not None else None, int(mode), N, pos_t.data_ptr(),
                                     radii_t.data_ptr(), ctypes.byref(lattice), int(rpp_t.dtype == torch.float32),
                                     rpp_t.data_ptr(), rpp_t.stride(1), zd.ctypes.data, ze.ctypes.data,
                                     ctypes.byref(ne)))
    return zd.reshape(N, 6, 6), ze[:ne.value].reshape(-1, 6, 6), off, src


def pcg_dev(ctx, net, mode, pos_t, radii_t, lattice, rpp_t, b_t, tol=1e-12, maxit=2000):
    """RPP x = b (columns of b_t, a (6N,) or (nrhs, 6N) FP64 tensor in the
    grand layout) by PCG in FP64 with preconditioner `mode`; returns x,
    iterations and the relative residual."""
    import torch
    N = radii_t.shape[0]
    b = b_t.reshape(-1, 6 * N).contiguous()
    x = torch.empty_like(b)
    it, res = ctypes.c_int32(0), ctypes.c_double(0.0)
    torch.cuda.synchronize(pos_t.device)
    ctx.check(_lib.rsd_lp_pcg_dev(ctx.h, net.h if net is not None else None, int(mode), N, pos_t.data_ptr(),
                                  radii_t.data_ptr(), ctypes.byref(lattice), rpp_t.data_ptr(), rpp_t.stride(1),
                                  b.shape[0], b.data_ptr(), x.data_ptr(), float(tol), int(maxit), ctypes.byref(it),
                                  ctypes.byref(res)))
    return x.reshape(b_t.shape), it.value, res.value


def mu_f_dimensionless(mu_f_in=1.0):
    """mu_f after dimentionless_calc/translate (src/mymodules.f90:816,846)."""
    return mu_f_in * (1.0 / PAI / mu_f_in)


def lubdat_dir():
    """The committed copy of the reference's lubrication tables."""
    return os.path.join(os.path.dirname(HERE), "tests", "golden", "lubdat")


from . import configs  # noqa: E402,F401
from . import driver  # noqa: E402,F401
from . import driver_files  # noqa: E402,F401
from . import ensemble  # noqa: E402,F401
from . import contact  # noqa: E402,F401


def driver_step(ctx: Context, tab: LubTab, precision=PREC_MIXED, fp64_fallback=False, on_fallback=None, **kw):
    """The fused step as the step callable of driver.run.  fp64_fallback:
    a mixed step whose refinement does not converge (RSD_ENOCONV) or whose
    FP32 factor is not positive definite (a positive INFO) is taken again in
    the plain FP64 form; on_fallback(T, reason) is told of each such step.
    kw: further STEPPER_Stokesian arguments (tol, max_iter, nb, use_lub)."""
    def step(conf, radii, T, dt, LB, gamma, mu_f, ews_err, Fe=None):
        try:
            out = STEPPER_Stokesian(ctx, tab, conf, radii, T, dt, LB, gamma, mu_f, ews_err, Fe=Fe,
                                    precision=precision, **kw)
            if out["rc"] == 0 or not fp64_fallback or precision == PREC_FP64:
                return out
            reason = "INFO %d" % out["rc"]
        except RSDError as e:
            if not (fp64_fallback and precision != PREC_FP64 and e.code == RSD_ENOCONV):
                raise
            reason = str(e)
        if on_fallback is not None:
            on_fallback(T, reason)
        kw64 = {k: v for k, v in kw.items() if k in ("nb", "use_lub")}
        return STEPPER_Stokesian(ctx, tab, conf, radii, T, dt, LB, gamma, mu_f, ews_err, Fe=Fe, precision=PREC_FP64,
                                 **kw64)
    return step
