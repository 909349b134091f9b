"""Generates overlap_gen.cuh: closed forms of the regularized pair blocks of
Regularization.f90 (Regular_ROTNE_PRAGER_IJ, 18-162), the blocks that
correction_method 2 adds for overlapping pairs (overlap_Regular_
CORRECTION_IJ, GRPY_YZD.f90:813-836).

    python gen_overlap.py        (needs sympy; run by build.py when the
                                  header is older than this script)

The derivative tensors of the regularized potential, Phi'(r) = erf(kap r)
(Init_DD_phir ... Init_DDD4_phir, 552-778, with erf1..erf5 the derivatives
of erf(kap r), 400-472), are taken as the Fortran writes them; before use
each is compared with sympy's own derivative of Phi at a sample point.  They
feed the same J/R/K chain and pair combinations as the Ewald real-space sum
(gen_ewald.pair_blocks) without the volume-fraction factor (phix = 1), and
each of the 60 outputs of a pair block (the order of gen_ewald.py) is
written as

    out_q = sum_t c_t * P_t(a_i, a_j) * g_t(r, F0, Ed, kap) * x^alpha

with F0 = erf(kap r) and Ed = 2 kap exp(-kap^2 r^2) / sqrt(pi):
rsd_reg_image evaluates the terms g x^alpha of one separation and
rsd_reg_epilogue applies the radius polynomials.  Outputs are before the
non-dimensionalisation (1/(6 a_i), 1/(6 a_i^3)) and 1/(pi mu_f).
"""
import os
import sys
import time

import sympy as sp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import gen_ewald as ge  # noqa: E402

OUT = os.path.join(HERE, "overlap_gen.cuh")
x, r, Ed, ai, aj, phix = ge.x, ge.r, ge.Ed, ge.ai, ge.aj, ge.phix
F0, kap = sp.symbols("F0 kap", positive=True)
R3 = range(3)
KD = ge.KD


def kijl(i, j, l):
    return KD(i, j) * x[l] + KD(i, l) * x[j] + KD(j, l) * x[i]


def kijlm(i, j, l, m):
    return (KD(i, j) * x[l] * x[m] + KD(i, l) * x[j] * x[m] + KD(j, l) * x[i] * x[m] + KD(i, m) * x[j] * x[l]
            + KD(j, m) * x[i] * x[l] + KD(l, m) * x[i] * x[j])


def rijl(i, j, l):
    return x[i] * x[j] * x[l]


def rijlm(i, j, l, m):
    return x[i] * x[j] * x[l] * x[m]


def IIiso(i, j, l, m):
    return KD(i, m) * KD(j, l) + KD(i, l) * KD(j, m) + KD(i, j) * KD(l, m)


I2_ = [(i, j) for i in R3 for j in R3]
I3_ = [(i, j, l) for i in R3 for j in R3 for l in R3]
I4 = [(i, j, l, m) for i in R3 for j in R3 for l in R3 for m in R3]


def phi_tensors():
    """Init_*_phir of Regularization.f90, symbolic in x, r, F0, Ed, kap."""
    rl2 = r * r * kap * kap
    f1 = Ed
    f2 = -2 * kap ** 2 * r * Ed
    f3 = 2 * kap ** 2 * Ed * (2 * rl2 - 1)
    f4 = -4 * kap ** 4 * r * Ed * (2 * rl2 - 3)
    f5 = 4 * kap ** 4 * Ed * (4 * rl2 ** 2 - 12 * rl2 + 3)
    t = {}
    t["DD"] = {(i, j): (KD(i, j) / r - x[i] * x[j] / r ** 3) * F0 + x[i] * x[j] / r ** 2 * f1 for i, j in I2_}
    t["DDD"] = {q: (-kijl(*q) / r ** 3 + 3 * rijl(*q) / r ** 5) * F0 + (kijl(*q) / r ** 2 - 3 * rijl(*q) / r ** 4) * f1
                + rijl(*q) / r ** 3 * f2 for q in I3_}
    t["DDDD"] = {q: (-IIiso(*q) / r ** 3 + 3 * kijlm(*q) / r ** 5 - 15 * rijlm(*q) / r ** 7) * F0
                 + (IIiso(*q) / r ** 2 - 3 * kijlm(*q) / r ** 4 + 15 * rijlm(*q) / r ** 6) * f1
                 + (kijlm(*q) / r ** 3 - 6 * rijlm(*q) / r ** 5) * f2 + rijlm(*q) / r ** 4 * f3 for q in I4}
    t["D2"] = 2 / r * F0 + f1
    t["DD2"] = {l: -2 * x[l] / r ** 3 * F0 + 2 * x[l] / r ** 2 * f1 + x[l] / r * f2 for l in R3}
    t["DDD2"] = {(l, m): (-2 * KD(l, m) / r ** 3 + 6 * x[l] * x[m] / r ** 5) * F0
                 + (2 * KD(l, m) / r ** 2 - 6 * x[l] * x[m] / r ** 4) * f1 + (KD(l, m) / r + x[l] * x[m] / r ** 3) * f2
                 + x[l] * x[m] / r ** 2 * f3 for l, m in I2_}
    t["DDDD2"] = {q: (6 * kijl(*q) / r ** 5 - 30 * rijl(*q) / r ** 7) * F0
                  + (-6 * kijl(*q) / r ** 4 + 30 * rijl(*q) / r ** 6) * f1 + (kijl(*q) / r ** 3 - 9 * rijl(*q) / r ** 5) * f2
                  + (kijl(*q) / r ** 2 - rijl(*q) / r ** 4) * f3 + rijl(*q) / r ** 3 * f4 for q in I3_}
    t["DDDDD2"] = {q: (6 * IIiso(*q) / r ** 5 - 30 * kijlm(*q) / r ** 7 + 210 * rijlm(*q) / r ** 9) * F0
                   + (-6 * IIiso(*q) / r ** 4 + 30 * kijlm(*q) / r ** 6 - 210 * rijlm(*q) / r ** 8) * f1
                   + (IIiso(*q) / r ** 3 - 9 * kijlm(*q) / r ** 5 + 75 * rijlm(*q) / r ** 7) * f2
                   + (IIiso(*q) / r ** 2 - kijlm(*q) / r ** 4 - 5 * rijlm(*q) / r ** 6) * f3
                   + (kijlm(*q) / r ** 3 - 4 * rijlm(*q) / r ** 5) * f4 + rijlm(*q) / r ** 4 * f5 for q in I4}
    t["D4"] = 4 / r * f2 + f3
    t["DD4"] = {l: -4 * x[l] / r ** 3 * f2 + 4 * x[l] / r ** 2 * f3 + x[l] / r * f4 for l in R3}
    t["DDD4"] = {(l, m): (-4 * KD(l, m) / r ** 3 + 12 * x[l] * x[m] / r ** 5) * f2
                 + (4 * KD(l, m) / r ** 2 - 12 * x[l] * x[m] / r ** 4) * f3
                 + (KD(l, m) / r + 3 * x[l] * x[m] / r ** 3) * f4 + x[l] * x[m] / r ** 2 * f5 for l, m in I2_}
    return t


def check_against_derivatives(t):
    """Each tensor against the derivative of Phi it stands for (DD = grad
    grad Phi, D2 = lap Phi, DD2 = grad D2, ..., DDD4 = grad grad lap^2 Phi)
    at one sample point, to 30 digits."""
    X = sp.symbols("X0:3", real=True)
    rr = sp.sqrt(X[0] ** 2 + X[1] ** 2 + X[2] ** 2)
    kv = sp.Rational(13, 10)
    grad_phi = [sp.erf(kv * rr) * X[i] / rr for i in R3]
    lap = lambda f: sum(sp.diff(f, X[i], 2) for i in R3)  # noqa: E731
    D2 = sum(sp.diff(grad_phi[i], X[i]) for i in R3)
    D4 = lap(D2)
    want = {"D2": D2, "D4": D4}
    want["DD"] = {(i, j): sp.diff(grad_phi[i], X[j]) for i, j in I2_}
    want["DDD"] = {(i, j, l): sp.diff(grad_phi[i], X[j], X[l]) for i, j, l in I3_}
    want["DDDD"] = {(i, j, l, m): sp.diff(grad_phi[i], X[j], X[l], X[m]) for i, j, l, m in I4}
    want["DD2"] = {l: sp.diff(D2, X[l]) for l in R3}
    want["DDD2"] = {(l, m): sp.diff(D2, X[l], X[m]) for l, m in I2_}
    want["DDDD2"] = {q: sp.diff(D2, X[q[0]], X[q[1]], X[q[2]]) for q in I3_}
    want["DDDDD2"] = {q: sp.diff(D2, X[q[0]], X[q[1]], X[q[2]], X[q[3]]) for q in I4}
    want["DD4"] = {l: sp.diff(D4, X[l]) for l in R3}
    want["DDD4"] = {(l, m): sp.diff(D4, X[l], X[m]) for l, m in I2_}
    pt = {X[0]: sp.Rational(3, 10), X[1]: sp.Rational(-7, 10), X[2]: sp.Rational(1, 2)}
    rv = sp.sqrt(sum(v ** 2 for v in pt.values()))
    sub = {x[i]: pt[X[i]] for i in R3}
    sub.update({r: rv, kap: kv, F0: sp.erf(kv * rv), Ed: 2 * kv * sp.exp(-kv ** 2 * rv ** 2) / sp.sqrt(sp.pi)})
    worst = 0
    for name, w in want.items():
        got = t[name]
        items = [(None, w, got)] if not isinstance(w, dict) else [(q, w[q], got[q]) for q in w]
        for q, a, b in items:
            va = sp.N(a.subs(pt), 40)
            vb = sp.N(b.subs(sub), 40)
            worst = max(worst, abs(va - vb))
            if abs(va - vb) > sp.Float("1e-30"):
                raise AssertionError("%s%s: Fortran form %s, derivative %s" % (name, q, vb, va))
    return worst


def regular_chain(t):
    Jr = {(i, j): KD(i, j) * t["D2"] - t["DD"][i, j] for i, j in I2_}
    D_Jr = {(i, j, l): KD(i, j) * t["DD2"][l] - t["DDD"][l, i, j] for i, j, l in I3_}
    DD_Jr = {(i, j, m, l): KD(i, j) * t["DDD2"][m, l] - t["DDDD"][m, l, i, j] for i, j, m, l in I4}
    D2_Jr = {(i, j): KD(i, j) * t["D4"] - t["DDD2"][i, j] for i, j in I2_}
    DD2_Jr = {(i, j, kk): KD(i, j) * t["DD4"][kk] - t["DDDD2"][kk, i, j] for i, j, kk in I3_}
    DDD2_Jr = {(i, j, l, kk): KD(i, j) * t["DDD4"][l, kk] - t["DDDDD2"][l, kk, i, j] for i, j, l, kk in I4}
    outs = ge.unique_outputs(*ge.pair_blocks(Jr, D_Jr, DD_Jr, D2_Jr, DD2_Jr, DDD2_Jr))
    return [sp.sympify(e).subs(phix, 1) for e in outs]


def emit(dec, mom):
    L = []
    L.append("// Generated by gen_overlap.py -- do not edit.  Closed forms of the regularized")
    L.append("// pair blocks of Regularization.f90 (Regular_ROTNE_PRAGER_IJ), as terms of one")
    L.append("// separation plus a per-pair epilogue.  See gen_overlap.py for the output order.")
    L.append("#pragma once")
    L.append("#define RSD_NMOM_REG %d" % len(mom))
    L.append("")
    fn_list = {}
    for g, xm in mom:
        fn_list.setdefault(sp.srepr(g), g)
    fns = list(fn_list.values())
    monos = sorted({xm for _, xm in mom if sum(xm) > 0}, key=lambda q: (sum(q), q))
    L.append("// The terms of the separation (x0,x1,x2), r = |x|, ir = 1/r, F0 = erf(kap r),")
    L.append("// Ed = 2 kap exp(-kap^2 r^2)/sqrt(pi), into acc[0..RSD_NMOM_REG).")
    L.append("template <typename T>")
    L.append("__device__ __forceinline__ void rsd_reg_image(T x0, T x1, T x2, T r, T ir, T F0, T Ed, T kap,")
    L.append("                                              T* __restrict__ acc) {")
    irs = sp.Symbol("ir")
    used = set()
    fexprs = []
    for g in fns:
        e = sp.expand(g.subs(r, 1 / irs))

        def pw(q):
            n = int(q.exp)
            if q.base == irs:
                nm = "ir%d" % n if n > 0 else "rp%d" % (-n)
            else:
                nm = "kap%d" % n
            used.add(nm)
            return sp.Symbol(nm)

        e = e.replace(lambda q: q.is_Pow and q.base in (irs, kap) and q.exp.is_Integer, pw)
        fexprs.append(e)

    def split(nm):
        for base, pre in (("ir", "ir"), ("r", "rp"), ("kap", "kap")):
            if nm.startswith(pre):
                return base, int(nm[len(pre):])

    for nm in sorted(used, key=lambda s_: split(s_)):
        base, n = split(nm)
        if n == 1:
            if nm != "r":
                L.append("  const T %s = %s;" % (nm, base))
            continue
        L.append("  const T %s = %s;" % (nm, " * ".join([base] * n)))
    rep, red = sp.cse(fexprs, symbols=sp.numbered_symbols("t"), optimizations="basic")
    for s_, e in rep:
        L.append("  const T %s = %s;" % (s_, sp.ccode(e)))
    fnames = []
    for i, e in enumerate(red):
        nm = "g%d" % i
        fnames.append(nm)
        L.append("  const T %s = %s;" % (nm, sp.ccode(e)))
    have = ge.emit_monomials(L, monos, "x", "T")
    fidx = {sp.srepr(g): i for i, g in enumerate(fns)}
    for m, (g, xm) in enumerate(mom):
        f = fnames[fidx[sp.srepr(g)]]
        mono = have.get(xm) if sum(xm) > 0 else None
        L.append("  acc[%d] = %s;" % (m, f if mono is None else "%s * %s" % (f, mono)))
    L.append("}")
    L.append("")
    L.append("// Regularized pair block (60 values) from the terms of rsd_reg_image.")
    L.append("template <typename T>")
    L.append("__device__ __forceinline__ void rsd_reg_epilogue(const T* __restrict__ acc, T ai, T aj, T* __restrict__ out) {")
    L.append("  const T ai2 = ai * ai, ai3 = ai2 * ai, ai4 = ai2 * ai2, ai5 = ai4 * ai, aj2 = aj * aj;")
    L.append("  const T aj3 = aj2 * aj, aj4 = aj2 * aj2; (void)aj3; (void)aj4; (void)ai4; (void)ai5;")
    for q, terms in enumerate(dec):
        if not terms:
            L.append("  out[%d] = T(0);" % q)
            continue
        parts = []
        for const, rm, m in terms:
            assert rm[2] == 0
            parts.append(" * ".join(["T(%s)" % sp.ccode(sp.N(const, 20))] + ge.radius_poly(rm) + ["acc[%d]" % m]))
        L.append("  out[%d] = %s;" % (q, " + ".join(parts)))
    L.append("}")
    return "\n".join(L) + "\n"


def main():
    t0 = time.time()
    t = phi_tensors()
    worst = check_against_derivatives(t)
    print("phi tensors match the derivatives of Phi (worst %.1e, %.1fs)" % (float(worst), time.time() - t0),
          file=sys.stderr)
    outs = regular_chain(t)
    dec, mom = ge.decompose(outs, x, (r, F0, Ed, kap))
    print("regularized terms %d (%.1fs)" % (len(mom), time.time() - t0), file=sys.stderr)
    with open(OUT, "w") as fp:
        fp.write(emit(dec, mom))
    print("wrote %s (%.1fs)" % (OUT, time.time() - t0), file=sys.stderr)


if __name__ == "__main__":
    main()
