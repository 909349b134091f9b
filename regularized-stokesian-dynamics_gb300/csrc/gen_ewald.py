"""Generate ewald_gen.cuh: closed forms of the Ewald pair sums.

Build-time tool (run by build.py when the header is missing or older than
this script).  It takes the derivative chain of Ewald_summation.f90 -- the
erfc(lambda r) derivatives (Init_erfc1..6, 658-743), their Cartesian tensors
(Init_*_rerfc, 808-1053), the J/R/K tensors (Init_*Jr/Ror/Kr, 427-650), the
pair combinations of PER_ROTNE_PRAGER_IJ (196-423) and the Y2 projections of
tensors.f90 (QQ_TR/GH_TR 993-1023) -- symbolically, and rewrites each of the
60 distinct outputs of one pair block (TT, RR symmetric 3x3; TR antisymmetric
3x3; QQ symmetric 5x5; G, H 3x5) as

    out_q = sum_t  c_t * P_t(a_i, a_j, phix) * MOM_m(t)

where every moment MOM_m = sum over images of  g_f(r) * x^alpha  (real space)
or  sum over k of  S(k) k^alpha * {cos,sin}(k.R)  (reciprocal space) does
not depend on the radii.  The kernels accumulate the moments per pair and
apply the radius polynomials once, in the epilogue.

Output order of the 60 values (0-based):
  0..5   TT  (00,01,02,11,12,22)
  6..11  RR  (00,01,02,11,12,22)
  12..14 TR  (01,02,12); TR(j,i) = -TR(i,j), TR(i,i) = 0
  15..29 QQ  (5x5 upper triangle, row-major: 00,01,..,04,11,..,44)
  30..44 G   (c,m) -> 30 + 5c + m
  45..59 H   (c,m) -> 45 + 5c + m
"""
import os
import sys
import time

import sympy as sp

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "ewald_gen.cuh")

x = sp.symbols("x0:3", real=True)
k = sp.symbols("k0:3", real=True)
r, E0, Ed, lam, ai, aj, phix, S = sp.symbols("r E0 Ed lam ai aj phix S", positive=True)
R3 = range(3)


def KD(i, j):
    return 1 if i == j else 0


def eps(i, j, l):
    return sp.LeviCivita(i, j, l)


def y2_basis():
    Y = {(m, i, j): 0 for m in range(5) for i in R3 for j in R3}
    s2 = 1 / sp.sqrt(2)
    s6 = 1 / sp.sqrt(6)
    Y[0, 0, 1] = Y[0, 1, 0] = s2
    Y[1, 1, 2] = Y[1, 2, 1] = -s2
    Y[2, 0, 0] = Y[2, 1, 1] = -s6
    Y[2, 2, 2] = sp.sqrt(sp.Rational(2, 3))
    Y[3, 0, 2] = Y[3, 2, 0] = -s2
    Y[4, 0, 0] = s2
    Y[4, 1, 1] = -s2
    return Y


Y2 = y2_basis()
half = sp.Rational(1, 2)


def pair_blocks(Jr, D_Jr, DD_Jr, D2_Jr, DD2_Jr, DDD2_Jr):
    """Pair combinations of PER_ROTNE_PRAGER_IJ given the J tensors (real
    space) or their Fourier counterparts; the same algebra in both sums."""
    Ror = {(i, j): sum(-half * eps(j, kk, l) * D_Jr[i, l, kk] for kk in R3 for l in R3) for i in R3 for j in R3}
    D_Ror = {(i, j, l): sum(-half * eps(j, m, n) * DD_Jr[i, n, l, m] for m in R3 for n in R3)
             for i in R3 for j in R3 for l in R3}
    D2_Ror = {(i, j): sum(-half * eps(j, kk, l) * DD2_Jr[i, l, kk] for kk in R3 for l in R3) for i in R3 for j in R3}
    Kr = {(i, j, kk): half * (D_Jr[i, j, kk] + D_Jr[i, kk, j]) for i in R3 for j in R3 for kk in R3}
    D_Kr = {(i, j, kk, l): half * (DD_Jr[i, j, l, kk] + DD_Jr[i, kk, l, j])
            for i in R3 for j in R3 for kk in R3 for l in R3}
    D2_Kr = {(i, j, kk): half * (DD2_Jr[i, j, kk] + DD2_Jr[i, kk, j]) for i in R3 for j in R3 for kk in R3}
    DD2_Kr = {(i, j, kk, l): half * (DDD2_Jr[i, j, l, kk] + DDD2_Jr[i, kk, l, j])
              for i in R3 for j in R3 for kk in R3 for l in R3}
    a3 = ai ** 3
    TT = {(i, j): sp.Rational(3, 4) * ai * Jr[i, j] + sp.Rational(3, 4) * ai * (ai ** 2 + aj ** 2) / 6 * D2_Jr[i, j] * phix
          for i in R3 for j in R3}
    RR = {(i, j): 3 * a3 / 8 * sum(eps(i, kk, l) * D_Ror[l, j, kk] for kk in R3 for l in R3) for i in R3 for j in R3}
    QQ = {(i, j, kk, l): -sp.Rational(3, 4) * a3 * half * (D_Kr[i, kk, l, j] + D_Kr[j, kk, l, i])
          - sp.Rational(3, 40) * a3 * (ai ** 2 + aj ** 2) * half * (DD2_Kr[i, kk, l, j] + DD2_Kr[j, kk, l, i])
          for i in R3 for j in R3 for kk in R3 for l in R3}
    GP = {(i, j, kk): -sp.Rational(3, 4) * ai * (Kr[i, j, kk] + (ai ** 2 / 6 + aj ** 2 / 10) * D2_Kr[i, j, kk])
          for i in R3 for j in R3 for kk in R3}
    HP = {(i, j, kk): -sp.Rational(3, 8) * a3 * sum(eps(i, l, m) * (D_Kr[m, j, kk, l] + aj ** 2 / 10 * DD2_Kr[m, j, kk, l])
                                                   for l in R3 for m in R3) for i in R3 for j in R3 for kk in R3}
    TR = {(i, j): sp.Rational(3, 4) * ai * Ror[i, j] + a3 / 8 * D2_Ror[i, j] for i in R3 for j in R3}
    QQ_TR = {(a, b): sum(QQ[i, j, kk, l] * Y2[a, i, j] * Y2[b, kk, l] for i in R3 for j in R3 for kk in R3 for l in R3)
             for a in range(5) for b in range(5)}
    G_TR = {(c, m): sum(GP[c, i, j] * Y2[m, i, j] for i in R3 for j in R3) for c in R3 for m in range(5)}
    H_TR = {(c, m): sum(HP[c, i, j] * Y2[m, i, j] for i in R3 for j in R3) for c in R3 for m in range(5)}
    return TT, RR, TR, QQ_TR, G_TR, H_TR


def unique_outputs(TT, RR, TR, QQ_TR, G_TR, H_TR):
    sym = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    outs = [TT[p] for p in sym] + [RR[p] for p in sym] + [TR[0, 1], TR[0, 2], TR[1, 2]]
    outs += [QQ_TR[a, b] for a in range(5) for b in range(a, 5)]
    outs += [G_TR[c, m] for c in R3 for m in range(5)]
    outs += [H_TR[c, m] for c in R3 for m in range(5)]
    assert len(outs) == 60
    return outs


def real_space_chain():
    """Ewald_summation.f90:658-1053 and 427-650, symbolic in x, r, E0 =
    erfc(lam r), Ed = 2 lam exp(-lam^2 r^2)/sqrt(pi)."""
    rl2 = r * r * lam * lam
    e1 = -Ed
    e2 = 2 * lam * lam * r * Ed
    e3 = -2 * lam * lam * Ed * (2 * rl2 - 1)
    e4 = 4 * lam ** 4 * r * Ed * (2 * rl2 - 3)
    e5 = -4 * lam ** 4 * Ed * (4 * rl2 ** 2 - 12 * rl2 + 3)
    e6 = 8 * lam ** 6 * r * Ed * (4 * rl2 ** 2 - 20 * rl2 + 15)

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

    I4 = [(i, j, l, m) for i in R3 for j in R3 for l in R3 for m in R3]
    I3_ = [(i, j, l) for i in R3 for j in R3 for l in R3]
    I2_ = [(i, j) for i in R3 for j in R3]
    DD = {(i, j): (KD(i, j) / r - x[i] * x[j] / r ** 3) * E0 + (KD(i, j) + x[i] * x[j] / r ** 2) * e1 + x[i] * x[j] / r * e2
          for i, j in I2_}
    DDD = {(i, j, l): (-kijl(i, j, l) / r ** 3 + 3 * rijl(i, j, l) / r ** 5) * E0
           - (-kijl(i, j, l) / r ** 2 + 3 * rijl(i, j, l) / r ** 4) * e1 + kijl(i, j, l) / r * e2 + rijl(i, j, l) / r ** 2 * e3
           for i, j, l in I3_}
    DDDD = {t: (-IIiso(*t) / r ** 3 + 3 * kijlm(*t) / r ** 5 - 15 * rijlm(*t) / r ** 7) * E0
            - (-IIiso(*t) / r ** 2 + 3 * kijlm(*t) / r ** 4 - 15 * rijlm(*t) / r ** 6) * e1
            + (IIiso(*t) / r - 3 * rijlm(*t) / r ** 5) * e2 + (kijlm(*t) / r ** 2 - 2 * rijlm(*t) / r ** 4) * e3
            + rijlm(*t) / r ** 3 * e4 for t in I4}
    D2 = 2 / r * E0 + 4 * e1 + r * e2
    DD2 = {l: -2 * x[l] / r ** 3 * E0 + 2 * x[l] / r ** 2 * e1 + 5 * x[l] / r * e2 + x[l] * e3 for l in R3}
    DDD2 = {(l, m): (-2 * KD(l, m) / r ** 3 + 6 * x[l] * x[m] / r ** 5) * E0
            - (-2 * KD(l, m) / r ** 2 + 6 * x[l] * x[m] / r ** 4) * e1 + (5 * KD(l, m) / r - 3 * x[l] * x[m] / r ** 3) * e2
            + (KD(l, m) + 5 * x[l] * x[m] / r ** 2) * e3 + x[l] * x[m] / r * e4 for l, m in I2_}
    DDDD2 = {t: (6 * kijl(*t) / r ** 5 - 30 * rijl(*t) / r ** 7) * E0 - (6 * kijl(*t) / r ** 4 - 30 * rijl(*t) / r ** 6) * e1
             + (-3 * kijl(*t) / r ** 3 + 3 * rijl(*t) / r ** 5) * e2 + (5 * kijl(*t) / r ** 2 - 13 * rijl(*t) / r ** 4) * e3
             + (kijl(*t) / r + 4 * rijl(*t) / r ** 3) * e4 + rijl(*t) / r ** 2 * e5 for t in I3_}
    DDDDD2 = {t: (6 * IIiso(*t) / r ** 5 - 30 * kijlm(*t) / r ** 7 + 210 * rijlm(*t) / r ** 9) * E0
              - (6 * IIiso(*t) / r ** 4 - 30 * kijlm(*t) / r ** 6 + 210 * rijlm(*t) / r ** 8) * e1
              + (-3 * IIiso(*t) / r ** 3 + 3 * kijlm(*t) / r ** 5 + 15 * rijlm(*t) / r ** 7) * e2
              + (5 * IIiso(*t) / r ** 2 - 13 * kijlm(*t) / r ** 4 + 55 * rijlm(*t) / r ** 6) * e3
              + (IIiso(*t) / r + 4 * kijlm(*t) / r ** 3 - 25 * rijlm(*t) / r ** 5) * e4
              + (kijlm(*t) / r ** 2 + 2 * rijlm(*t) / r ** 4) * e5 + rijlm(*t) / r ** 3 * e6 for t in I4}
    D4 = 12 / r * e2 + 8 * e3 + r * e4
    DD4 = {l: -12 * x[l] / r ** 3 * e2 + 12 * x[l] / r ** 2 * e3 + 9 * x[l] / r * e4 + x[l] * e5 for l in R3}
    DDD4 = {(l, m): (-12 * KD(l, m) / r ** 3 + 36 * x[l] * x[m] / r ** 5) * e2
            - (-12 * KD(l, m) / r ** 2 + 36 * x[l] * x[m] / r ** 4) * e3 + (9 * KD(l, m) / r + 3 * x[l] * x[m] / r ** 3) * e4
            + (KD(l, m) + 9 * x[l] * x[m] / r ** 2) * e5 + x[l] * x[m] / r * e6 for l, m in I2_}
    Jr = {(i, j): KD(i, j) * D2 - DD[i, j] for i, j in I2_}
    D_Jr = {(i, j, l): KD(i, j) * DD2[l] - DDD[l, i, j] for i, j, l in I3_}
    DD_Jr = {(i, j, m, l): KD(i, j) * DDD2[m, l] - DDDD[m, l, i, j] for i, j, m, l in I4}
    D2_Jr = {(i, j): KD(i, j) * D4 - DDD2[i, j] for i, j in I2_}
    DD2_Jr = {(i, j, kk): KD(i, j) * DD4[kk] - DDDD2[kk, i, j] for i, j, kk in I3_}
    DDD2_Jr = {(i, j, l, kk): KD(i, j) * DDD4[l, kk] - DDDDD2[l, kk, i, j] for i, j, l, kk in I4}
    return pair_blocks(Jr, D_Jr, DD_Jr, D2_Jr, DD2_Jr, DDD2_Jr)


def fourier_chain():
    """Ewald_summation.f90:1057-1257 with F_Jk = S (delta k^2 - k k) where
    S = 8 pi (1 + k^2/4lam^2 + k^4/8lam^4) exp(-k^2/4lam^2) / k^4.  Returns
    the cos- and sin-weighted parts of each pair block."""
    k2 = k[0] ** 2 + k[1] ** 2 + k[2] ** 2
    I2_ = [(i, j) for i in R3 for j in R3]
    F_Jk = {(i, j): S * (KD(i, j) * k2 - k[i] * k[j]) for i, j in I2_}
    F_DJk = {(i, j, l): k[l] * F_Jk[i, j] for i, j in I2_ for l in R3}
    F_DDJk = {(i, j, m, l): -k[m] * k[l] * F_Jk[i, j] for i, j in I2_ for m in R3 for l in R3}
    F_D2Jk = {(i, j): -k2 * F_Jk[i, j] for i, j in I2_}
    F_DD2Jk = {(i, j, l): k[l] * F_D2Jk[i, j] for i, j in I2_ for l in R3}
    # F_D2Kk = F_DD2Jk and F_DD2Kk(i,j,k,l) = k_k k_l |k|^2 F_Jk(i,j): these
    # replace the symmetrised D2_Kr / DD2_Kr of real space (1213-1257)
    F_DDD2Jk = {(i, j, l, kk): k[l] * k[kk] * k2 * F_Jk[i, j] for i, j in I2_ for l in R3 for kk in R3}
    Ror = {(i, j): sum(-half * eps(j, m, n) * F_DJk[i, n, m] for m in R3 for n in R3) for i, j in I2_}
    D_Ror = {(i, j, l): sum(-half * eps(j, m, n) * F_DDJk[i, n, l, m] for m in R3 for n in R3) for i, j in I2_ for l in R3}
    D2_Ror = {(i, j): sum(-half * eps(j, m, n) * F_DD2Jk[i, n, m] for m in R3 for n in R3) for i, j in I2_}
    Kr = {(i, j, kk): half * (F_DJk[i, j, kk] + F_DJk[i, kk, j]) for i, j in I2_ for kk in R3}
    D_Kr = {(i, j, kk, l): half * (F_DDJk[i, j, l, kk] + F_DDJk[i, kk, l, j]) for i, j in I2_ for kk in R3 for l in R3}
    D2_Kr = {(i, j, kk): F_DD2Jk[i, j, kk] for i, j in I2_ for kk in R3}
    DD2_Kr = {(i, j, kk, l): F_DDD2Jk[i, j, kk, l] for i, j in I2_ for kk in R3 for l in R3}
    a3 = ai ** 3
    TT = {(i, j): (sp.Rational(3, 4) * ai * F_Jk[i, j] + sp.Rational(3, 4) * ai * (ai ** 2 + aj ** 2) / 6 * F_D2Jk[i, j] * phix)
          for i, j in I2_}
    RR = {(i, j): 3 * a3 / 8 * sum(eps(i, kk, l) * D_Ror[l, j, kk] for kk in R3 for l in R3) for i, j in I2_}
    QQ = {(i, j, kk, l): -sp.Rational(3, 4) * a3 * half * (D_Kr[i, kk, l, j] + D_Kr[j, kk, l, i])
          - sp.Rational(3, 40) * a3 * (ai ** 2 + aj ** 2) * half * (DD2_Kr[i, kk, l, j] + DD2_Kr[j, kk, l, i])
          for i in R3 for j in R3 for kk in R3 for l in R3}
    GP = {(i, j, kk): sp.Rational(3, 4) * ai * (Kr[i, j, kk] + (ai ** 2 / 6 + aj ** 2 / 10) * D2_Kr[i, j, kk])
          for i in R3 for j in R3 for kk in R3}
    HP = {(i, j, kk): -sp.Rational(3, 8) * a3 * sum(eps(i, l, m) * (D_Kr[m, j, kk, l] + aj ** 2 / 10 * DD2_Kr[m, j, kk, l])
                                                   for l in R3 for m in R3) for i in R3 for j in R3 for kk in R3}
    TR = {(i, j): -(ai * sp.Rational(3, 4) * Ror[i, j] + a3 / 8 * D2_Ror[i, j]) for i, j in I2_}
    QQ_TR = {(a, b): sum(QQ[i, j, kk, l] * Y2[a, i, j] * Y2[b, kk, l] for i in R3 for j in R3 for kk in R3 for l in R3)
             for a in range(5) for b in range(5)}
    G_TR = {(c, m): sum(GP[c, i, j] * Y2[m, i, j] for i in R3 for j in R3) for c in R3 for m in range(5)}
    H_TR = {(c, m): sum(HP[c, i, j] * Y2[m, i, j] for i in R3 for j in R3) for c in R3 for m in range(5)}
    # cos-weighted: TT RR QQ H ; sin-weighted: G TR  (PER_ROTNE_PRAGER_IJ 357-412)
    return TT, RR, TR, QQ_TR, G_TR, H_TR


def decompose(outs, vars_, radial_syms):
    """Write each output as sum_t c_t * P_t(ai,aj,phix) * g_t * mono_t(vars_)
    with g_t free of numeric factors; returns per-output term lists and the
    moment list [(g, mono)]."""
    moments = {}
    order = []
    dec = []
    for e in outs:
        e = sp.expand(e)
        terms = []
        if e == 0:
            dec.append(terms)
            continue
        P = sp.Poly(e, *vars_, ai, aj, phix)
        for mono, coeff in P.terms():
            coeff = sp.factor(sp.nsimplify(coeff))
            const, g = coeff.as_independent(*radial_syms, as_Add=False)
            g = sp.simplify(g)
            c2, g2 = g.as_coeff_Mul()
            const = sp.nsimplify(const * c2)
            g = g2
            xm = mono[:3]
            rm = mono[3:]
            key = (sp.srepr(g), xm)
            if key not in moments:
                moments[key] = len(order)
                order.append((g, xm))
            terms.append((const, rm, moments[key]))
        dec.append(terms)
    return dec, order


def ccode(e, T="T"):
    s = sp.ccode(e)
    return s


def radius_poly(rm):
    a, b, p = rm
    parts = []
    if a:
        parts.append("ai%d" % a if a > 1 else "ai")
    if b:
        parts.append("aj%d" % b if b > 1 else "aj")
    if p:
        parts.append("phix" if p == 1 else "phix%d" % p)
    return parts


def mono_name(xm, base="x"):
    if sum(xm) == 0:
        return None
    return "%s%d%d%d" % ((base,) + tuple(xm))


def emit_monomials(lines, monos, base, T):
    """Emit the products x^alpha needed, each built from one of lower
    degree; returns {alpha: name}."""
    need = set()
    stack = [m for m in monos if sum(m) >= 2]
    plan = {}
    while stack:
        m = stack.pop()
        if m in need:
            continue
        need.add(m)
        i = max(range(3), key=lambda q: m[q])
        m1 = list(m)
        m1[i] -= 1
        m1 = tuple(m1)
        plan[m] = (m1, i)
        if sum(m1) >= 2:
            stack.append(m1)
    have = {(1, 0, 0): base + "0", (0, 1, 0): base + "1", (0, 0, 1): base + "2"}
    for m in sorted(need, key=lambda t: (sum(t), t)):
        m1, i = plan[m]
        nm = mono_name(m, base)
        lines.append("  const %s %s = %s * %s%d;" % (T, nm, have[m1], base, i))
        have[m] = nm
    return have


def gen():
    t0 = time.time()
    real = unique_outputs(*real_space_chain())
    four = fourier_chain()
    cosp = unique_outputs(four[0], four[1], {p: 0 for p in four[2]}, four[3], {p: 0 for p in four[4]}, four[5])
    sinp = unique_outputs({p: 0 for p in four[0]}, {p: 0 for p in four[1]}, four[2], {p: 0 for p in four[3]}, four[4],
                          {p: 0 for p in four[5]})
    print("chains built %.1fs" % (time.time() - t0), file=sys.stderr)
    dec_r, mom_r = decompose(real, x, (r, E0, Ed, lam))
    dec_c, mom_c = decompose(cosp, k, (S, lam))
    dec_s, mom_s = decompose(sinp, k, (S, lam))
    print("real moments %d, k cos moments %d, k sin moments %d (%.1fs)" % (len(mom_r), len(mom_c), len(mom_s),
                                                                          time.time() - t0), file=sys.stderr)
    L = []
    L.append("// Generated by gen_ewald.py -- do not edit.  Closed forms of the Ewald pair sums")
    L.append("// of Ewald_summation.f90 (PER_ROTNE_PRAGER_IJ), written as radius-independent")
    L.append("// moments plus a per-pair epilogue.  See gen_ewald.py for the output order.")
    L.append("#pragma once")
    L.append("#define RSD_NMOM_REAL %d" % len(mom_r))
    L.append("#define RSD_NMOM_KCOS %d" % len(mom_c))
    L.append("#define RSD_NMOM_KSIN %d" % len(mom_s))
    # ---- real-space image accumulation
    fn_list = {}
    for g, xm in mom_r:
        fn_list.setdefault(sp.srepr(g), g)
    fns = list(fn_list.values())
    monos = sorted({xm for _, xm in mom_r if sum(xm) > 0}, key=lambda t: (sum(t), t))
    L.append("")
    L.append("// Adds one real-space image at separation (x0,x1,x2), r = |x|, E0 = erfc(lam r),")
    # partitions of the moments into NP = 2..4 parts that share few radial
    # functions (whole g-groups, greedily balanced), for kernels that sum the
    # moments of one part per pass over the images
    fidx0 = {sp.srepr(g): i for i, g in enumerate(fns)}
    groups = {}
    for m, (g, xm) in enumerate(mom_r):
        groups.setdefault(fidx0[sp.srepr(g)], []).append(m)
    tables = {}
    for NP in (2, 3, 4):
        load = [0] * NP
        part = [0] * len(mom_r)
        for gi, ms in sorted(groups.items(), key=lambda kv: -len(kv[1])):
            pbest = min(range(NP), key=lambda p_: load[p_])
            for m in ms:
                part[m] = pbest
            load[pbest] += len(ms)
        tables[NP] = part
    L.append("// Part of real moment m when the moments are summed in NP passes (NP = 1..4):")
    L.append("// whole groups of moments that share a radial function, balanced by count.")
    L.append("__host__ __device__ constexpr int rsd_mom_part(int m, int NP) {")
    for NP in (2, 3, 4):
        L.append("  constexpr unsigned char p%d[%d] = {%s};" % (NP, len(mom_r), ", ".join(str(v) for v in tables[NP])))
    L.append("  return NP <= 1 ? 0 : NP == 2 ? p2[m] : NP == 3 ? p3[m] : p4[m];")
    L.append("}")
    L.append("")
    L.append("// Adds one real-space image at separation (x0,x1,x2), r = |x|, E0 = erfc(lam r),")
    L.append("// Ed = 2 lam exp(-lam^2 r^2)/sqrt(pi); lam2..lam10 are powers of lam.  A is the")
    L.append("// accumulator type (T, or a wider accumulator with fma(T, T, A) and A += T).")
    L.append("// With NP > 1 only the moments of part P (rsd_mom_part) are added.")
    L.append("template <typename T, typename A = T, int NP = 1, int P = 0>")
    L.append("__device__ __forceinline__ void rsd_real_image(T x0, T x1, T x2, T r, T ir, T E0, T Ed, T lam,")
    L.append("                                               A* __restrict__ acc) {")
    irs = sp.Symbol("ir")
    fexprs = []
    used = set()
    for g in fns:
        e = sp.expand(g.subs(r, 1 / irs))

        def pw(t):
            n = int(t.exp)
            if t.base == irs:
                nm = "ir%d" % n if n > 0 else "rp%d" % (-n)
            else:
                nm = "lam%d" % n
            used.add(nm)
            return sp.Symbol(nm)

        e = e.replace(lambda t: t.is_Pow and t.base in (irs, lam) and t.exp.is_Integer, pw)
        fexprs.append(e)
    def split(nm):
        for base, pre in (("ir", "ir"), ("r", "rp"), ("lam", "lam")):
            if nm.startswith(pre):
                return base, int(nm[len(pre):])

    for nm in sorted(used, key=lambda s_: split(s_)):
        base, n = split(nm)
        if n == 1:
            if base != "r" or nm != "r":
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
    have = emit_monomials(L, monos, "x", "T")
    fidx = {sp.srepr(g): i for i, g in enumerate(fns)}
    for m, (g, xm) in enumerate(mom_r):
        f = fnames[fidx[sp.srepr(g)]]
        mono = have.get(xm) if sum(xm) > 0 else None
        pre = "  if constexpr (rsd_mom_part(%d, NP) == P) " % m
        if mono is None:
            L.append(pre + "acc[%d] += %s;" % (m, f))
        else:
            L.append(pre + "acc[%d] = fma(%s, %s, acc[%d]);" % (m, f, mono, m))
    L.append("}")
    L.append("")

    def epilogue(name, dec, what):
        L.append("// %s" % what)
        L.append("template <typename T>")
        L.append("__device__ __forceinline__ void %s(const T* __restrict__ acc, T ai, T aj, T phix, T* __restrict__ out) {"
                 % name)
        L.append("  const T ai2 = ai * ai, ai3 = ai2 * ai, ai4 = ai2 * ai2, ai5 = ai4 * ai, aj2 = aj * aj;")
        L.append("  const T aj3 = aj2 * aj, aj4 = aj2 * aj2, phix2 = phix * phix; (void)aj3; (void)aj4; (void)phix2;")
        L.append("  (void)ai4; (void)ai5;")
        for q, terms in enumerate(dec):
            if not terms:
                L.append("  out[%d] = T(0);" % q)
                continue
            parts = []
            for const, rm, m in terms:
                c = sp.N(const, 20)
                rp = radius_poly(rm)
                f = ["T(%s)" % sp.ccode(c)] + rp + ["acc[%d]" % m]
                parts.append(" * ".join(f))
            L.append("  out[%d] = %s;" % (q, " + ".join(parts)))
        L.append("}")
        L.append("")

    epilogue("rsd_real_epilogue", dec_r, "Real-space pair block from the accumulated moments.")

    # the same epilogue as a sparse table: coefficients c[k] of the
    # (output, moment) pairs, formed once for given radii, then applied as
    # 60 chains of multiply-adds
    pairs = {}
    for q, terms in enumerate(dec_r):
        for const, rm, m in terms:
            pairs.setdefault((q, m), []).append((const, rm))
    keys = sorted(pairs)
    L.append("// The real-space epilogue as a table: c[k] (rsd_real_epi_coef) is the")
    L.append("// coefficient of moment m_k in output q_k (rsd_real_epi_apply).")
    L.append("#define RSD_REAL_EPI_NC %d" % len(keys))
    L.append("template <typename T>")
    L.append("__host__ __device__ inline void rsd_real_epi_coef(T ai, T aj, T phix, T* __restrict__ c) {")
    L.append("  const T ai2 = ai * ai, ai3 = ai2 * ai, ai4 = ai2 * ai2, ai5 = ai4 * ai, aj2 = aj * aj;")
    L.append("  const T aj3 = aj2 * aj, aj4 = aj2 * aj2, phix2 = phix * phix; (void)aj3; (void)aj4; (void)phix2;")
    L.append("  (void)ai4; (void)ai5;")
    for kk, key in enumerate(keys):
        parts = []
        for const, rm in pairs[key]:
            parts.append(" * ".join(["T(%s)" % sp.ccode(sp.N(const, 20))] + radius_poly(rm)))
        L.append("  c[%d] = %s;" % (kk, " + ".join(parts)))
    L.append("}")
    L.append("")
    # the same coefficients times the block scale of their output: s1 for
    # TT, TR, G and s3 for RR, QQ, H (the radius powers of scale_block)
    L.append("// rsd_real_epi_coef with each coefficient times the scale of its output:")
    L.append("// s3 for RR, QQ and H (outputs 6-11, 15-29, 45-59), s1 for the others.")
    L.append("template <typename T>")
    L.append("__host__ __device__ inline void rsd_real_epi_coef_scaled(T ai, T aj, T phix, T s1, T s3, T* __restrict__ c) {")
    L.append("  rsd_real_epi_coef<T>(ai, aj, phix, c);")
    for kk, (q, m) in enumerate(keys):
        a3 = (6 <= q < 12) or (15 <= q < 30) or q >= 45
        L.append("  c[%d] *= %s;" % (kk, "s3" if a3 else "s1"))
    L.append("}")
    L.append("")
    L.append("// Output q alone (q a compile-time constant after unrolling): the sum over")
    L.append("// its table entries of c[k] acc[m_k].")
    L.append("// With NP > 1 only the moments of part P (rsd_mom_part).")
    L.append("template <typename CT, typename A, typename O, int NP = 1, int P = 0>")
    L.append("__device__ __forceinline__ O rsd_real_epi_row(int q, const A* __restrict__ acc, const CT* __restrict__ c) {")
    L.append("  O o = O(0);")
    L.append("  switch (q) {")
    byq = {}
    for kk, (q, m) in enumerate(keys):
        byq.setdefault(q, []).append((kk, m))
    for q in range(60):
        if q not in byq:
            continue
        L.append("    case %d:" % q)
        for kk, m in byq[q]:
            L.append("      if constexpr (rsd_mom_part(%d, NP) == P) o = fma(c[%d], acc[%d], o);" % (m, kk, m))
        L.append("      break;")
    L.append("    default:")
    L.append("      break;")
    L.append("  }")
    L.append("  return o;")
    L.append("}")
    L.append("")
    L.append("// out[q] = sum over the table entries of output q of c[k] acc[m_k]; CT, A and O")
    L.append("// are the coefficient, moment and output types (fma(CT, A, O) -> O).")
    L.append("template <typename CT, typename A, typename O>")
    L.append("__device__ __forceinline__ void rsd_real_epi_apply(const A* __restrict__ acc, const CT* __restrict__ c,")
    L.append("                                                   O* __restrict__ out) {")
    L.append("#pragma unroll")
    L.append("  for (int q = 0; q < 60; q++) out[q] = O(0);")
    for kk, (q, m) in enumerate(keys):
        L.append("  out[%d] = fma(c[%d], acc[%d], out[%d]);" % (q, kk, m, q))
    L.append("}")
    L.append("")
    # ---- reciprocal-space weights: w[m] = S k^alpha for each moment
    for tag, mom, dec in (("kcos", mom_c, dec_c), ("ksin", mom_s, dec_s)):
        L.append("// Per-k weights of the %s moments: w[m] = g_m(S, lam) * k^alpha." % tag)
        L.append("template <typename T>")
        L.append("__device__ __host__ __forceinline__ void rsd_%s_weights(T k0, T k1, T k2, T S, T lam, T* __restrict__ w) {" % tag)
        L.append("  (void)lam;")
        monos = sorted({xm for _, xm in mom if sum(xm) > 0}, key=lambda t: (sum(t), t))
        have = emit_monomials(L, monos, "k", "T")
        for m, (g, xm) in enumerate(mom):
            mono = have.get(xm) if sum(xm) > 0 else None
            ge = sp.ccode(g)
            L.append("  w[%d] = (%s)%s;" % (m, ge, (" * " + mono) if mono else ""))
        L.append("}")
        L.append("")
        epilogue("rsd_%s_epilogue" % tag, dec, "Reciprocal-space (%s part) pair block from the moments." % tag)
    src = "\n".join(L) + "\n"
    with open(OUT, "w") as fp:
        fp.write(src)
    print("wrote %s (%.1fs)" % (OUT, time.time() - t0), file=sys.stderr)


if __name__ == "__main__":
    gen()
