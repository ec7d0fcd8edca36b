"""Generator of the straight-line FP64 sphere interaction code (``csrc/gen_sphere.cuh``).

Mathematics (restated from the reference's Eshelby sphere potentials,
integratorElastic3DHelper.cpp:41-750 and :2394-2624).  For a sphere of radius a
centred at the origin and a field point x, with u = |x|^2 / 2:

* J_m(u) = 4 pi a^3 / ((2m+1) (a^2+lambda)^(m+1/2)), lambda = max(|x|^2 - a^2, 0).
  Outside the sphere dJ_m/du = -(2m+3) J_{m+1}; inside J_m is constant.
* V_n = J_n / 2 - u J_{n+1}; dV_n/du = -J_{n+1} in both regions.
* Every potential of the source orders 0/1/2 is a polynomial prefactor times a
  radial function of u:
      phi    = V0                      psi    = Psi0,  dPsi0/du = V0 - a^2 V1
      phi_p  = a^2 x_p V1              psi_p  = a^2 x_p Q,  dQ/du = V1 - a^2 V2
      phi_pq = a^4 x_p x_q V2 - a^2 d_pq Q
      psi_pq = a^4 x_p x_q P - a^2 d_pq S,  dP/du = V2 - a^2 V3,
                                             d^2S/du^2 = V1 - 2 a^2 V2 + a^4 V3
  (only derivatives of order >= 1 of Psi0, Q, P, S are ever used).
* For a radial F(u), d^k F / dx_{i1..ik} = sum_j F^{(k-j)}(u) S_{k,j}(x), where
  S_{k,j} sums, over the ways of pairing j couples of equal indices, the product
  of x over the unpaired indices.

So one pair needs only the u-derivative "ladders" of J_m (the one place where
inside and outside differ) and polynomials in x.  The generator expands, at
concrete indices, the Eshelby-type tensors
  D(i,j,k,l;P;R) = [psi_P,klijR - 2 nu d_kl phi_P,ijR
                    - (1-nu)(phi_P,kjR d_il + phi_P,kiR d_jl + phi_P,ljR d_ik + phi_P,liR d_jk)]
                   / (8 pi (1-nu))                                          (:2394-2554)
and the per-pair blocks built from them, memoising every intermediate so each
is emitted once.  The emitted code is plain C++ with an ``IBEM_HD`` qualifier,
compiled for sm_103a by nvcc and, for checking, by the host compiler.
"""
from __future__ import annotations

import itertools
import math
import os
import re
from collections import OrderedDict

HERE = os.path.dirname(os.path.abspath(__file__))

# radial functions: name -> (kind, data)
#   ("J", m)                  J_m
#   ("V", n)                  V_n
#   ("LIN", [(coef_expr, fname)])  linear combination (coef in terms of a2)
#   ("PRIM", fname)           primitive: F' = fname
RADIAL = {
    "V0": ("V", 0), "V1": ("V", 1), "V2": ("V", 2), "V3": ("V", 3),
    "W0": ("LIN", [("1.0", "V0"), ("-a2", "V1")]),
    "W1": ("LIN", [("1.0", "V1"), ("-a2", "V2")]),
    "W2": ("LIN", [("1.0", "V2"), ("-a2", "V3")]),
    "UU": ("LIN", [("1.0", "V1"), ("-2.0*a2", "V2"), ("a4", "V3")]),
    "PSI0": ("PRIM", "W0"),
    "Q": ("PRIM", "W1"),
    "P": ("PRIM", "W2"),
    "S1": ("PRIM", "UU"),
    "S": ("PRIM", "S1"),
}


class Emitter:
    """Collects straight-line statements with memoisation by key."""

    def __init__(self, prefix: str = "t"):
        self.lines: list[str] = []
        self.memo: dict = {}
        self.n = 0
        self.prefix = prefix

    def new(self, expr: str, key=None) -> str:
        if key is not None and key in self.memo:
            return self.memo[key]
        name = f"{self.prefix}{self.n}"
        self.n += 1
        self.lines.append(f"const double {name} = {expr};")
        if key is not None:
            self.memo[key] = name
        return name


class Ladders:
    """u-derivative ladders of the radial functions (emitted lazily)."""

    def __init__(self, em: Emitter, maxk: int):
        self.em = em
        self.maxk = maxk
        self.jmax = 0
        self.used_j = set()

    def J(self, m: int, k: int) -> str:
        # k-th u-derivative of J_m: outside (-1)^k (2m+3)(2m+5)..(2m+2k+1) J_{m+k}; inside 0 (k>=1)
        if k == 0:
            self.used_j.add(m)
            return f"Jv[{m}]"
        self.used_j.add(m + k)
        c = 1
        for t in range(k):
            c *= (2 * m + 3 + 2 * t)
        c *= (-1) ** k
        return self.em.new(f"ext * ({float(c)!r} * Jv[{m + k}])", key=("J", m, k))

    def F(self, name: str, k: int) -> str:
        """k-th u-derivative of the radial function `name` (returns a symbol or '0.0')."""
        if name in ("RINV", "RLEN"):
            # r^s with s = -1 (1/R) or +1 (R): d^k/du^k r^s = s (s-2) .. (s-2k+2) r^(s-2k)
            sp = -1 if name == "RINV" else 1
            c = 1
            for t in range(k):
                c *= (sp - 2 * t)
            key = ("F", name, k)
            if key in self.em.memo:
                return self.em.memo[key]
            # r^(s-2k) = ir^(2k-s)
            e = 2 * k - sp
            powname = self.ipow(e)
            return self.em.new(f"{float(c)!r} * {powname}", key=key)
        kind, d = RADIAL[name]
        key = ("F", name, k)
        if key in self.em.memo:
            return self.em.memo[key]
        if kind == "J":
            return self.J(d, k)
        if kind == "V":
            n = d
            if k == 0:
                self.used_j.update([n, n + 1])
                return self.em.new(f"0.5 * Jv[{n}] - u * Jv[{n + 1}]", key=key)
            j = self.J(n + 1, k - 1)
            return self.em.new(f"-({j})", key=key)
        if kind == "LIN":
            parts = []
            for coef, f in d:
                s = self.F(f, k)
                parts.append(f"({coef}) * {s}")
            return self.em.new(" + ".join(parts), key=key)
        if kind == "PRIM":
            if k == 0:
                raise ValueError(f"value of primitive {name} requested")
            return self.F(d, k - 1)
        raise KeyError(name)


def _ipow_method(self, e: int) -> str:
    """1/r^e (e >= -1) as a memoised symbol."""
    if e == -1:
        return "rr"
    if e == 0:
        return "1.0"
    if e == 1:
        return "ir"
    key = ("ipow", e)
    if key in self.em.memo:
        return self.em.memo[key]
    half = self.ipow(e // 2)
    if e % 2 == 0:
        return self.em.new(f"{half} * {half}", key=key)
    return self.em.new(f"{half} * {half} * ir", key=key)


Ladders.ipow = _ipow_method


def multiset_key(K):
    return tuple(sorted(K))


class Tensors:
    """Symmetric derivatives of radial functions and the potential components."""

    def __init__(self, em: Emitter, lad: Ladders):
        self.em = em
        self.lad = lad

    def sym(self, fname: str, K) -> str:
        """d^|K| F / dx_K for radial F at the concrete multiset K."""
        K = multiset_key(K)
        key = ("sym", fname, K)
        if key in self.em.memo:
            return self.em.memo[key]
        k = len(K)
        cnt = [K.count(i) for i in range(3)]
        terms = []
        for j0 in range(cnt[0] // 2 + 1):
            for j1 in range(cnt[1] // 2 + 1):
                for j2 in range(cnt[2] // 2 + 1):
                    js = (j0, j1, j2)
                    j = sum(js)
                    mult = 1
                    for i in range(3):
                        mult *= math.comb(cnt[i], 2 * js[i]) * double_fact(2 * js[i] - 1)
                    xs = []
                    for i in range(3):
                        xs += [f"x{i}"] * (cnt[i] - 2 * js[i])
                    lad = self.lad.F(fname, k - j)
                    mono = self.mono(xs)
                    t = lad if mono == "1.0" else f"{lad} * {mono}"
                    if mult != 1:
                        t = f"{float(mult)!r} * {t}"
                    terms.append(t)
        return self.em.new(" + ".join(terms), key=key)

    def mono(self, xs) -> str:
        if not xs:
            return "1.0"
        xs = sorted(xs)
        key = ("mono", tuple(xs))
        if key in self.em.memo:
            return self.em.memo[key]
        if len(xs) == 1:
            return xs[0]
        # build from a shorter monomial
        prev = self.mono(xs[:-1])
        return self.em.new(f"{prev} * {xs[-1]}", key=key)

    # x_{P} F,K Leibniz expansion: prefactor indices pre (list), F radial
    def xpoly_deriv(self, pre, fname, K) -> str:
        """d_K [ prod_{c in pre} x_c  F(u) ] at concrete indices."""
        K = list(K)
        key = ("xpd", tuple(sorted(pre)), fname, multiset_key(K))
        if key in self.em.memo:
            return self.em.memo[key]
        terms = []
        # assign to each prefactor slot either nothing or one distinct K-slot with equal index
        slots = list(range(len(K)))

        def rec(pi, used, factor_x, count):
            if pi == len(pre):
                rest = [K[s] for s in slots if s not in used]
                terms.append((tuple(sorted(factor_x)), tuple(sorted(rest)), count))
                return
            c = pre[pi]
            rec(pi + 1, used, factor_x + [f"x{c}"], count)
            for s in slots:
                if s not in used and K[s] == c:
                    rec(pi + 1, used | {s}, factor_x, count)

        rec(0, frozenset(), [], 1)
        # combine identical terms
        acc = OrderedDict()
        for fx, rest, cnt in terms:
            acc[(fx, rest)] = acc.get((fx, rest), 0) + cnt
        parts = []
        for (fx, rest), cnt in acc.items():
            d = self.sym(fname, rest)
            mono = self.mono(list(fx))
            t = d if mono == "1.0" else f"{mono} * {d}"
            if cnt != 1:
                t = f"{float(cnt)!r} * {t}"
            parts.append(t)
        return self.em.new(" + ".join(parts), key=key)

    def phi(self, order, P, K) -> str:
        K = list(K)
        key = ("phi", order, tuple(P), multiset_key(K))
        if key in self.em.memo:
            return self.em.memo[key]
        if order == 0:
            v = self.sym("V0", K)
        elif order == 1:
            v = f"a2 * {self.xpoly_deriv([P[0]], 'V1', K)}"
        else:
            p, q = P
            v = f"a4 * {self.xpoly_deriv([p, q], 'V2', K)}"
            if p == q:
                v += f" - a2 * {self.sym('Q', K)}"
        return self.em.new(v, key=key)

    def psi(self, order, P, K) -> str:
        K = list(K)
        key = ("psi", order, tuple(P), multiset_key(K))
        if key in self.em.memo:
            return self.em.memo[key]
        if order == 0:
            v = self.sym("PSI0", K)
        elif order == 1:
            v = f"a2 * {self.xpoly_deriv([P[0]], 'Q', K)}"
        else:
            p, q = P
            v = f"a4 * {self.xpoly_deriv([p, q], 'P', K)}"
            if p == q:
                v += f" - a2 * {self.sym('S', K)}"
        return self.em.new(v, key=key)


def double_fact(n: int) -> int:
    r = 1
    while n > 1:
        r *= n
        n -= 2
    return r


SYM_PAIRS = [(i, j) for i in range(3) for j in range(i, 3)]


def units(layout: int):
    """Per-particle unknowns (order, i, j, P, column multiplier), reference order
    (configElastic3D.cpp:160-195); 60 stores order-2 coefficients for p <= q only."""
    u = [(0, i, j, (), 1.0) for (i, j) in SYM_PAIRS]
    u += [(1, i, j, (p,), 1.0) for (i, j) in SYM_PAIRS for p in range(3)]
    if layout == 24:
        return u
    for (i, j) in SYM_PAIRS:
        for p in range(3):
            for q in range(p if layout == 60 else 0, 3):
                u.append((2, i, j, (p, q), 2.0 if (layout == 60 and p != q) else 1.0))
    return u


MAPF = [[1, 2, 2], [0, 1, 2], [0, 0, 1]]


def d_parts(T: Tensors, order, P, i, j, k, l, R):
    """Return (psi, phi_ij, F4) symbols for D(i,j,k,l;P;R) without the material factor:
    D = c [psi - 2 nu d_kl phi_ij - (1-nu) F4]."""
    R = list(R)
    psi = T.psi(order, P, [k, l, i, j] + R)
    phi_ij = T.phi(order, P, [i, j] + R) if k == l else None
    f4 = []
    if i == l:
        f4.append(T.phi(order, P, [k, j] + R))
    if j == l:
        f4.append(T.phi(order, P, [k, i] + R))
    if i == k:
        f4.append(T.phi(order, P, [l, j] + R))
    if j == k:
        f4.append(T.phi(order, P, [l, i] + R))
    return psi, phi_ij, f4


def gen_block_function(name: str, layout: int, rows_sel, cols_sel) -> str:
    """Emit a device function computing the sub-block (rows_sel x cols_sel) of the
    per-pair inclusion block (integratorElastic3D.cpp:341-682):
        entry = map[m][n] * mult * fac * ( -sum_kl (C0-C1)_ijkl D(k,l,m,n;P;R) )
    The isotropic contrast turns the sum into
        -(dlam d_ij Tr + 2 dmu D_ij),  Tr = sum_k D(k,k,m,n)
    computed from the same components.  The self term (s == h) is added by the caller.
    Values are passed to `sink(row, col, v)` column by column."""
    U = units(layout)
    em = Emitter()
    lad = Ladders(em, 8)
    T = Tensors(em, lad)
    body = []
    for cc in cols_sel:
        co, m, n, P, mult = U[cc]
        for rr in rows_sel:
            ro, i, j, R, _ = U[rr]
            fac = 0.5 if ro == 2 else 1.0
            # 2 dmu D_ij
            psi, phi_ij, f4 = d_parts(T, co, P, i, j, m, n, R)
            # -(dlam d_ij Tr + 2 dmu D_ij); Tr = sum_k D(k,k,m,n)
            tr_terms = []
            if i == j:
                for kk in range(3):
                    ps, ph, f = d_parts(T, co, P, kk, kk, m, n, R)
                    tr_terms.append((ps, ph, f))
            expr = []
            # D_ij
            dij = em.new(_dexpr(psi, phi_ij, f4))
            expr.append(f"kmu * {dij}")
            if tr_terms:
                tr = em.new(" + ".join(_dexpr(*t) for t in tr_terms))
                expr.append(f"klam * {tr}")
            scale = MAPF[m][n] * mult * fac
            v = em.new(f"{float(scale)!r} * ({' + '.join(expr)})")
            em.lines.append(f"sink({rr}, {cc}, {v});")
    return _wrap(name, em, lad, body)


def _dexpr(psi, phi_ij, f4):
    """[psi - 2 nu d_kl phi_ij - (1-nu) F4] with nu-dependent constants tn2 = 2 nu, tn1 = 1 - nu."""
    s = psi
    if phi_ij is not None:
        s += f" - tn2 * {phi_ij}"
    if f4:
        s += f" - tn1 * ({' + '.join(f4)})"
    return f"({s})"


def _wrap(name, em: Emitter, lad: Ladders, body) -> str:
    jmax = max(lad.used_j) if lad.used_j else 0
    out = []
    out.append("template <class Sink>")
    out.append(f"IBEM_HD IBEM_INLINE void {name}(const double x0, const double x1, const double x2,")
    out.append("    const double a, const SphMat& mc, Sink& sink) {")
    out.append("  const double a2 = a * a; const double a4 = a2 * a2;")
    out.append("  const double u = 0.5 * (x0 * x0 + x1 * x1 + x2 * x2);")
    out.append("  const double lam = 2.0 * u - a2;")
    out.append("  const double ext = lam > 0.0 ? 1.0 : 0.0;")
    out.append("  const double rho2 = lam > 0.0 ? a2 + lam : a2;")
    out.append(f"  double Jv[{jmax + 1}];")
    out.append("  {")
    out.append("    // J_m = 4 pi a^3 / ((2m+1) rho^(2m+1)),  rho^2 = a^2 + lambda")
    out.append("    const double irho2 = 1.0 / rho2;")
    out.append("    double pw = 4.0 * IBEM_PI * a * a2 / sqrt(rho2);")
    out.append(f"    for (int m = 0; m <= {jmax}; ++m) {{ Jv[m] = pw / (2 * m + 1); pw *= irho2; }}")
    out.append("  }")
    out.append("  const double kmu = mc.kmu, klam = mc.klam, tn1 = mc.tn1, tn2 = mc.tn2;")
    out.append("  (void)kmu; (void)klam; (void)tn1; (void)tn2; (void)a4;")
    for ln in em.lines:
        out.append("  " + ln)
    for ln in body:
        out.append("  " + ln)
    out.append("}")
    return "\n".join(out)


def gen_field_function(name: str, layout: int) -> str:
    """Strain at a field point from one particle's eigenstrain (postprocessor,
    postProcessorElastic3D.cpp:407-470):  e_ij += sum_cols D(i,j,m,n;P) map mult E."""
    U = units(layout)
    em = Emitter()
    lad = Ladders(em, 8)
    T = Tensors(em, lad)
    body = []
    for r, (i, j) in enumerate(SYM_PAIRS):
        terms = []
        for cc, (co, m, n, P, mult) in enumerate(U):
            psi, phi_ij, f4 = d_parts(T, co, P, i, j, m, n, [])
            d = em.new(_dexpr(psi, phi_ij, f4))
            terms.append(f"{float(MAPF[m][n] * mult)!r} * {d} * E[{cc}]")
        v = em.new(" + ".join(terms))
        body.append(f"e[{r}] += kd * {v};")
    src = _wrap(name, em, lad, body)
    src = src.replace("template <class Sink>\n", "")
    src = src.replace("const SphMat& mc, Sink& sink) {",
                      "const SphMat& mc, const double* E, double* e) {\n  const double kd = mc.kd;")
    return src


def gen_node_function(name: str, layout: int) -> str:
    """Boundary-node rows of one particle's columns: get_addu/1/2
    (integratorElastic3D.cpp:30-133) with IGreen_01/11/21 (:2604-2624):
      H(3j+q, col) = map[m][n] mult sum_{jj,ll} C0(jj,ll,m,n) IGreen(q,jj,P,ll)
    IGreen(i,j,P,l) = (d_ij phi_P,l + d_il phi_P,j)/(8 pi mu0) - psi_P,ijl / (16 pi mu0 (1-nu0)).
    With isotropic C0: sum_{jj,ll} C0(jj,ll,m,n) IG(q,jj,ll) = lam0 d_mn sum_k IG(q,k,k)
                                                             + 2 mu0 IG(q,m,n) (IG sym in jj,ll)."""
    U = units(layout)
    em = Emitter()
    lad = Ladders(em, 8)
    T = Tensors(em, lad)
    body = []

    def ig(order, P, i, j, l):
        parts = []
        if i == j:
            parts.append(f"g1 * {T.phi(order, P, [l])}")
        if i == l:
            parts.append(f"g1 * {T.phi(order, P, [j])}")
        parts.append(f"-g2 * {T.psi(order, P, [i, j, l])}")
        return em.new(" + ".join(parts))

    for cc, (co, m, n, P, mult) in enumerate(U):
        for q in range(3):
            terms = [f"twomu0 * {ig(co, P, q, m, n)}"]
            if m == n:
                tr = " + ".join(ig(co, P, q, k, k) for k in range(3))
                terms.append(f"lam0 * ({tr})")
            v = em.new(f"{float(MAPF[m][n] * mult)!r} * ({' + '.join(terms)})")
            em.lines.append(f"sink({q}, {cc}, {v});")
    src = _wrap(name, em, lad, body)
    src = src.replace("const double kmu = mc.kmu, klam = mc.klam, tn1 = mc.tn1, tn2 = mc.tn2;",
                      "const double g1 = mc.g1, g2 = mc.g2, twomu0 = mc.twomu0, lam0 = mc.lam0;")
    src = src.replace("(void)kmu; (void)klam; (void)tn1; (void)tn2;", "(void)g1; (void)g2;")
    return src


FILE_HEAD = """// GENERATED by ibemproject_gb300/codegen.py -- do not edit by hand.
// Straight-line FP64 evaluation of the sphere interaction blocks of the 3D elastic
// iBEM path (restating integratorElastic3DHelper.cpp:41-750, :2394-2624 and
// integratorElastic3D.cpp:30-682 of the reference); see codegen.py for the derivation.
#pragma once
#include "gen_sphere_common.cuh"
"""

def gen_self_function(name: str, layout: int) -> str:
    """Self term of the diagonal pair block (s == h): map[m][n] C0_ijmn d(P,R) for
    rows and columns of equal order (integratorElastic3D.cpp:392-397, 509-523, 634-650).
    Compact order-2 rows/columns (p<=q) match only when (p,q) == (r,z)."""
    U = units(layout)
    body = []
    for rr, (ro, i, j, R, _) in enumerate(U):
        for cc, (co, m, n, P, _) in enumerate(U):
            if ro != co or tuple(R) != tuple(P):
                continue
            lam = 1 if (i == j and m == n) else 0
            mu = (1 if (i == m and j == n) else 0) + (1 if (i == n and j == m) else 0)
            if not lam and not mu:
                continue
            terms = []
            if lam:
                terms.append("mc.lam0")
            if mu:
                terms.append(f"{float(mu)!r} * mc.mu0")
            body.append(f"  sink({rr}, {cc}, {float(MAPF[m][n])!r} * ({' + '.join(terms)}));")
    return "\n".join(["template <class Sink>",
                      f"IBEM_HD IBEM_INLINE void {name}(const SphMat& mc, Sink& sink) {{"]
                     + body + ["}"])


def gen_bem_stress_function(name: str, order: int, W, dofs) -> str:
    """Stress (order 0) or its 1st/2nd gradient (W the derivative indices) at a point
    from a unit boundary displacement (Dsu) and traction (Dst) at a Gauss point,
    x = Gauss point - point: get_for_stress_BEM / BEM1 / BEM2 (BEMBuilderElastic3D.cpp:
    780-980, 429-672, 37-322) and get_for_stress_BEM_post (postProcessorElastic3D.cpp:
    32-114), with the contrast (dlam, dmu) a run-time argument.  Kelvin solution
    (integratorElastic3DHelper.cpp:2559-2593):  G_ij,K = A d_ij (1/R),K - B R,ijK,
    A = 1/(4 pi mu0), B = 1/(16 pi mu0 (1-nu0)).  Rows (k<=l) for the dof list `dofs`;
    Dsu[t*3+n], Dst[t*3+n] are written for n in dofs."""
    em = Emitter()
    lad = Ladders(em, 8)
    T = Tensors(em, lad)
    W = list(W)
    su = 1.0 if order % 2 == 0 else -1.0
    st = -su

    def G(i, j, K):
        K = list(K)
        key = ("G", i, j, multiset_key(K))
        if key in em.memo:
            return em.memo[key]
        parts = []
        if i == j:
            parts.append(f"kA * {T.sym('RINV', K)}")
        parts.append(f"-kB * {T.sym('RLEN', [i, j] + K)}")
        return em.new(" + ".join(parts), key=key)

    def TG(i, j):
        return em.new(" + ".join(G(l, i, [l, j] + W) for l in range(3)), key=("TG", i, j))

    body = []
    for t, (k, l) in enumerate(SYM_PAIRS):
        for n in dofs:
            # Dst
            parts = []
            if k == l:
                tg1 = em.new(" + ".join(G(n, i, [i] + W) for i in range(3)), key=("TG1", n))
                parts.append(f"dlam * {tg1}")
            parts.append(f"dmu * ({G(n, k, [l] + W)} + {G(n, l, [k] + W)})")
            body.append(f"Dst[{t * 3 + n}] = {st!r} * ({' + '.join(parts)});")
            # Dsu
            mparts = []
            for m in range(3):
                inner = []
                if k == l:
                    key = ("sgm", m, n)
                    if key not in em.memo:
                        sp = []
                        for i in range(3):
                            if m == n:
                                sp.append(f"lam0 * {TG(i, i)}")
                            if order == 0:
                                sp.append(f"2.0 * mu0 * {G(m, i, [n, i] + W)}")
                            else:
                                sp.append(f"mu0 * {G(m, i, [n, i] + W)}")
                                sp.append(f"mu0 * {G(n, i, [m, i] + W)}")
                        em.new(" + ".join(sp), key=key)
                    inner.append(f"dlam * {em.memo[key]}")
                dm = []
                if m == n:
                    dm.append(f"lam0 * ({TG(k, l)} + {TG(l, k)})")
                dm.append("mu0 * (" + " + ".join([G(m, k, [n, l] + W), G(m, l, [n, k] + W),
                                                  G(n, k, [m, l] + W), G(n, l, [m, k] + W)]) + ")")
                inner.append(f"dmu * ({' + '.join(dm)})")
                mparts.append(f"({' + '.join(inner)}) * nv{m}")
            body.append(f"Dsu[{t * 3 + n}] = {su!r} * ({' + '.join(mparts)});")
    out = ["IBEM_HD IBEM_INLINE void " + name +
           "(const double x0, const double x1, const double x2, const double nv0, const double nv1,",
           "    const double nv2, const BemMat& bm, const double dlam, const double dmu, double* Dsu,",
           "    double* Dst) {",
           "  const double u = 0.5 * (x0 * x0 + x1 * x1 + x2 * x2);",
           "  const double rr = sqrt(2.0 * u);",
           "  const double ir = 1.0 / rr;",
           "  const double kA = bm.kA, kB = bm.kB, lam0 = bm.lam0, mu0 = bm.mu0;",
           "  (void)kA; (void)kB; (void)lam0; (void)mu0; (void)rr;"]
    out += ["  " + ln for ln in em.lines]
    out += ["  " + ln for ln in body]
    out.append("}")
    return "\n".join(out)


HEADER = """// GENERATED by ibemproject_gb300/codegen.py -- do not edit by hand.
// Material constants and qualifiers shared by the generated sphere code.
#pragma once
#include <math.h>
#ifndef IBEM_HD
#ifdef __CUDACC__
#define IBEM_HD __host__ __device__
#define IBEM_INLINE __forceinline__
#else
#define IBEM_HD
#define IBEM_INLINE inline
#endif
#endif
#ifndef IBEM_PI
#define IBEM_PI 3.141592653589793
#endif

// Material constants folded for the generated code (filled by sph_mat_init).
struct SphMat {
  double kmu, klam;   // -2 dmu c, -dlam c   with c = 1 / (8 pi (1 - nu0))
  double tn1, tn2;    // 1 - nu0, 2 nu0
  double kd;          // c (field sums use D itself)
  double g1, g2;      // 1 / (8 pi mu0), 1 / (16 pi mu0 (1 - nu0))
  double twomu0, lam0, mu0;
  double dlam, dmu;
};

// Kelvin-solution constants of the boundary kernels.
struct BemMat {
  double kA, kB;      // 1 / (4 pi mu0), 1 / (16 pi mu0 (1 - nu0))
  double lam0, mu0;
  double dlam, dmu;   // (C0 - C1) contrast
};

IBEM_HD inline BemMat bem_mat_init(double E0, double nu0, double E1, double nu1) {
  BemMat m;
  const double mu0 = E0 / (2.0 * (1.0 + nu0));
  const double mu1 = E1 / (2.0 * (1.0 + nu1));
  m.lam0 = 2.0 * mu0 * nu0 / (1.0 - 2.0 * nu0);
  m.mu0 = mu0;
  m.kA = 1.0 / (4.0 * IBEM_PI * mu0);
  m.kB = 1.0 / (16.0 * IBEM_PI * mu0 * (1.0 - nu0));
  m.dlam = m.lam0 - 2.0 * mu1 * nu1 / (1.0 - 2.0 * nu1);
  m.dmu = mu0 - mu1;
  return m;
}

IBEM_HD inline SphMat sph_mat_init(double E0, double nu0, double E1, double nu1) {
  SphMat m;
  const double mu0 = E0 / (2.0 * (1.0 + nu0));
  const double mu1 = E1 / (2.0 * (1.0 + nu1));
  const double lam0 = 2.0 * mu0 * nu0 / (1.0 - 2.0 * nu0);
  const double lam1 = 2.0 * mu1 * nu1 / (1.0 - 2.0 * nu1);
  const double c = 1.0 / (8.0 * IBEM_PI * (1.0 - nu0));
  m.dlam = lam0 - lam1;
  m.dmu = mu0 - mu1;
  m.kmu = -2.0 * m.dmu * c;
  m.klam = -m.dlam * c;
  m.tn1 = 1.0 - nu0;
  m.tn2 = 2.0 * nu0;
  m.kd = c;
  m.g1 = 1.0 / (8.0 * IBEM_PI * mu0);
  m.g2 = 1.0 / (16.0 * IBEM_PI * mu0 * (1.0 - nu0));
  m.twomu0 = 2.0 * mu0;
  m.lam0 = lam0;
  m.mu0 = mu0;
  return m;
}
"""


_F32_LIT = re.compile(r"(?<![\w.])(\d+\.\d*(?:[eE][+-]?\d+)?)(?![\w.])")

F32_HEAD = """// GENERATED by ibemproject_gb300/codegen.py -- do not edit by hand.
// FP32 variant of the layout-24 sphere blocks for the matrix-free solver, which calls
// them in coordinates scaled by the source radius (a = 1), so that every intermediate is
// O(1) in single precision.  Same derivation as gen_sphere24.cuh.
#pragma once
#include "gen_sphere_common.cuh"

// Dimensionless material constants of the FP32 blocks (sph_matf_init: SphMat / mu0).
struct SphMatF {
  float kmu, klam, tn1, tn2;  // as SphMat, contrast terms divided by mu0
  float lam0, mu0;            // C0 / mu0 (self term): lam0 / mu0 and 1
};

IBEM_HD inline SphMatF sph_matf_init(const SphMat& m) {
  SphMatF f;
  const double s = 1.0 / m.mu0;
  f.kmu = (float)(m.kmu * s);
  f.klam = (float)(m.klam * s);
  f.tn1 = (float)m.tn1;
  f.tn2 = (float)m.tn2;
  f.lam0 = (float)(m.lam0 * s);
  f.mu0 = 1.0f;
  return f;
}
"""


F60_HEAD = """// GENERATED by ibemproject_gb300/codegen.py -- do not edit by hand.
// FP32 variant of the layout-60 sphere blocks for the matrix-free solver of quadratic
// realisations, called in coordinates scaled by the source radius (a = 1).  Same derivation
// as gen_sphere60.cuh.
#pragma once
#include "gen_sphere24_f32.cuh"   // SphMatF
"""


def to_f32(src: str, old_name: str, new_name: str) -> str:
    """Single-precision copy of a generated block function: the same straight-line
    arithmetic with float operands and literals."""
    out = src.replace(old_name + "(", new_name + "(")
    out = out.replace("const SphMat& mc", "const SphMatF& mc")
    out = out.replace("const double", "const float").replace("double Jv[", "float Jv[")
    out = out.replace("double pw", "float pw")
    out = out.replace("sqrt(", "sqrtf(").replace("IBEM_PI", "3.14159265358979f")
    out = _F32_LIT.sub(lambda m: m.group(1) + "f", out)
    return out


def generate(out_dir: str | None = None) -> dict:
    out_dir = out_dir or os.path.join(HERE, "csrc")
    files = {}
    # layout 24: blocks split by column order (rows all)
    files["gen_sphere_common.cuh"] = HEADER
    parts = [FILE_HEAD]
    U24 = units(24)
    for co in range(2):
        cols = [c for c in range(24) if U24[c][0] == co]
        for ro in range(2):
            rows = [r for r in range(24) if U24[r][0] == ro]
            parts.append(gen_block_function(f"sph_block24_c{co}_r{ro}", 24, rows, cols))
    parts.append(gen_field_function("sph_field24", 24))
    parts.append(gen_node_function("sph_node24", 24))
    parts.append(gen_self_function("sph_self24", 24))
    files["gen_sphere24.cuh"] = "\n\n".join(parts) + "\n"
    fparts = [F32_HEAD]
    for co in range(2):
        for ro in range(2):
            nm = f"sph_block24_c{co}_r{ro}"
            fparts.append(to_f32(parts[1 + 2 * co + ro], nm, nm.replace("block24", "block24f")))
    fparts.append(to_f32(gen_self_function("sph_self24", 24), "sph_self24", "sph_self24f"))
    files["gen_sphere24_f32.cuh"] = "\n\n".join(fparts) + "\n"
    for lay in (78, 60):
        U = units(lay)
        parts = [FILE_HEAD]
        for co in range(3):
            cols = [c for c in range(len(U)) if U[c][0] == co]
            for ro in range(3):
                rows = [r for r in range(len(U)) if U[r][0] == ro]
                parts.append(gen_block_function(f"sph_block{lay}_c{co}_r{ro}", lay, rows, cols))
        nblk = len(parts) - 1
        parts.append(gen_field_function(f"sph_field{lay}", lay))
        parts.append(gen_node_function(f"sph_node{lay}", lay))
        parts.append(gen_self_function(f"sph_self{lay}", lay))
        files[f"gen_sphere{lay}.cuh"] = "\n\n".join(parts) + "\n"
        if lay == 60:
            # FP32 blocks of the layout-60 matrix-free products (scaled coordinates, a = 1): the
            # large sub-blocks split into groups of 6 columns (one symmetric pair (m, n) each),
            # so that each kernel's straight-line code keeps its values in registers: the
            # order-1 columns of the order-2 rows in 3 groups, the order-2 columns of the
            # order-1 and order-2 rows in 6
            fparts = [F60_HEAD]
            def add(name, ro, cols):
                src = gen_block_function(name, 60, [r for r in range(len(U)) if U[r][0] == ro], cols)
                fparts.append(to_f32(src, name, name.replace("block60", "block60f")))
            for ro in range(3):
                for co in range(3):
                    cols = [c for c in range(len(U)) if U[c][0] == co]
                    if co == 2 and ro >= 1:
                        for g, pr in enumerate(SYM_PAIRS):
                            add(f"sph_block60_c2g{g}_r{ro}", ro, [c for c in cols if (U[c][1], U[c][2]) == pr])
                    elif co == 1 and ro == 2:
                        for g in range(3):
                            prs = SYM_PAIRS[2 * g:2 * g + 2]
                            add(f"sph_block60_c1g{g}_r2", ro, [c for c in cols if (U[c][1], U[c][2]) in prs])
                    else:
                        add(f"sph_block60m_c{co}_r{ro}", ro, cols)
            fparts.append(to_f32(gen_self_function("sph_self60", 60), "sph_self60", "sph_self60f"))
            files["gen_sphere60_f32.cuh"] = "\n\n".join(fparts) + "\n"
    # boundary stress kernels: one function per (order, W tuple, dof) and the
    # post-processing variant (order 0, all dofs)
    parts = [FILE_HEAD]
    for o in range(3):
        Ws = [()] if o == 0 else ([(w,) for w in range(3)] if o == 1 else
                                  [(w, z) for w in range(3) for z in range(3)])
        for W in Ws:
            for n in range(3):
                wn = "".join(str(v) for v in W)
                parts.append(gen_bem_stress_function(f"bem_stress_o{o}_w{wn}_n{n}", o, W, [n]))
    parts.append(gen_bem_stress_function("bem_stress_post", 0, (), [0, 1, 2]))
    files["gen_bem.cuh"] = "\n\n".join(parts) + "\n"
    for fn, src in files.items():
        path = os.path.join(out_dir, fn)
        old = open(path).read() if os.path.exists(path) else None
        if old != src:
            with open(path, "w") as f:
                f.write(src)
    return files


if __name__ == "__main__":
    fs = generate()
    for k, v in fs.items():
        print(k, len(v.splitlines()), "lines")
