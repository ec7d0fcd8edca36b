"""Derivation of the material coefficients of csrc/bem_contract.cuh (run by hand: about two
minutes with sympy; nothing imports it).

The boundary part of the post-processor's stress at a sample point is
    sigma_kl = sum_n Dsu[kl][n] u_n + Dst[kl][n] t_n,
Dsu and Dst being the Kelvin stress kernels that codegen.gen_bem_stress_function emits
(G_ij = A d_ij / R - B R_,ij and its derivatives; order 0, dlam = lam0, dmu = mu0).  This
script builds the same expressions symbolically, contracts them with symbolic u and t, and
solves for the coefficients of the isotropic basis tensors (seven in x, n, u; three in x, t)
at points with rational |x|, then checks the identity at every other sample.  It prints the
coefficients that bem_post_coef hard-codes and the number of equations left unsatisfied (0).
"""
import sympy as sp, itertools, random


def main():
    x = sp.symbols('x0:3', real=True); nv = sp.symbols('n0:3', real=True); uu = sp.symbols('u0:3', real=True); tt = sp.symbols('t0:3', real=True)
    A, B, lam, mu = sp.symbols('A B lam mu', positive=True)
    R = sp.sqrt(sum(xi**2 for xi in x))
    d = lambda i, j: 1 if i == j else 0
    Rd = {}
    def dR(idx):
        key = tuple(sorted(idx))
        if key not in Rd:
            e = R
            for i in key: e = sp.diff(e, x[i])
            Rd[key] = e
        return Rd[key]
    def G(i, j, K):   # G_ij,K = A d_ij (1/R),K - B R,ijK
        e = -B * dR([i, j] + list(K))
        if i == j:
            f = 1 / R
            for k in K: f = sp.diff(f, x[k])
            e += A * f
        return e
    def TG(i, j): return sum(G(l, i, [l, j]) for l in range(3))
    dlam, dmu, lam0, mu0 = lam, mu, lam, mu
    su, st = 1, -1
    SYM = [(i, j) for i in range(3) for j in range(i, 3)]
    sig = []
    for (k, l) in SYM:
        s_t = 0; s_u = 0
        for n in range(3):
            parts = dmu * (G(n, k, [l]) + G(n, l, [k]))
            if k == l: parts += dlam * sum(G(n, i, [i]) for i in range(3))
            s_t += st * parts * tt[n]
            mp = 0
            for m in range(3):
                inner = 0
                if k == l:
                    sg = sum((lam0 * TG(i, i) if m == n else 0) + 2 * mu0 * G(m, i, [n, i]) for i in range(3))
                    inner += dlam * sg
                dm = (lam0 * (TG(k, l) + TG(l, k)) if m == n else 0) + mu0 * (G(m, k, [n, l]) + G(m, l, [n, k]) + G(n, k, [m, l]) + G(n, l, [m, k]))
                inner += dmu * dm
                mp += inner * nv[m]
            s_u += su * mp * uu[n]
        sig.append((s_u, s_t))
    # basis
    dot = lambda a, b: sum(a[i] * b[i] for i in range(3))
    def basis_u(k, l):
        xn, xu, nu_ = dot(x, nv), dot(x, uu), dot(nv, uu)
        return [d(k, l) * nu_ / R**3, d(k, l) * xn * xu / R**5, x[k] * x[l] * nu_ / R**5, x[k] * x[l] * xn * xu / R**7,
                (nv[k] * uu[l] + nv[l] * uu[k]) / R**3, (nv[k] * x[l] + x[k] * nv[l]) * xu / R**5,
                (uu[k] * x[l] + x[k] * uu[l]) * xn / R**5]
    def basis_t(k, l):
        xt = dot(x, tt)
        return [d(k, l) * xt / R**3, x[k] * x[l] * xt / R**5, (tt[k] * x[l] + x[k] * tt[l]) / R**3]
    cu = sp.symbols('cu0:7'); ct = sp.symbols('ct0:3')
    pts = [(1, 2, 2), (2, 3, 6), (1, 4, 8), (4, 4, 7), (2, 6, 9), (6, 2, 3), (-2, 1, 2), (3, -6, 2), (8, 4, -1), (-4, 7, 4)]
    random.seed(1)
    eqs_u, eqs_t = [], []
    for p in pts:
        for trial in range(2):
            vals = {x[i]: p[i] for i in range(3)}
            vals.update({nv[i]: random.randint(-5, 5) for i in range(3)})
            vals.update({uu[i]: random.randint(-5, 5) for i in range(3)})
            vals.update({tt[i]: random.randint(-5, 5) for i in range(3)})
            for c, (k, l) in enumerate(SYM):
                lhs_u = sp.nsimplify(sp.simplify(sig[c][0].subs(vals)))
                lhs_t = sp.nsimplify(sp.simplify(sig[c][1].subs(vals)))
                eqs_u.append(sp.expand(sum(cu[a] * sp.nsimplify(b.subs(vals)) for a, b in enumerate(basis_u(k, l))) - lhs_u))
                eqs_t.append(sp.expand(sum(ct[a] * sp.nsimplify(b.subs(vals)) for a, b in enumerate(basis_t(k, l))) - lhs_t))
    sol_u = sp.solve(eqs_u[:60], cu, dict=True)
    sol_t = sp.solve(eqs_t[:30], ct, dict=True)
    print("u:", sol_u)
    print("t:", sol_t)
    su_ = sol_u[0]; st_ = sol_t[0]
    # verify on all equations
    bad = [e for e in eqs_u if sp.simplify(e.subs(su_)) != 0] + [e for e in eqs_t if sp.simplify(e.subs(st_)) != 0]
    print("residual equations:", len(bad))


if __name__ == "__main__":
    main()
