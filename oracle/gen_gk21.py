"""Derive the 21-point Gauss-Kronrod rule on [-1, 1] from first principles.

Used to generate ``oracle/gk21_nodes.h`` (the CPU oracle's QAGS) and
``imfit_gb300/csrc/gk21_nodes.cuh`` (the device line-of-sight integrator).
Run: ``python oracle/gen_gk21.py``.

Method (Kronrod 1965; see also Laurie 1997, Math. Comp. 66:1133):
  * the 10 Gauss nodes are the roots of the Legendre polynomial P_10;
  * the 11 Kronrod nodes are the roots of the Stieltjes polynomial E_11,
    the monic degree-11 polynomial with  int_{-1}^{1} P_10(x) E_11(x) x^k dx = 0
    for k = 0..10.  E_11 is odd, so only its odd coefficients are unknown and
    only odd k give non-trivial conditions (5 equations, 5 unknowns);
  * the 21 Kronrod weights make the rule exact for all polynomials of degree
    <= 31; by symmetry it is enough to match the even moments x^0..x^20;
  * the Gauss weights are 2 / ((1 - x^2) P_10'(x)^2).
Everything is done in 60-digit arithmetic and printed with 17 significant
digits, which round-trips IEEE doubles.

The output ordering follows the usual QK21 layout: xgk[0..10] descending
abscissae with xgk[1,3,5,7,9] the Gauss nodes and xgk[10] = 0; wgk matches
xgk; wg[0..4] are the Gauss weights of xgk[1,3,5,7,9].
"""
import os
import sys

import mpmath as mp

mp.mp.dps = 60
N = 10


def legendre_coeffs(n):
    """Coefficients c[k] of P_n(x) = sum c[k] x^k (Bonnet recursion)."""
    p0 = [mp.mpf(1)]
    p1 = [mp.mpf(0), mp.mpf(1)]
    if n == 0:
        return p0
    for k in range(1, n):
        # (k+1) P_{k+1} = (2k+1) x P_k - k P_{k-1}
        xp1 = [mp.mpf(0)] + p1
        pm = p0 + [mp.mpf(0)] * (len(xp1) - len(p0))
        nxt = [((2 * k + 1) * a - k * b) / (k + 1) for a, b in zip(xp1, pm)]
        p0, p1 = p1, nxt
    return p1


def poly_eval(c, x):
    s = mp.mpf(0)
    for a in reversed(c):
        s = s * x + a
    return s


def moment(k):
    """int_{-1}^{1} x^k dx"""
    return mp.mpf(0) if k % 2 else mp.mpf(2) / (k + 1)


def poly_moment(c, k):
    return mp.fsum(a * moment(j + k) for j, a in enumerate(c))


def main():
    P = legendre_coeffs(N)
    # Gauss nodes: positive roots of P_10
    gauss = sorted(
        [mp.findroot(lambda x: poly_eval(P, x), mp.cos(mp.pi * (i + 0.75) / (N + 0.5)))
         for i in range(N // 2)], reverse=True)
    dP = [j * a for j, a in enumerate(P)][1:]
    wg = [2 / ((1 - x ** 2) * poly_eval(dP, x) ** 2) for x in gauss]

    # Stieltjes polynomial E_11 = x^11 + sum_{m in {1,3,5,7,9}} e_m x^m
    odd = [1, 3, 5, 7, 9]
    A = mp.matrix(len(odd), len(odd))
    rhs = mp.matrix(len(odd), 1)
    for row, k in enumerate(odd):
        for col, m in enumerate(odd):
            A[row, col] = poly_moment(P, m + k)
        rhs[row] = -poly_moment(P, 11 + k)
    e = mp.lu_solve(A, rhs)
    E = [mp.mpf(0)] * 12
    E[11] = mp.mpf(1)
    for col, m in enumerate(odd):
        E[m] = e[col]
    # positive roots of E_11 interlace with the Gauss nodes: bracket them
    grid = [mp.mpf(1)] + gauss + [mp.mpf(0)]
    kron = []
    for lo, hi in zip(grid[1:], grid[:-1]):
        kron.append(mp.findroot(lambda x: poly_eval(E, x), (lo, hi), solver='anderson'))
    kron = sorted(kron, reverse=True)  # 5 positive Kronrod-only nodes

    xgk = []
    for i in range(5):
        xgk += [kron[i], gauss[i]]
    xgk.append(mp.mpf(0))
    # weights from even moments: sum_i w_i * (x_i^{2k}) over the symmetric rule
    M = mp.matrix(11, 11)
    b = mp.matrix(11, 1)
    for k in range(11):
        for i, x in enumerate(xgk):
            mult = 1 if i == 10 else 2
            M[k, i] = mult * x ** (2 * k)
        b[k] = moment(2 * k)
    wgk = mp.lu_solve(M, b)

    # self-checks: exactness to degree 31 and positivity
    for deg in range(0, 32, 2):
        s = wgk[10] * (0 if deg else 1) + mp.fsum(2 * wgk[i] * xgk[i] ** deg for i in range(10))
        if deg == 0:
            s = wgk[10] + mp.fsum(2 * wgk[i] for i in range(10))
        assert abs(s - moment(deg)) < mp.mpf(10) ** -50, deg
    assert all(w > 0 for w in wgk)
    return xgk, wgk, wg


def fmt(v):
    return mp.nstr(v, 17, min_fixed=-1, max_fixed=1, strip_zeros=False) if v != 0 else "0.0"


def emit(path, guard, qualifier, xgk, wgk, wg):
    lines = [
        "/* Generated by oracle/gen_gk21.py -- 21-point Gauss-Kronrod rule on [-1,1],",
        " * derived from the Legendre and Stieltjes polynomials (do not edit). */",
        f"#ifndef {guard}",
        f"#define {guard}",
        f"{qualifier} double GK21_XGK[11] = {{",
    ]
    lines += [f"  {fmt(v)}," for v in xgk] + ["};", f"{qualifier} double GK21_WGK[11] = {{"]
    lines += [f"  {fmt(v)}," for v in wgk] + ["};", f"{qualifier} double GK21_WG[5] = {{"]
    lines += [f"  {fmt(v)}," for v in wg] + ["};", "#endif", ""]
    with open(path, "w") as f:
        f.write("\n".join(lines))


if __name__ == "__main__":
    xgk, wgk, wg = main()
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    emit(os.path.join(root, "oracle", "gk21_nodes.h"), "IMFIT_ORACLE_GK21_NODES_H",
         "static const", xgk, wgk, wg)
    emit(os.path.join(root, "imfit_gb300", "csrc", "gk21_nodes.cuh"), "IMFIT_GB300_GK21_NODES_CUH",
         "__device__ __constant__ const", xgk, wgk, wg)
    sys.stdout.write("xgk=" + ", ".join(fmt(v) for v in xgk) + "\n")
