"""Generates o3g_gauss_poly.h: piecewise polynomials for the FP32 Gaussian core.

The library's Gaussian core (no counterpart in the reference) is, with q = d^2 / sigma^2
and rho = sqrt(q),

    r3  = G(q) / sigma^3,   G(q) = [erf(rho / sqrt 2) - sqrt(2/pi) rho exp(-q/2)] / rho^3,
    bbb = D(q) / sigma^5,   D(q) = 2 G'(q),

and G(q) = q^(-3/2) (the singular kernel) to float precision beyond q = 48.  On [0, 48] the
FP32 kernels evaluate G and D from the polynomials written here instead of erf/exp: one
polynomial of degree DEG in t = q * s + o (t in [-1, 1]) per interval [e_j, e_(j+1)] of
EDGES, fitted by least squares in the Chebyshev basis on a dense grid (near-minimax) and
converted to monomials for Horner's rule.  G and D are computed here in double: the Taylor
series for q < 1 (30 terms) and the closed form above.  The reported error includes the
rounding of q to float (up to 2.5 x 6e-8 relative for D ~ q^(-5/2)), which every float
evaluation of the core has.

Run from this directory:  python gauss_poly_gen.py   (rewrites o3g_gauss_poly.h and prints
the worst relative error of the fits evaluated in float32 with fused multiply-adds).
"""
import os

import numpy as np
from numpy.polynomial import chebyshev as C
from scipy.special import erf

# interval j = [(j/2)^2, ((j+1)/2)^2) for j < 13 and [42.25, 48] for j = 13, so that the
# kernels find j as floor(2 sqrt q) capped at 13
EDGES = [(j / 2.0) ** 2 for j in range(14)] + [48.0]
DEG = 6
# one interval's row: s, o, then (G_k, D_k) from k = DEG down to 0 (the order Horner's rule
# consumes them)
STRIDE = 2 + 2 * (DEG + 1)
CONST = np.sqrt(2.0 / np.pi)


def _coef(n):
    v = 1.0 / (2 * n + 1)
    for k in range(1, n):
        v /= 2 * k
    return v if n % 2 == 1 else -v


def gauss_G(q):
    q = np.asarray(q, dtype=np.float64)
    out = np.empty_like(q)
    s = q < 1.0
    g = np.zeros_like(q[s])
    for n in range(30, 0, -1):
        g = g * q[s] + _coef(n)
    out[s] = CONST * g
    ql = q[~s]
    rho = np.sqrt(ql)
    out[~s] = (erf(rho / np.sqrt(2.0)) - CONST * rho * np.exp(-0.5 * ql)) / rho ** 3
    return out


def gauss_D(q):
    q = np.asarray(q, dtype=np.float64)
    out = np.empty_like(q)
    s = q < 1.0
    gp = np.zeros_like(q[s])
    for n in range(30, 1, -1):
        gp = gp * q[s] + (n - 1) * _coef(n)
    out[s] = 2.0 * CONST * gp
    ql = q[~s]
    out[~s] = (CONST * np.exp(-0.5 * ql) - 3.0 * gauss_G(ql)) / ql
    return out


def _horner_f32(p, t):
    t = t.astype(np.float32)
    acc = np.full_like(t, np.float32(p[-1]))
    for a in p[-2::-1]:
        acc = (acc.astype(np.float64) * t + np.float64(np.float32(a))).astype(np.float32)
    return acc


def fit():
    table, worst = [], 0.0
    for lo, hi in zip(EDGES[:-1], EDGES[1:]):
        s, o = 2.0 / (hi - lo), -(hi + lo) / (hi - lo)
        q = np.linspace(lo, hi, 40001)
        t = q * s + o
        row = [s, o]
        polys = []
        for F in (gauss_G, gauss_D):
            y = F(q)
            p = C.cheb2poly(C.chebfit(t, y, DEG))
            # checked slightly beyond the interval: the index rounds q to an edge's side
            qq = np.linspace(lo - 1e-4 * (hi - lo), hi + 1e-4 * (hi - lo), 4001)
            qq = qq[qq >= 0]
            yy = F(qq)
            # t = fmaf(q, s, o) on the float inputs: one rounding
            tt = (qq.astype(np.float32).astype(np.float64) * np.float64(np.float32(s)) +
                  np.float64(np.float32(o))).astype(np.float32)
            worst = max(worst, float(np.max(np.abs(_horner_f32(p, tt) - yy) / np.abs(yy))))
            polys.append(p)
        for k in range(DEG, -1, -1):
            row += [polys[0][k], polys[1][k]]
        row += [0.0] * (STRIDE - len(row))
        table.append(row)
    return table, worst


def write(table, worst, path):
    # coefficient-major: entry k of every interval side by side, so the lanes of a warp
    # reading entry k of their own intervals touch one cache line
    names = ["s", "o"] + ["%s%d" % (f, k) for k in range(DEG, -1, -1) for f in ("G", "D")]
    lines = []
    for k in range(STRIDE):
        vals = ", ".join("%.9ef" % np.float32(row[k]) for row in table)
        lines.append("    // %s\n    %s," % (names[k] if k < len(names) else "pad", vals))
    body = "\n".join(lines)
    txt = f"""// o3g_gauss_poly.h -- GENERATED by gauss_poly_gen.py (do not edit): piecewise polynomials of
// the FP32 Gaussian core on q in [0, 48]: G(q) (r3 = G / sigma^3) and D(q) = 2 G'(q)
// (bbb = D / sigma^5), degree {DEG} in t = fma(q, s, o) per interval; float32 evaluation with
// fused multiply-adds from a float q stays within {worst:.2e} relative of the double-precision
// functions at the exact q (this includes the rounding of q itself).
#pragma once

namespace o3g {{

constexpr int kGaussPolyDeg = {DEG};
constexpr int kGaussPolyStride = {STRIDE};   // entries per interval: s, o, (G[k], D[k]) for k = {DEG}..0
constexpr int kGaussPolyN = {len(table)};        // intervals; interval j covers [(j/2)^2, ((j+1)/2)^2)
constexpr int kGaussPolyLast = {len(table) - 1};
// entry k of interval j at kGaussPoly[k * kGaussPolyN + j]
__device__ const __align__(16) float kGaussPoly[{STRIDE} * {len(table)}] = {{
{body}
}};

}}  // namespace o3g
"""
    with open(path, "w") as f:
        f.write(txt)


if __name__ == "__main__":
    tab, w = fit()
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "o3g_gauss_poly.h")
    write(tab, w, out)
    print("wrote %s; worst float32 relative error %.3e" % (out, w))
