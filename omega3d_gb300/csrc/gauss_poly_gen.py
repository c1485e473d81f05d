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

Run from this directory:  python gauss_poly_gen.py   (rewrites o3g_gauss_poly.h and
o3g_gauss_poly_ds.h and prints the worst relative error of each evaluation).
"""
import os

import numpy as np
from numpy.polynomial import chebyshev as C
from scipy.special import erf

# interval j = [j, j + 1) for j = 0..47, so that the kernels find j as the integer part of
# q (one conversion, no square root); degree 5 reaches the float rounding of q already
EDGES = [float(j) for j in range(49)]
DEG = 5
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
    # pair-interleaved and coefficient-major: the float pairs (s, o), (G_k, D_k) for
    # k = DEG..0 are entries e2 = 0..DEG+1, entry e2 of interval j at float2 index
    # e2 * N + j.  The lanes of a warp reading entry e2 of their own intervals touch one
    # 112-byte span, and one 8-byte load gives both Horner chains their coefficient.
    names = ["(s, o)"] + ["(G%d, D%d)" % (k, k) for k in range(DEG, -1, -1)]
    lines = []
    for e2 in range(STRIDE // 2):
        vals = ", ".join("%.9ef, %.9ef" % (np.float32(row[2 * e2]), np.float32(row[2 * e2 + 1])) for row in table)
        lines.append("    // %s\n    %s," % (names[e2], vals))
    body = "\n".join(lines)
    txt = f"""// o3g_gauss_poly.h -- GENERATED by gauss_poly_gen.py (do not edit): piecewise polynomials of
// the FP32 Gaussian core on q in [0, 48]: G(q) (r3 = G / sigma^3) and D(q) = 2 G'(q)
// (bbb = D / sigma^5), degree {DEG} in t = fma(q, s, o) per interval; float32 evaluation with
// fused multiply-adds from a float q stays within {worst:.2e} relative of the double-precision
// functions at the exact q (this includes the rounding of q itself).
#pragma once

namespace o3g {{

constexpr int kGaussPolyDeg = {DEG};
constexpr int kGaussPolyStride = {STRIDE};   // floats per interval: (s, o), (G[k], D[k]) for k = {DEG}..0
constexpr int kGaussPolyN = {len(table)};        // intervals; interval j covers [j, j + 1)
constexpr int kGaussPolyLast = {len(table) - 1};
// float pair e2 of interval j at kGaussPoly[2 (e2 * kGaussPolyN + j)], [.. + 1]
__device__ const __align__(16) float kGaussPoly[{STRIDE} * {len(table)}] = {{
{body}
}};

}}  // namespace o3g
"""
    with open(path, "w") as f:
        f.write(txt)


# ---- the accurate (double-single) evaluation: o3g_gauss_poly_ds.h ----------------------
# Degree DEG_DS in t = q s + o, with s and o the float32 values the kernel uses (the fit is
# made in that t, so the map itself adds no error).  The kernel runs Horner's rule in float
# for the coefficients of degree >= 3 (together at most 0.14 % of |G| or |D| on every
# interval, so their float rounding stays near 1e-10 relative) and in double-single
# arithmetic for degrees 2, 1, 0, whose coefficients are stored as (hi, lo) float pairs.
DEG_DS = 8
NDS = 3          # low-order coefficients kept as (hi, lo) pairs
STRIDE_DS = 2 + 2 * (DEG_DS + 1 - NDS) + 4 * NDS


def _split(v):
    hi = np.float32(v)
    return hi, np.float32(v - np.float64(hi))


def fit_ds():
    table, worst = [], 0.0
    for lo, hi in zip(EDGES[:-1], EDGES[1:]):
        s32, o32 = np.float32(2.0 / (hi - lo)), np.float32(-(hi + lo) / (hi - lo))
        s, o = np.float64(s32), np.float64(o32)
        q = np.linspace(lo, hi, 40001)
        t = q * s + o
        row = [s32, o32]
        polys = []
        for F in (gauss_G, gauss_D):
            y = F(q)
            polys.append(C.cheb2poly(C.chebfit(t, y, DEG_DS)))
            # the kernel's evaluation: float tail, then (hi, lo) steps (double stands in for
            # double-single arithmetic, which carries about 44 bits)
            qq = np.linspace(lo - 1e-4 * (hi - lo), hi + 1e-4 * (hi - lo), 4001)
            qq = qq[qq >= 0]
            tt = qq * s + o
            tf = tt.astype(np.float32)
            p = polys[-1]
            acc = np.full_like(tf, np.float32(p[DEG_DS]))
            for k in range(DEG_DS - 1, NDS - 1, -1):
                acc = (acc.astype(np.float64) * tf + np.float64(np.float32(p[k]))).astype(np.float32)
            v = acc.astype(np.float64)
            for k in range(NDS - 1, -1, -1):
                h, l = _split(p[k])
                v = v * tt + (np.float64(h) + np.float64(l))
            yy = F(qq)
            worst = max(worst, float(np.max(np.abs(v - yy) / np.abs(yy))))
        for k in range(DEG_DS, NDS - 1, -1):
            row += [np.float32(polys[0][k]), np.float32(polys[1][k])]
        for k in range(NDS - 1, -1, -1):
            gh, gl = _split(polys[0][k])
            dh, dl = _split(polys[1][k])
            row += [gh, gl, dh, dl]
        assert len(row) == STRIDE_DS
        table.append(row)
    return table, worst


def write_ds(table, worst, path):
    names = ["s", "o"] + ["%s%d" % (f, k) for k in range(DEG_DS, NDS - 1, -1) for f in ("G", "D")] + \
            ["%s%d%s" % (f, k, h) for k in range(NDS - 1, -1, -1) for f in ("G", "D") for h in ("hi", "lo")]
    lines = []
    for k in range(STRIDE_DS):
        vals = ", ".join("%.9ef" % np.float32(row[k]) for row in table)
        lines.append("    // %s\n    %s," % (names[k], vals))
    body = "\n".join(lines)
    txt = f"""// o3g_gauss_poly_ds.h -- GENERATED by gauss_poly_gen.py (do not edit): piecewise polynomials
// of the Gaussian core for the accurate (double-single) precision mode, on the intervals of
// o3g_gauss_poly.h: G(q) and D(q) = 2 G'(q), degree {DEG_DS} in t = q s + o (s, o the float
// values below).  Coefficients of degree >= {NDS} are floats (Horner in float); degrees
// {NDS - 1}..0 are (hi, lo) float pairs (Horner in double-single).  Evaluated that way from an
// exact q the result stays within {worst:.2e} relative of the double-precision functions.
#pragma once

namespace o3g {{

constexpr int kGaussDsDeg = {DEG_DS};
constexpr int kGaussDsPairs = {NDS};
constexpr int kGaussDsStride = {STRIDE_DS};   // s, o, (G[k], D[k]) for k = {DEG_DS}..{NDS}, then (G[k] hi, lo, D[k] hi, lo) for k = {NDS - 1}..0
// entry e of interval j at kGaussPolyDs[e * kGaussPolyN + j]
__device__ const __align__(16) float kGaussPolyDs[{STRIDE_DS} * {len(table)}] = {{
{body}
}};

}}  // namespace o3g
"""
    with open(path, "w") as f:
        f.write(txt)


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    tab, w = fit()
    out = os.path.join(here, "o3g_gauss_poly.h")
    write(tab, w, out)
    print("wrote %s; worst float32 relative error %.3e" % (out, w))
    tab, w = fit_ds()
    out = os.path.join(here, "o3g_gauss_poly_ds.h")
    write_ds(tab, w, out)
    print("wrote %s; worst relative error %.3e" % (out, w))
