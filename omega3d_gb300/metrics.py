"""Error measures used by the parity tests and the benchmark.

rel_err(test, ref): per-target relative error of a [k, n] field,
    e_i = |test_i - ref_i| / max(|ref_i|, floor * max_j |ref_j|)
with |.| the Euclidean norm over the k components (k = 3 for velocity, 9 for the
velocity gradient).  Returns (max_i e_i, rms_i e_i).

linf_err(test, ref): max_i |test_i - ref_i| / max_i |ref_i|, the error relative to the
field's largest magnitude.  Per-target relative errors of near-zero targets are bounded
below by FP32 rounding of the individual pair terms (a few 1e-7 of the terms' size),
which no summation scheme removes; the L-infinity form measures the sums' accuracy.
"""
import numpy as np


def _np(a):
    try:
        import torch
        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
    except Exception:  # pragma: no cover
        pass
    return np.asarray(a)


def rel_err(test, ref, floor=1e-6):
    t = _np(test).astype(np.float64)
    r = _np(ref).astype(np.float64)
    if r.ndim == 1:
        r = r[None, :]
        t = t[None, :]
    nr = np.sqrt((r * r).sum(axis=0))
    d = np.sqrt(((t - r) ** 2).sum(axis=0))
    if nr.size == 0:
        return 0.0, 0.0
    den = np.maximum(nr, floor * max(nr.max(), np.finfo(np.float64).tiny))
    e = d / den
    return float(e.max()), float(np.sqrt((e * e).mean()))


def linf_err(test, ref):
    t = _np(test).astype(np.float64)
    r = _np(ref).astype(np.float64)
    if r.ndim == 1:
        r = r[None, :]
        t = t[None, :]
    if r.size == 0:
        return 0.0
    nr = np.sqrt((r * r).sum(axis=0))
    d = np.sqrt(((t - r) ** 2).sum(axis=0))
    return float(d.max() / max(nr.max(), np.finfo(np.float64).tiny))
