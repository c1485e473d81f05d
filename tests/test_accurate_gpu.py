"""GPU tests of the accurate precision mode (O3G_PREC_ACCURATE): pair terms in double-single
FP32 arithmetic (exact separations, d^2, core factor and cross product as float pairs), the
velocity terms added unrounded into double-single running sums that the compensated
(Fast2Sum-folded) accumulators take over.

Tolerances against the FP64 oracle (per-target relative error, metrics.rel_err):
  * velocity per target <= 1e-6 everywhere, the accuracy form the mode exists for;
  * velocity L-infinity <= 1e-7: the terms carry about 44 bits (the Gaussian core's
    double-single polynomials are within 1.2e-10 of the function) and their sums are
    exact to that level, so the float outputs' own rounding (6e-8) is what remains;
  * gradients per target <= 1e-5 and L-infinity <= 1e-6 (their terms are formed in float
    from the double-single core, as in COMPENSATED);
  * and the velocity is at least as accurate as COMPENSATED on the same inputs.
Only the RM and Gaussian cores have the mode; the others return O3G_ERR_INVALID_ARG."""
import numpy as np
import pytest

import oracle as O
from omega3d_gb300 import _lib as L
from omega3d_gb300 import workloads as W
from omega3d_gb300.metrics import linf_err, rel_err

from test_pair_gpu import gpu_eval

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("core", ["rm", "gauss"])
@pytest.mark.parametrize("kind", ["particles", "fieldpoints"])
def test_accurate_matches_fp64_oracle(cuda, core, kind):
    x, s, r = W.gaussian_cloud(6000, seed=211, pos_std=0.2)
    if kind == "particles":
        tx, tr = x, r
    else:
        tx = np.random.default_rng(212).normal(scale=0.25, size=(3, 2500)).astype(np.float32)
        tr = None
    u64, g64 = O.points_affect_points(x, r, s, tx, tr, True, core, 2)
    ua, ga = gpu_eval(x, s, r, tx, tr, core=core, prec="accurate")
    uc, _ = gpu_eval(x, s, r, tx, tr, core=core, prec="compensated")
    ea, ec = rel_err(ua, u64)[0], rel_err(uc, u64)[0]
    assert ea <= 1e-6 and linf_err(ua, u64) <= 1e-7, (ea, linf_err(ua, u64))
    assert rel_err(ga, g64)[0] <= 1e-5 and linf_err(ga, g64) <= 1e-6
    assert ea <= ec


@pytest.mark.parametrize("core", ["rm", "gauss"])
def test_accurate_velocity_only_and_host_memory(cuda, core):
    x, s, r = W.gaussian_cloud(3000, seed=213, pos_std=0.2)
    u64, _ = O.points_affect_points(x, r, s, x, r, False, core, 2)
    ud, _ = gpu_eval(x, s, r, x, r, grads=False, core=core, prec="accurate")
    uh, _ = gpu_eval(x, s, r, x, r, grads=False, core=core, prec="accurate", on_device=False)
    assert rel_err(ud, u64)[0] <= 1e-6
    assert np.array_equal(ud.view(np.uint32), uh.view(np.uint32))


@pytest.mark.parametrize("core", ["wl", "exp", "v2"])
def test_accurate_other_cores_are_refused(cuda, core):
    x, s, r = W.gaussian_cloud(256, seed=214)
    with pytest.raises(L.O3GError) as ei:
        gpu_eval(x, s, r, x, r, core=core, prec="accurate")
    assert ei.value.status == 1
