"""Direct accuracy check of the fused kernels' reciprocal and square root.

The kernels replace IEEE division and square root by refinements of the hardware
estimates (nr_rcp / nr_sqrt / nr_rsqrt in hypar_gb300/csrc/gbh_device.cuh) and claim
a result within one unit in the last place.  gb_probe_rcp_sqrt evaluates them on
the GPU beside CUDA's correctly rounded 1/x and sqrt(x); both are compared with
numpy's correctly rounded results in units in the last place (ulp), and 1/sqrt(x)
with the extended-precision value rounded to double, over 1e6 inputs from each
range the path feeds them:

  * reciprocals of densities and of sums of squared sound speeds: 1e-3 .. 1e3,
  * reciprocals of WENO5 weight normalisations (sums of products of (beta + eps)^2
    terms, eps = 1e-6, so as small as ~1e-24 and as large as ~1e24): 1e-30 .. 1e30,
  * square roots of densities (Roe averages) and of gamma P / rho: 1e-6 .. 1e6.
"""
import numpy as np
import pytest

from hypar_gb300 import _lib

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

N = 1_000_000


def _log_uniform(rng, lo, hi, n):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n))


def _ulps(a, b):
    """|a - b| in units in the last place for positive finite doubles."""
    return np.abs(a.view(np.int64) - b.view(np.int64))


def _probe(x):
    L = _lib.lib()
    xd = torch.from_numpy(x).cuda()
    outs = [torch.empty_like(xd) for _ in range(5)]
    _lib.check(L.gb_probe_rcp_sqrt(xd.data_ptr(), *[o.data_ptr() for o in outs], x.size))
    return [o.cpu().numpy() for o in outs]


@pytest.mark.parametrize("lo,hi", [(1e-3, 1e3), (1e-30, 1e30), (1e-6, 1e6)])
def test_rcp_sqrt_within_one_ulp(built_lib, lo, hi):
    rng = np.random.default_rng(20261204)
    x = _log_uniform(rng, lo, hi, N)
    rcp_nr, rcp_ieee, sqrt_nr, sqrt_ieee, rsqrt_nr = _probe(x)
    rcp_exact = 1.0 / x
    sqrt_exact = np.sqrt(x)
    # CUDA's round-to-nearest intrinsics are the correctly rounded results numpy computes
    assert np.array_equal(rcp_ieee, rcp_exact)
    assert np.array_equal(sqrt_ieee, sqrt_exact)
    ur = _ulps(rcp_nr, rcp_exact)
    us = _ulps(sqrt_nr, sqrt_exact)
    assert int(ur.max()) <= 1, (int(ur.max()), float(x[np.argmax(ur)]))
    assert int(us.max()) <= 1, (int(us.max()), float(x[np.argmax(us)]))
    rsqrt_exact = (1.0 / np.sqrt(x.astype(np.longdouble))).astype(np.float64)
    uq = _ulps(rsqrt_nr, rsqrt_exact)
    assert int(uq.max()) <= 1, (int(uq.max()), float(x[np.argmax(uq)]))


def test_rcp_sqrt_empty_and_bad_arguments(built_lib):
    L = _lib.lib()
    _lib.check(L.gb_probe_rcp_sqrt(None, None, None, None, None, None, 0))
    assert L.gb_probe_rcp_sqrt(None, None, None, None, None, None, 4) == 1
    assert L.gb_probe_rcp_sqrt(None, None, None, None, None, None, -1) == 1
