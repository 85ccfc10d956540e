"""The kernels' Newton-Raphson reciprocal and square roots (st_common.cuh:
nr_rcp, nr_rsqrt, nr_sqrt, nr_sqrt_inv) against correctly rounded values
computed in extended precision, over positive normal inputs from 1e-30 to
1e30 plus the ranges the residual meets (densities, pressures, sound speeds)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ulps(a, exact):
    """Distance of a from the extended-precision value in units of the FP64
    spacing at the correctly rounded result."""
    ref = exact.astype(np.float64)
    return np.abs(a.astype(np.longdouble) - exact) / np.spacing(np.abs(ref)).astype(np.longdouble)


def test_newton_raphson_math_is_within_an_ulp_or_two(gpu_lib):
    import ctypes

    import torch
    rng = np.random.default_rng(2026)
    x = np.concatenate([10.0 ** rng.uniform(-30, 30, 200000), rng.uniform(0.5, 2.0, 200000),
                        rng.uniform(1e-3, 10.0, 200000), 1.0 + rng.standard_normal(50000) * 1e-8,
                        2.0 ** np.arange(-60, 61, dtype=np.float64)])
    xt = torch.tensor(x, device="cuda")
    out = torch.empty((x.size, 5), dtype=torch.float64, device="cuda")
    rc = gpu_lib.st_probe_nr_math(ctypes.c_void_p(xt.data_ptr()), x.size, ctypes.c_void_p(out.data_ptr()))
    assert rc == 0
    o = out.cpu().numpy()
    xl = x.astype(np.longdouble)
    rcp, rs = 1 / xl, 1 / np.sqrt(xl)
    sq = np.sqrt(xl)
    e = {"rcp": ulps(o[:, 0], rcp), "rsqrt": ulps(o[:, 1], rs), "sqrt": ulps(o[:, 2], sq),
         "sqrt_inv.root": ulps(o[:, 3], sq), "sqrt_inv.inv": ulps(o[:, 4], rs)}
    print({k: float(v.max()) for k, v in e.items()})
    # the correctly rounded value is within 0.5 ulp; the refined values within
    # about one more rounding of it
    assert e["rcp"].max() <= 1.5
    assert e["sqrt"].max() <= 1.5 and e["sqrt_inv.root"].max() <= 1.5
    assert e["rsqrt"].max() <= 2.5 and e["sqrt_inv.inv"].max() <= 2.5
