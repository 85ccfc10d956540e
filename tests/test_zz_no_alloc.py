"""The allocation-free norm entry point (st_norms_noalloc) agrees with the
context-based st_norms.

It exists for callers that cannot allocate device memory while running (an
application that reserved the device for its own pool, or a loop that cannot
afford cudaMalloc's synchronisation); its scratch is a fixed array inside the
library.  Kept in its own file so it is collected after every other test."""
import ctypes

import numpy as np
import pytest

from helpers import flat_plate
from structured_gb300 import case as C

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("turb", ["none", "sa"])
def test_norms_noalloc_matches_context_norms(gpu_lib, tmp_path, turb):
    import torch
    from structured_gb300.solver import EulerEquation
    lib = gpu_lib
    lib.st_norms_noalloc.restype = ctypes.c_int
    lib.st_norms_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_void_p]
    c = flat_plate(tmp_path, "na", 129, 65, turbulence=turb)
    xv, yv = C.load_grid(c)
    eq = EulerEquation(c, xv, yv)
    out = torch.zeros(8, dtype=torch.float64, device="cuda")
    for call in range(2):  # two calls in a row: the shared scratch is reused
        eq.calc_residual(C.perturbed_state(c, 60 + call))
        ref = eq.norms()
        _, rhs_dev, stream = eq.device_state()
        rc = lib.st_norms_noalloc(ctypes.c_void_p(rhs_dev), eq.nic * eq.njc, eq.nq,
                                  ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))
        assert rc == 0, lib.st_last_error()
        torch.cuda.synchronize()
        got = out[:eq.nq].cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=1e-13)


def test_norms_noalloc_rejects_oversized_components(gpu_lib):
    lib = gpu_lib
    lib.st_norms_noalloc.restype = ctypes.c_int
    lib.st_norms_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_void_p]
    dummy = ctypes.c_void_p(1)
    assert lib.st_norms_noalloc(dummy, 10, 9, dummy, None) == -1
    assert b"nq must be" in lib.st_last_error()
