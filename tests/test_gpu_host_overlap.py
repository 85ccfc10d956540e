"""Host-buffer entry points (st_residual, st_vjp, st_residual_vjp) against the
device-pointer ones they wrap, bit for bit.

The host-buffer calls overlap their copies with the pipeline: psi goes in on a
second stream while the forward passes run, the residual and the beta product
go out on it during the gather, and the last per-cell pass (k_cell, k_prim_adj)
runs in bands whose outputs go out while the next band computes.  Each call is
checked with pageable (numpy) and page-locked (pinned torch) buffers, twice in
a row with different psi so that a copy ordered against the wrong pass would
show, at order 2 and at the first-order lhs operator, SA and laminar.  The
513x257 grid gives two bands."""
import ctypes

import numpy as np
import pytest

from structured_gb300 import case as C

pytestmark = pytest.mark.gpu
SEED = 20261207


def plate(turb, ni=513, nj=257):
    import tempfile
    c = C.flat_plate_case(tempfile.gettempdir(), "ov", ni, nj, 0.3, 1e6, 1e-4, 1.08, turbulence=turb,
                          write_files=False)
    g = C.flat_plate_grid(ni, nj, h1=1e-4, ratio=1.08)
    return c, g.xv, g.yv, C.perturbed_state(c, SEED)


def pinned(shape):
    import torch
    return torch.empty(shape, dtype=torch.float64).pin_memory()


def dptr(t):
    return ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_double))


@pytest.mark.parametrize("lhs", [False, True])
@pytest.mark.parametrize("turb", ["sa", "none"])
def test_host_entry_points_match_device_ones(gpu_lib, turb, lhs):
    check_host_entry_points(turb, lhs, 513, 257)


def test_host_entry_points_in_eight_bands(gpu_lib):
    """1025x513: 524,288 cells, the full eight bands."""
    check_host_entry_points("sa", False, 1025, 513)


def check_host_entry_points(turb, lhs, ni, nj):
    import torch
    from structured_gb300.solver import EulerEquation
    c, xv, yv, q = plate(turb, ni, nj)
    eq = EulerEquation(c, xv, yv)
    eq.set_state(q)
    rng = np.random.default_rng(SEED)
    shape = q.shape
    nb = shape[:2]
    beta = 1.0 + 0.2 * rng.standard_normal(nb)
    eq.set_beta(beta)
    beta_d = torch.tensor(beta, device="cuda")
    lib = eq.lib
    for trial in range(2):
        psi = rng.standard_normal(shape)
        # device-pointer reference
        psi_d = torch.tensor(psi, device="cuda")
        rhs_d = torch.empty_like(psi_d)
        oq_d = torch.empty_like(psi_d)
        ob_d = torch.empty(nb, dtype=torch.float64, device="cuda")
        eq.residual_vjp_device(psi_d.data_ptr(), rhs_d.data_ptr(), oq_d.data_ptr(), ob_d.data_ptr(), lhs=lhs)
        torch.cuda.synchronize()
        ref = {"rhs": rhs_d.cpu().numpy(), "oq": oq_d.cpu().numpy(), "ob": ob_d.cpu().numpy()}
        eq.residual_device(eq.device_state()[0], rhs_d.data_ptr(), beta_ptr=beta_d.data_ptr(), lhs=lhs)
        torch.cuda.synchronize()
        ref_res = rhs_d.cpu().numpy()

        # pageable buffers: copies after the passes
        r, oq, ob = eq.residual_vjp(psi, lhs=lhs)
        assert np.array_equal(r, ref["rhs"]) and np.array_equal(oq, ref["oq"]) and np.array_equal(ob, ref["ob"])
        oq, ob = eq.vjp(psi, lhs=lhs)
        assert np.array_equal(oq, ref["oq"]) and np.array_equal(ob, ref["ob"])

        # page-locked buffers
        psi_h = pinned(shape)
        psi_h.copy_(torch.from_numpy(psi))
        r_h, oq_h, ob_h = pinned(shape), pinned(shape), pinned(nb)
        for t in (r_h, oq_h, ob_h):
            t.fill_(np.nan)
        assert lib.st_residual_vjp(eq.h, dptr(psi_h), dptr(r_h), dptr(oq_h), dptr(ob_h), int(lhs)) == 0
        assert np.array_equal(r_h.numpy(), ref["rhs"])
        assert np.array_equal(oq_h.numpy(), ref["oq"])
        assert np.array_equal(ob_h.numpy(), ref["ob"])
        oq_h.fill_(np.nan)
        ob_h.fill_(np.nan)
        assert lib.st_vjp(eq.h, dptr(psi_h), dptr(oq_h), dptr(ob_h), int(lhs)) == 0
        assert np.array_equal(oq_h.numpy(), ref["oq"]) and np.array_equal(ob_h.numpy(), ref["ob"])
        # one output only, the others null
        oq_h.fill_(np.nan)
        assert lib.st_residual_vjp(eq.h, dptr(psi_h), None, dptr(oq_h), None, int(lhs)) == 0
        assert np.array_equal(oq_h.numpy(), ref["oq"])
        ob_h.fill_(np.nan)
        assert lib.st_vjp(eq.h, dptr(psi_h), None, dptr(ob_h), int(lhs)) == 0
        assert np.array_equal(ob_h.numpy(), ref["ob"])

        # residual alone: copied out band by band behind the cell pass
        r_h.fill_(np.nan)
        assert lib.st_residual(eq.h, int(lhs), dptr(r_h)) == 0
        assert np.array_equal(r_h.numpy(), ref_res)
        r2 = np.empty(shape)
        assert lib.st_residual(eq.h, int(lhs), r2.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
        assert np.array_equal(r2, ref_res)
        del psi_d, rhs_d, oq_d, ob_d
    del beta_d
    eq.close()


def test_tiled_residual_path_with_page_locked_rhs(gpu_lib):
    """After the tiled sweeps the residual goes out whole, on the copy stream."""
    from structured_gb300.solver import EulerEquation
    c, xv, yv, q = plate("sa")
    eq = EulerEquation(c, xv, yv)
    ref = eq.calc_residual(q)
    if not eq.set_residual_path(True):
        eq.close()
        pytest.skip("tiled sweeps unavailable on this device")
    r_h = pinned(q.shape)
    r_h.fill_(np.nan)
    assert eq.lib.st_residual(eq.h, 0, dptr(r_h)) == 0
    assert np.array_equal(r_h.numpy(), ref)
    eq.close()
