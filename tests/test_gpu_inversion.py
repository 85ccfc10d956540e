"""The adjoint-driven field inversion (structured_gb300/inversion.py) and the
learned correction (structured_gb300/mlp.py) end to end on the GPU, on a
reduced SA plate (69x49, first cell 1e-7): the target Cf comes from the
solver itself with the seeded beta field of the inversion workload, and a few
L-BFGS iterations from beta = 1 (flow solves, adjoint solves and
(dR/dbeta)^T psi through the C ABI) must bring the plate Cf most of the way to
the target."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_field_inversion_reduces_cf_misfit(gpu_lib):
    from structured_gb300 import inversion as inv
    summary, arrays = inv.run_case(3e6, 0.0, 69, 49, max_iter=6, log=lambda m: print(m, flush=True))
    print({k: summary[k] for k in ("cf_err_base", "cf_err_inverted", "misfit_initial", "misfit_final",
                                   "iterations", "flow_solves", "wall_s")})
    assert summary["cf_err_base"] > 0.02  # the seeded beta field moves Cf by a few percent
    assert summary["misfit_final"] < 0.1 * summary["misfit_initial"]
    assert summary["cf_err_inverted"] < 0.35 * summary["cf_err_base"]
    # one history entry per accepted iterate, in time order
    assert len(arrays["iter_wall_s"]) >= 2 and np.all(np.diff(arrays["iter_wall_s"]) > 0)


def test_learned_correction_beats_plain_sa_on_held_out_case(gpu_lib, tmp_path):
    """The learned-correction workload on the reduced plate: inversions of
    three training cases (Re_L 1e6 at 0 deg, 3e6 at 0 and +2 deg) and of the
    held-out case (3e6 at -2 deg); the network trained on the training cases'
    (features, inverted beta) pairs by the GPU kernels, then fused into the SA
    source for the held-out solve from freestream.  Its plate Cf must be
    closer to the held-out inverted-beta solution than plain SA's by at least
    a third of plain SA's error."""
    from structured_gb300 import inversion as inv
    from structured_gb300 import mlp
    for re_l, ang in ((1e6, 0.0), (3e6, 0.0), (3e6, 2.0), (3e6, -2.0)):
        tag = "Re%.0e_a%+.0f" % (re_l, ang)
        summary, arrays = inv.run_case(re_l, ang, 69, 49, max_iter=10, log=lambda m: None)
        print(tag, {k: round(summary[k], 4) for k in ("cf_err_base", "cf_err_inverted", "wall_s")})
        # every inversion, the held-out one included, must have reached its target
        # (the comparison is against the held-out inverted-beta solution)
        assert summary["cf_err_inverted"] < 0.5 * summary["cf_err_base"], tag
        np.savez_compressed(os.path.join(tmp_path, "inversion_%s_69x49.npz" % tag), **arrays)
    res, params, loss = mlp.run(str(tmp_path), steps=1500, batch=4096, log=lambda m: print(m, flush=True))
    plain = res["plain_sa"]["cf_err_vs_inverted"]
    learned = res["learned"]["cf_err_vs_inverted"]
    print("held out: plain SA %.4f, learned %.4f (loss %.2e -> %.2e)"
          % (plain, learned, res["train"]["loss_first"], res["train"]["loss_last"]))
    assert res["learned"]["converged"] and res["inverted_beta"]["converged"]
    assert res["inverted_beta"]["cf_err_vs_inverted"] < 1e-6
    assert learned < (2.0 / 3.0) * plain
