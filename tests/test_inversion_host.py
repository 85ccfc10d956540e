"""Host logic of the field inversion (structured_gb300/inversion.py): the
L-BFGS direction and the plate weights, on CPU."""
import numpy as np

from structured_gb300 import inversion as inv


def test_lbfgs_on_a_quadratic_matches_conjugate_gradients():
    """With exact line minimisation on a quadratic, L-BFGS with full memory
    generates the conjugate-gradient iterates and ends at the minimiser in
    n steps."""
    rng = np.random.default_rng(1)
    n = 6
    A = rng.standard_normal((n, n))
    A = A @ A.T + n * np.eye(n)
    b = rng.standard_normal(n)
    x = np.zeros(n)
    S, Y = [], []
    g = A @ x - b
    for _ in range(n):
        d = inv.lbfgs_direction(g, S, Y)
        assert g @ d < 0
        t = -(g @ d) / (d @ A @ d)  # exact minimiser along d
        xn = x + t * d
        gn = A @ xn - b
        S.append(xn - x)
        Y.append(gn - g)
        x, g = xn, gn
    np.testing.assert_allclose(x, np.linalg.solve(A, b), rtol=1e-8, atol=1e-10)


def test_first_direction_is_scaled_steepest_descent():
    g = np.array([0.5, -2.0, 1.0])
    d = inv.lbfgs_direction(g, [], [])
    np.testing.assert_allclose(d, -g * (1e-2 / 2.0))


def test_plate_weights_cover_the_plate_faces_only(tmp_path):
    from structured_gb300 import workloads
    c = workloads.turbulent_plate(str(tmp_path), 41, 21, write_files=False)
    from structured_gb300 import case as C
    g = C.flat_plate_grid(41, 21, h1=1e-7, ratio=1.05)
    w = inv.plate_weights(c, g.xv)
    xm = 0.5 * (g.xv[:-1, 0] + g.xv[1:, 0])
    assert (w[xm < 0] == 0).all()
    assert abs(w.sum() - 1.0) < 1e-12  # the plate spans x in [0, 1]
