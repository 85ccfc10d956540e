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


def test_lbfgs_minimize_on_an_ill_conditioned_least_squares_problem():
    """The inversion's optimiser on a nonlinear least-squares problem with
    weights over four decades and a region where the objective is undefined
    (as a diverged flow solve leaves it): it backs off that region and
    converges."""
    rng = np.random.default_rng(7)
    n = 40
    w = 10.0 ** rng.uniform(0, 4, n)
    A = np.eye(n) + 0.1 * rng.standard_normal((n, n))
    x_true = 0.3 * rng.standard_normal(n)

    def r(x):
        return np.tanh(A @ x) + 0.5 * (A @ x) - (np.tanh(A @ x_true) + 0.5 * (A @ x_true))

    def evaluate(x):
        if np.abs(x).max() > 3.0:
            return np.inf, None, None
        z = A @ x
        res = r(x)
        jac = (1.0 - np.tanh(z) ** 2 + 0.5)[:, None] * A
        return float((w * res * res).sum()), 2.0 * jac.T @ (w * res), None

    seen = []
    x, f, g, _, it = inv.lbfgs_minimize(evaluate, np.zeros(n), 300, first_step=5.0, log=lambda m: None,
                                        on_accept=lambda it, x, f, aux, step: seen.append(f))
    # (scipy's L-BFGS-B with the same memory reaches 6e-5 here in 300 iterations)
    assert f < 1e-8 * evaluate(np.zeros(n))[0], (f, it)
    assert all(b <= a for a, b in zip(seen, seen[1:]))  # monotone accepted iterates
    np.testing.assert_allclose(x, x_true, atol=1e-2)


def test_metric_direction_and_cell_areas():
    """With a diagonal metric the first direction is -M g scaled to the step
    bound, and the two-loop recursion keeps the secant equation H y = s for
    the newest pair; cell areas of a unit-square grid sum to one."""
    rng = np.random.default_rng(3)
    g = rng.standard_normal(6)
    M = rng.uniform(0.1, 10.0, 6)
    d = inv.lbfgs_direction(g, [], [], first_step=0.2, metric=M)
    np.testing.assert_allclose(d, -M * g * (0.2 / np.abs(M * g).max()))
    s, y = rng.standard_normal(6), rng.standard_normal(6)
    y = y if (s @ y) > 0 else -y
    np.testing.assert_allclose(inv.lbfgs_direction(-y, [s], [y], metric=M), s, rtol=1e-12, atol=1e-12)
    xv, yv = np.meshgrid(np.linspace(0, 1, 5), np.linspace(0, 1, 9) ** 2, indexing="ij")
    assert abs(inv.cell_areas(xv, yv).sum() - 1.0) < 1e-14
