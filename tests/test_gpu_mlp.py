"""Learned SA correction on the GPU: the BF16 tensor-core MLP (inference and
training) against an FP32 numpy restatement that rounds to BF16 where the
kernels do, and the fused in-kernel beta against the same beta as a field."""
import numpy as np
import pytest

from helpers import flat_plate
from structured_gb300 import case as C

pytestmark = pytest.mark.gpu
H = 64


def bf16(x):
    """Round float32 to bfloat16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def unpack(p):
    """FP32 master layout: W1 [64][4] | b1 | W2 [64][64] | b2 | w3 | b3."""
    o = 0
    W1 = p[o:o + H * 4].reshape(H, 4); o += H * 4
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    return W1, b1, W2, b2, w3, p[o]


def ref_forward(p, x):
    W1, b1, W2, b2, w3, b3 = unpack(p)
    xb = bf16(x)
    h1 = bf16(np.tanh(xb @ bf16(W1).T + b1))
    h2 = bf16(np.tanh(h1 @ bf16(W2).T + b2))
    z = h2 @ bf16(w3) + b3
    return np.logaddexp(0.0, z), (xb, h1, h2, z)


def splitmix64(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)).astype(np.uint64)
    x = ((x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)).astype(np.uint64)
    x = ((x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)).astype(np.uint64)
    return x ^ (x >> np.uint64(31))


def make_eq(tmp_path):
    from structured_gb300.solver import EulerEquation
    c = flat_plate(tmp_path, "mlp", 41, 25, turbulence="sa", reynolds=5e6, h1=1e-6, ratio=1.15, mach=0.2)
    xv, yv = C.load_grid(c)
    eq = EulerEquation(c, xv, yv)
    q = C.perturbed_state(c, 91)
    eq.set_state(q)
    return c, eq, q


def features(eq):
    import torch
    f = torch.empty((eq.nic * eq.njc, 4), dtype=torch.float32, device="cuda")
    eq.sa_features_device(f.data_ptr())
    torch.cuda.synchronize()
    return f.cpu().numpy()


def random_params(eq, seed):
    eq.mlp_init(seed)
    p = eq.mlp_params()
    rng = np.random.default_rng(seed)
    p = p + rng.normal(0.0, 0.2, p.size).astype(np.float32)  # non-zero biases too
    eq.mlp_set_params(p)
    return p


def test_mlp_inference_matches_reference(gpu_lib, tmp_path):
    import torch
    c, eq, q = make_eq(tmp_path)
    f = features(eq)
    assert np.isfinite(f).all()
    assert (f[:, 0] >= 0).all() and (f[:, 0] <= 1).all() and (f[:, 3] >= 0).all() and (f[:, 3] <= 10).all()
    mean, std = f.mean(axis=0), f.std(axis=0) + 1e-6
    eq.mlp_set_normalization(mean, std)
    p = random_params(eq, 5)
    b = torch.empty(eq.nic * eq.njc, dtype=torch.float64, device="cuda")
    eq.mlp_beta_device(b.data_ptr())
    torch.cuda.synchronize()
    x = ((f - mean) * np.float32(1.0) / std).astype(np.float32)
    ref, _ = ref_forward(p, x)
    err = np.abs(b.cpu().numpy() - ref)
    print("inference: max %.3e, median %.3e, max |beta| %.3f" % (err.max(), np.median(err), np.abs(ref).max()))
    # The kernel rounds to BF16 where the restatement does; the two differ only
    # where FP32 accumulation order moves an activation across a BF16 rounding
    # boundary.  Bound: one BF16 ulp (2^-8 relative) of the largest beta.
    assert err.max() <= 2.0 ** -8 * np.abs(ref).max(), (err.max(), np.median(err))
    assert np.median(err) < 1e-5, np.median(err)


def test_fused_beta_equals_beta_field(gpu_lib, tmp_path):
    """Residual and JVP with the in-kernel network beta equal those with the
    network's beta written to the beta array (beta held fixed in the JVP)."""
    import torch
    c, eq, q = make_eq(tmp_path)
    f = features(eq)
    eq.mlp_set_normalization(f.mean(axis=0), f.std(axis=0) + 1e-6)
    random_params(eq, 6)
    b = torch.empty(eq.nic * eq.njc, dtype=torch.float64, device="cuda")
    eq.mlp_beta_device(b.data_ptr())
    torch.cuda.synchronize()
    beta = b.cpu().numpy().reshape(eq.nic, eq.njc)
    rng = np.random.default_rng(7)
    v = torch.tensor(rng.standard_normal(q.shape) * np.abs(q).mean(axis=(0, 1)), device="cuda")
    eq.mlp_enable(True)
    r1 = eq.calc_residual(q)
    j1 = torch.empty_like(v)
    eq.set_state(q)
    eq.jvp_device(v.data_ptr(), j1.data_ptr(), None)
    eq.mlp_enable(False)
    eq.set_beta(beta)
    r2 = eq.calc_residual(q)
    j2 = torch.empty_like(v)
    eq.set_state(q)
    eq.jvp_device(v.data_ptr(), j2.data_ptr(), None)
    torch.cuda.synchronize()
    assert np.array_equal(r1, r2)
    assert torch.equal(j1, j2)
    assert np.abs(beta - 1.0).max() > 1e-3  # the network is not the identity


def test_mlp_training_step_and_convergence(gpu_lib, tmp_path):
    import torch
    c, eq, q = make_eq(tmp_path)
    rng = np.random.default_rng(8)
    n = 8192
    feat = rng.standard_normal((n, 4)).astype(np.float32)
    target = (1.0 + 0.3 * np.tanh(feat[:, 0] - 0.5 * feat[:, 2])).astype(np.float32)
    eq.mlp_set_normalization(np.zeros(4, np.float32), np.ones(4, np.float32))
    eq.mlp_init(11)
    p0 = eq.mlp_params()
    ft = torch.tensor(feat, device="cuda")
    tt = torch.tensor(target, device="cuda")
    batch, seed = 256, 12345
    g_gpu, loss0 = eq.mlp_grad(ft.data_ptr(), tt.data_ptr(), n, batch, seed, step=0)
    loss1 = eq.mlp_train(ft.data_ptr(), tt.data_ptr(), n, 1, batch=batch, lr=1e-3, seed=seed)
    p1 = eq.mlp_params()
    assert loss0 == float(loss1[0])
    # numpy gradient on the same samples
    slot = np.arange(batch, dtype=np.uint64)
    idx = (splitmix64(np.uint64(seed) ^ splitmix64(np.uint64(0) * np.uint64(batch) + slot)) % np.uint64(n)).astype(np.int64)
    x, t = feat[idx], target[idx]
    W1, b1, W2, b2, w3, b3 = unpack(p0)
    y, (xb, h1, h2, z) = ref_forward(p0, x)
    assert abs(float(((y - t) ** 2).mean()) - float(loss1[0])) < 1e-3 * max(1.0, float(loss1[0]))
    dy = (2.0 / batch) * (y - t) / (1.0 + np.exp(-z))
    d2 = bf16(dy[:, None] * bf16(w3)[None, :] * (1 - h2 ** 2))
    d1 = bf16((d2 @ bf16(W2)) * (1 - h1 ** 2))
    g = np.concatenate([(d1.T @ xb).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0), h2.T @ dy, [dy.sum()]])
    # the training kernels' gradient in value: BF16 rounding of the backward
    # activations happens at the same points; FP32 accumulation order can move
    # a rounding by one BF16 ulp (2^-8 relative), which the bound allows per
    # entry on top of 1e-3 of the largest entry
    gmax = np.abs(g).max()
    err = np.abs(g_gpu - g)
    big = np.abs(g) > 1e-2 * gmax
    rel = err[big] / np.abs(g[big])
    print("gradient: max rel %.3e on %d entries above 1e-2 max, median %.3e; max abs / max %.3e"
          % (rel.max(), big.sum(), np.median(rel), err.max() / gmax))
    assert (err <= 2.0 ** -8 * np.abs(g) + 1e-3 * gmax).all(), (err / (np.abs(g) + 1e-3 * gmax)).max()
    assert np.median(rel) < 1e-3
    # the first Adam step from zero moments is -lr g / (|g| + 1e-8) of the
    # kernels' own gradient (bias-corrected moments g and g^2)
    step = p1 - p0
    expect = -1e-3 * g_gpu / (np.abs(g_gpu) + 1e-8)
    tol = 2e-7 + 4 * np.finfo(np.float32).eps * np.abs(p0).max()  # rounding of p0 - lr (...) in FP32
    assert np.abs(step - expect).max() <= tol, np.abs(step - expect).max()
    # a learnable target: the loss falls by an order of magnitude
    loss = eq.mlp_train(ft.data_ptr(), tt.data_ptr(), n, 400, batch=4096, lr=3e-3, seed=seed + 1)
    assert loss[-20:].mean() < 0.1 * loss[:5].mean(), (loss[:5], loss[-5:])
