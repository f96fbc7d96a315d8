"""Cost model: the hand-written MLP kernels against a plain PyTorch fp32
reference, the per-root level histograms against the trees, the logged
training data against the reference traversal counters, and the model
schedule against the static one (results must not depend on it)."""
from __future__ import annotations

import numpy as np
import pytest

from _util import INF32, assert_bc
from streamingbc_gb300 import graphs as G
from streamingbc_gb300 import native

pytestmark = pytest.mark.gpu

NIN, NH = 8, 64


def _split(P):
    o = 0
    W1 = P[o:o + NIN * NH].reshape(NIN, NH); o += NIN * NH
    b1 = P[o:o + NH]; o += NH
    W2 = P[o:o + NH * NH].reshape(NH, NH); o += NH * NH
    b2 = P[o:o + NH]; o += NH
    w3 = P[o:o + NH]; o += NH
    b3 = P[o:o + 1]; o += 1
    mu = P[o:o + NIN]; o += NIN
    isd = P[o:o + NIN]
    return W1, b1, W2, b2, w3, b3, mu, isd


def _torch_forward(P, x, grad=False):
    import torch
    t = [torch.tensor(a, dtype=torch.float32, requires_grad=grad) for a in _split(P)[:6]]
    mu, isd = (torch.tensor(a, dtype=torch.float32) for a in _split(P)[6:])
    W1, b1, W2, b2, w3, b3 = t
    xn = (torch.tensor(x, dtype=torch.float32) - mu) * isd
    h1 = torch.relu(xn @ W1 + b1)
    h2 = torch.relu(h1 @ W2 + b2)
    return h2 @ w3 + b3, t


def _random_params(rng):
    P = rng.normal(0, 0.3, size=NIN * NH + NH + NH * NH + NH + NH + 1 + 2 * NIN).astype(np.float32)
    P[-2 * NIN:-NIN] = rng.normal(0, 1, NIN)                # means
    P[-NIN:] = rng.uniform(0.5, 2.0, NIN).astype(np.float32)  # inverse std devs
    return P


def _small_forest():
    g = G.er(256, 1024, seed=5)
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, G.pick_roots(g.nv, 16, seed=5))
    f.static_init()
    return dg, f


def test_inference_matches_torch_fp32(sbc_lib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    dg, f = _small_forest()
    P = _random_params(rng)
    f.model_params(P)
    x = rng.normal(0, 2, size=(1000, NIN)).astype(np.float32)
    got = f.model_predict(x)
    with torch.no_grad():
        ref, _ = _torch_forward(P, x)
    ref = ref.numpy()
    np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-4 * max(1.0, float(np.abs(ref).max())))
    f.close()
    dg.close()


@pytest.mark.parametrize("n", [128, 300])
def test_gradient_matches_torch_autograd(sbc_lib, n):
    """One k_mlp_grad pass (mean squared error) against autograd; n = 300
    leaves a partly filled CTA."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n)
    dg, f = _small_forest()
    P = _random_params(rng)
    f.model_params(P)
    x = rng.normal(0, 2, size=(n, NIN)).astype(np.float32)
    y = rng.normal(0, 3, size=n).astype(np.float32)
    g, pred = f.model_grad(x, y)
    out, t = _torch_forward(P, x, grad=True)
    loss = ((out - torch.tensor(y)) ** 2).mean()
    loss.backward()
    ref = np.concatenate([p.grad.numpy().ravel() for p in t])
    np.testing.assert_allclose(pred, out.detach().numpy(), rtol=1e-4, atol=1e-4)
    scale = float(np.abs(ref).max())
    np.testing.assert_allclose(g, ref, rtol=1e-3, atol=1e-4 * scale)
    f.close()
    dg.close()


def _hist_from_dist(d):
    h = np.zeros((d.shape[0], 64), dtype=np.int64)
    for r in range(d.shape[0]):
        row = d[r][d[r] != INF32]
        h[r] = np.bincount(np.minimum(row, 63), minlength=64)
    return h


def test_level_histograms_stay_exact(sbc_lib):
    """After static init and after batches with re-levelling (case-2) jobs,
    each root's histogram equals the level counts of its tree."""
    g = G.rmat(14, 16, seed=3)
    roots = G.pick_roots(g.nv, 64, seed=3)
    ins = G.rmat_insertions(g, 14, 256, seed=3)
    dg = native.DeviceGraph(g.nv, g.off, g.adj)
    f = native.DeviceForest(dg, roots)
    f.static_init()
    np.testing.assert_array_equal(f.level_hist(), _hist_from_dist(f.dist()))
    case2 = 0
    for s in range(0, len(ins), 64):
        st = f.insert(ins[s:s + 64])
        case2 += st["case2"]
        np.testing.assert_array_equal(f.level_hist(), _hist_from_dist(f.dist()))
    assert case2 > 0
    f.close()
    dg.close()


def test_logging_training_and_model_schedule(sbc_lib):
    """Logged per-job costs add up to the reference traversal counter; a model
    trained on them beats predicting the mean; batches scheduled by the model
    (host and captured device batches) end exactly where the static schedule
    ends."""
    import torch
    g = G.rmat(14, 16, seed=7)
    roots = G.pick_roots(g.nv, 256, seed=7)
    ins = G.rmat_insertions(g, 14, 1024 + 512, seed=7)
    dgA = native.DeviceGraph(g.nv, g.off, g.adj)
    fA = native.DeviceForest(dgA, roots)
    dgB = native.DeviceGraph(g.nv, g.off, g.adj)
    fB = native.DeviceForest(dgB, roots)
    fA.static_init()
    fB.static_init()
    cap = 1 << 20
    fA.cost_log_start(cap)
    seen = 0
    for s in range(0, 1024, 64):
        st = fA.insert(ins[s:s + 64])
        fB.insert(ins[s:s + 64])
        n = fA.cost_log_stop()
        x, y = fA.cost_log_read(seen, n - seen)
        assert np.isfinite(x).all() and np.isfinite(y).all()
        touched = np.rint(np.expm1(y.astype(np.float64))).sum()
        assert touched == st["vertices"], (s, touched, st["vertices"])
        seen = n
        fA.cost_log_start(cap)
    fA.cost_log_stop()
    assert seen > 5000
    stats = fA.train_cost_model(epochs=20, batch=1024, lr=3e-3, val_frac=0.2, seed=3)
    assert stats["val_samples"] > 0
    assert stats["val_mae"] < 0.8 * stats["val_mae_mean"], stats
    fA.set_schedule(native.DeviceForest.SCHED_MODEL)
    rest = ins[1024:]
    d = torch.tensor(rest, dtype=torch.int32, device="cuda")
    du, dv = d[:, 0].contiguous(), d[:, 1].contiguous()
    dgA.reserve(rest)
    for k, s in enumerate(range(0, len(rest), 64)):
        if k == 0:
            ms_static, ms_model = fA.compare_schedules(rest[s:s + 64])
            assert ms_static > 0 and ms_model > 0
        elif k % 2 == 0:
            fA.insert(rest[s:s + 64])
        else:
            fA.insert_device(64, du[s:].data_ptr(), dv[s:].data_ptr())
            fA.sync()
        fB.insert(rest[s:s + 64])
    np.testing.assert_array_equal(fA.dist(), fB.dist())
    np.testing.assert_array_equal(fA.sigma(), fB.sigma())
    assert_bc(fA.bc(), fB.bc())
    fA.close()
    fB.close()
    dgA.close()
    dgB.close()
