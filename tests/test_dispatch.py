"""The learned dispatcher: descriptor generation and scoring on the CPU;
on the GPU the features kernel against numpy, the MLP inference and
training kernels against a PyTorch fp32 reference of the same network, a
small end-to-end sweep (autotune, train, evaluate), and gcvl_auto_run
computing what the default kernel computes."""
import numpy as np
import pytest

from neslgpu_gb300 import dispatch as D
from neslgpu_gb300 import workloads as W

F, H, K, STRIDE = 16, 64, 8, 24


@pytest.mark.parametrize("dist", D.DISTS)
def test_lengths_for(dist):
    r = W.rng(3)
    for n in (1 << 16, 100_003, 1 << 20):
        L = D.lengths_for(r, dist, n, 1 << 14)
        assert L.sum() == n and L.min() >= 0 and len(L) <= 1 << 14


def test_soft_targets_and_evaluate():
    t = np.array([[1.0, 1.01, 2.0, np.inf, np.inf, np.inf, ],
                  [2.0, np.inf, np.inf, np.inf, np.inf, 1.0]])
    T = D.soft_targets(t)
    assert np.allclose(T.sum(axis=1), 1.0)
    assert T[0, 0] > T[0, 1] > T[0, 2] and T[0, 3] == 0 and T[1, 5] > 0.99
    ev = D.evaluate(t, np.array([1, 0]))
    assert abs(ev["regret_mean"] - (0.01 + 1.0) / 2) < 1e-12
    assert abs(ev["speedup_vs_plain"] - 3.0 / 3.01) < 1e-12


def _torch_forward(p, X):
    torch = pytest.importorskip("torch")
    pt = torch.tensor(p, dtype=torch.float32)
    o = 0
    def take(k):
        nonlocal o
        v = pt[o:o + k]; o += k; return v
    W1 = take(F * H).view(F, H); b1 = take(H); W2 = take(H * H).view(H, H); b2 = take(H)
    W3 = take(H * K).view(H, K); b3 = take(K)
    x = torch.tensor(X[:, :F], dtype=torch.float32)
    h1 = torch.relu(x @ W1 + b1)
    h2 = torch.relu(h1 @ W2 + b2)
    z = h2 @ W3 + b3
    mask = torch.tensor(X[:, F:], dtype=torch.float32) > 0
    return z.masked_fill(~mask, float("-inf"))


def _random_rows(r, N):
    X = np.zeros((N, STRIDE), dtype=np.float32)
    X[:, :F] = r.random((N, F))
    X[:, F] = 1
    X[:, F + 1:F + 6] = r.random((N, 5)) < 0.6
    return X


@pytest.mark.gpu
def test_mlp_infer_matches_torch(gpu):
    c = gpu.cvl
    r = np.random.default_rng(5)
    p = D.init_params(c, 11)
    X = _random_rows(r, 333)
    P, XD, cls = D.DevF32(c, p), D.DevF32(c, X), D.DevF32(c, size=len(X))
    assert c.gcvl_mlp_infer(P.ptr, XD.ptr, len(X), cls.ptr) == 0
    got = cls.get(np.int32)
    for a in (P, XD, cls):
        a.free()
    z = _torch_forward(p, X).numpy()
    want = z.argmax(axis=1)
    srt = np.sort(z, axis=1)
    clear = (srt[:, -1] - srt[:, -2]) > 1e-4  # no near-tie at the top
    assert np.array_equal(got[clear], want[clear])
    assert np.all(X[np.arange(len(X)), F + got] > 0)  # never an invalid class


@pytest.mark.gpu
def test_mlp_train_steps_match_torch(gpu):
    """Two Adam steps over one full batch each: the kernel's parameters
    against autograd + Adam in fp32 (lr 1e-3, betas 0.9 / 0.999, eps 1e-8).
    The second step depends on the ratio of the two steps' gradients, so
    magnitudes are checked as well as signs."""
    torch = pytest.importorskip("torch")
    c = gpu.cvl
    r = np.random.default_rng(6)
    N, lr = 96, 1e-3
    X = _random_rows(r, N)
    times = np.where(X[:, F:F + 6] > 0, 1.0 + r.random((N, 6)), np.inf)
    T = D.soft_targets(times)
    p0 = D.init_params(c, 12)
    P, M = D.DevF32(c, p0), D.DevF32(c, np.zeros(2 * p0.size, dtype=np.float32))
    XD, TD = D.DevF32(c, X), D.DevF32(c, T)
    assert c.gcvl_mlp_train(P.ptr, M.ptr, XD.ptr, TD.ptr, N, 2, N, lr, 1, 0, None) == 0
    got = P.get()
    for a in (P, M, XD, TD):
        a.free()

    x = torch.tensor(X[:, :F])
    invalid = torch.tensor(X[:, F:]) <= 0
    tt = torch.tensor(T)
    p = torch.tensor(p0)
    m1 = torch.zeros_like(p)
    m2 = torch.zeros_like(p)
    for step in (1, 2):
        q = p.clone().requires_grad_(True)
        o, parts = 0, []
        for k in (F * H, H, H * H, H, H * K, K):
            parts.append(q[o:o + k]); o += k
        W1, b1, W2, b2, W3, b3 = parts
        h1 = torch.relu(x @ W1.view(F, H) + b1)
        h2 = torch.relu(h1 @ W2.view(H, H) + b2)
        z = (h2 @ W3.view(H, K) + b3).masked_fill(invalid, float("-inf"))
        logp = torch.log_softmax(z, dim=1)
        loss = -(tt * torch.where(tt > 0, logp, torch.zeros_like(logp))).sum() / N
        loss.backward()
        g = q.grad.detach()
        m1 = 0.9 * m1 + 0.1 * g
        m2 = 0.999 * m2 + 0.001 * g * g
        p = p - lr * (m1 / (1 - 0.9 ** step)) / (torch.sqrt(m2 / (1 - 0.999 ** step)) + 1e-8)
    want = p.numpy()
    moved = np.abs(want - p0) > 1e-4
    assert moved.sum() > 1000
    np.testing.assert_allclose(got[moved], want[moved], rtol=0, atol=2e-5)


def _features_numpy(lens, kind, is_double):
    n, m = int(lens.sum()), len(lens)
    mean = n / m
    var = max(0.0, float((lens.astype(np.float64) ** 2).mean() - mean * mean))
    f = np.zeros(16)
    f[0] = np.log2(n + 1) / 32; f[1] = np.log2(m + 1) / 32; f[2] = np.log2(mean + 1) / 24
    f[3] = np.log2(np.sqrt(var) + 1) / 24; f[4] = np.log2(lens.max() + 1) / 24
    f[5] = lens[lens >= 65536].sum() / n
    edges = [0, 4, 32, 256, 2048, 65536, 1 << 40]
    for k in range(6):
        f[6 + k] = ((lens >= edges[k]) & (lens < edges[k + 1])).mean()
    f[12 + kind] = 1; f[15] = is_double
    return f


@pytest.mark.gpu
@pytest.mark.parametrize("prim,kind,dbl", [("add_sez", 0, 0), ("add_red", 1, 1), ("rku_lez", 2, 0)])
def test_features_kernel(gpu, prim, kind, dbl):
    c = gpu.cvl
    r = W.rng(9)
    lens = D.lengths_for(r, "bimodal", 1 << 20, 1 << 18)
    sd, n, m = gpu.segd(lens)
    out = D.DevF32(c, size=STRIDE)
    assert c.gcvl_seg_features(prim.encode(), sd.ptr, n, m, out.ptr) == 0
    got = out.get()
    out.free()
    np.testing.assert_allclose(got[:16], _features_numpy(lens, kind, dbl), rtol=1e-5, atol=1e-6)
    mask = got[16:]
    assert mask[0] == 1
    if kind == 2:
        assert mask[1:5].sum() == 0 and mask[5] == (lens.max() <= 2048)
    else:
        assert mask[1:5].sum() == 4 and mask[5] == 0


@pytest.mark.gpu
def test_small_sweep_train_and_auto_run(gpu, oracle):
    c = gpu.cvl
    insts, X = D.sweep(48, seed=3, lo=12, hi=18, max_m=1 << 16, reps=1, cvl=c)
    for i in insts:
        assert np.isfinite(i.times[0]) and i.times[i.best] <= i.times[0]
    res = D.train(insts, X, seed=4, epochs=60, batch=16, cvl=c)
    assert res["loss_last"] < res["loss_first"]
    assert res["regret_mean"] >= 0 and res["speedup_vs_plain"] > 0
    # the installed model changes only how: gcvl_auto_run against the oracle
    from neslgpu_gb300 import ops
    c.gcvl_dispatch_set_model(res["params"].ctypes.data)
    try:
        r = W.rng(10)
        lens = W.geometric_lengths(r, 50_000, 40.0)
        x = r.integers(-100, 100, size=50_000).astype(np.int32)
        sd, n, m = gpu.segd(lens)
        xs, d = gpu.vec(x, "z"), gpu.out(n, "z")
        scr = gpu.units(c.gcvl_variant_scratch(b"add_sez", n, m))
        assert c.gcvl_auto_run(b"add_sez", d.ptr, xs.ptr, sd.ptr, n, m, scr.ptr) == 0
        np.testing.assert_array_equal(gpu.get(d, n), ops.scan_e(oracle, "add_sez", x, lens))
        assert 0 <= c.gcvl_dispatch_choice(b"add_sez", sd.ptr, n, m) < 5
    finally:
        c.gcvl_dispatch_set_model(None)
