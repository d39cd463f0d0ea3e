"""The moment-surrogate network: the CPU oracle (oracle/mlp.py) checked by
finite differences, and the GPU kernels (cusna_mlp_*) checked against it:
forward outputs, loss gradients, one Adam step and the input Jacobian.

Tolerances: the GPU rounds every product operand to bfloat16 and accumulates
in float32. Against the oracle with the same bfloat16 rounding the remaining
difference is float32 accumulation (plus rare one-ulp bfloat16 rounding flips
of an activation): relative error of the whole gradient vector <= 2e-3, of
forward outputs <= 2e-3. Against the unrounded float64 oracle (Jacobian, which
the GPU computes in float32 without rounding) <= 1e-4 relative."""
import numpy as np
import pytest

from oracle import mlp as OM

N_IN, H, N_OUT = 16, 64, 8


def _problem(seed=0, B=64, n_in=N_IN, hidden=H, n_out=N_OUT):
    rng = np.random.Generator(np.random.PCG64(seed))
    npar = OM.param_count(n_in, hidden, n_out)
    p = np.zeros(npar)
    W1, b1, W2, b2, W3, b3 = OM.unpack(p, n_in, hidden, n_out)
    W1[:] = rng.standard_normal(W1.shape) * np.sqrt(2.0 / n_in)
    b1[:] = 0.1 * rng.standard_normal(b1.shape)
    W2[:] = rng.standard_normal(W2.shape) * np.sqrt(2.0 / hidden)
    b2[:] = 0.1 * rng.standard_normal(b2.shape)
    W3[:] = rng.standard_normal(W3.shape) * np.sqrt(1.0 / hidden)
    b3[:] = 0.1 * rng.standard_normal(b3.shape)
    X = rng.standard_normal((B, n_in))
    T = rng.standard_normal((B, n_out))
    return p.astype(np.float32).astype(np.float64), X.astype(np.float32).astype(np.float64), \
        T.astype(np.float32).astype(np.float64)


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-30))


def test_oracle_gradient_matches_finite_differences():
    p, X, T = _problem(B=12, hidden=32)
    _, g = OM.loss_grad(p, X, T, N_IN, 32, N_OUT)
    rng = np.random.Generator(np.random.PCG64(1))
    idx = rng.choice(len(p), 60, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (OM.loss_grad(p + e, X, T, N_IN, 32, N_OUT)[0] -
              OM.loss_grad(p - e, X, T, N_IN, 32, N_OUT)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(g[i]), (i, fd, g[i])


def test_oracle_jacobian_matches_finite_differences():
    p, X, _ = _problem(B=3, hidden=32)
    J = OM.jacobian(p, X, N_IN, 32, N_OUT, 8)
    h = 1e-6
    for i in range(8):
        e = np.zeros(N_IN)
        e[i] = h
        fd = (OM.forward(p, X + e, N_IN, 32, N_OUT)[0] - OM.forward(p, X - e, N_IN, 32, N_OUT)[0]) / (2 * h)
        np.testing.assert_allclose(J[:, :, i], fd, rtol=1e-6, atol=1e-8)


def test_bf16_rounding_is_nearest_even():
    vals = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -3.14159, 0.0, 65504.0])
    r = OM.bf16_round(vals)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == 1.0
    assert abs(r[4] + 3.14159) < 2 ** -6 and r[5] == 0.0


def test_adam_oracle_first_step_is_signed_lr():
    p = np.array([1.0, -2.0, 0.5])
    g = np.array([0.3, -0.1, 0.0])
    p1, m, v = OM.adam(p, g, np.zeros(3), np.zeros(3), 1, lr=0.01)
    np.testing.assert_allclose(p1[:2], p[:2] - 0.01 * np.sign(g[:2]), rtol=1e-6)
    assert p1[2] == p[2]


# ---- GPU ---------------------------------------------------------------------
class _Gpu:
    def __init__(self, n_in=N_IN, hidden=H, n_out=N_OUT):
        import torch
        from cusna_gb300.abi import load_library
        self.torch = torch
        self.lib = load_library()
        self.dims = (n_in, hidden, n_out)
        self.dev = torch.device("cuda", 0)
        self.keep = []

    def t(self, a, dtype=None):
        """Device copy of a, kept alive as long as this object: a pointer taken
        from a temporary tensor would dangle once the tensor is freed."""
        dtype = dtype or self.torch.float32
        x = self.torch.from_numpy(np.ascontiguousarray(a)).to(self.dev, dtype)
        self.keep.append(x)
        return x

    def work(self, B):
        nb = int(self.lib.cusna_mlp_workspace_bytes(*self.dims, B))
        return self.torch.empty(nb, dtype=self.torch.uint8, device=self.dev), nb


@pytest.mark.gpu
def test_gpu_forward_matches_oracle():
    g = _Gpu()
    p, X, _ = _problem(B=100)           # batch not a multiple of 16: inference allows it
    w, nb = g.work(100)
    y = g.torch.empty((100, N_OUT), device=g.dev)
    st = g.lib.cusna_mlp_forward(g.t(p).data_ptr(), g.t(X).data_ptr(), 100, y.data_ptr(),
                                 w.data_ptr(), nb, N_IN, H, N_OUT, None)
    assert st == 0
    y = y.double().cpu().numpy()
    y_bf, _ = OM.forward(p, X, N_IN, H, N_OUT, bf16=True)
    y_64, _ = OM.forward(p, X, N_IN, H, N_OUT)
    assert _rel(y, y_bf) < 2e-3
    assert _rel(y, y_64) < 3e-2             # bfloat16 operands against exact arithmetic


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [(16, 64, 8), (16, 256, 8), (32, 128, 5)])
def test_gpu_gradient_matches_oracle(dims):
    n_in, hidden, n_out = dims
    g = _Gpu(*dims)
    B = 128
    p, X, T = _problem(seed=3, B=B, n_in=n_in, hidden=hidden, n_out=n_out)
    w, nb = g.work(B)
    grad = g.torch.zeros(len(p), device=g.dev)
    loss = g.torch.zeros(1, device=g.dev)
    st = g.lib.cusna_mlp_grad(g.t(p).data_ptr(), g.t(X).data_ptr(), g.t(T).data_ptr(), None, B,
                              grad.data_ptr(), loss.data_ptr(), w.data_ptr(), nb, n_in, hidden,
                              n_out, None)
    assert st == 0
    gg = grad.double().cpu().numpy()
    l_bf, g_bf = OM.loss_grad(p, X, T, n_in, hidden, n_out, bf16=True)
    l_64, g_64 = OM.loss_grad(p, X, T, n_in, hidden, n_out)
    assert abs(loss.item() - l_bf) <= 2e-3 * l_bf
    assert _rel(gg, g_bf) < 2e-3, _rel(gg, g_bf)
    assert _rel(gg, g_64) < 3e-2
    # every parameter block individually (a transposed or misplaced block would
    # not hide in the global norm)
    o = 0
    for sz in (hidden * n_in, hidden, hidden * hidden, hidden, n_out * hidden, n_out):
        assert _rel(gg[o:o + sz], g_bf[o:o + sz]) < 5e-3
        o += sz


@pytest.mark.gpu
def test_gpu_gradient_at_batch_1024_matches_oracle_and_repeats_exactly():
    """The surrogate's training batch (1024 rows, hidden width 256): the
    weight-gradient products reduce over the whole batch (K = 1024, sixteen
    chunks through the stage ring); the gradient matches the oracle's and two
    calls agree bit for bit."""
    n_in, hidden, n_out = 16, 256, 8
    g = _Gpu(n_in, hidden, n_out)
    B = 1024
    p, X, T = _problem(seed=21, B=B, n_in=n_in, hidden=hidden, n_out=n_out)
    w, nb = g.work(B)
    grads = []
    for _ in range(2):
        grad = g.torch.zeros(len(p), device=g.dev)
        st = g.lib.cusna_mlp_grad(g.t(p).data_ptr(), g.t(X).data_ptr(), g.t(T).data_ptr(), None,
                                  B, grad.data_ptr(), None, w.data_ptr(), nb, n_in, hidden,
                                  n_out, None)
        assert st == 0
        grads.append(grad.double().cpu().numpy())
    np.testing.assert_array_equal(grads[0], grads[1])
    _, g_bf = OM.loss_grad(p, X, T, n_in, hidden, n_out, bf16=True)
    assert _rel(grads[0], g_bf) < 2e-3, _rel(grads[0], g_bf)
    o = 0
    for sz in (hidden * n_in, hidden, hidden * hidden, hidden, n_out * hidden, n_out):
        assert _rel(grads[0][o:o + sz], g_bf[o:o + sz]) < 5e-3
        o += sz


@pytest.mark.gpu
def test_gpu_gradient_with_row_selection():
    g = _Gpu()
    p, X, T = _problem(seed=5, B=96)
    rows = np.array(list(range(95, 47, -1)) + list(range(0, 48, 3)) + list(range(1, 48, 3)), np.int32)[:64]
    B = 64
    w, nb = g.work(B)
    grad = g.torch.zeros(len(p), device=g.dev)
    st = g.lib.cusna_mlp_grad(g.t(p).data_ptr(), g.t(X).data_ptr(), g.t(T).data_ptr(),
                              g.t(rows, g.torch.int32).data_ptr(), B, grad.data_ptr(), None,
                              w.data_ptr(), nb, N_IN, H, N_OUT, None)
    assert st == 0
    _, g_bf = OM.loss_grad(p, X[rows], T[rows], N_IN, H, N_OUT, bf16=True)
    assert _rel(grad.double().cpu().numpy(), g_bf) < 2e-3


@pytest.mark.gpu
def test_gpu_adam_step_matches_oracle():
    g = _Gpu()
    B = 64
    p, X, T = _problem(seed=7, B=B)
    w, nb = g.work(B)
    P = g.t(p)
    grad = g.torch.zeros(len(p), device=g.dev)
    m = g.torch.zeros(len(p), device=g.dev)
    v = g.torch.zeros(len(p), device=g.dev)
    pc, mc, vc = p.copy(), np.zeros(len(p)), np.zeros(len(p))
    for step in (1, 2, 3):
        # the oracle step uses the GPU's gradient, so only the update is compared
        st = g.lib.cusna_mlp_train_step(P.data_ptr(), grad.data_ptr(), m.data_ptr(), v.data_ptr(),
                                        g.t(X).data_ptr(), g.t(T).data_ptr(), None, B, step,
                                        1e-3, 0.9, 0.999, 1e-8, None, w.data_ptr(), nb, N_IN,
                                        H, N_OUT, None)
        assert st == 0
        gs = grad.double().cpu().numpy()
        pc, mc, vc = OM.adam(pc, gs, mc, vc, step, lr=1e-3)
        np.testing.assert_allclose(P.double().cpu().numpy(), pc, rtol=0, atol=2e-6)


@pytest.mark.gpu
def test_gpu_jacobian_matches_oracle():
    g = _Gpu()
    p, X, _ = _problem(seed=9, B=5)
    w, nb = g.work(5)
    y = g.torch.empty((5, N_OUT), device=g.dev)
    J = g.torch.empty((5, N_OUT, 8), device=g.dev)
    st = g.lib.cusna_mlp_jacobian(g.t(p).data_ptr(), g.t(X).data_ptr(), 5, 8, y.data_ptr(),
                                  J.data_ptr(), w.data_ptr(), nb, N_IN, H, N_OUT, None)
    assert st == 0
    Jo = OM.jacobian(p, X, N_IN, H, N_OUT, 8)
    # the Jacobian reads float32 pre-activations of the bfloat16 forward pass
    assert _rel(J.double().cpu().numpy(), Jo) < 2e-2


@pytest.mark.gpu
def test_gpu_shape_errors():
    g = _Gpu()
    w, nb = g.work(32)
    grad = g.torch.zeros(10, device=g.dev)
    x = g.torch.zeros(1024, device=g.dev)
    # training batch not a multiple of 16
    assert g.lib.cusna_mlp_grad(x.data_ptr(), x.data_ptr(), x.data_ptr(), None, 24,
                                grad.data_ptr(), None, w.data_ptr(), nb, N_IN, H, N_OUT, None) == 2
    # workspace too small for the batch
    assert g.lib.cusna_mlp_forward(x.data_ptr(), x.data_ptr(), 64, x.data_ptr(), w.data_ptr(), nb,
                                   N_IN, H, N_OUT, None) == 2
    # n_in not a multiple of 16, n_out above 16
    assert g.lib.cusna_mlp_forward(x.data_ptr(), x.data_ptr(), 8, x.data_ptr(), w.data_ptr(), nb,
                                   12, H, N_OUT, None) == 2
    assert g.lib.cusna_mlp_forward(x.data_ptr(), x.data_ptr(), 8, x.data_ptr(), w.data_ptr(), nb,
                                   N_IN, H, 17, None) == 2
    assert g.lib.cusna_mlp_forward(None, x.data_ptr(), 8, x.data_ptr(), w.data_ptr(), nb,
                                   N_IN, H, N_OUT, None) == 1


@pytest.mark.gpu
def test_gpu_training_learns_a_smooth_map():
    """Adam on the GPU drives the loss on a smooth synthetic regression from
    its initial value to well below it (held-out rows)."""
    from cusna_gb300.surrogate import MlpSurrogate
    rng = np.random.Generator(np.random.PCG64(11))
    X = rng.standard_normal((8192, 16))
    A = rng.standard_normal((16, 8)) / 4
    Y = np.tanh(X @ A) + 0.5 * (X[:, :8] ** 2)
    net = MlpSurrogate(16, 8, 128, seed=1)
    info = net.fit(X, Y, epochs=60, batch=512, lr=3e-3, seed=2)
    hist = info["history"]
    assert hist[-1]["val"] < 0.1 * hist[0]["train"], hist[-1]
    Xt = rng.standard_normal((256, 16))
    Yt = np.tanh(Xt @ A) + 0.5 * (Xt[:, :8] ** 2)
    r2 = 1 - ((net.predict(Xt) - Yt) ** 2).sum() / ((Yt - Yt.mean(axis=0)) ** 2).sum()
    assert r2 > 0.9, r2


@pytest.mark.gpu
def test_gpu_train_steps_graph_replay_is_identical_to_direct_launches():
    """cusna_mlp_train_steps replayed from its CUDA graph gives bit-identical
    parameters to the same steps launched directly, across two replays with
    new minibatch rows and a new learning rate written between them; both
    agree with the single-step entry point up to float32 rounding of the
    bias corrections (device powf against host powf)."""
    from cusna_gb300.abi import adam_hyper_bytes
    g = _Gpu()
    B, S = 32, 3
    p, X, T = _problem(seed=13, B=256)
    w, nb = g.work(B)
    rng = np.random.Generator(np.random.PCG64(2))
    rows1 = rng.permutation(256)[:B * S].astype(np.int32)
    rows2 = rng.permutation(256)[:B * S].astype(np.int32)
    Xd, Td = g.t(X), g.t(T)
    out = []
    for graph in (1, 0):
        P = g.t(p)
        grad, m, v = (g.torch.zeros(len(p), device=g.dev) for _ in range(3))
        rows = g.torch.empty(B * S, dtype=g.torch.int32, device=g.dev)
        hyper = g.torch.from_numpy(adam_hyper_bytes(0, 1e-3)).to(g.dev)
        losses = g.torch.zeros(S, device=g.dev)
        for rr, lr in ((rows1, 1e-3), (rows2, 5e-4)):
            rows.copy_(g.torch.from_numpy(rr))
            hyper[4:8].copy_(g.torch.from_numpy(np.array([lr], np.float32).view(np.uint8)))
            st = g.lib.cusna_mlp_train_steps(P.data_ptr(), grad.data_ptr(), m.data_ptr(),
                                             v.data_ptr(), Xd.data_ptr(), Td.data_ptr(),
                                             rows.data_ptr(), B, S, hyper.data_ptr(),
                                             losses.data_ptr(), w.data_ptr(), nb, N_IN, H, N_OUT,
                                             graph, None)
            assert st == 0
        g.torch.cuda.synchronize()
        assert int(hyper[:4].cpu().numpy().view(np.int32)[0]) == 2 * S
        out.append(P.double().cpu().numpy())
    np.testing.assert_array_equal(out[0], out[1])
    # the single-step entry point, host-side bias corrections
    P = g.t(p)
    grad, m, v = (g.torch.zeros(len(p), device=g.dev) for _ in range(3))
    step = 0
    for rr, lr in ((rows1, 1e-3), (rows2, 5e-4)):
        rows = g.t(rr, g.torch.int32)
        for s in range(S):
            step += 1
            assert g.lib.cusna_mlp_train_step(P.data_ptr(), grad.data_ptr(), m.data_ptr(),
                                              v.data_ptr(), Xd.data_ptr(), Td.data_ptr(),
                                              rows.data_ptr() + 4 * s * B, B, step, lr, 0.9,
                                              0.999, 1e-8, None, w.data_ptr(), nb, N_IN, H,
                                              N_OUT, None) == 0
    np.testing.assert_allclose(P.double().cpu().numpy(), out[0], rtol=0, atol=1e-6)
