"""The warm-start MLP on the tensor cores (tcgen05, BF16 operands, FP32
accumulation) against the CPU oracle (oracle/mlp_oracle.py).

Bars: products within 1e-5 of exact (FP32 accumulation of exact BF16
products); forward outputs within 2e-3 and gradients within 1e-2
norm-relative of the oracle, which rounds in the same places (the residual
difference comes from BF16 roundings of activations that FP32 accumulation
order tips the other way, and erf/exp in FP32); a short training run lowers
the loss by 50x."""
import ctypes as C

import numpy as np
import pytest

import mlp_oracle as mo

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L():
    from pd_gpu1_gb300._lib import lib

    return lib()


def _dev(a, dtype):
    import torch

    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


@pytest.mark.parametrize("M,N,K,tr", [(128, 128, 64, 0), (300, 128, 200, 0), (257, 16, 16, 0), (1000, 128, 128, 0),
                                      (128, 128, 777, 1), (130, 256, 48, 0)])
def test_gemm_matches_exact(L, M, N, K, tr):
    import torch

    rng = np.random.default_rng(M + N + K)
    a = mo.bf16(rng.standard_normal((M, K)).astype(np.float32))
    b = mo.bf16(rng.standard_normal((N, K)).astype(np.float32))
    da = _dev(a.T.copy() if tr else a, torch.bfloat16)
    db = _dev(b, torch.bfloat16)
    dd = torch.zeros((M, N), dtype=torch.float32, device="cuda")
    assert L.pd_mlp_gemm(da.data_ptr(), db.data_ptr(), M, N, K, dd.data_ptr(), tr, None) == 0
    want = a.astype(np.float64) @ b.astype(np.float64).T
    got = dd.cpu().numpy().astype(np.float64)
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()


def _net(L, rows):
    st = C.c_int()
    n = L.pd_mlp_create(rows, C.byref(st))
    assert n, st.value
    return n


def _problem(seed, M):
    rng = np.random.default_rng(seed)
    x = np.zeros((M, 16), dtype=np.float32)
    x[:, :8] = rng.uniform(-1, 1, (M, 8))
    x = mo.bf16(x)
    t = np.stack([x[:, 0] + 0.3 * np.sin(3 * x[:, 5]), x[:, 1] - 0.2 * x[:, 6] ** 2], axis=1).astype(np.float32)
    return x, t


def test_forward_and_gradient_match_oracle(L):
    import torch

    M = 777
    p = mo.init_params(7)
    rng = np.random.default_rng(11)
    p = (p + 0.01 * rng.standard_normal(p.size)).astype(np.float32)  # nonzero biases
    x, t = _problem(5, M)
    n = _net(L, 1024)
    assert L.pd_mlp_set_params(n, p.ctypes.data, p.size) == 0
    dx, dt = _dev(x, torch.bfloat16), _dev(t, torch.float32)
    dy = torch.zeros((M, 2), dtype=torch.float32, device="cuda")
    assert L.pd_mlp_forward(n, dx.data_ptr(), M, dy.data_ptr(), None) == 0
    y_or, _ = mo.forward(p, x[:, :8])
    y = dy.cpu().numpy()
    assert np.abs(y - y_or).max() <= 2e-3 * np.abs(y_or).max()
    g = np.zeros(mo.N_PARAMS, dtype=np.float32)
    loss = C.c_float()
    assert L.pd_mlp_grad(n, dx.data_ptr(), dt.data_ptr(), M, g.ctypes.data, C.byref(loss), None) == 0
    g_or, loss_or = mo.grad(p, x[:, :8], t)
    assert loss.value == pytest.approx(loss_or, rel=1e-3)
    for name, (lo, hi) in _slices().items():
        err = np.linalg.norm(g[lo:hi] - g_or[lo:hi]) / np.linalg.norm(g_or[lo:hi])
        assert err <= 1e-2, (name, err)
    L.pd_mlp_destroy(n)


def test_fused_forward_equals_layer_by_layer(L):
    """The fused forward pass (one persistent kernel, the four layers per
    128-row tile with weights and activations on chip) against the layer-by-
    layer pass (one tensor-core product per layer through device memory):
    the same products and epilogues, so the outputs agree bit for bit.  Row
    counts: one partial tile (the input tile's missing rows read as zero), a
    full tile and one row, and a count that leaves a partial last tile and
    spans several passes of the persistent grid (the next input tile is
    fetched while the current one runs)."""
    import torch

    p = mo.init_params(3)
    rng = np.random.default_rng(5)
    p = (p + 0.05 * rng.standard_normal(p.size)).astype(np.float32)
    n = _net(L, 65536)
    assert L.pd_mlp_set_params(n, p.ctypes.data, p.size) == 0
    for M in (100, 129, 300_001):
        x, _ = _problem(9, M)
        dx = _dev(x, torch.bfloat16)
        y1 = torch.zeros((M, 2), dtype=torch.float32, device="cuda")
        y2 = torch.ones((M, 2), dtype=torch.float32, device="cuda")
        assert L.pd_mlp_forward(n, dx.data_ptr(), M, y1.data_ptr(), None) == 0
        assert L.pd_mlp_forward_layers(n, dx.data_ptr(), M, y2.data_ptr(), None) == 0
        a, b = y1.cpu().numpy(), y2.cpu().numpy()
        assert np.abs(a).max() > 0.0
        np.testing.assert_array_equal(a, b, err_msg=str(M))
    L.pd_mlp_destroy(n)


def _slices():
    out, o = {}, 0
    for name, shape in mo.SHAPES:
        k = int(np.prod(shape))
        out[name] = (o, o + k)
        o += k
    return out


def test_training_lowers_loss(L):
    import torch

    M = 8192
    x, t = _problem(9, M)
    n = _net(L, M)
    p = mo.init_params(3)
    assert L.pd_mlp_set_params(n, p.ctypes.data, p.size) == 0
    dx, dt = _dev(x, torch.bfloat16), _dev(t, torch.float32)
    loss = C.c_float()
    first = None
    for k in range(400):
        assert L.pd_mlp_train_step(n, dx.data_ptr(), dt.data_ptr(), M, C.c_float(3e-3), C.byref(loss), None) == 0
        if first is None:
            first = loss.value
    assert loss.value < first / 50.0, (first, loss.value)
    q = np.zeros(mo.N_PARAMS, dtype=np.float32)
    assert L.pd_mlp_get_params(n, q.ctypes.data, q.size) == 0
    assert np.isfinite(q).all() and not np.array_equal(q, p)
    L.pd_mlp_destroy(n)


@pytest.mark.parametrize("K", [64, 200])
def test_bounded_wait_gives_up_and_reports_timeout(L, K):
    """The tensor-core kernel's mbarrier wait is bounded.  With no product and
    no commit issued the barrier never completes: the kernel gives up after
    the given number of iterations, frees its tensor memory and returns, and
    the call reports PD_ERR_TIMEOUT (-7).  The same call with the products
    issued then completes and is exact, so the GPU and the context stay
    usable after a wait ran out (K = 200 also runs out inside the chunk loop,
    before the last chunk)."""
    import torch

    M, N = 256, 128
    rng = np.random.default_rng(K)
    a = mo.bf16(rng.standard_normal((M, K)).astype(np.float32))
    b = mo.bf16(rng.standard_normal((N, K)).astype(np.float32))
    da, db = _dev(a, torch.bfloat16), _dev(b, torch.bfloat16)
    dd = torch.zeros((M, N), dtype=torch.float32, device="cuda")
    rc = L.pd_mlp_gemm_wait_check(da.data_ptr(), db.data_ptr(), M, N, K, dd.data_ptr(), 0, 2000, 0, None)
    assert rc == -7
    assert float(dd.abs().max().item()) == 0.0  # gave up before its epilogue
    rc = L.pd_mlp_gemm_wait_check(da.data_ptr(), db.data_ptr(), M, N, K, dd.data_ptr(), 0, 2000000, 1, None)
    assert rc == 0
    want = a.astype(np.float64) @ b.astype(np.float64).T
    got = dd.cpu().numpy().astype(np.float64)
    assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max()
