"""The learned scheduler's network: the CPU oracle pinned by finite differences (CPU), the device's forward and
backward kernels against the oracle, training on the device, the claim order, and what the trained model gains over
ordering by query length (GPU)."""

import numpy as np
import pytest

from oracle import cost_model as CM


def _problem(seed, n):
    rng = np.random.default_rng(seed)
    X = rng.random((n, CM.F)).astype(np.float32) * np.array([1, 1, 1, 1, 1, 1], np.float32)
    work = rng.integers(0, 5000, n).astype(np.uint64)
    p = (rng.standard_normal(CM.PARAMS) * 0.3).astype(np.float32)
    return X, work, p


def test_oracle_gradient_matches_finite_differences():
    X, work, p = _problem(1, 64)
    p = p.astype(np.float64)
    _, g = CM.loss_grad(p, X, work)
    rng = np.random.default_rng(2)
    idx = rng.choice(CM.PARAMS, 80, replace=False)
    eps = 1e-6
    for i in idx:
        d = np.zeros(CM.PARAMS)
        d[i] = eps
        num = (CM.loss(p + d, X, work) - CM.loss(p - d, X, work)) / (2 * eps)
        assert num == pytest.approx(g[i], rel=1e-4, abs=1e-7), i


def test_oracle_layout_covers_every_parameter():
    assert CM.PARAMS == 1313
    p = np.arange(CM.PARAMS, dtype=np.float64)
    W1, b1, W2, b2, w3, b3 = CM.unpack(p)
    flat = np.concatenate([W1.ravel(), b1, W2.ravel(), b2, w3, [b3]])
    np.testing.assert_array_equal(flat, p)


# ---------------------------------------------------------------------------------------------------------------- GPU
def _dev(a):
    import torch

    a = np.ascontiguousarray(a)
    t = torch.from_numpy(a.view(np.int64) if a.dtype == np.uint64 else a).cuda()
    torch.cuda.synchronize()
    return t


@pytest.mark.gpu
def test_device_gradient_matches_oracle(gpu_lib):
    from hibf_gb300.scheduler import cost_model

    X, work, p = _problem(3, 3000)
    m = cost_model(seed=5)
    m.params = p
    dX, dW = _dev(X), _dev(work)
    loss, g = m.loss_grad(dX.data_ptr(), dW.data_ptr(), X.shape[0])
    ref_loss, ref_g = CM.loss_grad(p.astype(np.float64), X, work)
    assert loss == pytest.approx(ref_loss, rel=1e-4)
    # float32 accumulation over 3,000 samples in a different order: relative to the gradient's scale
    scale = np.abs(ref_g).max()
    np.testing.assert_allclose(g, ref_g, rtol=2e-3, atol=2e-4 * scale)


@pytest.mark.gpu
def test_device_forward_matches_oracle_and_training_converges(gpu_lib):
    import torch

    from hibf_gb300.scheduler import cost_model

    rng = np.random.default_rng(7)
    X = rng.random((20000, CM.F)).astype(np.float32)
    # a target the network can represent: work grows with f0 and f2, and only when f4 > 0.5
    work = np.expm1(2 + 6 * X[:, 0] + 3 * X[:, 2] * (X[:, 4] > 0.5)).astype(np.uint64)
    m = cost_model(seed=11)
    dX, dW = _dev(X), _dev(work)
    pred = torch.empty(X.shape[0], dtype=torch.float32, device="cuda")
    m.predict(dX.data_ptr(), X.shape[0], pred.data_ptr())
    torch.cuda.synchronize()
    y, _, _ = CM.forward(m.params, X)
    np.testing.assert_allclose(pred.cpu().numpy(), y, rtol=1e-4, atol=1e-4)
    loss0, _ = m.loss_grad(dX.data_ptr(), dW.data_ptr(), X.shape[0])
    loss = m.train(dX.data_ptr(), dW.data_ptr(), X.shape[0], steps=400, lr=1e-2)
    assert loss < 0.05 * loss0 and loss < 0.2
    assert loss == pytest.approx(CM.loss(m.params, X, work), rel=1e-3)


@pytest.mark.gpu
def test_order_is_a_stable_descending_permutation(gpu_lib):
    import torch

    from hibf_gb300.scheduler import cost_model

    m = cost_model()
    keys = np.array([3.0, 1.0, 3.0, 7.0, -1.0, 1.0, 7.0], np.float32)
    dk = _dev(keys)
    order = torch.empty(keys.size, dtype=torch.int32, device="cuda")
    m.sort_desc(dk.data_ptr(), keys.size, order.data_ptr())
    torch.cuda.synchronize()
    assert order.cpu().numpy().tolist() == [3, 6, 0, 2, 1, 5, 4]
