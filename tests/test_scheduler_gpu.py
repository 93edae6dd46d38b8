"""What the learned scheduler gains, measured: on the 8,192-user-bin workload's layout (user bins scaled to 1% so the
index builds in a second), a model trained on one batch's measured per-query work predicts another batch's work
better than the query length does (rank correlation), and the persistent kernel, claiming root tasks in the order of
its prediction, answers that batch faster than in query order (the kernel's claim order without a scheduler) by CUDA
events.  Ordering by query length, a heuristic that needs no model, is timed beside it and reported: on this
workload it captures nearly the same gain (the learned part's margin over it is within a few percent)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ranks(x):
    r = np.empty(x.size)
    r[np.argsort(x, kind="stable")] = np.arange(x.size)
    return r


def spearman(a, b):
    return float(np.corrcoef(_ranks(np.asarray(a, float)), _ranks(np.asarray(b, float)))[0, 1])


def _batch(wl, offs, first, n):
    import torch

    qo, thr = wl.query_offsets(first, n)
    v = wl.queries_host(offs, first, n, qo)
    dv = torch.from_numpy(v.view(np.int64)).cuda()
    dq = torch.from_numpy(qo.view(np.int64)).cuda()
    dt = torch.from_numpy(thr.view(np.int64)).cuda()
    return qo, thr, v, dv, dq, dt


def _features_and_work(agent, b, n):
    import torch

    qo, thr, v, dv, dq, dt = b
    feats = torch.zeros(n * 6, dtype=torch.float32, device="cuda")
    work = torch.zeros(n, dtype=torch.int64, device="cuda")
    agent.query_features(dv.data_ptr(), dq.data_ptr(), n, dt.data_ptr(), 32, feats.data_ptr())
    agent.set_work_out(work.data_ptr(), n)
    agent.query_batch_device(dv.data_ptr(), dq.data_ptr(), n, dt.data_ptr())
    agent.status()
    agent.set_work_out(None)
    torch.cuda.synchronize()
    return feats, work


def test_learned_order_shortens_the_measured_kernel(gpu_lib):
    import torch

    from hibf_gb300 import build as B
    from hibf_gb300.scheduler import cost_model
    from hibf_gb300.workloads import HIBF8192 as wl

    offs = wl.user_bin_offsets()
    sizes = np.maximum(1, np.floor(np.diff(offs.astype(np.float64)) * 0.01)).astype(np.uint64)
    offs = np.zeros(sizes.size + 1, np.uint64)
    np.cumsum(sizes, out=offs[1:])
    cfg = B.config(number_of_user_bins=wl.n_user_bins, number_of_hash_functions=wl.h, maximum_fpr=wl.fpr)
    hibf = B.build_synthetic(cfg, wl.layout_text(), wl.query.seed, offs)
    agent = hibf.membership_agent()
    n = 20000
    agent.reserve(n, 40_000_000, n * 8, n * 8)
    train = _batch(wl, offs, 0, n)
    test = _batch(wl, offs, 500_000, n)
    f_tr, w_tr = _features_and_work(agent, train, n)
    f_te, w_te = _features_and_work(agent, test, n)

    model = cost_model(seed=3)
    loss = model.train(f_tr.data_ptr(), w_tr.data_ptr(), n, steps=500, lr=1e-2)
    pred = torch.empty(n, dtype=torch.float32, device="cuda")
    model.predict(f_te.data_ptr(), n, pred.data_ptr())
    torch.cuda.synchronize()
    work = w_te.cpu().numpy().view(np.uint64).astype(np.float64)
    length = np.diff(test[0]).astype(np.float64)
    rho_learned = spearman(pred.cpu().numpy(), work)
    rho_length = spearman(length, work)
    assert loss < 1.0
    assert rho_learned > rho_length + 0.05, (rho_learned, rho_length)

    order = torch.empty(n, dtype=torch.int32, device="cuda")
    model.order(f_te.data_ptr(), n, order.data_ptr())
    torch.cuda.synchronize()
    learned = order.cpu().numpy().astype(np.int64)
    assert np.array_equal(np.sort(learned), np.arange(n))
    by_length = torch.from_numpy(np.argsort(-length, kind="stable").astype(np.int32)).cuda()
    qo, thr, v, dv, dq, dt = test

    def kernel_ms(d_order):
        agent.set_order(d_order.data_ptr() if d_order is not None else None, n)
        ks = []
        for _ in range(9):
            agent.query_batch_device(dv.data_ptr(), dq.data_ptr(), n, dt.data_ptr())
            agent.status()
            ks.append(agent.kernel_ms())
        agent.set_order(None)
        return float(np.median(ks[2:]))

    t_query, t_length, t_learned = (kernel_ms(o) for o in (None, by_length, order))
    # the model's order against the claim order without a scheduler; length order reported beside it
    assert t_learned < 0.95 * t_query, dict(query=t_query, length=t_length, learned=t_learned)
    print(f"kernel ms: query order {t_query:.4f}, length order {t_length:.4f}, learned order {t_learned:.4f}")

    # the ordered batch answers exactly as the unordered one
    base = agent.query_batch(v, qo, thr)
    agent.set_order(order.data_ptr(), n)
    got = agent.query_batch(v, qo, thr)
    agent.set_order(None)
    np.testing.assert_array_equal(base[0], got[0])
    np.testing.assert_array_equal(base[1], got[1])
