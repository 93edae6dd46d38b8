"""The learned scheduler: a small MLP (trained on the GPU by the library's own kernels) predicts each query's work
from cheap features, and the persistent kernel claims root tasks largest-first (see csrc/cost_model.cu).

    model = cost_model(seed=1)
    agent.query_features(d_values, d_qoff, nq, d_thr, probe=16, d_features=F)   # float32 [nq, 6]
    agent.set_work_out(W)                                                        # uint64 [nq] targets
    agent.query_batch_device(...)                                                # records the work
    model.train(F, W, nq, steps=300)
    model.order(F2, nq2, d_order)        # claim order for another batch
    agent.set_order(d_order)

Pointers are raw device addresses (e.g. torch tensor data_ptr()).  Only the order of tasks changes, so results are
the same with and without the scheduler.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N

FEATURES = 6
PARAMS = 1313


class cost_model:
    def __init__(self, seed: int = 1):
        self._m = None
        m = ctypes.c_void_p()
        N.call("hibf_gpu_cost_model_create", seed, ctypes.byref(m))
        self._m = m

    def __del__(self):
        if getattr(self, "_m", None):
            try:
                N.lib().hibf_gpu_cost_model_destroy(self._m)
            except Exception:
                pass
            self._m = None

    @property
    def params(self) -> np.ndarray:
        out = np.zeros(PARAMS, np.float32)
        N.call("hibf_gpu_cost_model_get_params", self._m, out.ctypes.data)
        return out

    @params.setter
    def params(self, p) -> None:
        p = np.ascontiguousarray(np.asarray(p, dtype=np.float32))
        if p.size != PARAMS:
            raise ValueError(f"expected {PARAMS} parameters")
        N.call("hibf_gpu_cost_model_set_params", self._m, p.ctypes.data)

    def loss_grad(self, d_features: int, d_work: int, n: int) -> tuple[float, np.ndarray]:
        g = np.zeros(PARAMS, np.float32)
        loss = ctypes.c_double(0)
        N.call("hibf_gpu_cost_model_loss_grad_d", self._m, d_features, d_work, n, g.ctypes.data, ctypes.byref(loss))
        return loss.value, g

    def train(self, d_features: int, d_work: int, n: int, steps: int = 300, lr: float = 1e-2) -> float:
        loss = ctypes.c_double(0)
        N.call("hibf_gpu_cost_model_train_d", self._m, d_features, d_work, n, steps, lr, ctypes.byref(loss))
        return loss.value

    def predict(self, d_features: int, n: int, d_pred: int, stream: int | None = None) -> None:
        N.call("hibf_gpu_cost_model_predict_d", self._m, d_features, n, d_pred, stream)

    def order(self, d_features: int, n: int, d_order: int, stream: int | None = None) -> None:
        N.call("hibf_gpu_cost_model_order_d", self._m, d_features, n, d_order, stream)

    def sort_desc(self, d_keys: int, n: int, d_order: int, stream: int | None = None) -> None:
        N.call("hibf_gpu_sort_desc_d", self._m, d_keys, n, d_order, stream)
