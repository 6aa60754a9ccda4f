"""Python interface of the learned warm start (C ABI: otfem_mlp_*).

A ``WarmStartNet`` owns a node-wise network and its training set on the GPU.
Typical use::

    net = WarmStartNet(capacity=2_000_000, seed=1)
    WarmStartNet.collect(h)                 # otfem_set_collect(h, 1)
    for step in ...:                        # plain solver steps
        simulate(h, ...); net.add_samples(h)
    net.fit_normalization(); net.train(epochs, batch=65536, lr=1e-3)
    net.attach(h)                           # then OTFEM_WARM_START_LEARNED
"""
import ctypes

import numpy as np

from . import capi

_fp = ctypes.POINTER(ctypes.c_float)


class WarmStartNet:
    """A node-wise MLP that predicts each node's velocity change for the CG
    initial guess, trained on the GPU by the library's own kernels."""

    def __init__(self, capacity=0, seed=0):
        self.lib = capi.lib()
        self.m = ctypes.c_void_p()
        capi.check(self.lib.otfem_mlp_create(int(capacity), int(seed), ctypes.byref(self.m)))

    def close(self):
        if self.m:
            self.lib.otfem_mlp_destroy(self.m)
            self.m = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- state ------------------------------------------------------------
    def state(self):
        out = np.zeros(capi.MLP_STATE_SIZE, np.float32)
        capi.check(self.lib.otfem_mlp_get_state(self.m, out.ctypes.data_as(_fp), out.size))
        return out

    def set_state(self, state):
        s = np.ascontiguousarray(state, np.float32)
        capi.check(self.lib.otfem_mlp_set_state(self.m, s.ctypes.data_as(_fp), s.size))

    # ---- training set -------------------------------------------------------
    @staticmethod
    def collect(handle, enable=True):
        capi.check(capi.lib().otfem_set_collect(handle, 1 if enable else 0))

    def add_samples(self, handle, fraction=1.0, seed=0):
        total = ctypes.c_int64()
        capi.check(self.lib.otfem_mlp_add_samples(self.m, handle, float(fraction), int(seed), ctypes.byref(total)))
        return total.value

    def num_samples(self):
        n = ctypes.c_int64()
        capi.check(self.lib.otfem_mlp_num_samples(self.m, ctypes.byref(n)))
        return n.value

    def clear_samples(self):
        capi.check(self.lib.otfem_mlp_clear_samples(self.m))

    # ---- training -----------------------------------------------------------
    def fit_normalization(self):
        capi.check(self.lib.otfem_mlp_fit_normalization(self.m))

    def train(self, epochs, batch=65536, lr=1e-3, seed=0):
        loss = ctypes.c_double()
        capi.check(self.lib.otfem_mlp_train(self.m, int(epochs), int(batch), float(lr), int(seed), ctypes.byref(loss)))
        return loss.value

    def evaluate(self):
        loss = ctypes.c_double()
        capi.check(self.lib.otfem_mlp_evaluate(self.m, ctypes.byref(loss)))
        return loss.value

    def gradient(self, x, y):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        g = np.zeros(capi.MLP_NUM_WEIGHTS, np.float32)
        loss = ctypes.c_double()
        capi.check(self.lib.otfem_mlp_gradient(self.m, x.ctypes.data_as(_fp), y.ctypes.data_as(_fp), x.shape[0],
                                               ctypes.byref(loss), g.ctypes.data_as(_fp)))
        return loss.value, g

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((x.shape[0], 3), np.float32)
        capi.check(self.lib.otfem_mlp_predict(self.m, x.ctypes.data_as(_fp), x.shape[0], y.ctypes.data_as(_fp)))
        return y

    # ---- use ----------------------------------------------------------------
    def attach(self, handle):
        capi.check(self.lib.otfem_set_mlp(handle, self.m))

    @staticmethod
    def detach(handle):
        capi.check(capi.lib().otfem_set_mlp(handle, None))


# offsets in the network state (include/otfem_gpu.h, OTFEM_MLP_STATE_SIZE)
_W4, _B4, _MU_Y = 9536, 9728, 9731 + 36


def extrapolation_state(state):
    """The state with the output layer and target mean zeroed: its guess is
    v + dv_prev, the extrapolation of the velocity the network corrects."""
    s = np.array(state, np.float32, copy=True)
    s[_W4:_B4 + 3] = 0.0
    s[_MU_Y:_MU_Y + 3] = 0.0
    return s


def node_features(handle, num_nodes):
    """The network inputs of every node in the handle's last step (N x 18)."""
    out = np.zeros((num_nodes, 18), np.float32)
    capi.check(capi.lib().otfem_get_features(handle, out.ctypes.data_as(_fp), out.size))
    return out
