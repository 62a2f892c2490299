"""Learned morphogen surrogate: network, training dataset and attachment to a simulation.

The network (MLP 48 -> 128 -> 128 -> 16, GELU) predicts one morphogen stage's concentration
increment from a particle's concentrations, its diffusion neighbours' mean concentrations and
its gene bits.  Training data are captured from plain steps; training runs on the GPU with
the library's BF16 tensor-core kernels; in-step inference runs on tcgen05 tensor cores.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from ._abi import MgError, load


def _check(lib, status, what=""):
    if status != A.MG_OK:
        msg = (lib.mg_last_error(None) or b"").decode()
        raise MgError(status, f"{what}: {msg}" if what else msg)


class Mlp:
    """One network on the device (FP32 master weights, Adam state, BF16 and inference copies)."""

    def __init__(self, seed: int = 0):
        self.lib = load()
        h = C.c_void_p()
        _check(self.lib, self.lib.mg_mlp_create(int(seed), C.byref(h)), "mg_mlp_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.mg_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.empty(A.P_COUNT, np.float32)
        _check(self.lib, self.lib.mg_mlp_get_params(self.h, out.ctypes.data, out.size))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        _check(self.lib, self.lib.mg_mlp_set_params(self.h, p.ctypes.data, p.size))

    def norm(self) -> np.ndarray:
        out = np.empty(A.NORM_COUNT, np.float32)
        _check(self.lib, self.lib.mg_mlp_get_norm(self.h, out.ctypes.data, out.size))
        return out

    def set_norm(self, n: np.ndarray) -> None:
        n = np.ascontiguousarray(n, np.float32)
        _check(self.lib, self.lib.mg_mlp_set_norm(self.h, n.ctypes.data, n.size))

    def gradients(self, x: np.ndarray, y: np.ndarray):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        g = np.empty(A.P_COUNT, np.float32)
        loss = C.c_double()
        _check(self.lib, self.lib.mg_mlp_gradients(self.h, x.ctypes.data, y.ctypes.data, len(x),
                                                   g.ctypes.data, C.byref(loss)))
        return g, loss.value

    def infer(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        y = np.empty((len(x), A.MLP_OUT), np.float32)
        _check(self.lib, self.lib.mg_mlp_infer(self.h, x.ctypes.data, len(x), y.ctypes.data))
        return y

    def fit_normalization(self, ds: "Dataset") -> None:
        _check(self.lib, self.lib.mg_mlp_fit_normalization(self.h, ds.h))

    def train(self, ds: "Dataset", steps: int, batch: int = 65536, lr: float = 1e-3,
              seed: int = 0) -> np.ndarray:
        curve = np.empty(steps, np.float32)
        _check(self.lib, self.lib.mg_mlp_train(self.h, ds.h, steps, batch, lr, seed, curve.ctypes.data))
        return curve


class Dataset:
    """(features, morphogen increment) pairs on the device, captured from plain steps."""

    def __init__(self, capacity: int):
        self.lib = load()
        h = C.c_void_p()
        _check(self.lib, self.lib.mg_dataset_create(int(capacity), C.byref(h)), "mg_dataset_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.mg_dataset_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def capture(self, fs, flags: int = A.STEP_PHYSICS) -> None:
        _check(self.lib, self.lib.mg_dataset_capture(self.h, fs.h, flags), "mg_dataset_capture")

    def __len__(self) -> int:
        n = C.c_uint64()
        _check(self.lib, self.lib.mg_dataset_size(self.h, C.byref(n)))
        return int(n.value)

    def read(self, first: int, n: int):
        x = np.empty((n, A.MLP_IN), np.float32)
        y = np.empty((n, A.MLP_OUT), np.float32)
        _check(self.lib, self.lib.mg_dataset_read(self.h, first, n, x.ctypes.data, y.ctypes.data))
        return x, y


def attach(fs, mlp: Mlp | None, judge_period: int = 10, judge_stride: int = 64,
           threshold: float = 1e-3) -> None:
    lib = load()
    _check(lib, lib.mg_set_surrogate(fs.h, mlp.h if mlp is not None else None, judge_period,
                                     judge_stride, threshold), "mg_set_surrogate")


def stats(fs, reset: bool = False):
    lib = load()
    j, t, w = C.c_uint64(), C.c_uint64(), C.c_float()
    _check(lib, lib.mg_surrogate_stats(fs.h, C.byref(j), C.byref(t), C.byref(w), 1 if reset else 0))
    return int(j.value), int(t.value), float(w.value)
