"""The learned dispatcher: an MLP trained on the GPU by the library's own
CUDA kernels (ndconv_mlp_*), mapping 16 shape / mode features of an
instance to predicted log-time (log ms) per algorithm variant.

Candidates (outputs, in order): direct FP32, direct 3xBF16 split, FFT
full N-d, FFT row-spectral, and the two with power-of-two lengths (the
ndconv_algo codes in CANDIDATES).  Every candidate meets the same error
bound, so the pick changes only the time, never the result beyond it.
"""
import ctypes
import json
import math
import os

import numpy as np
import torch

from . import _abi
from .dispatch import N_FEATURES, features

CANDIDATES = [_abi.ALGO_DIRECT, _abi.ALGO_DIRECT_BF16X3, _abi.ALGO_FFT_ND, _abi.ALGO_FFT_RS,
              _abi.ALGO_FFT_ND_POW2, _abi.ALGO_FFT_RS_POW2]
N_HIDDEN = 64
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "dispatcher_mlp.json")


def _fp(t):
    return ctypes.cast(ctypes.c_void_p(t.data_ptr()), ctypes.POINTER(ctypes.c_float))


class MLP:
    """ndconv_mlp handle with input standardisation kept on the host."""

    def __init__(self, n_in=N_FEATURES, n_hidden=N_HIDDEN, n_out=len(CANDIDATES), seed=0):
        self.dims = (n_in, n_hidden, n_out)
        h = ctypes.c_void_p()
        st = _abi.lib().ndconv_mlp_create(n_in, n_hidden, n_out, seed, ctypes.byref(h))
        if st:
            raise RuntimeError(_abi.last_error())
        self._h = h
        self.mu = np.zeros(n_in)
        self.sd = np.ones(n_in)
        self.trained = np.ones(n_out)  # outputs that saw at least one timing

    def close(self):
        if self._h:
            _abi.lib().ndconv_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_params(self):
        return int(_abi.lib().ndconv_mlp_param_count(self._h))

    def get_params(self):
        buf = np.zeros(self.n_params, np.float32)
        st = _abi.lib().ndconv_mlp_params(self._h, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                           buf.size, 0)
        if st:
            raise RuntimeError(_abi.last_error())
        return buf

    def set_params(self, p):
        buf = np.ascontiguousarray(p, dtype=np.float32)
        assert buf.size == self.n_params
        st = _abi.lib().ndconv_mlp_params(self._h, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                           buf.size, 1)
        if st:
            raise RuntimeError(_abi.last_error())

    # ---- raw (already standardised) device-side calls
    def forward_raw(self, x):
        x = x.contiguous().float().cuda()
        y = torch.empty((x.shape[0], self.dims[2]), device=x.device)
        st = _abi.lib().ndconv_mlp_forward(self._h, _fp(x), x.shape[0], _fp(y),
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        if st:
            raise RuntimeError(_abi.last_error())
        return y

    def gradient_raw(self, x, t, m):
        x, t, m = [a.contiguous().float().cuda() for a in (x, t, m)]
        g = torch.empty(self.n_params, device=x.device)
        loss = torch.empty(1, device=x.device)
        st = _abi.lib().ndconv_mlp_gradient(self._h, _fp(x), _fp(t), _fp(m), x.shape[0], _fp(g), _fp(loss),
                                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        if st:
            raise RuntimeError(_abi.last_error())
        return g, float(loss.item())

    def train_raw(self, x, t, m, epochs=200, batch=256, lr=2e-3, seed=0):
        x, t, m = [a.contiguous().float().cuda() for a in (x, t, m)]
        fl = ctypes.c_float()
        st = _abi.lib().ndconv_mlp_train(self._h, _fp(x), _fp(t), _fp(m), x.shape[0], epochs, batch,
                                         ctypes.c_float(lr), seed, ctypes.byref(fl),
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        if st:
            raise RuntimeError(_abi.last_error())
        return fl.value

    # ---- feature-level API
    def standardise(self, F):
        return (np.asarray(F, np.float64) - self.mu) / self.sd

    def fit(self, F, logt, mask, epochs=200, batch=256, lr=2e-3, seed=0):
        """Train on features F [n, 16], targets log-ms [n, k], mask [n, k]."""
        F = np.asarray(F, np.float64)
        self.trained = (np.asarray(mask) > 0).any(0).astype(np.float64)
        self.mu = F.mean(0)
        self.sd = np.where(F.std(0) > 1e-9, F.std(0), 1.0)
        x = torch.tensor(self.standardise(F), dtype=torch.float32)
        t = torch.tensor(np.where(mask > 0, logt, 0.0), dtype=torch.float32)
        return self.train_raw(x, t, torch.tensor(mask, dtype=torch.float32), epochs, batch, lr, seed)

    def predict(self, F):
        x = torch.tensor(self.standardise(F), dtype=torch.float32)
        return self.forward_raw(x).cpu().numpy().astype(np.float64)

    def pick(self, F, available=None):
        """ndconv_algo code of the fastest predicted available candidate per row."""
        pred = self.predict(F)
        if available is not None:
            pred = np.where(np.asarray(available) > 0, pred, np.inf)
        return [CANDIDATES[int(i)] for i in np.argmin(pred, axis=1)]

    def save(self, path=DEFAULT_WEIGHTS, extra=None):
        os.makedirs(os.path.dirname(path), exist_ok=True)
        d = {"dims": list(self.dims), "candidates": CANDIDATES, "mu": list(self.mu), "sd": list(self.sd),
             "trained": [float(v) for v in self.trained], "params": [float(v) for v in self.get_params()]}
        if extra:
            d.update(extra)
        with open(path, "w") as f:
            json.dump(d, f)

    @classmethod
    def load(cls, path=DEFAULT_WEIGHTS):
        with open(path) as f:
            d = json.load(f)
        net = cls(*d["dims"])
        net.mu, net.sd = np.array(d["mu"]), np.array(d["sd"])
        net.trained = np.array(d.get("trained", [1.0] * net.dims[2]))
        net.set_params(np.array(d["params"], np.float32))
        return net


class MLPDispatcher:
    """choose(specs) -> ndconv_algo per instance from the trained network;
    candidates that a build does not provide (mask) are never picked."""

    def __init__(self, net=None, available=None):
        self.net = net if net is not None else MLP.load()
        avail = available if available is not None else default_available()
        # never pick an output the network was not trained on
        self.available = np.asarray(avail, np.float64) * (self.net.trained > 0)

    def choose(self, specs):
        F = np.array([features(s) for s in specs])
        return self.net.pick(F, np.tile(self.available, (len(specs), 1)))


def default_available():
    """1 for each candidate this library build provides."""
    lib = _abi.lib()
    has_bf16 = hasattr(lib, "ndconv_conv_bf16x3")
    return np.array([0.0 if (c == _abi.ALGO_DIRECT_BF16X3 and not has_bf16) else 1.0 for c in CANDIDATES])


def log_ms(t):
    return math.log(max(t, 1e-6))
