"""Learned near-field preconditioner: host side of the network and tokens.

The network (16 -> 128 -> 128 -> 2, ReLU; BF16 parameters and activations,
FP32 accumulation) is trained and evaluated by the library's own CUDA kernels
(mlf_mlp_*); the tokens and targets come from a context's near field and an
exact preconditioner (mlf_lp_tokens), and mlf_lp_install writes the
prediction into the context's preconditioner slot.  Device buffers are torch
CUDA tensors (memory only: all arithmetic runs in the library).  No
counterpart in the reference.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._capi import MLFError, load

TARGETS = {"none": 0, "own": 1, "nbhd": 2}


def _p(t):
    return C.c_void_p(t.data_ptr())


def _ck(code, net=None):
    if code != 0:
        msg = load().mlf_mlp_last_error(net).decode() if net else ""
        raise MLFError(code, msg)


class MLP:
    def __init__(self, seed: int = 0, device: int = 0):
        h = C.c_void_p()
        _ck(load().mlf_mlp_create(C.byref(h), int(device), C.c_ulonglong(seed)))
        self._h = h
        self.nparam = load().mlf_mlp_nparam()

    def close(self):
        if getattr(self, "_h", None):
            load().mlf_mlp_free(self._h)
            self._h = None

    __del__ = close

    @property
    def handle(self):
        return self._h

    def params(self):
        P = np.zeros(self.nparam, dtype=np.float32)
        nrm = np.zeros(32, dtype=np.float32)
        _ck(load().mlf_mlp_get_params(self._h, P.ctypes.data, nrm.ctypes.data), self._h)
        return P, nrm

    def set_params(self, P=None, norm=None):
        Pc = None if P is None else np.ascontiguousarray(P, dtype=np.float32)
        Nc = None if norm is None else np.ascontiguousarray(norm, dtype=np.float32)
        _ck(load().mlf_mlp_set_params(self._h, None if Pc is None else Pc.ctypes.data,
                                      None if Nc is None else Nc.ctypes.data), self._h)

    def fit_norm(self, X):
        """mu, sd of the token features (binary and constant columns kept at 0, 1)."""
        import torch
        mu = X.mean(0).double().cpu().numpy()
        sd = X.double().std(0).cpu().numpy() + 1e-6
        for q in (3, 15):
            mu[q], sd[q] = 0.0, 1.0
        self.set_params(None, np.concatenate([mu, sd]).astype(np.float32))
        return mu, sd

    def forward(self, X):
        import torch
        Y = torch.empty((X.shape[0], 2), dtype=torch.float32, device=X.device)
        _ck(load().mlf_mlp_forward(self._h, _p(X), X.shape[0], _p(Y), None), self._h)
        return Y

    def grad(self, X, T):
        G = np.zeros(self.nparam, dtype=np.float32)
        loss = C.c_double()
        _ck(load().mlf_mlp_grad(self._h, _p(X), _p(T), X.shape[0], G.ctypes.data, C.byref(loss)), self._h)
        return loss.value, G

    def train(self, X, T, steps=2000, batch=8192, lr=1e-3, seed=1):
        hist = np.zeros(steps, dtype=np.float32)
        _ck(load().mlf_mlp_train(self._h, _p(X), _p(T), X.shape[0], int(steps), int(batch), C.c_float(lr),
                                 C.c_ulonglong(seed), hist.ctypes.data), self._h)
        return hist


def tokens(m, target="nbhd"):
    """(X [ntok, 16], T [ntok, 2]) CUDA tensors for the context `m`; target
    'own' needs m.nearinv(own_only=True) first, 'nbhd' m.nearinv()."""
    import torch
    tk = TARGETS[target] if isinstance(target, str) else int(target)
    n = C.c_longlong()
    L = load()
    code = L.mlf_lp_tokens(m.handle, tk, None, None, 0, C.byref(n))
    if code:
        raise MLFError(code, L.mlf_last_error(m.handle).decode())
    X = torch.empty((n.value, 16), dtype=torch.float32, device="cuda")
    T = torch.empty((n.value, 2), dtype=torch.float32, device="cuda") if tk else None
    code = L.mlf_lp_tokens(m.handle, tk, _p(X), None if T is None else _p(T), n.value, C.byref(n))
    if code:
        raise MLFError(code, L.mlf_last_error(m.handle).decode())
    return X, T


def install(m, net: MLP) -> int:
    """Replace m's preconditioner by the network's prediction; returns the
    number of non-finite outputs (zeroed)."""
    bad = C.c_int()
    L = load()
    code = L.mlf_lp_install(m.handle, net.handle, C.byref(bad))
    if code:
        raise MLFError(code, L.mlf_last_error(m.handle).decode())
    return bad.value
