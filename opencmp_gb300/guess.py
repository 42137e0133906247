"""Learned Krylov initial guess for implicit time stepping.

OpenCMP starts each step's Krylov solve from the previous step's solution
(``opencmp/models/base_model.py:925-937``). :class:`LearnedGuess` replaces that start by
``u^n + scale * MLP(features)``, where, per dof, the features are the last k-1 solution differences
and the Jacobi correction ``D^-1 (b - A u^n)`` of the previous-step guess, all divided by the norm
of that dof's differences. The network (``ocmp_guess_*`` in ``csrc/ocmp_guess.cu``) is trained on
trajectories the solver itself produced, with the library's own forward, backward and Adam
kernels. The solve still runs to the same FP64 residual tolerance, so the guess only changes how
many iterations that takes; if a prediction starts worse than the previous step's solution would
have, the run falls back to the previous-step guess.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional

import numpy as np
import torch

from . import _lib as LB
from .fem import Matrix, Space, _ptr, _stream


class GuessNet:
    """The per-dof MLP (hidden width 32, FP32) and its Adam state on the device."""

    def __init__(self, n_features: int, seed: int = 0):
        h = C.c_void_p()
        LB.call('ocmp_guess_create', n_features, C.c_uint64(seed), C.byref(h))
        self.h = h
        self.F = n_features
        self.nparams = LB.load().ocmp_guess_nparams(self.h)

    def __del__(self):
        if getattr(self, 'h', None) and LB._lib is not None:
            LB._lib.ocmp_guess_destroy(self.h)
            self.h = None

    def params(self) -> np.ndarray:
        p = np.empty(self.nparams, np.float32)
        LB.call('ocmp_guess_params', self.h, _ptr(p), 0)
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        LB.call('ocmp_guess_params', self.h, _ptr(p), 1)

    def forward(self, X: torch.Tensor, Y: torch.Tensor, stream=None):
        LB.call('ocmp_guess_forward', self.h, _ptr(X), X.shape[0], _ptr(Y), _stream(stream))

    def loss_grad(self, X: torch.Tensor, T: torch.Tensor, want_grad: bool = False, stream=None):
        loss = C.c_double(0)
        g = np.empty(self.nparams, np.float32) if want_grad else None
        LB.call('ocmp_guess_loss_grad', self.h, _ptr(X), _ptr(T), X.shape[0], C.byref(loss),
                _ptr(g) if want_grad else None, _stream(stream))
        return loss.value, g

    def adam_step(self, lr: float, stream=None):
        LB.call('ocmp_guess_adam_step', self.h, C.c_float(lr), _stream(stream))


class LearnedGuess:
    """History of the last ``k`` solutions on the device and the network that extrapolates them."""

    def __init__(self, space: Space, k: int = 4, use_residual: bool = True, seed: int = 0):
        if not 2 <= k <= 4:
            raise ValueError('k must be 2..4')
        self.space = space
        self.n = space.ndof
        self.k = k
        self.use_q = use_residual
        self.F = (k - 1) + (1 if use_residual else 0)
        self.net = GuessNet(self.F, seed)
        dev = 'cuda'
        self.hist: List[torch.Tensor] = []
        self._ring = [torch.zeros(self.n, dtype=torch.float64, device=dev) for _ in range(k)]
        self._head = 0
        self.X = torch.empty(self.n, self.F, dtype=torch.float32, device=dev)
        self.Y = torch.empty(self.n, dtype=torch.float32, device=dev)
        self.q = torch.empty(self.n, dtype=torch.float64, device=dev)
        self.scale = torch.ones(self.n, dtype=torch.float64, device=dev)
        self._free = torch.as_tensor(space.FreeDofs().astype(np.uint8), device=dev)
        self.samples_X: List[torch.Tensor] = []
        self.samples_T: List[torch.Tensor] = []
        self.enabled = True
        self.judge_window = 3
        self._base_it: List[int] = []
        self._base_r0: List[float] = []
        self._net_it: List[int] = []
        self.fallback_reason = None

    # ---------------------------------------------------------------- history
    def reset(self):
        self.hist = []

    def push(self, u: torch.Tensor):
        """Record the newest solution (copied into the device ring)."""
        buf = self._ring[self._head]
        buf.copy_(u)
        self._head = (self._head + 1) % self.k
        self.hist = [buf] + self.hist[:self.k - 1]

    @property
    def ready(self) -> bool:
        return len(self.hist) >= self.k

    # ---------------------------------------------------------------- features / prediction
    def _features(self, A: Optional[Matrix], b: Optional[torch.Tensor], stream=None):
        L = LB.load()
        st = _stream(stream)
        h = self.hist
        qp = None
        if self.use_q:
            LB.check(L.ocmp_jacobi_residual(A.h, _ptr(b), _ptr(h[0]), _ptr(self.q), st))
            qp = _ptr(self.q)
        arr = (C.c_void_p * 4)(*[C.c_void_p(t.data_ptr()) for t in h[:self.k]] + [None] * (4 - self.k))
        LB.check(L.ocmp_guess_features(self.n, self.k, arr, qp, _ptr(self.scale), _ptr(self.X), self.F, st))

    def predict(self, x: torch.Tensor, A: Optional[Matrix] = None, b: Optional[torch.Tensor] = None, stream=None):
        """x = u^n + scale * MLP(features); falls back to x = u^n until the history is full."""
        if not (self.ready and self.enabled):
            x.copy_(self.hist[0] if self.hist else x)
            return False
        self._features(A, b, stream)
        self.net.forward(self.X, self.Y, stream)
        LB.check(LB.load().ocmp_guess_apply(self.n, _ptr(self.hist[0]), _ptr(self.Y), _ptr(self.scale),
                                            _ptr(self._free), _ptr(x), _stream(stream)))
        return True

    def judge(self, info, used: bool):
        """Convergence is the guess's judge. Steps solved from the previous-step guess set the
        baseline (iterations, initial residual); the network is switched off for the rest of the run
        if one of its guesses starts worse than that baseline, or if over ``judge_window`` steps it
        does not reduce the Krylov iterations."""
        if not used:
            self._base_it.append(info.iterations)
            self._base_r0.append(info.relres0)
            return
        self._net_it.append(info.iterations)
        if not self._base_it:
            return
        if info.relres0 > np.mean(self._base_r0):
            self.enabled, self.fallback_reason = False, 'initial residual above the previous-step guess'
        elif len(self._net_it) >= self.judge_window and \
                np.mean(self._net_it[-self.judge_window:]) >= np.mean(self._base_it[-self.judge_window:]):
            self.enabled, self.fallback_reason = False, 'no fewer Krylov iterations than the previous-step guess'

    def reset_judge(self):
        self.enabled = True
        self._base_it, self._base_r0, self._net_it = [], [], []
        self.fallback_reason = None

    # ---------------------------------------------------------------- training
    def collect(self, u_next: torch.Tensor, A: Optional[Matrix] = None, b: Optional[torch.Tensor] = None):
        """Store one training sample: features at step n and target (u^{n+1} - u^n) / scale."""
        if not self.ready:
            return
        self._features(A, b)
        T = torch.empty(self.n, dtype=torch.float32, device='cuda')
        LB.check(LB.load().ocmp_guess_target(self.n, _ptr(u_next), _ptr(self.hist[0]), _ptr(self.scale), _ptr(T),
                                             _stream(None)))
        self.samples_X.append(self.X.clone())
        self.samples_T.append(T)

    def train(self, steps: int = 300, batch: int = 1 << 17, lr: float = 3e-3, seed: int = 0) -> List[float]:
        """Adam on random contiguous row windows of the stored samples; returns the loss history."""
        if not self.samples_X:
            raise RuntimeError('no training samples collected')
        rng = np.random.default_rng(seed)
        losses = []
        for it in range(steps):
            s = int(rng.integers(len(self.samples_X)))
            nb = min(batch, self.n)
            off = int(rng.integers(0, self.n - nb + 1))
            X = self.samples_X[s][off:off + nb]
            T = self.samples_T[s][off:off + nb]
            loss, _ = self.net.loss_grad(X, T)
            self.net.adam_step(lr * (0.5 * (1 + np.cos(np.pi * it / steps))) + 1e-5)
            losses.append(loss)
        return losses

    def eval_loss(self) -> float:
        """Mean loss of the network over every stored sample (all rows)."""
        tot = 0.0
        for X, T in zip(self.samples_X, self.samples_T):
            tot += self.net.loss_grad(X, T)[0]
        return tot / max(1, len(self.samples_X))

    def drop_samples(self):
        self.samples_X.clear()
        self.samples_T.clear()
