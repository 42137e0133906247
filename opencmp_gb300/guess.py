"""Learned Krylov initial guess for implicit time stepping.

OpenCMP starts each step's Krylov solve from the previous step's solution
(``opencmp/models/base_model.py:925-937``). :class:`LearnedGuess` starts it from

    x = u^n + D_1 + ... + D_p  +  S_{k-1} * MLP(D_1 / S_1, ..., D_{k-1} / S_{k-1}),

where D_j is the j-th backward difference in time of the last k solutions at a dof and S_j its
root mean square over the free dofs: the degree-p extrapolation in time plus a per-dof network's
correction (``ocmp_guess_*`` in ``csrc/ocmp_guess.cu``). The history is kept on the device as the
table of backward differences itself, in double-float (pairs of FP32 values). The network is trained on trajectories
the solver itself produced, with the library's own forward, backward and Adam kernels, to minimise
the FP64 relative residual its guess leaves (|A e| / |b|, through A and its transpose).

The extrapolation alone is the fallback: it is used until the history is full and the network is
trained, and for the rest of a run once the judge (:meth:`LearnedGuess.judge`) sees the network's
guess start a solve no better than the extrapolation did. The solve always runs to the same FP64
residual tolerance, so the guess only changes how many iterations that takes.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, List

import numpy as np
import torch

from . import _lib as LB
from .fem import Matrix, Space, _ptr, _stream

NET, PROBE, FALLBACK = 'network', 'probe', 'fallback'


class GuessNet:
    """The per-dof MLP (hidden width 16, FP32) and its Adam state on the device. A new network has
    zero output: its output layer and linear skip start at zero."""

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
        """Mean squared error against T and its parameter gradient."""
        loss = C.c_double(0)
        g = np.empty(self.nparams, np.float32) if want_grad else None
        LB.call('ocmp_guess_loss_grad', self.h, _ptr(X), _ptr(T), X.shape[0], C.byref(loss),
                _ptr(g) if want_grad else None, _stream(stream))
        return loss.value, g

    def backward(self, X: torch.Tensor, dY: torch.Tensor, want_grad: bool = False, stream=None):
        """Parameter gradient of sum_r dY_r y_r (kept on the device for :meth:`adam_step`)."""
        g = np.empty(self.nparams, np.float32) if want_grad else None
        LB.call('ocmp_guess_backward', self.h, _ptr(X), _ptr(dY), X.shape[0], _ptr(g) if want_grad else None,
                _stream(stream))
        return g

    def adam_step(self, lr: float, stream=None):
        LB.call('ocmp_guess_adam_step', self.h, C.c_float(lr), _stream(stream))


class LearnedGuess:
    """History of the last ``k`` solutions on the device, the degree-``base_order`` extrapolation and
    the network that corrects it (``k - 1`` features)."""

    def __init__(self, space: Space, k: int = 5, base_order: int = 3, seed: int = 0):
        if not 2 <= k <= 6:
            raise ValueError('k must be 2..6')
        if not 0 <= base_order < k:
            raise ValueError('base_order must be 0..k-1')
        self.space = space
        self.n = space.ndof
        self.k = k
        self.base_order = base_order
        self.F = k - 1
        self.net = GuessNet(self.F, seed)
        dev = 'cuda'
        self.m = 0  # valid rows of the difference table
        self.tab = torch.zeros(k, self.n, 2, dtype=torch.float32, device=dev)
        self.X = torch.empty(self.n, self.F, dtype=torch.float32, device=dev)
        self.Y = torch.empty(self.n, dtype=torch.float32, device=dev)
        self.dY = torch.empty(self.n, dtype=torch.float32, device=dev)
        self.scales = torch.ones(32, dtype=torch.float64, device=dev)
        self._free = torch.as_tensor(space.FreeDofs().astype(np.uint8), device=dev)
        self.samples: List[Dict] = []
        self.trained = False
        self.enabled = True
        self.judge_window = 3
        self.probe_every = 8
        self.fallback_reason = None
        self.reset_judge()

    # ---------------------------------------------------------------- history
    def reset(self):
        self.m = 0

    def push(self, u: torch.Tensor, stream=None):
        """Add the newest solution to the difference table."""
        LB.call('ocmp_guess_push', self.n, self.k, self.m, _ptr(self.tab), _ptr(u), _stream(stream))
        self.m = min(self.m + 1, self.k)

    @property
    def ready(self) -> bool:
        return self.m >= self.k

    # ---------------------------------------------------------------- prediction
    def _scales(self, X=None, stream=None):
        LB.call('ocmp_guess_features', self.net.h, self.n, self.k, _ptr(self.tab), _ptr(self._free),
                _ptr(self.scales), _ptr(X), _stream(stream))

    def extrapolate(self, x: torch.Tensor, order=None, stream=None):
        """The fallback: x = u^n + D_1 + ... + D_p with p = min(order, history - 1)."""
        if self.m == 0:
            raise RuntimeError('no history')
        p = min(self.base_order if order is None else order, self.m - 1)
        LB.call('ocmp_guess_predict', None, self.n, self.m, _ptr(self.tab), _ptr(self._free), None, p, _ptr(x),
                _stream(stream))

    def predict(self, x: torch.Tensor, stream=None) -> str:
        """Writes the guess into x; returns which guess it was: ``'network'``, ``'probe'`` (the
        extrapolation, solved on alternate steps of the judge's evaluation window and every
        ``probe_every``-th step after it) or ``'fallback'`` (the extrapolation)."""
        if not (self.ready and self.enabled and self.trained):
            self.extrapolate(x, stream=stream)
            return FALLBACK
        self._count += 1
        probe = self._probe_next if self._evaluating else self._count % self.probe_every == 0
        if probe:
            self.extrapolate(x, stream=stream)
            self._probe_next = False
            return PROBE
        self._scales(stream=stream)
        LB.call('ocmp_guess_predict', self.net.h, self.n, self.k, _ptr(self.tab), _ptr(self._free),
                _ptr(self.scales), self.base_order, _ptr(x), _stream(stream))
        self._probe_next = self._evaluating
        return NET

    def judge(self, info, kind: str):
        """Convergence is the guess's judge. Over an evaluation window of ``2 judge_window`` steps
        the network's guess alternates with the extrapolation (probe steps), and after it every
        ``probe_every``-th step is a probe. The network is switched off for the rest of the run as
        soon as its recent steps (the last ``2 judge_window``) do not take fewer Krylov iterations on
        average than the recent probes (the last ``judge_window``), or if one of its guesses starts
        a solve with a larger initial FP64 residual than the probes' mean."""
        if kind == PROBE:
            self._base_it.append(info.iterations)
            self._base_r0.append(info.relres0)
        elif kind == NET:
            self._net_it.append(info.iterations)
            if self._base_r0 and info.relres0 > np.mean(self._base_r0[-self.judge_window:]):
                self.enabled, self.fallback_reason = False, 'initial residual above the extrapolation'
                return
        else:
            return
        W = self.judge_window
        if len(self._net_it) >= W and len(self._base_it) >= W:
            self._evaluating = False
            if np.mean(self._net_it[-2 * W:]) >= np.mean(self._base_it[-W:]):
                self.enabled, self.fallback_reason = False, 'no fewer Krylov iterations than the extrapolation'

    def reset_judge(self):
        self.enabled = True
        self._evaluating = True
        self._probe_next = True
        self._count = 0
        self._base_it, self._base_r0, self._net_it = [], [], []
        self.fallback_reason = None

    # ---------------------------------------------------------------- training
    def collect(self, u_next: torch.Tensor, A: Matrix, b: torch.Tensor):
        """Store one training sample from a solved step: features and target of the history before
        it, the step's matrix A (kept by reference: it must keep these values until training ends)
        and right-hand side b. The sample's weight makes the extrapolation's loss 1."""
        if not self.ready:
            return
        X = torch.empty(self.n, self.F, dtype=torch.float32, device='cuda')
        self._scales(X)
        T = torch.empty(self.n, dtype=torch.float32, device='cuda')
        LB.call('ocmp_guess_target', self.n, self.k, _ptr(self.tab), _ptr(self._free), _ptr(self.scales),
                self.base_order, _ptr(u_next), _ptr(T), _stream(None))
        smp = dict(X=X, T=T, S=self.scales[self.F - 1:self.F].clone(), A=A, b=b.clone(), w=1.0)
        self.Y.zero_()
        base = self._loss(smp, self.Y, want_grad=False)
        smp['w'] = 1.0 / base if base > 0 else 1.0
        smp['r0_extrap'] = float(np.sqrt(base))
        self.samples.append(smp)

    def _loss(self, smp, Y, want_grad=True) -> float:
        loss = C.c_double(0)
        LB.call('ocmp_guess_residual_loss', self.net.h, smp['A'].h, _ptr(Y), _ptr(smp['T']), _ptr(smp['S']),
                _ptr(smp['b']), smp['w'], C.byref(loss), _ptr(self.dY), _stream(None))
        return loss.value

    def train(self, steps: int = 300, lr: float = 3e-3, seed: int = 0) -> List[float]:
        """Adam over the stored samples (one whole step per iteration, cosine learning rate) on the
        weighted residual loss; returns the loss history (1 = the extrapolation's residual).

        The mean loss over all samples is evaluated ten times along the way, and the parameters with
        the lowest one are kept, the untrained network (mean loss 1) included: on few samples from a
        fast transient the steps can overshoot, and training then never ends worse than the
        extrapolation on its own samples."""
        if not self.samples:
            raise RuntimeError('no training samples collected')
        rng = np.random.default_rng(seed)
        losses = []
        best_p, best = self.net.params(), self.eval_loss()
        every = max(1, steps // 10)
        for it in range(steps):
            smp = self.samples[int(rng.integers(len(self.samples)))]
            self.net.forward(smp['X'], self.Y)
            losses.append(self._loss(smp, self.Y))
            self.net.backward(smp['X'], self.dY)
            self.net.adam_step(lr * (0.5 * (1 + np.cos(np.pi * it / steps))) + 1e-5)
            if (it + 1) % every == 0 or it + 1 == steps:
                cur = self.eval_loss()
                if cur < best:
                    best_p, best = self.net.params(), cur
        self.net.set_params(best_p)
        self.trained = True
        return losses

    def eval_loss(self) -> float:
        """Mean weighted residual loss of the network over the stored samples (1 = extrapolation)."""
        tot = 0.0
        for smp in self.samples:
            self.net.forward(smp['X'], self.Y)
            tot += self._loss(smp, self.Y)
        return tot / max(1, len(self.samples))

    def drop_samples(self):
        self.samples.clear()
