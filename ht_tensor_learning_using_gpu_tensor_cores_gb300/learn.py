"""Learned per-mode sketch for the leaf range finder.

The leaf eigen-solver started from a block S (n x s) and run for one
iteration is a randomized range finder on the mode Gram: Y = G S, Q = orth(Y),
leaf basis = top-k Rayleigh-Ritz vectors of span(Q).  With a Gaussian S this is
the textbook method (the reference's rsvd draws a Gaussian test matrix,
third_order_tensor_decompsition/CUDA/Optimized/kernel.cu:595-680).  Here S is
trained, per mode, on Grams that the engine itself produces from a family of
tensors, to minimise the energy the subspace misses:

    L(S) = mean_b [ 1 - tr(Q_b^T G_b Q_b) / tr(G_b) ].

Forward and adjoint run in the library's own kernels (``ht_sketch_loss_grad``:
the three n x n by n x s products in FP32, the s x s algebra of CholeskyQR in
FP64), the update is Adam (``ht_sketch_adam``).  The trained S is used through
the ordinary C ABI: ``decompose(..., sketch=[S_0, S_1, S_2], eig_iters=1)``;
``sketch=None`` keeps the Gaussian start block, which stays the default and the
yardstick of the learned one.
"""
from __future__ import annotations

import ctypes
from ctypes import c_double, c_void_p
from typing import List, Sequence, Tuple

import numpy as np

from ._lib import check, lib


def _ptr(t):
    return c_void_p(t.data_ptr())


def family_grams(seeds: Sequence[int], n: int, precision: str = "bf16", device="cuda"):
    """Mode Grams of the separable-bumps family at n^3 (synth.bumps): a
    (len(seeds), 3, n, n) float32 CUDA tensor (column-major n x n blocks; Grams
    are symmetric) and their traces (len(seeds), 3)."""
    import torch
    from . import mode_gram, synth
    G = torch.empty((len(seeds), 3, n, n), dtype=torch.float32, device=device)
    for i, sd in enumerate(seeds):
        X = synth.bumps(n, seed=int(sd), assemble_on=torch.device(device))
        for m in range(3):
            G[i, m] = mode_gram(X, (n, n, n), m, precision=precision)
        del X
    tr = torch.diagonal(G, dim1=2, dim2=3).sum(-1).contiguous()
    return G, tr


def gaussian_sketch(n: int, s: int, seed: int = 0, device="cuda"):
    import torch
    g = torch.Generator(device="cpu").manual_seed(int(seed))
    S = torch.randn((s, n), generator=g, dtype=torch.float32) / np.sqrt(n)
    return S.to(device).t()   # n x s, column-major storage


def loss_grad(G, trG, S, stream=None):
    """(per-Gram losses as numpy, gradient n x s as a torch tensor) for the batch
    G (B x n x n), traces trG (B), sketch S (n x s column-major)."""
    import torch
    B, n = int(G.shape[0]), int(G.shape[-1])
    s = int(S.shape[1])
    if S.stride() != (1, n):
        raise ValueError("S must be column-major n x s (e.g. a transposed contiguous s x n tensor)")
    grad = torch.empty((s, n), dtype=torch.float32, device=G.device).t()
    loss = (c_double * B)()
    st = torch.cuda.current_stream(G.device).cuda_stream if stream is None else stream
    check(lib().ht_sketch_loss_grad(_ptr(G.contiguous()), _ptr(trG.contiguous()), B, n, s, _ptr(S), _ptr(grad), loss,
                                    c_void_p(st)))
    return np.array(loss[:], dtype=np.float64), grad


class SketchTrainer:
    """Adam on one mode's sketch."""

    def __init__(self, n: int, s: int, seed: int = 0, lr: float = 2e-3, device="cuda"):
        import torch
        self.S = gaussian_sketch(n, s, seed, device).contiguous().t().contiguous().t()   # own storage, column-major
        self.m = torch.zeros_like(self.S)
        self.v = torch.zeros_like(self.S)
        self.lr, self.step_no = float(lr), 0

    def step(self, G, trG) -> float:
        import torch
        loss, grad = loss_grad(G, trG, self.S)
        self.step_no += 1
        st = torch.cuda.current_stream(G.device).cuda_stream
        check(lib().ht_sketch_adam(_ptr(self.S), _ptr(grad), _ptr(self.m), _ptr(self.v), self.S.numel(),
                                   ctypes.c_float(self.lr), self.step_no, c_void_p(st)))
        return float(loss.mean())


def train_mode_sketches(G_train, tr_train, s: int = 34, steps: int = 2000, batch: int = 32, lr: float = 2e-3,
                        seed: int = 0, log_every: int = 0) -> Tuple[List, dict]:
    """One sketch per mode trained on G_train[:, m] (N x n x n): ``steps`` Adam
    steps on random minibatches of ``batch`` Grams.  Returns the sketches
    (n x s, column-major) and the loss history per mode."""
    import torch
    N, modes, n = int(G_train.shape[0]), int(G_train.shape[1]), int(G_train.shape[-1])
    rng = np.random.default_rng(seed)
    sketches, hist = [], {}
    for m in range(modes):
        tr = SketchTrainer(n, s, seed=seed + 17 * m, lr=lr, device=G_train.device)
        h = []
        for it in range(steps):
            idx = torch.as_tensor(rng.choice(N, size=min(batch, N), replace=False), device=G_train.device)
            G = G_train[idx, m].contiguous()
            t = tr_train[idx, m].contiguous()
            h.append(tr.step(G, t))
            if log_every and it % log_every == 0:
                print(f"mode {m} step {it} loss {h[-1]:.4e}", flush=True)
        sketches.append(tr.S)
        hist[m] = h
    return sketches, hist


def heldout_loss(G, trG, S) -> np.ndarray:
    """Per-Gram forward loss of sketch S on G (B x n x n)."""
    loss, _ = loss_grad(G.contiguous(), trG.contiguous(), S)
    return loss


def to_bf16(S):
    """The sketch as stored for use: BF16-rounded values (kept in an FP32 tensor)."""
    import torch
    return S.to(torch.bfloat16).to(torch.float32).t().contiguous().t()


__all__ = ["family_grams", "gaussian_sketch", "loss_grad", "SketchTrainer", "train_mode_sketches", "heldout_loss",
           "to_bf16"]
