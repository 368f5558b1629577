"""HT tensor layer: a fully connected layer whose weight is held in HT format.

Mirrors the reference's HT layer (``HT_tensor_layer/FC_MNIST/mnist_ht.py``):

* :func:`ht_init` is ``ht(data, rank, N, M)`` (``mnist_ht.py:167-197``): an HT
  decomposition of an ``nn.Linear`` weight reshaped to
  ``(N0*M0, N1*M1, N2*M2)`` with the tree {1,2},{3} -> {1},{2}, returning
  ``u1 (N0, M0, r), u2 (N1, M1, r), u3 (N2, M2, r), b2 (r, r, r), b1 (r, r)``.
  The decomposition runs on the GPU through :func:`decompose`.
* :class:`HTLinear` is the layer of ``tNet`` (``mnist_ht.py:199-245``): the same
  five parameters plus a bias shaped ``(M0, M1, M2)``, and a forward equal to
  the reference's einsum chain
  ``zabc,ade -> zabcd,def -> zabcde,afd -> zabcd,ce -> zabcd,aed`` plus bias.

The forward and backward run in ``libhtgb.so`` (``ht_layer_forward`` /
``ht_layer_backward``): the weight is formed from the factors on the GPU and
the batch goes through one GEMM (FP32 SIMT, or tcgen05 on BF16 operands with
``precision="bf16"``).  There is no PyTorch fallback.
"""
from __future__ import annotations

import ctypes
from ctypes import c_void_p
from typing import Sequence

import torch

from ._lib import PREC_BF16, PREC_FP32, HtLayerShape, check, lib

_PREC = {"fp32": PREC_FP32, "bf16": PREC_BF16}


def layer_shape(n: Sequence[int], m: Sequence[int], ranks: Sequence[int]) -> HtLayerShape:
    """ranks = (r_u1, r_u2, r_u3, r_b2): u_j is (n[j], m[j], ranks[j]), b2 is
    (ranks[0], ranks[1], ranks[3]) and b1 is (ranks[3], ranks[2])."""
    s = HtLayerShape()
    for j in range(3):
        s.n[j], s.m[j] = int(n[j]), int(m[j])
    for j in range(4):
        s.r[j] = int(ranks[j])
    return s


_SHAPES = {}


def shape_of(u1, u2, u3, b2, b1) -> HtLayerShape:
    """The C shape struct of a factor set (cached by the factors' shapes: the C
    side only reads it)."""
    key = (tuple(u1.shape), tuple(u2.shape), tuple(u3.shape), tuple(b2.shape), tuple(b1.shape))
    sh = _SHAPES.get(key)
    if sh is None:
        sh = _make_shape(u1, u2, u3, b2, b1)
        if len(_SHAPES) >= 256:
            _SHAPES.clear()
        _SHAPES[key] = sh
    return sh


def _make_shape(u1, u2, u3, b2, b1) -> HtLayerShape:
    for name, t, d in (("u1", u1, 3), ("u2", u2, 3), ("u3", u3, 3), ("b2", b2, 3), ("b1", b1, 2)):
        if t.dim() != d:
            raise ValueError(f"{name} must have {d} dimensions")
    if (b2.shape[0], b2.shape[1]) != (u1.shape[2], u2.shape[2]) or tuple(b1.shape) != (b2.shape[2], u3.shape[2]):
        raise ValueError("factor ranks do not chain: need b2 (r_u1, r_u2, r), b1 (r, r_u3)")
    return layer_shape([u1.shape[0], u2.shape[0], u3.shape[0]], [u1.shape[1], u2.shape[1], u3.shape[1]],
                       [u1.shape[2], u2.shape[2], u3.shape[2], b2.shape[2]])


def _dev(t):
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32):
        raise TypeError("HT layer tensors must be float32 CUDA tensors")
    return t if t.is_contiguous() else t.contiguous()


def _stream(t):
    return c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def release() -> None:
    """Free the layer workspace of the current device."""
    check(lib().ht_layer_release())


def layer_weight(u1, u2, u3, b2, b1):
    """The dense weight (M0*M1*M2, N0*N1*N2) of the layer (an ``nn.Linear``
    weight: y = x W^T)."""
    sh = shape_of(u1, u2, u3, b2, b1)
    f = [_dev(t) for t in (u1, u2, u3, b2, b1)]
    nin = sh.n[0] * sh.n[1] * sh.n[2]
    nout = sh.m[0] * sh.m[1] * sh.m[2]
    W = torch.empty((nout, nin), dtype=torch.float32, device=u1.device)
    check(lib().ht_layer_weight(ctypes.byref(sh), *[c_void_p(t.data_ptr()) for t in f], c_void_p(W.data_ptr()),
                                _stream(W)))
    return W


def layer_forward(x, u1, u2, u3, b2, b1, bias=None, relu: bool = False, precision: str = "fp32"):
    """y (batch, M0*M1*M2) for x (batch, N0*N1*N2) (or (batch, N0, N1, N2))."""
    sh = shape_of(u1, u2, u3, b2, b1)
    nin = sh.n[0] * sh.n[1] * sh.n[2]
    nout = sh.m[0] * sh.m[1] * sh.m[2]
    x2 = _dev(x.reshape(x.shape[0], -1))
    if x2.shape[1] != nin:
        raise ValueError(f"x has {x2.shape[1]} features, the layer takes {nin}")
    f = [_dev(t) for t in (u1, u2, u3, b2, b1)]
    keep_bias = _dev(bias).reshape(-1) if bias is not None else None
    bp = c_void_p(keep_bias.data_ptr()) if keep_bias is not None else None
    y = torch.empty((x2.shape[0], nout), dtype=torch.float32, device=x.device)
    check(lib().ht_layer_forward(ctypes.byref(sh), *[c_void_p(t.data_ptr()) for t in f], bp, 1 if relu else 0,
                                 _PREC[precision], c_void_p(x2.data_ptr()), x2.shape[0], c_void_p(y.data_ptr()),
                                 _stream(y)))
    return y


def layer_backward(x, dy, u1, u2, u3, b2, b1, need_dx: bool = True, need_dbias: bool = True,
                   precision: str = "fp32"):
    """(dx, du1, du2, du3, db2, db1, dbias) of sum(dy * (x W^T + bias))."""
    sh = shape_of(u1, u2, u3, b2, b1)
    x2 = _dev(x.reshape(x.shape[0], -1))
    dy2 = _dev(dy.reshape(dy.shape[0], -1))
    f = [_dev(t) for t in (u1, u2, u3, b2, b1)]
    grads = [torch.empty_like(t) for t in f]
    dx = torch.empty_like(x2) if need_dx else None
    nout = sh.m[0] * sh.m[1] * sh.m[2]
    dbias = torch.empty(nout, dtype=torch.float32, device=x.device) if need_dbias else None
    p = lambda t: c_void_p(t.data_ptr()) if t is not None else None
    check(lib().ht_layer_backward(ctypes.byref(sh), *[p(t) for t in f], _PREC[precision], p(x2), p(dy2),
                                  x2.shape[0], p(dx), *[p(g) for g in grads], p(dbias), _stream(x2)))
    return (dx.reshape(x.shape) if dx is not None else None, *grads, dbias)


class HTLayerFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, u1, u2, u3, b2, b1, bias, precision):
        ctx.save_for_backward(x, u1, u2, u3, b2, b1)
        ctx.precision = precision
        ctx.has_bias = bias is not None
        return layer_forward(x, u1, u2, u3, b2, b1, bias, False, precision)

    @staticmethod
    def backward(ctx, dy):
        x, u1, u2, u3, b2, b1 = ctx.saved_tensors
        dx, du1, du2, du3, db2, db1, dbias = layer_backward(
            x, dy, u1, u2, u3, b2, b1, need_dx=ctx.needs_input_grad[0], need_dbias=ctx.has_bias,
            precision=ctx.precision)
        return dx, du1, du2, du3, db2, db1, dbias, None


def ht_layer(x, u1, u2, u3, b2, b1, bias=None, precision: str = "fp32"):
    """Differentiable HT layer: y = x W(u1, u2, u3, b2, b1)^T + bias."""
    return HTLayerFunction.apply(x, u1, u2, u3, b2, b1, bias.reshape(-1) if bias is not None else None, precision)


def ht_init(weight, rank: int, N: Sequence[int], M: Sequence[int], precision: str = "fp32"):
    """Mirror of ``ht(data, rank, N, M)`` (mnist_ht.py:167-197): HT factors of an
    ``nn.Linear`` weight (out x in), reshaped C-order to
    ``(N0*M0, N1*M1, N2*M2)``, ranks ``rank`` at every node.  Returns
    ``(u1, u2, u3, b2, b1)`` as contiguous float32 tensors on the weight's
    CUDA device.  The eigenvectors come out in descending eigenvalue order (the
    reference takes ``torch.eig``'s unsorted first columns)."""
    from . import decompose
    from .tree import DimTree
    a, b, c = N[0] * M[0], N[1] * M[1], N[2] * M[2]
    X = _dev(weight).reshape(a, b, c)     # C-order (a, b, c) = column-major (c, b, a)
    # column-major modes: 0 = c, 1 = b, 2 = a.  Nodes: 1 = {a, b}, 2 = {c},
    # 3 = {b} (the reference's node 4), 4 = {a} (the reference's node 3)
    tree = DimTree(3, [(0, 1, 2), (1, 2), (0,), (1,), (2,)], [1, 3, -1, -1, -1], [2, 4, -1, -1, -1],
                   ranks=[1, rank, rank, rank, rank])
    res = decompose(X, tree, dims=(c, b, a), precision=precision)
    u1 = res.U[4].contiguous().reshape(N[0], M[0], rank)
    u2 = res.U[3].contiguous().reshape(N[1], M[1], rank)
    u3 = res.U[2].contiguous().reshape(N[2], M[2], rank)
    b2 = res.B[1].permute(1, 0, 2).contiguous()
    b1 = res.B[0][:, :, 0].contiguous()
    return u1, u2, u3, b2, b1


class HTLinear(torch.nn.Module):
    """The reference's HT layer as an ``nn.Module``: parameters ``u1, u2, u3, b2,
    b1`` and ``bias`` (shaped ``(M0, M1, M2)``), forward ``x W^T + bias`` on the
    GPU.  Build it from an existing weight with :meth:`from_linear` (the
    reference's ``ht()`` initialisation) or with random factors."""

    def __init__(self, N: Sequence[int], M: Sequence[int], rank: int, bias: bool = True,
                 precision: str = "fp32", device="cuda"):
        super().__init__()
        self.N, self.M, self.rank, self.precision = tuple(N), tuple(M), int(rank), precision
        r = int(rank)
        g = lambda *s: torch.nn.Parameter(torch.randn(*s, device=device) / max(1.0, float(s[0] * s[-1])) ** 0.5)
        self.u1 = g(N[0], M[0], r)
        self.u2 = g(N[1], M[1], r)
        self.u3 = g(N[2], M[2], r)
        self.b2 = g(r, r, r)
        self.b1 = g(r, r)
        self.bias = torch.nn.Parameter(torch.zeros(M[0], M[1], M[2], device=device)) if bias else None

    @classmethod
    def from_linear(cls, linear, rank: int, N: Sequence[int], M: Sequence[int], precision: str = "fp32"):
        w = linear.weight.detach().to(device="cuda", dtype=torch.float32)
        layer = cls(N, M, rank, bias=linear.bias is not None, precision=precision, device=w.device)
        with torch.no_grad():
            for p, v in zip((layer.u1, layer.u2, layer.u3, layer.b2, layer.b1), ht_init(w, rank, N, M)):
                p.copy_(v)
            if linear.bias is not None:
                layer.bias.copy_(linear.bias.detach().reshape(M[0], M[1], M[2]))
        return layer

    def weight(self):
        return layer_weight(self.u1, self.u2, self.u3, self.b2, self.b1)

    def forward(self, x):
        y = ht_layer(x.reshape(x.shape[0], -1), self.u1, self.u2, self.u3, self.b2, self.b1, self.bias,
                     self.precision)
        return y
