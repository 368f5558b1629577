"""Generate golden vectors by running the reference's own Python HT statements.

Run where a checkout of the reference is available, naming its root in
HT_REFERENCE_DIR (required; there is no default):

    HT_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py

The reference scripts
  third_order_tensor_decompsition/Python/HT_TensorLy.py
  third_order_tensor_decompsition/Python/HT_TensorNetwork.py
  fourth_order_tensor_decomposition/single_GPU/Python/HT_4d_TensorNetwork.py
are executed unmodified except for the problem size line ``n=...`` (the
shipped sizes, 160 / 560 / 120, give fixtures of many MB).  For the HT tensor
layer (HT_tensor_layer/FC_MNIST/mnist_ht.py) the ``ht()`` function and the
einsum chain of ``tNet.forward`` are executed as written (``make_ht_layer``).  Their third-party
dependencies are not installed here, so this script supplies small stand-ins
that restate the published semantics of the calls the scripts make:

* tensorly (unpinned; API as in tensorly 0.4-0.8, pytorch backend):
  ``unfold(T, m) = moveaxis(T, m, 0).reshape(shape[m], -1)``, ``fold`` its
  inverse, ``tenalg.multi_mode_dot`` (a chain of ``mode_dot``; ``transpose=True``
  uses the transposed matrices), ``tensor_to_vec``/``vec_to_tensor`` (C-order
  reshape), ``tensor`` (to a torch tensor).
* tensornetwork (unpinned): ``ncon`` with the standard convention (positive
  labels are summed, negative labels -1, -2, ... give the output axes in that
  order), evaluated with ``torch.einsum``.
* ``torch.eig`` (removed in torch 2.x): LAPACK ``?geev`` with right eigenvectors
  only, eigenvalues returned as an (n, 2) [real, imag] tensor -- the routine and
  return convention torch.eig had on CPU.
* ``cuda:0`` / ``.cuda()`` / ``torch.cuda.synchronize``: the scripts run on CPU.

Inputs are seeded (numpy / torch RNG) before each run.  Outputs are stored as
float32 arrays in the reference's own (C-order, torch) index convention; the
tests map them to the column-major convention of this project.
"""
from __future__ import annotations

import os
import re
import sys
import types

import numpy as np
import torch

REF = os.environ.get("HT_REFERENCE_DIR", "")
OUT = os.path.dirname(os.path.abspath(__file__))


# --------------------------------------------------------------------- shims
def _install_shims():
    def unfold(tensor, mode):
        return torch.moveaxis(tensor, mode, 0).reshape(tensor.shape[mode], -1)

    def fold(unfolded, mode, shape):
        full = list(shape)
        mode_dim = full.pop(mode)
        full.insert(0, mode_dim)
        return torch.moveaxis(unfolded.reshape(full), 0, mode)

    def mode_dot(tensor, matrix, mode):
        new_shape = list(tensor.shape)
        new_shape[mode] = matrix.shape[0]
        res = matrix @ unfold(tensor, mode)
        return fold(res, mode, new_shape)

    def multi_mode_dot(tensor, matrix_or_vec_list, modes=None, skip=None, transpose=False):
        if modes is None:
            modes = range(len(matrix_or_vec_list))
        res = tensor
        for i, (m, mode) in enumerate(zip(matrix_or_vec_list, modes)):
            if skip is not None and i == skip:
                continue
            res = mode_dot(res, m.T if transpose else m, mode)
        return res

    def tensor(data, device=None, dtype=None, **kw):
        return torch.as_tensor(np.asarray(data) if not torch.is_tensor(data) else data, dtype=dtype)

    tl = types.ModuleType("tensorly")
    tl.unfold, tl.fold, tl.tensor = unfold, fold, tensor
    tl.tensor_to_vec = lambda t: t.reshape(-1)
    tl.vec_to_tensor = lambda v, shape: v.reshape(shape)
    tl.set_backend = lambda name: None
    tl.tenalg = types.ModuleType("tensorly.tenalg")
    tl.tenalg.multi_mode_dot = multi_mode_dot
    tl.tenalg.mode_dot = mode_dot
    tl.decomposition = types.ModuleType("tensorly.decomposition")
    tl.decomposition.__all__ = []
    tl.__all__ = ["unfold", "fold", "tensor_to_vec", "vec_to_tensor"]
    sys.modules["tensorly"] = tl
    sys.modules["tensorly.tenalg"] = tl.tenalg
    sys.modules["tensorly.decomposition"] = tl.decomposition

    def ncon(tensors, network, **kw):
        letters = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"
        lab = {}
        specs = []
        for idx in network:
            s = ""
            for v in idx:
                if v not in lab:
                    lab[v] = letters[len(lab)]
                s += lab[v]
            specs.append(s)
        outs = sorted([v for v in lab if v < 0], reverse=True)
        return torch.einsum(",".join(specs) + "->" + "".join(lab[v] for v in outs), *tensors)

    tn = types.ModuleType("tensornetwork")
    tn.ncon = ncon
    tn.set_default_backend = lambda name: None
    sys.modules["tensornetwork"] = tn

    def eig(A, eigenvectors=False):
        from scipy.linalg import lapack
        a = A.detach().cpu().numpy()
        geev = lapack.sgeev if a.dtype == np.float32 else lapack.dgeev
        wr, wi, vl, vr, info = geev(a, compute_vl=0, compute_vr=1 if eigenvectors else 0)
        e = torch.as_tensor(np.stack([wr, wi], axis=1))
        v = torch.as_tensor(vr) if eigenvectors else torch.empty(0)
        return e, v

    torch.eig = eig
    torch.cuda.synchronize = lambda *a, **k: None
    torch.Tensor.cuda = lambda self, *a, **k: self


def _source(rel, n):
    src = open(os.path.join(REF, rel), encoding="utf-8").read()
    src, cnt = re.subn(r"(?m)^n\s*=\s*\d+\s*$", f"n={n}", src)
    assert cnt == 1, rel
    return src


def _run(rel, n, seed, split_marker=None):
    src = _source(rel, n)
    np.random.seed(seed)
    torch.manual_seed(seed)
    ns = {"__name__": "__ref__"}
    if split_marker is None:
        exec(compile(src, rel, "exec"), ns)
        return ns, ns
    i = src.index(split_marker)
    exec(compile(src[:i], rel, "exec"), ns)
    snap = {k: (list(v) if isinstance(v, list) else v) for k, v in ns.items()}
    exec(compile(src[i:], rel, "exec"), ns)
    return snap, ns


def _np(t):
    return t.detach().cpu().numpy().astype(np.float32)


def make_tensorly(n, seed):
    rel = "third_order_tensor_decompsition/Python/HT_TensorLy.py"
    snap, ns = _run(rel, n, seed, split_marker="#还原")
    U, B = snap["U"], snap["B"]
    out = dict(X=_np(ns["X"]), U1=_np(U[1]), U2=_np(U[2]), U3=_np(U[3]), U4=_np(U[4]),
               B1=_np(B[1]), B0=_np(B[0]), err=np.float32(float(ns["err"])),
               k=np.array(ns["k"], dtype=np.int32), n=np.int32(n), seed=np.int32(seed))
    np.savez_compressed(os.path.join(OUT, f"ref_tensorly_3d_n{n}_s{seed}.npz"), **out)
    return out


def make_tensornetwork_3d(n, seed):
    rel = "third_order_tensor_decompsition/Python/HT_TensorNetwork.py"
    snap, ns = _run(rel, n, seed, split_marker="#还原原始tensor")
    Un, B = snap["U_node"], snap["B"]
    out = dict(X=_np(ns["U"][0]), U1=_np(Un[1].reshape(n * n, -1)), U2=_np(Un[2]), U3=_np(Un[3]),
               U4=_np(Un[4]), B1=_np(B[1]), B0=_np(B[0]), err=np.float32(float(ns["err"])),
               k=np.array(ns["k"], dtype=np.int32), n=np.int32(n), seed=np.int32(seed))
    np.savez_compressed(os.path.join(OUT, f"ref_tensornetwork_3d_n{n}_s{seed}.npz"), **out)
    return out


def make_tensornetwork_4d(n, seed):
    rel = "fourth_order_tensor_decomposition/single_GPU/Python/HT_4d_TensorNetwork.py"
    _, ns = _run(rel, n, seed)
    U, B = ns["U"], ns["B"]
    X = ns["U"][0]
    out = dict(X=_np(X), U1=_np(U[1].reshape(n * n, -1)), U2=_np(U[2].reshape(n * n, -1)),
               U3=_np(U[3]), U4=_np(U[4]), U5=_np(U[5]), U6=_np(U[6]),
               B0=_np(B[0]), B1=_np(B[1]), B2=_np(B[2]),
               k=np.array(ns["k"], dtype=np.int32), n=np.int32(n), seed=np.int32(seed))
    np.savez_compressed(os.path.join(OUT, f"ref_tensornetwork_4d_n{n}_s{seed}.npz"), **out)
    return out


def make_ht_layer(seed, N=(4, 4, 6), M=(4, 5, 4), rank=4, batch=5):
    """The HT tensor layer of HT_tensor_layer/FC_MNIST/mnist_ht.py: its ``ht()``
    initialisation (lines 167-197) run as written on a seeded weight, and the
    einsum chain of ``tNet.forward`` (lines 233-240) on a seeded input, with the
    gradients torch autograd gives that chain for a seeded output cotangent.  The
    module's other lines (datasets, training loop, thop/torchvision imports) are
    not executed; the reshape to the layer's (N0, N1, N2) input is restated for
    these small sizes."""
    rel = "HT_tensor_layer/FC_MNIST/mnist_ht.py"
    src = open(os.path.join(REF, rel), encoding="utf-8").read()
    i = src.index("def ht(data,rank,N,M):")
    j = src.index("# ht tensor layer", i)
    ns = {"torch": torch, "tn": sys.modules["tensornetwork"]}
    exec(compile(src[i:j], rel, "exec"), ns)
    k = src.index("def forward(self, x):", src.index("class tNet"))
    body = src[k:src.index("x = x + self.b1", k) + len("x = x + self.b1")]
    chain = [l.strip() for l in body.splitlines() if l.strip().startswith("x = torch.einsum(")]
    assert len(chain) == 5, chain
    torch.manual_seed(seed)
    nin, nout = int(np.prod(N)), int(np.prod(M))
    W = torch.randn(nout, nin) / np.sqrt(nin)
    u1, u2, u3, b2, b1 = ns["ht"](W, rank, list(N), list(M))
    x0 = torch.randn(batch, nin)
    bias0 = torch.randn(*M)
    dy = torch.randn(batch, nout)
    params = [t.detach().clone().float().requires_grad_(True) for t in (u1, u2, u3, b2, b1, bias0, x0)]
    self_ = types.SimpleNamespace(u1_1=params[0], u2_1=params[1], u3_1=params[2], b2_1=params[3], b1_1=params[4],
                                  b1=params[5])
    loc = {"torch": torch, "self": self_, "x": torch.reshape(params[6], (batch, *N))}
    for line in chain:
        exec(line, {}, loc)
    exec("x = x + self.b1", {}, loc)
    y = torch.reshape(loc["x"], (batch, nout))
    y.backward(dy)
    names = ["u1", "u2", "u3", "b2", "b1", "bias", "x"]
    out = dict(W=_np(W), N=np.array(N, dtype=np.int32), M=np.array(M, dtype=np.int32), rank=np.int32(rank),
               y=_np(y), dy=_np(dy), seed=np.int32(seed))
    for nm, t in zip(names, params):
        out[nm] = _np(t)
        out["g_" + nm] = _np(t.grad)
    np.savez_compressed(os.path.join(OUT, f"ref_htlayer_s{seed}.npz"), **out)
    return out


if __name__ == "__main__":
    if not REF or not os.path.isdir(REF):
        sys.exit("set HT_REFERENCE_DIR to the root of a reference checkout")
    _install_shims()
    torch.set_num_threads(4)
    for n, seed in [(24, 1), (32, 2)]:
        o = make_tensorly(n, seed)
        print("tensorly 3d", n, seed, "err", float(o["err"]))
    for n, seed in [(16, 4), (20, 5)]:
        o = make_tensornetwork_3d(n, seed)
        print("tensornetwork 3d", n, seed, "err", float(o["err"]))
    for n, seed in [(20, 6)]:
        o = make_tensornetwork_4d(n, seed)
        print("tensornetwork 4d", n, seed, "k", o["k"].tolist())
    for seed in (7,):
        o = make_ht_layer(seed)
        print("ht layer", seed, "y", o["y"].shape)
