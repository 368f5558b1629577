"""GB300-native hierarchical Tucker (HT) decomposition.

Host-side mirror of the reference's entry points
(``third_order_tensor_decompsition/CUDA/Optimized/function.h:6`` ``htd``,
``fourth_order_tensor_decomposition/single_GPU/CUDA/Optimized/function.h:6``
``htd4``) over the C ABI in ``include/htgb.h``.  All compute runs in the
hand-written sm_103a kernels of ``libhtgb.so``; there is no CPU fallback.

Tensors are column-major (first index fastest), as in the reference's CUDA
code.  A numpy input is a Fortran-ordered array of shape ``dims``; a torch
CUDA input is a contiguous tensor whose memory is the column-major tensor,
i.e. a C-contiguous tensor of shape ``dims[::-1]``.

    import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht
    tree = ht.reference_tree_3d([1, 32, 32, 32, 32])
    res = ht.decompose(X, tree, precision="bf16", compute_error=True)
    res.U[3], res.B[1], res.report["rel_err"]
"""
from __future__ import annotations

import ctypes
from ctypes import c_double, c_int, c_long, c_ulonglong, c_void_p
from dataclasses import dataclass, field
from typing import Dict, Optional, Sequence

import numpy as np

from . import htformat, synth
from ._lib import (FLAG_COMPUTE_ERROR, HTError, HtBatchReport, HtConfig, HtReport, HtTree, LEAF_GRAM, LEAF_SKETCH, PREC_BF16,
                   PREC_FP32, check, lib)
from .tree import (DimTree, balanced_tree_4d, left_first_tree_3d, middle_tree_3d, reference_tree_3d,
                   uniform_ranks)

__all__ = ["DimTree", "reference_tree_3d", "left_first_tree_3d", "middle_tree_3d", "balanced_tree_4d",
           "uniform_ranks", "decompose", "decompose_streaming", "reconstruct_error", "reconstruct", "evaluate", "htformat", "htd", "htd4", "HTResult", "HTError", "synth",
           "workspace_size", "release_workspace", "kernel_launch_count", "BatchDecomposer", "release_batch"]

_PREC = {"fp32": PREC_FP32, "bf16": PREC_BF16}


_TREE_STRUCTS: Dict[tuple, HtTree] = {}


def _tree_struct(tree: DimTree) -> HtTree:
    """The C struct of a tree (cached by the tree's contents: the C side only
    reads it)."""
    key = (tree.order, tuple(tree.left), tuple(tree.right), tuple(tree.ranks), tuple(map(tuple, tree.modes)))
    t = _TREE_STRUCTS.get(key)
    if t is None:
        t = _make_tree_struct(tree)
        if len(_TREE_STRUCTS) >= 256:
            _TREE_STRUCTS.clear()
        _TREE_STRUCTS[key] = t
    return t


def _make_tree_struct(tree: DimTree) -> HtTree:
    f = tree.as_struct_fields()
    t = HtTree()
    t.order, t.n_nodes = f["order"], f["n_nodes"]
    for name in ("parent", "left", "right", "mode_mask", "rank"):
        arr = getattr(t, name)
        for i, v in enumerate(f[name]):
            arr[i] = int(v) if v is not None else -1
    return t


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


@dataclass
class HTResult:
    """U[t] for leaves (n_t x k_t, column-major), B[t] for interior nodes and the
    root (k_left x k_right x k_t, column-major) and the run report."""
    tree: DimTree
    dims: tuple
    U: Dict[int, object] = field(default_factory=dict)
    B: Dict[int, object] = field(default_factory=dict)
    report: Dict[str, object] = field(default_factory=dict)


def _dims_of(x, tree: DimTree, dims: Optional[Sequence[int]]):
    if dims is not None:
        dims = tuple(int(d) for d in dims)
    elif _is_torch(x):
        if x.dim() != tree.order:
            raise ValueError("pass dims= for a torch tensor that is not shaped dims[::-1]")
        dims = tuple(int(d) for d in reversed(x.shape))
    else:
        if x.ndim != tree.order:
            raise ValueError("pass dims= for a flat numpy buffer")
        dims = tuple(int(d) for d in x.shape)
    if len(dims) != tree.order:
        raise ValueError(f"tree has order {tree.order}, dims has {len(dims)} entries")
    return dims


def _host_input(x, dims):
    a = np.asarray(x)
    if a.dtype != np.float32:
        raise TypeError("the tensor must be float32")
    if a.ndim == len(dims) and tuple(a.shape) == tuple(dims):
        a = np.asfortranarray(a)
        return a, a.ctypes.data
    a = np.ascontiguousarray(a).reshape(-1)
    if a.size != int(np.prod(dims)):
        raise ValueError("buffer size does not match dims")
    return a, a.ctypes.data


def _out_buffers(tree: DimTree, dims, like):
    U, B = {}, {}
    if like is None:
        for t in tree.leaves():
            U[t] = np.zeros((dims[tree.modes[t][0]], tree.ranks[t]), dtype=np.float32, order="F")
        for t in [0] + tree.interior():
            kl, kr = tree.ranks[tree.left[t]], tree.ranks[tree.right[t]]
            B[t] = np.zeros((kl, kr, tree.ranks[t]), dtype=np.float32, order="F")
        ptr = lambda a: a.ctypes.data
    else:
        # column-major factors allocated directly (one torch call each); the
        # call writes every element, so they are not cleared
        import torch
        dev = like.device
        for t in tree.leaves():
            n, k = dims[tree.modes[t][0]], tree.ranks[t]
            U[t] = torch.empty_strided((n, k), (1, n), dtype=torch.float32, device=dev)
        for t in [0] + tree.interior():
            kl, kr, kt = tree.ranks[tree.left[t]], tree.ranks[tree.right[t]], tree.ranks[t]
            B[t] = torch.empty_strided((kl, kr, kt), (1, kl, kl * kr), dtype=torch.float32, device=dev)
        ptr = lambda a: a.data_ptr()
    uptr = (c_void_p * 7)()
    bptr = (c_void_p * 7)()
    for t, a in U.items():
        uptr[t] = ptr(a)
    for t, a in B.items():
        bptr[t] = ptr(a)
    return U, B, uptr, bptr


_LEAF = {"gram": LEAF_GRAM, "sketch": LEAF_SKETCH}


_CONFIGS: Dict[tuple, HtConfig] = {}


def _config(precision: str, oversample: int, eig_iters: int, power_steps: int, seed: int, flags: int,
            sketch=None, eig_tol: float = 0.0, leaf_method: str = "gram") -> tuple:
    """(ht_config_t, objects to keep alive during the call).  Configurations
    without sketch blocks are cached: the C side only reads them."""
    if sketch is None:
        key = (precision, oversample, eig_iters, power_steps, seed, flags, eig_tol, leaf_method)
        cfg = _CONFIGS.get(key)
        if cfg is None:
            cfg, _ = _make_config(precision, oversample, eig_iters, power_steps, seed, flags, None, eig_tol,
                                  leaf_method)
            if len(_CONFIGS) >= 256:
                _CONFIGS.clear()
            _CONFIGS[key] = cfg
        return cfg, []
    return _make_config(precision, oversample, eig_iters, power_steps, seed, flags, sketch, eig_tol, leaf_method)


def _make_config(precision: str, oversample: int, eig_iters: int, power_steps: int, seed: int, flags: int,
                 sketch=None, eig_tol: float = 0.0, leaf_method: str = "gram") -> tuple:
    cfg = HtConfig()
    check(lib().ht_config_default(ctypes.byref(cfg)))
    if precision not in _PREC:
        raise ValueError(f"precision must be one of {sorted(_PREC)}")
    if leaf_method not in _LEAF:
        raise ValueError(f"leaf_method must be one of {sorted(_LEAF)}")
    cfg.precision = _PREC[precision]
    cfg.leaf_method = _LEAF[leaf_method]
    cfg.oversample = int(oversample)
    cfg.eig_iters = int(eig_iters)
    cfg.power_steps = int(power_steps)
    cfg.seed = int(seed)
    cfg.flags = int(flags)
    cfg.eig_tol = float(eig_tol)
    keep = []
    if sketch is not None:
        for m, s in enumerate(sketch):
            if s is None:
                continue
            if _is_torch(s):
                if s.dim() != 2 or s.dtype.is_floating_point is False:
                    raise TypeError("a sketch is a 2-D float tensor (n_m x (k + oversample))")
                s = s.float()
                if s.stride() != (1, s.shape[0]):   # the C ABI reads column-major n x s
                    s = s.t().contiguous().t()
                keep.append(s)
                cfg.sketch[m] = s.data_ptr()
            else:
                a = np.asfortranarray(np.asarray(s, dtype=np.float32))
                keep.append(a)
                cfg.sketch[m] = a.ctypes.data
    return cfg, keep


def decompose(x, tree: DimTree, dims: Optional[Sequence[int]] = None, precision: str = "bf16", oversample: int = 16,
              eig_iters: int = 0, power_steps: int = 1, seed: int = 1234, compute_error: bool = False,
              sketch=None, eig_tol: float = 0.0, stream=None, leaf_method: str = "gram") -> HTResult:
    """HT decomposition of a column-major 3rd/4th-order float32 tensor.

    precision="bf16": BF16 tcgen05 GEMMs with FP32 accumulation (the mixed path);
    precision="fp32": every product in FP32 on CUDA cores (the plain path).
    eig_iters: subspace iterations of the leaf solver (0: 10 on FP32, 6 on BF16).
    leaf_method="gram": leaf bases from the mode Grams (subspace iteration,
    eig_iters); "sketch": from the Gram-free range finder on X_(t)
    (power_steps applications of X_(t) X_(t)^T as streaming products, a
    Nystrom core; the interior node from a Householder TSQR).
    sketch: optional per-mode blocks (n_m x (k+p)): the eigen-solver's start
    block ("gram") or the range finder's block S ("sketch").
    """
    dims = _dims_of(x, tree, dims)
    tree.check_ranks(dims)
    flags = FLAG_COMPUTE_ERROR if compute_error else 0
    cfg, keep = _config(precision, oversample, eig_iters, power_steps, seed, flags, sketch, eig_tol, leaf_method)
    ts = _tree_struct(tree)
    cdims = (c_long * 4)(*dims)
    if _is_torch(x):
        import torch
        if not x.is_cuda or x.dtype != torch.float32 or not x.is_contiguous():
            raise TypeError("torch input must be a contiguous float32 CUDA tensor")
        xptr, like = x.data_ptr(), x
        if stream is None:
            stream = torch.cuda.current_stream(x.device).cuda_stream
    else:
        xa, xptr = _host_input(x, dims)
        keep.append(xa)
        like = None
    U, B, uptr, bptr = _out_buffers(tree, dims, like)
    rep = HtReport()
    st = lib().ht_decompose(c_void_p(xptr), cdims, len(dims), ctypes.byref(ts), ctypes.byref(cfg), uptr, bptr,
                            ctypes.byref(rep), c_void_p(stream) if stream else None)
    check(st)
    report = {
        "rel_err": rep.rel_err if compute_error else None,
        "norm_x": rep.norm_x,
        "ms_total": rep.ms_total,
        "ms_stage": {name: rep.ms_stage[i] for i, name in
                     enumerate(["convert", "grams", "eig", "core_pass", "transfer", "error", "h2d", "d2h"])},
        "eig_residual": {t: rep.eig_residual[t] for t in tree.leaves()},
        "gpu_launches": rep.gpu_launches,
        "path": {"tcgen05": bool(rep.path_flags & 1), "simt": bool(rep.path_flags & 2)},
    }
    del keep
    return HTResult(tree, dims, U, B, report)


def decompose_streaming(x, tree: DimTree, slab_bytes: int, dims: Optional[Sequence[int]] = None,
                        precision: str = "bf16", oversample: int = 16, eig_iters: int = 0, seed: int = 1234,
                        compute_error: bool = False, stream=None) -> HTResult:
    """Out-of-core HT decomposition of a 3rd-order float32 tensor that stays in
    host memory (a Fortran-ordered numpy array of shape dims, or a flat buffer
    with dims=): X is streamed through two device slab buffers of at most
    slab_bytes together (ht_decompose_streaming).  Factors come back as numpy
    arrays.  Page-locked host memory (e.g. from torch's pin_memory) gives the
    full copy bandwidth."""
    if _is_torch(x):   # a contiguous CPU tensor shaped dims[::-1] (its memory is the column-major tensor)
        import torch
        if x.is_cuda or x.dtype != torch.float32 or not x.is_contiguous():
            raise TypeError("decompose_streaming reads a contiguous float32 host tensor; use decompose for device "
                            "tensors")
        dims = tuple(int(d) for d in (dims if dims is not None else reversed(x.shape)))
        keep, xptr = [x], x.data_ptr()
    else:
        dims = _dims_of(x, tree, dims)
        arr, xptr = _host_input(x, dims)
        keep = [arr]
    if len(dims) != 3:
        raise ValueError("decompose_streaming handles 3rd-order tensors")
    tree.check_ranks(dims)
    flags = FLAG_COMPUTE_ERROR if compute_error else 0
    cfg, keep2 = _config(precision, oversample, eig_iters, 1, seed, flags)
    ts = _tree_struct(tree)
    U, B, uptr, bptr = _out_buffers(tree, dims, None)
    rep = HtReport()
    check(lib().ht_decompose_streaming(c_void_p(xptr), (c_long * 4)(*dims), 3, ctypes.byref(ts), ctypes.byref(cfg),
                                       uptr, bptr, ctypes.c_ulonglong(int(slab_bytes)), ctypes.byref(rep),
                                       c_void_p(stream) if stream else None))
    report = {
        "rel_err": rep.rel_err if compute_error else None,
        "norm_x": rep.norm_x,
        "ms_total": rep.ms_total,
        "ms_stage": {name: rep.ms_stage[i] for i, name in
                     enumerate(["pass_grams_12", "pass_gram_3", "eig", "core_pass", "transfer", "error_pass"])},
        "gpu_launches": rep.gpu_launches,
        "path": {"tcgen05": bool(rep.path_flags & 1), "simt": bool(rep.path_flags & 2)},
    }
    del keep, keep2
    return HTResult(tree, dims, U, B, report)


class BatchDecomposer:
    """Many tensors per call through ht_decompose_batched, with output buffers
    that stay fixed between calls so that the recorded CUDA graph is replayed.

        bd = BatchDecomposer(trees, dims_list, precision="bf16", compute_error=True)
        results, report = bd(tensors)      # tensors: contiguous float32 CUDA tensors,
                                           # shaped dims[::-1] (column-major memory)

    The input tensors must also stay the same objects (same device addresses)
    for the graph to be replayed; new contents are fine."""

    def __init__(self, trees: Sequence[DimTree], dims: Sequence[Sequence[int]], precision: str = "bf16",
                 compute_error: bool = True, oversample: int = 16, eig_iters: int = 0, seed: int = 1234,
                 device=None, tuning=None):
        """tuning: None keeps the default launch shape and the given eig_iters /
        oversample; "auto" takes them from the autotuner's table for the bucket
        of the batch's largest dimension (autotune.lookup); a dict with keys
        lanes, eig_ctas, eig_iters, oversample sets them explicitly."""
        import torch
        from . import autotune
        if len(trees) != len(dims) or not trees:
            raise ValueError("one tree per tensor, at least one tensor")
        if tuning == "auto":
            tuning = autotune.lookup(dims, precision=precision)
        self.tuning = dict(tuning) if tuning is not None else None
        if self.tuning is not None:
            eig_iters, oversample = int(self.tuning["eig_iters"]), int(self.tuning["oversample"])
        order = trees[0].order
        if any(t.order != order for t in trees):
            raise ValueError("every tensor of a batch has the same order")
        self.trees = list(trees)
        self.dims = [tuple(int(v) for v in d) for d in dims]
        for t, d in zip(self.trees, self.dims):
            t.check_ranks(d)
        self.order = order
        self.count = len(trees)
        self.compute_error = compute_error
        flags = FLAG_COMPUTE_ERROR if compute_error else 0
        self.cfg, self._keep = _config(precision, oversample, eig_iters, 1, seed, flags, None, 0.0)
        dev = torch.device("cuda") if device is None else torch.device(device)
        self.U, self.B = [], []
        self.uptr = (c_void_p * (7 * self.count))()
        self.bptr = (c_void_p * (7 * self.count))()
        like = torch.empty(1, device=dev)
        for i, (t, d) in enumerate(zip(self.trees, self.dims)):
            U, B, up, bp = _out_buffers(t, d, like)
            self.U.append(U)
            self.B.append(B)
            for k in range(7):
                self.uptr[7 * i + k] = up[k]
                self.bptr[7 * i + k] = bp[k]
        self.ts = (HtTree * self.count)(*[_tree_struct(t) for t in self.trees])
        self.cdims = (c_long * (order * self.count))(*[v for d in self.dims for v in d])
        self.xptr = (c_void_p * self.count)()
        self.rel = (c_double * self.count)()

    def __call__(self, tensors, stream=None):
        import torch
        if len(tensors) != self.count:
            raise ValueError(f"expected {self.count} tensors")
        for i, (x, d) in enumerate(zip(tensors, self.dims)):
            if not (_is_torch(x) and x.is_cuda and x.dtype == torch.float32 and x.is_contiguous()):
                raise TypeError("batched inputs must be contiguous float32 CUDA tensors")
            if tuple(reversed(x.shape)) != d and x.numel() != int(np.prod(d)):
                raise ValueError(f"tensor {i} does not match dims {d}")
            self.xptr[i] = x.data_ptr()
        if stream is None:
            stream = torch.cuda.current_stream(tensors[0].device).cuda_stream
        t = self.tuning or {"lanes": 0, "eig_ctas": 0}
        check(lib().ht_batch_set_tuning(int(t["lanes"]), int(t["eig_ctas"])))
        rep = HtBatchReport()
        check(lib().ht_decompose_batched(self.count, self.xptr, self.cdims, self.order, self.ts, ctypes.byref(self.cfg),
                                         self.uptr, self.bptr, self.rel if self.compute_error else None,
                                         ctypes.byref(rep), c_void_p(stream)))
        results = []
        for i in range(self.count):
            report = {"rel_err": self.rel[i] if self.compute_error else None}
            results.append(HTResult(self.trees[i], self.dims[i], self.U[i], self.B[i], report))
        summary = {"rel_err_p50": rep.rel_err_p50, "rel_err_p99": rep.rel_err_p99, "rel_err_max": rep.rel_err_max,
                   "ms_total": rep.ms_total, "gpu_launches": rep.gpu_launches, "graph_replayed": bool(rep.graph_replayed),
                   "lanes": rep.lanes, "grouped": bool(rep.grouped),
                   "ms_phase": {name: rep.ms_phase[i] for i, name in enumerate(
                       ["conversion_grams", "leaf_solver", "core_pass", "transfer_tails", "error_pass",
                        "copies"])},
                   "note": (lib().ht_last_error() or b"").decode()}
        return results, summary


def release_batch():
    """Free the batched path's cached CUDA graph and workspace."""
    check(lib().ht_release_batch())


def _factor_ptrs(U: Dict[int, object], B: Dict[int, object], keep: list):
    """C pointer tables of column-major factors (numpy or torch; copies are kept alive in keep)."""
    uptr = (c_void_p * 7)()
    bptr = (c_void_p * 7)()

    def p(a):
        if _is_torch(a):
            # factors must be column-major
            if a.dim() == 2 and a.stride() != (1, a.shape[0]):
                a = a.t().contiguous().t()
            keep.append(a)
            return a.data_ptr()
        a = np.asfortranarray(np.asarray(a, dtype=np.float32))
        keep.append(a)
        return a.ctypes.data

    for t, a in U.items():
        uptr[t] = p(a)
    for t, a in B.items():
        if _is_torch(a) and a.dim() == 3:
            a = a.permute(2, 1, 0).contiguous().permute(2, 1, 0)
        bptr[t] = p(a)
    return uptr, bptr


def _factor_device(U: Dict[int, object], B: Dict[int, object]):
    """The CUDA device of torch factors, or None for host factors."""
    for a in list(U.values()) + list(B.values()):
        if _is_torch(a) and a.is_cuda:
            return a.device
    return None


def reconstruct(tree: DimTree, U: Dict[int, object], B: Dict[int, object], dims: Sequence[int], stream=None,
                out=None):
    """The full tensor Xhat of an HT representation, computed on the GPU.

    Torch CUDA factors give a torch tensor shaped ``dims[::-1]`` (its memory is
    the column-major tensor); host factors give a Fortran-ordered numpy array
    of shape ``dims``.  ``out`` (a contiguous float32 CUDA tensor of prod(dims)
    elements) receives the result instead of a new tensor.  The reference forms
    Xhat only to measure the error (3D/Opt/htd_tensorcore.cu:295-331)."""
    dims = tuple(int(d) for d in dims)
    ts = _tree_struct(tree)
    keep = []
    uptr, bptr = _factor_ptrs(U, B, keep)
    dev = _factor_device(U, B)
    if out is not None:
        if not (_is_torch(out) and out.is_cuda and out.is_contiguous() and out.numel() == int(np.prod(dims))):
            raise ValueError("out must be a contiguous CUDA tensor with prod(dims) elements")
        optr = out.data_ptr()
        if stream is None:
            import torch
            stream = torch.cuda.current_stream(out.device).cuda_stream
    elif dev is not None:
        import torch
        out = torch.empty(tuple(reversed(dims)), dtype=torch.float32, device=dev)
        optr = out.data_ptr()
        if stream is None:
            stream = torch.cuda.current_stream(dev).cuda_stream
    else:
        out = np.empty(dims, dtype=np.float32, order="F")
        optr = out.ctypes.data
    check(lib().ht_reconstruct((c_long * 4)(*dims), len(dims), ctypes.byref(ts), uptr, bptr, c_void_p(optr),
                               c_void_p(stream) if stream else None))
    return out


def evaluate(tree: DimTree, U: Dict[int, object], B: Dict[int, object], dims: Sequence[int], idx, stream=None):
    """Entries Xhat[idx[e, 0], ..., idx[e, order-1]] (0-based) of an HT
    representation without forming Xhat.  idx: (count, order) integers, numpy or
    torch; the result matches idx's library (numpy float32 or torch float32 on
    idx's device)."""
    dims = tuple(int(d) for d in dims)
    ts = _tree_struct(tree)
    keep = []
    uptr, bptr = _factor_ptrs(U, B, keep)
    if _is_torch(idx):
        import torch
        ix = idx.to(torch.int64).contiguous()
        if ix.dim() != 2 or ix.shape[1] != len(dims):
            raise ValueError("idx must be (count, order)")
        count = ix.shape[0]
        out = torch.empty(count, dtype=torch.float32, device=ix.device)
        iptr, optr = ix.data_ptr(), out.data_ptr()
        if stream is None and ix.is_cuda:
            stream = torch.cuda.current_stream(ix.device).cuda_stream
    else:
        ix = np.ascontiguousarray(np.asarray(idx, dtype=np.int64))
        if ix.ndim != 2 or ix.shape[1] != len(dims):
            raise ValueError("idx must be (count, order)")
        count = ix.shape[0]
        out = np.empty(count, dtype=np.float32)
        iptr, optr = ix.ctypes.data, out.ctypes.data
    check(lib().ht_evaluate((c_long * 4)(*dims), len(dims), ctypes.byref(ts), uptr, bptr, c_void_p(iptr),
                            count, c_void_p(optr), c_void_p(stream) if stream else None))
    return out


def reconstruct_error(x, tree: DimTree, U: Dict[int, object], B: Dict[int, object],
                      dims: Optional[Sequence[int]] = None, stream=None) -> float:
    """||X - Xhat||_F / ||X||_F computed on the GPU without materialising Xhat."""
    dims = _dims_of(x, tree, dims)
    ts = _tree_struct(tree)
    cdims = (c_long * 4)(*dims)
    keep = []
    if _is_torch(x):
        import torch
        xptr = x.data_ptr()
        if stream is None:
            stream = torch.cuda.current_stream(x.device).cuda_stream
    else:
        xa, xptr = _host_input(x, dims)
        keep.append(xa)
    uptr, bptr = _factor_ptrs(U, B, keep)
    out = c_double(0.0)
    check(lib().ht_reconstruct_error(c_void_p(xptr), cdims, len(dims), ctypes.byref(ts), uptr, bptr,
                                     ctypes.byref(out), c_void_p(stream) if stream else None))
    return float(out.value)


def htd(x: np.ndarray, k: Sequence[int]) -> float:
    """Mirror of ``float htd(dt *x, long a, long b, long c, int *k)``
    (3D/Opt/function.h:6): x is a host a x b x c column-major tensor, k the
    5 ranks by node id; returns the relative reconstruction error."""
    a = np.asfortranarray(np.asarray(x, dtype=np.float32))
    if a.ndim != 3:
        raise ValueError("htd takes a 3rd-order tensor")
    kk = (c_int * 5)(*[int(v) for v in k])
    e = lib().htd(c_void_p(a.ctypes.data), a.shape[0], a.shape[1], a.shape[2], kk)
    if e < 0:
        raise HTError(1, lib().ht_last_error().decode(errors="replace"))
    return float(e)


def htd4(x: np.ndarray, k: Sequence[int]) -> None:
    """Mirror of ``void htd4(dt *X, long a, long b, long c, long d, int *k, ...)``
    (4D/Opt/function.h:6); prints the error rate as the reference does."""
    a = np.asfortranarray(np.asarray(x, dtype=np.float32))
    if a.ndim != 4:
        raise ValueError("htd4 takes a 4th-order tensor")
    kk = (c_int * 7)(*[int(v) for v in k])
    lib().htd4(c_void_p(a.ctypes.data), a.shape[0], a.shape[1], a.shape[2], a.shape[3], kk, None, None)


def workspace_size(dims: Sequence[int], tree: DimTree, precision: str = "bf16", compute_error: bool = False) -> int:
    cfg, _ = _config(precision, 16, 10, 1, 1234, FLAG_COMPUTE_ERROR if compute_error else 0)
    out = c_ulonglong(0)
    check(lib().ht_workspace_size((c_long * 4)(*dims), len(dims), ctypes.byref(_tree_struct(tree)),
                                  ctypes.byref(cfg), ctypes.byref(out)))
    return int(out.value)


def release_workspace() -> None:
    check(lib().ht_release_workspace())


def kernel_launch_count() -> int:
    return int(lib().ht_kernel_launch_count())


def _prim_input(x, dims):
    if _is_torch(x):
        return x, x.data_ptr(), x
    a, p = _host_input(x, dims)
    return a, p, None


def _prim_view(dims, lo, hi):
    L = int(np.prod(dims[:lo])) if lo > 0 else 1
    N = int(np.prod(dims[lo:hi + 1]))
    R = int(np.prod(dims[hi + 1:])) if hi + 1 < len(dims) else 1
    return L, N, R


def _prim_out(shape, like):
    if like is None:
        a = np.zeros(shape, dtype=np.float32, order="F")
        return a, a.ctypes.data
    import torch
    t = torch.zeros(tuple(reversed(shape)), dtype=torch.float32, device=like.device).t()
    return t, t.data_ptr()


def _prim_mat(m, like):
    if _is_torch(m):
        m = m.t().contiguous().t() if m.stride(0) != 1 else m
        return m, m.data_ptr()
    a = np.asfortranarray(np.asarray(m, dtype=np.float32))
    return a, a.ctypes.data


def _stream_of(like):
    if like is None:
        return None
    import torch
    return c_void_p(torch.cuda.current_stream(like.device).cuda_stream)


def mode_gram(x, dims: Sequence[int], lo: int, hi: Optional[int] = None, precision: str = "bf16"):
    """G = X_(g) X_(g)^T for the contiguous mode group lo..hi (0-based)."""
    hi = lo if hi is None else hi
    dims = tuple(int(d) for d in dims)
    keep, xp, like = _prim_input(x, dims)
    L, N, R = _prim_view(dims, lo, hi)
    out, op = _prim_out((N, N), like)
    check(lib().ht_mode_gram(c_void_p(xp), (c_long * 4)(*dims), len(dims), lo, hi, _PREC[precision], c_void_p(op),
                             _stream_of(like)))
    return out


def mode_product(x, dims: Sequence[int], lo: int, W, hi: Optional[int] = None, precision: str = "bf16"):
    """Z ((L*R) x k) = X_(g)^T W: the mode-group product with W (N x k)."""
    hi = lo if hi is None else hi
    dims = tuple(int(d) for d in dims)
    keep, xp, like = _prim_input(x, dims)
    L, N, R = _prim_view(dims, lo, hi)
    Wk, wp = _prim_mat(W, like)
    k = int(Wk.shape[1])
    out, op = _prim_out((L * R, k), like)
    check(lib().ht_mode_product(c_void_p(xp), (c_long * 4)(*dims), len(dims), lo, hi, c_void_p(wp), k,
                                _PREC[precision], c_void_p(op), _stream_of(like)))
    return out


def corange_product(x, dims: Sequence[int], lo: int, Q, hi: Optional[int] = None, precision: str = "bf16"):
    """Z (N x k) = X_(g) Q: contract every mode outside the group with Q ((L*R) x k)."""
    hi = lo if hi is None else hi
    dims = tuple(int(d) for d in dims)
    keep, xp, like = _prim_input(x, dims)
    L, N, R = _prim_view(dims, lo, hi)
    Qk, qp = _prim_mat(Q, like)
    k = int(Qk.shape[1])
    out, op = _prim_out((N, k), like)
    check(lib().ht_corange_product(c_void_p(xp), (c_long * 4)(*dims), len(dims), lo, hi, c_void_p(qp), k,
                                   _PREC[precision], c_void_p(op), _stream_of(like)))
    return out


def tsqr(A):
    """R factor (k x k, upper triangular, non-negative diagonal) of a tall-skinny
    float32 matrix A (m x k, k <= 64) by the GPU Householder TSQR (ht_tsqr).
    A: a numpy array (any order) or a float32 CUDA tensor of shape (m, k) whose
    columns are contiguous (e.g. the transpose of a contiguous (k, m) tensor).
    Returns the same kind as A."""
    if _is_torch(A):
        import torch
        if not A.is_cuda or A.dtype != torch.float32 or A.dim() != 2 or A.stride(0) != 1:
            raise TypeError("A must be a float32 CUDA tensor (m, k) with contiguous columns")
        m, k = int(A.shape[0]), int(A.shape[1])
        R = torch.empty((k, k), dtype=torch.float32, device=A.device).t()   # column-major storage
        check(lib().ht_tsqr(c_void_p(A.data_ptr()), m, k, max(int(A.stride(1)), m), c_void_p(R.data_ptr()),
                            c_void_p(torch.cuda.current_stream(A.device).cuda_stream)))
        return R
    a = np.asfortranarray(np.asarray(A, dtype=np.float32))
    m, k = a.shape
    R = np.zeros((k, k), dtype=np.float32, order="F")
    check(lib().ht_tsqr(c_void_p(a.ctypes.data), m, k, m, c_void_p(R.ctypes.data), None))
    return R


__all__ += ["mode_gram", "mode_product", "corange_product", "tsqr"]
