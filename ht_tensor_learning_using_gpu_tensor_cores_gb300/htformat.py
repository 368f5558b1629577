"""HT-format storage: a decomposition's tree, dimensions and factors in one file.

The reference keeps its factors only in device memory for the length of one
``htd`` call and frees them after measuring the error
(``third_order_tensor_decompsition/CUDA/Optimized/htd_tensorcore.cu:333-350``);
it has no file format.  This one is a numpy ``.npz`` archive:

* ``format``       the string ``"htgb-ht/1"``
* ``dims``         int64[order]
* ``mode_mask``    int64[n_nodes], bit m set when node t holds mode m
* ``left``, ``right``  int64[n_nodes], -1 for leaves
* ``ranks``        int64[n_nodes], ranks[0] = 1
* ``U<t>``         float32 (n_t, k_t) for each leaf t, column-major values
* ``B<t>``         float32 (k_left, k_right, k_t) for the root and each interior node

Arrays are stored with their logical shapes (numpy keeps the element order),
so ``np.load`` of the file gives the factors directly.  Loading validates the
tree and every factor's shape before returning.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, Sequence

import numpy as np

from .tree import DimTree

FORMAT = "htgb-ht/1"


@dataclass
class HTTensor:
    """A tensor in HT format: tree (with ranks), dims, leaf bases U and transfer tensors B."""
    tree: DimTree
    dims: tuple
    U: Dict[int, np.ndarray]
    B: Dict[int, np.ndarray]

    def n_parameters(self) -> int:
        return int(sum(a.size for a in self.U.values()) + sum(a.size for a in self.B.values()))

    def compression(self) -> float:
        """Dense entries per stored parameter."""
        return float(np.prod(self.dims)) / max(self.n_parameters(), 1)


def _host(a) -> np.ndarray:
    if type(a).__module__.startswith("torch"):
        a = a.detach().cpu().numpy()
    return np.asarray(a, dtype=np.float32)


def factor_shapes(tree: DimTree, dims: Sequence[int]) -> Dict[str, tuple]:
    shapes = {}
    for t in tree.leaves():
        shapes[f"U{t}"] = (int(dims[tree.modes[t][0]]), tree.ranks[t])
    for t in [0] + tree.interior():
        shapes[f"B{t}"] = (tree.ranks[tree.left[t]], tree.ranks[tree.right[t]], tree.ranks[t])
    return shapes


def from_result(res) -> HTTensor:
    """An HTTensor on the host from a decompose() result (numpy or torch factors)."""
    return HTTensor(res.tree, tuple(int(d) for d in res.dims), {t: _host(a) for t, a in res.U.items()},
                    {t: _host(a) for t, a in res.B.items()})


def save(path: str, tree: DimTree, dims: Sequence[int], U: Dict[int, object], B: Dict[int, object]) -> None:
    """Write an HT representation (numpy or torch factors) to ``path`` (.npz)."""
    dims = tuple(int(d) for d in dims)
    tree.check_ranks(dims)
    shapes = factor_shapes(tree, dims)
    arrays = {"format": np.array(FORMAT), "dims": np.array(dims, np.int64),
              "mode_mask": np.array([tree.mode_mask(t) for t in range(tree.n_nodes)], np.int64),
              "left": np.array(tree.left, np.int64), "right": np.array(tree.right, np.int64),
              "ranks": np.array(tree.ranks, np.int64)}
    for name, shape in shapes.items():
        src = U if name[0] == "U" else B
        t = int(name[1:])
        if t not in src:
            raise ValueError(f"missing factor {name}")
        a = _host(src[t])
        if a.shape != shape:
            raise ValueError(f"{name} has shape {a.shape}, expected {shape}")
        arrays[name] = a
    with open(path, "wb") as f:
        np.savez(f, **arrays)


def load(path: str) -> HTTensor:
    """Read an HT representation written by :func:`save`."""
    with np.load(path, allow_pickle=False) as z:
        if "format" not in z.files or str(z["format"]) != FORMAT:
            raise ValueError(f"{path}: not an {FORMAT} file")
        dims = tuple(int(d) for d in z["dims"])
        masks = [int(m) for m in z["mode_mask"]]
        modes = [tuple(m for m in range(len(dims)) if mask >> m & 1) for mask in masks]
        tree = DimTree(len(dims), modes, [int(v) for v in z["left"]], [int(v) for v in z["right"]])
        tree = tree.with_ranks([int(v) for v in z["ranks"]])
        tree.check_ranks(dims)
        U, B = {}, {}
        for name, shape in factor_shapes(tree, dims).items():
            if name not in z.files:
                raise ValueError(f"{path}: missing factor {name}")
            a = np.asarray(z[name], dtype=np.float32)
            if a.shape != shape:
                raise ValueError(f"{path}: {name} has shape {a.shape}, expected {shape}")
            (U if name[0] == "U" else B)[int(name[1:])] = a
    return HTTensor(tree, dims, U, B)
