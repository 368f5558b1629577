"""Dimension trees for hierarchical Tucker (HT) decomposition.

A dimension tree is a binary tree whose root holds all modes of the tensor and
whose leaves hold one mode each.  Nodes are numbered as in the reference:

* 3rd order (``third_order_tensor_decompsition/CUDA/Optimized/ht_init.cu:16-20``,
  ``Python/HT_TensorLy.py:23-24``): 0 = root {1,2,3}, 1 = {1,2}, 2 = {3},
  3 = {1}, 4 = {2}.  The rank vector ``k[]`` is indexed by node id and
  ``k[0] = 1``.
* 4th order (``fourth_order_tensor_decomposition/single_GPU/CUDA/Optimized/
  ht_init.cu:19-23``): 0 = root, 1 = {1,2}, 2 = {3,4}, 3..6 = leaves {1}..{4}.

Modes are 0-based here.  Tensors are column-major (first index fastest), as
in the reference's CUDA code (``htd_tensorcore.cu:12``): element
``(i1, i2, i3)`` of an ``n1 x n2 x n3`` tensor sits at ``i1 + n1*i2 + n1*n2*i3``.
The matricisation ``X_(t)`` of node ``t`` has one row per multi-index over the
modes of ``t`` (lowest mode fastest) and one column per multi-index over the
remaining modes (lowest mode fastest).

Constraint: for every interior node below the root, all modes of the left
child precede all modes of the right child.  Then the row index of ``X_(t)`` is
``row_left + n_left * row_right`` and ``B_t`` (shape ``k_left x k_right x k_t``,
column-major) satisfies ``U_t = (U_right kron U_left) B_t``, the layout the
reference's ``ttm`` writes (``CUDA/Optimized/ttm.cu:2-36``).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

MAX_NODES = 7


@dataclass
class DimTree:
    order: int
    modes: List[Tuple[int, ...]]          # node -> sorted tuple of modes
    left: List[int]                       # -1 for leaves
    right: List[int]
    parent: List[int] = field(default_factory=list)
    ranks: List[int] = field(default_factory=list)

    def __post_init__(self):
        n = len(self.modes)
        if n != 2 * self.order - 1:
            raise ValueError(f"a binary dimension tree of order {self.order} has {2*self.order-1} nodes, got {n}")
        if n > MAX_NODES:
            raise ValueError("at most 7 nodes (order <= 4) are supported")
        self.parent = [-1] * n
        for t in range(n):
            l, r = self.left[t], self.right[t]
            if (l < 0) != (r < 0):
                raise ValueError(f"node {t} must have zero or two children")
            if l >= 0:
                self.parent[l] = t
                self.parent[r] = t
                if set(self.modes[l]) | set(self.modes[r]) != set(self.modes[t]) or set(self.modes[l]) & set(self.modes[r]):
                    raise ValueError(f"children of node {t} must partition its modes")
                if t != 0 and max(self.modes[l]) > min(self.modes[r]):
                    raise ValueError(f"node {t}: left child's modes must precede the right child's")
            elif len(self.modes[t]) != 1:
                raise ValueError(f"leaf {t} must hold exactly one mode")
        if tuple(sorted(self.modes[0])) != tuple(range(self.order)):
            raise ValueError("node 0 must be the root holding every mode")
        if not self.ranks:
            self.ranks = [1] + [0] * (n - 1)

    # ------------------------------------------------------------------ queries
    @property
    def n_nodes(self) -> int:
        return len(self.modes)

    def is_leaf(self, t: int) -> bool:
        return self.left[t] < 0

    def leaves(self) -> List[int]:
        return [t for t in range(self.n_nodes) if self.is_leaf(t)]

    def interior(self) -> List[int]:
        """Interior nodes other than the root."""
        return [t for t in range(1, self.n_nodes) if not self.is_leaf(t)]

    def leaf_of_mode(self, m: int) -> int:
        for t in self.leaves():
            if self.modes[t][0] == m:
                return t
        raise KeyError(m)

    def mode_mask(self, t: int) -> int:
        mask = 0
        for m in self.modes[t]:
            mask |= 1 << m
        return mask

    def with_ranks(self, ranks: Sequence[int]) -> "DimTree":
        ranks = list(int(r) for r in ranks)
        if len(ranks) != self.n_nodes:
            raise ValueError(f"need {self.n_nodes} ranks, got {len(ranks)}")
        ranks[0] = 1
        return DimTree(self.order, list(self.modes), list(self.left), list(self.right), ranks=ranks)

    def check_ranks(self, dims: Sequence[int]) -> None:
        """Ranks must be admissible: 1 <= k_t <= rows of X_(t), and for interior
        nodes k_t <= k_left * k_right (the transfer tensor's row count)."""
        for t in range(1, self.n_nodes):
            rows = 1
            for m in self.modes[t]:
                rows *= int(dims[m])
            cols = 1
            for m in range(self.order):
                if m not in self.modes[t]:
                    cols *= int(dims[m])
            k = self.ranks[t]
            if k < 1 or k > rows or k > cols:
                raise ValueError(f"rank of node {t} ({k}) must lie in [1, min({rows}, {cols})]")
            if not self.is_leaf(t):
                kl, kr = self.ranks[self.left[t]], self.ranks[self.right[t]]
                if k > kl * kr:
                    raise ValueError(f"rank of node {t} ({k}) exceeds k_left*k_right = {kl*kr}")

    def as_struct_fields(self):
        """Fields of the C ``ht_tree_t`` (see include/htgb.h)."""
        n = self.n_nodes
        pad = lambda v: list(v) + [-1] * (MAX_NODES - len(v))
        return dict(order=self.order, n_nodes=n, parent=pad(self.parent), left=pad(self.left),
                    right=pad(self.right), mode_mask=pad([self.mode_mask(t) for t in range(n)]),
                    rank=pad(self.ranks))


def reference_tree_3d(k: Optional[Sequence[int]] = None) -> DimTree:
    """Tree of ``htd`` / ``HT_TensorLy.py``: root -> {1,2},{3}; {1,2} -> {1},{2}."""
    t = DimTree(3, [(0, 1, 2), (0, 1), (2,), (0,), (1,)], [1, 3, -1, -1, -1], [2, 4, -1, -1, -1])
    return t.with_ranks(k) if k is not None else t


def left_first_tree_3d(k: Optional[Sequence[int]] = None) -> DimTree:
    """Tree root -> {1},{2,3}; {2,3} -> {2},{3}.  Node ids: 1 = {1}, 2 = {2,3},
    3 = {2}, 4 = {3}."""
    t = DimTree(3, [(0, 1, 2), (0,), (1, 2), (1,), (2,)], [1, -1, 3, -1, -1], [2, -1, 4, -1, -1])
    return t.with_ranks(k) if k is not None else t


def middle_tree_3d(k: Optional[Sequence[int]] = None) -> DimTree:
    """Tree root -> {2},{1,3}; {1,3} -> {1},{3}.  Node ids: 1 = {2}, 2 = {1,3},
    3 = {1}, 4 = {3}."""
    t = DimTree(3, [(0, 1, 2), (1,), (0, 2), (0,), (2,)], [1, -1, 3, -1, -1], [2, -1, 4, -1, -1])
    return t.with_ranks(k) if k is not None else t


def balanced_tree_4d(k: Optional[Sequence[int]] = None) -> DimTree:
    """Tree of ``htd4``: root -> {1,2},{3,4}; {1,2} -> {1},{2}; {3,4} -> {3},{4}."""
    t = DimTree(4, [(0, 1, 2, 3), (0, 1), (2, 3), (0,), (1,), (2,), (3,)],
                [1, 3, 5, -1, -1, -1, -1], [2, 4, 6, -1, -1, -1, -1])
    return t.with_ranks(k) if k is not None else t


def uniform_ranks(tree: DimTree, r: int, interior: Optional[int] = None) -> DimTree:
    ranks = [1] + [(interior if (interior is not None and not tree.is_leaf(t)) else r) for t in range(1, tree.n_nodes)]
    return tree.with_ranks(ranks)
