"""Seeded synthetic tensor families for the HT decomposition path.

The reference generates its test tensors with ``genHtensor``
(``third_order_tensor_decompsition/CUDA/Optimized/kernel.cu:115-224``): random
leaf bases and transfer tensors with ranks drawn from 3..7 under
``srand(time(NULL))``, multiplied out with cuBLAS.  The families here are
seeded (numpy ``default_rng``) so that every run, test and benchmark is
reproducible:

* ``exact_ht``       -- exact HT tensor of given HT ranks plus relative Gaussian noise
                        (QR-orthonormalised Gaussian leaf bases, Gaussian transfer tensors).
* ``odeco``          -- sum_r d_r a_r (x) b_r (x) c_r with orthonormal factors, so every
                        matricisation has singular values |d_r| = r**-decay.
* ``bumps``          -- samples of a sum of separable Gaussian bumps on [0,1]^3.
* ``reference_style``-- the reference's own recipe (uniform [-1,1) factors, ranks 3..7).
* ``batch_family``   -- many small uneven exact-HT tensors.

All tensors are float32, column-major: a numpy array of shape ``dims`` with
Fortran order (``X[i,j,l]`` at flat ``i + n1*j + n1*n2*l``).  For tensors too
large to assemble comfortably on the host, ``assemble_on`` takes a torch
device; the returned torch tensor has shape ``dims[::-1]`` (C-contiguous), which
is the same memory as the column-major tensor.
"""
from __future__ import annotations

from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .tree import DimTree


def _orth(rng: np.random.Generator, n: int, k: int) -> np.ndarray:
    q, r = np.linalg.qr(rng.standard_normal((n, k)))
    return q * np.sign(np.diag(r))


def _node_basis(tree: DimTree, dims: Sequence[int], U: Dict[int, np.ndarray], B: Dict[int, np.ndarray], t: int) -> np.ndarray:
    if tree.is_leaf(t):
        return U[t]
    l, r = tree.left[t], tree.right[t]
    Ul = _node_basis(tree, dims, U, B, l)
    Ur = _node_basis(tree, dims, U, B, r)
    kl, kr = Ul.shape[1], Ur.shape[1]
    Bt = B[t].reshape(kl * kr, -1, order="F")
    # rows: idx_left + n_left * idx_right  ->  kron(U_right, U_left)
    out = np.empty((Ul.shape[0] * Ur.shape[0], Bt.shape[1]), dtype=Ul.dtype)
    tmp = Ul @ Bt.reshape(kl, kr * Bt.shape[1], order="F")          # n_l x (kr*kt)
    tmp = tmp.reshape(Ul.shape[0], kr, Bt.shape[1], order="F")
    # out[il + nl*ir, c] = sum_b tmp[il, b, c] * Ur[ir, b]
    out3 = np.einsum("ibc,jb->ijc", tmp, Ur, optimize=True)
    out[:] = out3.reshape(Ul.shape[0] * Ur.shape[0], Bt.shape[1], order="F")
    return out


def ht_full(tree: DimTree, dims: Sequence[int], U: Dict[int, np.ndarray], B: Dict[int, np.ndarray]) -> np.ndarray:
    """Multiply out an HT representation into a full column-major tensor."""
    l, r = tree.left[0], tree.right[0]
    Ul = _node_basis(tree, dims, U, B, l)
    Ur = _node_basis(tree, dims, U, B, r)
    M = Ul @ B[0].reshape(Ul.shape[1], Ur.shape[1], order="F") @ Ur.T   # X_(left)
    return fold(M, tree.modes[l], dims)


def fold(M: np.ndarray, row_modes: Sequence[int], dims: Sequence[int]) -> np.ndarray:
    """Inverse of the matricisation with rows over ``row_modes``."""
    d = len(dims)
    rest = [m for m in range(d) if m not in row_modes]
    perm = list(row_modes) + rest
    T = M.reshape([dims[m] for m in perm], order="F")
    inv = np.argsort(perm)
    return np.asfortranarray(np.transpose(T, inv))


def exact_ht(dims: Sequence[int], tree: DimTree, noise_rel: float = 0.0, seed: int = 0,
             dtype=np.float32) -> np.ndarray:
    """Exact HT tensor with HT ranks ``tree.ranks`` plus i.i.d. N(0, noise_rel*rms) noise."""
    rng = np.random.default_rng(seed)
    U, B = {}, {}
    for t in tree.leaves():
        U[t] = _orth(rng, int(dims[tree.modes[t][0]]), tree.ranks[t])
    for t in [0] + tree.interior():
        kl, kr = tree.ranks[tree.left[t]], tree.ranks[tree.right[t]]
        B[t] = rng.standard_normal((kl, kr, tree.ranks[t]))
    X = ht_full(tree, dims, U, B)
    if noise_rel > 0:
        rms = np.sqrt(np.mean(X * X))
        X = X + noise_rel * rms * rng.standard_normal(X.shape)
    return np.asfortranarray(X.astype(dtype))


def exact_ht_device(dims: Sequence[int], tree: DimTree, noise_rel: float = 0.0, seed: int = 0, device="cuda"):
    """``exact_ht`` assembled on a torch device: the same seeded factors, the
    noise drawn by torch's generator.  Returns the column-major tensor as a
    contiguous torch tensor of shape ``dims[::-1]``.  Requires every interior
    node's left modes to precede its right modes (true of the reference trees)."""
    import torch
    rng = np.random.default_rng(seed)
    U, B = {}, {}
    for t in tree.leaves():
        U[t] = _orth(rng, int(dims[tree.modes[t][0]]), tree.ranks[t])
    for t in [0] + tree.interior():
        kl, kr = tree.ranks[tree.left[t]], tree.ranks[tree.right[t]]
        B[t] = rng.standard_normal((kl, kr, tree.ranks[t]))
    f = lambda a: torch.as_tensor(a, dtype=torch.float32, device=device)

    def basis(t):   # (prod of node dims with the lowest mode slowest) x k_t
        if tree.is_leaf(t):
            return f(U[t])
        L, R = basis(tree.left[t]), basis(tree.right[t])
        T = torch.einsum("pa,qb,abc->pqc", L, R, f(B[t]))
        return T.reshape(-1, T.shape[-1])

    l, r = tree.left[0], tree.right[0]
    L, R = basis(l), basis(r)
    Xc = (L @ f(B[0]).reshape(L.shape[1], R.shape[1]) @ R.T).reshape(*[int(d) for d in dims])   # X[i0, i1, ...]
    if noise_rel > 0:
        g = torch.Generator(device=device).manual_seed(int(seed))
        rms = torch.sqrt(torch.mean(Xc * Xc))
        Xc = Xc + noise_rel * rms * torch.randn(Xc.shape, generator=g, device=device)
    return Xc.permute(*reversed(range(len(dims)))).contiguous()


def odeco_factors(n: int, order: int = 3, decay: float = 1.5, seed: int = 0, R: Optional[int] = None):
    """Orthonormal factors A_t (n x R) and weights d_r = +-r**-decay."""
    rng = np.random.default_rng(seed)
    R = n if R is None else R
    A = [_orth(rng, n, R) for _ in range(order)]
    d = (np.arange(1, R + 1, dtype=np.float64) ** -decay) * rng.choice([-1.0, 1.0], size=R)
    return A, d


def odeco_optimal_error(n: int, k: int, decay: float = 1.5, R: Optional[int] = None) -> float:
    """Relative error of the best rank-k truncation: sqrt(sum_{r>k} d_r^2 / sum_r d_r^2).
    With orthonormal factors this is also the exact HT truncation error at
    rank k on every node."""
    R = n if R is None else R
    w = np.arange(1, R + 1, dtype=np.float64) ** (-2 * decay)
    return float(np.sqrt(w[k:].sum() / w.sum()))


def _cp_assemble_numpy(A: List[np.ndarray], d: np.ndarray, dtype) -> np.ndarray:
    if len(A) == 3:
        a, b, c = A
        n1, n2, n3 = a.shape[0], b.shape[0], c.shape[0]
        X = np.empty((n1, n2, n3), dtype=dtype, order="F")
        for l in range(n3):
            X[:, :, l] = (a * (d * c[l])) @ b.T
        return X
    a, b, c, e = A
    X = np.empty((a.shape[0], b.shape[0], c.shape[0], e.shape[0]), dtype=dtype, order="F")
    for m in range(e.shape[0]):
        for l in range(c.shape[0]):
            X[:, :, l, m] = (a * (d * c[l] * e[m])) @ b.T
    return X


def _cp_assemble_torch(A: List[np.ndarray], d: np.ndarray, device, chunk: int = 32):
    import torch
    if len(A) != 3:
        raise ValueError("device assembly supports order 3")
    a, b, c = (torch.as_tensor(x, dtype=torch.float32, device=device) for x in A)
    dd = torch.as_tensor(d, dtype=torch.float32, device=device)
    n1, n2, n3 = a.shape[0], b.shape[0], c.shape[0]
    out = torch.empty((n3, n2, n1), dtype=torch.float32, device=device)
    for l0 in range(0, n3, chunk):
        l1 = min(n3, l0 + chunk)
        W = b.unsqueeze(0) * (dd * c[l0:l1]).unsqueeze(1)        # (L, n2, R)
        torch.matmul(W, a.T, out=out[l0:l1])                    # (L, n2, n1): [l, j, i]
    return out


def odeco(n: int, order: int = 3, decay: float = 1.5, seed: int = 0, R: Optional[int] = None,
          assemble_on=None):
    """Orthogonally decomposable tensor: every unfolding has singular values r**-decay."""
    A, d = odeco_factors(n, order, decay, seed, R)
    if assemble_on is not None:
        return _cp_assemble_torch(A, d, assemble_on)
    return _cp_assemble_numpy(A, d, np.float32)


def bump_factors(n: int, seed: int = 0, min_bumps: int = 8, max_bumps: int = 32):
    """Separable Gaussian bumps: f = sum_b amp_b * g_b(x) g_b(y) g_b(z) on the grid i/(n-1)."""
    rng = np.random.default_rng(seed)
    nb = int(rng.integers(min_bumps, max_bumps + 1))
    centres = rng.uniform(0.0, 1.0, size=(nb, 3))
    widths = rng.uniform(0.02, 0.2, size=nb)
    amps = rng.standard_normal(nb)
    grid = np.linspace(0.0, 1.0, n)
    A = [np.exp(-((grid[:, None] - centres[None, :, m]) ** 2) / (2.0 * widths[None, :] ** 2)) for m in range(3)]
    return A, amps


def bumps(n: int, seed: int = 0, assemble_on=None, min_bumps: int = 8, max_bumps: int = 32):
    A, amps = bump_factors(n, seed, min_bumps, max_bumps)
    if assemble_on is not None:
        return _cp_assemble_torch(A, amps, assemble_on)
    return _cp_assemble_numpy(A, amps, np.float32)


def reference_style(n: int, seed: int = 0) -> Tuple[np.ndarray, List[int]]:
    """The reference's ``genHtensor`` recipe (kernel.cu:115-204), seeded: HT ranks
    drawn from 3..7, all factor entries uniform in [-1, 1), tree {1,2},{3}."""
    from .tree import reference_tree_3d
    rng = np.random.default_rng(seed)
    k = [1] + [int(v) for v in rng.integers(3, 8, size=4)]
    tree = reference_tree_3d(k)
    U = {t: rng.uniform(-1.0, 1.0, size=(n, k[t])) for t in (2, 3, 4)}
    B = {1: rng.uniform(-1.0, 1.0, size=(k[3], k[4], k[1])), 0: rng.uniform(-1.0, 1.0, size=(k[1], k[2], 1))}
    X = ht_full(tree, (n, n, n), U, B)
    return np.asfortranarray(X.astype(np.float32)), k


def batch_family(count: int, seed: int = 0, dim_range=(32, 160), rank_range=(8, 16), noise_rel: float = 1e-3,
                 device=None):
    """``count`` exact-HT 3rd-order tensors, dims ~ U[dim_range], ranks ~ U[rank_range].
    With ``device`` the tensors are assembled there (``exact_ht_device``: torch
    tensors shaped dims[::-1], column-major memory); otherwise numpy arrays."""
    from .tree import reference_tree_3d
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        dims = tuple(int(v) for v in rng.integers(dim_range[0], dim_range[1] + 1, size=3))
        r = [1] + [int(v) for v in rng.integers(rank_range[0], rank_range[1] + 1, size=4)]
        # admissible ranks: k_{12} <= k1*k2, k_{12} <= n3, leaves <= n
        r[3] = min(r[3], dims[0]); r[4] = min(r[4], dims[1]); r[2] = min(r[2], dims[2])
        r[1] = min(r[1], r[3] * r[4], dims[2])
        tree = reference_tree_3d(r)
        s_i = int(rng.integers(0, 2**31 - 1))
        X = exact_ht(dims, tree, noise_rel, seed=s_i) if device is None else \
            exact_ht_device(dims, tree, noise_rel, seed=s_i, device=device)
        out.append((X, tree))
    return out
