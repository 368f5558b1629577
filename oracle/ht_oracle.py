"""CPU oracle for the hierarchical Tucker (HT) decomposition path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; it is
used by ``tests/``, by ``__graft_entry__.smoke()`` as the checker, and by
``bench.py``'s CPU-baseline leg (``cpu_baseline`` / ``--impl reference``).

It is a numpy restatement of the reference's HT algorithm (root-to-leaf
"hierarchical SVD"), following

* ``third_order_tensor_decompsition/Python/HT_TensorLy.py:52-82``  (CPU statement,
  tree and node numbering at ``:23-24``),
* ``third_order_tensor_decompsition/CUDA/Optimized/htd_batch.cu:78-165``  (plain
  FP32 CUDA path: leaf Gram + eigendecomposition, QR-SVD for node {1,2},
  ``ttm`` for the transfer tensors, reconstruction + error ``:196-244``),
* ``fourth_order_tensor_decomposition/single_GPU/Python/HT_4d_TensorNetwork.py:44-69``
  and ``.../CUDA/Optimized/htd4_tensorcore.cu:2-291`` for the 4th-order tree.

Per node t below the root:
  leaf t      U_t = top-k_t eigenvectors of X_(t) X_(t)^T      (htd_batch.cu:83-117, HT_TensorLy.py:61-66)
  interior t  U_t = top-k_t left singular vectors of X_(t)     (htd_batch.cu:146 -> kernel.cu:719, HT_TensorLy.py:55-59)
  interior t  B_t = (U_right kron U_left)^T U_t, stored k_l x k_r x k_t  (ttm.cu:2-36, HT_TensorLy.py:68-72)
  root        B_0 = U_left^T X_(left) U_right                  (htd_batch.cu:165, HT_TensorLy.py:68-72)
Reconstruction and error follow htd_batch.cu:196-244 / HT_TensorLy.py:76-82.

Documented deviations from the reference (both are fixes, not choices):
* eigenvectors are taken in DESCENDING eigenvalue order.  ``HT_TensorLy.py:64-66``
  takes the first k columns of the unsorted ``torch.eig`` output and the CUDA
  code copies the last k columns of the ascending ``syevd`` output; both mean
  "top-k" only by accident of ordering.  ``eig_order="geev"`` reproduces the
  Python statement's unsorted choice exactly (LAPACK ``?geev``, which is what
  ``torch.eig`` called) so the oracle can be pinned to the reference's own
  outputs.
* the interior node uses an exact SVD (the Optimized CUDA ``rsvd`` SVDs only
  the leading ks x ks block of B, ``kernel.cu:641-657``).

Tensors are column-major numpy arrays (Fortran order) as in the reference's
CUDA code (``htd_tensorcore.cu:12``).

Pinned to the reference's own outputs (tests/golden/, made by
tests/golden/make_golden.py, which runs the reference's Python as written):
the decomposition and its error by tests/test_oracle_golden.py (HT_TensorLy.py,
HT_TensorNetwork.py, HT_4d_TensorNetwork.py); the HT tensor layer
(``ht_layer_chain``, ``ht_layer_weight``, ``ht_layer_unfoldings``,
``ht_layer_transfers``) by tests/test_oracle_htlayer_golden.py
(HT_tensor_layer/FC_MNIST/mnist_ht.py).  The learned-sketch objective and its
adjoint have no counterpart in the reference; they are checked against finite
differences (tests/test_sketch_oracle.py).
"""
from __future__ import annotations

from typing import Dict, Sequence, Tuple

import numpy as np


class OTree:
    """The oracle's own description of a dimension tree: per node the sorted
    modes, the children (-1 for leaves) and the rank; node 0 is the root.  It
    is built from plain lists or copied out of any object carrying ``order``,
    ``modes``, ``left``, ``right`` and ``ranks`` (the product's tree class), so
    the oracle shares no mapping code with the product."""

    def __init__(self, order, modes, left, right, ranks):
        self.order = int(order)
        self.modes = [tuple(sorted(int(m) for m in ms)) for ms in modes]
        self.left = [int(v) for v in left]
        self.right = [int(v) for v in right]
        self.ranks = [int(v) for v in ranks]
        self.n_nodes = len(self.modes)
        if self.n_nodes != 2 * self.order - 1 or self.modes[0] != tuple(range(self.order)):
            raise ValueError("not a binary dimension tree with node 0 the root")

    def is_leaf(self, t: int) -> bool:
        return self.left[t] < 0

    def leaves(self):
        return [t for t in range(self.n_nodes) if self.is_leaf(t)]

    def interior(self):
        return [t for t in range(1, self.n_nodes) if not self.is_leaf(t)]


def as_tree(tree) -> OTree:
    if isinstance(tree, OTree):
        return tree
    return OTree(tree.order, tree.modes, tree.left, tree.right, tree.ranks)


def fold(M: np.ndarray, row_modes: Sequence[int], dims: Sequence[int]) -> np.ndarray:
    """Inverse of ``unfold``: the column-major tensor of shape ``dims`` whose
    matricisation with rows over ``row_modes`` is M."""
    rest = [m for m in range(len(dims)) if m not in row_modes]
    perm = list(row_modes) + rest
    T = np.reshape(M, [int(dims[m]) for m in perm], order="F")
    return np.asfortranarray(np.transpose(T, np.argsort(perm)))


def unfold(X: np.ndarray, row_modes: Sequence[int]) -> np.ndarray:
    """Matricisation X_(t): rows over ``row_modes`` (lowest fastest), columns over
    the remaining modes (lowest fastest).  For the reference tree this is
    X_(1) = X as a x (bc) (ld a), X_(12) = X as (ab) x c, X_(3) = X_(12)^T."""
    d = X.ndim
    rest = [m for m in range(d) if m not in row_modes]
    rows = int(np.prod([X.shape[m] for m in row_modes]))
    return np.reshape(np.transpose(X, list(row_modes) + rest), (rows, -1), order="F")


def top_eigvecs(G: np.ndarray, k: int, eig_order: str = "desc") -> Tuple[np.ndarray, np.ndarray]:
    """Top-k eigenpairs of a symmetric Gram.  ``eig_order='geev'`` returns the
    first k columns of LAPACK ?geev's unsorted output (torch.eig semantics,
    HT_TensorLy.py:64-66)."""
    if eig_order == "geev":
        from scipy.linalg import lapack
        geev = lapack.sgeev if G.dtype == np.float32 else lapack.dgeev
        wr, wi, vl, vr, info = geev(G, compute_vl=0, compute_vr=1)
        if info != 0:
            raise RuntimeError(f"geev failed: info={info}")
        return wr[:k], vr[:, :k]
    w, V = np.linalg.eigh(G)
    idx = np.argsort(w)[::-1][:k]
    return w[idx], V[:, idx]


def ht_decompose(X: np.ndarray, tree, dtype=np.float64, eig_order: str = "desc",
                 interior_svd: bool = True):
    """Root-to-leaf HT decomposition (the reference algorithm).

    Returns (U, B, info): U[t] for every non-root node (leaves and interior
    nodes), B[t] (k_l x k_r x k_t, Fortran order) for interior nodes and the
    root (k_l x k_r x 1)."""
    tree = as_tree(tree)
    X = np.asarray(X, dtype=dtype)
    if not X.flags.f_contiguous:
        X = np.asfortranarray(X)
    U: Dict[int, np.ndarray] = {}
    evals: Dict[int, np.ndarray] = {}
    for t in range(1, tree.n_nodes):
        A = unfold(X, tree.modes[t])
        k = tree.ranks[t]
        if tree.is_leaf(t) or not interior_svd:
            G = A @ A.T
            w, V = top_eigvecs(G, k, eig_order)
            U[t] = np.ascontiguousarray(V)
            evals[t] = w
        else:
            Us, s, _ = np.linalg.svd(A, full_matrices=False)
            U[t] = Us[:, :k]
            evals[t] = s[:k] ** 2
    B: Dict[int, np.ndarray] = {}
    for t in tree.interior():
        l, r = tree.left[t], tree.right[t]
        B[t] = transfer_tensor(U[t], U[l], U[r])
    l, r = tree.left[0], tree.right[0]
    M = U[l].T @ unfold(X, tree.modes[l]) @ U[r]
    B[0] = M.reshape(M.shape[0], M.shape[1], 1, order="F")
    return U, B, {"evals": evals}


def transfer_tensor(Ut: np.ndarray, Ul: np.ndarray, Ur: np.ndarray) -> np.ndarray:
    """B_t = (U_r kron U_l)^T U_t as a k_l x k_r x k_t Fortran array (ttm.cu:2-36)."""
    nl, kl = Ul.shape
    nr, kr = Ur.shape
    kt = Ut.shape[1]
    T = Ut.reshape(nl, nr, kt, order="F")
    Bt = np.einsum("ijc,ia,jb->abc", T, Ul, Ur, optimize=True)
    return np.asfortranarray(Bt)


def node_basis(tree, U: Dict[int, np.ndarray], B: Dict[int, np.ndarray], t: int) -> np.ndarray:
    """Reconstructed basis of node t: U_t for leaves, (U_r kron U_l) B_t above."""
    tree = as_tree(tree)
    if tree.is_leaf(t):
        return U[t]
    l, r = tree.left[t], tree.right[t]
    Ul = node_basis(tree, U, B, l)
    Ur = node_basis(tree, U, B, r)
    kt = B[t].shape[2]
    T = np.einsum("ia,jb,abc->ijc", Ul, Ur, B[t], optimize=True)
    return T.reshape(Ul.shape[0] * Ur.shape[0], kt, order="F")


def ht_reconstruct(tree, dims: Sequence[int], U: Dict[int, np.ndarray], B: Dict[int, np.ndarray]) -> np.ndarray:
    """Full tensor from (U_leaf, B_t) (htd_batch.cu:196-224, HT_TensorLy.py:76-81)."""
    tree = as_tree(tree)
    l, r = tree.left[0], tree.right[0]
    Ul = node_basis(tree, U, B, l)
    Ur = node_basis(tree, U, B, r)
    M = Ul @ B[0][:, :, 0] @ Ur.T
    return fold(M, tree.modes[l], dims)


def ht_entries(tree, U: Dict[int, np.ndarray], B: Dict[int, np.ndarray], idx: np.ndarray) -> np.ndarray:
    """Entries Xhat[idx[e]] contracted leaf-to-root without forming Xhat: a leaf
    contributes the row U_t[i_m, :], an interior node
    v_t[c] = sum_{a,b} B_t[a, b, c] v_l[a] v_r[b], and the root's v_0[0] is the
    entry.  The same contraction as ht_reconstruct's node bases
    (htd_batch.cu:196-224), restricted to one row of each."""
    tree = as_tree(tree)
    idx = np.asarray(idx, dtype=np.int64)

    def vec(t):
        if tree.is_leaf(t):
            return U[t][idx[:, tree.modes[t][0]], :].astype(np.float64)
        vl, vr = vec(tree.left[t]), vec(tree.right[t])
        return np.einsum("ea,eb,abc->ec", vl, vr, np.asarray(B[t], np.float64), optimize=True)

    return vec(0)[:, 0]


def rel_error(X: np.ndarray, Xh: np.ndarray) -> float:
    """||X - Xhat||_F / ||X||_F in float64 (htd_batch.cu:237-244)."""
    X = np.asarray(X, dtype=np.float64)
    return float(np.linalg.norm((X - np.asarray(Xh, dtype=np.float64)).ravel()) / np.linalg.norm(X.ravel()))


def ht_error(X: np.ndarray, tree, U, B) -> float:
    tree = as_tree(tree)
    return rel_error(X, ht_reconstruct(tree, X.shape, U, B))


# ----------------------------------------------------------------- comparators
def principal_angles(U1: np.ndarray, U2: np.ndarray) -> np.ndarray:
    """Principal angles (radians) between span(U1) and span(U2); inputs need not
    be orthonormal."""
    Q1, _ = np.linalg.qr(np.asarray(U1, dtype=np.float64))
    Q2, _ = np.linalg.qr(np.asarray(U2, dtype=np.float64))
    s = np.linalg.svd(Q1.T @ Q2, compute_uv=False)
    return np.arccos(np.clip(s, -1.0, 1.0))


def orthogonality_defect(U: np.ndarray) -> float:
    U = np.asarray(U, dtype=np.float64)
    return float(np.abs(U.T @ U - np.eye(U.shape[1])).max())


def procrustes_align(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """Orthogonal Q minimising ||A Q - B||_F."""
    u, _, vt = np.linalg.svd(np.asarray(A, dtype=np.float64).T @ np.asarray(B, dtype=np.float64))
    return u @ vt


def tree_energy_bound(tree) -> float:
    """Quasi-optimality constant of root-to-leaf HT truncation: sqrt(2d-3)."""
    tree = as_tree(tree)
    return float(np.sqrt(2 * tree.order - 3))


# ---------------------------------------------------------------- learned sketch
# The learned start block of the leaf range finder has no counterpart in the
# reference (its rsvd draws a Gaussian test matrix, 3D/Opt/kernel.cu:595-680);
# these are the float64 statements of the training objective and its gradient
# that the GPU forward/adjoint kernels are checked against.
# A column of Y = G S whose CholeskyQR pivot (Schur complement) falls below
# SKETCH_DROP times its squared norm lies in the span of the earlier columns
# to rounding: it is left out of Q (rank-deficient Y, e.g. a Gram of rank
# below the sketch width).  The GPU kernel (csrc/learn.cu) applies the same rule.
SKETCH_DROP = 1e-8


def _sketch_parts(G: np.ndarray, S: np.ndarray):
    """Y = G S, C = Y^T Y, the kept columns K of the pivot-dropping Cholesky."""
    G = np.asarray(G, np.float64)
    Y = G @ np.asarray(S, np.float64)
    C = Y.T @ Y
    s = C.shape[0]
    A = C.copy()
    keep = np.ones(s, dtype=bool)
    d0 = np.diag(C).copy()
    for j in range(s):
        d = A[j, j]
        if not d > SKETCH_DROP * d0[j]:
            keep[j] = False
            continue
        r = A[j, j + 1:] / np.sqrt(d)
        A[j + 1:, j + 1:] -= np.outer(r, r)
    return G, Y, C, keep


def sketch_loss(G: np.ndarray, S: np.ndarray) -> float:
    """1 - tr(Q^T G Q) / tr(G), Q an orthonormal basis of G S (of its kept
    columns when G S is rank deficient)."""
    G, Y, C, K = _sketch_parts(G, S)
    if not K.any():
        return 1.0
    H = Y[:, K].T @ G @ Y[:, K]
    return float(1.0 - np.trace(np.linalg.solve(C[np.ix_(K, K)], H)) / np.trace(G))


def sketch_grad(G: np.ndarray, S: np.ndarray) -> np.ndarray:
    """d sketch_loss / dS: on the kept columns K, -(2 / tr G) G E C^-1 with
    Y = G S, C = Y_K^T Y_K, E = G Y_K - Y_K C^-1 (Y_K^T G Y_K); zero elsewhere."""
    G, Y, C, K = _sketch_parts(G, S)
    out = np.zeros((G.shape[0], C.shape[0]))
    if not K.any():
        return out
    YK = Y[:, K]
    CK = C[np.ix_(K, K)]
    P = G @ YK
    X = np.linalg.solve(CK, YK.T @ P)
    E = P - YK @ X
    out[:, K] = -(2.0 / np.trace(G)) * (G @ E) @ np.linalg.inv(CK)
    return out


# ------------------------------------------------------------- HT tensor layer
def ht_layer_chain(x: np.ndarray, u1, u2, u3, b2, b1, bias=None) -> np.ndarray:
    """The reference's HT layer forward, step for step
    (HT_tensor_layer/FC_MNIST/mnist_ht.py:233-241): x (batch, N0*N1*N2) ->
    y (batch, M0*M1*M2), float64."""
    f = lambda a: np.asarray(a, dtype=np.float64)
    u1, u2, u3, b2, b1 = f(u1), f(u2), f(u3), f(b2), f(b1)
    batch = x.shape[0]
    t = f(x).reshape(batch, u1.shape[0], u2.shape[0], u3.shape[0])
    t = np.einsum("zabc,ade->zbcde", t, u1)
    t = np.einsum("zabcd,def->zabcef", t, b2)
    t = np.einsum("zabcde,afd->zbcef", t, u2)
    t = np.einsum("zabcd,ce->zabde", t, b1)
    t = np.einsum("zabcd,aed->zbce", t, u3)
    if bias is not None:
        t = t + f(bias).reshape(t.shape[1:])
    return t.reshape(batch, -1)


def ht_layer_weight(u1, u2, u3, b2, b1) -> np.ndarray:
    """Dense weight W (M0*M1*M2, N0*N1*N2) with chain(x) = x W^T: the chain applied
    to the identity."""
    nin = u1.shape[0] * u2.shape[0] * u3.shape[0]
    return ht_layer_chain(np.eye(nin), u1, u2, u3, b2, b1).T.copy()


def ht_layer_init(weight: np.ndarray, rank: int, N: Sequence[int], M: Sequence[int]):
    """The reference's ``ht(data, rank, N, M)`` (mnist_ht.py:167-197) in float64:
    leaves 3, 4, 2 from the top eigenvectors of the unfolding Grams (descending
    order; the reference takes torch.eig's unsorted first columns), node 1 from
    the SVD of the (a*b) x c unfolding, then the two ncon contractions."""
    a, b, c = N[0] * M[0], N[1] * M[1], N[2] * M[2]
    X, U3m, U4m, U2m, U1m = ht_layer_unfoldings(weight, N, M)
    leaf = lambda A: top_eigvecs(A @ A.T, rank)[1]
    U3, U4, U2 = leaf(U3m), leaf(U4m), leaf(U2m)
    U1 = np.linalg.svd(U1m, full_matrices=False)[0][:, :rank].reshape(a, b, rank)
    B1, B0 = ht_layer_transfers(X, U1, U2, U3, U4)
    return (U3.reshape(N[0], M[0], rank), U4.reshape(N[1], M[1], rank), U2.reshape(N[2], M[2], rank), B1, B0)


def ht_layer_unfoldings(weight: np.ndarray, N: Sequence[int], M: Sequence[int]):
    """The tensor view X (a, b, c) of the weight and its four unfoldings as the
    reference's ``ht()`` forms them (mnist_ht.py:168-177): nodes 3 (a x bc),
    4 (b x ac), 2 (c x ab) and 1 (ab x c), float64."""
    a, b, c = N[0] * M[0], N[1] * M[1], N[2] * M[2]
    X = np.asarray(weight, dtype=np.float64).reshape(a, b, c)
    return X, X.reshape(a, b * c), X.transpose(1, 0, 2).reshape(b, a * c), X.transpose(2, 0, 1).reshape(c, a * b), \
        X.reshape(a * b, c)


def ht_layer_transfers(X: np.ndarray, U1: np.ndarray, U2: np.ndarray, U3: np.ndarray, U4: np.ndarray):
    """The two ncon contractions of ``ht()`` (mnist_ht.py:195-196): B1 (r3, r4, r1)
    from node 1's basis U1 (a, b, r1) and the leaves U3 (a, r3), U4 (b, r4); B0
    (r1, r2) from X, U1 and U2 (c, r2)."""
    B1 = np.einsum("abk,ai,bj->ijk", U1, U3, U4)
    B0 = np.einsum("abc,abi,cj->ij", X, U1, U2)
    return B1, B0

