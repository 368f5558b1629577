"""HT-format operations on the GPU: full reconstruction (ht_reconstruct) and
entry evaluation (ht_evaluate), checked against the oracle's reconstruction
(htd_batch.cu:196-224 restated) and its leaf-to-root entry contraction, and
pinned on the reference's own factors from tests/golden/.

Tolerances (FP32 arithmetic throughout):
  reconstruction   ||Xhat_gpu - Xhat_oracle||_F / ||Xhat_oracle||_F <= 1e-5
  entries          max |x_gpu - x_oracle| <= 1e-5 * max |Xhat_oracle|
  reference error  |err(X, Xhat_gpu) - err_reference| <= 1e-6 + 1e-4 err_reference
"""
import glob
import os

import numpy as np
import pytest
import torch

import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht
from ht_tensor_learning_using_gpu_tensor_cores_gb300 import htformat, synth
from ht_tensor_learning_using_gpu_tensor_cores_gb300._lib import HTError
from ht_tensor_learning_using_gpu_tensor_cores_gb300.tree import DimTree
import ht_oracle as O

pytestmark = pytest.mark.gpu

REC_TOL = 1e-5
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def random_factors(tree, dims, seed):
    rng = np.random.default_rng(seed)
    U = {t: np.asfortranarray(rng.standard_normal((dims[tree.modes[t][0]], tree.ranks[t])).astype(np.float32))
         for t in tree.leaves()}
    B = {}
    for t in [0] + tree.interior():
        kl, kr = tree.ranks[tree.left[t]], tree.ranks[tree.right[t]]
        B[t] = np.asfortranarray(rng.standard_normal((kl, kr, tree.ranks[t])).astype(np.float32))
    return U, B


def to_torch_factors(U, B):
    Ut = {t: torch.from_numpy(np.ascontiguousarray(a.T)).cuda().t() for t, a in U.items()}
    Bt = {t: torch.from_numpy(np.ascontiguousarray(a.transpose(2, 1, 0))).cuda().permute(2, 1, 0)
          for t, a in B.items()}
    return Ut, Bt


def gpu_tensor_to_numpy(x, dims):
    """A torch tensor shaped dims[::-1] (the column-major tensor) as a Fortran numpy array."""
    return np.asfortranarray(x.cpu().numpy().transpose(tuple(range(len(dims)))[::-1]))


CASES = [
    (ht.reference_tree_3d, (40, 24, 56), [1, 12, 6, 5, 7]),          # root -> {1,2},{3}: X_(01) = W U_2^T
    (ht.left_first_tree_3d, (33, 48, 20), [1, 9, 11, 6, 8]),         # root -> {1},{2,3}: X_(0) = U_0 W^T
    (ht.middle_tree_3d, (21, 35, 64), [1, 13, 17, 9, 8]),            # root -> {2},{1,3}: slab-batched
    (ht.reference_tree_3d, (129, 1, 67), [1, 3, 1, 3, 1]),           # a mode of size one
    (ht.balanced_tree_4d, (12, 10, 14, 9), [1, 7, 6, 4, 5, 3, 6]),
    (ht.reference_tree_3d, (300, 260, 200), [1, 64, 48, 32, 40]),     # ranks at the 64 limit, several tiles
]


@pytest.mark.parametrize("mk,dims,k", CASES)
@pytest.mark.parametrize("where", ["device", "host"])
def test_reconstruct_matches_oracle(mk, dims, k, where):
    tree = mk(k)
    U, B = random_factors(tree, dims, seed=sum(dims) + len(k))
    ref = O.ht_reconstruct(tree, dims, {t: a.astype(np.float64) for t, a in U.items()},
                           {t: a.astype(np.float64) for t, a in B.items()})
    if where == "device":
        Ut, Bt = to_torch_factors(U, B)
        X = gpu_tensor_to_numpy(ht.reconstruct(tree, Ut, Bt, dims), dims)
    else:
        X = ht.reconstruct(tree, U, B, dims)
        assert isinstance(X, np.ndarray) and X.flags.f_contiguous and X.shape == dims
    assert rel(X, ref) <= REC_TOL, rel(X, ref)


@pytest.mark.parametrize("mk,dims,k", CASES)
def test_evaluate_matches_oracle(mk, dims, k):
    tree = mk(k)
    U, B = random_factors(tree, dims, seed=7 * sum(dims))
    rng = np.random.default_rng(3)
    idx = np.stack([rng.integers(0, d, size=3001) for d in dims], axis=1)
    idx[0] = 0
    idx[1] = [d - 1 for d in dims]
    Uo = {t: a.astype(np.float64) for t, a in U.items()}
    Bo = {t: a.astype(np.float64) for t, a in B.items()}
    want = O.ht_entries(tree, Uo, Bo, idx)
    full = O.ht_reconstruct(tree, dims, Uo, Bo)
    assert np.allclose(want, full[tuple(idx.T)], rtol=1e-10, atol=1e-10 * np.abs(full).max())
    scale = np.abs(full).max()
    got_host = ht.evaluate(tree, U, B, dims, idx)
    assert np.abs(got_host - want).max() <= 1e-5 * scale
    Ut, Bt = to_torch_factors(U, B)
    got_dev = ht.evaluate(tree, Ut, Bt, dims, torch.from_numpy(idx).cuda())
    assert got_dev.is_cuda
    assert np.abs(got_dev.cpu().numpy() - want).max() <= 1e-5 * scale


def test_evaluate_edge_cases():
    tree = ht.balanced_tree_4d([1, 3, 2, 2, 2, 2, 1])
    dims = (5, 4, 3, 2)
    U, B = random_factors(tree, dims, seed=11)
    assert ht.evaluate(tree, U, B, dims, np.zeros((0, 4), np.int64)).shape == (0,)
    bad = np.array([[0, 0, 0, 0], [0, 4, 0, 0]], np.int64)       # mode 2 has size 4
    with pytest.raises(HTError, match="outside"):
        ht.evaluate(tree, U, B, dims, bad)
    with pytest.raises(HTError, match="outside"):
        ht.evaluate(tree, U, B, dims, torch.tensor([[-1, 0, 0, 0]], device="cuda"))
    # the context stays usable after a rejected call
    good = ht.evaluate(tree, U, B, dims, np.array([[4, 3, 2, 1]], np.int64))
    want = O.ht_entries(tree, U, B, np.array([[4, 3, 2, 1]]))
    assert abs(float(good[0]) - float(want[0])) <= 1e-5 * max(abs(float(want[0])), 1.0)


def test_reconstruct_rejects_missing_factor():
    tree = ht.reference_tree_3d([1, 2, 2, 2, 2])
    dims = (4, 4, 4)
    U, B = random_factors(tree, dims, seed=1)
    del B[1]
    with pytest.raises(HTError, match="missing factor"):
        ht.reconstruct(tree, U, B, dims)


# ------------------------------------------------- pinned on the reference's factors
def _golden3(path):
    """Reference factors of a 3rd-order fixture in the column-major convention:
    node 1 = modes (1,2) [ref B1], 2 = (0,) [ref U2], 3 = (1,) [ref U4], 4 = (2,) [ref U3]."""
    z = np.load(path)
    k = [int(v) for v in z["k"]]
    X = np.asfortranarray(z["X"].transpose(2, 1, 0))
    tree = DimTree(3, [(0, 1, 2), (1, 2), (0,), (1,), (2,)], [1, 3, -1, -1, -1], [2, 4, -1, -1, -1],
                   ranks=[1, k[1], k[2], k[4], k[3]])
    f = lambda a: np.asfortranarray(a, dtype=np.float32)
    U = {2: f(z["U2"]), 3: f(z["U4"]), 4: f(z["U3"])}
    B = {1: f(z["B1"].transpose(1, 0, 2)), 0: f(z["B0"].reshape(k[1], k[2], 1))}
    return z, X, tree, U, B


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLD, "ref_*_3d_*.npz"))), ids=os.path.basename)
def test_reconstruct_reference_factors(path):
    """The reference's own factors (leaf bases, B1, B0) through ht_reconstruct
    reproduce the error the reference printed for them."""
    z, X, tree, U, B = _golden3(path)
    Xh = ht.reconstruct(tree, U, B, X.shape)
    err = O.rel_error(X, Xh)
    assert abs(err - float(z["err"])) <= 1e-6 + 1e-4 * float(z["err"]), (err, float(z["err"]))


def test_reconstruct_reference_factors_4d():
    """The 4th-order fixture's tree puts modes {3,4} left of the root; the engine
    wants {1,2} left, so the root's children swap and B0 transposes."""
    path = os.path.join(GOLD, "ref_tensornetwork_4d_n20_s6.npz")
    z = np.load(path)
    k = [int(v) for v in z["k"]]
    X = np.asfortranarray(z["X"].transpose(3, 2, 1, 0))
    # column-major fixture tree: 1 = (2,3) with leaves 3 = (2,) [ref U4], 4 = (3,) [ref U3];
    # 2 = (0,1) with leaves 5 = (0,) [ref U6], 6 = (1,) [ref U5]
    tree = ht.balanced_tree_4d([1, k[2], k[1], k[6], k[5], k[4], k[3]])
    f = lambda a: np.asfortranarray(a, dtype=np.float32)
    U = {3: f(z["U6"]), 4: f(z["U5"]), 5: f(z["U4"]), 6: f(z["U3"])}
    B = {1: f(z["B2"].transpose(1, 0, 2)), 2: f(z["B1"].transpose(1, 0, 2)),
         0: f(z["B0"].T.reshape(k[2], k[1], 1))}
    Xh = ht.reconstruct(tree, U, B, X.shape)
    ref = O.ht_reconstruct(tree, X.shape, {t: a.astype(np.float64) for t, a in U.items()},
                           {t: a.astype(np.float64) for t, a in B.items()})
    assert rel(Xh, ref) <= REC_TOL
    assert O.rel_error(X, Xh) < 1e-4      # the fixture's tensor is exactly of these ranks


# ------------------------------------------------- decompose -> save -> load -> use
@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_roundtrip_through_file(tmp_path, prec):
    dims = (96, 80, 112)
    tree = ht.reference_tree_3d([1, 10, 8, 6, 7])
    X = synth.exact_ht(dims, tree, noise_rel=1e-3, seed=5)
    Xd = torch.from_numpy(np.ascontiguousarray(X.transpose(2, 1, 0))).cuda()
    res = ht.decompose(Xd, tree, precision=prec, compute_error=True)
    path = str(tmp_path / "x.npz")
    htformat.save(path, res.tree, res.dims, res.U, res.B)
    h = htformat.load(path)
    assert h.dims == dims and h.tree.ranks == tree.ranks
    assert h.compression() > 100
    Xh = ht.reconstruct(h.tree, h.U, h.B, h.dims)
    err = O.rel_error(X, Xh)
    assert abs(err - res.report["rel_err"]) <= 1e-5 + 1e-4 * err
    assert abs(ht.reconstruct_error(X, h.tree, h.U, h.B) - err) <= 1e-5 + 1e-4 * err
    idx = np.array([[0, 0, 0], [95, 79, 111], [17, 3, 64]], np.int64)
    assert np.allclose(ht.evaluate(h.tree, h.U, h.B, h.dims, idx), Xh[tuple(idx.T)], rtol=1e-5,
                       atol=1e-5 * np.abs(Xh).max())


def test_reconstruct_full_size_matches_error_pass():
    """1024^3, ranks 32, mixed precision: Xhat from ht_reconstruct gives the same
    relative error as the fused error pass (a size-independent check)."""
    n, r = 1024, 32
    tree = ht.reference_tree_3d([1, r, r, r, r])
    X = synth.exact_ht_device((n, n, n), tree, noise_rel=1e-3, seed=9)
    res = ht.decompose(X, tree, precision="bf16", compute_error=True)
    Xh = ht.reconstruct(tree, res.U, res.B, (n, n, n))
    num = den = 0.0
    for s in range(0, n, 128):       # slabs of the slowest mode, accumulated in FP64
        d = (X[s:s + 128] - Xh[s:s + 128]).double()
        num += float(torch.sum(d * d))
        den += float(torch.sum(X[s:s + 128].double() ** 2))
    del Xh
    err = (num / den) ** 0.5
    assert abs(err - res.report["rel_err"]) <= 1e-6 + 1e-4 * err, (err, res.report["rel_err"])
