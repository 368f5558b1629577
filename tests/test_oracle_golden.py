"""Pin the CPU oracle to the reference's own outputs.

The fixtures in tests/golden/ were produced by running the reference's Python
statements (HT_TensorLy.py, HT_TensorNetwork.py, HT_4d_TensorNetwork.py) with
tests/golden/make_golden.py.  They are stored in the reference's C-order torch
convention; this file maps them onto the column-major convention used by the
oracle and the engine (C-mode m <-> column-major mode d-1-m).
"""
import glob
import os

import numpy as np
import pytest

import ht_oracle as O
from ht_tensor_learning_using_gpu_tensor_cores_gb300.tree import DimTree

GOLD = os.path.join(os.path.dirname(__file__), "golden")
FIX3 = sorted(glob.glob(os.path.join(GOLD, "ref_*_3d_*.npz")))
FIX4 = sorted(glob.glob(os.path.join(GOLD, "ref_*_4d_*.npz")))


def _load3(path):
    z = np.load(path)
    k = [int(v) for v in z["k"]]
    X = np.asfortranarray(z["X"].transpose(2, 1, 0))
    # reference nodes: 1 = C{0,1}, 2 = C{2}, 3 = C{0}, 4 = C{1}
    # column-major: 1 = (1,2), 2 = (0,), 3 = (1,) [ref 4], 4 = (2,) [ref 3]
    tree = DimTree(3, [(0, 1, 2), (1, 2), (0,), (1,), (2,)], [1, 3, -1, -1, -1], [2, 4, -1, -1, -1],
                   ranks=[1, k[1], k[2], k[4], k[3]])
    U = {1: z["U1"].astype(np.float64), 2: z["U2"].astype(np.float64),
         3: z["U4"].astype(np.float64), 4: z["U3"].astype(np.float64)}
    B = {1: np.asfortranarray(z["B1"].transpose(1, 0, 2).astype(np.float64)),
         0: z["B0"].astype(np.float64).reshape(k[1], k[2], 1)}
    return z, X, tree, U, B


def _load4(path):
    z = np.load(path)
    k = [int(v) for v in z["k"]]
    X = np.asfortranarray(z["X"].transpose(3, 2, 1, 0))
    tree = DimTree(4, [(0, 1, 2, 3), (2, 3), (0, 1), (2,), (3,), (0,), (1,)],
                   [1, 3, 5, -1, -1, -1, -1], [2, 4, 6, -1, -1, -1, -1],
                   ranks=[1, k[1], k[2], k[4], k[3], k[6], k[5]])
    U = {1: z["U1"], 2: z["U2"], 3: z["U4"], 4: z["U3"], 5: z["U6"], 6: z["U5"]}
    U = {t: v.astype(np.float64) for t, v in U.items()}
    B = {1: np.asfortranarray(z["B1"].transpose(1, 0, 2).astype(np.float64)),
         2: np.asfortranarray(z["B2"].transpose(1, 0, 2).astype(np.float64)),
         0: z["B0"].astype(np.float64).reshape(k[1], k[2], 1)}
    return z, X, tree, U, B


def test_fixtures_present():
    assert len(FIX3) >= 4 and len(FIX4) >= 1


@pytest.mark.parametrize("path", FIX3, ids=os.path.basename)
def test_reconstruction_matches_reference_error(path):
    """The reference's factors, pushed through the oracle's reconstruction and
    error, give the error the reference printed (same B layout, same formula)."""
    z, X, tree, U, B = _load3(path)
    err = O.ht_error(X, tree, U, B)
    assert abs(err - float(z["err"])) <= 1e-7 + 1e-4 * float(z["err"])


@pytest.mark.parametrize("path", [p for p in FIX3 if "tensorly" in p], ids=os.path.basename)
def test_oracle_reproduces_reference_decomposition(path):
    """FP32 oracle with the reference's unsorted geev eigen-ordering reproduces
    the reference run: same error to 1e-6 absolute, same subspaces."""
    z, X, tree, Uref, Bref = _load3(path)
    U, B, _ = O.ht_decompose(X, tree, dtype=np.float32, eig_order="geev")
    err = O.ht_error(X, tree, U, B)
    assert abs(err - float(z["err"])) <= 1e-6
    for t in range(1, 5):
        assert O.principal_angles(U[t], Uref[t]).max() < 2e-3
    # transfer tensors agree after aligning the per-node bases
    Ual = {t: Uref[t] for t in Uref}
    Q = {t: O.procrustes_align(U[t], Uref[t]) for t in range(1, 5)}
    B1 = np.einsum("abc,ax,by,cz->xyz", B[1], Q[3], Q[4], Q[1])
    assert np.abs(B1 - Bref[1]).max() < 5e-3 * np.abs(Bref[1]).max()
    del Ual


@pytest.mark.parametrize("path", FIX3, ids=os.path.basename)
def test_fp64_oracle_at_least_as_accurate(path):
    z, X, tree, _, _ = _load3(path)
    U, B, _ = O.ht_decompose(X, tree, dtype=np.float64)
    err = O.ht_error(X, tree, U, B)
    assert err <= float(z["err"]) + 1e-7
    # the inputs are exactly low rank: FP64 recovers them to rounding level of the FP32 input
    assert err < 1e-6


@pytest.mark.parametrize("path", FIX4, ids=os.path.basename)
def test_4d_oracle_vs_reference(path):
    z, X, tree, Uref, Bref = _load4(path)
    err_ref = O.ht_error(X, tree, Uref, Bref)
    U, B, _ = O.ht_decompose(X, tree, dtype=np.float64)
    err = O.ht_error(X, tree, U, B)
    assert err <= err_ref + 1e-7
    assert err < 1e-6
    # FP32 with sorted eigenvectors.  (Unsorted geev ordering is rounding-dependent
    # here: on this input the numpy Gram makes geev list a noise eigenvalue second
    # for one leaf, which is the reference's HT_TensorLy.py:64-66 defect.)
    U32, B32, _ = O.ht_decompose(X, tree, dtype=np.float32, eig_order="desc")
    assert O.ht_error(X, tree, U32, B32) < 10 * err_ref + 1e-5
    for t in (1, 2):   # interior bases come from SVDs of the same matrices
        assert O.principal_angles(U32[t], Uref[t]).max() < 1e-2
