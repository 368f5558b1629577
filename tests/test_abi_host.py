"""CPU tests of the C ABI boundary and the host-side logic (no GPU needed).

The library must load and export every entry point include/htgb.h declares;
argument validation and workspace sizing run without a device; compute calls
fail loudly (HT_ERR_NO_DEVICE) instead of falling back to the CPU.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht
from ht_tensor_learning_using_gpu_tensor_cores_gb300 import _lib, synth
from ht_tensor_learning_using_gpu_tensor_cores_gb300.tree import DimTree

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "htgb.h")


def _have_lib():
    return os.path.exists(_lib.LIB_PATH)


pytestmark = pytest.mark.skipif(not _have_lib(), reason="libhtgb.so not built (run __graft_entry__.build())")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:ht_status_t|float|void|const char \*|unsigned long long)\s*\*?\s*(\w+)\s*\(", src,
                       flags=re.M)
    return sorted(set(names))


def test_header_declares_expected_entry_points():
    names = declared_functions()
    assert set(names) == set(_lib.EXPORTED), names


def test_library_exports_every_declared_symbol():
    L = ctypes.CDLL(_lib.LIB_PATH)
    for name in declared_functions():
        assert hasattr(L, name), name


def test_reference_trees_match_reference_numbering():
    L = _lib.lib()
    t = _lib.HtTree()
    k = (ctypes.c_int * 5)(1, 10, 11, 12, 13)
    assert L.ht_tree_reference_3d(ctypes.byref(t), k) == 0
    assert t.order == 3 and t.n_nodes == 5
    assert list(t.mode_mask)[:5] == [7, 3, 4, 1, 2]          # root, {1,2}, {3}, {1}, {2}
    assert list(t.left)[:5] == [1, 3, -1, -1, -1]
    assert list(t.right)[:5] == [2, 4, -1, -1, -1]
    assert list(t.parent)[:5] == [-1, 0, 0, 1, 1]
    assert list(t.rank)[:5] == [1, 10, 11, 12, 13]
    t4 = _lib.HtTree()
    k4 = (ctypes.c_int * 7)(1, 2, 3, 4, 5, 6, 7)
    assert L.ht_tree_balanced_4d(ctypes.byref(t4), k4) == 0
    assert list(t4.mode_mask)[:7] == [15, 3, 12, 1, 2, 4, 8]
    # the Python tree builders agree with the C ones
    py = ht._tree_struct(ht.reference_tree_3d([1, 10, 11, 12, 13]))
    for f in ("mode_mask", "left", "right", "parent", "rank"):
        assert list(getattr(py, f))[:5] == list(getattr(t, f))[:5], f


def _validate(tree: DimTree, dims):
    L = _lib.lib()
    ts = ht._tree_struct(tree)
    return L.ht_tree_validate(ctypes.byref(ts), (ctypes.c_long * 4)(*dims), len(dims))


@pytest.mark.parametrize("tree", [ht.reference_tree_3d([1, 4, 4, 4, 4]), ht.left_first_tree_3d([1, 4, 4, 4, 4]),
                                  ht.middle_tree_3d([1, 4, 4, 4, 4])])
def test_validate_accepts_3d_trees(tree):
    assert _validate(tree, (8, 9, 10)) == 0


def test_validate_accepts_4d_balanced():
    assert _validate(ht.balanced_tree_4d([1, 6, 6, 3, 3, 3, 3]), (8, 8, 8, 8)) == 0


@pytest.mark.parametrize("ranks,dims,status", [
    ([1, 4, 4, 4, 4], (8, 8, 0), 1),          # zero dim
    ([1, 4, 4, 9, 4], (8, 8, 8), 1),          # leaf rank above its dimension
    ([1, 20, 4, 4, 4], (8, 8, 8), 1),         # interior rank above k_l * k_r
    ([1, 0, 4, 4, 4], (8, 8, 8), 1),          # zero rank
    ([1, 65, 65, 65, 65], (100, 100, 100), 6),  # ranks above 64 unsupported
])
def test_validate_rejects(ranks, dims, status):
    t = ht.reference_tree_3d([1, 4, 4, 4, 4])
    ts = ht._tree_struct(t)
    for i, r in enumerate(ranks):
        ts.rank[i] = r
    L = _lib.lib()
    assert L.ht_tree_validate(ctypes.byref(ts), (ctypes.c_long * 4)(*dims), 3) == status
    assert len(L.ht_last_error()) > 0


def test_validate_rejects_bad_structure():
    L = _lib.lib()
    ts = ht._tree_struct(ht.reference_tree_3d([1, 4, 4, 4, 4]))
    ts.mode_mask[3] = 3            # leaf holding two modes
    assert L.ht_tree_validate(ctypes.byref(ts), (ctypes.c_long * 4)(8, 8, 8), 3) == 1
    ts = ht._tree_struct(ht.reference_tree_3d([1, 4, 4, 4, 4]))
    ts.parent[3] = 2               # inconsistent parent
    assert L.ht_tree_validate(ctypes.byref(ts), (ctypes.c_long * 4)(8, 8, 8), 3) == 1
    ts = ht._tree_struct(ht.reference_tree_3d([1, 4, 4, 4, 4]))
    assert L.ht_tree_validate(ctypes.byref(ts), (ctypes.c_long * 4)(8, 8, 8, 8), 4) == 1   # order mismatch
    assert L.ht_tree_validate(ctypes.byref(ts), (ctypes.c_long * 4)(8, 8, 8), 5) == 6      # order unsupported


def test_workspace_size_runs_without_gpu():
    tree = ht.reference_tree_3d([1, 32, 32, 32, 32])
    small = ht.workspace_size((64, 64, 64), tree)
    big = ht.workspace_size((1024, 1024, 1024), tree)
    assert 0 < small < big
    # the BF16 copy of a 4 GiB tensor plus the Grams must fit in the plan
    assert big > 1024 ** 3 * 2
    assert big < 16 * 1024 ** 3
    t4 = ht.balanced_tree_4d([1, 48, 48, 24, 24, 24, 24])
    assert ht.workspace_size((128, 128, 128, 128), t4) > 128 ** 4 * 2


def test_compute_fails_loudly_without_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    X = np.zeros((8, 8, 8), dtype=np.float32, order="F")
    with pytest.raises(ht.HTError) as ei:
        ht.decompose(X, ht.reference_tree_3d([1, 2, 2, 2, 2]))
    assert ei.value.status == 7
    with pytest.raises(ht.HTError):
        ht.mode_gram(X, X.shape, 0)
    assert ht.htd.__doc__


def test_config_defaults():
    cfg = _lib.HtConfig()
    assert _lib.lib().ht_config_default(ctypes.byref(cfg)) == 0
    assert cfg.precision == _lib.PREC_BF16 and cfg.oversample == 16 and cfg.eig_iters == 0   # 0: per-precision default
    assert cfg.seed == 1234 and cfg.power_steps == 1
    assert _lib.lib().ht_status_string(5) == b"kernel wait timed out"


# --------------------------------------------------------- host-side logic
def test_dimtree_validation_python():
    with pytest.raises(ValueError):
        DimTree(3, [(0, 1, 2), (1, 0), (2,), (0,), (1,)], [1, 4, 3, -1, -1], [2, 3, 4, -1, -1])
    with pytest.raises(ValueError):
        ht.reference_tree_3d([1, 4, 4, 4, 4]).check_ranks((2, 8, 8))


def test_odeco_generator_spectrum():
    n, k = 24, 6
    X = synth.odeco(n, seed=3).astype(np.float64)
    s = np.linalg.svd(X.reshape(n, n * n, order="F"), compute_uv=False)
    np.testing.assert_allclose(s, np.arange(1, n + 1) ** -1.5, rtol=1e-5, atol=1e-7)
    import ht_oracle as O
    tree = ht.reference_tree_3d([1, k, k, k, k])
    U, B, _ = O.ht_decompose(X, tree)
    assert abs(O.ht_error(X, tree, U, B) - synth.odeco_optimal_error(n, k)) < 1e-6


def test_exact_ht_generator_has_ht_rank():
    tree = ht.left_first_tree_3d([1, 3, 4, 3, 2])
    X = synth.exact_ht((10, 9, 8), tree, noise_rel=0.0, seed=5)
    import ht_oracle as O
    U, B, _ = O.ht_decompose(X, tree)
    assert O.ht_error(X, tree, U, B) < 1e-5


def test_bumps_and_batch_family():
    X = synth.bumps(24, seed=1)
    assert X.shape == (24, 24, 24) and np.isfinite(X).all()
    fam = synth.batch_family(3, seed=2)
    for X, tree in fam:
        tree.check_ranks(X.shape)
        assert 32 <= min(X.shape) and max(X.shape) <= 160


@pytest.mark.parametrize("lang,compiler,flags", [("c", "gcc", ["-std=c99"]), ("c++", "g++", ["-std=c++17"])])
def test_header_compiles_and_links_from_c_and_cpp(tmp_path, lang, compiler, flags):
    """A caller of the reference's entry points, in C or C++, compiles against
    include/htgb.h alone (no CUDA headers) and links against libhtgb.so."""
    import shutil
    import subprocess
    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not installed")
    src = tmp_path / ("caller.c" if lang == "c" else "caller.cpp")
    src.write_text(
        '#include "htgb.h"\n'
        "#include <stdio.h>\n"
        "int main(void) {\n"
        "  ht_config_t cfg; ht_tree_t tree; int k[5] = {1, 4, 4, 4, 4}; long dims[3] = {8, 8, 8};\n"
        "  if (ht_config_default(&cfg) != HT_OK) return 1;\n"
        "  if (ht_tree_reference_3d(&tree, k) != HT_OK) return 2;\n"
        "  if (ht_tree_validate(&tree, dims, 3) != HT_OK) return 3;\n"
        "  float (*f3)(float *, long, long, long, int *) = htd;\n"
        "  void (*f4)(float *, long, long, long, long, int *, void *, void *) = htd4;\n"
        "  printf(\"%s %d\\n\", ht_status_string(HT_OK), f3 != 0 && f4 != 0);\n"
        "  return 0;\n"
        "}\n")
    exe = tmp_path / "caller"
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = [compiler, *flags, "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
           "-L", libdir, "-lhtgb", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, (run.returncode, run.stderr)
    assert run.stdout.split()[-1] == "1"


def test_ctypes_structs_match_the_header(tmp_path):
    """Every ABI struct that the Python layer mirrors has the header's size
    (compiled with gcc against include/htgb.h alone)."""
    import ctypes
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc not installed")
    pairs = [("ht_tree_t", _lib.HtTree), ("ht_config_t", _lib.HtConfig), ("ht_report_t", _lib.HtReport),
             ("ht_batch_report_t", _lib.HtBatchReport), ("ht_layer_shape_t", _lib.HtLayerShape)]
    src = tmp_path / "sizes.c"
    src.write_text('#include "htgb.h"\n#include <stdio.h>\nint main(void) {\n' +
                   "".join(f'  printf("%zu\\n", sizeof({name}));\n' for name, _ in pairs) + "  return 0;\n}\n")
    exe = tmp_path / "sizes"
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60).stdout.split()
    for (name, cls), size in zip(pairs, out):
        assert ctypes.sizeof(cls) == int(size), (name, ctypes.sizeof(cls), size)
