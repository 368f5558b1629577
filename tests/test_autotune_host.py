"""Host logic of the batched path's autotuner: the table lookup by the
batch's largest dimension (no GPU)."""
from ht_tensor_learning_using_gpu_tensor_cores_gb300 import autotune


def test_lookup_picks_the_bucket_of_the_largest_dimension():
    table = {"precision": "bf16", "buckets": [
        {"lo": 1, "hi": 64, "config": {"lanes": 32, "eig_ctas": 3, "eig_iters": 4, "oversample": 8}},
        {"lo": 65, "hi": 160, "config": {"lanes": 16, "eig_ctas": 6, "eig_iters": 6, "oversample": 16}}]}
    assert autotune.lookup([(40, 50, 60), (20, 64, 33)], table)["lanes"] == 32
    assert autotune.lookup([(40, 50, 60), (20, 65, 33)], table)["eig_ctas"] == 6
    assert autotune.lookup([(400, 50, 60)], table) == autotune.DEFAULT
    assert autotune.lookup([(40, 50, 60)], table, precision="fp32") == autotune.DEFAULT
    assert autotune.lookup([(40, 50, 60)], None if autotune.load_table() else {}) is not None


def test_committed_table_is_well_formed():
    t = autotune.load_table()
    if t is None:
        return
    for b in t["buckets"]:
        assert b["lo"] <= b["hi"]
        assert set(b["config"]) == set(autotune.DEFAULT)
        assert b["tensors_per_s"] >= 0.95 * b["default_tensors_per_s"]
