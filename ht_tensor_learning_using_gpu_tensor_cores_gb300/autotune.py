"""Autotuner of the batched path (``ht_decompose_batched``), per size bucket.

Batches whose modes are all at most ``GROUPED_MAX_DIM`` run as grouped stages
(one launch per stage for every tensor); what moves them is how many subspace
iterations and how much oversampling the leaf solver needs before the error
stops moving.  Larger tensors run as per-tensor chains spread over concurrent
streams ("lanes"), where the number of lanes and the CTAs each lane's
cooperative eigen-solver takes matter as well.  ``tune_batched`` times
every candidate on a sample batch of a size bucket, keeps the candidates whose
p99 and maximum relative errors stay within a relative slack of the default
configuration's, and returns the fastest.  ``tune_table`` does this for a list
of buckets and writes the table (JSON) that ``BatchDecomposer(tuning="auto")``
reads: the batch's largest dimension picks the bucket.

The reference has no batched path (its size sweeps call htd() once per tensor,
``third_order_tensor_decompsition/CUDA/Optimized/ht_init.cu:9-47``).
"""
from __future__ import annotations

import itertools
import json
import os
import time
from typing import Dict, List, Optional, Sequence, Tuple

from ._lib import check, lib

TABLE_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning", "batched_gb300.json")
DEFAULT = {"lanes": 16, "eig_ctas": 0, "eig_iters": 10, "oversample": 16}
CANDIDATES = {"lanes": (8, 16, 32), "eig_ctas": (0, 3, 6), "eig_iters": (10, 6, 4), "oversample": (16, 8)}
# the library groups the stages of a batch whose modes are all at most this
GROUPED_MAX_DIM = 512
CANDIDATES_GROUPED = {"lanes": (16,), "eig_ctas": (0,), "eig_iters": (10, 6, 4), "oversample": (16, 8)}


def set_launch_shape(lanes: int, eig_ctas: int) -> None:
    """Lanes and eigen-solver CTA cap of later batched calls on the current device."""
    check(lib().ht_batch_set_tuning(int(lanes), int(eig_ctas)))


def _time_config(trees, dims, tensors, cfg: Dict, precision: str, repeats: int) -> Tuple[float, Dict]:
    import torch
    from . import BatchDecomposer, release_batch
    set_launch_shape(cfg["lanes"], cfg["eig_ctas"])
    bd = BatchDecomposer(trees, dims, precision=precision, compute_error=True, eig_iters=cfg["eig_iters"],
                         oversample=cfg["oversample"])
    for _ in range(2):                      # records and replays the graph
        bd(tensors)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(repeats):
        _, rep = bd(tensors)
    wall = (time.perf_counter() - t0) / repeats
    del bd
    release_batch()
    return wall, rep


def tune_batched(trees: Sequence, dims: Sequence[Sequence[int]], tensors: Sequence, precision: str = "bf16",
                 candidates: Optional[Dict] = None, err_slack: float = 1e-3, repeats: int = 3) -> Dict:
    """The fastest candidate configuration for one batch whose p99 and maximum
    relative errors exceed the default configuration's by at most a factor
    (1 + err_slack).  Returns the choice, its tensors/s and errors, and the
    default's."""
    grouped = max(max(int(v) for v in d) for d in dims) <= GROUPED_MAX_DIM
    cand = candidates or (CANDIDATES_GROUPED if grouped else CANDIDATES)
    base_wall, base = _time_config(trees, dims, tensors, DEFAULT, precision, repeats)
    best, best_wall, best_rep = dict(DEFAULT), base_wall, base
    tried = []
    keys = ("lanes", "eig_ctas", "eig_iters", "oversample")
    for values in itertools.product(*(cand[k] for k in keys)):
        cfg = dict(zip(keys, values))
        if cfg == DEFAULT:
            continue
        wall, rep = _time_config(trees, dims, tensors, cfg, precision, repeats)
        ok = (rep["rel_err_p99"] <= base["rel_err_p99"] * (1 + err_slack) and
              rep["rel_err_max"] <= base["rel_err_max"] * (1 + err_slack))
        tried.append({**cfg, "tensors_per_s": len(tensors) / wall, "rel_err_p99": rep["rel_err_p99"], "ok": ok})
        if ok and wall < best_wall:
            best, best_wall, best_rep = cfg, wall, rep
    set_launch_shape(DEFAULT["lanes"], DEFAULT["eig_ctas"])
    return {"config": best, "tensors_per_s": len(tensors) / best_wall,
            "rel_err_p50": best_rep["rel_err_p50"], "rel_err_p99": best_rep["rel_err_p99"],
            "default_tensors_per_s": len(tensors) / base_wall, "default_rel_err_p99": base["rel_err_p99"],
            "candidates_tried": len(tried) + 1, "precision": precision}


def tune_table(buckets: Sequence[Tuple[int, int]], count: int = 256, rank_range=(8, 16), precision: str = "bf16",
               seed: int = 0, path: Optional[str] = TABLE_PATH, candidates: Optional[Dict] = None) -> Dict:
    """Tune each size bucket (lo, hi) on a seeded family of `count` exact-HT
    tensors with every dimension drawn from [lo, hi] (synth.batch_family) and
    write the table to `path` (None: do not write)."""
    from . import synth
    table = {"device": _device_name(), "precision": precision, "buckets": []}
    for i, (lo, hi) in enumerate(buckets):
        fam = synth.batch_family(count, seed=seed + i, dim_range=(lo, hi), rank_range=rank_range, device="cuda")
        tensors = [x for x, _ in fam]
        trees = [t for _, t in fam]
        dims = [tuple(reversed(x.shape)) for x in tensors]
        res = tune_batched(trees, dims, tensors, precision=precision, candidates=candidates)
        table["buckets"].append({"lo": lo, "hi": hi, "tensors": count, **res})
        del fam, tensors
    if path:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as f:
            json.dump(table, f, indent=1)
    return table


def _device_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name()
    except Exception:
        return "unknown"


def load_table(path: str = TABLE_PATH) -> Optional[Dict]:
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


def lookup(dims: Sequence[Sequence[int]], table: Optional[Dict] = None, precision: str = "bf16") -> Dict:
    """The tuned configuration for a batch: the bucket that holds its largest
    dimension (the default configuration when no table or bucket matches)."""
    table = load_table() if table is None else table
    if not table or table.get("precision") != precision:
        return dict(DEFAULT)
    biggest = max(max(int(v) for v in d) for d in dims)
    for b in table["buckets"]:
        if b["lo"] <= biggest <= b["hi"]:
            return dict(b["config"])
    return dict(DEFAULT)


__all__ = ["tune_batched", "tune_table", "load_table", "lookup", "set_launch_shape", "DEFAULT", "CANDIDATES",
           "CANDIDATES_GROUPED", "GROUPED_MAX_DIM", "TABLE_PATH"]
