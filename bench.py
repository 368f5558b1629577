"""Benchmark: HT decomposition of a 1024^3 FP32 tensor at rank 32 on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (the headline configuration): a 1024 x 1024 x 1024 FP32 tensor
(4 GiB) whose every matricisation has singular values r^-1.5 (orthonormal
Gaussian factors, seeded), reference dimension tree {1,2,3}->{1,2},{3}, rank 32
at every node.  One step = one full decomposition (leaf bases U_t and transfer
tensors B_t) by the mixed-precision path (BF16 tcgen05 GEMMs, FP32
accumulation) with the tensor resident in HBM.  The tensor (4 GiB) is 32x the
L2, so no flush is needed between steps.

Also measured, outside the headline value: the plain FP32 path (FP32 CUDA-core
GEMMs) on the same GPU, the end-to-end time through the C ABI with the tensor
in pinned host memory (host->device copy inside the timed region), the
relative errors against the FP64 optimum (exact for this family), the
roofline of the dominant kernel (the BF16 Gram), and the CPU baseline: the
numpy restatement of the reference's HT_TensorLy.py on the host cores.

--impl reference: times the reference's CPU implementation of the path (the
numpy port of HT_TensorLy.py; the Python statement itself needs tensorly and
torch.eig, neither available) on this machine's host cores, on the full
1024^3 tensor (one decomposition, a few minutes; the line's `steps` counts the
full-size decompositions timed).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_FULL, RANK, DECAY = 1024, 32, 1.5
CPU_SAMPLE_N = 704   # about 10-15 s of the CPU port on 16 host cores
METRIC = "HT-decomp ms @1024^3 r32, err<=1e-3 vs FP64: mixed/learned vs plain FP32"
# DRAM bytes (read + write) of one leaf-Gram launch at 1024^3, from a one-pass ncu capture:
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum --clock-control none
#       -k 'regex:tc_gemm_kernel|convert_bf16' -c 8 python bench.py --steps 2 --warmup 1 --mixed-only --no-cpu
# (2.149e9 read + ~0 written per Gram launch; X in BF16 is 2.147e9 bytes)
GRAM_DRAM_BYTES_PER_LAUNCH = 2.149e9


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.rows, self.proc, self.dev = [], None, device_index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) >= 9:
                for nm, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ CPU leg
def blas_info():
    """(threads, BLAS library) numpy uses: threadpoolctl when present, else
    numpy's build configuration and the host's core count."""
    try:
        import threadpoolctl
        info = threadpoolctl.threadpool_info()
        threads = max((i.get("num_threads", 1) for i in info), default=os.cpu_count())
        blas = ",".join(sorted({f"{i.get('internal_api', '?')} {i.get('version', '')}".strip() for i in info}))
        return int(threads), blas
    except Exception:
        pass
    try:
        import numpy as np
        b = np.show_config(mode="dicts")["Build Dependencies"]["blas"]
        blas = f"{b.get('name', '?')} {b.get('version', '')}".strip()
    except Exception:
        blas = "unknown"
    threads = int(os.environ.get("OPENBLAS_NUM_THREADS", os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)))
    return threads, blas


def cpu_decompose(n):
    """The reference's CPU path, the numpy port of HT_TensorLy.py (FP32: leaf
    Grams + eigh, SVD of the n^2 x n unfolding for node {1,2}, transfer
    contractions), on an n^3 tensor of the headline family.  Timed region: the
    decomposition, X -> (U_t, B_t), the region the GPU headline times.
    Returns (seconds, rel_err or None); the error pass runs after the timed
    region and only for n <= 704 (the full-size reconstruction would double
    the CPU time)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ht_oracle as O
    from ht_tensor_learning_using_gpu_tensor_cores_gb300 import synth, tree as T
    X = synth.odeco(n, decay=DECAY, seed=1)
    tr = T.reference_tree_3d([1, RANK, RANK, RANK, RANK])
    t0 = time.perf_counter()
    U, B, _ = O.ht_decompose(X, tr, dtype=np.float32)
    t = time.perf_counter() - t0
    err = O.ht_error(X, tr, U, B) if n <= 704 else None
    return t, err


def cpu_baseline(sample_n=CPU_SAMPLE_N):
    """Bounded sample for the GPU line: the CPU path on a sample_n^3 tensor of the
    same family, scaled by (N/sample_n)^4 (the operation count of the Gram GEMMs
    and of the n^2 x n SVD) to the full size.  The reference arm
    (--impl reference) measures the full size instead."""
    t, err = cpu_decompose(sample_n)
    scale = (N_FULL / sample_n) ** 4
    threads, blas = blas_info()
    return {"value": t * scale * 1e3, "unit": "ms", "cores": threads, "kind": "port",
            "sample": f"FP32 decomposition of a {sample_n}^3 tensor of the same family (numpy port of "
                      f"HT_TensorLy.py), {t:.2f} s measured, scaled x{scale:.2f} by the n^4 operation count to "
                      f"{N_FULL}^3 (extrapolated; --impl reference measures {N_FULL}^3)",
            "blas": blas, "sample_seconds": t, "sample_err": err, "extrapolated": True}


def run_reference(args, world, rank):
    """The reference's CPU implementation at the benchmark configuration itself:
    one full 1024^3 rank-32 decomposition (a few minutes of host time), after
    `warmup` untimed runs on a 64^3 sample (imports, BLAS thread pools).  Each
    full-size run is one step; --ref-steps sets how many (default 1, so the
    whole run stays within a few minutes); the line's `steps` is the number
    actually timed."""
    if rank != 0:
        return
    for _ in range(max(0, args.warmup)):
        cpu_decompose(64)
    n = args.ref_n
    secs = []
    for _ in range(max(1, args.ref_steps)):
        t, _ = cpu_decompose(n)
        secs.append(t)
    v = statistics.median(secs) * 1e3
    threads, blas = blas_info()
    cb = {"value": v, "unit": "ms", "cores": threads, "kind": "port",
          "sample": f"{len(secs)} full FP32 decomposition(s) of the {n}^3 rank-{RANK} tensor (numpy port of "
                    f"HT_TensorLy.py), measured, not scaled",
          "blas": blas, "seconds": secs}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "ms", "n_gpus": args.gpus,
            "steps": len(secs), "steps_requested": args.steps, "warmup": args.warmup, "ms_per_step": v,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"HT decomposition {n}^3 rank {RANK}, reference tree, r^-1.5 spectrum",
                       "path": "numpy port of HT_TensorLy.py on host cores",
                       "timed_region": "decomposition X -> (U_t, B_t), as the GPU headline"},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU leg
def secondary_configs(ht, synth, torch, stream, steps=10, warmup=3):
    import numpy as np
    """c1 (256^3, tree {1},{2,3}, ranks 16, exact HT + 1e-3 noise) and c3 (128^4,
    balanced tree, leaf ranks 24, interior 48, exact HT + 1e-4 noise): ms per
    decomposition of the mixed and the plain FP32 paths, device-resident input,
    and the relative error of each (the noise level is the attainable error).
    c4 (512 small tensors): tensors/s through the batched C ABI, wall clock per
    call (graph replay + error readback), and the p50 / p99 relative error."""
    cfgs = [("c1", (256, 256, 256), ht.left_first_tree_3d([1, 16, 16, 16, 16]), 1e-3),
            ("c3", (128, 128, 128, 128), ht.balanced_tree_4d([1, 48, 48, 24, 24, 24, 24]), 1e-4)]
    out = {}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for name, dims, tree, noise in cfgs:
        X = synth.exact_ht_device(dims, tree, noise, seed=21, device="cuda")
        rec = {"dims": list(dims), "ranks": list(tree.ranks), "noise_rel": noise}
        for prec, key in (("bf16", "mixed"), ("fp32", "plain")):
            rec[key + "_rel_err"] = ht.decompose(X, tree, precision=prec, compute_error=True).report["rel_err"]
            for _ in range(warmup):
                ht.decompose(X, tree, precision=prec)
            torch.cuda.synchronize()
            ev0.record(stream)
            for _ in range(steps):
                ht.decompose(X, tree, precision=prec)
            ev1.record(stream)
            torch.cuda.synchronize()
            rec[key + "_ms"] = ev0.elapsed_time(ev1) / steps
        rec["speedup_vs_plain_fp32"] = rec["plain_ms"] / rec["mixed_ms"]
        out[name] = rec
        del X
    # c4: 512 tensors, dims ~ U[32, 160], ranks ~ U[8, 16], exact HT + 1e-3 noise,
    # through the batched C ABI (the recorded CUDA graph replayed on fixed buffers;
    # every stage one launch for the whole batch); tensors/s from the host's wall
    # clock per call (graph launch, error readback), device time beside it
    fam = synth.batch_family(512, seed=31, device="cuda")
    trees = [t for _, t in fam]
    xs = [x for x, _ in fam]
    dims = [tuple(reversed(x.shape)) for x in xs]
    rec = {"tensors": len(xs), "dims": "U[32,160]^3", "ranks": "U[8,16]", "noise_rel": 1e-3,
           "input_bytes": int(sum(x.numel() for x in xs) * 4)}
    from ht_tensor_learning_using_gpu_tensor_cores_gb300 import autotune
    rec["tuned_config"] = autotune.lookup(dims, precision="bf16")
    for prec, key, tuning in (("bf16", "mixed_tuned", "auto"), ("bf16", "mixed", None), ("fp32", "plain", None)):
        bd = ht.BatchDecomposer(trees, dims, precision=prec, compute_error=True, tuning=tuning)
        _, rep = bd(xs)                      # records the graph
        for _ in range(2):
            _, rep = bd(xs)
        torch.cuda.synchronize()
        reps = 5
        t0 = time.perf_counter()
        dev_ms = []
        for _ in range(reps):
            _, rep = bd(xs)
            dev_ms.append(rep["ms_total"])
        wall = (time.perf_counter() - t0) / reps
        rec[key] = {"tensors_per_s": len(xs) / wall, "ms_per_batch": wall * 1e3,
                    "device_ms_per_batch": statistics.median(dev_ms), "rel_err_p50": rep["rel_err_p50"],
                    "rel_err_p99": rep["rel_err_p99"], "graph_replayed": rep["graph_replayed"],
                    "lanes": rep["lanes"], "gpu_launches_per_batch": rep["gpu_launches"],
                    "grouped_stages": rep["grouped"], "device_ms_per_phase": rep["ms_phase"]}
        del bd
    ht.release_batch()
    out["c4"] = rec
    del fam, xs
    torch.cuda.empty_cache()
    out["c5"] = learned_sketch_config(ht, synth, torch, stream)
    torch.cuda.empty_cache()
    out["ht_format"] = ht_format_config(ht, synth, torch, stream)
    torch.cuda.empty_cache()
    out["out_of_core"] = out_of_core_config(ht, synth, torch)
    torch.cuda.empty_cache()
    out["ht_layer"] = ht_layer_config(torch, stream)
    torch.cuda.empty_cache()
    return out


def _event_ms(torch, stream, fn, iters, warmup=3):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(iters):
        fn()
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / iters


def _reference_chain(torch, x, u1, u2, u3, b2, b1, bias):
    """The reference's HT layer forward (HT_tensor_layer/FC_MNIST/mnist_ht.py:233-241),
    PyTorch einsum on the same GPU, FP32 (TF32 off)."""
    batch = x.shape[0]
    t = x.reshape(batch, u1.shape[0], u2.shape[0], u3.shape[0])
    t = torch.einsum("zabc,ade->zbcde", t, u1)
    t = torch.einsum("zabcd,def->zabcef", t, b2)
    t = torch.einsum("zabcde,afd->zbcef", t, u2)
    t = torch.einsum("zabcd,ce->zabde", t, b1)
    t = torch.einsum("zabcd,aed->zbce", t, u3)
    return (t + bias).reshape(batch, -1)


def ht_layer_config(torch, stream):
    """HT tensor layer (the reference's tNet / AlexNet_ht layer): ms per forward and
    per forward+backward through ht_layer_forward / ht_layer_backward (BF16 tcgen05
    and FP32 products), beside the reference's own einsum chain run by PyTorch on
    the same GPU.  Random factors of the reference's shapes; device-resident batch."""
    import numpy as np
    from ht_tensor_learning_using_gpu_tensor_cores_gb300 import htlayer
    out = {}
    allow = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    for name, N, M, r, batches in (("mnist_fc1", (8, 8, 16), (8, 8, 16), 16, (128, 65536)),
                                   ("alexnet_fc6", (16, 16, 25), (16, 16, 16), 16, (256, 8192))):
        g = torch.Generator(device="cuda").manual_seed(0)
        mk = lambda *s: (torch.randn(*s, device="cuda", generator=g) / np.sqrt(s[0] * s[-1])).contiguous()
        f = [mk(N[0], M[0], r), mk(N[1], M[1], r), mk(N[2], M[2], r), mk(r, r, r), mk(r, r)]
        bias = torch.randn(*M, device="cuda")
        for B in batches:
            x = torch.randn(B, int(np.prod(N)), device="cuda")
            rec = {"N": list(N), "M": list(M), "rank": r, "batch": B}
            it = 20 if B <= 1024 else 5
            rec["reference_chain_fwd_ms"] = _event_ms(torch, stream, lambda: _reference_chain(torch, x, *f, bias), it)
            for prec in ("bf16", "fp32"):
                rec[f"{prec}_fwd_ms"] = _event_ms(
                    torch, stream, lambda: htlayer.layer_forward(x, *f, bias=bias, precision=prec), it)
            ps = [t.clone().requires_grad_(True) for t in f]
            bs = bias.clone().requires_grad_(True)

            def ref_step():
                _reference_chain(torch, x, *ps, bs).sum().backward()

            def our_step(prec):
                htlayer.ht_layer(x, *ps, bs, prec).sum().backward()

            rec["reference_chain_fwdbwd_ms"] = _event_ms(torch, stream, ref_step, it)
            for prec in ("bf16", "fp32"):
                rec[f"{prec}_fwdbwd_ms"] = _event_ms(torch, stream, lambda: our_step(prec), it)
            rec["samples_per_s_bf16_fwd"] = B / (rec["bf16_fwd_ms"] * 1e-3)
            rec["speedup_bf16_fwd_vs_reference_chain"] = rec["reference_chain_fwd_ms"] / rec["bf16_fwd_ms"]
            rec["speedup_fp32_fwd_vs_reference_chain"] = rec["reference_chain_fwd_ms"] / rec["fp32_fwd_ms"]
            rec["speedup_bf16_fwdbwd_vs_reference_chain"] = rec["reference_chain_fwdbwd_ms"] / rec["bf16_fwdbwd_ms"]
            out[f"{name}_b{B}"] = rec
            del x, ps, bs
    torch.backends.cuda.matmul.allow_tf32 = allow
    htlayer.release()
    return out


def ht_format_config(ht, synth, torch, stream, n=1024, k=32):
    """HT-format operations on the headline's factors (1024^3, rank 32):
    ht_reconstruct (the full 4 GiB tensor, GB/s of output) and ht_evaluate
    (entries/s for 2^20 random index tuples)."""
    tree = ht.reference_tree_3d([1, k, k, k, k])
    X = synth.exact_ht_device((n, n, n), tree, noise_rel=1e-3, seed=3)
    res = ht.decompose(X, tree, precision="bf16")
    del X
    torch.cuda.empty_cache()
    out = torch.empty((n, n, n), dtype=torch.float32, device="cuda")
    rec_ms = _event_ms(torch, stream, lambda: ht.reconstruct(tree, res.U, res.B, (n, n, n), out=out), 5)
    del out
    cnt = 1 << 20
    idx = torch.randint(0, n, (cnt, 3), device="cuda", dtype=torch.int64)
    ev_ms = _event_ms(torch, stream, lambda: ht.evaluate(tree, res.U, res.B, (n, n, n), idx), 5)
    return {"n": n, "rank": k, "reconstruct_ms": rec_ms,
            "reconstruct_write_GBps": n ** 3 * 4 / (rec_ms * 1e-3) / 1e9,
            "evaluate_entries": cnt, "evaluate_ms": ev_ms, "evaluate_entries_per_s": cnt / (ev_ms * 1e-3)}


def out_of_core_config(ht, synth, torch, n=1024, k=32, slab_gib=1.0):
    """The headline tensor (1024^3, rank 32) decomposed from page-locked host memory
    through ht_decompose_streaming with 1 GiB of device slab buffers (a quarter of
    the tensor): three passes over host X, BF16 products.  Reports ms per
    decomposition (wall clock around the synchronous call), the host bytes
    streamed and the effective host->device rate, and the error against the
    in-core path on the same tensor."""
    tree = ht.reference_tree_3d([1, k, k, k, k])
    Xd = synth.odeco(n, decay=DECAY, seed=1, assemble_on=torch.device("cuda"))
    e_in = ht.decompose(Xd, tree, precision="bf16", compute_error=True).report["rel_err"]
    Xh = Xd.cpu().pin_memory()
    del Xd
    torch.cuda.empty_cache()
    slab = int(slab_gib * (1 << 30))
    r = ht.decompose_streaming(Xh, tree, slab_bytes=slab, precision="bf16", compute_error=True)
    ht.decompose_streaming(Xh, tree, slab_bytes=slab, precision="bf16")
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        rr = ht.decompose_streaming(Xh, tree, slab_bytes=slab, precision="bf16")
    ms = (time.perf_counter() - t0) * 1e3 / reps
    streamed = 3 * n ** 3 * 4
    del Xh
    ht.release_workspace()
    return {"n": n, "rank": k, "slab_buffer_bytes": slab, "passes": 3, "ms": ms,
            "host_bytes_streamed": streamed, "effective_h2d_GBps": streamed / (ms * 1e-3) / 1e9,
            "stage_ms": rr.report["ms_stage"], "rel_err": r.report["rel_err"], "rel_err_in_core": e_in}


def learned_sketch_config(ht, synth, torch, stream, n=512, k=24, p=10, n_train=256, n_test=64, steps=2000):
    """c5: separable-bumps family at n^3, target rank k.  Per-mode sketches of
    width k+p are trained for `steps` Adam steps (batch 32) by the library's
    forward/adjoint kernels on the mode Grams of n_train family members (BF16
    tcgen05 Grams); compared on n_test held-out seeds with the Gaussian start
    block (the training's initial sketch) and the exact Gram path."""
    import numpy as np
    from ht_tensor_learning_using_gpu_tensor_cores_gb300 import learn
    s = k + p
    t0 = time.perf_counter()
    Gtr, ttr = learn.family_grams(range(10000, 10000 + n_train), n, precision="bf16")
    Gte, tte = learn.family_grams(range(20000, 20000 + n_test), n, precision="bf16")
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    t0 = time.perf_counter()
    sketches, hist = learn.train_mode_sketches(Gtr, ttr, s=s, steps=steps, batch=32, lr=2e-3, seed=0)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    gauss = [learn.gaussian_sketch(n, s, seed=17 * m) for m in range(3)]   # the trainers' initial sketches
    learned = [learn.to_bf16(S) for S in sketches]
    rec = {"n": n, "rank": k, "sketch_width": s, "train_grams": 3 * n_train, "heldout_tensors": n_test,
           "steps": steps, "data_s": t_data, "train_s": t_train,
           "train_loss_first_last": {m: [hist[m][0], hist[m][-1]] for m in hist}}
    lg = np.concatenate([learn.heldout_loss(Gte[:, m], tte[:, m], gauss[m]) for m in range(3)])
    ll = np.concatenate([learn.heldout_loss(Gte[:, m], tte[:, m], learned[m]) for m in range(3)])
    rec["heldout_missed_energy"] = {"gaussian_mean": float(lg.mean()), "learned_mean": float(ll.mean()),
                                    "gaussian_p99": float(np.quantile(lg, 0.99)),
                                    "learned_p99": float(np.quantile(ll, 0.99))}
    # below the family's rank the sketch is a choice: width 6, trained on the same
    # Grams, held-out missed energy against the Gaussian start and the best
    # subspace of that width (top-6 eigenvectors of each Gram)
    sn = 6
    narrow, _ = learn.train_mode_sketches(Gtr, ttr, s=sn, steps=400, batch=16, lr=2e-3, seed=1)
    g0 = [learn.gaussian_sketch(n, sn, seed=1 + 17 * m) for m in range(3)]
    lgn = np.concatenate([learn.heldout_loss(Gte[:, m], tte[:, m], g0[m]) for m in range(3)])
    lln = np.concatenate([learn.heldout_loss(Gte[:, m], tte[:, m], narrow[m]) for m in range(3)])
    ev = torch.linalg.eigvalsh(Gte.double()).flip(-1)
    best = (1.0 - ev[..., :sn].sum(-1) / ev.sum(-1)).reshape(-1).cpu().numpy()
    rec["below_rank_width6"] = {"gaussian_missed_energy_mean": float(lgn.mean()),
                                "learned_missed_energy_mean": float(lln.mean()),
                                "best_subspace_missed_energy_mean": float(best.mean()),
                                "gap_closed": float((lgn.mean() - lln.mean()) / max(lgn.mean() - best.mean(), 1e-30))}
    del Gtr, Gte
    tree = ht.reference_tree_3d([1, k, k, k, k])
    variants = (("exact_gram", {}), ("gaussian_1it", {"eig_iters": 1, "oversample": p}),
                ("learned_1it", {"eig_iters": 1, "oversample": p, "sketch": learned}),
                ("gaussian_range_finder", {"leaf_method": "sketch", "oversample": p, "power_steps": 0}),
                ("learned_range_finder", {"leaf_method": "sketch", "oversample": p, "power_steps": 0,
                                          "sketch": learned}))
    errs = {v: [] for v, _ in variants}
    ms = {}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for i, sd in enumerate(range(20000, 20016)):
        X = synth.bumps(n, seed=sd, assemble_on=torch.device("cuda"))
        for v, kw in variants:
            errs[v].append(ht.decompose(X, tree, precision="bf16", compute_error=True, **kw).report["rel_err"])
            if i == 0:
                for _ in range(3):
                    ht.decompose(X, tree, precision="bf16", **kw)
                torch.cuda.synchronize()
                ev0.record(stream)
                for _ in range(10):
                    ht.decompose(X, tree, precision="bf16", **kw)
                ev1.record(stream)
                torch.cuda.synchronize()
                ms[v] = ev0.elapsed_time(ev1) / 10
        del X
    rec["heldout_rel_err_mean"] = {v: float(np.mean(e)) for v, e in errs.items()}
    rec["heldout_rel_err_max"] = {v: float(np.max(e)) for v, e in errs.items()}
    rec["heldout_rel_err_max_minus_exact_gram"] = {v: float(np.max(np.array(e) - np.array(errs["exact_gram"])))
                                                   for v, e in errs.items()}
    rec["variants"] = {"gram_1it": "leaf solver on the mode Gram, one iteration from the start block",
                       "range_finder": "Gram-free range finder (Y = X (X^T S), Nystrom core), no power step"}
    rec["ms_per_decomposition"] = ms
    return rec


def run_ours(args, world, rank, local):
    import numpy as np
    import torch
    import ht_tensor_learning_using_gpu_tensor_cores_gb300 as ht
    from ht_tensor_learning_using_gpu_tensor_cores_gb300 import synth

    torch.cuda.set_device(local)
    if args.fourth_order_only:
        # profiling mode: only the 128^4 mixed-path decomposition (leaf ranks 24,
        # interior 48, exact HT + 1e-4 noise), warm-up + timed steps, no other work
        tree4 = ht.balanced_tree_4d([1, 48, 48, 24, 24, 24, 24])
        X4 = synth.exact_ht_device((128,) * 4, tree4, 1e-4, seed=21, device="cuda")
        for _ in range(args.warmup + args.steps):
            ht.decompose(X4, tree4, precision="bf16")
        torch.cuda.synchronize()
        if rank == 0:
            print(json.dumps({"fourth_order_only": True, "steps": args.steps, "warmup": args.warmup}), flush=True)
        return
    if args.batch_only:
        # profiling mode: only the batched configuration (512 tensors, dims
        # U[32,160]^3, ranks U[8,16]), mixed path, warm-up + timed batches
        fam = synth.batch_family(512, seed=31, device="cuda")
        xs = [x for x, _ in fam]
        bd = ht.BatchDecomposer([t for _, t in fam], [tuple(reversed(x.shape)) for x in xs], precision="bf16",
                                compute_error=True)
        for _ in range(args.warmup + args.steps):
            _, rep = bd(xs)
        torch.cuda.synchronize()
        if rank == 0:
            print(json.dumps({"batch_only": True, "steps": args.steps, "warmup": args.warmup,
                              "device_ms_per_batch": rep["ms_total"]}), flush=True)
        return
    n, k = args.n, RANK
    tree = ht.reference_tree_3d([1, k, k, k, k])
    X = synth.odeco(n, decay=DECAY, seed=1 + rank, assemble_on=torch.device("cuda", local))   # column-major memory
    torch.cuda.synchronize()
    e_opt = synth.odeco_optimal_error(n, k, DECAY)
    stream = torch.cuda.current_stream()

    def one(prec, compute_error=False):
        return ht.decompose(X, tree, precision=prec, compute_error=compute_error)

    if args.mixed_only or args.sketch_only:
        # profiling modes: only the headline step (or the Gram-free range-finder
        # path on the same tensor), warm-up + timed steps, no other work
        kw = {"leaf_method": "sketch", "oversample": 10, "power_steps": 1} if args.sketch_only else {}
        for _ in range(args.warmup + args.steps):
            ht.decompose(X, tree, precision="bf16", **kw)
        torch.cuda.synchronize()
        if rank == 0:
            print(json.dumps({"mixed_only": bool(args.mixed_only), "sketch_only": bool(args.sketch_only),
                              "steps": args.steps, "warmup": args.warmup}), flush=True)
        return

    # correctness of both paths against the FP64 optimum (not timed)
    mixed = one("bf16", compute_error=True)
    plain = one("fp32", compute_error=True)
    err_mixed, err_plain = mixed.report["rel_err"], plain.report["rel_err"]

    # ---- headline: mixed path, device-resident input
    for _ in range(args.warmup):
        one("bf16")
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    l0 = ht.kernel_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stage_ms = []
    ev0.record(stream)
    for _ in range(args.steps):
        r = one("bf16")
        stage_ms.append(r.report["ms_stage"])
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clocks = clk.stop()
    launches = (ht.kernel_launch_count() - l0) / max(1, args.steps)
    ms = ev0.elapsed_time(ev1) / max(1, args.steps)
    ms = allmax(ms, world)

    # ---- plain FP32 path on the same GPU (denominator of the headline ratio)
    one("fp32")
    torch.cuda.synchronize()
    psteps = max(1, min(args.steps, 5))
    ev0.record(stream)
    for _ in range(psteps):
        one("fp32")
    ev1.record(stream)
    torch.cuda.synchronize()
    ms_plain = ev0.elapsed_time(ev1) / psteps

    # ---- end to end through the C ABI with the tensor in pinned host memory
    Xh = torch.empty(X.shape, dtype=torch.float32, pin_memory=True)
    Xh.copy_(X)
    Xh_np = Xh.numpy()   # shares the pinned buffer; memory is the column-major tensor
    dims = (n, n, n)
    flat = Xh_np.reshape(-1)
    ht.decompose(flat, tree, dims=dims, precision="bf16")   # warm: workspace sized for host input
    torch.cuda.synchronize()
    e2e_steps = max(1, min(args.steps, 5))
    e2e_h2d_ms, e2e_step_ms = [], []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()   # each call returns with U, B on the host: the step is synchronous
        res_h = ht.decompose(flat, tree, dims=dims, precision="bf16")
        e2e_step_ms.append((time.perf_counter() - t0) * 1e3)
        e2e_h2d_ms.append(res_h.report["ms_stage"]["h2d"])
    e2e_mean_ms = allmax(statistics.fmean(e2e_step_ms), world)
    e2e_ms = allmax(statistics.median(e2e_step_ms), world)
    d2h = sum(int(np.asarray(a).nbytes) for a in list(res_h.U.values()) + list(res_h.B.values()))
    h2d = n * n * n * 4

    # ---- Gram-free leaf range finder (HT_LEAF_SKETCH) on the same tensor: the
    # configuration's oversampling 10 and one power step, BF16 products
    sk_kw = {"leaf_method": "sketch", "oversample": 10, "power_steps": 1}
    sk_res = ht.decompose(X, tree, precision="bf16", compute_error=True, **sk_kw)
    for _ in range(max(3, args.warmup)):
        ht.decompose(X, tree, precision="bf16", **sk_kw)
    torch.cuda.synchronize()
    sk_steps = max(1, min(args.steps, 10))
    sk_stage = []
    ev0.record(stream)
    for _ in range(sk_steps):
        sk_stage.append(ht.decompose(X, tree, precision="bf16", **sk_kw).report["ms_stage"])
    ev1.record(stream)
    torch.cuda.synchronize()
    ms_sketch = ev0.elapsed_time(ev1) / sk_steps

    # ---- leaf principal angles against the exact subspaces (the family's
    # leading factor columns, closed form), per path
    A_true, _ = synth.odeco_factors(n, 3, DECAY, seed=1 + rank)

    def max_angles(res):
        out = {}
        for t in tree.leaves():
            m = tree.modes[t][0]
            At = torch.as_tensor(A_true[m][:, :k], dtype=torch.float64, device=X.device)
            sv = torch.linalg.svdvals(At.T @ res.U[t].double())
            out[f"mode{m}"] = float(torch.arccos(sv.clamp(max=1.0)).max())
        return out

    angles = {"mixed": max_angles(mixed), "plain_fp32": max_angles(plain), "sketch": max_angles(sk_res)}

    # ---- the other single-tensor configurations (not the headline): c1 and c3
    others = secondary_configs(ht, synth, torch, stream) if rank == 0 else None

    # ---- roofline of the dominant kernel: the BF16 Gram (3 launches per step)
    pk = peaks()
    grams_ms = statistics.median([s["grams"] for s in stage_ms]) / 3.0   # per launch (+ its reduction)
    gram_flops = float(n) ** 2 * float(n) ** 2               # SYRK of one mode: n^2 K, K = n^2
    achieved = gram_flops / (grams_ms * 1e-3) / 1e12
    tiles = -(-n // 256)
    issued = tiles * (tiles + 1) / 2 * 256.0 * 256.0 * 2.0 * float(n) ** 2   # per launch
    stage_med = {kk: statistics.median([s[kk] for s in stage_ms]) for kk in stage_ms[0]}
    cpu = cpu_baseline(args.cpu_sample) if (rank == 0 and not args.no_cpu) else None

    if rank == 0:
        line = {
            "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
            "data": "synthetic",
            "config": {"workload": f"HT decomposition {n}^3 FP32 rank {k}, reference tree {{1,2,3}}->{{1,2}},{{3}}, "
                                   f"r^-{DECAY} spectrum on every matricisation",
                       "n": n, "rank": k, "path": "mixed: BF16 tcgen05 Gram/TTM, FP32 accumulation",
                       "l2_policy": "inputs larger than L2 (4 GiB vs 129 MB), no flush",
                       "parallelism": f"replicas x{world}"},
            "plain_fp32_ms": ms_plain, "speedup_vs_plain_fp32": ms_plain / ms,
            "rel_err": {"mixed": err_mixed, "plain_fp32": err_plain, "fp64_optimum": e_opt,
                        "mixed_minus_fp64": err_mixed - e_opt, "plain_minus_fp64": err_plain - e_opt},
            "stage_ms": stage_med,
            "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "h2d_ms": statistics.median(e2e_h2d_ms),
                    "host_link_GBps": h2d / (statistics.median(e2e_h2d_ms) * 1e-3) / 1e9,
                    "mean_ms": e2e_mean_ms, "steps": e2e_steps, "statistic": "median of per-step wall times",
                    "note": "the copy runs in slabs on a side stream; conversion and the mode-1/2 Gram shares overlap it"},
            "roofline": {"bound": "tensor", "kernel": "tc_gemm_kernel<256,2> (leaf Grams: 3 launches + their "
                                                      "reductions, per launch)",
                         "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                         "frac": achieved / pk["bf16_tflops"],
                         "traffic": GRAM_DRAM_BYTES_PER_LAUNCH if n == N_FULL else None,
                         "traffic_unit": "bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)",
                         "algorithmic_bytes_per_launch": 2 * float(n) ** 3,
                         "flop_per_launch": float(n) ** 4,
                         "issued_flop_per_launch": issued,
                         "issued_frac": issued / (grams_ms * 1e-3) / 1e12 / pk["bf16_tflops"],
                         "issued_note": "tcgen05 work actually issued: the upper triangle of 256 x 256 tiles, "
                                        "diagonal tiles in full",
                         "peak_source": pk["source"] + " bf16 burst"},
            "leaf_principal_angles_rad": angles,
            "sketch_path": {
                "what": "leaf bases from the Gram-free range finder (block width k+10, one power step, Nystrom "
                        "core), interior node from the Householder TSQR of X_(12) V; BF16 products",
                "ms": ms_sketch, "rel_err": sk_res.report["rel_err"],
                "rel_err_minus_fp64": sk_res.report["rel_err"] - e_opt,
                "speedup_vs_plain_fp32": ms_plain / ms_sketch,
                "stage_ms": {kk: statistics.median([s_[kk] for s_ in sk_stage]) for kk in sk_stage[0]},
                "streaming_products": 12,
                "products_GBps": 12 * 2.0 * float(n) ** 3 / (statistics.median([s_["grams"] for s_ in sk_stage])
                                                              * 1e-3) / 1e9,
                "products_GBps_note": "12 passes over BF16 X (2 applications of X X^T per mode, 2 products each) "
                                      "over the whole range-finder stage, CholeskyQR and Nystrom included",
                "hbm_peak_GBps": pk["hbm_gbs"]},
            "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": launches,
            "other_configs": others,
        }
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=N_FULL)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=CPU_SAMPLE_N,
                    help="edge of the cubic sample the GPU line's CPU baseline decomposes (scaled by n^4 to 1024^3)")
    ap.add_argument("--ref-n", type=int, default=N_FULL, help="--impl reference: edge of the decomposed tensor")
    ap.add_argument("--ref-steps", type=int, default=1, help="--impl reference: full-size decompositions timed")
    ap.add_argument("--mixed-only", action="store_true",
                    help="run only the headline mixed-path steps (for profiler launch lists)")
    ap.add_argument("--batch-only", action="store_true",
                    help="run only the batched 512-tensor configuration (for profiler launch lists)")
    ap.add_argument("--sketch-only", action="store_true",
                    help="run only the Gram-free range-finder path on the headline tensor (for profiler launch lists)")
    ap.add_argument("--fourth-order-only", action="store_true",
                    help="run only the 128^4 mixed-path steps (for profiler launch lists)")
    args = ap.parse_args()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
