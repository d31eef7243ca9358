#!/usr/bin/env python
"""Headline benchmark: apply throughput (Mpts/s) of the strong-recursive-
skeletonization FMM, 3D Laplace, N = 1,000,000 points uniform in [0,1]^3
(numpy default_rng(0)), charges RandomState(1).randn, tol 1e-6, leaf 400 —
plus the build time and the plain-FP64 apply beside the mixed one.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one apply of the built operator to one charge vector.  ``value`` is
device-resident throughput (inputs in HBM, CUDA events on the launch stream);
``e2e`` is the same metric through the C ABI with pinned host buffers
(host->device copy of x and device->host copy of y inside the timed region).
Multi-GPU runs are independent replicas (one instance per rank, no
collective on the data path); ``value`` sums all ranks.
``--impl reference`` times the reference algorithm's CPU implementation (the
oracle port of skelfmm's batched apply) on the host cores.
"""

from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

WORKLOAD = "laplace_3d uniform cube N=1e6 tol=1e-6 leaf=400"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=1_000_000)
    p.add_argument("--tol", type=float, default=1e-6)
    p.add_argument("--leaf", type=int, default=400)
    p.add_argument("--fp64-steps", type=int, default=2)
    p.add_argument("--ncheck", type=int, default=2000)
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def workload(n, seed=0):
    pts = np.random.default_rng(seed).random((n, 3))
    x = np.random.RandomState(1).randn(n)
    return pts, x


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([s.strip() for s in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        smax = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(np.max(smax)) if smax else None,
                "reasons": reasons, "samples": len(self.samples)}


def measured_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def profiled_traffic(name):
    """Per-launch DRAM bytes of a kernel from a committed ncu summary, or None."""
    path = os.path.join(HERE, "profiles", name)
    try:
        text = open(path).read()
    except OSError:
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", text)
    return float(m.group(1)) if m else None


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        return dist, rank, ws
    return None, 0, 1


def cpu_baseline_sample(f, x, budget_s=15.0):
    """Reference algorithm (oracle port: FP64 dense kernel blocks) on the host
    cores, over a sample of target boxes of the same build; throughput scaled
    by pair evaluations (plus the measured upward/downward passes)."""
    from oracle import skel_oracle as O

    rb = f.plan.rb
    nb = rb.nboxes
    rng = np.random.default_rng(0)
    order = rng.permutation(nb)
    work = np.array([(rb.box_off[b + 1] - rb.box_off[b]) *
                     sum(rb.box_off[s + 1] - rb.box_off[s] for s in rb.list_src[rb.list_off[b]:rb.list_off[b + 1]])
                     for b in range(nb)], dtype=np.float64)
    total = float(work.sum())
    q = np.zeros(rb.nentries)
    q[rb.perm_entry] = x[rb.perm_point]
    qh = q.copy()
    nthreads = os.cpu_count() or 1
    done_pairs, secs, i = 0, 0.0, 0
    while secs < budget_s and i < nb:
        chunk = [b for b in order[i:i + 4 * nthreads] if work[b] > 0]
        i += 4 * nthreads
        t0 = time.perf_counter()
        res = O.translation_sample("laplace_3d", 0.0, rb.entry_xyz, None, rb.box_off, rb.box_rank,
                                   rb.list_off, rb.list_src, rb.list_kind, q, qh, chunk, nthreads)
        secs += time.perf_counter() - t0
        done_pairs += sum(r[2] for r in res)
    rate = done_pairs / secs
    t_apply = total / rate
    return {"value": rb.npoints / t_apply / 1e6, "unit": "Mpts/s", "cores": nthreads, "kind": "port",
            "sample": f"{done_pairs:.3g} of {total:.3g} kernel evaluations ({100 * done_pairs / total:.2f}%) "
                      f"in {secs:.1f} s, FP64 numpy dense blocks, {nthreads} threads; apply time scaled by "
                      f"evaluation count"}


def run_ours(args):
    import torch

    from skelfmm_gb300 import _lib, operators
    from skelfmm_gb300.skel_fmm import SkelFMM

    dist, rank, ws = dist_setup()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    pts, x = workload(args.n, seed=rank)
    n = args.n

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    # first use of the library/CUDA context outside the timed build
    SkelFMM(pts[:2000], operators.LAPLACE_3D, tol=args.tol, leaf_size=args.leaf, precision="mixed")
    barrier()
    t0 = time.perf_counter()
    f = SkelFMM(pts, operators.LAPLACE_3D, tol=args.tol, leaf_size=args.leaf, precision="mixed")
    torch.cuda.synchronize(dev)
    build_s = time.perf_counter() - t0
    plan = f.plan
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    xt = torch.from_numpy(x).to(dev)
    yt = torch.empty_like(xt)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > L2 (126 MB)

    def timed(prec, steps, warmup):
        for _ in range(warmup):
            plan.apply_device(xt, yt, prec, sp)
        barrier()
        evs = []
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.apply_device(xt, yt, prec, sp)
            e1.record(stream)
            evs.append((e0, e1))
        barrier()
        ms = [a.elapsed_time(b) for a, b in evs]
        return float(np.mean(ms)), ms

    with ClockSampler(dev.index) as clk:
        ms_mixed, ms_list = timed(_lib.PREC_MIXED, args.steps, args.warmup)
    clocks = clk.summary()
    ms_t = torch.tensor([ms_mixed], device=dev)
    if dist is not None:
        dist.all_reduce(ms_t, op=dist.ReduceOp.MAX)
    ms_step = float(ms_t.item())

    # e2e through the C ABI with pinned host buffers
    xh = torch.from_numpy(x).pin_memory()
    yh = torch.empty_like(xh).pin_memory()
    for _ in range(args.warmup):
        plan.apply_host(xh, yh, _lib.PREC_MIXED, sp)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        plan.apply_host(xh, yh, _lib.PREC_MIXED, sp)
    barrier()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_t = torch.tensor([e2e_s], device=dev)
    if dist is not None:
        dist.all_reduce(e2e_t, op=dist.ReduceOp.MAX)
    e2e_s = float(e2e_t.item())

    # plain FP64 apply (the parity path) for the mixed/FP64 ratio
    ms_fp64 = None
    y64 = None
    if args.fp64_steps > 0:
        ms_fp64, _ = timed(_lib.PREC_FP64, args.fp64_steps, 1)
        y64 = yt.cpu().numpy()
    plan.apply_device(xt, yt, _lib.PREC_MIXED, sp)
    torch.cuda.synchronize(dev)
    ymix = yt.cpu().numpy()
    idx = np.random.default_rng(0).choice(n, size=min(args.ncheck, n), replace=False)
    yd = f.direct_apply(x, idx)
    den = np.abs(yd).max()
    err_mixed = float(np.abs(ymix[idx] - yd).max() / den)
    err_fp64 = None if y64 is None else float(np.abs(y64[idx] - yd).max() / den)

    # roofline of the dominant stage (translations, mixed).  Units are kernel
    # evaluations counted from the built lists.  Per evaluation the algorithm
    # needs 3 FP32 subtractions, 3 FMA-pipe ops for r^2, 1 rsqrt (XU pipe) and
    # one FMA per direction it feeds: 7 FMA-pipe ops on the per-direction
    # path, 8 on the symmetric path (one evaluation feeds both directions).
    # GB300: 128 FMA-pipe lanes/clk/SM; the XU pipe (32 lanes/clk/SM by ncu
    # pct_of_peak of sm__inst_executed_pipe_xu) is not binding.
    # peak = 152 SMs x 128/ops evaluations/clk x max SM clock.  The timed
    # launch covers the whole translation stage (on the symmetric path the
    # evaluation kernel plus the partial-sum reduction).
    peaks, src = measured_peaks()
    t_ms = plan.time_translations(_lib.PREC_MIXED, reps=5, stream=sp)
    info = plan.info
    pairs = int(info.npairs_fused)
    evals = int(info.npairs_evaluated_mixed)
    sym = evals < pairs
    ops = 8 if sym else 7
    achieved = evals / (t_ms * 1e-3) / 1e9
    sm_mhz = float(peaks.get("sm_max_mhz", 2070.0))
    peak = 152 * (128.0 / ops) * sm_mhz * 1e6 / 1e9
    kern = "k_translate_sym<LAPLACE_3D> + k_sym_reduce" if sym else "k_translate_f32x2<LAPLACE_3D>"
    roofline = {
        "bound": "fp32-fma", "kernel": kern, "achieved": round(achieved, 1),
        "peak": round(peak, 1), "unit": "Geval/s", "frac": round(achieved / peak, 4),
        "traffic": profiled_traffic("translate_sym_lap3d_1M.md" if sym else "translate_lap3d_1M.md"),
        "peak_source": f"152 SMs x 128/{ops} evaluations/clk (FP32 FMA pipe, {ops} ops per evaluation) x "
                       f"sm_max_mhz {sm_mhz:.0f} ({src} MEASURED_PEAKS.json clock); XU (rsqrt) not binding",
        "evaluations_per_launch": evals, "pairs_per_launch": pairs, "launch_ms": round(t_ms, 4),
        "pairs_per_s_G": round(pairs / (t_ms * 1e-3) / 1e9, 1),
    }
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(f, x)
    value = n * ws / (ms_step * 1e-3) / 1e6
    line = {
        "metric": "apply Mpts/s, 3D Laplace N=1M tol 1e-6 (mixed FP32-kernel apply; plain FP64 apply and build s alongside)",
        "value": round(value, 2), "unit": "Mpts/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 kernel eval, f64 accumulation", "data": "synthetic",
        "config": {"workload": WORKLOAD, "N": n, "tol": args.tol, "leaf_size": args.leaf,
                   "charges": "RandomState(1).randn", "points": "default_rng(rank).random((N,3))",
                   "l2": "256 MB buffer zeroed between timed steps (outside the step events); working set ~1 GB",
                   "parallelism": f"replicas x{ws}"},
        "e2e": {"value": round(n * ws / e2e_s / 1e6, 2), "unit": "Mpts/s", "h2d_bytes_per_step": n * 8,
                "d2h_bytes_per_step": n * 8, "ms_per_step": round(e2e_s * 1e3, 3)},
        "gpu_launches": int(info.launches_mixed) * args.steps,
        "build_s": round(build_s, 3),
        "fp64_ms_per_step": None if ms_fp64 is None else round(ms_fp64, 3),
        "mixed_over_fp64": None if ms_fp64 is None else round(ms_fp64 / ms_step, 2),
        "err_mixed_vs_fp64_direct": err_mixed, "err_fp64_vs_fp64_direct": err_fp64, "ncheck": len(idx),
        "roofline": roofline, "clocks": clocks,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


def run_reference(args):
    """The reference algorithm on the host cores (oracle port), bounded sample per step."""
    import multiprocessing as mp

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import skel_oracle as O
    from skelfmm_gb300.tree import BalancedTree

    pts, x = workload(args.n)
    n = args.n
    ctx = mp.get_context("spawn")
    ncores = os.cpu_count() or 1
    t0 = time.perf_counter()
    tree = BalancedTree(pts, args.leaf)
    # one BLAS thread per pool worker (the workers read these at import; a
    # multi-threaded BLAS in every worker oversubscribes the cores)
    blas_env = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in blas_env}
    os.environ.update({k: "1" for k in blas_env})
    try:
        pool = ctx.Pool(ncores)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    with pool:
        ob = O.OracleBuild(tree, O.OPERATORS["laplace_3d"], 0.0, args.tol).skel_tree(500, pool=pool)
    build_s = time.perf_counter() - t0
    oa = O.OracleApply(ob, nthreads=ncores)
    # ragged view of the oracle build for sampled translations
    nb = ob.nboxes
    bs = ob.bs_list
    off = np.zeros(nb + 1, dtype=np.int64)
    np.cumsum(bs, out=off[1:])
    xyz = np.concatenate([tree.XX[ob.pid[b]] for b in range(nb) if bs[b] > 0])
    work = {}
    for u, s in np.vstack((ob.leaf_uskel_from_qskel_list, ob.tree_uskel_from_qskel_list)):
        work.setdefault(int(u), []).append((int(s), 0))
    for u, s in ob.uskel_from_q_list:
        work.setdefault(int(u), []).append((int(s), 1))
    for u, s in ob.u_from_qskel_list:
        work.setdefault(int(u), []).append((int(s), 2))
    for u, s in ob.u_from_q_list:
        work.setdefault(int(u), []).append((int(s), 3))
    lo = np.zeros(nb + 1, dtype=np.int64)
    srcs, kinds = [], []
    for b in range(nb):
        lst = work.get(b, [])
        lo[b + 1] = lo[b] + len(lst)
        srcs += [s for s, _ in lst]
        kinds += [k for _, k in lst]
    srcs = np.array(srcs, dtype=np.int64)
    kinds = np.array(kinds, dtype=np.int64)
    wcost = np.array([bs[b] * sum(bs[s] for s in srcs[lo[b]:lo[b + 1]]) for b in range(nb)], dtype=np.float64)
    total = float(wcost.sum())
    t0 = time.perf_counter()
    qv, qhv = oa.upward(x)
    t_up = time.perf_counter() - t0
    q = np.concatenate([qv[b] for b in range(nb) if bs[b] > 0])
    qh = np.concatenate([qhv[b] for b in range(nb) if bs[b] > 0])
    rng = np.random.default_rng(0)
    per_step = max(1e8, total / 200.0)

    def step():
        sel, acc = [], 0.0
        while acc < per_step:
            b = int(rng.integers(nb))
            if wcost[b] > 0:
                sel.append(b)
                acc += wcost[b]
        t = time.perf_counter()
        res = O.translation_sample("laplace_3d", 0.0, xyz, None, off, ob.rank_list, lo, srcs, kinds, q, qh,
                                   sel, ncores)
        dt = time.perf_counter() - t
        return sum(r[2] for r in res), dt

    for _ in range(args.warmup):
        step()
    pairs, secs = 0, 0.0
    for _ in range(args.steps):
        p_, s_ = step()
        pairs += p_
        secs += s_
    rate = pairs / secs
    t_apply = total / rate + 2 * t_up
    value = n / t_apply / 1e6
    line = {
        "metric": "apply Mpts/s, 3D Laplace N=1M tol 1e-6 (mixed FP32-kernel apply; plain FP64 apply and build s alongside)",
        "impl": "reference", "value": round(value, 4), "unit": "Mpts/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_apply * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "N": n, "tol": args.tol, "leaf_size": args.leaf},
        "build_s": round(build_s, 2),
        "cpu_baseline": {"value": round(value, 4), "unit": "Mpts/s", "cores": ncores, "kind": "port",
                         "sample": f"{args.steps} steps x ~{per_step:.3g} kernel evaluations of random target "
                                   f"boxes ({100 * pairs / total:.2f}% of one apply), FP64 dense numpy blocks; "
                                   f"apply time = evaluations / rate + upward/downward passes"},
        "e2e": {"value": round(value, 4), "unit": "Mpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
