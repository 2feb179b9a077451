"""Benchmark: L1 pdist of 100,000 float32 PCFs (L ~ Poisson(256) + 2,
N(0,1) values, last value 0, Exp(1) gaps) on one GB300.

A step is one full pdist pass over the whole problem (4,999,950,000 pairs)
with the CSR input and the 20 GB condensed output resident in HBM.
Prints one JSON line (see the keys below).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--n N]

``--impl reference`` times the reference's CPU algorithm (the oracle's C
restatement of stablebear's CPU pairwise task, all host threads) on bounded
row samples of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PCF pairs/s, L1 pdist N=100k fp32, 1 GB300"
UNIT = "pairs/s"
W_SEG = 5  # algorithmic FP32 lane-ops per merged segment (compare, dt, diff, scale, accumulate)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=100_000, help="PCFs (the benchmark workload is 100000)")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-sample-rows", type=int, default=0, help="rows in the CPU baseline sample (0 = auto)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ref-kernel", action="store_true",
                    help="skip the reference's own CUDA kernel on the same problem after the timed region")
    ap.add_argument("--order", type=int, default=0, choices=[0, 1],
                    help="processing order of the device entry: 0 length order (default), 1 caller order")
    ap.add_argument("--variant", type=int, default=0, choices=range(0, 9),
                    help="kernel variant of the engine (0 automatic; 4 hybrid, 5 shared memory, 6 time-windowed; "
                         "7 replicated row with one unified load per step, 8 merge path: measurement only)")
    ap.add_argument("--lengths", default="",
                    help="LO:HI: breakpoint counts ~ U{LO..HI} instead of the headline's Poisson(256)+2 "
                         "(a measurement workload, not the headline)")
    ap.add_argument("--window-cap", type=int, default=0,
                    help="time-windowed kernel: elements of a PCF per window (0 automatic)")
    ap.add_argument("--config", default="large",
                    choices=["large", "plain", "stable_rank", "batched", "fwdbwd", "dense", "ref_gpu_kernel"],
                    help="large: the headline workload; the others print their own report line; "
                         "ref_gpu_kernel (with --impl reference): the reference's own CUDA block kernel "
                         "on the headline workload's shape at --n PCFs")
    return ap.parse_args()


# ---- the other workloads (reported beside the headline) -----------------------

def _time_device(fn, steps, warmup):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def _device_problem(pts, off):
    import torch
    return torch.from_numpy(pts).cuda(), torch.from_numpy(off.astype(np.int64)).cuda()


def _traffic_per_launch(kernel, n):
    """DRAM bytes (read + write) per launch from the committed ncu capture
    ``profiles/traffic.json``, scaled from the captured case by output pairs
    (the traffic is the condensed output stream); None without a capture."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "profiles", "traffic.json")
    try:
        with open(path) as fh:
            e = json.load(fh).get(kernel)
    except (OSError, ValueError):
        return None
    if not e:
        return None
    return float(e["bytes"]) * (n * (n - 1) // 2) / float(e["pairs"])


def _hbm_peak():
    """HBM copy bandwidth (GB/s) from the measured-peaks file beside this
    script, else one earlier GB300 measurement."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback (6.8 TB/s, one earlier GB300 measurement)"


def run_aux(args):
    import torch
    from stablebear_gb300 import _native as nat, synthetic
    from oracle import oracle as orc
    lib = nat.lib()
    st = lambda: ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    threads = os.cpu_count() or 1
    rep = {"config_name": args.config, "data": "synthetic"}
    if args.variant:
        nat.check(lib.sbg_set_tuning(0, 0, args.variant, 0, 0))
        rep["variant"] = args.variant
    if args.window_cap:
        nat.check(lib.sbg_set_window_cap(args.window_cap))
        rep["window_cap"] = args.window_cap

    def single(pts, off, opc, p, skip, out, lmax):
        dp, do = _device_problem(pts, off)
        n = len(off) - 1
        return lambda: nat.check(lib.sbg_pairwise_device(nat.F32 if pts.dtype == np.float32 else nat.F64, opc, p, skip,
                                                         dp.data_ptr(), do.data_ptr(), n, None, None, 0, None, None,
                                                         lmax, out.data_ptr(), 0, 0, 0, st()))

    if args.config == "plain":
        pts, off = synthetic.plain_l1(1000, seed=0)
        n = 1000
        out = torch.empty(n * (n - 1) // 2, device="cuda")
        f = single(pts, off, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, out, int(np.diff(off.astype(np.int64)).max()))
        ms = _time_device(f, max(args.steps, 20), max(args.warmup, 3))
        ref = orc.evaluate(pts, off, threads=threads)
        t0 = time.perf_counter()
        orc.evaluate(pts, off, threads=threads)
        cpu_s = time.perf_counter() - t0
        rep.update({"workload": "L1 pdist N=1000 f32, L~U{10..200}", "pairs": n * (n - 1) // 2,
                    "gpu_ms": ms, "gpu_pairs_per_s": n * (n - 1) / 2 / (ms / 1e3),
                    "segments": synthetic.segment_count(off, pts, 1),
                    "cpu_pairs_per_s": n * (n - 1) / 2 / cpu_s, "cpu_cores": threads,
                    "max_rel_err_vs_reference_cpu": float(np.max(np.abs(out.cpu().numpy() - ref) / np.maximum(np.abs(ref), 1e-30)))})
    elif args.config == "stable_rank":
        n = args.n if args.n != 100_000 else 20_000
        pts, off = synthetic.stable_rank(n, seed=0)
        lmax = int(np.diff(off.astype(np.int64)).max())
        rows = np.unique(np.random.default_rng(1).integers(1, n, size=24)).astype(np.uint64)
        for name, opc, p, skip in (("l2_kernel", nat.OP_L2_INNER, 1.0, nat.SKIP_LOWER),
                                   ("l2_pdist", nat.OP_LP, 2.0, nat.SKIP_LOWER_NODIAG)):
            cnt = int(lib.sbg_output_count(skip, n, n))
            out = torch.empty(cnt, dtype=torch.float64, device="cuda")
            f = single(pts, off, opc, p, skip, out, lmax)
            ms = _time_device(f, max(1, args.steps // 2), 1)
            mode = orc.MODE_KERNEL if skip == nat.SKIP_LOWER else orc.MODE_PDIST
            oop = orc.OP_L2 if skip == nat.SKIP_LOWER else orc.OP_LP
            t0 = time.perf_counter()
            vals, starts = orc.evaluate_rows(pts, off, rows, op=oop, p=p, mode=mode, threads=threads)
            cpu_s = time.perf_counter() - t0
            truth, _ = orc.evaluate_rows(pts, off, rows[:6], op=oop, p=p, mode=mode, truth=True, threads=threads)
            host = out.cpu().numpy()
            per = 1 if skip == nat.SKIP_LOWER else 0
            got = np.concatenate([host[(int(i) * (int(i) + 1) // 2 if per else int(i) * (int(i) - 1) // 2):
                                       (int(i) * (int(i) + 1) // 2 if per else int(i) * (int(i) - 1) // 2) + int(i) + per]
                                  for i in rows])
            gt = got[: int(starts[min(6, len(rows))])]
            floor = 1.0 if skip == nat.SKIP_LOWER else 1e-300
            rep[name] = {"gpu_ms": ms, "pairs": cnt, "gpu_pairs_per_s": cnt / (ms / 1e3),
                         "segments": synthetic.segment_count(off, pts, 2 if per else 1),
                         "cpu_pairs_per_s": int(starts[-1]) / cpu_s, "cpu_cores": threads,
                         "max_rel_err_vs_reference_cpu": float(np.max(np.abs(got - vals) / np.maximum(np.abs(vals), floor))),
                         "max_rel_err_vs_fp64_oracle": float(np.max(np.abs(gt - truth) / np.maximum(np.abs(truth), floor)))}
            del out
        rep.update({"workload": f"N={n} f64 stable-rank-like, L=round(exp(U[ln16,ln4096]))", "lmax": lmax})
    elif args.config == "batched":
        from stablebear_gb300.batch import PairwiseBatch
        probs = synthetic.batched_betti(512, seed=0)
        pairs = sum((len(o) - 1) * (len(o) - 2) // 2 for _, o in probs)
        segs = sum(synthetic.segment_count(o, p_, 1) for p_, o in probs)
        for name, op, p in (("l1", "l1", 1.0), ("l2", "lp", 2.0)):
            b = PairwiseBatch(probs, op=op, p=p, graph=True)
            b.run()
            torch.cuda.synchronize()
            tuned = b.autotune()
            ms_b = _time_device(b.run, max(3, args.steps), 2)
            info = b.info()
            # the plain single-problem path, one launch per problem
            outs = [o for o in b.outputs]
            fns = [single(pp, oo, nat.OP_L1 if op == "l1" else nat.OP_LP, p, nat.SKIP_LOWER_NODIAG, out_,
                          int(np.diff(oo.astype(np.int64)).max())) for (pp, oo), out_ in zip(probs, outs)]
            ms_plain = _time_device(lambda: [f() for f in fns], 2, 1)
            # parity: two problems against the oracle
            errs = []
            b.run()
            torch.cuda.synchronize()
            for k in (0, 255):
                pp, oo = probs[k]
                want = orc.evaluate(pp, oo, op=orc.OP_L1 if op == "l1" else orc.OP_LP, p=p, threads=threads)
                got = b.outputs[k].cpu().numpy()
                errs.append(float(np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-30))))
            rep[name] = {"batched_ms": ms_b, "batched_pairs_per_s": pairs / (ms_b / 1e3),
                         "batched_segments_per_s": segs / (ms_b / 1e3), "plain_loop_ms": ms_plain,
                         "plain_loop_pairs_per_s": pairs / (ms_plain / 1e3), "speedup_vs_plain": ms_plain / ms_b,
                         "autotuned_ms": tuned, "launch": info, "max_rel_err_vs_reference_cpu": max(errs)}
            b.close()
            # the same batch with the window cap among the tuned settings
            bw = PairwiseBatch(probs, op=op, p=p, graph=True, tune_window=True)
            bw.run()
            torch.cuda.synchronize()
            tuned_w = bw.autotune()
            ms_w = _time_device(bw.run, max(3, args.steps), 2)
            bw.run()
            torch.cuda.synchronize()
            errs_w = []
            for k in (0, 255):
                pp, oo = probs[k]
                want = orc.evaluate(pp, oo, op=orc.OP_L1 if op == "l1" else orc.OP_LP, p=p, threads=threads)
                got = bw.outputs[k].cpu().numpy()
                errs_w.append(float(np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-30))))
            rep[name]["tune_window"] = {"batched_ms": ms_w, "autotuned_ms": tuned_w, "launch": bw.info(),
                                        "max_rel_err_vs_reference_cpu": max(errs_w)}
            bw.close()
        rep.update({"workload": "512 problems, N_i~U{50..2000}, L~U{8..1024}, f32 Betti-like", "pairs": pairs,
                    "segments": segs})
    elif args.config == "fwdbwd":
        from stablebear_gb300 import autograd as ag
        pts, off = synthetic.differentiation(4096, seed=0)
        n = 4096
        P = torch.tensor(pts, device="cuda", requires_grad=True)
        O = torch.tensor(off.astype(np.int64), device="cuda")
        G = torch.randn(n, n, device="cuda", generator=torch.Generator("cuda").manual_seed(0))
        G = G + G.T
        lmax = int(np.diff(off.astype(np.int64)).max())
        segs_kernel = synthetic.segment_count(off, pts, 2)
        segs_dist = synthetic.segment_count(off, pts, 1)
        for name in ("l2_kernel", "l2"):
            diag = name == "l2_kernel"

            def fwd():
                # the longest PCF's length is known on the host, as for the device entry
                return ag.l2_kernel(P, O, max_points=lmax) if diag else ag.pdist(P, O, p=2, max_points=lmax)

            def fwdbwd():
                P.grad = None
                M = fwd()
                L = (G * ag.condensed_to_dense(M, n, diagonal=diag)).sum()
                L.backward()

            with torch.no_grad():
                ms_f = _time_device(fwd, max(5, args.steps), 3)
            ms_fb = _time_device(fwdbwd, max(5, args.steps), 3)
            pairs = n * (n + 1) // 2 if diag else n * (n - 1) // 2
            # rectangles walked: the forward's; the backward recomputes the same
            # merge of every off-diagonal pair (the diagonal in closed form)
            segs = segs_kernel if diag else segs_dist
            ms_b = ms_fb - ms_f
            rep[name] = {"forward_ms": ms_f, "forward_pairs_per_s": pairs / (ms_f / 1e3),
                         "fwd_bwd_ms": ms_fb, "fwd_bwd_pairs_per_s": pairs / (ms_fb / 1e3),
                         "backward_ms": ms_b, "backward_over_forward": ms_b / ms_f,
                         "forward_rect_per_s": segs / (ms_f / 1e3), "backward_rect_per_s": segs_dist / (ms_b / 1e3),
                         "backward_rate_vs_forward": (segs_dist / (ms_b / 1e3)) / (segs / (ms_f / 1e3))}
        rep.update({"workload": "N=4096 f32, L~U{16..512}, upstream G symmetric N(0,1); grads w.r.t. values and times",
                    "segments_kernel": segs_kernel, "segments_pdist": segs_dist})
    elif args.config == "dense":
        from stablebear_gb300 import device as dev
        n = args.n
        cnt = n * (n - 1) // 2
        g = torch.Generator("cuda").manual_seed(0)
        cond = torch.rand(cnt, device="cuda", generator=g)
        dense = torch.empty((n, n), device="cuda")
        hbm, src = _hbm_peak()
        to_dense = lambda: dev.condensed_to_dense(cond, n, "distance", out=dense)
        ms_d = _time_device(to_dense, max(3, args.steps), max(3, args.warmup))
        # spot check: rows against the condensed storage
        rows = [0, 1, n // 2, n - 1]
        errs = 0
        for i in rows:
            r = dense[i].cpu().numpy()
            lo = cond[i * (i - 1) // 2: i * (i - 1) // 2 + i].cpu().numpy() if i else np.zeros(0, np.float32)
            col = np.array([cond[j * (j - 1) // 2 + i].item() for j in range(i + 1, min(n, i + 65))], np.float32)
            errs += int(not (np.array_equal(r[:i], lo) and r[i] == 0 and np.array_equal(r[i + 1:i + 1 + len(col)], col)))
        ms_c = _time_device(lambda: dev.dense_to_condensed(dense, "distance", check=False), max(3, args.steps),
                            max(3, args.warmup))
        back_ok = bool(torch.equal(dev.dense_to_condensed(dense, "distance"), cond))
        bytes_d = cnt * 4 + n * n * 4     # read each condensed value once, write both dense copies
        bytes_c = n * n * 4 + cnt * 4     # read the dense matrix once, write the condensed storage
        rep.update({"workload": f"DistanceMatrix N={n} f32 in HBM: condensed -> dense and back",
                    "condensed_to_dense": {"ms": ms_d, "algorithmic_bytes": bytes_d, "gbs": bytes_d / ms_d / 1e6,
                                           "frac_of_hbm_peak": bytes_d / ms_d / 1e6 / hbm, "rows_checked": len(rows),
                                           "row_mismatches": errs},
                    "dense_to_condensed": {"ms": ms_c, "algorithmic_bytes": bytes_c, "gbs": bytes_c / ms_c / 1e6,
                                           "frac_of_hbm_peak": bytes_c / ms_c / 1e6 / hbm, "round_trip_equal": back_ok},
                    "hbm_peak_gbs": hbm, "hbm_peak_source": src})
    print(json.dumps(rep), flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


LENGTHS = ""  # --lengths LO:HI (a measurement workload); empty: the headline's Poisson(256)+2


def workload(n, seed):
    from stablebear_gb300 import synthetic
    if LENGTHS:
        lo, hi = (int(x) for x in LENGTHS.split(":"))
        return synthetic.gaussian(n, synthetic.uniform_lengths(lo, hi), np.float32, seed)
    pts, off = synthetic.large_l1(n, seed=seed)
    return pts, off


def lengths_text():
    if LENGTHS:
        lo, hi = LENGTHS.split(":")
        return f"L~U{{{lo}..{hi}}}"
    return "L~Poisson(256)+2"


def _generator_hash():
    """Hash of the synthetic-data generator, so a result names the exact inputs."""
    import hashlib
    from stablebear_gb300 import synthetic
    with open(synthetic.__file__, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()[:16]


def config(args, n, ws):
    return {"workload": f"L1 pdist, N={n} float32 PCFs, {lengths_text()}, N(0,1) values, Exp(1) gaps, seed=0",
            "n_pcfs": n, "pairs_per_step": n * (n - 1) // 2,
            "output": "condensed DistanceMatrix float32 kept in HBM",
            "l2": "inputs (CSR) and output larger than L2; no flush",
            "processing_order": "caller" if getattr(args, "order", 0) == 1 else "length order in 1024-PCF windows",
            "generator_sha256": _generator_hash(),
            "kernel_variant": getattr(args, "variant", 0) or "automatic",
            "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"}


def sample_rows(n, target_pairs, seed=1):
    """Rows spread over the whole triangle whose partner counts sum to about
    target_pairs (row i has i partners in the lower triangle)."""
    rng = np.random.default_rng(seed)
    k = max(1, int(target_pairs / max(1, n / 2)))
    rows = np.unique(rng.integers(1, n, size=k)).astype(np.uint64)
    return rows


# The CPU legs (cpu_baseline and the reference arm) time the same sample:
# rows of the same triangle holding about CPU_SAMPLE_PAIRS pairs, handed to
# the threads in pieces of CPU_CHUNK pairs so that no thread idles behind a
# long row, by the oracle's -O3 host-CPU builds with and without FMA
# contraction.
CPU_SAMPLE_PAIRS = 5.0e7
CPU_CHUNK = 4096
CPU_BUILDS = ("o3_fast", "o3_off")


def cpu_sample_rows(n, sample_rows_arg=0):
    target = sample_rows_arg * n / 2 if sample_rows_arg else CPU_SAMPLE_PAIRS
    return sample_rows(n, min(target, n * (n - 1) / 2))


def cpu_baseline(pts, off, rows, threads, build="o3_fast"):
    from oracle import oracle as orc
    t0 = time.perf_counter()
    vals, starts = orc.evaluate_rows(pts, off, rows, op=orc.OP_L1, mode=orc.MODE_PDIST, threads=threads,
                                     chunk=CPU_CHUNK, build=build)
    dt = time.perf_counter() - t0
    pairs = int(starts[-1])
    return pairs / dt, dt, pairs, vals, starts


def cpu_flags(build):
    from oracle import build_oracle as bo
    return f"gcc -O3 {bo.native_cpu_flag()} -ffp-contract={build[3:]}"


# ---- clocks --------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, mx, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        load = [s for s in sm if mx and s > 0.3 * mx] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


# ---- reference arm ---------------------------------------------------------------

def run_reference_gpu_kernel(args):
    """The reference's own CUDA block kernel (a cubin of its headers, driven
    tile by tile with its scheduler's parameters) on the headline workload's
    PCFs at N = --n: the tile kernels' device time, CSR resident."""
    import torch
    from oracle import oracle as orc
    from stablebear_gb300 import synthetic
    ok = orc.ref_gpu_kernel_available()
    if ok is not True:
        print(json.dumps({"impl": "reference", "config_name": "ref_gpu_kernel", "unavailable": ok}), flush=True)
        return
    n = args.n
    pts, off = workload(n, seed=0)
    pairs = n * (n - 1) // 2
    segs = synthetic.segment_count(off, pts, 1)
    dp = torch.from_numpy(pts).cuda()
    do = torch.from_numpy(off.astype(np.int64)).cuda()
    torch.cuda.synchronize()
    steps = args.steps if n <= 30_000 else 1
    runs = [orc.ref_gpu_triangle(dp.data_ptr(), do.data_ptr(), n) for _ in range(steps)]
    ms = min(r[0] for r in runs)
    tiles = runs[0][1]
    cfg = config(args, n, 1)
    cfg["processing_order"] = "caller order, tiles of the reference scheduler"
    cfg["kernel_variant"] = "the reference's block kernel"
    line = {"impl": "reference", "config_name": "ref_gpu_kernel", "metric": METRIC, "value": pairs / (ms / 1e3),
            "unit": UNIT, "n_gpus": 1, "steps": steps, "ms_per_step": ms, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic", "config": cfg,
            "segments_per_s": segs / (ms / 1e3), "tiles": tiles,
            "kernel": "sb::internal::cuda_pcf_block_integrate<float, float, OperationL1Dist> compiled from the "
                      "reference's headers for sm_103a; block 1x32; tiles of the reference scheduler "
                      "(32 splits, min side sqrt(SMs*1024), 80% of free memory)",
            "timed": "the tile kernels only (CSR resident on the device; no tile clearing, copies or host scatter)"}
    if n <= 30_000:
        hout = np.full(pairs, np.nan, np.float32)
        orc.ref_gpu_triangle(dp.data_ptr(), do.data_ptr(), n, host_out=hout)
        rows = np.unique(np.linspace(1, n - 1, 24).astype(np.uint64))
        want, starts = orc.evaluate_rows(pts, off, rows)
        got = np.concatenate([hout[int(i) * (int(i) - 1) // 2: int(i) * (int(i) - 1) // 2 + int(i)] for i in rows])
        line["max_rel_err_vs_reference_cpu"] = float(np.max(np.abs(got.astype(np.float64) - want) /
                                                            np.maximum(np.abs(want), 1e-30)))
    print(json.dumps(line), flush=True)


def run_reference_aux(args):
    """The reference's own CUDA block kernel on the other workloads (the
    reference has no batched launch: one tiled run per problem; no
    gradients, no device dense expansion)."""
    import torch
    from oracle import oracle as orc
    from stablebear_gb300 import synthetic
    rep = {"impl": "reference", "config_name": args.config, "data": "synthetic",
           "kernel": "the reference's sb::internal::cuda_pcf_block_integrate (cubin of its headers), tiles of its "
                     "scheduler, block 1x32; tile kernels only, CSR resident"}
    ok = orc.ref_gpu_kernel_available()
    if ok is not True or args.config in ("fwdbwd", "dense"):
        rep["unavailable"] = ok if ok is not True else (
            "the reference has no gradients" if args.config == "fwdbwd" else
            "the reference expands matrices on the host (py_distance_matrix.hpp:37-49), not on the device")
        print(json.dumps(rep), flush=True)
        return

    def dev(pts, off):
        return torch.from_numpy(pts).cuda(), torch.from_numpy(off.astype(np.int64)).cuda()

    def sample_err(pts, off, n, dt, kw, oracle_kw, rows):
        hout = np.full(n * (n + 1) // 2 if kw.get("kernel") else n * (n - 1) // 2, np.nan, dt)
        dp, do = dev(pts, off)
        orc.ref_gpu_triangle(dp.data_ptr(), do.data_ptr(), n, host_out=hout, dtype=dt, **kw)
        want, starts = orc.evaluate_rows(pts, off, rows, **oracle_kw)
        per = 1 if kw.get("kernel") else 0
        got = np.concatenate([hout[(int(i) * (int(i) + 1) // 2 if per else int(i) * (int(i) - 1) // 2):][: int(i) + per]
                              for i in rows]).astype(np.float64)
        floor = 1.0 if per else 1e-300
        return float(np.max(np.abs(got - want) / np.maximum(np.abs(want), floor)))

    if args.config == "plain":
        pts, off = synthetic.plain_l1(1000, seed=0)
        dp, do = dev(pts, off)
        ms = min(orc.ref_gpu_triangle(dp.data_ptr(), do.data_ptr(), 1000)[0] for _ in range(max(3, args.steps)))
        rep.update({"workload": "L1 pdist N=1000 f32, L~U{10..200}", "gpu_ms": ms,
                    "gpu_pairs_per_s": 499500 / (ms / 1e3),
                    "max_rel_err_vs_reference_cpu": sample_err(pts, off, 1000, np.float32, {}, {},
                                                               np.arange(1, 1000, 37, dtype=np.uint64))})
    elif args.config == "stable_rank":
        n = args.n if args.n != 100_000 else 20_000
        pts, off = synthetic.stable_rank(n, seed=0)
        dp, do = dev(pts, off)
        rows = np.unique(np.random.default_rng(1).integers(1, n, size=24)).astype(np.uint64)
        for name, kw, okw in (("l2_kernel", {"kernel": True}, {"op": orc.OP_L2, "mode": orc.MODE_KERNEL}),
                              ("l2_pdist", {"op": "lp", "p": 2.0}, {"op": orc.OP_LP, "p": 2.0})):
            ms, tiles = orc.ref_gpu_triangle(dp.data_ptr(), do.data_ptr(), n, dtype=np.float64, **kw)
            cnt = n * (n + 1) // 2 if kw.get("kernel") else n * (n - 1) // 2
            rep[name] = {"gpu_ms": ms, "tiles": tiles, "pairs": cnt, "gpu_pairs_per_s": cnt / (ms / 1e3),
                         "max_rel_err_vs_reference_cpu": sample_err(pts, off, n, np.float64, kw, okw, rows[:6])}
        rep["workload"] = f"N={n} f64 stable-rank-like, L=round(exp(U[ln16,ln4096]))"
    elif args.config == "batched":
        probs = synthetic.batched_betti(512, seed=0)
        pairs = sum((len(o) - 1) * (len(o) - 2) // 2 for _, o in probs)
        devs = [dev(p_, o) for p_, o in probs]
        for name, kw in (("l1", {}), ("l2", {"op": "lp", "p": 2.0})):
            ms = 0.0
            for (p_, o), (dp, do) in zip(probs, devs):
                ms += orc.ref_gpu_triangle(dp.data_ptr(), do.data_ptr(), len(o) - 1, **kw)[0]
            rep[name] = {"gpu_ms": ms, "gpu_pairs_per_s": pairs / (ms / 1e3)}
        p0, o0 = probs[0]
        rep["max_rel_err_vs_reference_cpu"] = sample_err(p0, o0, len(o0) - 1, np.float32, {}, {},
                                                         np.arange(1, len(o0) - 1, 41, dtype=np.uint64))
        rep.update({"workload": "512 problems, N_i~U{50..2000}, L~U{8..1024}, f32 Betti-like; one tiled "
                                "reference run per problem", "pairs": pairs})
    print(json.dumps(rep), flush=True)


def run_reference(args, ws, rank):
    if rank != 0:
        return
    if args.config == "ref_gpu_kernel":
        run_reference_gpu_kernel(args)
        return
    if args.config != "large":
        run_reference_aux(args)
        return
    pts, off = workload(args.n, seed=0)
    threads = os.cpu_count() or 1
    # The same row sample as the GPU arm's cpu_baseline leg, split over the
    # timed steps (step k takes rows[k::K]), so that the K steps together
    # time the whole sample.  Warm-up steps time both builds on the same
    # slices; the faster build is the one timed.
    rows = cpu_sample_rows(args.n, args.cpu_sample_rows)
    steps = max(1, args.steps)
    slices = [rows[k::steps] for k in range(steps)]
    warm = {b: [] for b in CPU_BUILDS}
    for w in range(max(len(CPU_BUILDS), args.warmup)):
        b = CPU_BUILDS[w % len(CPU_BUILDS)]
        r, _, _, _, _ = cpu_baseline(pts, off, slices[w % steps], threads, build=b)
        warm[b].append(r)
    build = max(CPU_BUILDS, key=lambda b: statistics.median(warm[b]))
    times, pairs_tot = [], 0
    for k in range(steps):
        r, dt, pairs, _, _ = cpu_baseline(pts, off, slices[k], threads, build=build)
        times.append(dt)
        pairs_tot += pairs
    value = pairs_tot / sum(times)
    cfg = config(args, args.n, ws)
    cfg["processing_order"] = "caller order (sampled rows, all host threads)"
    cfg["kernel_variant"] = "the reference's CPU algorithm"
    sample = (f"{len(rows)} random rows (seed 1) of the N={args.n} triangle, {pairs_tot} pairs over {steps} steps "
              f"(step k: rows k, k+{steps}, ...), pieces of {CPU_CHUNK} pairs over {threads} threads; "
              f"oracle C restatement of the reference CPU pairwise task, {cpu_flags(build)}")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                             "build": cpu_flags(build),
                             "warmup_rates": {cpu_flags(b): statistics.median(v) for b, v in warm.items()}},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)


# ---- GPU arm -------------------------------------------------------------------

def main():
    global LENGTHS
    args = parse()
    LENGTHS = args.lengths
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.config == "ref_gpu_kernel":
        raise SystemExit("--config ref_gpu_kernel times the reference's kernel: use it with --impl reference")
    if args.config != "large":
        if rank == 0:
            run_aux(args)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    import stablebear_gb300 as sb
    from stablebear_gb300 import _native as nat, synthetic

    n = args.n
    pts, off = workload(n, seed=rank)
    lens = np.diff(off.astype(np.int64))
    lmax = int(lens.max())
    pairs = n * (n - 1) // 2
    segs = synthetic.segment_count(off, pts, 1)

    dev = torch.device("cuda", local)
    dp = torch.from_numpy(pts).to(dev)
    do = torch.from_numpy(off.astype(np.int64)).to(dev)
    out = torch.empty(pairs, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    sptr = ctypes.c_void_p(stream.cuda_stream)
    lib = nat.lib()

    if args.order or args.variant:
        sb.set_tuning(order=args.order, variant=args.variant)
    if args.window_cap:
        sb.set_window_cap(args.window_cap)

    def step():
        nat.check(lib.sbg_pairwise_device(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, dp.data_ptr(),
                                          do.data_ptr(), n, None, None, 0, None, None, lmax, out.data_ptr(), 0, 0, 0,
                                          sptr))

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    launches0 = lib.sbg_kernel_launches()
    evs[0].record(stream)
    for k in range(args.steps):
        step()
        evs[k + 1].record(stream)
    torch.cuda.synchronize()
    launches = int(lib.sbg_kernel_launches() - launches0)
    if dist:
        dist.barrier()
    clk = clocks.stop()
    per = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    total_ms = evs[0].elapsed_time(evs[-1])
    if dist:
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_step = total_ms / args.steps
    value = ws * pairs * args.steps / (total_ms / 1e3)

    # parity on sampled rows of the device result against the oracle
    parity = None
    cpu = None
    rows = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rows = cpu_sample_rows(n, args.cpu_sample_rows)
        builds = {}
        for b in CPU_BUILDS:
            rate_b, dt_b, npairs, vals_b, starts = cpu_baseline(pts, off, rows, threads, build=b)
            builds[b] = (rate_b, dt_b, vals_b)
        best = max(CPU_BUILDS, key=lambda b: builds[b][0])
        rate, dt = builds[best][0], builds[best][1]
        # parity against the reference's algorithm without contraction (bit
        # for bit the oracle build that the golden tests pin)
        vals = builds["o3_off"][2]
        host = out.cpu().numpy() if pairs <= 6_000_000_000 else None
        got = np.concatenate([host[int(i) * (int(i) - 1) // 2: int(i) * (int(i) - 1) // 2 + int(i)] for i in rows])
        rel = np.abs(got.astype(np.float64) - vals) / np.maximum(np.abs(vals.astype(np.float64)), 1e-30)
        from oracle import oracle as orc
        trows = rows[:: max(1, len(rows) // 12)]
        tv, _ = orc.evaluate_rows(pts, off, trows, truth=True, threads=threads)
        gt = np.concatenate([host[int(i) * (int(i) - 1) // 2: int(i) * (int(i) - 1) // 2 + int(i)] for i in trows])
        relt = np.abs(gt.astype(np.float64) - tv) / np.maximum(np.abs(tv), 1e-30)
        parity = {"rows_checked": int(len(rows)), "pairs_checked": int(npairs),
                  "max_rel_err_vs_reference_cpu": float(rel.max()),
                  "max_rel_err_vs_fp64_oracle": float(relt.max()), "tolerance": 1e-5,
                  "ok": bool(rel.max() <= 1e-5 and relt.max() <= 1e-5)}
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{len(rows)} random rows (seed 1) of the same N={n} triangle, {npairs} pairs, {dt:.1f} s, "
                         f"pieces of {CPU_CHUNK} pairs over {threads} threads; oracle C restatement of the "
                         f"reference CPU pairwise task, {cpu_flags(best)}",
               "builds": {cpu_flags(b): {"value": builds[b][0], "seconds": builds[b][1]} for b in CPU_BUILDS},
               "max_rel_diff_contracted_vs_not": float(np.max(
                   np.abs(builds["o3_fast"][2].astype(np.float64) - vals) / np.maximum(np.abs(vals), 1e-30)))}
        del host, builds

    # end to end through the public C ABI with host buffers: host CSR in,
    # host DistanceMatrix storage out, every step.  Both output routes are
    # timed; `e2e` reports the library's default route.
    e2e = None
    if rank == 0 and not args.no_e2e:
        hout = np.empty(pairs, dtype=np.float32)
        hout[:] = 0  # touch the pages outside the timed region
        offs = np.ascontiguousarray(off)
        pg, hpt = ctypes.c_int(0), ctypes.c_int(0)
        nat.check(lib.sbg_host_memory_access(ctypes.byref(pg), ctypes.byref(hpt)))
        routes = {}
        for name, mode in (("staged", 1), ("direct", 2)):
            if mode == 2 and not (pg.value and hpt.value):
                routes[name] = {"available": False}
                continue
            nat.check(lib.sbg_set_output_mode(mode))

            def e2e_step():
                nat.check(lib.sbg_pairwise_host(nat.F32, nat.OP_L1, 1.0, nat.SKIP_LOWER_NODIAG, nat.ptr(pts),
                                                nat.ptr(offs), n, None, None, 0, nat.ptr(hout), 0))

            e2e_step()
            t0 = time.perf_counter()
            for _ in range(args.e2e_steps):
                e2e_step()
            dt = (time.perf_counter() - t0) / args.e2e_steps
            chk = hout[-1000:].astype(np.float64)
            routes[name] = {"value": pairs / dt, "ms_per_step": dt * 1e3,
                            "matches_device_result": bool(np.array_equal(hout[-1000:], out[-1000:].cpu().numpy()))}
        nat.check(lib.sbg_set_output_mode(0))
        default = routes["staged"]
        e2e = {"value": default["value"], "unit": UNIT, "h2d_bytes_per_step": int(pts.nbytes + offs.nbytes),
               "d2h_bytes_per_step": int(hout.nbytes), "ms_per_step": default["ms_per_step"],
               "steps": args.e2e_steps, "route": "staged",
               "api": "sbg_pairwise_host (host CSR in, host DistanceMatrix storage out)", "routes": routes,
               "host_memory_access": {"pageable": pg.value, "uses_host_page_tables": hpt.value}}
        del hout

    # The reference's own CUDA block kernel (cuda_pcf_kernel.cuh:95-136, tiles
    # of its scheduler, pcf_block_op.cuh:165-171) on the same device-resident
    # problem, once, after the timed region: its tile kernels' device time,
    # and sampled rows against the reference's CPU algorithm.
    ref_kernel = None
    if rank == 0 and not args.no_ref_kernel:
        from oracle import oracle as orc
        ok = orc.ref_gpu_kernel_available()
        if ok is not True:
            ref_kernel = {"unavailable": ok}
        else:
            krows = sample_rows(n, min(2.0e6, pairs))
            ms_r, tiles_r, rvals, rstarts = orc.ref_gpu_triangle_rows(dp.data_ptr(), do.data_ptr(), n, krows)
            want, _ = orc.evaluate_rows(pts, off, krows, chunk=CPU_CHUNK)
            err = np.abs(rvals.astype(np.float64) - want) / np.maximum(np.abs(want.astype(np.float64)), 1e-30)
            ref_kernel = {"ms": ms_r, "pairs_per_s": pairs / (ms_r / 1e3), "segments_per_s": segs / (ms_r / 1e3),
                          "tiles": tiles_r, "max_rel_err_vs_reference_cpu": float(np.nanmax(err)),
                          "all_sampled_entries_written": bool(not np.isnan(rvals).any()),
                          "rows_checked": int(len(krows)), "pairs_checked": int(rstarts[-1]),
                          "this_library_speedup_device": ms_r / ms_step,
                          "kernel": "sb::internal::cuda_pcf_block_integrate<float, float, OperationL1Dist> "
                                    "(a cubin of the reference's headers, sm_103a), block 1x32, tiles of the "
                                    "reference scheduler (32 splits, min side sqrt(SMs*1024), 80% of free memory)",
                          "timed": "the tile kernels only (CSR resident; no tile clearing, copies or host scatter)"}
            torch.cuda.synchronize()

    # roofline of the pair kernel: the nominal FP32 issue rate, SMs x 128
    # lanes x the SM clock sampled during the timed region; the FFMA probe
    # measured in the same run is reported beside it
    from stablebear_gb300 import roofline
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 0
    peak_measured = roofline.fp32_peak(local)
    peak_nominal = sms * 128 * mhz * 1e6 / 1e12 if mhz else None
    achieved = segs * W_SEG / (ms_step / 1e3) / 1e12
    traffic = _traffic_per_launch("pairs_kernel_l1_f32", n)
    # The pipe that actually bounds the kernel: every merged rectangle brings
    # one new 8-byte (t, v) element per lane out of shared memory; the peak is
    # 128 B per clock per SM at the sampled SM clock.
    smem_peak = 128.0 * sms * mhz * 1e6 / 1e12 if mhz else None
    smem_ach = segs * 8.0 / (ms_step / 1e3) / 1e12
    smem_view = {"achieved": smem_ach, "peak": smem_peak, "unit": "TB/s",
                 "frac": (smem_ach / smem_peak) if smem_peak else None,
                 "work_model": "8 B of (t, v) per lane per merged rectangle, from shared memory",
                 "peak_source": f"128 B/clk/SM x {sms} SMs x sampled SM clock"}
    # The hardware floor of any design that brings one new 8-byte (t, v)
    # element per lane per rectangle out of shared memory: 256 B per
    # warp-step of 32 rectangles is two wavefronts, at most one wavefront per
    # SM per clock.
    if mhz:
        ceiling = sms * mhz * 1e6 * 32 / 2.0
        smem_view["wavefront_ceiling"] = {
            "rect_per_s": ceiling, "achieved_rect_per_s": segs / (ms_step / 1e3),
            "frac": segs / (ms_step / 1e3) / ceiling,
            "model": "2 shared-memory wavefronts (256 B) per warp-step of 32 rectangles, 1 wavefront per SM per "
                     f"clock x {sms} SMs x sampled SM clock"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": config(args, n, ws),
        "segments_per_s": segs * ws / (ms_step / 1e3), "segments_per_step": segs,
        "roofline": {"bound": "fp32_issue", "achieved": achieved,
                     "peak": peak_nominal if peak_nominal else peak_measured["value"], "unit": "T lane-op/s",
                     "frac": achieved / (peak_nominal if peak_nominal else peak_measured["value"]),
                     "traffic": traffic,
                     "peak_source": (f"nominal: {sms} SMs x 128 FP32 lanes x {mhz:.0f} MHz (SM clock sampled "
                                     "during the timed region)") if peak_nominal else peak_measured["source"],
                     "peak_measured": peak_measured["value"], "peak_measured_source": peak_measured["source"],
                     "frac_of_measured": achieved / peak_measured["value"],
                     "work_model": f"{W_SEG} FP32 lane-ops per merged segment x {segs} segments per launch"},
        "hbm_output_stream": {"bytes_per_launch": pairs * 4, "achieved_gbs": pairs * 4 / (ms_step / 1e3) / 1e9},
        "smem_view": smem_view,
        "clocks": clk, "gpu_launches": launches, "step_ms": per,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if parity:
        line["parity"] = parity
    if e2e:
        line["e2e"] = e2e
    if ref_kernel:
        line["reference_gpu_kernel"] = ref_kernel
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
