"""MLS setup+apply throughput on GB300 (DataTransferKit MovingLeastSquaresOperator path).

Workload (default, "mixed_8m"): 8,000,000 sources and 8,000,000 targets
U[0,1]^3 (seeds 6, 7), Quadratic3 basis, Wendland<4>, k = 32 -- the
configuration the headline metric is quoted on.  One step = one operator
setup (search, weights, moments, pseudo-inverse, coefficients) plus one
apply over all targets.  ``value`` is targets/s of the mixed FP32/FP64 form
with inputs resident in HBM; the plain FP64 form (the reference algorithm) is
timed on the same inputs and reported beside it (``fp64_form``,
``mixed_over_fp64``), with the relative L2 error of both against the FP64 CPU
oracle on every target and the neighbour rows compared with the oracle's
(``accuracy``).  ``e2e`` is the same metric through the public host-buffer
call (``transfer_host``, the C entry ``dtk_mls_transfer_host``): the H2D
copies of the points and the source field from pinned memory and the D2H copy
of the target field are inside the timed region, overlapped with the work as
that call does.  ``cpu_baseline`` is that oracle run, timed: the CPU
restatement of the reference on all host threads over the whole workload.

At N=1 the line also carries ``rows``: short measurements (CUDA events,
one warm-up, three steps) of the other workloads of the path -- the plain
10k transfer, the FP64 form at 2M points with every neighbour row and value
checked against the oracle, the 256-problem batched radius transfer, and the
1M-point adjoint.  ``--detail FILE`` writes the full record (notes, stage
splits, per-problem errors) beside the one-line summary.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU (torchrun, one process per GPU): one shared target set of N x 8M
points U[0,1]^3 (seed 7) is cut into N Morton-ordered slices
(``sharding.target_shard``), one per rank, with the sources replicated; each
rank builds its own tree and operator, with no data-path collective
("scaling": "weak": 8M targets per GPU at every N).  Timing takes the max
over ranks.  ``--impl reference`` times the CPU restatement of the reference
algorithm (the oracle, all host threads) on the whole workload of one rank
every step.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "MLS setup+apply targets/s on 1 GB300: mixed vs FP64 form at ≤1e-6 rel L2 err"
UNIT = "targets/s"
WORKLOADS = {
    # name: (n_src, n_tgt, src_seed, tgt_seed, rbf, basis, k)
    "mixed_8m": (8_000_000, 8_000_000, 6, 7, 2, 2, 32),
    "fp64_2m": (2_000_000, None, 3, 4, 1, 2, 32),  # 126^3 jittered-grid targets
    "mixed_1m": (1_000_000, 1_000_000, 6, 7, 2, 2, 32),  # profiling size (ncu captures)
}
# workloads measured by their own functions below (also run alone with --workload)
ROW_WORKLOADS = ("fp64_2m", "batch_256", "batch_32", "adjoint_1m")
RBF_NAMES = {1: "Wendland<2>", 2: "Wendland<4>"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="mixed_8m", choices=sorted(set(WORKLOADS) | set(ROW_WORKLOADS)))
    ap.add_argument("--sample", type=int, default=20000,
                    help="targets of the CPU sample behind the per-target extrapolation")
    ap.add_argument("--oracle-targets", type=int, default=0,
                    help="targets checked against the oracle (0 = all)")
    ap.add_argument("--detail", default="", help="write the full record to this JSON file")
    ap.add_argument("--no-rows", action="store_true",
                    help="skip the side measurements of the other workloads")
    ap.add_argument("--profile-only", action="store_true",
                    help="run only the timed steps of both forms (for profiler captures)")
    return ap.parse_args()


def make_inputs(name, rank=0, world=1):
    """Sources (replicated) and this rank's targets: its Morton-ordered slice
    of one shared set of world x n_tgt targets (the whole set when world = 1)."""
    from datatransferkit_gb300 import synthetic as syn
    from datatransferkit_gb300.sharding import target_shard
    n_src, n_tgt, s_seed, t_seed, rbf, basis, k = WORKLOADS[name]
    src = syn.uniform_points(n_src, s_seed)
    if n_tgt is None:
        tgt = syn.jittered_grid(126, t_seed)
    else:
        tgt = syn.uniform_points(n_tgt * world, t_seed)
        if world > 1:
            tgt = np.ascontiguousarray(tgt[target_shard(tgt, rank, world)])
    return src, tgt, rbf, basis, k


def config_of(name, n_src, n_tgt_per_rank):
    """The workload's config, the same keys and values in both arms."""
    _, _, _, _, rbf, basis, k = WORKLOADS[name]
    return {"workload": name, "n_sources": int(n_src), "n_targets_per_gpu": int(n_tgt_per_rank),
            "basis": {1: "Linear3", 2: "Quadratic3"}[basis], "rbf": RBF_NAMES[rbf], "k": k,
            "l2_flush": f"inputs larger than L2 ({n_src * 24 / 1e6:.0f} MB of source coordinates)"}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples every 200 ms, each stamped with the host clock when
    it arrives; the summary keeps the samples of a window (the timed region),
    all samples when none fell inside it."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.rows = []  # (host time, fields)
        self.proc = None
        self.device_index = device_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 8:
                self.rows.append((time.monotonic(), parts))

    def wait_first(self, timeout: float = 3.0):
        """Until the first sample arrives (nvidia-smi starting up), at most timeout seconds."""
        end = time.monotonic() + timeout
        while self.proc is not None and not self.rows and time.monotonic() < end and self.proc.poll() is None:
            time.sleep(0.02)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0: float | None = None, t1: float | None = None):
        rows = list(self.rows)
        window = "timed region"
        if t0 is not None and t1 is not None:
            # a sample arrives up to one period after it was taken
            inside = [r for r in rows if t0 <= r[0] <= t1 + 0.25]
            if inside:
                rows = inside
            else:
                window = "sampler run (no sample inside the timed region)"
        rows = [r[1] for r in rows]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        smax = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, v in zip(names, r[4:8]):
                if v.lower() in ("active", "1"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(rows), "window": window}


# ---------------------------------------------------------------------------
# algorithmic FLOP counts (FP64) of the setup kernels
# ---------------------------------------------------------------------------
def fp64_form_flops(n_tgt, k, m, rotations):
    """Reference algorithm: per rotation the off-diagonal norm scan 2m(m-1),
    the 2x2 SVD ~30 (transcendentals counted once), the E row/column, U column
    and V column-0 rotations 3*(6m) + 6; per target-neighbour the gather,
    distance, weight, basis and symmetric moments ~ 30 + m + m(m+1), and the
    coefficients ~ 30 + 2m; per target row 0 of the pseudo-inverse 2m^2 + m."""
    per_rot = 2 * m * (m - 1) + 30 + 18 * m + 6
    per_nb = (30 + m + m * (m + 1)) + (30 + 2 * m)
    return rotations * per_rot + n_tgt * k * per_nb + n_tgt * (2 * m * m + m)


def mixed_form_fp32_ops(n_tgt, k, m):
    """Mixed form (Cholesky path), FP32-pipe operations (an FMA counts as one
    operation).  Per neighbour: the centring, three times 3 x 4; the moment
    pass (basis m - 4, weight ~13, m products, m(m+1)/2 FMAs); the double-float
    residual (basis TwoProds 2(m - 4), weight 13, compensated dot 12m, weight
    product 3, update 12m); the double-float coefficient dot (2(m - 4) + 13 +
    12m + 4).  Per target: Cholesky and triangular inverse ~m^3/3, the bound
    m(m+1)/2, two preconditioner applications 2 m(m+1)."""
    nu = m * (m + 1) // 2
    per_nb = (36 + (m - 4 + 13 + m + nu) + (2 * (m - 4) + 13 + 24 * m + 3)
              + (2 * (m - 4) + 13 + 12 * m + 4))
    return n_tgt * (k * per_nb + m ** 3 // 3 + nu + 2 * m * (m + 1))


def measure_fp32_peak(torch, dev):
    """cuBLAS FP32 GEMM rate (no TF32): the FP32-pipe analogue of the measured bf16 peak."""
    n = 8192
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.rand(n, n, dtype=torch.float32, device=dev)
    b = torch.rand(n, n, dtype=torch.float32, device=dev)
    best = 0.0
    for _ in range(4):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12)
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b
    return best


def measure_fp64_peak(torch, dev):
    """cuBLAS DGEMM rate (the FP64 analogue of the measured bf16 peak)."""
    n = 4096
    a = torch.rand(n, n, dtype=torch.float64, device=dev)
    b = torch.rand(n, n, dtype=torch.float64, device=dev)
    best = 0.0
    for _ in range(4):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12)
    del a, b
    return best


def read_profile_traffic(name, key):
    """dram bytes per unit of a kernel from a committed ncu summary."""
    f = ROOT / "profiles" / name
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith(key + "="):
            return float(line.split("=", 1)[1])
    return None


def hbm_peak():
    """Measured HBM copy rate (GB/s) of this machine, else the stated fallback."""
    f = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(f.read_text())["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s"


# ---------------------------------------------------------------------------
# CPU oracle: the whole workload, timed
# ---------------------------------------------------------------------------
def cpu_oracle_full(src, tgt, rbf, basis, k, fields):
    """The FP64 CPU oracle (all host threads) over every target: index build
    and kNN query, setup, and one apply per field.  Timed from the search to
    the first apply (one setup + apply, the GPU step's work)."""
    from oracle import cpu
    threads = cpu.max_threads()
    t0 = time.perf_counter()
    off, idx, _ = cpu.knn(src, tgt, k)
    t1 = time.perf_counter()
    coeff, _, _, under = cpu.mls_coefficients(src, tgt, off, idx, rbf, basis)
    ys = [cpu.apply(off, idx, coeff, fields[0])]
    t2 = time.perf_counter()
    ys += [cpu.apply(off, idx, coeff, f) for f in fields[1:]]
    return dict(seconds=t2 - t0, search_s=t1 - t0, setup_apply_s=t2 - t1, threads=threads,
                offset=off, idx=idx, ys=ys, underdetermined=under)


def cpu_oracle_extrapolated(src, tgt, vals, rbf, basis, k, sample):
    """The per-target extrapolation kept beside the full run: the index build
    over all sources (warm, best of two) plus `sample` targets' kNN query,
    setup and apply, scaled to the whole target set."""
    from oracle import cpu
    sub = tgt[:sample]
    cpu.knn(src[:1000], tgt[:10], k)  # load and warm the library
    t_build = float("inf")
    for _ in range(2):
        t0 = time.perf_counter()
        cpu.knn(src, tgt[:1], k)
        t_build = min(t_build, time.perf_counter() - t0)
    t0 = time.perf_counter()
    off, idx, _ = cpu.knn(src, sub, k)
    t_knn = time.perf_counter() - t0
    t0 = time.perf_counter()
    coeff, _, _, _ = cpu.mls_coefficients(src, sub, off, idx, rbf, basis)
    cpu.apply(off, idx, coeff, vals)
    t_setup = time.perf_counter() - t0
    per_target = (max(t_knn - t_build, 0.0) + t_setup) / len(sub)
    return len(tgt) / (t_build + len(tgt) * per_target)


# ---------------------------------------------------------------------------
# reference arm: the CPU restatement of the reference, the whole workload per step
# ---------------------------------------------------------------------------
def run_reference(args, rank, world):
    if rank != 0:
        return
    from datatransferkit_gb300 import synthetic as syn
    src, tgt, rbf, basis, k = make_inputs(args.workload, 0, world)
    vals = syn.smooth_field(src)
    secs, last = [], None
    for it in range(args.warmup + args.steps):
        r = cpu_oracle_full(src, tgt, rbf, basis, k, [vals])
        if it >= args.warmup:
            secs.append(r["seconds"])
        last = r
        del r
    mean_s = float(np.mean(secs))
    value = len(tgt) / mean_s
    extrap = cpu_oracle_extrapolated(src, tgt, vals, rbf, basis, k, args.sample)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": mean_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded U[0,1]^3 clouds)",
        "config": config_of(args.workload, len(src), len(tgt)),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": last["threads"], "kind": "port",
                         "sample": (f"every step the whole workload: {len(src)}-source index build, "
                                    f"kNN, FP64 setup and apply of all {len(tgt)} targets"),
                         "stage_s": {"search": last["search_s"], "setup_apply": last["setup_apply_s"]},
                         "extrapolated_from_sample": {"value": extrap, "sample_targets": args.sample}},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# side measurements: the other workloads of the path, one GPU
# ---------------------------------------------------------------------------
def _event_time(torch, stream, fn, steps, warmup):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def row_plain_10k(torch, dtk, syn, dev, stream):
    """Plain transfer: 10k / 10k U[0,1]^3 (seeds 1, 2), Quadratic3, Wendland<2>,
    k = 20, FP64; rows and values against the oracle, and the approximation
    error against f at the targets."""
    from oracle import cpu as ocpu
    src, tgt = syn.uniform_points(10_000, 1), syn.uniform_points(10_000, 2)
    vals = syn.smooth_field(src)
    s_d, t_d, v_d = (torch.from_numpy(a).to(dev) for a in (src, tgt, vals))
    out = torch.empty(len(tgt), dtype=torch.float64, device=dev)
    W2, Q = dtk.Wendland(2), dtk.MultivariatePolynomialBasis(dtk.Quadratic, 3)
    holder = {}

    def step():
        holder["op"] = dtk.MovingLeastSquaresOperator(None, s_d, t_d, W2, Q, k=20, precision="fp64")
        holder["op"].apply(v_d, out)

    ms = _event_time(torch, stream, step, 3, 1)
    ref = ocpu.mls_transfer(src, tgt, vals, 1, 2, k=20)
    y = out.cpu().numpy()
    _, idx, _ = holder["op"].csr()
    f_t = syn.smooth_field(tgt)
    return {"value": len(tgt) / (ms / 1e3), "ms": ms,
            "rows_bit_exact": bool(np.array_equal(idx.cpu().numpy(), ref["idx"])),
            "rel_l2_vs_oracle": float(np.linalg.norm(y - ref["target"]) / np.linalg.norm(ref["target"])),
            "rel_l2_vs_f": float(np.linalg.norm(y - f_t) / np.linalg.norm(f_t))}


def row_fp64_2m(torch, dtk, syn, dev, stream, n_check=0, profile_only=False):
    """Plain FP64 form at scale: 2M U[0,1]^3 sources, 2M targets on a jittered
    126^3 grid, Quadratic3, Wendland<2>, k = 32; every neighbour row compared
    with the oracle's and every value by relative L2 (n_check > 0: the first
    n_check targets only)."""
    from oracle import cpu as ocpu
    src, tgt, rbf, basis_id, k = make_inputs("fp64_2m")
    vals = syn.smooth_field(src)
    s_d, t_d, v_d = (torch.from_numpy(a).to(dev) for a in (src, tgt, vals))
    out = torch.empty(len(tgt), dtype=torch.float64, device=dev)
    W2, Q = dtk.Wendland(2), dtk.MultivariatePolynomialBasis(dtk.Quadratic, 3)
    ops = []

    def step():
        op = dtk.MovingLeastSquaresOperator(None, s_d, t_d, W2, Q, k=k, precision="fp64")
        op.apply(v_d, out)
        ops.append(op.stage_times_ms)

    ms = _event_time(torch, stream, step, 1 if profile_only else 3, 1)
    if profile_only:
        return {"profile_only": True, "workload": "fp64_2m", "ms_per_step": ms}
    op = dtk.MovingLeastSquaresOperator(None, s_d, t_d, W2, Q, k=k, precision="fp64")
    op.apply(v_d, out)
    _, idx, _ = op.csr()
    sub = tgt if n_check <= 0 else tgt[:n_check]
    r = cpu_oracle_full(src, sub, rbf, basis_id, k, [vals])
    y = out[: len(sub)].cpu().numpy()
    y_ref = r["ys"][0]
    return {"value": len(tgt) / (ms / 1e3), "ms": ms,
            "stages_ms": {"search": float(np.mean([t[0] for t in ops[1:]])),
                          "setup": float(np.mean([t[1] for t in ops[1:]]))},
            "rows_checked": len(sub),
            "rows_bit_exact": bool(np.array_equal(idx[: len(r["idx"])].cpu().numpy(), r["idx"])),
            "rel_l2_vs_oracle": float(np.linalg.norm(y - y_ref) / np.linalg.norm(y_ref))}


def row_batch(torch, dtk, syn, dev, stream, n_problems=256, profile_only=False):
    """Batched uneven transfers: 256 problems (fewer for profiler captures), sizes log-uniform 1e3..1e5,
    Gaussian-mixture sources (8 clusters, sigma 0.02..0.2), U[0,1]^3 targets,
    radius 0.05, linear/quadratic alternating, Wendland<2>, FP64.  One step =
    batch setup (one search, one persistent setup launch) + one graph-replayed
    apply; beside it, a re-setup on the kept rows + apply, both graph replays."""
    from oracle import cpu as ocpu
    probs = syn.batched_problems(n_problems, 5)
    W2 = dtk.Wendland(2)
    B = {1: dtk.MultivariatePolynomialBasis(dtk.Linear, 3), 2: dtk.MultivariatePolynomialBasis(dtk.Quadratic, 3)}
    inputs = [dict(source_points=torch.from_numpy(p["src"]).to(dev),
                   target_points=torch.from_numpy(p["tgt"]).to(dev), rbf=W2, basis=B[p["basis"]],
                   radius=0.05) for p in probs]
    vals = np.concatenate([syn.smooth_field(p["src"]) for p in probs])
    v_d = torch.from_numpy(vals).to(dev)
    n_tgt = sum(len(p["tgt"]) for p in probs)
    out = torch.empty(n_tgt, dtype=torch.float64, device=dev)
    holder = {}

    def step():
        b = dtk.MovingLeastSquaresBatch(inputs, precision="fp64")
        b.apply(v_d, out, graph=True)
        holder["b"] = b

    ms = _event_time(torch, stream, step, 1 if profile_only else 3, 1)
    if profile_only:
        return {"profile_only": True, "workload": f"batch_{n_problems}", "ms_per_step": ms}
    b = holder["b"]
    ms_graph = _event_time(torch, stream, lambda: b.apply(v_d, out, graph=True), 20, 3)
    ms_direct = _event_time(torch, stream, lambda: b.apply(v_d, out, graph=False), 20, 3)
    # re-setup on the same coordinates with the create's rows, replayed from
    # its CUDA graph (one persistent launch), then the graph-replayed apply;
    # the coefficients must come out bit for bit as the create's
    _, _, c0 = b.csr()

    def resetup_step():
        b.resetup()
        b.apply(v_d, out, graph=True)

    ms_resetup = _event_time(torch, stream, resetup_step, 5, 3)
    off, idx, coeff = b.csr()
    resetup_bitwise = bool(torch.equal(coeff, c0))
    off = off.cpu().numpy()
    rows = np.diff(off)
    y = out.cpu().numpy()
    # oracle on the smallest and the largest problem, beside the oracle's own
    # spread (its distance to its multiply-add-contracted build): rows with
    # fewer neighbours than basis terms make the reference algorithm itself
    # reproducible only to that spread
    sizes = [len(p["src"]) for p in probs]
    errs = {}
    for p in (int(np.argmin(sizes)), int(np.argmax(sizes))):
        pr = probs[p]
        f = vals[b.source_offsets[p]:b.source_offsets[p + 1]]
        ref = ocpu.mls_transfer(pr["src"], pr["tgt"], f, 1, pr["basis"], r=0.05)
        _, spread = ocpu.rounding_spread(pr["src"], pr["tgt"], ref["offset"], ref["idx"], 1, pr["basis"], f,
                                         ref["coeff"])
        yp = y[b.target_offsets[p]:b.target_offsets[p + 1]]
        errs[f"p{p}_n{sizes[p]}"] = {
            "rel_l2": float(np.linalg.norm(yp - ref["target"]) / max(np.linalg.norm(ref["target"]), 1e-300)),
            "oracle_spread": float(spread)}
    return {"value": n_tgt / (ms / 1e3), "ms": ms, "n_targets": int(n_tgt), "nnz": int(off[-1]),
            "stages_ms": dict(zip(("search", "setup", "host"), b.stage_times_ms)),
            "apply_ms": {"graph": ms_graph, "direct": ms_direct},
            "resetup_apply_ms": ms_resetup, "resetup_bitwise": resetup_bitwise,
            "tuned": b.config,
            "rel_l2_vs_oracle": errs,
            "detail": {"row_length": {"mean": float(rows.mean()), "p50": float(np.percentile(rows, 50)),
                                      "p99": float(np.percentile(rows, 99)), "max": int(rows.max())},
                       "n_sources": int(sum(sizes))}}


def row_adjoint_1m(torch, dtk, syn, dev, stream, profile_only=False):
    """Adjoint: 1M/1M U[0,1]^3, Quadratic3, Wendland<2>, k = 32, FP64;
    L = 1/2 ||T f - g||^2, g = f + 0.05 cos(4 pi z) at the targets.  One step =
    setup + forward + adjoint (source values and source coordinates)."""
    src = syn.uniform_points(1_000_000, 12)
    tgt = syn.uniform_points(1_000_000, 13)
    f = syn.smooth_field(src)
    g = syn.smooth_field(tgt) + 0.05 * np.cos(4 * np.pi * tgt[:, 2])
    s_d, t_d, f_d, g_d = (torch.from_numpy(a).to(dev) for a in (src, tgt, f, g))
    y = torch.empty(len(tgt), dtype=torch.float64, device=dev)
    W2, Q = dtk.Wendland(2), dtk.MultivariatePolynomialBasis(dtk.Quadratic, 3)
    holder = {}

    def step():
        op = dtk.MovingLeastSquaresOperator(None, s_d, t_d, W2, Q, k=32, keep_points=True)
        op.apply(f_d, y)
        holder["g"] = op.apply_adjoint(y - g_d, f_d, coords=True)
        holder["op"] = op

    ms = _event_time(torch, stream, step, 1 if profile_only else 3, 1)
    if profile_only:
        return {"profile_only": True, "workload": "adjoint_1m", "ms_per_step": ms}
    op = holder["op"]
    ms_adj = _event_time(torch, stream, lambda: op.apply_adjoint(y - g_d, f_d, coords=True), 3, 1)
    ms_adj_v = _event_time(torch, stream, lambda: op.apply_adjoint(y - g_d), 5, 1)
    return {"value": len(tgt) / (ms / 1e3), "ms": ms,
            "adjoint_ms": {"values_and_coords": ms_adj, "values_only": ms_adj_v}}


def run_row_workload(args):
    """One of the other workloads alone (``--workload batch_256`` etc.)."""
    import torch
    import datatransferkit_gb300 as dtk
    from datatransferkit_gb300 import synthetic as syn
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    po = args.profile_only
    if args.workload == "fp64_2m":
        r = row_fp64_2m(torch, dtk, syn, dev, stream, args.oracle_targets, po)
    elif args.workload.startswith("batch_"):
        r = row_batch(torch, dtk, syn, dev, stream, int(args.workload.split("_")[1]), po)
    else:
        r = row_adjoint_1m(torch, dtk, syn, dev, stream, po)
    print(json.dumps(r), flush=True)


def run_rows(args, dev, stream):
    import torch
    import datatransferkit_gb300 as dtk
    from datatransferkit_gb300 import synthetic as syn
    rows = {}
    for name, fn in (("plain_10k", lambda: row_plain_10k(torch, dtk, syn, dev, stream)),
                     ("fp64_2m", lambda: row_fp64_2m(torch, dtk, syn, dev, stream, args.oracle_targets)),
                     ("batch_256", lambda: row_batch(torch, dtk, syn, dev, stream)),
                     ("adjoint_1m", lambda: row_adjoint_1m(torch, dtk, syn, dev, stream))):
        t0 = time.perf_counter()
        rows[name] = fn()
        rows[name]["wall_s"] = round(time.perf_counter() - t0, 1)
        torch.cuda.empty_cache()
    return rows


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args, rank, world, local_rank):
    import torch
    import datatransferkit_gb300 as dtk
    from datatransferkit_gb300 import synthetic as syn

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    src, tgt, rbf, basis_id, k = make_inputs(args.workload, rank, world)
    vals = syn.smooth_field(src)
    front = syn.front_field(src)
    RBF = {1: dtk.Wendland(2), 2: dtk.Wendland(4)}[rbf]
    BASIS = {1: dtk.MultivariatePolynomialBasis(dtk.Linear, 3),
             2: dtk.MultivariatePolynomialBasis(dtk.Quadratic, 3)}[basis_id]
    m = BASIS.size
    n_tgt = len(tgt)

    s_d = torch.from_numpy(src).to(dev)
    t_d = torch.from_numpy(tgt).to(dev)
    v_d = torch.from_numpy(vals).to(dev)
    out = torch.empty(n_tgt, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    def max_over_ranks(x):
        if world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())

    def step(precision, record):
        op = dtk.MovingLeastSquaresOperator(None, s_d, t_d, RBF, BASIS, k=k, precision=precision)
        op.apply(v_d, out)
        if record is not None:
            record.append((op.stage_times_ms, op.rotations, op.rotations_fp32, op.nnz,
                           op.search_times_ms))
        return op

    def timed(precision, steps, warmup):
        # the sampler starts before the warm-up, so that its first samples
        # are in by the time the timed region starts
        with ClockSampler(dev.index) as clk:
            clk.wait_first()
            for _ in range(warmup):
                step(precision, None)
            rec = []
            barrier()
            launches0 = dtk.kernel_launch_count()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0 = time.monotonic()
            e0.record(stream)
            for _ in range(steps):
                step(precision, rec)
            e1.record(stream)
            barrier()
            t1 = time.monotonic()
        launches = (dtk.kernel_launch_count() - launches0) // steps
        ms = max_over_ranks(e0.elapsed_time(e1) / steps)
        return ms, rec, clk.summary(t0, t1), launches

    # -- headline: mixed form, inputs resident ---------------------------------
    ms_mixed, rec_mixed, clocks, launches = timed("mixed", args.steps, args.warmup)
    # -- FP64 form on the same inputs -------------------------------------------
    ms_fp64, rec_fp64, clocks64, _ = timed("fp64", max(2, args.steps // 2), 1)
    if args.profile_only:
        if rank == 0:
            print(json.dumps({"profile_only": True, "ms_mixed": ms_mixed, "ms_fp64": ms_fp64,
                              "workload": args.workload}), flush=True)
        return

    # -- e2e through the public API with host buffers -----------------------------
    src_h = torch.from_numpy(src).pin_memory()
    tgt_h = torch.from_numpy(tgt).pin_memory()
    val_h = torch.from_numpy(vals).pin_memory()
    out_h = torch.empty(n_tgt, dtype=torch.float64).pin_memory()

    def e2e_step():
        # the public host-buffer call: points and values in from pinned host
        # memory, results out, copies overlapped with the work
        dtk.MovingLeastSquaresOperator.transfer_host(None, src_h, tgt_h, val_h, out_h, RBF, BASIS, k=k,
                                                     precision="mixed")

    for _ in range(max(1, args.warmup - 1)):
        e2e_step()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    barrier()
    ms_e2e = max_over_ranks(e0.elapsed_time(e1) / args.steps)

    # -- both forms against the FP64 oracle: every target (rank 0's shard) --------
    acc, cpu = {}, None
    n_chk = n_tgt if args.oracle_targets <= 0 else min(n_tgt, args.oracle_targets)
    res = {}
    for name, field in (("smooth", vals), ("front", front)):
        f_d = torch.from_numpy(field).to(dev)
        for prec in ("mixed", "fp64"):
            op = dtk.MovingLeastSquaresOperator(None, s_d, t_d, RBF, BASIS, k=k, precision=prec)
            op.apply(f_d, out)
            res[name, prec] = out[:n_chk].cpu().numpy()
            if prec == "fp64" and name == "smooth":
                idx_gpu = op.csr()[1][: n_chk * k].cpu().numpy()
            del op
        del f_d
    if rank == 0:
        cpu = cpu_oracle_full(src, tgt[:n_chk], rbf, basis_id, k, [vals, front])
        for j, name in enumerate(("smooth", "front")):
            y_ref = cpu["ys"][j]
            nrm = np.linalg.norm(y_ref)
            acc[name] = {prec: float(np.linalg.norm(res[name, prec] - y_ref) / nrm)
                         for prec in ("mixed", "fp64")}
        acc["neighbour_rows_bit_exact"] = bool(np.array_equal(idx_gpu, cpu["idx"]))
        acc["targets_checked"] = int(n_chk)
        cpu_value = n_chk / cpu["seconds"]
        cpu_extrap = cpu_oracle_extrapolated(src, tgt, vals, rbf, basis_id, k, args.sample)
        del cpu["ys"], cpu["idx"], cpu["offset"]
    del res

    rows = run_rows(args, dev, stream) if (world == 1 and not args.no_rows) else None

    if rank != 0:
        return
    # -- rooflines: per stage, and the dominant kernel (the kNN query) -------------
    setup_ms = float(np.mean([r[0][1] for r in rec_mixed]))
    search_ms = float(np.mean([r[0][0] for r in rec_mixed]))
    query_ms = float(np.mean([r[4][1] for r in rec_mixed]))
    build_ms = float(np.mean([r[4][0] for r in rec_mixed]))
    ops32 = mixed_form_fp32_ops(n_tgt, k, m)
    achieved = ops32 / (setup_ms / 1e3) / 1e12          # Top/s, FMA = 1 operation
    peak = measure_fp32_peak(torch, dev) / 2.0           # FMA operations/s of the SGEMM
    peak64 = measure_fp64_peak(torch, dev)
    hbm, hbm_src = hbm_peak()
    traffic_pt = read_profile_traffic("setup_mixed_traffic.txt", "bytes_per_target")
    traffic_q = read_profile_traffic("knn_traffic.txt", "bytes_per_query")
    instr_q = read_profile_traffic("knn_traffic.txt", "warp_instructions_per_query")
    # kNN query launch, algorithmic bytes: per query its 64-byte record, k
    # indices and k sorted positions out and the offset; per source its FP64 +
    # FP32 sorted copies and its index
    q_bytes = n_tgt * (64 + 8 * k + 4) + len(src) * (24 + 12 + 4)
    q_gbs = q_bytes / (query_ms / 1e3) / 1e9
    # the issue ruler: warp instructions (ncu count per query) over the SMs'
    # issue rate, one warp instruction per cycle per scheduler at the sampled clock
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    clk_mhz = clocks.get("sm_mhz") or 2070.0
    issue_peak = n_sm * 4 * clk_mhz * 1e6
    issue_frac = (instr_q * n_tgt / (query_ms / 1e3) / issue_peak) if instr_q else None
    # apply alone (CUDA events on the launching stream, inputs resident)
    op_m = dtk.MovingLeastSquaresOperator(None, s_d, t_d, RBF, BASIS, k=k, precision="mixed")
    apply_ms = _event_time(torch, stream, lambda: op_m.apply(v_d, out), 10, 3)
    a_bytes = op_m.nnz * (4 + 4) + 8 * len(src) + 8 * n_tgt + 4 * (n_tgt + 1)
    a_gbs = a_bytes / (apply_ms / 1e3) / 1e9
    del op_m
    stage_fracs = {"query": (q_gbs / hbm, query_ms), "setup": (achieved / peak, setup_ms),
                   "apply": (a_gbs / hbm, apply_ms)}
    combined = (sum(f * t for f, t in stage_fracs.values()) / sum(t for _, t in stage_fracs.values()))
    setup64_ms = float(np.mean([r[0][1] for r in rec_fp64]))
    rot_fp64_form = float(np.mean([r[1] for r in rec_fp64]))
    flops64 = fp64_form_flops(n_tgt, k, m, rot_fp64_form)
    total_targets = n_tgt * world
    value = total_targets / (ms_mixed / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_mixed, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded U[0,1]^3 clouds)",
        "config": config_of(args.workload, len(src), n_tgt),
        "form": "mixed",
        "fp64_form": {"value": total_targets / (ms_fp64 / 1e3), "ms_per_step": ms_fp64},
        "mixed_over_fp64": ms_fp64 / ms_mixed,
        "accuracy": acc,
        "e2e": {"value": total_targets / (ms_e2e / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": int(src_h.numel() * 8 + tgt_h.numel() * 8 + val_h.numel() * 8),
                "d2h_bytes_per_step": int(out_h.numel() * 8)},
        "roofline": {"bound": "hbm", "kernel": "k_knn", "achieved": q_gbs, "peak": hbm, "unit": "GB/s",
                     "frac": q_gbs / hbm, "traffic": (traffic_q * n_tgt) if traffic_q else None,
                     "launch_ms": query_ms, "issue_frac": issue_frac},
        "cpu_baseline": ({"value": cpu_value, "unit": UNIT, "cores": cpu["threads"], "kind": "port",
                          "sample": f"whole workload, all {n_chk} targets, timed"} if cpu else None),
        "gpu_launches": int(launches),
        "clocks": clocks,
        "stages_ms": {"build": build_ms, "query": query_ms, "setup": setup_ms,
                      "apply": ms_mixed - search_ms - setup_ms, "fp64_setup": setup64_ms},
    }
    if rows is not None:
        line["rows"] = {name: {k2: v for k2, v in r.items() if k2 not in ("detail", "stages_ms")}
                        for name, r in rows.items()}
    detail = dict(line)
    detail.update({
        "roofline_detail": {
            "peak_source": hbm_src, "algorithmic_bytes": q_bytes,
            "note": ("the dominant kernel of a mixed step; algorithmic bytes = N_t (64 + 8k + 4) "
                     "+ N_s (24 + 12 + 4); traffic = the ncu DRAM bytes per query of profiles/knn_traffic.txt "
                     "x N_t; issue_frac = ncu warp instructions per query x N_t / launch time / "
                     "(SMs x 4 schedulers x sampled SM clock)")},
        "roofline_stages": {
            "query": {"bound": "hbm", "achieved": q_gbs, "peak": hbm, "unit": "GB/s",
                      "frac": q_gbs / hbm, "ms": query_ms, "issue_frac": issue_frac},
            "setup": {"bound": "fp32", "kernel": "k_setup_mixed<10>", "achieved": achieved,
                      "peak": peak, "unit": "T FP32 ops/s (FMA = 1)", "frac": achieved / peak, "ms": setup_ms,
                      "peak_source": "measured cuBLAS SGEMM 8192^3 (no TF32) in this run, FMA/s",
                      "traffic": (traffic_pt * n_tgt) if traffic_pt else None},
            "apply": {"bound": "hbm", "kernel": "k_apply_pos (+ k_permute_values)", "achieved": a_gbs, "peak": hbm,
                      "unit": "GB/s", "frac": a_gbs / hbm, "ms": apply_ms},
            "time_weighted_frac": combined},
        "fp64_form_detail": {"setup_ms": setup64_ms,
                             "setup_fp64_tflops": flops64 / (setup64_ms / 1e3) / 1e12,
                             "setup_fp64_frac_of_dgemm": flops64 / (setup64_ms / 1e3) / 1e12 / peak64,
                             "dgemm_tflops": peak64, "clocks": clocks64},
        "rotations_per_target": {
            "mixed_fp32": float(np.mean([r[2] for r in rec_mixed])) / n_tgt,
            "fp64_form": rot_fp64_form / n_tgt},
        "cpu_detail": ({"seconds": cpu["seconds"], "search_s": cpu["search_s"],
                        "setup_apply_s": cpu["setup_apply_s"],
                        "extrapolated_from_sample": {"value": cpu_extrap, "sample_targets": args.sample}}
                       if cpu else None),
        "rows": rows,
    })
    if args.detail:
        Path(args.detail).write_text(json.dumps(detail, indent=1))
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload in ROW_WORKLOADS:
        if rank == 0:
            run_row_workload(args)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
