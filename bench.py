"""Benchmarks of the semiring sparse path on one GB300 (N replicas under torchrun).

Default workload (`spmv_csr_rmat22`, the R-MAT scale-22 configuration): plus-times
Float32 SpMV over the CSR of an R-MAT graph (a=0.57, b=0.19, c=0.19, edge factor 16,
symmetrised, self-loops removed, values uniform [0,1)), x uniform [0,1).  A step is
one gpu_spmv! over the whole matrix.  `value` = GB/s of algorithmic bytes
4(n+1) + 8 nnz + 4n (x) + 4n (y) with inputs resident in HBM (the ~1 GB matrix is
larger than L2, so no flush is needed); `e2e` = the same call through the public API
with x copied in from pinned host memory and y copied out every step.  The line also
carries the same graph's SELL-C-sigma SpMV, SpMM (32 row-major columns), BFS,
Bellman-Ford and batched BFS / shortest-path throughput under "secondary".

Other workloads (`--workload`, one JSON line each): bfs_rmat24, sssp_rmat24,
bfs_grid4096, sssp_grid4096 (BFS / Bellman-Ford GTEPS), serve (continuous-batching
server, queries/s with p50/p99 latency against the one-query-at-a-time path),
multigraph (1000 Erdos-Renyi graphs in one launch).

--impl reference times the reference algorithm's CPU path (the C restatement of the
reference kernels, OpenMP over every host core) on the same inputs built on the host.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                       [--workload NAME] [--no-cpu]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "gpugraphs.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

RMAT = dict(a=0.57, b=0.19, c=0.19, edge_factor=16, seed=1)
FALLBACK_HBM_GBS = 6800.0
I32MAX = 2 ** 31 - 1


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def traffic_from_profiles(workload):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary
    (profiles/traffic.txt lines: `workload kernel bytes_per_launch`), else None."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    try:
        for line in open(p):
            f = line.split()
            if len(f) >= 3 and f[0] == workload and not line.startswith("#"):
                return float(f[2])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during a timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(value, device=None):
    """The largest of a per-rank float over the process group (timings: the job is as
    slow as its slowest rank); the value itself without a group of more than one rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_gbs(ws, bytes_per_rank, ms):
    """Whole-job GB/s: every rank moved bytes_per_rank in ms (the max over ranks)."""
    return ws * bytes_per_rank / (ms * 1e-3) / 1e9


def spmv_bytes(n, nnz):
    return 4 * (n + 1) + 8 * nnz + 4 * n + 4 * n


def bfs_bytes(n, nnz):
    return 4 * (n + 1) + 4 * nnz + 4 * n


def sssp_bytes(n, nnz):
    return 4 * (n + 1) + 8 * nnz + 4 * n


# ---------------------------------------------------------------------------------
# timing helpers (CUDA events on the launching stream, synchronize on both sides)
# ---------------------------------------------------------------------------------

def time_steps(fn, steps, warmup=3):
    import torch
    for _ in range(max(warmup, 3)):
        fn()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        fn()
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def time_host(fn, reps, warmup=1):
    """Host wall time of synchronous calls (BFS / SSSP return after the search)."""
    import torch
    for _ in range(warmup):
        fn(0)
    torch.cuda.synchronize()
    ts = []
    for i in range(reps):
        t0 = time.perf_counter()
        fn(i)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    return ts


def reached_edges(A, dist):
    """m_cc: stored entries of the reached vertices / 2 (symmetric graphs, Graph500)."""
    import torch
    rp = A.rowptr.to(torch.int64)
    deg = rp[1:] - rp[:-1]
    return int(deg[dist != I32MAX].sum().item()) // 2


def sources_for(A, k, seed):
    """k seeded non-isolated vertices (1-based)."""
    import numpy as np
    import torch
    rp = A.rowptr.to(torch.int64)
    nz = torch.nonzero((rp[1:] - rp[:-1]) > 0).flatten().cpu().numpy()
    rng = np.random.default_rng(seed)
    return (nz[rng.integers(0, len(nz), k)] + 1).astype(np.int64)


# ---------------------------------------------------------------------------------
# default workload: SpMV on R-MAT scale 22 (+ secondary measurements)
# ---------------------------------------------------------------------------------

def rmat(scale, wkind, device):
    from gpugraphs import generators as gen
    return gen.rmat(scale, RMAT["edge_factor"], RMAT["a"], RMAT["b"], RMAT["c"], seed=RMAT["seed"],
                    wkind=wkind, device=device)


def secondary_rmat22(device, A, x):
    import numpy as np
    import torch
    import gpugraphs as G
    from gpugraphs import generators as gen
    out = {}
    n, nnz = A.n, A.nnz()
    y = torch.zeros(n, dtype=torch.float32, device=device)
    S = G.SparseGPUMatrixSELL(A, 32, A.n)
    ms = time_steps(lambda: G.gpu_spmv_(y, S, x), 20)
    out["sell_spmv_rmat22"] = {"gbs": round(spmv_bytes(n, nnz) / ms / 1e6, 1), "ms": round(ms, 4),
                               "C": 32, "sigma": n, "n_stored": S.n_stored}
    del S
    X = torch.rand((n, 32), dtype=torch.float32, device=device)
    Y = torch.zeros((n, 32), dtype=torch.float32, device=device)
    ms = time_steps(lambda: G.gpu_spmm_(Y, A, X), 5)
    b = 4 * (n + 1) + 8 * nnz + 4 * n * 32 * 2
    out["spmm_rmat22_k32"] = {"gbs_algorithmic": round(b / ms / 1e6, 1), "ms": round(ms, 3),
                              "layout": "row-major"}
    del X, Y
    out.update(secondary_sparse_vector(device, A))
    P = rmat(22, gen.W_PATTERN, device)
    src = sources_for(P, 256, 7)
    d = G.bfs_distances(P, int(src[0]))
    mcc = reached_edges(P, d)
    ts = time_host(lambda i: G.bfs_distances(P, int(src[i % 16])), 8)
    t = statistics.median(ts)
    out["bfs_rmat22"] = {"gteps": round(mcc / t / 1e9, 2), "ms": round(t * 1e3, 3), "m_cc": mcc}
    tb = time_host(lambda i: G.bfs_distances_batch(P, src), 2)
    tbm = statistics.median(tb)
    out["bfs_batch256_rmat22"] = {"queries_per_s": round(256 / tbm, 1), "ms": round(tbm * 1e3, 2),
                                  "aggregate_gteps": round(256 * mcc / tbm / 1e9, 1),
                                  "speedup_vs_single": round((256 / tbm) / (1 / t), 2)}
    del P
    W = rmat(22, gen.W_INT_1_255, device)
    ts = time_host(lambda i: G.shortest_path(W, int(src[i % 16])), 3)
    t1 = statistics.median(ts)
    out["sssp_rmat22_int"] = {"gteps": round(mcc / t1 / 1e9, 2), "ms": round(t1 * 1e3, 2)}
    tb = time_host(lambda i: G.shortest_path(W, src), 1)
    tbm = statistics.median(tb)
    out["sssp_batch256_rmat22_int"] = {"queries_per_s": round(256 / tbm, 1), "ms": round(tbm * 1e3, 1),
                                       "speedup_vs_single": round((256 / tbm) / (1 / t1), 2)}
    del W
    t0 = time.time()
    res = G.autotune(A, spmm_k=32)
    res["tune_s"] = round(time.time() - t0, 1)
    res["spmv_gbs"] = round(spmv_bytes(n, nnz) / res["spmv_ms"] / 1e6, 1)
    out["autotune_rmat22"] = res
    return out


def secondary_sparse_vector(device, A):
    """SpMSpV over 1% of the vertices of R-MAT s22 (plus-times Float32; the matrix is
    symmetric, so the column lists pushed have the row lengths), and the element-wise /
    reduce entry points over 2^28 Float32 values (HBM-bound)."""
    import numpy as np
    import torch
    import gpugraphs as G
    out = {}
    n = A.n
    deg = np.diff(A.rowptr.cpu().numpy().astype(np.int64))
    rng = np.random.default_rng(5)
    ind = np.sort(rng.choice(n, n // 100, replace=False)).astype(np.int32) + 1
    xv = G.SparseGPUVector(n, ind, rng.random(len(ind)).astype(np.float32))
    y = torch.zeros(n, dtype=torch.float32, device=device)
    rows = G.gpu_spmspv_(y, A, xv)
    reached = rows.long().cpu().numpy() - 1
    pushed, pulled = int(deg[ind - 1].sum()), int(deg[reached].sum())
    ts = time_host(lambda i: G.gpu_spmspv_(y, A, xv), 10)
    t = statistics.median(ts)
    b = 4 * pushed + 8 * pulled + 8 * len(reached) + 8 * len(ind)
    out["spmspv_rmat22_1pct"] = {"ms": round(t * 1e3, 3), "x_nnz": len(ind), "rows_reached": len(reached),
                                 "entries_pushed": pushed, "entries_pulled": pulled,
                                 "gbs_algorithmic": round(b / t / 1e9, 1),
                                 "note": "synchronous call incl. validation sync and result count"}
    N = 1 << 28
    a = torch.rand(N, device=device)
    b2 = torch.rand(N, device=device)
    z = torch.empty(N, device=device)
    ms = time_steps(lambda: G.gpu_ewise_(z, a, b2, G.GPUGraphs_min), 10)
    out["ewise_min_f32_2p28"] = {"ms": round(ms, 3), "gbs": round(12 * N / ms / 1e6, 1)}
    ts = time_host(lambda i: G.gpu_reduce(a, G.GPUGraphs_add), 10)
    t = statistics.median(ts)
    out["reduce_add_f32_2p28"] = {"ms": round(t * 1e3, 3), "gbs": round(4 * N / t / 1e9, 1)}
    del a, b2, z
    return out


def measure_spmv(A, x, steps, warmup, device, ws, sample_clocks=True):
    """Times `steps` plus-times SpMVs y = A x with inputs resident in HBM (CUDA events
    on the launching stream), the main kernel alone under the library's launch tracer,
    and the same call end to end with host buffers.  Returns a dict of the figures."""
    import torch
    import torch.distributed as dist
    import gpugraphs as G
    n, nnz = A.n, A.nnz()
    y = torch.zeros(n, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device)

    def step():
        G.gpu_spmv_(y, A, x)

    for _ in range(max(warmup, 3)):
        step()
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clk = ClockSampler(device.index or 0) if sample_clocks else None
    if clk:
        clk.start()
        time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    ms = ev0.elapsed_time(ev1)
    clocks = None
    if clk:
        t_end = time.time() + 1.0  # keep the sampler on the same work a little longer
        while time.time() < t_end:
            for _ in range(50):
                step()
            torch.cuda.synchronize()
        clocks = clk.stop()
    ms = max_over_ranks(ms, device)
    per_step_ms = ms / steps
    B = spmv_bytes(n, nnz)

    # roofline of the dominant kernel: the same K steps again under the library's
    # launch tracer, which brackets the matrix-streaming kernel of every call with
    # CUDA events on the launching stream and counts every kernel launch
    from gpugraphs.tracing import launch_trace
    with launch_trace(device) as tr:
        for _ in range(steps):
            step()
    kernel_ms = tr.kernel_ms / max(tr.timed, 1)

    # e2e through the public API with host buffers
    # every step copies its x from pinned host memory and reads its y back; the copies
    # of neighbouring steps overlap the SpMV on two side streams (double buffers)
    xh = x.cpu().pin_memory()
    yh = [torch.empty(n, dtype=torch.float32).pin_memory() for _ in range(2)]
    xd = [torch.empty_like(x) for _ in range(2)]
    yd = [torch.empty_like(y) for _ in range(2)]
    cin, cout = torch.cuda.Stream(device), torch.cuda.Stream(device)
    ev_in = [torch.cuda.Event() for _ in range(2)]
    ev_used = [torch.cuda.Event() for _ in range(2)]   # SpMV of the buffer pair done
    ev_freed = [torch.cuda.Event() for _ in range(2)]  # its y copied out

    def e2e_steps(k):
        start = torch.cuda.Event()
        start.record(stream)
        cin.wait_event(start)
        cout.wait_event(start)
        for i in range(k):
            b = i & 1
            with torch.cuda.stream(cin):
                cin.wait_event(ev_used[b])  # step i - 2 has read xd[b]
                xd[b].copy_(xh, non_blocking=True)
                ev_in[b].record(cin)
            stream.wait_event(ev_in[b])
            stream.wait_event(ev_freed[b])  # step i - 2's y has left yd[b]
            G.gpu_spmv_(yd[b], A, xd[b])
            ev_used[b].record(stream)
            with torch.cuda.stream(cout):
                cout.wait_event(ev_used[b])
                yh[b].copy_(yd[b], non_blocking=True)
                ev_freed[b].record(cout)
        for b in range(2):
            stream.wait_event(ev_freed[b])

    e2e_steps(max(warmup, 3))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    e2e_steps(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / steps
    assert bool(torch.equal(yd[(steps - 1) & 1].cpu(), yh[(steps - 1) & 1]))
    peak, peak_kind = peak_hbm()
    achieved = B / (kernel_ms * 1e-3) / 1e9
    return {"y": y, "per_step_ms": per_step_ms, "value": aggregate_gbs(ws, B, per_step_ms),
            "kernel_ms": kernel_ms, "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
            "frac": achieved / peak, "bytes": B, "launches": tr.launches, "clocks": clocks,
            "e2e": aggregate_gbs(ws, B, max_over_ranks(e2e_ms, device)), "e2e_ms": e2e_ms}


def run_spmv_rmat(args, scale=22):
    import torch
    import torch.distributed as dist
    import gpugraphs as G
    from gpugraphs import generators as gen

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=device)
    A = rmat(scale, gen.W_U01_F32, device)
    x = gen.uniform_vector(A.n, seed=2, device=device)
    if args.sell_variant or args.hot_cols or args.layout == "sell":
        from gpugraphs import tuning
        tuning.apply(A, {"spmv_kernel": "sell", "slice_size": 32, "sigma": A.m})
        G.gpu_spmv_(torch.zeros(A.n, device=device), A, x)  # builds the SELL-32 copy
        choice = {"sell_variant": args.sell_variant or "registers"}
        if args.hot_cols:
            choice["hot_cols"] = args.hot_cols
        tuning.apply(A, choice)
    if args.layout == "window_tiles":
        from gpugraphs import tuning
        tuning.apply(A, {"spmv_kernel": "window_tiles"})
    n, nnz = A.n, A.nnz()
    m = measure_spmv(A, x, args.steps, args.warmup, device, ws)
    y = m.pop("y")
    workload = "spmv_csr_rmat%d" % scale
    traffic = traffic_from_profiles(workload)
    layout = G.spmv_layout(A)
    if layout == "window_tiles":
        kernel_label = ("k_spmv_pipe (tail rows) + k_spmv_win (column-window tiles: rows sorted "
                        "by length, x windows of 16384 relabelled columns staged in shared memory)")
    elif G.spmv_hub_rows(A) > 0:
        kernel_label = ("k_sell_hot32 (SELL-32 copy sorted by row length, relabelled columns) "
                        "+ k_hubwin / k_hw_combine (the %d hub rows folded from shared-memory "
                        "column windows)" % G.spmv_hub_rows(A))
    else:
        kernel_label = ({"registers": "k_sell_hot32", "bulk_copy": "k_sell_tma32",
                         "hub_windows": "k_sell_hot32"}[
            args.sell_variant or "registers"]
            + " (SELL-32 copy sorted by row length, relabelled columns)")
    # parity of this run's own output, every row, after the timed region
    parity = {}
    if rank == 0 and not args.no_parity:
        parity["spmv_rmat%d" % scale] = spmv_parity(A, x, y)
    secondary = {}
    if not args.no_secondary and scale == 22:
        secondary = secondary_rmat22(device, A, x)
    cpu = cpu_baseline_spmv(A, x) if (rank == 0 and not args.no_cpu) else None
    if not args.no_secondary and scale == 22:
        del A, x, y
        torch.cuda.empty_cache()
        secondary.update(secondary_large(args, device, parity, rank))
    out = {
        "metric": "SpMV GB/s (plus-times Float32, CSR, R-MAT scale %d)" % scale,
        "value": round(m["value"], 2), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": round(m["per_step_ms"], 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded R-MAT generator on the device)",
        "config": {"workload": workload, "n": n, "nnz": nnz, "format": "CSR",
                   "semiring": "(mul, add, second)",
                   "l2": "inputs larger than L2 (CSR %.2f GB)" % ((4 * (n + 1) + 8 * nnz) / 1e9),
                   "parallelism": "replicas" if ws > 1 else "single"},
        "roofline": {"bound": "hbm", "achieved": round(m["achieved"], 2), "peak": m["peak"],
                     "unit": "GB/s", "frac": round(m["frac"], 4), "traffic": traffic,
                     "peak_kind": m["peak_kind"], "algorithmic_bytes": m["bytes"],
                     "kernel_ms": round(m["kernel_ms"], 5),
                     "kernel": kernel_label},
        "e2e": {"value": round(m["e2e"], 2), "unit": "GB/s", "h2d_bytes_per_step": 4 * n,
                "d2h_bytes_per_step": 4 * n,
                "schedule": "x of step i+1 copied in and y of step i-1 copied out on two side "
                            "streams while step i's SpMV runs (double buffers)"},
        "gpu_launches": m["launches"],
        "clocks": m["clocks"],
        "parity": parity,
        "secondary": secondary,
    }
    if cpu is not None:
        out["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def spmv_parity(A, x, y):
    """Every row of this run's SpMV output against an FP64 product (rel err <= 1e-5)
    and against the oracle's storage-order fold (csr_spmv_kernel!), bit for bit on
    the rows of <= 128 entries (the SELL-32 copy folds those in storage order)."""
    import numpy as np
    import scipy.sparse as sp
    from oracle import oracle as O
    rp, cv, nz = A.rowptr.cpu().numpy(), A.colval.cpu().numpy(), A.nzval.cpu().numpy()
    xh, yh = x.cpu().numpy(), y.cpu().numpy()
    M = sp.csr_matrix((nz.astype(np.float64), cv - 1, rp - 1), shape=(A.m, A.n))
    ref = M @ xh.astype(np.float64)
    d = np.abs(yh.astype(np.float64) - ref)
    err = float(np.max(np.where(ref != 0, d / np.where(ref != 0, np.abs(ref), 1.0), d)))
    yo = np.empty(A.m, np.float32)
    O.spmv_plus_times_f32(rp, cv, nz, xh, yo)
    short = np.diff(rp) <= 128
    exact = int(np.count_nonzero(yh[short] == yo[short]))
    return {"rows": int(A.m), "max_rel_err_vs_fp64": err, "rows_le_128_entries": int(short.sum()),
            "rows_le_128_bit_exact_vs_oracle": exact,
            "ok": bool(err <= 1e-5 and exact == int(short.sum()))}


def cpu_baseline_spmv(A, x, budget_s=8.0):
    """csr_spmv_kernel! (plus-times) restated in C (oracle), OpenMP over all host cores,
    on the same graph copied to the host."""
    import numpy as np
    from oracle import oracle as O
    rowptr, colval, nzval = A.rowptr.cpu().numpy(), A.colval.cpu().numpy(), A.nzval.cpu().numpy()
    xh = x.cpu().numpy()
    y = np.zeros(A.m, np.float32)
    O.spmv_plus_times_f32(rowptr, colval, nzval, xh, y)
    times = []
    t_end = time.time() + budget_s
    while (time.time() < t_end or len(times) < 3) and len(times) < 50:
        t0 = time.perf_counter()
        O.spmv_plus_times_f32(rowptr, colval, nzval, xh, y)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    return {"value": round(spmv_bytes(A.n, A.nnz()) / t / 1e9, 3), "unit": "GB/s",
            "cores": O.num_threads(), "kind": "port",
            "sample": "%d full SpMVs over the same R-MAT CSR (median)" % len(times)}


# ---------------------------------------------------------------------------------
# BFS / SSSP workloads (R-MAT scale 24, 4096 x 4096 grid)
# ---------------------------------------------------------------------------------

def search_graph(kind, graph, device):
    """The configured search graphs: R-MAT (Bool pattern for BFS, Int32 weights 1..255
    for shortest paths) or the 4096 x 4096 grid (pattern / Float32 weights [1, 10))."""
    from gpugraphs import generators as gen
    if graph.startswith("rmat"):
        sc = int(graph[4:])
        A = rmat(sc, gen.W_PATTERN if kind == "bfs" else gen.W_INT_1_255, device)
        cfg = "R-MAT scale %d, edge factor 16, symmetrised" % sc + (
            ", Bool pattern" if kind == "bfs" else ", Int32 weights 1..255")
    else:
        A = gen.grid(4096, 4096, seed=4, wkind=gen.W_PATTERN if kind == "bfs" else gen.W_F32_1_10,
                     device=device)
        cfg = "4096x4096 4-neighbour grid" + (", Bool pattern" if kind == "bfs" else
                                               ", Float32 weights [1,10)")
    return A, cfg


def hop_levels(A, s, device):
    """BFS level count from s on A's pattern (a search's hop eccentricity + 1)."""
    import torch
    import gpugraphs as G
    P = A if A.dtype == torch.bool else G.SparseGPUMatrixCSR(
        A.m, A.n, A.rowptr, A.colval, torch.ones(A.nnz(), dtype=torch.bool, device=device))
    lv = G.bfs_distances(P, int(s))
    return int(lv[lv != I32MAX].max().item()) + 1


def search_parity(A, kind, s, d):
    """One search's result against the oracle's full-size cross-checks: BFS levels
    and CSR parents by frontier BFS, shortest paths by Dijkstra (bit for bit; both
    pinned against the restated reference loops in the CPU tests)."""
    import numpy as np
    import gpugraphs as G
    from oracle import oracle as O
    rp, cv = A.rowptr.cpu().numpy(), A.colval.cpu().numpy()
    t0 = time.perf_counter()
    if kind == "bfs":
        ref, _ = O.bfs_levels_fast(A.n, rp, cv, None, s, symmetric=True)
        lev_ok = bool(np.array_equal(d.cpu().numpy(), ref))
        par = G.bfs_parents(A, s).cpu().numpy()
        par_ok = bool(np.array_equal(par, O.bfs_parents_fast(A.n, rp, cv, s, 1, dist=ref)))
        out = {"source": int(s), "levels_equal": lev_ok, "parents_equal": par_ok,
               "ok": lev_ok and par_ok, "oracle": "frontier BFS; parents from levels (CSR rule)"}
    else:
        ref = O.sssp_dijkstra(A.n, rp, cv, A.nzval.cpu().numpy(), s, symmetric=True)
        got = d.cpu().numpy()
        ok = bool(np.array_equal(got.view(np.int32), ref.view(np.int32)))
        out = {"source": int(s), "distances_equal": ok, "ok": ok,
               "oracle": "Dijkstra in the distance type (%s)" % got.dtype}
    out["check_s"] = round(time.perf_counter() - t0, 1)
    return out


def run_search(args, kind, graph):
    import numpy as np
    import torch
    import gpugraphs as G

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    A, cfg = search_graph(kind, graph, device)
    n, nnz = A.n, A.nnz()
    src = sources_for(A, 64, 11)
    run = (lambda i: G.bfs_distances(A, int(src[i % len(src)]))) if kind == "bfs" else \
        (lambda i: G.shortest_path(A, int(src[i % len(src)])))
    d0 = run(0)
    if kind == "bfs":
        mcc = reached_edges(A, d0)
    else:
        unreached = torch.isinf(d0) if d0.is_floating_point() else (d0 == I32MAX)
        mcc = reached_edges(A, torch.where(unreached, I32MAX, 0).to(torch.int32))
    clk = ClockSampler(local)
    clk.start()
    ts = time_host(run, args.steps, warmup=max(args.warmup, 3))
    clocks = clk.stop()
    t = sum(ts) / len(ts)
    value = mcc / t / 1e9
    B = (bfs_bytes if kind == "bfs" else sssp_bytes)(n, nnz)
    peak, peak_kind = peak_hbm()
    # e2e: every query's result copied back to pinned host memory; the copy of query i
    # runs on a side stream while query i + 1 searches (two host buffers)
    host = [torch.empty(n, dtype=d0.dtype).pin_memory() for _ in range(2)]
    side = torch.cuda.Stream(device)
    cur_s = torch.cuda.current_stream(device)

    def e2e_run(k):
        t0 = time.perf_counter()
        for i in range(k):
            d = run(i)
            side.wait_stream(cur_s)
            with torch.cuda.stream(side):
                host[i & 1].copy_(d, non_blocking=True)
                d.record_stream(side)
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / k

    e2e_run(1)
    e2e = mcc / e2e_run(max(3, args.steps // 2)) / 1e9
    out = {
        "metric": "%s GTEPS (%s)" % ("BFS" if kind == "bfs" else "Bellman-Ford", cfg),
        "value": round(value * ws, 3), "unit": "GTEPS", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": round(t * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32" if kind == "bfs" else str(d0.dtype).split(".")[-1],
        "data": "synthetic (seeded generator on the device), %d seeded sources" % len(src),
        "config": {"workload": "%s_%s" % (kind, graph), "n": n, "nnz": nnz, "m_cc": mcc,
                   "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "achieved": round(B / t / 1e9, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(B / t / 1e9 / peak, 4), "traffic": traffic_from_profiles("%s_%s" % (kind, graph)),
                     "peak_kind": peak_kind, "algorithmic_bytes": B},
        "e2e": {"value": round(e2e * ws, 3), "unit": "GTEPS", "h2d_bytes_per_step": 8,
                "d2h_bytes_per_step": n * d0.element_size(),
                "schedule": "each query's result copied to pinned host memory on a side stream "
                            "while the next query searches"},
        "gpu_launches": None,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline_search(A, kind, int(src[0]), mcc,
                                                  hop_levels(A, src[0], device))
    if rank == 0 and not args.no_parity:
        out["parity"] = search_parity(A, kind, int(src[0]), d0)
    if rank == 0:
        print(json.dumps(out), flush=True)


def secondary_large(args, device, parity, rank):
    """The configurations beyond the scale-22 graph, each measured briefly: plus-times
    SpMV on R-MAT scale 24 (the 70%-of-HBM target configuration), BFS and shortest
    paths on R-MAT scale 24 and on the 4096 x 4096 grid, and a summary of the serving
    loop.  One search of each large graph is checked against the oracle."""
    import torch
    import gpugraphs as G
    from gpugraphs import generators as gen
    out = {}
    t0 = time.time()
    A = rmat(24, gen.W_U01_F32, device)
    x = gen.uniform_vector(A.n, seed=2, device=device)
    m = measure_spmv(A, x, 10, 3, device, 1, sample_clocks=False)
    out["spmv_csr_rmat24"] = {
        "n": A.n, "nnz": A.nnz(), "ms": round(m["per_step_ms"], 4), "gbs": round(m["value"], 1),
        "kernel_ms": round(m["kernel_ms"], 4), "kernel_gbs": round(m["achieved"], 1),
        "frac": round(m["frac"], 4), "peak": m["peak"], "e2e_gbs": round(m["e2e"], 1),
        "layout": G.spmv_layout(A), "hub_rows_from_windows": G.spmv_hub_rows(A)}
    del A, x, m
    torch.cuda.empty_cache()
    for kind, graph, reps, budget in (("bfs", "rmat24", 8, 40), ("sssp", "rmat24", 4, 4),
                                      ("bfs", "grid4096", 4, 40), ("sssp", "grid4096", 3, 6)):
        A, cfg = search_graph(kind, graph, device)
        src = sources_for(A, 64, 11)
        run = (lambda i: G.bfs_distances(A, int(src[i % len(src)]))) if kind == "bfs" else \
            (lambda i: G.shortest_path(A, int(src[i % len(src)])))
        d0 = run(0)
        unreached = torch.isinf(d0) if d0.is_floating_point() else (d0 == I32MAX)
        mcc = reached_edges(A, torch.where(unreached, I32MAX, 0).to(torch.int32))
        ts = time_host(run, reps, warmup=2)
        t = sum(ts) / len(ts)
        lv = hop_levels(A, src[0], device)
        B = (bfs_bytes if kind == "bfs" else sssp_bytes)(A.n, A.nnz())
        rec = {"gteps": round(mcc / t / 1e9, 3), "ms": round(t * 1e3, 3), "searches": reps,
               "levels_from_first_source": lv, "n": A.n, "nnz": A.nnz(), "m_cc": mcc,
               "gbs_algorithmic": round(B / t / 1e9, 1), "graph": cfg}
        if rank == 0 and not args.no_cpu:
            rec["cpu_baseline"] = cpu_baseline_search(A, kind, int(src[0]), mcc, lv, budget=budget)
        if rank == 0 and not args.no_parity and (kind, graph) in (("bfs", "rmat24"), ("sssp", "grid4096")):
            parity["%s_%s" % (kind, graph)] = search_parity(A, kind, int(src[0]), d0)
        out["%s_%s" % (kind, graph)] = rec
        del A, d0, run
        torch.cuda.empty_cache()
    out["serve_summary"] = serve_summary(device)
    torch.cuda.empty_cache()
    mgm = multigraph_measure(device, 1000, 10, 3, parity=rank == 0 and not args.no_parity)
    if "parity" in mgm:
        parity["multigraph_1000"] = mgm.pop("parity")
    out["multigraph_1000"] = mgm
    out["large_configs_s"] = round(time.time() - t0, 1)
    return out


def cpu_baseline_search(A, kind, s, mcc, levels_full, budget=40):
    """The reference algorithm (level-synchronous masked-SpMV BFS, bfs.jl:31-73, or
    Jacobi Bellman-Ford, shortest_path.jl:34-83, restated in C with OpenMP) from one
    source.  At most `budget` levels / rounds run; a longer search is scaled to
    `levels_full` levels (the BFS level count of this source -- exact for BFS, a lower
    bound on the Jacobi round count, which favours the CPU)."""
    from oracle import oracle as O
    rp, cv, nz = A.rowptr.cpu().numpy(), A.colval.cpu().numpy(), A.nzval.cpu().numpy()
    t0 = time.perf_counter()
    if kind == "bfs":
        _, lv = O.bfs_levels(A.n, rp, cv, nz, s, max_levels=budget)
        done = lv > 0
        ran = abs(lv)
    else:
        _, lv = O.sssp(A.n, rp, cv, nz, [s], max_rounds=budget)
        done = lv > 0
        ran = budget if lv < 0 else lv
    t = time.perf_counter() - t0
    if done:
        sample = "whole search from 1 source (%d %s)" % (ran, "levels" if kind == "bfs" else "rounds")
    else:
        t = t / ran * levels_full
        sample = ("first %d %s from 1 source, time scaled to %d levels" %
                  (ran, "levels" if kind == "bfs" else "Jacobi rounds", levels_full))
    return {"value": round(mcc / t / 1e9, 5), "unit": "GTEPS", "cores": O.num_threads(),
            "kind": "port", "sample": sample}


# ---------------------------------------------------------------------------------
# SpMM: R-MAT scale 22, 32 row-major dense columns
# ---------------------------------------------------------------------------------

def run_batch(args):
    """Batched searches on R-MAT scale 22: 256 BFS sources as one bit-packed search and
    256 Int32 shortest-path sources as eight 32-column groups run at once, against the
    same sources one at a time (queries/s, results compared column by column)."""
    import statistics
    import torch
    import gpugraphs as G
    from gpugraphs import generators as gen
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    P = rmat(22, gen.W_PATTERN, device)
    src = sources_for(P, 256, 7)
    steps = max(1, min(args.steps, 5))
    tb = time_host(lambda i: G.bfs_distances_batch(P, src), steps, warmup=max(args.warmup, 1))
    ts = time_host(lambda i: G.bfs_distances(P, int(src[i % 16])), 16)
    Db = G.bfs_distances_batch(P, src)
    same_bfs = all(bool((Db[:, q] == G.bfs_distances(P, int(src[q]))).all()) for q in range(0, 256, 37))
    del P
    W = rmat(22, gen.W_INT_1_255, device)
    tsb = time_host(lambda i: G.shortest_path(W, src), steps, warmup=1)
    tss = time_host(lambda i: G.shortest_path(W, int(src[i % 16])), 6)
    Ds = G.shortest_path(W, src)
    same_sssp = all(bool((Ds[:, q] == G.shortest_path(W, int(src[q]))).all()) for q in (0, 37, 100, 255))
    qb, q1 = 256 / statistics.median(tb), 1 / statistics.median(ts)
    qsb, qs1 = 256 / statistics.median(tsb), 1 / statistics.median(tss)
    out = {
        "metric": "batched BFS queries/s (256 sources, R-MAT scale 22)", "value": round(qb, 1),
        "unit": "queries/s", "n_gpus": 1, "steps": steps, "warmup": max(args.warmup, 1),
        "ms_per_step": round(statistics.median(tb) * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded R-MAT generator on the device)",
        "config": {"workload": "batch_rmat22", "bfs_sources": 256, "sssp_sources": 256},
        "bfs": {"batch_queries_per_s": round(qb, 1), "single_queries_per_s": round(q1, 1),
                "speedup": round(qb / q1, 2), "equal_to_single": same_bfs},
        "sssp_int32": {"batch_queries_per_s": round(qsb, 1), "single_queries_per_s": round(qs1, 1),
                       "speedup": round(qsb / qs1, 2), "equal_to_single": same_sssp},
    }
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_spmm(args):
    """plus-times Float32 SpMM Y = A X on the R-MAT scale-22 CSR with X of n x 32
    row-major uniform [0,1) (the SpMM half of the scale-22 configuration).  A step is
    one gpu_spmm_ call; algorithmic bytes 4(n+1) + 8 nnz + 4nk (X once) + 4nk (Y)."""
    import torch
    import gpugraphs as G
    from gpugraphs import generators as gen
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    A = rmat(22, gen.W_U01_F32, device)
    n, nnz, k = A.n, A.nnz(), 32
    X = torch.rand((n, k), dtype=torch.float32, device=device)
    Y = torch.empty((n, k), dtype=torch.float32, device=device)
    clk = ClockSampler(local)
    clk.start()
    ms = time_steps(lambda: G.gpu_spmm_(Y, A, X), args.steps, warmup=max(args.warmup, 3))
    clocks = clk.stop()
    from gpugraphs.tracing import launch_trace
    with launch_trace(device) as tr:
        for _ in range(args.steps):
            G.gpu_spmm_(Y, A, X)
    B = 4 * (n + 1) + 8 * nnz + 4 * n * k * 2
    peak, peak_kind = peak_hbm()
    out = {
        "metric": "SpMM GB/s (plus-times Float32, CSR, R-MAT scale 22, 32 row-major columns)",
        "value": round(ws * B / ms / 1e6, 2), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded R-MAT generator on the device)",
        "config": {"workload": "spmm_rmat22", "n": n, "nnz": nnz, "k": k, "layout": "row-major",
                   "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "achieved": round(B / ms / 1e6, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(B / ms / 1e6 / peak, 4), "traffic": None, "peak_kind": peak_kind,
                     "algorithmic_bytes": B, "gathered_bytes": nnz * k * 4},
        "e2e": None, "gpu_launches": tr.launches, "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_sparse_vector(args):
    """SpMSpV over 1% of the vertices of R-MAT scale 22 (plus-times Float32), e-wise min
    and reduce over 2^28 Float32 values: the sparse-vector, e-wise and reduce entry
    points on their own.  The line's value is the SpMSpV's algorithmic GB/s."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    from gpugraphs import generators as gen
    A = rmat(22, gen.W_U01_F32, device)
    clk = ClockSampler(local)
    clk.start()
    sec = secondary_sparse_vector(device, A)
    clocks = clk.stop()
    sv = sec["spmspv_rmat22_1pct"]
    peak, peak_kind = peak_hbm()
    out = {
        "metric": "SpMSpV GB/s (plus-times Float32, x on 1% of R-MAT scale 22's vertices)",
        "value": sv["gbs_algorithmic"], "unit": "GB/s", "n_gpus": ws, "steps": 10, "warmup": 1,
        "ms_per_step": sv["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded R-MAT generator on the device)",
        "config": {"workload": "sparse_vector_rmat22", "n": A.n, "nnz": A.nnz(),
                   "x_nnz": sv["x_nnz"]},
        "roofline": {"bound": "hbm", "achieved": sv["gbs_algorithmic"], "peak": peak, "unit": "GB/s",
                     "frac": round(sv["gbs_algorithmic"] / peak, 4), "traffic": None,
                     "peak_kind": peak_kind},
        "e2e": None, "clocks": clocks, "secondary": sec,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------------
# serving: Poisson arrivals over 16 resident graphs, continuous batching
# ---------------------------------------------------------------------------------

class ServeMix:
    """16 resident R-MAT graphs (scales 16..23, one Int32- and one Float32-weighted per
    scale); requests: 1/3 BFS (Int32 graphs), 1/3 shortest paths (any graph), 1/3
    20-step plus-times SpMV iterations (Float32 graphs); graph and source seeded."""

    def __init__(self, device):
        import numpy as np
        from gpugraphs import generators as gen
        self.graphs = []
        for sc in range(16, 24):
            self.graphs.append(rmat(sc, gen.W_INT_1_255, device))
            self.graphs.append(rmat(sc, gen.W_U01_F32, device))
        self.ints = [i for i in range(16) if i % 2 == 0]
        self.flts = [i for i in range(16) if i % 2 == 1]
        self.xs = {g: gen.uniform_vector(self.graphs[g].n, seed=100 + g, device=device)
                   for g in self.flts}
        self.rng = np.random.default_rng(9)

    KINDS = ("bfs", "sssp", "spmv_x20")

    def draw(self):
        rng = self.rng
        kind = int(rng.integers(0, 3))
        if kind == 0:
            g = int(rng.choice(self.ints))
        elif kind == 1:
            g = int(rng.integers(0, 16))
        else:
            g = int(rng.choice(self.flts))
        return kind, g, int(rng.integers(1, self.graphs[g].n + 1))

    def plain(self, nq):
        """The same mix one query at a time through the single-query functions, every
        graph's per-matrix analysis built first: (queries/s, latencies in s)."""
        import torch
        import gpugraphs as G
        for g in range(16):
            for kind in ((0, 1) if g in self.ints else (1, 2)):
                _single(G, self.graphs, self.xs, kind, g, 1)
        torch.cuda.synchronize()
        lat = []
        self.plain_kinds = []
        t0 = time.perf_counter()
        for _ in range(nq):
            kind, g, s = self.draw()
            t1 = time.perf_counter()
            _single(G, self.graphs, self.xs, kind, g, s)
            torch.cuda.synchronize()
            lat.append(time.perf_counter() - t1)
            self.plain_kinds.append(kind)
        return nq / (time.perf_counter() - t0), lat

    def poisson(self, srv, ids, lam, nreq):
        """Open-loop Poisson submissions at rate lam; the server's own submit->result
        latencies give p50 / p99."""
        import numpy as np
        gaps = self.rng.exponential(1.0 / lam, nreq)
        reqs = [self.draw() for _ in range(nreq)]
        t_start = time.perf_counter()
        t_next = t_start
        kind_of = {}
        for i, (kind, g, s) in enumerate(reqs):
            t_next += gaps[i]
            while time.perf_counter() < t_next:
                pass
            if kind == 0:
                rid = srv.submit_bfs(ids[g], s)
            elif kind == 1:
                rid = srv.submit_sssp(ids[g], s)
            else:
                rid = srv.submit_spmv_iter(ids[g], self.xs[g], steps=20)
            kind_of[rid] = kind
        t_sub = time.perf_counter() - t_start
        done = srv.wait(timeout=600)
        t_all = time.perf_counter() - t_start
        lat = np.array(sorted(v[1] for v in done.values()))
        per_kind = {}
        for k, name in enumerate(self.KINDS):
            lk = np.array([v[1] for r, v in done.items() if kind_of.get(r) == k])
            if len(lk):
                per_kind[name] = {"n": int(len(lk)), "p50_ms": round(float(np.percentile(lk, 50)) * 1e3, 3),
                                  "p99_ms": round(float(np.percentile(lk, 99)) * 1e3, 3)}
        return {"lambda": lam, "requests": nreq, "offered_qps": round(nreq / t_sub, 1),
                "qps": round(nreq / t_all, 1), "p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 3),
                "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 3), "per_kind": per_kind}


def serve_summary(device):
    """Serving at a low and a saturating rate (lambda = 1e2 and 1e4 requests/s) against
    the one-query-at-a-time path: queries/s and p50 / p99 latency."""
    import numpy as np
    from gpugraphs.serving import Server
    t0 = time.time()
    mix = ServeMix(device)
    plain_qps, pl = mix.plain(60)
    srv = Server(reserve_bytes=1 << 30, device=device.index or 0)
    ids = [srv.add_graph(A) for A in mix.graphs]
    low = mix.poisson(srv, ids, 1e2, 200)
    high = mix.poisson(srv, ids, 1e4, 2000)
    srv.close()
    pl = np.array(pl)
    pk = np.array(mix.plain_kinds)
    plain_kind = {name: round(float(np.percentile(pl[pk == k], 50)) * 1e3, 3)
                  for k, name in enumerate(mix.KINDS) if (pk == k).any()}
    return {"lambda_1e2": low, "lambda_1e4": high, "plain_p50_ms_per_kind": plain_kind,
            "best_qps": max(low["qps"], high["qps"]),
            "plain": {"qps": round(plain_qps, 1), "p50_ms": round(float(np.percentile(pl, 50)) * 1e3, 3),
                      "p99_ms": round(float(np.percentile(pl, 99)) * 1e3, 3)},
            "speedup_vs_plain": round(max(low["qps"], high["qps"]) / plain_qps, 2),
            "p50_low_load_vs_plain": round(low["p50_ms"] / (float(np.percentile(pl, 50)) * 1e3), 2),
            "mix": "1/3 BFS, 1/3 SSSP, 1/3 SpMV x20 over 16 R-MAT graphs (scales 16..23)",
            "took_s": round(time.time() - t0, 1)}


def run_serve(args):
    """Poisson-rate sweep of the serving loop (ServeMix) and per-kind saturation, against
    the same kind of mix one query at a time through the single-query functions."""
    import numpy as np
    import torch
    import gpugraphs as G
    from gpugraphs.serving import Server

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    mix = ServeMix(device)
    graphs, ints, xs, rng = mix.graphs, mix.ints, mix.xs, mix.rng
    nplain = max(30, args.steps)
    plain_qps, plain_lat = mix.plain(nplain)

    srv = Server(reserve_bytes=1 << 30, device=local)
    ids = [srv.add_graph(A) for A in graphs]
    sweep = []
    clk = ClockSampler(local)
    clk.start()
    for lam in (1e2, 3e2, 1e3, 3e3, 1e4, 3e4, 1e5):
        sweep.append(mix.poisson(srv, ids, lam, int(min(lam * 2.0, 3000))))
    # per kind at saturation (every request submitted at once) against the same kind
    # one query at a time
    per_kind = {}
    for kind, name in ((0, "bfs"), (1, "sssp")):
        pool = ints if kind == 0 else list(range(16))
        reqs = [(int(rng.choice(pool)),) for _ in range(1500)]
        reqs = [(g, int(rng.integers(1, graphs[g].n + 1))) for (g,) in reqs]
        t0 = time.perf_counter()
        for g, s in reqs:
            (srv.submit_bfs if kind == 0 else srv.submit_sssp)(ids[g], s)
        done = srv.wait(timeout=600)
        t_all = time.perf_counter() - t0
        lat = np.array(sorted(v[1] for v in done.values()))
        tp = time.perf_counter()
        for g, s in reqs[:40]:
            _single(G, graphs, xs, kind, g, s)
            torch.cuda.synchronize()
        plain_k = 40 / (time.perf_counter() - tp)
        per_kind[name] = {"served_qps": round(len(reqs) / t_all, 1),
                          "p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 3),
                          "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 3),
                          "plain_qps": round(plain_k, 1),
                          "speedup_vs_plain": round(len(reqs) / t_all / plain_k, 2)}
    clocks = clk.stop()
    st = srv.stats()
    srv.close()
    best = max(sweep, key=lambda r: r["qps"])
    pl = np.array(plain_lat)
    out = {
        "metric": "serving queries/s (BFS / shortest path / 20-step SpMV mix, 16 resident R-MAT graphs)",
        "value": best["qps"] * ws, "unit": "queries/s", "n_gpus": ws, "steps": len(sweep),
        "warmup": 3, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32/f32", "data": "synthetic (seeded R-MAT graphs, seeded Poisson arrivals)",
        "config": {"workload": "serve", "graphs": "R-MAT scales 16..23 x {Int32 1..255, Float32 [0,1)}",
                   "mix": "1/3 BFS, 1/3 SSSP, 1/3 SpMV x20", "l2": "graphs larger than L2 (scales >= 21)"},
        "sweep": sweep,
        "plain_path": {"qps": round(plain_qps, 1), "p50_ms": round(float(np.percentile(pl, 50)) * 1e3, 3),
                       "p99_ms": round(float(np.percentile(pl, 99)) * 1e3, 3), "queries": nplain},
        "speedup_vs_plain": round(best["qps"] / plain_qps, 2),
        "per_kind_saturation": per_kind,
        "server_stats": st,
        "e2e": None, "gpu_launches": None, "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)


def _single(G, graphs, xs, kind, g, s):
    A = graphs[g]
    if kind == 0:
        return G.bfs_distances(A, s)
    if kind == 1:
        return G.shortest_path(A, s)
    import torch
    y = xs[g]
    out = torch.empty_like(y)
    for _ in range(20):
        G.gpu_spmv_(out, A, y)
        y, out = out, y
    return y


# ---------------------------------------------------------------------------------
# many graphs: 1000 Erdos-Renyi graphs in one launch
# ---------------------------------------------------------------------------------

def multigraph_measure(device, ng, steps, warmup, parity=True):
    """1000 symmetric Erdos-Renyi graphs, n = round(10^U[3,6]), average degree U[4,32]
    (seed 2), Float32 values U[0,1).  One plus-times SpMV over all graphs in one launch,
    one BFS and one shortest-path search per graph in one persistent cooperative launch
    each (CUDA graphs), against the same work as one call per graph; with `parity`,
    sampled graphs (every 100th and the last three, whose entry offsets in the
    concatenation pass 2^31) are checked against the oracle."""
    import numpy as np
    import scipy.sparse as sp
    import torch
    import gpugraphs as G
    from gpugraphs import generators as gen
    from gpugraphs.multigraph import MultiGraph

    rng = np.random.default_rng(2)
    ns = np.round(10 ** rng.uniform(3, 6, ng)).astype(np.int64)
    degs = rng.uniform(4, 32, ng)
    t0 = time.time()
    # d / 2 undirected edges per vertex, mirrored: about d stored entries per row
    graphs = [gen.erdos_renyi(int(n), float(d) / 2, seed=1000 + i, wkind=gen.W_U01_F32,
                              symmetric=True, device=device) for i, (n, d) in enumerate(zip(ns, degs))]
    mg = MultiGraph(graphs)
    build_s = time.time() - t0
    N, NNZ = mg.total_n, mg.total_nnz
    x = gen.uniform_vector(N, seed=3, device=device)
    y = torch.empty(N, dtype=torch.float32, device=device)
    ms = time_steps(lambda: mg.spmv(x, y), steps, warmup=max(warmup, 3))
    B = spmv_bytes(N, NNZ) + 8 * (ng + 1)
    xs = mg.split(x)
    ys = [torch.empty_like(v) for v in xs]

    def per_graph():
        for A, xv, yv in zip(graphs, xs, ys):
            G.gpu_spmv_(yv, A, xv)

    ms_loop = time_steps(per_graph, max(3, steps // 4), warmup=1)
    src = [int(rng.integers(1, int(n) + 1)) for n in ns]
    d = torch.empty(N, dtype=torch.int32, device=device)  # fixed buffer: the CUDA graph is reused
    mg.bfs(src, d)
    torch.cuda.synchronize()
    tb = time_host(lambda i: mg.bfs(src, d), max(3, steps // 4), warmup=1)
    t_bfs = statistics.median(tb)
    reached = int((d != I32MAX).sum().item())
    # traversed edges: entries of reached vertices, halved (symmetric graphs)
    mcc = 0
    for A, dv in zip(graphs, mg.split(d)):
        mcc += reached_edges(A, dv)
    # the one-call-per-graph path: bfs_distances needs the Bool pattern of each graph
    pats = [G.SparseGPUMatrixCSR(A.m, A.n, A.rowptr, A.colval,
                                 torch.ones(A.nnz(), dtype=torch.bool, device=device)) for A in graphs]
    tl = time_host(lambda i: [G.bfs_distances(P, s) for P, s in zip(pats, src)], 1, warmup=1)
    same_bfs = all(torch.equal(dv, G.bfs_distances(P, s))
                   for P, s, dv in list(zip(pats, src, mg.split(d)))[:: max(1, ng // 20)])
    del pats
    t_loop = statistics.median(tl)
    dsp = torch.empty(N, dtype=torch.float32, device=device)
    mg.sssp(src, dsp)
    torch.cuda.synchronize()
    tsp = statistics.median(time_host(lambda i: mg.sssp(src, dsp), 2, warmup=0))
    out = {"graphs": ng, "total_n": N, "total_nnz": NNZ, "build_s": round(build_s, 1),
           "spmv_ms": round(ms, 4), "spmv_gbs": round(B / ms / 1e6, 2), "spmv_bytes": B,
           "spmv_per_graph_ms": round(ms_loop, 3), "spmv_speedup_of_one_launch": round(ms_loop / ms, 2),
           "bfs_ms": round(t_bfs * 1e3, 3), "bfs_gteps": round(mcc / t_bfs / 1e9, 2),
           "bfs_levels": mg.last_levels, "bfs_reached": reached,
           "bfs_per_graph_calls_ms": round(t_loop * 1e3, 1),
           "bfs_speedup_of_one_launch": round(t_loop / t_bfs, 2), "bfs_equal_to_per_graph": same_bfs,
           "sssp_ms": round(tsp * 1e3, 3), "sssp_rounds": mg.last_rounds}
    if parity:
        from oracle import oracle as O
        t1 = time.time()
        idx = sorted(set(range(0, ng, 100)) | {ng - 3, ng - 2, ng - 1})
        offs = [sum(A.nnz() for A in graphs[:g]) for g in (idx[-3], idx[-1])]
        ok_bfs = ok_sp = ok_mv = True
        worst = 0.0
        yl, dl, sl = mg.split(y), mg.split(d), mg.split(dsp)
        for g in idx:
            A = graphs[g]
            rp, cv, nz = A.rowptr.cpu().numpy(), A.colval.cpu().numpy(), A.nzval.cpu().numpy()
            lv, _ = O.bfs_levels_fast(A.n, rp, cv, None, src[g], symmetric=True)
            ok_bfs &= bool(np.array_equal(dl[g].cpu().numpy(), lv))
            ref = O.sssp_dijkstra(A.n, rp, cv, nz, src[g], symmetric=True)
            ok_sp &= bool(np.array_equal(sl[g].cpu().numpy().view(np.int32), ref.view(np.int32)))
            M = sp.csr_matrix((nz.astype(np.float64), cv - 1, rp - 1), shape=(A.n, A.n))
            r64 = M @ xs[g].cpu().numpy().astype(np.float64)
            dd = np.abs(yl[g].cpu().numpy().astype(np.float64) - r64)
            err = float(np.max(np.where(r64 != 0, dd / np.where(r64 != 0, np.abs(r64), 1), dd))) if A.n else 0.0
            worst = max(worst, err)
        ok_mv = worst <= 1e-5
        out["parity"] = {"graphs_checked": len(idx), "entry_offset_of_last_checked": offs[-1],
                         "bfs_levels_equal": ok_bfs, "sssp_equal": ok_sp,
                         "spmv_max_rel_err_vs_fp64": worst, "ok": bool(ok_bfs and ok_sp and ok_mv),
                         "oracle": "frontier BFS, Float32 Dijkstra, FP64 SpMV", "check_s": round(time.time() - t1, 1)}
    return out


def run_multigraph(args):
    """The many-graph workload (multigraph_measure) as one JSON line."""
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    clk = ClockSampler(local)
    clk.start()
    m = multigraph_measure(device, args.graphs, args.steps, args.warmup,
                           parity=rank == 0 and not args.no_parity)
    clocks = clk.stop()
    peak, peak_kind = peak_hbm()
    out = {
        "metric": "multi-graph SpMV GB/s (1000 Erdos-Renyi graphs, one launch)",
        "value": round(ws * m["spmv_gbs"], 2), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": m["spmv_ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Erdos-Renyi generator on the device)",
        "config": {"workload": "multigraph", "graphs": m["graphs"], "total_n": m["total_n"],
                   "total_nnz": m["total_nnz"], "n": "round(10^U[3,6])", "avg_degree": "U[4,32]",
                   "build_s": m["build_s"],
                   "l2": "inputs larger than L2 (%.1f GB CSR)" % ((4 * m["total_n"] + 8 * m["total_nnz"]) / 1e9)},
        "roofline": {"bound": "hbm", "achieved": m["spmv_gbs"], "peak": peak, "unit": "GB/s",
                     "frac": round(m["spmv_gbs"] / peak, 4), "traffic": None, "peak_kind": peak_kind,
                     "algorithmic_bytes": m["spmv_bytes"]},
        "detail": m, "e2e": None, "gpu_launches": args.steps, "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------------
# reference arm
# ---------------------------------------------------------------------------------

def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    import numpy as np
    from oracle import oracle as O
    t0 = time.time()
    n = 1 << 22
    s, d, w = O.gen_rmat(22, RMAT["edge_factor"] * n, RMAT["a"], RMAT["b"], RMAT["c"], RMAT["seed"], 1)
    rowptr, colval, nzval = O.coo_to_csr(n, s, d, w, symmetrize=True, drop_loops=True)
    del s, d, w
    x = O.gen_uniform_f32(n, 2)
    y = np.zeros(n, np.float32)
    build_s = time.time() - t0
    for _ in range(max(args.warmup, 1)):
        O.spmv_plus_times_f32(rowptr, colval, nzval, x, y)
    times = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        O.spmv_plus_times_f32(rowptr, colval, nzval, x, y)
        times.append(time.perf_counter() - t1)
    per = sum(times) / len(times)
    B = spmv_bytes(n, len(colval))
    val = B / per / 1e9
    out = {
        "impl": "reference",
        "metric": "SpMV GB/s (plus-times Float32, CSR, R-MAT scale 22)",
        "value": round(val, 3), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 1), "ms_per_step": round(per * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded R-MAT generator, host copy)",
        "config": {"workload": "spmv_csr_rmat22", "n": n, "nnz": int(len(colval)), "format": "CSR",
                   "semiring": "(mul, add, second)"},
        "cpu_baseline": {"value": round(val, 3), "unit": "GB/s", "cores": O.num_threads(),
                         "kind": "port",
                         "sample": "%d full SpMVs (C restatement of csr_spmv_kernel!, OpenMP); "
                                   "host graph build %.1f s untimed" % (args.steps, build_s)},
        "e2e": {"value": round(val, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="spmv_csr_rmat22")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-secondary", action="store_true", help="headline SpMV only")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the checks of this run's results against the oracle")
    ap.add_argument("--graphs", type=int, default=1000, help="graph count of --workload multigraph")
    ap.add_argument("--sell-variant", default=None, choices=["registers", "bulk_copy", "hub_windows"],
                    help="SpMV workloads: kernel variant over the SELL-32 copy (default: built-in)")
    ap.add_argument("--layout", default=None, choices=["sell", "window_tiles"],
                    help="spmv workloads: run this plus-times layout instead of the built-in choice")
    ap.add_argument("--hot-cols", type=int, default=0,
                    help="SpMV workloads: x values staged in shared memory (default: built-in)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "spmv_csr_rmat22":
        run_spmv_rmat(args, 22)
    elif args.workload == "spmv_csr_rmat24":
        run_spmv_rmat(args, 24)
    elif args.workload in ("bfs_rmat24", "sssp_rmat24", "bfs_grid4096", "sssp_grid4096",
                           "bfs_rmat22", "sssp_rmat22"):
        kind, graph = args.workload.split("_")
        if args.steps == 50:
            args.steps = 8
        run_search(args, kind, graph)
    elif args.workload == "batch_rmat22":
        run_batch(args)
    elif args.workload == "spmm_rmat22":
        run_spmm(args)
    elif args.workload == "sparse_vector_rmat22":
        run_sparse_vector(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "multigraph":
        run_multigraph(args)
    else:
        raise SystemExit("unknown workload %s" % args.workload)


if __name__ == "__main__":
    main()
