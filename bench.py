"""Benchmark of the semiring SpMV hot path on one GB300 (N replicas under torchrun).

Default workload: plus-times Float32 SpMV over the CSR of an R-MAT scale-22 graph
(a=0.57, b=0.19, c=0.19, edge factor 16, symmetrised, self-loops removed, values
uniform [0,1)), x uniform [0,1) -- the SpMV half of the R-MAT scale-22 config.  A
step is one gpu_spmv! over the whole matrix.  `value` is GB/s of algorithmic bytes
4(n+1) + 8 nnz + 4n (x) + 4n (y) with all inputs resident in HBM (the matrix, ~1 GB,
is larger than L2); `e2e` times the same call through the public API with x in
pinned host memory copied in and y copied out every step.

--impl reference times the reference algorithm's CPU path (the C restatement of
csr_spmv_kernel!, OpenMP over every host core) on the same graph built on the host.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                       [--workload NAME]
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


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def traffic_from_profiles(workload):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary
    (profiles/traffic.txt: `workload kernel bytes_per_launch` lines), else None."""
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
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

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
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ---------------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------------

def spmv_bytes(n, nnz):
    return 4 * (n + 1) + 8 * nnz + 4 * n + 4 * n


def build_rmat22(device):
    from gpugraphs import generators as gen
    A = gen.rmat(22, RMAT["edge_factor"], RMAT["a"], RMAT["b"], RMAT["c"], seed=RMAT["seed"],
                 wkind=gen.W_U01_F32, device=device)
    x = gen.uniform_vector(A.n, seed=2, device=device)
    return A, x


def run_ours(args):
    import torch
    import torch.distributed as dist

    import gpugraphs as G

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=device)
    A, x = build_rmat22(device)
    n, nnz = A.n, A.nnz()
    y = torch.zeros(n, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device)

    def step():
        G.gpu_spmv_(y, A, x)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    clk = ClockSampler(local)
    clk.start()
    time.sleep(0.3)  # let the sampler see the start of the timed region
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    ms = ev0.elapsed_time(ev1)
    # hold the clock sampler over a longer window of the same work
    t_end = time.time() + 1.0
    while time.time() < t_end:
        for _ in range(50):
            step()
        torch.cuda.synchronize()
    clocks = clk.stop()
    if ws > 1:
        t = torch.tensor([ms], device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    per_step_ms = ms / args.steps
    B = spmv_bytes(n, nnz)
    value = ws * B / (per_step_ms * 1e-3) / 1e9

    # kernel-level roofline: average launch duration of the SpMV kernel (one per step)
    achieved = B / (per_step_ms * 1e-3) / 1e9
    peak, peak_kind = peak_hbm()
    traffic = traffic_from_profiles("spmv_csr_rmat22")

    # e2e through the public API with host buffers
    xh = x.cpu().pin_memory()
    yh = torch.empty(n, dtype=torch.float32).pin_memory()
    xd = torch.empty_like(x)
    for _ in range(3):
        xd.copy_(xh, non_blocking=True)
        G.gpu_spmv_(y, A, xd)
        yh.copy_(y, non_blocking=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        xd.copy_(xh, non_blocking=True)
        G.gpu_spmv_(y, A, xd)
        yh.copy_(y, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e_ms_t = torch.tensor([e2e_ms], device=device)
    if ws > 1:
        dist.all_reduce(e2e_ms_t, op=dist.ReduceOp.MAX)
    e2e_val = ws * B / (float(e2e_ms_t.item()) * 1e-3) / 1e9

    # parity spot check of this run's output against an FP64 product on 4096 rows
    rows = torch.arange(0, n, max(1, n // 4096), device=device)[:4096]
    ok = spot_check(A, x, y, rows)

    cpu = cpu_baseline(A, x) if (rank == 0 and not args.no_cpu) else None
    out = {
        "metric": "SpMV GB/s (plus-times Float32, CSR, R-MAT scale 22)",
        "value": round(value, 2), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": round(per_step_ms, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded R-MAT generator on the device)",
        "config": {"workload": "spmv_csr_rmat22", "n": n, "nnz": nnz, "format": "CSR",
                   "semiring": "(mul, add, second)", "l2": "inputs larger than L2 (CSR %.2f GB)" % (
                       (4 * (n + 1) + 8 * nnz) / 1e9), "parallelism": "replicas" if ws > 1 else "single"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "peak_kind": peak_kind, "algorithmic_bytes": B},
        "e2e": {"value": round(e2e_val, 2), "unit": "GB/s", "h2d_bytes_per_step": 4 * n,
                "d2h_bytes_per_step": 4 * n},
        "gpu_launches": args.steps,
        "clocks": clocks,
        "parity_spot_check": ok,
    }
    if cpu is not None:
        out["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(out), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def spot_check(A, x, y, rows):
    import numpy as np
    import torch
    rp = A.rowptr.cpu().numpy().astype(np.int64)
    r = rows.cpu().numpy()
    cv = A.colval
    nz = A.nzval
    xs = x.double()
    worst = 0.0
    for i in r:
        lo, hi = rp[i] - 1, rp[i + 1] - 1
        if hi == lo:
            ref = 0.0
        else:
            idx = torch.arange(lo, hi, device=x.device)
            ref = float((nz[idx].double() * xs[cv[idx].long() - 1]).sum())
        got = float(y[i])
        if ref != 0:
            worst = max(worst, abs(got - ref) / abs(ref))
        elif got != 0:
            worst = max(worst, abs(got))
    return {"rows": int(len(r)), "max_rel_err_vs_fp64": worst, "ok": worst <= 1e-5}


def cpu_baseline(A, x, budget_s=10.0):
    """The reference's csr_spmv_kernel! restated in C (oracle), OpenMP over all host
    cores, timed on the same graph copied to the host."""
    import numpy as np
    from oracle import oracle as O
    rowptr = A.rowptr.cpu().numpy()
    colval = A.colval.cpu().numpy()
    nzval = A.nzval.cpu().numpy()
    xh = x.cpu().numpy()
    y = np.zeros(A.m, np.float32)
    O.spmv_plus_times_f32(rowptr, colval, nzval, xh, y)  # warm-up
    times = []
    t_end = time.time() + budget_s
    while time.time() < t_end or len(times) < 3:
        t0 = time.perf_counter()
        O.spmv_plus_times_f32(rowptr, colval, nzval, xh, y)
        times.append(time.perf_counter() - t0)
        if len(times) >= 50:
            break
    t = statistics.median(times)
    B = spmv_bytes(A.n, A.nnz())
    return {"value": round(B / t / 1e9, 3), "unit": "GB/s", "cores": O.num_threads(),
            "kind": "port", "sample": "%d full SpMVs over the same R-MAT s22 CSR (median)" % len(times)}


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
    cores = O.num_threads()
    out = {
        "impl": "reference",
        "metric": "SpMV GB/s (plus-times Float32, CSR, R-MAT scale 22)",
        "value": round(val, 3), "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 1), "ms_per_step": round(per * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded R-MAT generator, host copy)",
        "config": {"workload": "spmv_csr_rmat22", "n": n, "nnz": int(len(colval)), "format": "CSR",
                   "semiring": "(mul, add, second)"},
        "cpu_baseline": {"value": round(val, 3), "unit": "GB/s", "cores": cores, "kind": "port",
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
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
