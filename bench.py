"""Benchmark: fp64 Jacobi-PCG time-to-tolerance on the 27-point 160^3
variable-coefficient diffusion system, one GB300 per rank.

A step is one complete solve from x0 = 0 to ||r|| <= 1e-10 ||b|| (recursive
residual, the xJPCG stop rule).  The headline metric is solves/s (= 1 /
time-to-tolerance per GPU, summed over ranks; ranks are independent replicas:
the path has no data exchange).

  value  inputs resident in HBM: xJPCG_gbSolveDevice on the stored matrix,
         device-timed with CUDA events on the library's stream.
  e2e    the reference-facing call xJPCG_cooSolver(MODE_DEFAULT) from pinned
         host COO arrays: H2D copies, COO->CSR conversion, SpMV layouts and
         the tuner's choice (timed on the first call, reused while the
         structure fingerprint matches), the solve and the D2H copy of x
         inside the timed region; W untimed calls first, as for value.
  roofline  the tuner's SpMV timed alone (20 launches) against the measured
         HBM copy bandwidth, with its fraction of the FP64 issue rate this
         GPU measured in the same run (xJPCG_gbDiagFp64Rate); other_layouts
         times the int16-offset and int32-column sliced layouts the same way.
  cpu_baseline  one complete oracle solve of the same system on all host
         cores (rank 0, N = 1).
  extras (rank 0; --no-extras skips them): mixed vs fp64 on 160^3 and on
         the Zipf 2M system, with the FP32 SpMV's roofline; the 4,096-system
         batch in both precisions; the 96^3 adjoint; the device time of the
         signature exporter on the bench matrix.  Each extra carries the
         oracle's CPU time for the same work on all host cores.  A compact
         "summary" of the extras is the line's last key.

``--impl reference`` times the oracle (the C/OpenMP restatement of the
reference's JPCG; the reference itself only runs on an Alveo U280) on the
host cores: every step, warm-up included, is one complete solve of the same
system from x0 = 0 to the same tolerance.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = {"workload": "jpcg_fp64_diffusion27", "grid": "160^3", "n": 4096000, "nnz": 109215352,
            "stencil": "27-point variable-coefficient diffusion, log-normal(0,1.5) conductances, seed 1",
            "tol": 1e-10, "max_iter": 20000, "precond": "jacobi", "index": "int32", "dtype": "f64",
            "l2": "inputs larger than L2 (matrix 1.3 GB)"}
METRIC = "fp64 JPCG time-to-1e-10 relative residual, 27-pt 160^3 (solves/s = 1/time-to-tol)"
# Nominal FP64 issue rate of GB300 (1.25 TFLOP/s fp64: 2 DFMA per clock per SM
# at 2.07 GHz on 152 SMs), reported beside the rate measured in the run.
FP64_DFMA_NOMINAL = 152 * 2 * 2.07e9


def bench_config(world: int) -> dict:
    """The workload description both arms print as `config`."""
    return dict(WORKLOAD, parallelism="replicas" if world > 1 else "single")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nx", type=int, default=160)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the mixed-precision, batched and adjoint measurements")
    ap.add_argument("--profile", choices=["spmv", "solve", "mixed", "batched", "adjoint", "export", "fp64"],
                    default=None,
                    help="profiling driver for ncu: set the matrix, then run --reps plain SpMVs "
                         "(spmv), one resident fp64 solve (solve) or one mixed solve (mixed); or one batched "
                         "solve of --systems systems (batched); or the adjoint solve and gradients on "
                         "--nx^3 (adjoint); or the signature export of the matrix (export); or the FP64 "
                         "issue-rate probe at several lengths (fp64, prints its rates); no timing line")
    ap.add_argument("--systems", type=int, default=4096)
    ap.add_argument("--workload", choices=["diffusion27", "zipf"], default="diffusion27",
                    help="matrix of --profile: diffusion27(--nx) or the 2M-row Zipf SPD system")
    ap.add_argument("--reps", type=int, default=4)
    ap.add_argument("--zipf-n", type=int, default=2_000_000,
                    help="rows of the Zipf SPD system of --profile --workload zipf")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Ranks:
    """The timing protocol across ranks: a barrier on both sides of the timed
    region and the maximum of the per-rank times.  The GPU arm runs it over
    NCCL with CUDA tensors; with a gloo group it uses CPU tensors."""

    def __init__(self, world: int, device: str):
        self.world = world
        self.device = device

    def barrier(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.barrier()

    def max(self, v: float) -> float:
        if self.world == 1:
            return v
        import torch
        import torch.distributed as dist
        t = torch.tensor([v], dtype=torch.float64, device=self.device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())


def replicas_value(world: int, steps: int, t_max: float) -> float:
    """Whole-job throughput of independent replicas: every rank ran `steps`
    steps, the slowest in t_max seconds."""
    return world * steps / t_max


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
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
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(layout):
    """DRAM bytes per SpMV launch of `layout` from the committed ncu summary
    (or None when no capture of that kernel is committed)."""
    p = os.path.join(ROOT, "profiles", "spmv_diffusion27_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f).get(layout)
        if d:
            return d.get("dram_bytes_per_launch_full"), d.get("source", p)
    return None, None


def run_profile(args):
    """Profiling driver: the matrix is set through xJPCG_cooSolver (maxIter 0),
    then --reps plain SpMVs (xJPCG_gbSpmv on device vectors), one resident
    solve (xJPCG_gbSolveDevice) or one mixed solve (xJPCG_gbMixedSolve).
    XJPCG_SPMV_LANES forces a layout and skips the tuner's launches."""
    import torch
    import hpc_gb300 as X
    from hpc_gb300 import workloads as W
    if args.profile == "fp64":
        with X.JPCG() as h:
            for iters in (4096, 16384, 65536):
                rate, ms = h.fp64_rate(iters)
                print("fp64 probe iters=%d: %.3f ms, %.1f G DFMA/s" % (iters, ms, rate / 1e9), flush=True)
        return
    if args.profile == "batched":
        systems = W.batched_stencils(count=args.systems, seed=3)
        h = X.JPCG()
        for prec in (0, 1):
            st, _, res = h.batch_solve(systems, 20000, 1e-10, precision=prec)
            print("batched precision=%d status=%d converged=%d" % (prec, st, int(np.sum(res["status"] == 0))),
                  flush=True)
        h.close()
        return
    if args.profile == "adjoint":
        prob = W.adjoint_problem(args.nx, seed=4)
        n = args.nx ** 3
        s = W.assemble_edges(n, prob.edge_i, prob.edge_j, np.exp(prob.theta), W.ghost_diagonal7(prob.shape, prob.ghost))
        h = X.JPCG()
        r = h.csr_solve(n, s.rowptr, s.col, s.val, s.diag, prob.b, 20000, 1e-12)
        st, lam, grad, it, res = h.adjoint(r.x - 0.5 * r.x, s.diag, 20000, 1e-12, grad_a=True)
        g = h.edge_grad(prob.edge_i, prob.edge_j, np.exp(prob.theta))
        print("adjoint forward=%d adjoint=%d status=%d" % (r.iters, it, st), flush=True)
        h.close()
        return
    sysm = W.diffusion27(args.nx) if args.workload == "diffusion27" else W.zipf_spd(args.zipf_n, seed=2)
    rows, cols, vals = sysm.coo()
    h = X.JPCG()
    r = h.coo_solve(sysm.n, rows, cols, vals, sysm.diag, sysm.b, 0, 1e-10)
    inf = h.info()
    print("matrix n=%d nnz=%d layout=%s status=%d" % (sysm.n, sysm.nnz, LAYOUTS[inf.spmvLayout][0], r.status),
          flush=True)
    d_b = torch.from_numpy(sysm.b).cuda()
    d_y = torch.zeros_like(d_b)
    if args.profile == "export":
        for _ in range(args.reps):
            files = h.export_signature()
        print("export bytes=%d" % sum(len(v) for v in files.values()), flush=True)
    elif args.profile == "spmv":
        for _ in range(args.reps):
            h.spmv(d_b.data_ptr(), d_y.data_ptr(), on_device=True)
    elif args.profile == "solve":
        d_diag = torch.from_numpy(sysm.diag).cuda()
        st, it, res = h.solve_device(d_b.data_ptr(), d_diag.data_ptr(), d_y.data_ptr(), 20000, 1e-10)
        print("solve status=%d iters=%d res=%.3e" % (st, it, res), flush=True)
    else:
        d_diag = torch.from_numpy(sysm.diag).cuda()
        m = h.mixed_solve(d_b.data_ptr(), d_diag.data_ptr(), 20000, 1e-10, x=d_y.data_ptr(), on_device=True)
        inf = h.info()
        print("mixed status=%d iters=%d refreshes=%d res=%.3e layout32=%s" % (
            m.status, m.iters, inf.outerSweeps, m.res, LAYOUTS[inf.spmvLayout32][0]), flush=True)
    torch.cuda.synchronize()
    h.close()


# SpMV layouts as reported by xJPCG_gbGetInfo().spmvLayout
LAYOUTS = {0: ("csr_staged", "spmv_ws_kernel (TMA-staged CSR fp64 SpMV)", 4),
           1: ("sliced", "spmv_sell_kernel<double,U,int> (SELL-32 fp64 SpMV, int32 columns)", 4),
           2: ("merge_path", "spmv_merge_kernel (merge-path CSR fp64 SpMV)", 4),
           3: ("sliced16", "spmv_sell_kernel<double,U,int16_t> (SELL-32 fp64 SpMV, int16 column offsets)", 2),
           4: ("sliced_sorted", "spmv_sellsort_kernel<double,U> (length-sorted SELL-32 fp64 SpMV, long rows per warp)",
               4),
           5: ("sliced_shared", "spmv_sellpat_kernel<double,U> (SELL-32 fp64 SpMV, column offsets shared per slice)",
               0)}


def spmv_bytes(n, nnz, col_bytes=4):
    # 8 B value + the stored column width per entry, row pointers, x read
    # once, y written once.
    return (8 + col_bytes) * nnz + 4 * (n + 1) + 8 * n + 8 * n


def iter_bytes(n, nnz, col_bytes=4):
    # SpMV + 10 vector streams of 8 B (update: r, Ap, J read, r written;
    # p kernel: x, p, r, J read, x, p written).
    return spmv_bytes(n, nnz, col_bytes) + 80 * n


def cpu_solve(sysm, tol=1e-10, max_iter=20000, nthreads=0):
    """One complete oracle JPCG solve (x0 = 0 to tol) on the host cores:
    (wall seconds, iterations run)."""
    import oracle
    oracle.build()
    t0 = time.perf_counter()
    r = oracle.jpcg(sysm.rowptr, sysm.col, sysm.val, sysm.diag, sysm.b, max_iter, tol, nthreads=nthreads)
    return time.perf_counter() - t0, r["k"]


def _timed(fn, reps=3):
    """Median wall time of fn() over reps (device work synchronised inside)."""
    import torch
    ts = []
    out = None
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts)), out


def mixed_vs_fp64(X, sysm, name, tight_tol=1e-14, cpu_s=None):
    """fp64 JPCG and the reliable-update mixed solver on the same system, both
    to 1e-10, with their errors against a tight FP64 oracle solve, and the
    oracle's fp64 time-to-tolerance on the host cores (cpu_s when the caller
    already timed it)."""
    import torch
    import oracle
    h = X.JPCG()
    r = h.csr_solve(sysm.n, sysm.rowptr, sysm.col, sysm.val, sysm.diag, sysm.b, 0, 1e-10)
    d_b = torch.from_numpy(sysm.b).cuda()
    d_d = torch.from_numpy(sysm.diag).cuda()
    d_x = torch.zeros_like(d_b)
    _timed(lambda: h.solve_device(d_b.data_ptr(), d_d.data_ptr(), d_x.data_ptr(), 20000, 1e-10), 1)
    t64, (st64, it64, _) = _timed(lambda: h.solve_device(d_b.data_ptr(), d_d.data_ptr(), d_x.data_ptr(), 20000,
                                                         1e-10))
    x64 = d_x.cpu().numpy()
    _timed(lambda: h.mixed_solve(d_b.data_ptr(), d_d.data_ptr(), 20000, 1e-10, x=d_x.data_ptr(), on_device=True), 1)
    tm, m = _timed(lambda: h.mixed_solve(d_b.data_ptr(), d_d.data_ptr(), 20000, 1e-10, x=d_x.data_ptr(),
                                         on_device=True))
    inf = h.info()
    xm = d_x.cpu().numpy()
    # FP32 SpMV on the HBM roofline: 4 B values + the layout's column bytes
    # per entry, row pointers, x read once and y written once in FP32
    ms32 = h.spmv_tuning32()[inf.spmvCfg32] if inf.spmvCfg32 < 64 else -1.0
    b32 = (4 + LAYOUTS[inf.spmvLayout32][2]) * sysm.nnz + 4 * (sysm.n + 1) + 8 * sysm.n
    peak, _ = measured_peak()
    gbs32 = b32 / (ms32 / 1e3) / 1e9 if ms32 > 0 else None
    tight = oracle.jpcg(sysm.rowptr, sysm.col, sysm.val, sysm.diag, sysm.b, 200000, tight_tol)["x"]
    nt = np.linalg.norm(tight)
    cpu_iters = None
    if cpu_s is None:
        cpu_s, cpu_iters = cpu_solve(sysm)
    out = {"system": name, "n": sysm.n, "nnz": sysm.nnz, "fp64_time_to_tol_s": t64, "fp64_iters": it64,
           "cpu_fp64_time_to_tol_s": cpu_s, "cpu_fp64_iters": cpu_iters, "cpu_cores": oracle.max_threads(),
           "cpu_kind": "port (oracle JPCG, one complete solve to 1e-10, all host cores)",
           "fp64_status": st64, "mixed_time_to_tol_s": tm, "mixed_fp32_iters": inf.innerIters,
           "mixed_refreshes": inf.outerSweeps, "mixed_status": m.status, "speedup": t64 / tm,
           "fp64_err_vs_oracle": float(np.linalg.norm(x64 - tight) / nt),
           "mixed_err_vs_oracle": float(np.linalg.norm(xm - tight) / nt),
           "mixed_true_relres": float(oracle.true_relres(sysm.rowptr, sysm.col, sysm.val, sysm.b, xm)),
           "oracle": "oracle JPCG to %g (FP64, CPU)" % tight_tol,
           "spmv_layout": LAYOUTS[inf.spmvLayout][0], "spmv_layout_fp32": LAYOUTS[inf.spmvLayout32][0],
           "spmv_fp32_ms": (h.spmv_tuning32()[inf.spmvCfg32] if inf.spmvCfg32 < 64 else None),
           "spmv_fp64_ms": h.spmv_tuning()[inf.spmvCfg][4],
           "spmv_fp32_shape": (list(h.spmv_tuning()[inf.spmvCfg32][:4]) if inf.spmvCfg32 < 64 else None),
           "spmv_tuning_fp32_ms": [round(v, 4) for v in h.spmv_tuning32()],
           "spmv_fp32_roofline": {"bytes_per_launch": b32, "achieved_gbs": gbs32,
                                  "frac": (gbs32 / peak if gbs32 else None), "peak_gbs": peak,
                                  "note": "tuner's median time of the chosen FP32 configuration"}}
    h.close()
    return out


def cpu_batch(systems, tol=1e-10, max_iter=20000):
    """The oracle's fp64 JPCG on every system, one system per host thread,
    all host cores busy (ctypes releases the GIL during each solve): (wall
    seconds, systems that met tol, threads)."""
    from concurrent.futures import ThreadPoolExecutor
    import oracle
    oracle.build()
    threads = oracle.max_threads()

    def one(s):
        r = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, s.b, max_iter, tol, nthreads=1)
        return int(r["status"] == 0 and r["res"] <= tol)

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        ok = sum(ex.map(one, sorted(systems, key=lambda s: -s.n)))  # largest first: even finish
    return time.perf_counter() - t0, ok, threads


def batched_measure(X, count=4096):
    from hpc_gb300 import workloads as W
    systems = W.batched_stencils(count=count, seed=3)
    h = X.JPCG()
    out = {"systems": count, "rows": int(sum(s.n for s in systems)), "nnz": int(sum(s.nnz for s in systems))}
    import oracle
    # error against a tight FP64 oracle solve on a sample of the systems
    sample = list(range(0, count, max(1, count // 16)))[:16]
    tight = {i: oracle.jpcg(systems[i].rowptr, systems[i].col, systems[i].val, systems[i].diag, systems[i].b,
                            200000, 1e-14)["x"] for i in sample}
    for prec, key in ((0, "fp64"), (1, "mixed")):
        st, _, res = h.batch_solve(systems, 20000, 1e-10, precision=prec)  # includes tuning on first use
        st, xs, res = h.batch_solve(systems, 20000, 1e-10, precision=prec)
        inf = h.info()
        err = max(float(np.linalg.norm(xs[i] - tight[i]) / np.linalg.norm(tight[i])) for i in sample)
        out[key] = {"status": st, "device_ms": inf.batchMs, "systems_per_s": count / (inf.batchMs / 1e3),
                    "converged": int(np.sum((res["status"] == 0) & (res["res"] <= 1e-10))),
                    "iters_total": int(res["itersRun"].sum()), "threads": inf.batchThreads,
                    "lanes": inf.batchLanes, "smem_rows": inf.batchSmemRows, "grid": inf.batchGrid,
                    "sliced": bool(inf.batchSliced),
                    "max_err_vs_oracle_sample": err,
                    "oracle": "oracle JPCG to 1e-14 (FP64, CPU) on %d sampled systems" % len(sample)}
    h.close()
    t_cpu, ok, threads = cpu_batch(systems)
    out["cpu_baseline"] = {"value": count / t_cpu, "unit": "systems/s", "seconds": t_cpu, "converged": ok,
                           "cores": threads, "kind": "port",
                           "sample": "all %d systems, fp64 oracle JPCG to 1e-10, one system per host thread" % count}
    return out


def adjoint_measure(X, nx=96):
    import torch
    from hpc_gb300 import workloads as W
    prob = W.adjoint_problem(nx, seed=4)
    n = nx ** 3
    ghost = W.ghost_diagonal7(prob.shape, prob.ghost)
    s = W.assemble_edges(n, prob.edge_i, prob.edge_j, np.exp(prob.theta), ghost)
    h = X.JPCG()
    # every host array of the timed calls in pinned memory, as the e2e inputs are
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    p_b, p_diag = pin(prob.b), pin(s.diag)
    p_x, p_lam = pin(np.zeros(n)), pin(np.zeros(n))
    tf, r = _timed(lambda: h.csr_solve(n, s.rowptr, s.col, s.val, p_diag, p_b, 20000, 1e-12, x=p_x,
                                       mode=X.MODE_KEEP_MATRIX if h.info().n == n else X.MODE_DEFAULT), 3)
    p_gin = pin(r.x - 0.5 * r.x)  # any right-hand side of the right size for the timing
    ta, (st, lam, _, it, res) = _timed(lambda: h.adjoint(p_gin, p_diag, 20000, 1e-12, lam=p_lam), 3)
    p_i, p_j, p_c = pin(prob.edge_i), pin(prob.edge_j), pin(np.exp(prob.theta))
    p_g = pin(np.zeros(prob.edge_i.size))
    tg, _ = _timed(lambda: h.edge_grad(p_i, p_j, p_c, out=p_g), 3)
    h.close()
    # The same gradient on the host cores: the oracle's forward and adjoint
    # solves (A is symmetric) and the per-edge formula -c (l_i - l_j)(x_i - x_j).
    import oracle
    oracle.build()
    c = np.exp(prob.theta)
    t0 = time.perf_counter()
    xf = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, prob.b, 20000, 1e-12)["x"]
    t1 = time.perf_counter()
    lam_c = oracle.jpcg(s.rowptr, s.col, s.val, s.diag, xf - 0.5 * xf, 20000, 1e-12)["x"]
    t2 = time.perf_counter()
    _ = -c * (lam_c[prob.edge_i] - lam_c[prob.edge_j]) * (xf[prob.edge_i] - xf[prob.edge_j])
    t3 = time.perf_counter()
    return {"grid": "%d^3" % nx, "n": n, "edges": int(prob.edge_i.size), "forward_solve_s": tf,
            "forward_iters": r.iters, "adjoint_solve_s": ta, "adjoint_iters": it, "edge_gradient_s": tg,
            "gradient_s": tf + ta + tg,
            "tol": 1e-12, "note": "host-array calls from pinned host buffers (H2D/D2H inside; the conductances "
                                  "exp(theta) computed before the timed calls, as on the CPU side); gradient checked "
                                  "in tests/test_gpu_adjoint.py",
            "cpu_baseline": {"value": t3 - t0, "unit": "s per gradient (forward + adjoint + edge gradient)",
                             "forward_s": t1 - t0, "adjoint_s": t2 - t1, "edge_gradient_s": t3 - t2,
                             "cores": oracle.max_threads(), "kind": "port",
                             "sample": "one complete gradient on the %d^3 system: oracle JPCG forward and adjoint "
                                       "solves to 1e-12 and the edge formula in numpy" % nx}}


def export_measure(X, sysm, reps=3):
    """Device time of the signature exporter (the reference's host
    partitioner, gen_signature.hpp:41-73, on the GPU) for the bench matrix.
    The matrix is set again before each rep so that the layout is rebuilt."""
    import ctypes as C
    import torch
    h = X.JPCG()
    ts = []
    sig = X.GbSignature()
    for _ in range(reps + 1):
        h.csr_solve(sysm.n, sysm.rowptr, sysm.col, sysm.val, sysm.diag, sysm.b, 0, 1e-10)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = h.lib.xJPCG_gbExportSignature(h.h, C.byref(sig))
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
        if st != X.SUCCESS:
            raise RuntimeError(h.last_message())
    out_bytes = sig.rbParamBytes + sig.parParamBytes + sum(sig.nnzValBytes[c] for c in range(16))
    h.close()
    return {"partition_s": float(np.median(ts[1:])), "signature_bytes": int(out_bytes),
            "call": "xJPCG_gbExportSignature on the stored matrix (device buffers; the copy out is separate)",
            "reference_partitioner": "SpmPar::partitionCooMat compiled from the reference sources runs on the "
                                     "build host only (oracle/time_ref_partition.py), not here"}


def summarize(line: dict) -> dict:
    """A few numbers of the line, repeated as its last key so that a reader
    of the line's tail sees them."""
    r = lambda v, d=3: None if v is None else round(float(v), d)
    s = {"solves_per_s": r(line["value"]), "e2e_solves_per_s": r((line.get("e2e") or {}).get("value")),
         "iter_ms": r(line.get("iter_ms"), 4), "spmv_hbm_frac": r(line["roofline"]["frac"]),
         "spmv_fp64_issue_frac": r(line["roofline"]["fp64_issue"]["frac"]),
         "fp64_peak_gdfma_s": r(line["roofline"]["fp64_issue"]["peak_gdfma_s"], 1),
         "cpu_solves_per_s": r((line.get("cpu_baseline") or {}).get("value"), 4)}
    for m in line.get("mixed", []):
        s["mixed_speedup_" + m["system"]] = r(m["speedup"])
        s["mixed_err_" + m["system"]] = float("%.2e" % m["mixed_err_vs_oracle"])
        s["cpu_fp64_s_" + m["system"]] = r(m.get("cpu_fp64_time_to_tol_s"))
    b = line.get("batched")
    if b:
        s["batched_fp64_ms"] = r(b["fp64"]["device_ms"], 1)
        s["batched_mixed_ms"] = r(b["mixed"]["device_ms"], 1)
        s["batched_cpu_systems_per_s"] = r(b["cpu_baseline"]["value"], 1)
    a = line.get("adjoint")
    if a:
        s["adjoint_gradient_ms"] = r(1e3 * a["gradient_s"], 1)
        s["adjoint_cpu_gradient_ms"] = r(1e3 * a["cpu_baseline"]["value"], 1)
    e = line.get("signature_export")
    if e:
        s["signature_export_ms"] = r(1e3 * e["partition_s"], 2)
    return s


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    from hpc_gb300 import workloads as W
    import oracle
    oracle.build()
    sysm = W.diffusion27(args.nx)
    threads = oracle.max_threads()
    # Every step, warm-up included, is one complete solve from x0 = 0 to the
    # tolerance, so the timed region is the K solves themselves.
    for _ in range(args.warmup):
        cpu_solve(sysm)
    t0 = time.perf_counter()
    steps = [cpu_solve(sysm) for _ in range(args.steps)]
    total = time.perf_counter() - t0
    iters = int(np.median([k for _, k in steps]))
    ttt = total / args.steps
    value = args.steps / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ttt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(args.gpus),
            "time_to_tol_s": ttt, "iters": iters, "step_s": [round(s, 3) for s, _ in steps],
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                             "sample": "%d complete solves of the 160^3 system (%d iterations each) on %d host "
                                       "threads, %d untimed before them" % (args.steps, iters, threads,
                                                                            args.warmup)},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args):
    import ctypes as C
    import torch
    import torch.distributed as dist

    import hpc_gb300 as X
    from hpc_gb300 import workloads as W

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    ranks = Ranks(world, "cuda")
    barrier, max_over_ranks = ranks.barrier, ranks.max

    sysm = W.diffusion27(args.nx)
    n, nnz = sysm.n, sysm.nnz
    rows, cols, vals = sysm.coo()
    # pinned host copies of the step's inputs for the end-to-end measurement
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    h_rows, h_cols, h_vals = pin(rows), pin(cols), pin(vals)
    h_diag, h_b = pin(sysm.diag), pin(sysm.b)
    h_x = torch.zeros(n, dtype=torch.float64).pin_memory()
    np_ = lambda t: t.numpy()

    h = X.JPCG()
    stream = torch.cuda.ExternalStream(h.stream())
    max_iter, tol = WORKLOAD["max_iter"], WORKLOAD["tol"]

    def e2e_step():
        r = h.coo_solve(n, np_(h_rows), np_(h_cols), np_(h_vals), np_(h_diag), np_(h_b), max_iter, tol,
                        x=np_(h_x))
        if r.status != X.SUCCESS:
            raise RuntimeError(r.message)
        return r

    r0 = e2e_step()  # sets the matrix, tunes the SpMV
    info = h.info()
    tuning = h.spmv_tuning()
    d_b = torch.from_numpy(sysm.b).cuda()
    d_diag = torch.from_numpy(sysm.diag).cuda()
    d_x = torch.zeros(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()

    def solve():
        st, it, res = h.solve_device(d_b.data_ptr(), d_diag.data_ptr(), d_x.data_ptr(), max_iter, tol)
        if st != X.SUCCESS:
            raise RuntimeError(h.last_message())
        return it

    for _ in range(max(args.warmup, 3)):
        solve()
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    iters = []
    ev0.record(stream)
    for _ in range(args.steps):
        iters.append(solve())
        iters[-1] = h.info().itersRun
    ev1.record(stream)
    torch.cuda.synchronize()
    clock_info = clocks.stop()
    barrier()
    t = ev0.elapsed_time(ev1) / 1e3
    t = max_over_ranks(t)
    ttt = t / args.steps
    value = replicas_value(world, args.steps, t)
    k_iters = int(np.median(iters))
    # per solve: the init kernel, then whole passes of the loop body (kernels
    # past the stop in the last pass launch and return at once)
    inf_l = h.info()
    per_pass = inf_l.kernelsPerIter * inf_l.loopUnroll
    launches = sum(1 + per_pass * -(-k // inf_l.loopUnroll) for k in iters)

    # Dominant kernel: the SpMV, timed alone on the same stream and matrix.
    spmv_ms = None
    reps = 20
    with torch.cuda.stream(stream):
        for _ in range(3):
            h.spmv(d_b.data_ptr(), d_x.data_ptr(), on_device=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            h.spmv(d_b.data_ptr(), d_x.data_ptr(), on_device=True)
        e1.record(stream)
    torch.cuda.synchronize()
    spmv_ms = e0.elapsed_time(e1) / reps
    peak, peak_kind = measured_peak()
    layout, kernel_name, col_bytes = LAYOUTS[info.spmvLayout]
    B = spmv_bytes(n, nnz, col_bytes)
    achieved = B / (spmv_ms / 1e3) / 1e9
    traffic, traffic_src = committed_traffic(layout)
    iter_ms = ttt * 1e3 / max(k_iters, 1)
    iter_gbs = iter_bytes(n, nnz, col_bytes) / (iter_ms / 1e3) / 1e9

    # End to end through the reference-facing COO call with host buffers.
    e2e = None
    if not args.no_e2e:
        for _ in range(args.warmup):  # untimed, as for the resident steps
            e2e_step()
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step_s, step_phases = [], []
        for _ in range(args.steps):
            ts = time.perf_counter()
            e2e_step()
            step_s.append(time.perf_counter() - ts)
            m_, i_ = h.metrics(), h.info()
            step_phases.append([round(m_.m_matProc, 4), round(i_.uploadMs / 1e3, 4), round(i_.uploadIdxMs / 1e3, 4),
                                round(i_.uploadValMs / 1e3, 4), round(i_.tuneMs / 1e3, 4), round(m_.m_solver, 4)])
        torch.cuda.synchronize()
        te = max_over_ranks(time.perf_counter() - t0)
        met, inf_e = h.metrics(), h.info()
        e2e = {"value": replicas_value(world, args.steps, te), "unit": "solves/s",
               "h2d_bytes_per_step": int(4 * nnz + 4 * nnz + 8 * nnz + 8 * n + 8 * n),
               "d2h_bytes_per_step": int(8 * n + 256), "time_to_tol_s": te / args.steps,
               "call": "xJPCG_cooSolver(MODE_DEFAULT), pinned host COO arrays", "step_s": step_s,
               "step_phases_s": {"columns": ["matProc", "upload", "upload_indices", "upload_values", "tuning",
                                                 "solver"], "steps": step_phases},
               "last_call_phases_s": {"matProc (H2D, conversion, layouts, tuning)": met.m_matProc,
                                      "of which SpMV tuning": inf_e.tuneMs / 1e3,
                                      "of which H2D of the COO arrays": inf_e.uploadMs / 1e3,
                                      "vecProc": met.m_vecProc, "solver (incl. D2H of x)": met.m_solver}}

    # The FP64 issue ceiling of this GPU, measured now (register-resident DFMA
    # chains on every SM, best of three launches): the fp64 kernels are held
    # against it beside the HBM roofline.
    fp64_rate, fp64_ms = h.fp64_rate()

    # The other sliced layouts, forced one at a time and timed the same way:
    # the tuner's choice moves the fewest bytes but is bound by FP64 issue,
    # so the layouts that carry column bytes sit higher on the HBM roofline.
    alt_layouts = []
    for lanes in (-3, -1):
        try:
            h.set_spmv_lanes(lanes)
        except X.XJPCGError:
            continue
        alt = h.info().spmvLayout
        if alt == info.spmvLayout:
            continue
        with torch.cuda.stream(stream):
            for _ in range(3):
                h.spmv(d_b.data_ptr(), d_x.data_ptr(), on_device=True)
            e0.record(stream)
            for _ in range(reps):
                h.spmv(d_b.data_ptr(), d_x.data_ptr(), on_device=True)
            e1.record(stream)
        torch.cuda.synchronize()
        ms_alt = e0.elapsed_time(e1) / reps
        name_alt, kern_alt, cb_alt = LAYOUTS[alt]
        b_alt = spmv_bytes(n, nnz, cb_alt)
        alt_layouts.append({"layout": name_alt, "kernel": kern_alt, "launch_ms": ms_alt, "bytes_per_launch": b_alt,
                            "achieved": b_alt / (ms_alt / 1e3) / 1e9, "frac": b_alt / (ms_alt / 1e3) / 1e9 / peak,
                            "fp64_issue_frac": nnz / (ms_alt / 1e3) / fp64_rate,
                            "traffic": committed_traffic(name_alt)[0]})
    h.set_spmv_lanes(0)  # back to the tuned choice

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        import oracle
        cpu_s, cpu_iters = cpu_solve(sysm)
        xs = np.asarray(sysm.b)
        oracle.spmv(sysm.rowptr, sysm.col, sysm.val, xs)
        t0 = time.perf_counter()
        for _ in range(5):
            oracle.spmv(sysm.rowptr, sysm.col, sysm.val, xs)
        spmv_cpu_s = (time.perf_counter() - t0) / 5
        cpu = {"value": 1.0 / cpu_s, "unit": "solves/s", "cores": oracle.max_threads(),
               "kind": "port", "spmv_gbs": spmv_bytes(n, nnz) / spmv_cpu_s / 1e9,
               "spmv_note": "oracle CSR SpMV (12 B per entry), all host cores, 5 launches",
               "sample": "one complete oracle JPCG solve of the 160^3 system to 1e-10 (%.2f s, %d iterations) "
                         "on all host cores" % (cpu_s, cpu_iters)}

    extras = {}
    if rank == 0 and not args.no_extras:
        from hpc_gb300 import workloads as W
        extras["mixed"] = [mixed_vs_fp64(X, sysm, "diffusion27_160", cpu_s=(1.0 / cpu["value"] if cpu else None)),
                           mixed_vs_fp64(X, W.zipf_spd(2_000_000, seed=2), "zipf_spd_2M")]
        extras["batched"] = batched_measure(X)
        extras["adjoint"] = adjoint_measure(X)
        extras["signature_export"] = export_measure(X, sysm)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": ttt * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": bench_config(world),
                "spmv_choice": {"lanes": info.spmvLanes, "grid": info.spmvGrid, "cfg": info.spmvCfg,
                                "tuning": [list(t) for t in tuning]},
                "time_to_tol_s": ttt, "iters": k_iters, "iter_ms": iter_ms, "iter_gbs": iter_gbs,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic,
                             "kernel": kernel_name, "layout": layout,
                             "bytes_per_launch": B, "bytes_formula": "(8 + %d) nnz + 4 (n + 1) + 16 n" % col_bytes,
                             "launch_ms": spmv_ms,
                             "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                             "traffic_source": traffic_src,
                             "fp64_issue": {"achieved_gdfma_s": nnz / (spmv_ms / 1e3) / 1e9,
                                            "peak_gdfma_s": fp64_rate / 1e9,
                                            "frac": nnz / (spmv_ms / 1e3) / fp64_rate,
                                            "peak_source": "measured in this run (xJPCG_gbDiagFp64Rate: "
                                                           "register-resident DFMA chains on every SM, "
                                                           "%.2f ms best of 3)" % fp64_ms,
                                            "nominal_gdfma_s": FP64_DFMA_NOMINAL / 1e9,
                                            "note": "one DFMA per stored entry; the SpMV is bound by whichever "
                                                    "fraction is higher"},
                             "other_layouts": alt_layouts},
                "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clock_info,
                "loop": "conditional-graph" if h.info().loopMode == 1 else "host"}
        line.update(extras)
        line["summary"] = summarize(line)
        print(json.dumps(line), flush=True)
    h.close()
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.profile:
        run_profile(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
