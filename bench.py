"""Benchmark: f64-accurate solves/s on the batched uneven-solve mix.

Workload (one step = one pass over the whole batch): 20,000 SPD systems A = G G^T + n I
(Cholesky) and 20,000 general systems A = U(-1,1) + n I (PartialPivLu), n log-uniform
in [8, 512], one N(0,1) right-hand side each, seed 0. The timed path is the mixed-
precision batched solver (FP32 factor, FP64 residual / update / backward-error test,
FP64 refactor for any system that does not converge), graph-captured, one plan.

  value            solves/s with inputs resident in HBM (device-pointer C entry point)
  e2e              solves/s through the host-pointer C entry point: every step copies
                   A and b from pinned host memory and x, info, iters, berr back
  plain_fp64_gpu   solves/s of the same batch factored and solved entirely in FP64
  cpu_baseline     the oracle (C restatement of rulinalg's algorithms) on a bounded
                   sample of the same systems, 1 thread

--impl reference times the oracle on all host threads instead (the reference crate is
Rust and cannot be built on this machine; its algorithms are restated in oracle/).
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "f64-accurate solves/s (batched uneven mix: 20k SPD Cholesky + 20k general LU, n log-uniform [8,512])"
U64 = 2.0 ** -53


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--count-spd", type=int, default=20000)
    p.add_argument("--count-lu", type=int, default=20000)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--cpu-sample-gflop", type=float, default=8.0,
                   help="CPU baseline sample size in GFLOP of factorisation work")
    p.add_argument("--skip-e2e", action="store_true")
    p.add_argument("--skip-cpu", action="store_true")
    p.add_argument("--workload", default="batch", choices=["batch", "dense", "mixed", "serve", "factors"],
                   help="batch (default): the headline batched mix, followed by the other configurations as "
                        "sub-objects of the same line; dense / mixed / serve: only that configuration, as its "
                        "own line (GEMM sweep + FP64 LU; single-system mixed precision; served stream; "
                        "single factorisations: LU, Cholesky, QR, FullPivLu)")
    p.add_argument("--configs", default="1,2,3,4f,5",
                   help="configurations reported beside the headline: 1 (LU n=1024), 2 (GEMM sweep, FP64 LU), "
                        "3 (mixed single systems), 4f (f32 SPD half of the batch), 5 (served stream); '' for none")
    p.add_argument("--sizes", default="", help="comma-separated sizes for dense / mixed")
    p.add_argument("--kappas", default="1e2,1e6,1e10", help="mixed: condition numbers")
    p.add_argument("--nrhs", default="1,64", help="mixed: right-hand-side counts")
    p.add_argument("--gen", default="haar", choices=["haar", "uniform"],
                   help="mixed: A = U diag(sigma) V^T (haar) or U(-1,1) + n/2 I (uniform, no factorisation "
                        "needed to build it; kappa is then ignored)")
    p.add_argument("--lambdas", default="1000,10000,50000", help="serve: arrival rates (requests/s)")
    p.add_argument("--serve-seconds", type=float, default=60.0, help="serve: stream length per rate")
    p.add_argument("--serve-workers", type=int, default=0, help="serve: worker threads (0: the library's default)")
    p.add_argument("--tune", default="", help="library tunables set before the run: key=value[,key=value] with "
                                              "the RL_TUNE_* keys of include/rulinalg_gb300.h")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def aggregate_max(value: float, world: int, device=None) -> float:
    """Max over ranks (the job ends when the slowest replica ends)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons, sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._th = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([c.strip() for c in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._th.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def parse_cpulist(text: str) -> set:
    cpus = set()
    for part in text.strip().split(","):
        if not part:
            continue
        if "-" in part:
            a, b = part.split("-")
            cpus.update(range(int(a), int(b) + 1))
        else:
            cpus.add(int(part))
    return cpus


def pin_near_gpu(index: int) -> str:
    """Restricts this process to the host CPUs local to GPU `index` (sysfs local_cpulist of
    its PCI function), so that the pinned host buffers the end-to-end leg allocates and
    first touches sit in the memory attached to that GPU's host link. Returns what was
    done, for the JSON line."""
    try:
        import torch
        p = torch.cuda.get_device_properties(index)
        bdf = f"{p.pci_domain_id:04x}:{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0"
    except Exception:
        try:
            out = subprocess.run(["nvidia-smi", "-i", str(index), "--query-gpu=pci.bus_id", "--format=csv,noheader"],
                                 capture_output=True, text=True, timeout=10).stdout.strip()
            dom, bus, rest = out.split(":")
            bdf = f"{int(dom, 16):04x}:{bus.lower()}:{rest.lower()}"
        except Exception as e:  # no affinity information: leave the process as it is
            return f"unchanged ({type(e).__name__})"
    try:
        cpus = parse_cpulist(Path(f"/sys/bus/pci/devices/{bdf}/local_cpulist").read_text())
        allowed = os.sched_getaffinity(0)
        use = cpus & allowed
        if not use or use == allowed:
            return f"unchanged (local CPUs of {bdf}: {len(cpus)}, allowed {len(allowed)})"
        os.sched_setaffinity(0, use)
        return f"{len(use)} CPUs local to GPU {bdf} (of {len(allowed)})"
    except Exception as e:
        return f"unchanged ({type(e).__name__})"


def flops_of(n, kind):
    n = n.astype(np.float64)
    return float(np.sum(np.where(kind == 1, n ** 3 / 3.0, 2.0 * n ** 3 / 3.0)))


def cpu_sample(n, kind, gflop, seed):
    """A seeded sample of system indices whose factorisation work is ~gflop."""
    rng = np.random.default_rng(seed + 99)
    order = rng.permutation(len(n))
    w = np.where(kind[order] == 1, n[order].astype(np.float64) ** 3 / 3.0, 2.0 * n[order].astype(np.float64) ** 3 / 3.0)
    k = int(np.searchsorted(np.cumsum(w), gflop * 1e9)) + 1
    return np.sort(order[:max(1, min(k, len(n)))])


def run_oracle(idx, n, kind, a_host, b_host, threads):
    import oracle as O
    a_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)])
    b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))])
    sn = n[idx]
    sk = kind[idx]
    sa = np.concatenate([a_host[a_off[i]:a_off[i + 1]] for i in idx])
    sb = np.concatenate([b_host[b_off[i]:b_off[i + 1]] for i in idx])
    sa_off = np.concatenate([[0], np.cumsum(sn.astype(np.int64) ** 2)[:-1]])
    sb_off = np.concatenate([[0], np.cumsum(sn.astype(np.int64))[:-1]])
    t0 = time.perf_counter()
    info = O.batch_solve(sn, sk, sa_off, sa, sb_off, sb, threads=threads)
    dt = time.perf_counter() - t0
    return dt, info


def workloads_module():
    """rulinalg_gb300/workloads.py loaded by its path: the package's __init__ loads the
    CUDA library, which the reference arm must not map (it is numpy-only)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("rl_bench_workloads", ROOT / "rulinalg_gb300" / "workloads.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def batch_config(args, world, n):
    """The `config` of the headline line, identical in both arms."""
    a_gb = float(np.sum(np.asarray(n, dtype=np.float64) ** 2)) * 8 / 1e9
    return {"workload": "batched uneven solves: 20k SPD (Cholesky) + 20k general (PartialPivLu)",
            "count_spd": args.count_spd, "count_lu": args.count_lu, "n_range": [8, 512], "rhs": 1,
            "seed": args.seed, "parallelism": f"replicas x{world}",
            "l2": f"inputs {a_gb:.1f} GB of f64 matrices > 129 MB L2, no flush needed"}


def reference_arm(args, rank, world):
    """The reference's algorithms (the oracle's C restatement of PartialPivLu / Cholesky
    decompose + solve) on all host threads, on a seeded quarter of the batch's work."""
    if rank != 0:
        return
    n, kind, a, b = workloads_module().mixed_batch(args.count_spd, args.count_lu, seed=args.seed)
    threads = os.cpu_count() or 1
    idx = cpu_sample(n, kind, flops_of(n, kind) / 4e9, args.seed)
    for _ in range(max(0, args.warmup)):
        run_oracle(idx[: max(1, len(idx) // 8)], n, kind, a, b, threads)
    times = []
    for _ in range(args.steps):
        dt, info = run_oracle(idx, n, kind, a, b, threads)
        times.append(dt)
    v = len(idx) / statistics.mean(times)
    sample = (f"each step: {len(idx)} of {len(n)} systems, a seeded sample carrying a quarter of the batch's "
              f"factorisation work ({flops_of(n[idx], kind[idx]) / 1e9:.1f} of {flops_of(n, kind) / 1e9:.1f} GFLOP); "
              f"{threads} POSIX threads taking systems from a shared counter (the reference crate itself is "
              f"single-threaded); rulinalg-algorithm restatement in C (oracle/), -O2 -ffp-contract=off")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": batch_config(args, world, n),
        "cpu_baseline": {"value": v, "unit": "solves/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "rulinalg is Rust with no toolchain on this machine; its algorithms run as the C restatement in "
                "oracle/ (no CUDA library is loaded by this arm)",
    }), flush=True)


def event_times(fn, steps, warmup, stream, flush=None):
    """CUDA-event times (ms) of `steps` calls of fn on `stream`, after `warmup` calls; when
    `flush` is given it is overwritten before every call (L2 flush, outside the events)."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    out = []
    for _ in range(steps):
        if flush is not None:
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        out.append(e0.elapsed_time(e1))
    return out


FP64_PEAK_TFLOPS = 1.25  # GB300's FP64 rate (nominal; rl_dgemm_dev sustains it at n = 8192)


def peaks():
    return json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}


def profile_traffic(a_bytes: float, path=None):
    """DRAM bytes per launch of the batched kernel for a batch of a_bytes matrix bytes,
    from the committed ncu summary's line `traffic_per_launch_bytes: T @ M` (T bytes for
    a batch of M matrix bytes), scaled by matrix bytes; None without that line."""
    path = path or ROOT / "profiles" / "batch_solve_kernel_mixed_40k_mix.md"
    if not Path(path).exists():
        return None
    for line in Path(path).read_text().splitlines():
        if line.startswith("traffic_per_launch_bytes:") and "@" in line:
            t, m = line.split(":", 1)[1].split("@")
            return float(t) * a_bytes / float(m)
    return None


def tf32x3_ceiling_tflops():
    """FP32-accurate ceiling of the 3xTF32 tensor-core GEMM: the TF32 rate (half the
    measured bf16 burst rate) over the three TF32 products per FP32 product."""
    return peaks().get("bf16_tflops", 1900.0) / 2.0 / 3.0


def config1(dev):
    """PartialPivLu decompose + solve, f64, n = 1024, A = U(-1,1) + I (seed 0), b = A x_true:
    permutation against the oracle, L/U normwise errors, backward and forward errors."""
    import hashlib

    import torch
    import oracle as O
    import rulinalg_gb300 as rl
    from rulinalg_gb300._lib import SolveInfo
    import ctypes as C
    from rulinalg_gb300.workloads import config1_lu
    n = 1024
    a, x_true, b = config1_lu(n, seed=0)
    olu, operm, st, gap = O.lu_decompose(a, gaps=True)
    t0 = time.perf_counter()
    lu = rl.PartialPivLu.decompose(a)
    x = lu.solve(b)
    host_ms = 1e3 * (time.perf_counter() - t0)
    lref, uref = np.tril(olu, -1), np.triu(olu)
    fro = lambda m: float(np.sqrt(np.sum(m * m)))
    xo, _ = O.lu_solve(olu, operm, b)
    r = b - a @ x
    berr = float(np.max(np.abs(r)) / (np.max(np.sum(np.abs(a), 1)) * np.max(np.abs(x)) + np.max(np.abs(b))))
    stream = torch.cuda.current_stream()
    ta, tb = torch.from_numpy(a).to(dev), torch.from_numpy(b.reshape(n, 1)).to(dev)
    tx = torch.zeros_like(tb)
    info = SolveInfo()
    call = lambda: rl.lib.rl_dsolve_fp64_dev(n, 1, 0, ta.data_ptr(), n, tb.data_ptr(), 1, tx.data_ptr(), 1,
                                             C.byref(info), stream.cuda_stream)
    ms = statistics.median(event_times(call, 5, 3, stream))
    return {"workload": "PartialPivLu decompose + solve, f64, n=1024, U(-1,1)+I seed 0, b = A x_true",
            "perm_bit_identical_to_oracle": bool(np.array_equal(lu.p.perm, operm)),
            "perm_sha256": hashlib.sha256(lu.p.perm.astype("<u8").tobytes()).hexdigest()[:16],
            "min_pivot_gap": float(gap[:-1].min()),
            "l_rel_err_vs_oracle": fro(np.tril(lu.lu, -1) - lref) / fro(lref),
            "u_rel_err_vs_oracle": fro(np.triu(lu.lu) - uref) / fro(uref),
            "berr": berr, "berr_within": berr <= n * U64 * 10,
            "fwd_err_vs_oracle": float(np.max(np.abs(x - xo)) / np.max(np.abs(xo))),
            "fwd_err_vs_x_true": float(np.max(np.abs(x - x_true)) / np.max(np.abs(x_true))),
            "device_ms": ms, "host_api_ms": host_ms,
            "tflops": (2.0 * n ** 3 / 3.0 + 2.0 * n * n) / (ms / 1e3) / 1e12}


def config2(dev, sizes=(1024, 2048, 4096, 8192), steps=3, warm=3):
    """Square GEMM sweep (N(0,1), seeded), f32 and f64, and the plain FP64 LU solve at the
    largest size: TFLOP/s, fraction of the FP64 rate / the 3xTF32 ceiling, cuBLAS beside
    it for context, and the normwise accuracy bound n eps ||A||_F ||B||_F against an FP64
    product."""
    import torch
    import rulinalg_gb300 as rl
    from rulinalg_gb300.workloads import config1_lu
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    ceil32 = tf32x3_ceiling_tflops()
    sweep = []
    for n in sizes:
        g = torch.Generator(device=dev)
        g.manual_seed(n)
        a64 = torch.randn(n, n, dtype=torch.float64, device=dev, generator=g)
        b64 = torch.randn(n, n, dtype=torch.float64, device=dev, generator=g)
        for dt, fn_name, eps in ((torch.float32, "rl_sgemm_dev", 2.0 ** -24), (torch.float64, "rl_dgemm_dev", U64)):
            a, b = a64.to(dt), b64.to(dt)
            c = torch.empty(n, n, dtype=dt, device=dev)
            f = getattr(rl.lib, fn_name)
            call = lambda: f(n, n, n, a.data_ptr(), n, b.data_ptr(), n, c.data_ptr(), n, sh)
            ms = statistics.median(event_times(call, steps, warm, stream, flush))
            ref = a.double() @ b.double()
            err = float(torch.linalg.norm(c.double() - ref))
            bound = n * eps * float(torch.linalg.norm(a.double())) * float(torch.linalg.norm(b.double()))
            cub = statistics.median(event_times(lambda: torch.matmul(a, b, out=c), steps, warm, stream, flush))
            tf = 2.0 * n ** 3 / (ms / 1e3) / 1e12
            peak = FP64_PEAK_TFLOPS if dt == torch.float64 else ceil32
            sweep.append({"n": n, "dtype": "f64" if dt == torch.float64 else "f32", "ms": ms, "tflops": tf,
                          "frac": tf / peak, "peak_tflops": peak, "cublas_tflops": 2.0 * n ** 3 / (cub / 1e3) / 1e12,
                          "err_over_bound": err / bound, "within": err <= bound})
            del ref
        del a64, b64
    n = max(sizes)
    a_h, x_true, b_h = config1_lu(n, seed=0)
    a = torch.from_numpy(a_h).to(dev)
    b = torch.from_numpy(b_h).to(dev).reshape(n, 1)
    x = torch.empty_like(b)
    call = lambda: rl.lib.rl_dsolve_fp64_dev(n, 1, 0, a.data_ptr(), n, b.data_ptr(), 1, x.data_ptr(), 1, None, sh)
    ms = statistics.median(event_times(call, 2, 1, stream, flush))
    r = (b - a @ x).abs().max().item()
    berr = r / (a.abs().sum(1).max().item() * x.abs().max().item() + b.abs().max().item())
    tf = (2.0 * n ** 3 / 3.0 + 2.0 * n * n) / (ms / 1e3) / 1e12
    return {"workload": "square GEMM C = A B, N(0,1), f32 (tcgen05 3xTF32) and f64 (DFMA); plain FP64 LU solve",
            "peaks": {"f64_tflops": FP64_PEAK_TFLOPS, "f64_source": "GB300 FP64 rate (nominal)",
                      "f32_tflops": ceil32, "f32_source": "MEASURED_PEAKS bf16 burst / 2 (TF32) / 3 (3xTF32), of measured"},
            "gemm": sweep,
            "fp64_lu_solve": {"n": n, "ms": ms, "tflops": tf, "frac_of_fp64_rate": tf / FP64_PEAK_TFLOPS,
                              "berr": berr, "within": berr <= n * U64 * 10},
            "l2": "256 MB buffer overwritten before every timed call"}


def config3(dev, sizes=(4096, 8192, 16384), kappas=(1e2, 1e6, 1e10), nrhs_list=(1, 64), gen="haar"):
    """Mixed-precision single-system LU solves (FP32 factor, FP64 refinement, GMRES-IR,
    FP64 refactor) against the plain FP64 GPU solve: A = U diag(sigma) V^T, Haar U, V,
    sigma geometric from 1 to 1/kappa, 1 and 64 N(0,1) right-hand sides. Forward error of
    the mixed solution against the plain FP64 GPU solution (all sizes) and against the
    FP64 oracle (n = 4096, elimination rows over all host threads)."""
    import torch
    import ctypes as C
    import rulinalg_gb300 as rl
    from rulinalg_gb300._lib import SolveInfo
    from rulinalg_gb300.workloads import conditioned_system
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    paths = {0: "refinement", 1: "gmres-ir", 2: "fp64"}
    cases = []
    for n in sizes:
        reps = 3 if n <= 8192 else 1
        for kappa in kappas:
            if gen == "haar":
                a, bfull = conditioned_system(n, kappa, 64, seed=n + int(np.log10(kappa)), device=dev)
            else:
                g = torch.Generator(device=dev)
                g.manual_seed(n)
                a = torch.rand(n, n, dtype=torch.float64, device=dev, generator=g) * 2 - 1
                a += torch.eye(n, dtype=torch.float64, device=dev) * (n / 2)
                bfull = torch.randn(n, 64, dtype=torch.float64, device=dev, generator=g)
            xo_all = None
            if n == 4096 and 64 in nrhs_list and gen == "haar":
                import oracle as O
                ah, bh = a.cpu().numpy(), bfull.cpu().numpy()
                lu, perm, st = O.lu_decompose(ah, threads=os.cpu_count() or 1)
                xo_all, _ = O.solve_columns(lu, perm, bh, threads=os.cpu_count() or 1)
            for nrhs in nrhs_list:
                b = bfull[:, :nrhs].contiguous()
                row = {"n": n, "kappa": kappa, "nrhs": nrhs}
                xs = {}
                for name, fn in (("mixed", rl.lib.rl_dsolve_mixed_dev), ("fp64", rl.lib.rl_dsolve_fp64_dev)):
                    x = torch.empty_like(b)
                    info = SolveInfo()
                    call = lambda: fn(n, nrhs, 0, a.data_ptr(), n, b.data_ptr(), nrhs, x.data_ptr(), nrhs,
                                      C.byref(info), sh)
                    ms = statistics.median(event_times(call, reps, 1, stream))
                    row[name] = {"ms": ms, "berr": info.berr, "iters": info.iters, "gmres_iters": info.gmres_iters,
                                 "path": paths.get(info.path, info.path), "within": info.berr <= n * U64 * 10}
                    xs[name] = x
                fe = torch.linalg.norm(xs["mixed"] - xs["fp64"], dim=0) / torch.linalg.norm(xs["fp64"], dim=0)
                row["mixed"]["fwd_err_vs_fp64_gpu"] = float(fe.max())
                if xo_all is not None:
                    xo = torch.from_numpy(np.ascontiguousarray(xo_all[:, :nrhs])).to(dev)
                    fo = torch.linalg.norm(xs["mixed"] - xo, dim=0) / torch.linalg.norm(xo, dim=0)
                    row["mixed"]["fwd_err_vs_oracle"] = float(fo.max())
                row["speedup"] = row["fp64"]["ms"] / row["mixed"]["ms"]
                cases.append(row)
            del a, bfull
    sp = [c["speedup"] for c in cases]
    return {"workload": "A = U diag(sigma) V^T (Haar U, V; sigma geometric 1 .. 1/kappa), nrhs N(0,1)",
            "geomean_speedup_mixed_over_fp64": float(np.exp(np.mean(np.log(sp)))),
            "all_within": all(c["mixed"]["within"] for c in cases), "cases": cases}


def factors(n: int = 4096, reps: int = 3):
    """Single factorisations through the host-pointer entry points (each call copies A in
    and the factor out): PartialPivLu and Cholesky in f32 and f64, Householder QR of an
    n x n and of a 2n x n matrix in f32 and f64, FullPivLu in f64. Median wall time of
    `reps` calls after one warm-up; GFLOP/s on the reference's flop counts (LU 2/3 n^3,
    Cholesky 1/3 n^3, QR 2 m n^2 - 2/3 n^3), and for FullPivLu the bytes its passes move
    (each step reads and writes the trailing block: about n^3/3 elements each way)."""
    import rulinalg_gb300 as rl
    rng = np.random.default_rng(n)
    g = rng.standard_normal((n, n))
    spd = g @ g.T / n + np.eye(n)
    gen = rng.uniform(-1, 1, (n, n)) + np.eye(n)
    tall = rng.standard_normal((2 * n, n))
    out = {"workload": f"single factorisations, n = {n} (QR also 2n x n)", "n": n, "runs": []}

    def timed(name, fn, flops=None, bytes_moved=None):
        fn()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        ms = 1e3 * statistics.median(ts)
        row = {"op": name, "ms_host_api": ms}
        if flops:
            row["gflops"] = flops / (ms / 1e3) / 1e9
        if bytes_moved:
            row["gbs"] = bytes_moved / (ms / 1e3) / 1e9
        out["runs"].append(row)

    for dt in (np.float32, np.float64):
        tag = "f32" if dt == np.float32 else "f64"
        timed(f"lu_{tag}", lambda: rl.PartialPivLu.decompose(gen.astype(dt)), 2.0 * n ** 3 / 3)
        timed(f"cholesky_{tag}", lambda: rl.Cholesky.decompose(spd.astype(dt)), n ** 3 / 3.0)
        timed(f"qr_{tag}", lambda: rl.HouseholderQr.decompose(gen.astype(dt)), 4.0 * n ** 3 / 3)
        timed(f"qr_tall_{tag}", lambda: rl.HouseholderQr.decompose(tall.astype(dt)),
              2.0 * 2 * n * n * n - 2.0 * n ** 3 / 3)
    timed("full_piv_lu_f64", lambda: rl.FullPivLu.decompose(gen), 2.0 * n ** 3 / 3, 2 * 8 * n ** 3 / 3.0)
    return out


def config4_f32(dev, args):
    """The f32 half of the SPD set: 20,000 Cholesky systems as Matrix<f32> (FP32 plan,
    graph-captured, device pointers)."""
    import torch
    import rulinalg_gb300 as rl
    n, kind, a, b = workloads_module().mixed_batch(args.count_spd, 0, seed=args.seed, device=dev, dtype=np.float32)
    count = len(n)
    stream = torch.cuda.current_stream()
    plan = rl.BatchPlan(n, kind, rl.PREC_FP32)
    x = torch.zeros_like(b)
    info = torch.zeros(count, dtype=torch.int32, device=dev)
    berr = torch.zeros(count, dtype=torch.float64, device=dev)
    call = lambda: plan.solve_dev(a.data_ptr(), b.data_ptr(), x.data_ptr(), info.data_ptr(), 0, berr.data_ptr(),
                                  stream.cuda_stream)
    ms = statistics.mean(event_times(call, max(3, args.steps), max(3, args.warmup), stream))
    plan.close()
    limit = torch.from_numpy(n.astype(np.float64) * 2.0 ** -24 * 10).to(dev)
    return {"workload": f"{count} SPD systems A = G G^T + n I in f32 (Cholesky, FP32 plan)",
            "solves_per_s": count / (ms / 1e3), "ms_per_step": ms, "all_ok": bool((info == 0).all()),
            "max_berr": float(berr.max()), "berr_within_n_u32_10": bool((berr <= limit).all())}


def config5(dev, args):
    """The served stream: Poisson arrivals at each lambda for args.serve_seconds s, sizes
    log-uniform in [16, 4096], kinds 50% LU / 30% Cholesky / 20% QR least squares (m = 2n,
    N(0,1)), 30% of requests re-solving a resident LU factor with a new right-hand side.
    Matrices come from a seeded pool that the requests cycle through (read-only host
    arrays); results land in per-entry output slots (their values are not read: every
    result's f64 accuracy is the backward error the server reports). Admission by HBM
    footprint; backpressure: at most max_pending requests in the server, the rest refused
    (RL_ERR_BUSY) and counted."""
    import rulinalg_gb300 as rl
    from rulinalg_gb300._lib import REQUEST_DTYPE
    wl = workloads_module()
    rng = np.random.default_rng(args.seed)
    per_kind = 24
    pool = {0: [], 1: [], 2: []}
    for kind in (0, 1, 2):
        for nn in wl.log_uniform_sizes(per_kind, 16, 4096, rng):
            nn = int(nn)
            if kind == 0:
                a = rng.uniform(-1, 1, (nn, nn)) + nn * np.eye(nn)
            elif kind == 1:
                u = rng.uniform(-1, 1, (nn, nn))
                a = 0.5 * (u + u.T) + nn * np.eye(nn)
            else:
                a = rng.standard_normal((2 * nn, nn))
            pool[kind].append((np.ascontiguousarray(a), rng.standard_normal(a.shape[0]),
                               [np.zeros(nn) for _ in range(4)]))
    max_pending = 2048
    srv = rl.Server(max_pending=max_pending, workers=args.serve_workers)
    resident = []
    for nn in wl.log_uniform_sizes(8, 16, 4096, rng):
        nn = int(nn)
        a = rng.uniform(-1, 1, (nn, nn)) + nn * np.eye(nn)
        t, _ = srv.submit(rl.REQ_LU, a, rng.standard_normal(nn), retain=True)
        resident.append((srv.wait(t)["factor"], nn, rng.standard_normal(nn), [np.zeros(nn) for _ in range(4)]))
    names = {0: "lu", 1: "cholesky", 2: "lstsq", 3: "resolve"}
    runs = []
    for lam in [float(v) for v in args.lambdas.split(",")]:
        count = int(lam * args.serve_seconds)
        arrivals = np.cumsum(rng.exponential(1.0 / lam, count))
        req = np.zeros(count, dtype=REQUEST_DTYPE)
        is_res = rng.random(count) < 0.3
        kinds = rng.choice(3, size=count, p=[0.5, 0.3, 0.2])
        which = rng.integers(0, per_kind, count)
        rwhich = rng.integers(0, len(resident), count)
        slot = np.arange(count) % 4
        kind_of = np.where(is_res, 3, kinds)
        req["kind"] = kind_of
        for k in (0, 1, 2):
            for e in range(per_kind):
                sel = (~is_res) & (kinds == k) & (which == e)
                if not sel.any():
                    continue
                a, b, xs = pool[k][e]
                req["m"][sel] = a.shape[0]
                req["n"][sel] = a.shape[1]
                req["a"][sel] = a.ctypes.data
                req["b"][sel] = b.ctypes.data
                req["x"][sel] = np.array([x.ctypes.data for x in xs], dtype=np.uint64)[slot[sel]]
        for e, (h, nn, b, xs) in enumerate(resident):
            sel = is_res & (rwhich == e)
            req["factor"][sel] = h
            req["m"][sel] = nn
            req["n"][sel] = nn
            req["b"][sel] = b.ctypes.data
            req["x"][sel] = np.array([x.ctypes.data for x in xs], dtype=np.uint64)[slot[sel]]
        srv.reset_stats()
        t0 = time.perf_counter()
        res = srv.replay_arrays(arrivals, req)
        wall = time.perf_counter() - t0
        st = srv.stats()
        ok = res["status"] == 0
        busy = res["status"] == 37
        by_kind = {}
        for k, nm in names.items():
            sel = ok & (kind_of == k)
            lat = np.sort(res["latency_us"][sel]) / 1e3
            if len(lat):
                by_kind[nm] = {"completed": int(sel.sum()), "p50_ms": float(lat[len(lat) // 2]),
                               "p99_ms": float(lat[min(len(lat) - 1, int(0.99 * len(lat)))])}
        sq = ok & (kind_of != 2)
        lat = np.sort(res["latency_us"][ok]) / 1e3
        runs.append({"lambda": lam, "seconds": args.serve_seconds, "offered": count, "accepted": int((~busy).sum()),
                     "rejected_busy": int(busy.sum()), "completed_ok": int(ok.sum()),
                     "failed": int((~ok & ~busy).sum()), "solves_per_s": float(ok.sum() / wall), "wall_s": wall,
                     "p50_ms": float(lat[len(lat) // 2]) if len(lat) else None,
                     "p99_ms": float(lat[min(len(lat) - 1, int(0.99 * len(lat)))]) if len(lat) else None,
                     "by_kind": by_kind, "batches": st["batches"], "batched_requests": st["batched_requests"],
                     "bytes_peak": st["bytes_peak"],
                     "max_berr_lu_chol_resolve": float(res["berr"][sq].max()) if sq.any() else None})
    srv.close()
    return {"workload": "Poisson stream, sizes log-uniform [16,4096], 50% LU / 30% Cholesky / 20% QR LS (m=2n), "
                        "30% re-solves of resident factors",
            "pool_per_kind": per_kind, "resident_factors": len(resident), "max_pending": max_pending,
            "workers": args.serve_workers or "default", "runs": runs}


def main():
    args = parse()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        dist.init_process_group(backend)
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    import torch
    import rulinalg_gb300 as rl
    from rulinalg_gb300.workloads import mixed_batch

    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    if not rl.device_available():
        raise SystemExit("rulinalg_gb300: no usable sm_103 GPU")
    affinity = pin_near_gpu(local)
    for kv in filter(None, args.tune.split(",")):
        k, v = kv.split("=")
        rl.tune_set(int(k), int(float(v)))
    if args.workload != "batch":
        sizes = tuple(int(v) for v in args.sizes.split(",")) if args.sizes else None
        with ClockSampler(local) as clk:
            if args.workload == "dense":
                out = config2(dev, sizes or (1024, 2048, 4096, 8192))
            elif args.workload == "factors":
                out = factors(sizes[0] if sizes else 4096)
            elif args.workload == "mixed":
                out = config3(dev, sizes or (4096, 8192, 16384), tuple(float(v) for v in args.kappas.split(",")),
                              tuple(int(v) for v in args.nrhs.split(",")), args.gen)
            else:
                out = config5(dev, args)
        out["clocks"] = clk.summary()
        if rank == 0:
            print(json.dumps({"workload": args.workload, **out}), flush=True)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    n, kind, a, b = mixed_batch(args.count_spd, args.count_lu, seed=args.seed, device=dev)
    count = len(n)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    a_bytes = a.numel() * 8
    b_bytes = b.numel() * 8

    def alloc_out():
        return (torch.zeros_like(b), torch.zeros(count, dtype=torch.int32, device=dev),
                torch.zeros(count, dtype=torch.int32, device=dev), torch.zeros(count, dtype=torch.float64, device=dev))

    def time_plan(precision, steps, warmup):
        plan = rl.BatchPlan(n, kind, precision)
        x, info, iters, berr = alloc_out()
        call = lambda: plan.solve_dev(a.data_ptr(), b.data_ptr(), x.data_ptr(), info.data_ptr(), iters.data_ptr(),
                                      berr.data_ptr(), sh)
        for _ in range(warmup):
            call()
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        l0 = rl.launch_count()
        with ClockSampler(local) as clk:
            t0 = time.perf_counter()
            for e0, e1 in ev:
                e0.record(stream)
                call()
                e1.record(stream)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
        launches = rl.launch_count() - l0
        per = [e0.elapsed_time(e1) for e0, e1 in ev]
        res = dict(ms=per, wall=wall, launches=launches, clocks=clk.summary(),
                   info=info.cpu().numpy(), iters=iters.cpu().numpy(), berr=berr.cpu().numpy(), x=x)
        plan.close()
        return res

    # autotuned launch shape and size classes for each plan (rulinalg_gb300/autotune.py),
    # cached for this run only, so every bench run tunes on its own GPU
    import tempfile
    from rulinalg_gb300 import autotune
    tune_cache = Path(tempfile.mkdtemp()) / "autotune.json"
    tuned = {}
    tuned["fp64"] = autotune.tune(n, kind, rl.PREC_FP64, a, b, reps=2, cache=tune_cache)
    fp64 = time_plan(rl.PREC_FP64, max(2, args.steps // 3), 1)
    tuned["mixed"] = autotune.tune(n, kind, rl.PREC_MIXED, a, b, reps=3, cache=tune_cache)
    mixed = time_plan(rl.PREC_MIXED, args.steps, args.warmup)

    ms_mixed = aggregate_max(sum(mixed["ms"]) / len(mixed["ms"]), world, dev)
    ms_fp64 = aggregate_max(sum(fp64["ms"]) / len(fp64["ms"]), world, dev)
    value = world * count / (ms_mixed / 1e3)
    v_fp64 = world * count / (ms_fp64 / 1e3)

    # e2e: host pointers (pinned), copies inside the timed region, through the C ABI.
    e2e = None
    if not args.skip_e2e:
        a_h = a.cpu().pin_memory()
        b_h = b.cpu().pin_memory()
        x_h = torch.zeros(b.numel(), dtype=torch.float64).pin_memory()
        i_h = torch.zeros(count, dtype=torch.int32).pin_memory()
        it_h = torch.zeros(count, dtype=torch.int32).pin_memory()
        be_h = torch.zeros(count, dtype=torch.float64).pin_memory()
        plan = rl.BatchPlan(n, kind, rl.PREC_MIXED)
        import ctypes as C
        f64p = C.POINTER(C.c_double)
        i32p = C.POINTER(C.c_int32)
        args_c = (plan._h, C.cast(a_h.data_ptr(), f64p), C.cast(b_h.data_ptr(), f64p), C.cast(x_h.data_ptr(), f64p),
                  C.cast(i_h.data_ptr(), i32p), C.cast(it_h.data_ptr(), i32p), C.cast(be_h.data_ptr(), f64p))
        for _ in range(max(1, args.warmup)):
            assert rl.lib.rl_dbatch_solve(*args_c) == 0
        torch.cuda.synchronize()
        # this host's pinned host-to-device rate for the same buffer (one plain copy),
        # which bounds the end-to-end step (the upload is overlapped with the solve)
        dst = torch.empty_like(a)
        t0 = time.perf_counter()
        dst.copy_(a_h, non_blocking=True)
        torch.cuda.synchronize()
        h2d_gbs = a_bytes / (time.perf_counter() - t0) / 1e9
        del dst
        ts = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            assert rl.lib.rl_dbatch_solve(*args_c) == 0
            ts.append(time.perf_counter() - t0)
        plan.close()
        e2e_s = aggregate_max(statistics.mean(ts), world, dev)
        e2e = {"value": world * count / e2e_s, "unit": "solves/s", "ms_per_step": 1e3 * e2e_s,
               "h2d_bytes_per_step": int(a_bytes + b_bytes),
               "d2h_bytes_per_step": int(b_bytes + count * (4 + 4 + 8)),
               "ms_steps": [round(1e3 * t, 2) for t in ts], "host_affinity": affinity,
               "h2d_gbs_pinned": h2d_gbs, "upload_ms_at_that_rate": 1e3 * (a_bytes + b_bytes) / (h2d_gbs * 1e9),
               "timing": "host clock around each rl_dbatch_solve call (pinned host buffers in, results out)"}
        assert np.array_equal(x_h.numpy(), mixed["x"].cpu().numpy()), "host and device entry points disagree"

    # accuracy of both paths (f64 backward error bound n 2^-53 10)
    limit = n.astype(np.float64) * U64 * 10
    acc = {
        "bound": "berr <= n * 2^-53 * 10 (normwise, inf-norms)",
        "mixed_max_berr": float(mixed["berr"].max()), "mixed_all_within": bool((mixed["berr"] <= limit).all()),
        "mixed_all_ok": bool((mixed["info"] == 0).all()),
        "fp64_max_berr": float(fp64["berr"].max()), "fp64_all_within": bool((fp64["berr"] <= limit).all()),
        "fallbacks": int((mixed["iters"] < 0).sum()),
        "refinement_steps_hist": np.bincount(mixed["iters"][mixed["iters"] >= 0]).tolist(),
    }
    # roofline of the dominant kernel (the mixed batched solve): FP32 factor flops and
    # FP64 refinement flops against measured peaks; HBM bytes = the f64 matrices read once.
    fl32 = flops_of(n, kind) + float(np.sum(2.0 * n.astype(np.float64) ** 2 * (mixed["iters"].clip(0) + 1)))
    fl64 = float(np.sum(2.0 * n.astype(np.float64) ** 2 * (mixed["iters"].clip(0) + 1)))
    t_k = ms_mixed / 1e3
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    alg_bytes = a_bytes + 2 * b_bytes
    # DRAM traffic per launch from the committed ncu summary of this kernel (one launch on
    # a 6,000-system batch of the same mix), scaled here by matrix bytes to this batch.
    traffic = profile_traffic(a_bytes)
    fp64_peak = FP64_PEAK_TFLOPS
    fp64_floor_ms = fl64 / (fp64_peak * 1e12) * 1e3
    roofline = {"bound": "hbm", "achieved": alg_bytes / t_k / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "frac": alg_bytes / t_k / 1e9 / hbm_peak, "traffic": traffic,
                "traffic_rate_gbs": traffic / t_k / 1e9 if traffic else None,
                "traffic_source": "not measured in this run: ncu dram__bytes_read+write of one launch of a smaller "
                                  "batch of the same mix, scaled by matrix bytes (profiles/"
                                  "batch_solve_kernel_mixed_40k_mix.md)",
                "kernel": "batch_solve_kernel<double,float,true> (graph: memset + main pass + FP64 fallback pass)",
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6.8 TB/s",
                "compute": {"fp32_tflops": fl32 / t_k / 1e12, "fp32_simt_peak_tflops": 80.5,
                            "fp32_peak_source": "152 SMs x 128 FP32 lanes x 2 flops x 2.07 GHz (nominal)",
                            "fp64_tflops": fl64 / t_k / 1e12, "fp64_peak_tflops": fp64_peak,
                            "fp64_floor_ms": fp64_floor_ms, "frac_of_fp64_floor": fp64_floor_ms / ms_mixed,
                            "note": "HBM is not the binding unit (algorithmic bytes are 1/10 of the DRAM "
                                    "traffic, which runs at ~30% of peak); the binding throughput floor is "
                                    "the FP64 pipe for the refinement residuals (fp64_floor_ms), the kernel "
                                    "itself is latency-bound per CTA (profiles/)"}}

    cpu = None
    if rank == 0 and not args.skip_cpu:
        a_h = a.cpu().numpy()
        b_h = b.cpu().numpy()
        idx = cpu_sample(n, kind, args.cpu_sample_gflop, args.seed)
        dt, info = run_oracle(idx, n, kind, a_h, b_h, 1)
        cpu = {"value": len(idx) / dt, "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": f"{len(idx)} of {count} systems, seeded sample ({flops_of(n[idx], kind[idx]) / 1e9:.1f} "
                         f"GFLOP of factorisation), rulinalg-algorithm restatement in C, 1 thread"}

    # forward error of every solution against the FP64 oracle's (all systems, all host threads)
    if rank == 0 and not args.skip_cpu:
        import oracle as O
        a_h = a.cpu().numpy()
        b_h = b.cpu().numpy()
        a_off = np.concatenate([[0], np.cumsum(n.astype(np.int64) ** 2)])[:-1]
        b_off = np.concatenate([[0], np.cumsum(n.astype(np.int64))])[:-1]
        xo = b_h.copy()
        t0 = time.perf_counter()
        oinfo = O.batch_solve(n, kind, a_off, a_h.copy(), b_off, xo, threads=os.cpu_count() or 1)
        t_or = time.perf_counter() - t0
        xm = mixed["x"].cpu().numpy()
        num = np.maximum.reduceat(np.abs(xm - xo), b_off)
        den = np.maximum.reduceat(np.abs(xo), b_off)
        fe = num / den
        acc["fwd_err_vs_oracle"] = {"max": float(fe.max()), "p99": float(np.quantile(fe, 0.99)),
                                    "oracle_all_ok": bool((oinfo == 0).all()),
                                    "norm": "||x - x_oracle||_inf / ||x_oracle||_inf per system",
                                    "oracle_seconds": t_or, "oracle_threads": os.cpu_count() or 1}

    lat = sorted(mixed["ms"])
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_mixed, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 factor + f64 refinement", "data": "synthetic",
        "config": batch_config(args, world, n),
        "plain_fp64_gpu": {"value": v_fp64, "unit": "solves/s", "ms_per_step": ms_fp64,
                           "speedup_mixed_over_fp64": value / v_fp64},
        "batch_latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
        "autotune": {k: {"choice": v["choice"], "tuned_ms": v["ms"], "default_ms": v["default_ms"],
                         "trials": len(v["trials"])} for k, v in tuned.items()},
        "accuracy": acc,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(mixed["launches"]),
        "clocks": mixed["clocks"],
    }
    # the other configurations, each measured on its own (rank 0; replicas would repeat them)
    wanted = [c for c in args.configs.split(",") if c]
    if rank == 0 and wanted:
        del a, b
        torch.cuda.empty_cache()
        configs = {}
        with ClockSampler(local) as clk:
            for key, name, fn in (("1", "config1_lu_1024", lambda: config1(dev)),
                                  ("2", "config2_gemm_and_fp64_lu", lambda: config2(dev)),
                                  ("3", "config3_mixed_single_system", lambda: config3(dev)),
                                  ("4f", "config4_f32_spd_half", lambda: config4_f32(dev, args)),
                                  ("5", "config5_served_stream", lambda: config5(dev, args))):
                if key in wanted:
                    t0 = time.perf_counter()
                    try:
                        configs[name] = fn()
                    except Exception as e:  # reported in the line; the headline stands on its own
                        import traceback
                        traceback.print_exc()
                        configs[name] = {"error": f"{type(e).__name__}: {e}"}
                    configs[name]["wall_s"] = time.perf_counter() - t0
                    torch.cuda.synchronize()
                    torch.cuda.empty_cache()
        configs["clocks"] = clk.summary()
        line["configs"] = configs
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
