"""Benchmark: fused Lanczos steps on the 2x14 two-hole t-J ladder (k = (0, 0)).

One "step" is one Lanczos step of the spectrum/ground-state recursion over the
whole sector (H.v + a_k dot + axpy + b_{k+1} norm): the fused H.v kernel
(ed_lanczos_hv) plus the in-place update (ed_lanczos_update).  Default: mixed
precision (FP32 vectors, FP64 reductions); the plain FP64 GPU path is timed
beside it, and the ground energy of both forms is compared (relative
difference reported as delta_E_rel).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

--impl reference times the reference's CPU path (stored-matrix SpMV in the
reference's row-major Hermitian-triangle form + the numpy vector operations of
_lanczos_vec_iteration), run through the CPU oracle port on a bounded row
sample of the same sector and scaled to one full step.

N > 1 (torchrun): every rank runs an independent replica of the workload
(the path does not shard within a sector); value = steps of all ranks / max time.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Lanczos steps/s & H·v HBM GB/s, 2×14 t-J: mixed vs FP64 GPU at ΔE≤1e-10"
UNIT = "Lanczos steps/s"
SECTOR = (14, 2, 13, 0, 0)
WEIGHTS = {"tl": 1.0, "tr": 1.0, "jl": 0.5, "jr": 0.5}
KERNEL_VERSION = "v9"  # the H.v kernel generation the committed traffic figure was captured on


def workload_name(sector) -> str:
    L, nh, nd, kx, ky = sector
    sz2 = 2 * L - nh - 2 * nd
    return (f"2x{L} t-J ladder, {nh} holes, 2Sz={sz2}, k=({kx},{ky}), t=1, J=0.5: "
            "fused Lanczos step over the full sector")


def peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms while running; mark() before and
    after the timed region selects the samples taken during it (plus the first one after)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread is not None:
                self.thread.join(timeout=2)

    def wait_first(self, timeout_s: float = 3.0) -> None:
        """Block until the sampler has produced a sample (nvidia-smi takes a moment to start)."""
        t_end = time.perf_counter() + timeout_s
        while self.proc is not None and not self.lines and time.perf_counter() < t_end:
            time.sleep(0.02)

    def mark(self) -> int:
        return len(self.lines)

    def wait_one_more(self, n: int, timeout_s: float = 0.5) -> None:
        t_end = time.perf_counter() + timeout_s
        while self.proc is not None and len(self.lines) <= n and time.perf_counter() < t_end:
            time.sleep(0.01)

    def summary(self, lo: int = 0, hi: int | None = None) -> dict:
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[lo: None if hi is None else hi + 1]:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def ncu_traffic(workload_key: str, kind_rows: tuple[int, int, int]) -> float | None:
    """DRAM bytes of one fused H.v step (all row kinds) from the committed ncu summary: its bytes
    per row of each kind times this sector's rows of that kind, if the summary covers this workload
    and kernel generation."""
    p = ROOT / "profiles" / "lanczos_hv_2x14_traffic.txt"
    if not p.exists():
        return None
    fields = {}
    for line in p.read_text().splitlines():
        if ":" in line and not line.startswith("#"):
            k, v = line.split(":", 1)
            fields[k.strip()] = v.strip()
    if fields.get("workload") != workload_key or fields.get("kernel_version") != KERNEL_VERSION:
        return None
    per_row = [float(fields["dram_bytes_per_row_free"]), float(fields["dram_bytes_per_row_stabiliser"]),
               float(fields.get("dram_bytes_per_row_orbit_walk", fields["dram_bytes_per_row_stabiliser"]))]
    return sum(r * b for r, b in zip(kind_rows, per_row))


def aggregate_replicas(ms_local: list[float], steps: int, world: int, device=None) -> tuple[list[float], float]:
    """Max over ranks of the per-step times (the slowest replica bounds the job) and the whole-job
    throughput: all ranks' steps divided by that time.  Replicas exchange nothing else."""
    if world > 1:
        import torch

        t = torch.tensor(ms_local, dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = [float(v) for v in t.cpu()]
    else:
        ms = list(ms_local)
    return ms, world * 1000.0 / ms[0]


# ----------------------------------------------------------------------------- engine arm

def run_engine(args, rank: int, world: int) -> dict | None:
    import torch

    from exactdiag_gb300.engine import DeviceSector
    from exactdiag_gb300.lanczos import ground_state

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    t0 = time.perf_counter()
    sec = DeviceSector(*SECTOR)
    torch.cuda.synchronize()
    t_basis = time.perf_counter() - t0
    n = sec.n
    K, W = args.steps, args.warmup

    from exactdiag_gb300 import autotune

    tuned = {}

    def timed_steps(precision: str):
        dt = sec.dtype(precision)
        if args.launch:
            minb, ctas = (int(t) for t in args.launch.split(","))
            autotune.set_launch(sec, minb, ctas)
            tuned[precision] = {"min_ctas_per_sm": minb, "ctas_per_sm": ctas, "grid": autotune.get_launch(sec)[1],
                                "fixed": True}
        else:
            tuned[precision] = autotune.tune(sec, WEIGHTS, dt, use_cache=False)
        rng = np.random.default_rng(0)
        v0 = torch.as_tensor(rng.uniform(-1, 1, n), device=dev).to(dt)
        buf = [v0.clone(), torch.zeros_like(v0)]
        scal = torch.zeros(2 * (K + W) + 4, dtype=torch.float64, device=dev)
        norm = torch.zeros(1, dtype=torch.float64, device=dev)
        sec.normalize(buf[0], norm)

        def step(k, ev=None):
            v, other = buf[k % 2], buf[(k + 1) % 2]
            if ev is not None:
                ev[0].record()
            sec.lanczos_hv(WEIGHTS, v, other if k > 0 else None, other, scal[2 * k: 2 * k + 4])
            if ev is not None:
                ev[1].record()
            sec.lanczos_update(v, other, scal[2 * k: 2 * k + 4])

        with ClockSampler(dev.index) as clocks:
            clocks.wait_first()
            for k in range(W):
                step(k)
            torch.cuda.synchronize()
            if world > 1:
                torch.distributed.barrier()
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
            start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            lo = clocks.mark()
            start.record()
            for k in range(W, W + K):
                step(k, evs[k - W])
            stop.record()
            torch.cuda.synchronize()
            hi = clocks.mark()
            clocks.wait_one_more(hi)
        if world > 1:
            torch.distributed.barrier()
        total_ms = start.elapsed_time(stop)
        hv_ms = [a.elapsed_time(b) for a, b in evs]
        return total_ms, hv_ms, clocks.summary(lo, hi), dt

    total_mixed, hv_mixed, clocks, dt_mixed = timed_steps("fp32")
    total_fp64, hv_fp64, _, dt64 = timed_steps("fp64")
    (ms_mixed, ms_fp64), value = aggregate_replicas([total_mixed / K, total_fp64 / K], K, world, dev)

    # roofline of the dominant kernel (fused H.v of the step): algorithmic bytes per launch
    s_bytes = torch.empty(0, dtype=dt_mixed).element_size()
    bytes_per_row = 8 + 1 + 3 * s_bytes  # key, orbit size, v_k, v_{k-1}, y
    hv_avg_ms = float(np.mean(hv_mixed))
    achieved = n * bytes_per_row / (hv_avg_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    s64 = torch.empty(0, dtype=dt64).element_size()
    hv64_gbs = n * (8 + 1 + 3 * s64) / (float(np.mean(hv_fp64)) * 1e-3) / 1e9

    # end to end through the C ABI with host buffers: pinned host v0 -> device, one ed_lanczos_step
    # per step with the step's (a_k, b_{k+1}) read back to the host
    e2e = None
    if rank == 0:
        autotune.set_launch(sec, tuned["fp32"]["min_ctas_per_sm"], tuned["fp32"]["ctas_per_sm"])
        e2e = e2e_steps(sec, K, dt_mixed)

    energy = {}
    if not args.no_energy and rank == 0:
        g64 = ground_state(sec, WEIGHTS, args.energy_steps, precision="fp64", seed=1)
        gmx = ground_state(sec, WEIGHTS, args.energy_steps, precision="mixed", seed=1)
        energy = {
            "E0_fp64": g64["E0"], "E0_mixed": gmx["E0"],
            "delta_E_rel": abs(gmx["E0"] - g64["E0"]) / abs(g64["E0"]),
            "lanczos_steps": args.energy_steps, "refine_steps_fp64": gmx.get("refine_steps"),
            "mixed_residual": gmx.get("residual"),
        }

    if rank != 0:
        return None
    traffic = ncu_traffic(workload_name(SECTOR), autotune.kind_rows(sec))
    return {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": ms_mixed,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {
            "workload": workload_name(SECTOR),
            "sector": {"num_rungs": SECTOR[0], "num_holes": SECTOR[1], "num_down_spins": SECTOR[2],
                       "kx": SECTOR[3], "ky": SECTOR[4]},
            "n_representatives": n,
            "precision": "mixed: FP32 vectors and per-term arithmetic, FP64 reductions",
            "start_vector": "np.random.default_rng(0).uniform(-1, 1, n)",
            "l2_policy": f"inputs larger than L2: each FP32 vector {n * s_bytes / 1e6:.0f} MB, key table "
                         f"{n * 8 / 1e6:.0f} MB",
            "basis_build_s": t_basis,
            "fp64_steps_per_s": world * 1000.0 / ms_fp64,
            "fp64_ms_per_step": ms_fp64,
            "mixed_over_fp64": ms_fp64 / ms_mixed,
            "hv_gbs_mixed": achieved,
            "hv_gbs_fp64": hv64_gbs,
            "bytes_per_row_mixed": bytes_per_row,
            "parallelism": "replicas" if world > 1 else "single GPU",
            "launch": {p: {k: v for k, v in r.items() if k != "candidates"} for p, r in tuned.items()},
            **energy,
        },
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": traffic,
                     "kernel": "lanczos_hv_kernel<float,false,*,kind> for each block kind + lanczos_scalars_kernel (ed_lanczos_hv)",
                     "algorithmic_bytes_per_launch": n * bytes_per_row},
        "e2e": e2e,
        "gpu_launches": K * autotune.step_launches(sec),
        "clocks": clocks,
        "cpu_baseline": None if args.no_cpu else cpu_baseline(args),
    }


def e2e_steps(sec, K: int, dt) -> dict:
    import torch

    from exactdiag_gb300 import _native as nat
    from exactdiag_gb300.engine import _ptr, _stream_ptr, weights_tuple

    lib = nat.load()
    n = sec.n
    host_v0 = torch.as_tensor(np.random.default_rng(0).uniform(-1, 1, n)).to(dt).pin_memory()
    host_scal = torch.zeros(4, dtype=torch.float64).pin_memory()
    code = sec._code(torch.empty(n, dtype=dt, device=sec.device))
    w = nat.weights_array(weights_tuple(WEIGHTS))
    buf = [torch.empty(n, dtype=dt, device=sec.device), torch.empty(n, dtype=dt, device=sec.device)]
    scal = torch.zeros(2 * K + 4, dtype=torch.float64, device=sec.device)
    norm = torch.zeros(1, dtype=torch.float64, device=sec.device)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    start.record()
    buf[0].copy_(host_v0, non_blocking=True)
    sec.normalize(buf[0], norm)
    for k in range(K):
        v, other = buf[k % 2], buf[(k + 1) % 2]
        nat.check("ed_lanczos_step", lib.ed_lanczos_step(sec.handle, w, code, _ptr(v), _ptr(other if k else None),
                                                         _ptr(other), _ptr(scal[2 * k: 2 * k + 4]), _stream_ptr()))
        host_scal.copy_(scal[2 * k: 2 * k + 4], non_blocking=True)
        torch.cuda.current_stream().synchronize()  # the host reads a_k, b_{k+1} every step
    stop.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    return {"value": K / wall, "unit": UNIT, "h2d_bytes_per_step": n * host_v0.element_size() / K,
            "d2h_bytes_per_step": 32, "note": "host-driven steps through the C ABI: start vector copied from "
            "pinned host memory inside the timed region (bytes amortised over the steps), the step's "
            "a_k, b_{k+1} read back to the host after every step", "device_ms": start.elapsed_time(stop)}


# ----------------------------------------------------------------------------- CPU baseline (oracle port)

class CpuReference:
    """The reference's CPU step on the same sector, timed on a bounded row sample.

    Setup (untimed): the sector's basis by the oracle; for `sample_rows` evenly spaced rows, each
    term's stored row in the reference's row-major Hermitian-triangle format (entries with column
    >= row, int16 value indices into a table of unique values).  A timed step: the four terms' SpMV
    passes over those rows (or_spmv_triangle_rows, single thread) and the vector operations of
    _lanczos_vec_iteration on `vec_sample` elements, both scaled by n / sample to one full step.
    """

    def __init__(self, sector, sample_rows: int = 4000, vec_sample: int = 4_000_000):
        from oracle import oracle as O

        O.build(ref=False)
        self.O = O
        self.lib = O.lib()
        sec = O.Sector(*sector)
        t0 = time.perf_counter()
        sp, orb = O.basis(sec)
        self.t_basis = time.perf_counter() - t0
        self.n = n = len(sp)
        # contiguous chunks of rows at evenly spaced offsets keep the x locality a full pass has
        chunk = 1024
        nchunks = max(1, sample_rows // chunk)
        starts = np.linspace(0, max(0, n - chunk), nchunks).astype(np.int64)
        self.rows = rows = np.unique(np.concatenate([np.arange(s0, min(n, s0 + chunk)) for s0 in starts]))
        self.vec_sample = min(vec_sample, n)
        i64p = ctypes.POINTER(ctypes.c_int64)
        f64p = ctypes.POINTER(ctypes.c_double)
        self.mats = []
        for t, term in enumerate(O.TERMS):
            nnz = ctypes.c_int64()
            colptr = np.empty(len(rows) + 1, np.int64)
            args = (*sec.args(), t, 1, sp.ctypes.data_as(i64p), orb.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                    ctypes.c_int64(n), rows.ctypes.data_as(i64p), ctypes.c_int64(len(rows)))
            self.lib.or_term_columns_subset(*args, colptr.ctypes.data_as(i64p), None, None, None,
                                            ctypes.c_int64(0), ctypes.byref(nnz))
            cols = np.empty(nnz.value, np.int64)
            vre = np.empty(nnz.value)
            vim = np.empty(nnz.value)
            self.lib.or_term_columns_subset(*args, colptr.ctypes.data_as(i64p), cols.ctypes.data_as(i64p),
                                            vre.ctypes.data_as(f64p), vim.ctypes.data_as(f64p),
                                            ctypes.c_int64(nnz.value), ctypes.byref(nnz))
            # row-major triangle storage holds conj of the column-major values (cython_sparse_matrices.pyx:149-155)
            vals = np.conj(vre + 1j * vim)
            uniq, inv = np.unique(np.round(vals, 12), return_inverse=True)
            self.mats.append((term, colptr, cols, inv.astype(np.int16), np.ascontiguousarray(uniq, np.complex128)))
        del sp, orb
        self.x = np.random.default_rng(0).uniform(-1, 1, n).astype(np.complex128)
        self.y = np.zeros(n, np.complex128)

    def step_seconds(self, seed: int = 0) -> float:
        i64p = ctypes.POINTER(ctypes.c_int64)
        vp = ctypes.c_void_p
        rows = self.rows
        t0 = time.perf_counter()
        for term, colptr, cols, vidx, vals in self.mats:
            self.lib.or_spmv_triangle_rows(ctypes.c_int64(len(rows)), rows.ctypes.data_as(i64p),
                                           colptr.ctypes.data_as(i64p), cols.ctypes.data_as(i64p),
                                           vidx.ctypes.data_as(ctypes.POINTER(ctypes.c_int16)), vp(vals.ctypes.data),
                                           vp(self.x.ctypes.data), vp(self.y.ctypes.data),
                                           ctypes.c_double(WEIGHTS[term]), ctypes.c_double(0.0))
        t_spmv = time.perf_counter() - t0
        m = self.vec_sample
        rng = np.random.default_rng(seed)
        vn = rng.uniform(-1, 1, m).astype(np.complex128)
        vnm = rng.uniform(-1, 1, m).astype(np.complex128)
        hvn = rng.uniform(-1, 1, m).astype(np.complex128)
        t0 = time.perf_counter()
        an = np.real(np.vdot(vn, hvn))
        vnp = hvn - an * vn - 0.5 * vnm
        bnp = np.linalg.norm(vnp)
        vnp /= bnp
        t_vec = time.perf_counter() - t0
        return t_spmv * self.n / len(rows) + t_vec * self.n / m

    def sample_text(self) -> str:
        return (f"{len(self.rows)} rows (1024-row chunks at evenly spaced offsets) of the {self.n}-row sector (SpMV of the 4 stored term "
                f"matrices in the reference's row-major Hermitian-triangle passes) + the _lanczos_vec_iteration "
                f"vector ops on {self.vec_sample} elements, complex128, each scaled by n/sample to one full step; "
                "one thread because the reference's multi-threaded SpMV races (wrong results beyond 1 thread)")


def cpu_baseline(args) -> dict:
    ref = CpuReference(SECTOR, args.cpu_sample_rows, args.cpu_vec_sample)
    ref.step_seconds(0)
    times = [ref.step_seconds(k + 1) for k in range(3)]
    return {"value": 1.0 / float(np.mean(times)), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": ref.sample_text(), "setup_basis_s": ref.t_basis}


def run_reference(args, rank: int) -> dict | None:
    if rank != 0:
        return None
    K, W = args.steps, args.warmup
    ref = CpuReference(SECTOR, args.cpu_sample_rows, args.cpu_vec_sample)
    for k in range(W):
        ref.step_seconds(k)
    times = [ref.step_seconds(W + k) for k in range(K)]
    ms = 1000.0 * float(np.mean(times))
    value = 1000.0 / ms
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": W, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": workload_name(SECTOR), "n_representatives": ref.n, "precision": "complex128 (reference)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port", "sample": ref.sample_text()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--energy-steps", type=int, default=160)
    ap.add_argument("--no-energy", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-sample-rows", type=int, default=4000)
    ap.add_argument("--cpu-vec-sample", type=int, default=4_000_000)
    ap.add_argument("--sector", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--launch", default=None, metavar="MINB,CTAS",
                    help="fix the free-row step kernel's launch (register variant 3|4, CTAs per SM, 0 = all that fit) "
                         "instead of tuning it")
    args = ap.parse_args()
    if args.sector:
        global SECTOR
        SECTOR = tuple(int(v) for v in args.sector.split(","))
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        out = run_reference(args, rank)
        if out is not None:
            print(json.dumps(out))
        return
    if world > 1:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group("nccl")
    out = run_engine(args, rank, world)
    if out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
