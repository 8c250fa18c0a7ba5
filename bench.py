"""Benchmark: fused Lanczos steps on the 2x14 two-hole t-J ladder (k = (0, 0)).

One "step" is one Lanczos step of the ground-state / spectrum recursion over the whole sector
(H.v + a_k dot + axpy + b_{k+1} norm): the fused H.v kernels (ed_lanczos_hv) plus the in-place
update (ed_lanczos_update).  `value` is the mixed-precision form (FP32 vectors, FP64 reductions).
The line also carries the plain FP64 GPU form, the time each form takes to a converged ground
energy, and under `extra` the other measured workloads:

* config2: the 2x12 two-hole ladder, all 24 momentum sectors: steps/s and H.v GB/s of both forms on
  a real and a complex sector, and every sector's ground energy in both forms (worst dE, total time);
* config3: S^z_q recursions into the 24 2x12 target sectors (m = 150): one batched recursion against
  24 sequential ones, complex64 and complex128;
* config5: the 2x16 two-hole ladder (2.4e9 representatives): both forms' steps/s, GB/s and ground
  energy.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference] [--no-extra]

--impl reference times the reference's CPU step (its stored-matrix SpMV in the row-major
Hermitian-triangle form plus the numpy vector operations of _lanczos_vec_iteration) through the
oracle's restatement, on a bounded row sample of the same sector: first one process, then one
single-threaded process per host core at once (throughput mode).  `ms_per_step` is the wall time of
one sample step; `value` scales the samples to full steps.

N > 1 (torchrun): every rank runs an independent replica of the workload (the path does not shard
within a sector); value = steps of all ranks / max time.
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
# the kernel generation the committed ncu traffic summary was captured on
KERNEL_VERSION = "seg_step_kernel v9"
TRAFFIC_FILE = ROOT / "profiles" / "seg_step_2x14_traffic.txt"


def workload_name(sector) -> str:
    L, nh, nd, kx, ky = sector
    sz2 = 2 * L - nh - 2 * nd
    return (f"2x{L} t-J ladder, {nh} holes, 2Sz={sz2}, k=({kx},{ky}), t=1, J=0.5: "
            "fused Lanczos step over the full sector")


def bench_config(n: int) -> dict:
    """The workload, identical in both arms."""
    L, nh, nd, kx, ky = SECTOR
    return {
        "workload": workload_name(SECTOR),
        "sector": {"num_rungs": L, "num_holes": nh, "num_down_spins": nd, "kx": kx, "ky": ky},
        "n_representatives": int(n),
        "weights": dict(WEIGHTS),
        "start_vector": "np.random.default_rng(0).uniform(-1, 1, n)",
        "l2_policy": f"inputs larger than L2: every vector >= {n * 4 / 1e6:.0f} MB (FP32), no flush",
    }


def peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bytes_per_row(elem: int) -> int:
    """Algorithmic bytes per row of one fused step: the packed 8-byte representative, the orbit byte,
    reading v_k and v_{k-1} and writing v_{k+1}."""
    return 8 + 1 + 3 * elem


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


def ncu_traffic(workload_key: str) -> float | None:
    """DRAM bytes (read + write) of the fused H.v of one step, all its launches, from the committed
    ncu summary captured on this workload and kernel generation; None when it does not cover them."""
    if not TRAFFIC_FILE.exists():
        return None
    fields = {}
    for line in TRAFFIC_FILE.read_text().splitlines():
        if ":" in line and not line.startswith("#"):
            k, v = line.split(":", 1)
            fields[k.strip()] = v.strip()
    if fields.get("workload") != workload_key or fields.get("kernel_version") != KERNEL_VERSION:
        return None
    return float(fields["dram_bytes_per_hv_pass"])


def aggregate_replicas(ms_local: list[float], world: int, device=None) -> tuple[list[float], float]:
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

def _vec(n: int, seed: int, dt, dev):
    import torch

    return torch.as_tensor(np.random.default_rng(seed).uniform(-1, 1, n), device=dev).to(dt)


def step_timing(sec, dt, K: int, W: int, clocks: ClockSampler | None = None, world: int = 1) -> dict:
    """W untimed fused steps, then K timed ones (CUDA events on the launching stream, synchronised on
    both sides; a barrier between ranks).  Returns the total ms of the K steps and each step's H.v ms."""
    import torch

    n, dev = sec.n, sec.device
    buf = [_vec(n, 0, dt, dev), torch.zeros(n, dtype=dt, device=dev)]
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

    for k in range(W):
        step(k)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    lo = clocks.mark() if clocks else 0
    start.record()
    for k in range(W, W + K):
        step(k, evs[k - W])
    stop.record()
    torch.cuda.synchronize()
    out = {"total_ms": start.elapsed_time(stop), "hv_ms": [a.elapsed_time(b) for a, b in evs]}
    if clocks:
        hi = clocks.mark()
        clocks.wait_one_more(hi)
        out["clocks"] = clocks.summary(lo, hi)
    if world > 1:
        torch.distributed.barrier()
    del buf
    return out


def form_rates(sec, dt, K: int, W: int) -> dict:
    """steps/s, H.v GB/s and roofline fraction of one form on a sector (launch tuned first)."""
    import torch

    from exactdiag_gb300 import autotune

    rec = autotune.ensure(sec, WEIGHTS, dt)
    t = step_timing(sec, dt, K, W)
    elem = torch.empty(0, dtype=dt).element_size()
    hv = float(np.mean(t["hv_ms"]))
    gbs = sec.n * bytes_per_row(elem) / (hv * 1e-3) / 1e9
    peak, _ = peaks()
    out = {"dtype": str(dt).replace("torch.", ""), "steps_per_s": 1000.0 * K / t["total_ms"],
           "ms_per_step": t["total_ms"] / K, "hv_ms": hv, "hv_gbs": gbs, "frac": gbs / peak}
    if rec:
        out["launch"] = {k: rec.get(k) for k in ("min_ctas_per_sm", "ctas_per_sm", "rows_per_lane", "staged",
                                                 "window", "chunk_rows")}
    return out


def ground_energy_pair(sec, seed: int, max_steps: int = 400) -> dict:
    """Both forms' converged ground energy and their time to it (launch tuning done beforehand)."""
    from exactdiag_gb300 import autotune
    from exactdiag_gb300.lanczos import ground_state

    for prec in ("fp32", "fp64"):
        autotune.ensure(sec, WEIGHTS, sec.dtype(prec))
    g64 = ground_state(sec, WEIGHTS, max_steps, precision="fp64", seed=seed)
    gmx = ground_state(sec, WEIGHTS, max_steps, precision="mixed", seed=seed)
    return {
        "E0_fp64": g64["E0"], "E0_mixed": gmx["E0"],
        "delta_E_rel": abs(gmx["E0"] - g64["E0"]) / abs(g64["E0"]),
        "time_to_E0_fp64_s": g64["time_s"], "time_to_E0_mixed_s": gmx["time_s"],
        "speedup": g64["time_s"] / gmx["time_s"],
        "steps_fp64": g64["steps"], "steps_fp32": gmx["steps"], "refine_steps_fp64": gmx["refine_steps"],
        "mixed_fp32_stage_s": gmx["time_fp32_s"], "mixed_refine_s": gmx["time_refine_s"],
        "mixed_kept_fp32_vectors": gmx["kept_vectors"], "mixed_residual": gmx["residual"],
    }


def extra_config2(K: int, W: int) -> dict:
    """2x12 two-hole ladder: both forms' rates on a real and a complex sector, ground energy of all 24."""
    import torch

    from exactdiag_gb300.engine import DeviceSector

    out = {"workload": "2x12 t-J ladder, 2 holes, 2Sz=0, all 12 kx x 2 ky sectors, t=1, J=0.5", "rates": []}
    for kx, ky in ((0, 0), (3, 0)):
        sec = DeviceSector(12, 2, 11, kx, ky)
        rec = {"k": [kx, ky], "n": sec.n}
        for prec in ("fp32", "fp64"):
            rec["mixed" if prec == "fp32" else "fp64"] = form_rates(sec, sec.dtype(prec), K, W)
        out["rates"].append(rec)
        sec.close()
    worst, t64, tmx, per = 0.0, 0.0, 0.0, []
    for kx in range(12):
        for ky in (0, 1):
            sec = DeviceSector(12, 2, 11, kx, ky)
            g = ground_energy_pair(sec, seed=0)
            worst = max(worst, g["delta_E_rel"])
            t64 += g["time_to_E0_fp64_s"]
            tmx += g["time_to_E0_mixed_s"]
            per.append({"k": [kx, ky], "n": sec.n, "E0": g["E0_fp64"], "dE_rel": g["delta_E_rel"]})
            sec.close()
            torch.cuda.empty_cache()
    out.update({"worst_delta_E_rel": worst, "all_sectors_time_to_E0_fp64_s": t64,
                "all_sectors_time_to_E0_mixed_s": tmx, "sectors": per})
    return out


def extra_config3(m: int = 150) -> dict:
    """S^z_q targets of the 2x12 two-hole ladder (k = q, all 24): one batched recursion of m steps
    against 24 sequential ones, same seeded start vectors; both return the same coefficients."""
    import torch

    from exactdiag_gb300 import autotune
    from exactdiag_gb300.engine import DeviceSector, batch_lanczos
    from exactdiag_gb300.lanczos import lanczos_coefficients

    secs = [DeviceSector(12, 2, 11, qx, qy) for qx in range(12) for qy in (0, 1)]
    total = sum(s.n for s in secs)
    out = {"workload": f"24 S^z_q target sectors of the 2x12 two-hole ladder, m={m}, seeded start vectors",
           "rows_per_step": total}
    for dt in (torch.complex64, torch.complex128):
        for s in secs:
            autotune.ensure(s, WEIGHTS, dt)
        autotune.ensure(secs[0], WEIGHTS, dt)  # the batch runs with the first sector's launch
        v0s = [_vec(s.n, 100 + i, dt, s.device) for i, s in enumerate(secs)]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        first = batch_lanczos(secs, WEIGHTS, v0s, m)
        t1 = time.perf_counter()
        again = batch_lanczos(secs, WEIGHTS, v0s, m)
        t2 = time.perf_counter()
        seq = [lanczos_coefficients(s, WEIGHTS, v, m) for s, v in zip(secs, v0s)]
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        same = all(np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) for a, b in zip(first, seq))
        same = same and all(np.array_equal(a[0], b[0]) for a, b in zip(first, again))
        steps = sum(len(c[0]) for c in seq)
        out[str(dt).replace("torch.", "")] = {
            "batched_first_call_s": t1 - t0, "batched_replay_s": t2 - t1, "sequential_s": t3 - t2,
            "batched_over_sequential": (t3 - t2) / (t1 - t0),
            "batched_steps_per_s": steps / (t1 - t0), "sequential_steps_per_s": steps / (t3 - t2),
            "coefficients_identical": bool(same)}
        del v0s, first, again, seq
        torch.cuda.empty_cache()
    for s in secs:
        s.close()
    return out


def extra_config5(K: int = 5, W: int = 3) -> dict:
    """2x16 two-hole ladder, k = (0, 0): both forms' rates and ground energy."""
    import torch

    from exactdiag_gb300.engine import DeviceSector

    t0 = time.perf_counter()
    sec = DeviceSector(16, 2, 15, 0, 0)
    torch.cuda.synchronize()
    out = {"workload": "2x16 t-J ladder, 2 holes, 2Sz=0, k=(0,0), t=1, J=0.5", "n": sec.n,
           "sector_build_s": time.perf_counter() - t0}
    for prec in ("fp32", "fp64"):
        out["mixed" if prec == "fp32" else "fp64"] = form_rates(sec, sec.dtype(prec), K, W)
        torch.cuda.empty_cache()
    out.update(ground_energy_pair(sec, seed=0))
    sec.close()
    torch.cuda.empty_cache()
    return out


def e2e_steps(sec, K: int, dt) -> dict:
    """Host-driven steps through the C ABI: the start vector copied from pinned host memory inside
    the timed region, and each step's a_k, b_{k+1} read back to the host after the step."""
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


def run_engine(args, rank: int, world: int) -> dict | None:
    import torch

    from exactdiag_gb300 import autotune
    from exactdiag_gb300.engine import DeviceSector

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    t0 = time.perf_counter()
    sec = DeviceSector(*SECTOR)
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    n = sec.n
    K, W = args.steps, args.warmup

    tuned, timed = {}, {}
    with ClockSampler(dev.index) as clocks:
        clocks.wait_first()
        for prec in ("fp32", "fp64"):
            dt = sec.dtype(prec)
            if args.launch:
                minb, ctas = (int(t) for t in args.launch.split(","))
                autotune.set_launch(sec, minb, ctas)
                tuned[prec] = {"min_ctas_per_sm": minb, "ctas_per_sm": ctas, "grid": autotune.get_launch(sec)[1],
                               "fixed": True}
            else:
                tuned[prec] = autotune.tune(sec, WEIGHTS, dt, use_cache=False)
            timed[prec] = step_timing(sec, dt, K, W, clocks if prec == "fp32" else None, world)
    dt32, dt64 = sec.dtype("fp32"), sec.dtype("fp64")
    (ms_mixed, ms_fp64), value = aggregate_replicas([timed["fp32"]["total_ms"] / K, timed["fp64"]["total_ms"] / K],
                                                    world, dev)

    # roofline of the dominant kernel (the fused H.v of the step, all its launches): algorithmic bytes
    # per launch group over its CUDA-event time
    s32, s64 = (torch.empty(0, dtype=d).element_size() for d in (dt32, dt64))
    hv_ms = float(np.mean(timed["fp32"]["hv_ms"]))
    achieved = n * bytes_per_row(s32) / (hv_ms * 1e-3) / 1e9
    hv64_ms = float(np.mean(timed["fp64"]["hv_ms"]))
    hv64_gbs = n * bytes_per_row(s64) / (hv64_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()

    e2e = None
    if rank == 0:
        if args.launch:
            autotune.set_launch(sec, tuned["fp32"]["min_ctas_per_sm"], tuned["fp32"]["ctas_per_sm"])
        else:
            autotune.apply(sec, tuned["fp32"])
        e2e = e2e_steps(sec, K, dt32)

    extra = {"fp64": {"steps_per_s": world * 1000.0 / ms_fp64, "ms_per_step": ms_fp64, "hv_ms": hv64_ms,
                      "hv_gbs": hv64_gbs, "frac": hv64_gbs / peak},
             "mixed": {"hv_ms": hv_ms, "hv_gbs": achieved, "frac": achieved / peak},
             "mixed_over_fp64_per_step": ms_fp64 / ms_mixed,
             "sector_build_s": t_build,
             "autotune": {p: dict(r) for p, r in tuned.items()},
             "parallelism": "replicas" if world > 1 else "single GPU"}
    if rank == 0 and not args.no_energy:
        g = ground_energy_pair(sec, seed=1)
        extra["time_to_E0"] = g
    launches = K * autotune.step_launches(sec)
    sec.close()
    torch.cuda.empty_cache()
    if rank == 0 and not args.no_extra:
        todo = args.extra.split(",") if args.extra else ["config2", "config3", "config5"]
        if "config2" in todo:
            extra["config2"] = extra_config2(10, 3)
        if "config3" in todo:
            extra["config3"] = extra_config3()
        if "config5" in todo:
            extra["config5"] = extra_config5()

    if rank != 0:
        return None
    time_to_e0 = extra.get("time_to_E0", {})
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
        "config": bench_config(n),
        "precision": "mixed: FP32 vectors and per-term arithmetic, FP64 reductions",
        "fp64_steps_per_s": world * 1000.0 / ms_fp64,
        "time_to_E0_mixed_s": time_to_e0.get("time_to_E0_mixed_s"),
        "time_to_E0_fp64_s": time_to_e0.get("time_to_E0_fp64_s"),
        "delta_E_rel": time_to_e0.get("delta_E_rel"),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": ncu_traffic(workload_name(SECTOR)),
                     "kernel": "fused H.v of the step: seg_step_kernel<float,false,MINB,true,NR> (free blocks) + "
                               "expand_cand_kernel + lanczos_hv_kernel<float,false,4,1> (stabiliser blocks) + "
                               "lanczos_scalars_kernel (ed_lanczos_hv)",
                     "algorithmic_bytes_per_launch": n * bytes_per_row(s32)},
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": timed["fp32"].get("clocks"),
        "extra": extra,
        "cpu_baseline": None if args.no_cpu else cpu_baseline(args),
    }


# ----------------------------------------------------------------------------- CPU reference (oracle port)

class CpuReference:
    """The reference's CPU step on one sector, timed on a bounded row sample (or on every row).

    Setup (untimed): the sector's basis by the oracle; for the sampled rows (`chunks` runs of
    `chunk` consecutive rows at evenly spaced offsets, or every row), each term's stored row in the
    reference's row-major Hermitian-triangle format (entries with column >= row, int16 indices into a
    table of unique values).  A step: a write of a buffer larger than the host's last-level cache
    (untimed, so that no step finds the previous one's rows cached, as a full step would not), then
    the four terms' SpMV over the sampled rows (explicit pass, then the conjugate scatter;
    or_spmv_triangle_rows, one thread) and the vector operations of _lanczos_vec_iteration on
    `vec_sample` elements, each part scaled by n / sample to the full step it stands for.
    """

    FLUSH_BYTES = 256 << 20

    def __init__(self, sector, chunks: int = 32, chunk: int = 16384, vec_sample: int = 4_000_000,
                 every_row: bool = False):
        from oracle import oracle as O

        O.build(ref=False)
        self.lib = O.lib()
        sec = O.Sector(*sector)
        t0 = time.perf_counter()
        sp, orb = O.basis(sec)
        self.t_basis = time.perf_counter() - t0
        self.n = n = len(sp)
        if every_row:
            rows = np.arange(n, dtype=np.int64)
        else:
            starts = np.linspace(0, max(0, n - chunk), max(1, chunks)).astype(np.int64)
            rows = np.unique(np.concatenate([np.arange(s0, min(n, s0 + chunk)) for s0 in starts]))
        self.rows = np.ascontiguousarray(rows, np.int64)
        self.chunks = 1 if every_row else max(1, chunks)
        self.vec_sample = min(vec_sample, n)
        i64p = ctypes.POINTER(ctypes.c_int64)
        f64p = ctypes.POINTER(ctypes.c_double)
        self.mats = []
        t0 = time.perf_counter()
        for t, term in enumerate(O.TERMS):
            nnz = ctypes.c_int64()
            colptr = np.empty(len(self.rows) + 1, np.int64)
            args = (*sec.args(), t, 1, sp.ctypes.data_as(i64p), orb.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                    ctypes.c_int64(n), self.rows.ctypes.data_as(i64p), ctypes.c_int64(len(self.rows)))
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
            del vre, vim, vals
        self.t_matrices = time.perf_counter() - t0
        self.nnz = sum(len(m[2]) for m in self.mats)
        del sp, orb
        self.x = np.random.default_rng(0).uniform(-1, 1, n).astype(np.complex128)
        self.y = np.zeros(n, np.complex128)
        rng = np.random.default_rng(1)
        m = self.vec_sample
        self.vn, self.vnm, self.hvn = (rng.uniform(-1, 1, m).astype(np.complex128) for _ in range(3))
        self.flush = np.zeros(self.FLUSH_BYTES // 8)

    def own_output(self) -> None:
        """A private y and flush buffer (throughput-mode children write their own)."""
        self.y = np.zeros(self.n, np.complex128)
        self.flush = np.zeros(self.FLUSH_BYTES // 8)

    def flush_cache(self) -> None:
        self.flush += 1.0

    def spmv_seconds(self) -> float:
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
        return time.perf_counter() - t0

    def vec_seconds(self) -> float:
        """_lanczos_vec_iteration's vector operations (cython_lanczos_diagonalization.pyx:50-61)."""
        vn, vnm, hvn = self.vn, self.vnm, self.hvn
        t0 = time.perf_counter()
        an = np.real(np.vdot(vn, hvn))
        vnp = hvn - an * vn - 0.5 * vnm
        bnp = np.linalg.norm(vnp)
        vnp /= bnp
        return time.perf_counter() - t0

    def step(self) -> tuple[float, float]:
        """(seconds of this sample step, the full step it stands for); the cache flush before it is
        not counted."""
        self.flush_cache()
        ts = self.spmv_seconds()
        tv = self.vec_seconds()
        return ts + tv, ts * self.n / len(self.rows) + tv * self.n / self.vec_sample

    def sample_text(self) -> str:
        run = len(self.rows) // max(1, self.chunks)
        return (f"{len(self.rows)} rows ({self.chunks} runs of {run} rows at evenly spaced offsets) of the "
                f"{self.n}-row sector, the host cache flushed before each step: SpMV of "
                "the 4 stored term matrices in the reference's row-major Hermitian-triangle passes, plus the "
                f"_lanczos_vec_iteration vector ops on {self.vec_sample} elements, complex128; each part scaled "
                "by n/sample to one full step")


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def mem_available_bytes() -> int | None:
    try:
        for line in pathlib.Path("/proc/meminfo").read_text().splitlines():
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) * 1024
    except OSError:
        pass
    return None


def cpu_baseline(args) -> dict:
    """One single-threaded process of the reference arm's sample steps (the engine line's baseline)."""
    ref = CpuReference(SECTOR, args.cpu_chunks, args.cpu_chunk, args.cpu_vec_sample)
    ref.step()
    steps = [ref.step() for _ in range(3)]
    full = float(np.mean([s[1] for s in steps]))
    return {"value": 1.0 / full, "unit": UNIT, "cores": 1, "kind": "port", "sample": ref.sample_text(),
            "sample_step_s": float(np.mean([s[0] for s in steps])), "setup_basis_s": ref.t_basis}


def _throughput_child(ref: CpuReference, K: int, W: int, barrier, conn) -> None:
    """W + K sample steps in lock step with the other processes: every process flushes its cache,
    then all start the timed part together, and none flushes again before all have finished it (so
    the flushes never overlap another process's timed work)."""
    ref.own_output()
    out = []
    for k in range(W + K):
        ref.flush_cache()
        barrier.wait()
        ts = ref.spmv_seconds()
        tv = ref.vec_seconds()
        barrier.wait()
        if k >= W:
            out.append((ts + tv, ts * ref.n / len(ref.rows) + tv * ref.n / ref.vec_sample))
    conn.send(out)
    conn.close()


def run_reference(args, rank: int) -> dict | None:
    """The reference arm: single process, then throughput mode (one single-threaded process per
    host core, min(sectors, cores, memory), all stepping at once)."""
    if rank != 0:
        return None
    import multiprocessing as mp

    K, W = args.steps, args.warmup
    t_setup = time.perf_counter()
    ref = CpuReference(SECTOR, args.cpu_chunks, args.cpu_chunk, args.cpu_vec_sample)
    t_setup = time.perf_counter() - t_setup
    for _ in range(W):
        ref.step()
    single = [ref.step() for _ in range(K)]
    single_full = float(np.mean([s[1] for s in single]))

    cores = host_cores()
    n_sectors = 2 * SECTOR[0]  # the ladder's (kx, ky) sectors of this filling
    per_child = ref.n * 16 + 6 * ref.vec_sample * 16 + CpuReference.FLUSH_BYTES
    avail = mem_available_bytes()
    procs = min(n_sectors, cores)
    if avail is not None:
        procs = max(1, min(procs, int(0.5 * avail // per_child)))
    # fork: this arm never touches CUDA, and the children share the basis-derived tables read-only
    ctx = mp.get_context("fork")
    barrier = ctx.Barrier(procs + 1)
    pipes, children = [], []
    for _ in range(procs):
        a, b = ctx.Pipe(duplex=False)
        p = ctx.Process(target=_throughput_child, args=(ref, K, W, barrier, b))
        p.start()
        pipes.append(a)
        children.append(p)
    # the parent keeps step with the children (two barriers per step) and times the K timed steps
    for k in range(W + K):
        if k == W:
            t0 = time.perf_counter()
        barrier.wait()
        barrier.wait()
    wall = time.perf_counter() - t0
    results = [a.recv() for a in pipes]
    for p in children:
        p.join()
    child_full = [float(np.mean([s[1] for s in r])) for r in results]
    value = sum(1.0 / f for f in child_full)  # full-sector steps/s of all processes together
    sample_ms = 1000.0 * wall / K
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": W,
        "ms_per_step": sample_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128", "data": "synthetic", "impl": "reference",
        "config": bench_config(ref.n),
        "precision": "complex128 (the reference's value type)",
        "timing": {
            "ms_per_step_is": "wall time of one sample step of the throughput run (all processes at once, "
                              "each flushing its cache before the step); K of them are the timed region",
            "value_is": f"sum over {procs} processes of 1 / (their mean full-step time, each sample step scaled "
                        "by n/sample)",
            "full_step_s_throughput_mean": float(np.mean(child_full)),
            "single_process_steps_per_s": 1.0 / single_full,
            "single_process_full_step_s": single_full,
            "single_process_sample_step_ms": 1000.0 * float(np.mean([s[0] for s in single])),
            "processes": procs, "host_cores": cores, "sectors_of_this_filling": n_sectors,
            "setup_s": t_setup, "nnz_sampled": ref.nnz,
        },
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                         "sample": ref.sample_text() + f"; throughput mode: {procs} single-threaded processes "
                         f"on {cores} host cores, each stepping its own copy of the output vector (the reference's "
                         "multi-threaded SpMV races, so one thread per process)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--no-energy", action="store_true", help="skip the time-to-E0 runs")
    ap.add_argument("--no-extra", action="store_true", help="skip the 2x12 and 2x16 workloads")
    ap.add_argument("--extra", default=None, help="comma list of config2,config3,config5 (default: all)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-chunks", type=int, default=32, help="runs of consecutive rows in the CPU sample")
    ap.add_argument("--cpu-chunk", type=int, default=16384, help="rows per run of the CPU sample")
    ap.add_argument("--cpu-vec-sample", type=int, default=4_000_000)
    ap.add_argument("--sector", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--launch", default=None, metavar="MINB,CTAS",
                    help="fix the free-row step kernel's launch (register variant 2|3|4, CTAs per SM, 0 = all "
                         "that fit) instead of tuning it")
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
