"""Checks the reference arm's CPU timing (TEST INFRASTRUCTURE ONLY; needs the reference tree).

On one sector small enough to store whole (default: 2x12, two holes, k = (0, 0), 8.1e6 rows):

1. every row of the four term matrices in the reference's row-major Hermitian-triangle storage;
2. one SpMV pass per term by the reference's own code -- general/cpp_sparse_dot.h:59-71 and
   :104-138 as general/cython_sparse_dot.pyx:40-80 calls them at num_threads = 1, compiled from the
   reference tree into oracle/_ref (ref_sparse_matrix_dot_row_major) -- and by the oracle's
   restatement (or_spmv_triangle_rows, what bench.py's reference arm runs), on the same rows and
   vectors; their outputs must agree bit for bit and their times are compared;
3. one full CPU step (the four SpMVs plus _lanczos_vec_iteration's vector operations on n
   elements) against the full-step time bench.py extrapolates from its row sample.

    EXACTDIAG_REF_SRC=<reference>/src/exactdiag python oracle/cpu_step_check.py [--sector 12,2,11,0,0]

Prints one JSON line.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import pathlib
import sys
import time

import numpy as np

# the repository root in place of this script's folder (whose oracle.py would shadow the package)
sys.path[0] = str(pathlib.Path(__file__).resolve().parent.parent)

from bench import WEIGHTS, CpuReference  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--sector", default="12,2,11,0,0")
    ap.add_argument("--repeats", type=int, default=7)
    args = ap.parse_args()
    sector = tuple(int(v) for v in args.sector.split(","))
    O.build(ref=True)
    ref = O.ref_lib()
    if ref is None:
        raise SystemExit("oracle/_ref is not built (set EXACTDIAG_REF_SRC)")
    ref.ref_sparse_matrix_dot_row_major.restype = ctypes.c_int

    full = CpuReference(sector, every_row=True, vec_sample=1 << 62)
    sample = CpuReference(sector)
    n, nnz = full.n, full.nnz
    i64p = ctypes.POINTER(ctypes.c_int64)
    vp = ctypes.c_void_p
    y_ref = np.zeros(n, np.complex128)

    def reference_spmv() -> float:
        y_ref[:] = 0
        t0 = time.perf_counter()
        for term, colptr, cols, vidx, vals in full.mats:
            rc = ref.ref_sparse_matrix_dot_row_major(
                ctypes.c_int64(n), colptr.ctypes.data_as(i64p), cols.ctypes.data_as(i64p),
                vidx.ctypes.data_as(ctypes.POINTER(ctypes.c_int16)), vp(vals.ctypes.data), vp(full.x.ctypes.data),
                vp(y_ref.ctypes.data), ctypes.c_double(WEIGHTS[term]), ctypes.c_double(0.0))
            assert rc == 0
        return time.perf_counter() - t0

    # interleaved repeats (this host's timings drift): each a flushed cache, then one measurement
    t_ref, t_port, t_vec, est = [], [], [], []
    identical = True
    sample.step()
    for rep in range(args.repeats):
        full.flush_cache()
        t_ref.append(reference_spmv())
        full.y[:] = 0
        full.flush_cache()
        t_port.append(full.spmv_seconds())
        identical = identical and bool(np.array_equal(y_ref, full.y))
        full.flush_cache()
        t_vec.append(full.vec_seconds())  # _lanczos_vec_iteration's vector operations on n elements
        est.append(sample.step()[1])
    med = lambda v: float(np.median(v))  # noqa: E731
    measured_full_step = med(t_port) + med(t_vec)
    measured_full_step_ref = med(t_ref) + med(t_vec)
    extrapolated = med(est)
    print(json.dumps({
        "sector": sector, "n": n, "nnz_stored": nnz,
        "repeats": args.repeats,
        "reference_spmv_s": med(t_ref), "port_spmv_s": med(t_port),
        "port_over_reference_time": med(t_port) / med(t_ref),
        "outputs_bit_identical": identical,
        "vector_ops_full_s": med(t_vec),
        "full_step_measured_port_s": measured_full_step,
        "full_step_measured_reference_spmv_s": measured_full_step_ref,
        "full_step_extrapolated_s": extrapolated,
        "extrapolation_error": extrapolated / measured_full_step - 1.0,
        "extrapolation_error_vs_reference_code": extrapolated / measured_full_step_ref - 1.0,
        "sample": sample.sample_text(),
        "threads": 1,
    }))


if __name__ == "__main__":
    main()
