"""CPU: host-side logic of bench.py -- the DRAM-traffic figure of the committed capture and the
clock samples of the timed region."""

import pytest


def test_traffic_read_only_for_the_captured_workload_and_kernel(tmp_path, monkeypatch):
    import bench

    key = bench.workload_name(bench.SECTOR)
    f = tmp_path / "traffic.txt"
    f.write_text(f"# ncu summary\nworkload: {key}\nkernel_version: {bench.KERNEL_VERSION}\n"
                 "dram_bytes_per_hv_pass: 3.5e9\n")
    monkeypatch.setattr(bench, "TRAFFIC_FILE", f)
    assert bench.ncu_traffic(key) == pytest.approx(3.5e9)
    assert bench.ncu_traffic("another workload") is None
    f.write_text(f"workload: {key}\nkernel_version: an older kernel\ndram_bytes_per_hv_pass: 1\n")
    assert bench.ncu_traffic(key) is None
    monkeypatch.setattr(bench, "TRAFFIC_FILE", tmp_path / "absent.txt")
    assert bench.ncu_traffic(key) is None


def test_committed_traffic_summary_matches_the_bench_workload():
    import bench

    if not bench.TRAFFIC_FILE.exists():
        pytest.skip("no traffic capture committed for this kernel generation")
    assert bench.ncu_traffic(bench.workload_name(bench.SECTOR)) is not None


def test_cpu_reference_every_row_spmv_equals_the_oracle_hamiltonian():
    """The reference arm's stored-triangle SpMV over every row is H x (the oracle's matrix)."""
    import numpy as np

    import bench
    from oracle import oracle as O

    sector = (5, 2, 4, 1, 0)
    ref = bench.CpuReference(sector, every_row=True, vec_sample=1000)
    ref.y[:] = 0
    ref.spmv_seconds()
    sec = O.Sector(*sector)
    bas = O.basis(sec)
    h = O.hamiltonian(sec, bench.WEIGHTS, bas)
    want = h @ ref.x
    assert np.allclose(ref.y, want, rtol=0, atol=1e-12 * np.max(np.abs(want)))


def test_cpu_reference_sample_scales_to_a_full_step():
    import bench

    ref = bench.CpuReference((6, 2, 5, 0, 0), chunks=4, chunk=64, vec_sample=500)
    assert len(ref.rows) == 256 and ref.rows[0] == 0 and ref.rows[-1] == ref.n - 1
    wall, full = ref.step()
    assert 0 < wall and full > wall


def test_clock_summary_counts_only_the_marked_window():
    import bench

    s = bench.ClockSampler(0)
    line = "0, {mhz}, 2070, 800.0, 0x0, {hw}, Not Active, Not Active, {cap}"
    s.lines = [line.format(mhz=1200, hw="Active", cap="Not Active"),  # during the warm-up
               line.format(mhz=2070, hw="Not Active", cap="Not Active"),
               line.format(mhz=2055, hw="Not Active", cap="Active"),
               line.format(mhz=2070, hw="Not Active", cap="Not Active"),  # first sample after the region
               line.format(mhz=900, hw="Active", cap="Not Active")]
    out = s.summary(1, 3)
    assert out["samples"] == 3
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]
    whole = s.summary()
    assert whole["samples"] == 5 and "hw_slowdown" in whole["reasons"]


def test_clock_sampler_without_nvidia_smi_reports_no_samples():
    import bench

    s = bench.ClockSampler(0)
    s.wait_first(timeout_s=0.01)  # no process: returns at once
    assert s.summary(s.mark(), s.mark())["samples"] == 0
