"""CPU: host-side logic of bench.py -- the DRAM-traffic figure of the committed capture and the
clock samples of the timed region."""

import pytest


def test_traffic_scales_per_kind_rows_of_the_bench_workload():
    import bench

    key = bench.workload_name(bench.SECTOR)
    fields = {}
    for line in (bench.ROOT / "profiles" / "lanczos_hv_2x14_traffic.txt").read_text().splitlines():
        if ":" in line and not line.startswith("#"):
            k, v = line.split(":", 1)
            fields[k.strip()] = v.strip()
    assert fields["workload"] == key
    assert fields["kernel_version"] == bench.KERNEL_VERSION
    free, stab = float(fields["dram_bytes_per_row_free"]), float(fields["dram_bytes_per_row_stabiliser"])
    rows = (1000, 10, 0)
    assert bench.ncu_traffic(key, rows) == pytest.approx(1000 * free + 10 * stab)
    # bytes per row above the algorithmic 20 (key, v_k, v_{k-1}, y): the gathers' misses
    assert free >= 20 and stab >= 20
    assert bench.ncu_traffic("another workload", rows) is None


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
