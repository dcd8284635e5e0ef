"""Host-side pieces of bench.py: the byte counts behind the roofline fields and the
ncu traffic figure of the default configuration (no GPU needed)."""

import pytest

import bench


def test_algorithmic_bytes_formula():
    # B = 2(8r + 4) + 4(2 + 2 S_total + P_seg + 1) with S_total = 11, P_seg = 5.
    assert bench.algorithmic_bytes_per_segment_step(1.0) == 2 * 12 + 4 * (2 + 22 + 5 + 1)
    assert bench.algorithmic_bytes_per_segment_step(302.5) == pytest.approx(2 * (8 * 302.5 + 4) + 120)


def test_format_bytes_add_the_step_state_to_the_stored_propagator():
    # Per half step: the row's stored propagator bytes + V r/w, kI, kG, 3 HH gates,
    # 3 HH coefficients, na8 open state and coefficient (4 B each); per step the
    # mechanism pass reads V and reads + writes 11 states.
    assert bench.format_bytes_per_segment_step(0.0) == 2 * 12 * 4 + 4 + 2 * 11 * 4
    # A row of 100 stored 4 B values with u16 columns, an 8 B row pointer and the leak.
    b = bench.format_bytes_per_segment_step(100 * 6 + 8 + 4)
    assert b - bench.format_bytes_per_segment_step(0.0) == 2 * (100 * 6 + 12)


def _defaults():
    """The parser's defaults, read from bench.main's argument definitions."""
    import inspect
    import re
    src = inspect.getsource(bench.main)
    fmt = re.search(r'"--format", default="(\w+)"', src).group(1)
    tol = float(re.search(r'"--tol", type=float, default=([0-9.e-]+)\)', src).group(1))
    lump = int(re.search(r'"--lump", type=int, default=(\d)', src).group(1))
    return fmt, tol, lump


def test_default_configuration_has_an_ncu_traffic_figure():
    assert _defaults() in bench.NCU_TRAFFIC_PER_SEGMENT_STEP


def test_both_arms_name_the_same_workload():
    name = bench.workload_name(1024, 500, 20000)
    assert name.startswith("batched: 1024 neurons, log-uniform 500-20000 segments")


def test_wide_bytes_count_windows_rows_and_state():
    # Per half step: 20 B per quad window (16 B values + 4 B base), row pointer (8 B)
    # and leak, x, kG and kI read, next x and V written; with calcium 8 B per stored
    # entry, its row pointer and leak, scratch read, c and next scratch written; per
    # step the HH gates (read and written) with their 3 coefficients, and the calcium
    # pump's 3 states (read and written), dc/dt and the influx and efflux coefficients.
    no_ca = bench.wide_bytes_per_segment_step(0.0, 0.0, calcium=False)
    assert no_ca == 2 * (8 + 4 + 12 + 8) + 2 * 12 + 12
    assert bench.wide_bytes_per_segment_step(10.0, 0.0, calcium=False) - no_ca == 2 * 10 * 20
    ca = bench.wide_bytes_per_segment_step(0.0, 0.0)
    assert ca - no_ca == 2 * (8 + 4 + 12) + 2 * 12 + 12
    assert bench.wide_bytes_per_segment_step(0.0, 5.0) - ca == 2 * 5 * 8
