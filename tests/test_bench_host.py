"""bench.py's clock record on the CPU: the summary of nvidia-smi rows (SM
clock median and maximum, the throttle reasons seen as Active during the timed
region), from rows written as nvidia-smi writes them, without a GPU."""
import bench


def _row(sm, mx, hw="Not Active", hwt="Not Active", swt="Not Active", cap="Not Active"):
    return [x.strip() for x in f"0, {sm}, {mx}, 612.40, 0x0000000000000000, {hw}, {hwt}, {swt}, {cap}".split(",")]


def _summary(rows):
    s = bench.ClockSampler()
    s.rows = rows
    return s.summary()


def test_clean_run():
    s = _summary([_row(2070, 2070), _row(2070, 2070), _row(2055, 2070)])
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 3}


def test_throttle_reasons_are_reported():
    s = _summary([_row(2070, 2070), _row(1800, 2070, hw="Active"), _row(1900, 2070, cap="Active"),
                  _row(1700, 2070, hwt="Active", swt="Active")])
    assert s["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_power_cap", "sw_thermal_slowdown"]
    assert s["sm_mhz"] == 1850.0 and s["samples"] == 4


def test_unreadable_values_and_no_rows():
    s = _summary([_row("[N/A]", "[N/A]"), _row(2070, 2070)])
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert _summary([])["reasons"] == ["nvidia-smi unavailable"]
