"""CPU tests of the bench's host logic: the clock record taken during the
timed region (median SM clock, the throttle reasons seen) from nvidia-smi's
CSV, and the per-group roofline table (algorithmic bytes over event time
against the HBM peak, FP64-pipe fractions from the per-point op counts)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


class _Proc:
    """stands in for the nvidia-smi process the sampler started"""
    def terminate(self):
        pass

    def wait(self, t=None):
        return 0


def _sampled(tmp_path, lines):
    c = bench.Clocks(0)
    c.path = str(tmp_path / "clocks.csv")
    with open(c.path, "w") as f:
        f.write("\n".join(lines) + "\n")
    c.fh = open(c.path, "a")
    c.p = _Proc()
    return c.stop()


def test_clock_record_median_and_reasons(tmp_path):
    na, act = "Not Active", "Active"
    rows = ["0, %d, 2070, 900.5, 0x0, %s, %s, %s, %s" % (mhz, na, na, na, cap)
            for mhz, cap in ((2070, na), (2055, act), (1980, na), (2070, na), (2040, act))]
    rows.insert(2, "garbage line")
    rows.append("0, [N/A], 2070, 0, 0x0, %s, %s, %s, %s" % (na, na, na, na))
    out = _sampled(tmp_path, rows)
    assert out["samples"] == 5
    assert out["sm_mhz"] == 2055.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]


def test_clock_record_flags_thermal_slowdown(tmp_path):
    out = _sampled(tmp_path, ["0, 1800, 2070, 1300, 0x60, Not Active, Active, Not Active, Active"])
    assert out["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]


def test_clock_record_without_sampler():
    c = bench.Clocks(0)
    c.p = None
    assert c.stop() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_group_table_fractions():
    prof = {"mg": (200.0, 1000), "eno_yz": (100.0, 20), "net": (0.0, 0)}
    pbytes = {"mg": 1.0e12, "eno_yz": 2.0e11}
    npts = 1.0e7
    t = bench.group_table(prof, pbytes, peak_hbm=6000.0, fp64_rate=5.0e11, npts=npts, ncell=npts)
    assert t["mg"]["gbs"] == pytest.approx(1000.0 / 0.2)
    assert t["mg"]["hbm_frac"] == pytest.approx(5000.0 / 6000.0)
    assert "fp64_frac" not in t["mg"]
    ops = bench.FP64_OPS["eno_yz"]
    assert t["eno_yz"]["fp64_frac"] == pytest.approx(ops * npts * 20 / 0.1 / 5.0e11)
    assert t["net"] == {"ms": 0.0, "launches": 0, "gbytes": 0.0}
