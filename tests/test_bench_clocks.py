"""bench.py's clock record: nvidia-smi samples taken during the timed region
are reduced to the median SM clock, the maximum clock and power, and the
throttle reasons seen active (a run with a thermal or hardware slowdown is
not a valid measurement)."""
import bench


class _Done:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def sampler_over(tmp_path, text):
    path = tmp_path / "clocks.csv"
    path.write_text(text)
    s = bench.ClockSampler.__new__(bench.ClockSampler)
    s.path = str(path)
    s.fh = open(path, "a")
    s.proc = _Done()
    return s


def test_clean_samples(tmp_path):
    rows = "\n".join(f"{mhz}, 2070, {w}, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"
                     for mhz, w in ((2070, 410.5), (2055, 420.0), (2070, 415.0)))
    out = sampler_over(tmp_path, rows + "\n").stop()
    assert out == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "power_w_max": 420.0, "samples": 3, "reasons": []}
    assert not (tmp_path / "clocks.csv").exists()


def test_reasons_are_reported(tmp_path):
    rows = ["1800, 2070, 1390.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
            "1650, 2070, 1400.0, 0x0000000000000048, Not Active, Active, Not Active, Not Active",
            "garbage line"]
    out = sampler_over(tmp_path, "\n".join(rows) + "\n").stop()
    assert out["samples"] == 2
    assert out["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert out["sm_mhz"] == 1725.0


def test_no_samples(tmp_path):
    assert sampler_over(tmp_path, "").stop() is None
