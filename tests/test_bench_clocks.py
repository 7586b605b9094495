"""The bench's clock record: nvidia-smi lines and NVML samples reduce to the median SM
clock under load and the union of the throttle reasons seen (no GPU needed)."""
import bench


def test_nvidia_smi_lines_only():
    c = bench.ClockSampler(0)
    c.lines = ["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
               "0, 2055, 2070, 1200.5, 0x4, Not Active, Not Active, Not Active, Active",
               "garbage"]
    s = c.summary()
    assert s["samples"] == 2 and s["sm_mhz"] == 2062.5 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]


def test_nvml_samples_take_precedence_and_reasons_merge():
    c = bench.ClockSampler(0)
    c.lines = ["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active"]
    c.nv = [(2070.0, 0), (2040.0, 0x4), (2070.0, 0x8 | 0x1)]
    c.nv_max = 2070.0
    s = c.summary()
    assert s["samples"] == 3 and s["sm_mhz"] == 2070.0 and s["sm_min_mhz"] == 2040.0
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]
    assert s["nvidia_smi"] == {"sm_mhz": 2070.0, "samples": 1}


def test_nvml_index_follows_visible_devices(monkeypatch):
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "5,3")
    assert bench.ClockSampler(1)._nvml_index() == 3
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "GPU-abc")
    assert bench.ClockSampler(1)._nvml_index() == 1


def test_short_region_falls_back_to_bracketing_samples():
    c = bench.ClockSampler(0)
    c.lines = ["0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active"]
    c.bracket = [(2070.0, 0), (2055.0, 0x20)]
    s = c.summary()
    assert s["samples"] == 2 and s["sm_mhz"] == 2062.5 and s["reasons"] == ["sw_thermal_slowdown"]
    assert "before and just after" in s["source"]
