"""bench.py host logic without a GPU: the clock summary of the timed region
and the workload config shared by both arms."""
import bench


def _row(mhz, hw_slowdown="Not Active"):
    return [str(mhz), "2070", "500.0", "0x0", hw_slowdown, "Not Active", "Not Active", "Not Active"]


def test_clock_summary_keeps_the_timed_window():
    c = bench.ClockSampler(0)
    c.rows = [(0.0, _row(1000, "Active")), (1.0, _row(2070)), (1.2, _row(2065)), (5.0, _row(900))]
    s = c.summary(0.9, 1.1)  # a sample arrives up to one period late: [0.9, 1.35]
    assert s["samples"] == 2 and s["sm_mhz"] == 2067.5 and s["reasons"] == []
    assert s["window"] == "timed region" and s["sm_max_mhz"] == 2070
    s = c.summary(3.0, 3.1)  # nothing inside: every sample, said so
    assert s["samples"] == 4 and s["reasons"] == ["hw_slowdown"] and s["window"].startswith("sampler run")
    assert bench.ClockSampler(0).summary(0.0, 1.0)["reasons"] == ["unsampled"]


def test_both_arms_share_the_config():
    a = bench.config_of("mixed_8m", 8_000_000, 8_000_000)
    assert a == bench.config_of("mixed_8m", 8_000_000, 8_000_000)
    assert a["workload"] == "mixed_8m" and a["k"] == 32 and a["basis"] == "Quadratic3" and a["rbf"] == "Wendland<4>"
