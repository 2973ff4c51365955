"""Host-side pieces of bench.py (no GPU): the figures the bench line copies from the committed ncu
summaries exist and parse, the algorithmic byte model is the one the roofline divides by, and both
arms of the bench describe their workload with the same config object."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def bench():
    sys.path.insert(0, str(ROOT))
    import bench as b

    return b


@pytest.mark.parametrize("kernel", ["k_pair32", "k_pair64"])
def test_profile_figures_of_the_roofline_kernels_exist(bench, kernel):
    traffic, src = bench.load_traffic(kernel)
    assert src is not None and (ROOT / src).is_file()
    assert traffic is not None and traffic > 1e8  # bytes per launch of a full-size capture
    issue, src2 = bench.load_profile_value("issue_active_pct", kernel)
    assert src2 == src and 0.0 < issue <= 100.0


def test_fp32_pair_profile_reports_the_l1_figure(bench):
    l1, src = bench.load_profile_value("l1tex_throughput_pct", "k_pair32")
    assert src is not None and 0.0 < l1 <= 100.0


def test_byte_model(bench):
    # compulsory bytes per RHS stage: FP64 352 B per fluid + 88 B per wall particle, FP32 248 + 56;
    # the pair kernel's share (pair + fused update) of it
    assert bench.BYTES_STAGE == {"float64": (352, 88), "float32": (248, 56)}
    for prec in ("float64", "float32"):
        pf, pw = bench.BYTES_PAIR[prec]
        sf, sw = bench.BYTES_STAGE[prec]
        assert 0 < pf <= sf and 0 < pw <= sw


def test_both_arms_share_the_config_object(bench):
    a = bench.workload_config(bench.CFG1, 968750, 876666)
    b = bench.workload_config(bench.CFG1, 968750, 876666)
    assert a == b
    assert a["particles"] == 968750 + 876666
    assert a["dx"] == 0.008 and a["dt"] == 5e-5


def test_measured_peak_is_used(bench):
    peak, kind = bench.load_peaks()
    if (ROOT / "MEASURED_PEAKS.json").exists():
        assert kind == "measured" and peak > 1000.0
    else:
        assert kind == "fallback" and peak == 6800.0
