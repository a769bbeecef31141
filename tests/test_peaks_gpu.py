"""oh_measure_issue_peaks: the compute-side roofline denominators measured
on the GPU (scalar and packed FP32 FMA issue rates, sin.approx results)."""
import pytest

from openholo_gb300 import _lib

pytestmark = pytest.mark.gpu


def test_issue_peaks_are_plausible(ctx):
    pk = _lib.measure_issue_peaks(0)
    # four FMA warp instructions per SM per clock at some clock between 0.5 and 2.5 GHz
    assert 500 < pk["sm_mhz_implied"] < 2500
    assert pk["ffma2_warp_inst_per_s"] > 0.4 * pk["ffma_warp_inst_per_s"]
    # the multi-function unit runs well below the FMA lanes
    assert 0 < pk["mufu_per_s"] < 32 * pk["ffma_warp_inst_per_s"]
