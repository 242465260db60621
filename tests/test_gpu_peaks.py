"""The device-peak microbenchmark (include/wavetorch_gb300_testing.h,
wt_test_device_peaks) that gives the fused kernels' roofline its
denominators: FP32 FFMA issue rate and shared-memory load bandwidth."""
import pytest

pytestmark = pytest.mark.gpu


def test_device_peaks_are_plausible(cuda):
    """The FFMA rate lies between half and all of the SMs' 128 FP32 lanes per
    clock at the clock the kernel measured; the shared-memory rate is of the
    order of 128 bytes per clock per SM."""
    import bench
    p = bench.device_peaks(cuda)
    assert p["sm_count"] > 0 and 500 < p["sm_mhz"] < 3000
    lanes = p["sm_count"] * 128 * p["sm_mhz"] * 1e6
    assert 0.5 * lanes < p["ffma_per_s"] <= 1.05 * lanes
    assert abs(p["warp_inst_per_s"] * 32 - p["ffma_per_s"]) < 1e-6 * p["ffma_per_s"]
    assert 0.3 * lanes < p["smem_bytes_per_s"] <= 4 * lanes
