"""The roofline denominators measured on the device (gbde_measure_fma_peak):
FP64 and FP32 FMA throughput, and the rate of the SDE kernels' FP32 normal
stream.  Checked for plausibility on GB300 (FP32 far above FP64, a normal
stream far below the FP32 FMA rate) and for the rejection of unknown kinds."""
import pytest


@pytest.mark.gpu
def test_measured_peaks(capi):
    ctx = capi.context(0)
    fp64, fp32, normals = ctx.fma_peak(0), ctx.fma_peak(1), ctx.fma_peak(2)
    assert 0.1 < fp64 < 100.0          # TFLOP/s
    assert fp32 > 10.0 * fp64
    assert 1e-3 < normals < fp32        # 10^12 normals/s
    with pytest.raises(capi.GBDEError):
        ctx.fma_peak(3)
