"""The FP64 issue-rate diagnostic (xJPCG_gbDiagFp64Rate), the ceiling the
fp64 kernels are held against: it must report a rate of the right order for a
GB300 (nominal 1.25 TFLOP/s fp64 = 0.63 T DFMA/s) and scale with the work."""
import pytest

import hpc_gb300 as X

pytestmark = pytest.mark.gpu


def test_fp64_rate_is_plausible(handle):
    rate, ms = handle.fp64_rate(16384)
    assert ms > 0.0
    assert 0.2e12 < rate < 2.0e12
    rate2, ms2 = handle.fp64_rate(4096)
    assert 0.5 * rate < rate2 < 1.5 * rate  # same rate on a quarter of the work
    assert ms2 < ms


def test_fp64_rate_rejects_bad_arguments(handle):
    with pytest.raises(X.XJPCGError):
        handle.fp64_rate(0)
