"""The SpMV host classes (include/spmvHost_gb300.hpp) compile into an
application that links against libXilinxPcg.so.  CPU only: the application is
built, not run (its run is tests/test_gpu_spmv_host.py)."""
import subprocess

import pytest

from spmv_host_util import build_app

pytestmark = pytest.mark.skipif(subprocess.run(["which", "g++"], capture_output=True).returncode != 0,
                                reason="needs g++")


def test_spmv_host_app_builds(tmp_path):
    exe = build_app(str(tmp_path))
    out = subprocess.run(["nm", "-u", exe], capture_output=True, text=True, check=True).stdout
    for sym in ("xJPCG_gbCreateHandleOnDevice", "xJPCG_gbSetSignatureMatrix", "xJPCG_gbSignatureSpmv",
                "xJPCG_gbStoreYFrames"):
        assert sym in out
