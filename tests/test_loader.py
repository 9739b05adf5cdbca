"""The dlopen loader (libXilinxPcg_loader.a, hpc_gb300/csrc/pcg_loader.c)
against the behaviour of the reference's pcg/sw/src/pcg_loader.c: a C
application linked with the loader instead of the library.  CPU only: no call
here launches device work."""
from __future__ import annotations

import os
import subprocess

import pytest

from loader_util import INCLUDE, LIBDIR, build_app, fields, run_app

pytestmark = pytest.mark.skipif(subprocess.run(["which", "gcc"], capture_output=True).returncode != 0,
                                reason="needs gcc")


@pytest.fixture(scope="module")
def app(tmp_path_factory):
    from hpc_gb300 import build as B
    B.build_library()
    return build_app(str(tmp_path_factory.mktemp("loader")))


def test_library_absent_gives_dynamic_loading_error(app, tmp_path):
    r = run_app(app, ["errstr"], str(tmp_path))  # an empty directory: the library cannot be found
    f = fields(r.stdout)
    assert r.returncode == 0
    assert f["str6"] == "Dynamic"  # "Dynamic loading error", answered by the loader itself
    assert "Dynamic loading error" in r.stdout
    assert "unavailable" in r.stdout  # str3 could not reach the library
    assert f["peek"] == "6"  # the stored loading error, reported without the library
    assert "cannot open libXilinxPcgStatic.so" in r.stdout
    r = run_app(app, ["create"], str(tmp_path))
    assert fields(r.stdout)["create"] == "6"


def test_library_present_forwards_calls(app):
    r = run_app(app, ["errstr"], LIBDIR)
    f = fields(r.stdout)
    assert r.returncode == 0
    assert f["str3"] == "XJPCG_STATUS_INVALID_VALUE"
    assert "Dynamic loading error" in r.stdout
    # the library's own answer for a null handle (pcg.cpp:185-189)
    assert f["peek"] == "1"


def test_missing_symbol_gives_dynamic_loading_error(app, tmp_path):
    stub = os.path.join(str(tmp_path), "libXilinxPcgStatic.so")
    subprocess.run(["gcc", "-shared", "-fPIC", "-I" + INCLUDE, os.path.join(os.path.dirname(__file__), "c",
                                                                             "stub_library.c"), "-o", stub],
                   check=True)
    r = run_app(app, ["errstr"], str(tmp_path))
    assert fields(r.stdout)["str3"] == "stub"
    r = run_app(app, ["create"], str(tmp_path))
    f = fields(r.stdout)
    assert f["create"] == "6"
    assert "cannot find symbol xJPCG_createHandle" in r.stdout


def test_loader_exports_the_api():
    from hpc_gb300 import build as B
    loader = B.build_loader()
    out = subprocess.run(["nm", "-g", "--defined-only", loader], capture_output=True, text=True, check=True).stdout
    names = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert names == {"xJPCG_createHandle", "xJPCG_destroyHandle", "xJPCG_getMetrics", "xJPCG_peekAtLastStatus",
                     "xJPCG_getLastMessage", "xJPCG_getErrorString", "xJPCG_cscSymSolver", "xJPCG_cooSolver"}
