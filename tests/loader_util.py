"""Builds the loader test application (tests/c/loader_app.c linked against
libXilinxPcg_loader.a) for the loader tests."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "hpc_gb300")


def build_app(outdir: str) -> str:
    from hpc_gb300 import build as B
    loader = B.build_loader()
    exe = os.path.join(outdir, "loader_app")
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-I" + INCLUDE, os.path.join(HERE, "c", "loader_app.c"),
                    loader, "-ldl", "-lm", "-o", exe], check=True)
    return exe


def run_app(exe: str, args, libdir: str | None, timeout: int = 300) -> subprocess.CompletedProcess:
    env = dict(os.environ)
    env["LD_LIBRARY_PATH"] = libdir or ""
    return subprocess.run([exe] + list(args), env=env, capture_output=True, text=True, timeout=timeout)


def fields(text: str) -> dict:
    out = {}
    for line in text.splitlines():
        for tok in line.split(" "):
            if "=" in tok:
                k, v = tok.split("=", 1)
                out.setdefault(k, v)
    return out
