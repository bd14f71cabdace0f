"""The request server's output arena allocator (csrc/nbg_arena.hpp), host only:
a randomised C++ check against a brute-force model (first fit, no overlap,
merged free runs, exact used count, whole again after releasing all)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "nbodygradient.jl_gb300", "csrc")


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_arena_against_model(tmp_path):
    exe = str(tmp_path / "arena_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", CSRC, os.path.join(HERE, "native", "arena_check.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout
