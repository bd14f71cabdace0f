"""The C ABI library: it builds, loads, exports every symbol include/nbg.h
declares, and reports errors cleanly (these checks need no GPU)."""
import ctypes
import os
import re
import subprocess

import pytest

import nbg
from conftest import ROOT, has_gpu

HEADER = os.path.join(ROOT, "include", "nbg.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nbg_[a-z0-9_]+)\s*\(", src)))


def test_header_declarations_match_binding():
    decl = declared_functions()
    assert decl, "no declarations found"
    assert sorted(nbg._lib.EXPORTS) == decl


def test_library_exports_every_declared_symbol():
    path = nbg.build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (nbg_[a-z0-9_]+)$", out, flags=re.M))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    L = nbg._lib.load()
    for f in declared_functions():
        assert hasattr(L, f)


def test_built_for_sm_103a():
    path = nbg.build.build()
    out = subprocess.run(["cuobjdump", "--list-elf", path], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump not available")
    assert "sm_103a" in out.stdout


def test_version_and_error_buffer():
    L = nbg._lib.load()
    assert L.nbg_version() >= 100
    buf = ctypes.create_string_buffer(64)
    assert L.nbg_last_error(buf, 64) == 0
    assert L.nbg_last_error(None, 0) == nbg._lib.NBG_EINVAL


def test_null_arguments_are_rejected_without_a_gpu():
    L = nbg._lib.load()
    assert L.nbg_set_tuning(None, 16, 0) == nbg._lib.NBG_EINVAL
    assert L.nbg_last_timing(None, None, None, None, None) == nbg._lib.NBG_EINVAL
    assert L.nbg_integrate_transits(None, 3, 0, 0.5, 10.0, 1, *([None] * 11), 10, None, None, None, None) \
        == nbg._lib.NBG_EINVAL
    assert "NULL" in nbg._lib.last_error()


@pytest.mark.skipif(has_gpu(), reason="checks the no-GPU error path")
def test_context_creation_fails_loudly_without_gpu():
    with pytest.raises(nbg.NbgError):
        nbg.Context(0)
