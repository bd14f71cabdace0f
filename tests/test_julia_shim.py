"""The Julia shim's ccall signatures against the C ABI (static check, no Julia).

Julia is not installed where the tests run, so NbgCuda.jl cannot be executed;
this test parses every ccall in it and checks the argument types, position by
position, and the return type against the prototype in include/nbg.h.  The
argument lists are also checked against the reference-side arrays they pass
(a State{Float64} / TransitTiming{Float64} field for every array pointer).
"""
import os
import re

from conftest import ROOT

SHIM = os.path.join(ROOT, "nbodygradient.jl_gb300", "julia", "NbgCuda.jl")
HEADER = os.path.join(ROOT, "include", "nbg.h")

# C parameter type (const and names stripped) -> the Julia ccall type it must be bound with
C_TO_JULIA = {
    "nbg_context*": {"Ptr{Cvoid}"},
    "nbg_context**": {"Ref{Ptr{Cvoid}}", "Ptr{Ptr{Cvoid}}"},
    "int": {"Cint"},
    "int32_t": {"Int32", "Cint"},
    "int64_t": {"Int64"},
    "size_t": {"Csize_t", "UInt"},
    "double": {"Cdouble", "Float64"},
    "double*": {"Ptr{Float64}", "Ptr{Cdouble}"},
    "uint8_t*": {"Ptr{Bool}", "Ptr{UInt8}"},  # Julia's Bool is one byte (State.pair)
    "int64_t*": {"Ptr{Int64}"},
    "uint32_t*": {"Ptr{UInt32}"},
    "char*": {"Ptr{UInt8}", "Ptr{Cchar}"},
}


def _split_top(s):
    """Split at top-level commas (braces and parentheses nest)."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({":
            depth += 1
        elif ch in ")}":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def header_prototypes():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    protos = {}
    for m in re.finditer(r"\b([a-z0-9_]+\*?)\s+\**(nbg_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", src):
        ret, name, params = m.group(1), m.group(2), m.group(3)
        types = []
        for p in _split_top(params):
            if p == "void":
                continue
            p = re.sub(r"\bconst\b", "", p)
            p = re.sub(r"\s*\*\s*", "*", p).strip()
            m2 = re.match(r"^(.*?)\s*([A-Za-z_]\w*)$", p)  # the type, then the parameter's name
            types.append(m2.group(1).replace(" ", ""))
        protos[name] = (ret, types)
    return protos


def shim_ccalls():
    src = open(SHIM).read()
    calls = []
    for m in re.finditer(r"ccall\(\(:(nbg_[a-z0-9_]+),\s*LIB\),\s*(\w+),", src):
        name, ret = m.group(1), m.group(2)
        # the type tuple: the parenthesised group right after the return type
        i = src.index("(", m.end())
        depth, j = 0, i
        while True:
            if src[j] == "(":
                depth += 1
            elif src[j] == ")":
                depth -= 1
                if depth == 0:
                    break
            j += 1
        types = [t for t in _split_top(src[i + 1:j]) if t]
        # the argument values: up to the ccall's closing parenthesis
        k, depth2 = j + 1, 1
        while depth2:
            if src[k] == "(":
                depth2 += 1
            elif src[k] == ")":
                depth2 -= 1
            k += 1
        args = [a for a in _split_top(src[j + 1:k - 1]) if a]
        calls.append((name, ret, types, args))
    return calls


def test_every_ccall_matches_the_header():
    protos = header_prototypes()
    calls = shim_ccalls()
    names = {c[0] for c in calls}
    assert {"nbg_create", "nbg_last_error", "nbg_integrate_transits", "nbg_integrate_transit_parameters",
            "nbg_integrate", "nbg_integrate_steps", "nbg_integrate_cartesian"} <= names
    for name, ret, types, args in calls:
        assert name in protos, name
        cret, ctypes_ = protos[name]
        assert ret == "Cint" and cret == "int", (name, ret, cret)
        assert len(types) == len(ctypes_), (name, len(types), len(ctypes_))
        assert len(args) == len(types), (name, "values", len(args), "types", len(types))
        for pos, (jt, ct) in enumerate(zip(types, ctypes_)):
            assert ct in C_TO_JULIA, (name, pos, ct)
            assert jt in C_TO_JULIA[ct], (name, pos, "Julia %s for C %s" % (jt, ct))


def test_transit_calls_pass_the_reference_fields_in_order():
    """The array arguments of the transit calls are the State / TransitTiming fields the C ABI names."""
    calls = {c[0]: c for c in shim_ccalls()}
    _, _, _, args = calls["nbg_integrate_transits"]
    assert args[6] in ("t", "s.t")  # s.t, the one-element time vector
    assert args[7:] == ["s.x", "s.v", "s.m", "s.xerror", "s.verror", "s.jac_step", "s.jac_error", "s.dqdt", "s.pair",
                        "s.jac_init", "tt.ntt", "tt.tt", "tt.dtdq0", "tt.dtdelements", "tt.count"]
    assert args[2] == "tt.ti - 1" and args[3] == "intr.h" and args[4] == "intr.tmax"
    _, _, _, args = calls["nbg_integrate_transit_parameters"]
    assert args[-4:] == ["ttbv.ttbv", "ttbv.dtbvdq0", "ttbv.dtbvdelements", "ttbv.count"]
