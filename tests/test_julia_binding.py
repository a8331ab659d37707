"""The Julia binding (geostatsprocesses.jl_gb300/julia/GeoStatsProcessesGPU.jl)
cannot run here: no Julia toolchain.  These CPU checks read it as text and
hold it to the C ABI: every symbol it ccalls is declared in include/geosgs.h
and exported by the library, and its struct mirrors list the C structs'
fields in order with the same sizes (so the layouts agree)."""
import ctypes as C
import os
import re

from geosgs import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JL = os.path.join(ROOT, "geostatsprocesses.jl_gb300", "julia", "GeoStatsProcessesGPU.jl")
HEADER = os.path.join(ROOT, "include", "geosgs.h")

JULIA_SIZES = {"Int32": 4, "UInt32": 4, "Int64": 8, "UInt64": 8, "Float64": 8, "Float32": 4}


def _julia_structs(src):
    out = {}
    for m in re.finditer(r"^struct (\w+)\n(.*?)^end", src, re.S | re.M):
        out[m.group(1)] = re.findall(r"^\s*(\w+)::([\w{},]+)", m.group(2), re.M)
    return out


def _jsize(t, structs):
    if t in JULIA_SIZES:
        return JULIA_SIZES[t]
    if t.startswith("Ptr{"):
        return 8
    m = re.fullmatch(r"NTuple\{(\d+),(\w+)\}", t)
    if m:
        return int(m.group(1)) * _jsize(m.group(2), structs)
    return sum(_jsize(ft, structs) for _, ft in structs[t])


def test_ccalled_symbols_are_declared_and_exported():
    src = open(JL).read()
    header = open(HEADER).read()
    names = sorted(set(re.findall(r"ccall\(\(:(\w+),\s*libgeosgs\)", src)))
    assert "sgs_plan_set_multivariate" in names and "sgs_plan_simulate_indicator" in names
    for n in names:
        assert re.search(r"\b%s\s*\(" % n, header), n
        assert n in _abi.EXPORTS, n


def test_struct_mirrors_match_the_c_layout():
    structs = _julia_structs(open(JL).read())
    pairs = {"SgsVariogram": _abi.SgsVariogram, "SgsBall": _abi.SgsBall, "SgsProblem": _abi.SgsProblem}
    for jname, ct in pairs.items():
        jf = structs[jname]
        cf = ct._fields_
        assert [n for n, _ in jf] == [n for n, _ in cf], jname
        for (n, jt), (_, ctype) in zip(jf, cf):
            assert _jsize(jt, structs) == C.sizeof(ctype), (jname, n)
