"""The Julia binding's struct mirrors (mavi.jl_gb300/julia/MaviCUDA.jl) have the
byte layout of the C structs of include/mavi_cuda.h. Julia isbits structs are
laid out with C alignment rules, so the layout is computed from the field types
here and compared with the ctypes mirror (itself checked against the C compiler
in test_abi.py). No Julia and no GPU needed."""
import ctypes as C
import re

from conftest import ROOT

SHIM = ROOT / "mavi.jl_gb300" / "julia" / "MaviCUDA.jl"
CONSTS = {"MAX_SPACES": 4, "MAX_LINES": 16, "MAX_TYPES": 4}
PRIM = {"Int32": 4, "Int64": 8, "UInt64": 8, "Float64": 8}

# Julia struct -> ctypes struct and the names whose offsets must agree
PAIRS = {
    "CSpace": ("MaviSpace", None),
    "CRingsCfg": ("MaviRingsCfg", {"inter": "inter_k_rep"}),
    "CDynamicCfg": ("MaviDynamicCfg", None),
    "CReplicaParams": ("MaviReplicaParams", None),
    "COptions": ("MaviOptions", None),
    "CSourceEntry": ("MaviSourceEntry", None),
    "CSpawnBox": ("MaviSpawnBox", None),
    "CInvasion": ("MaviInvasion", None),
}


def _structs(text):
    out = {}
    for m in re.finditer(r"^struct (\w+)\n(.*?)^end", text, flags=re.S | re.M):
        fields = []
        for line in m.group(2).splitlines():
            line = line.split("#")[0]
            for part in line.split(";"):
                part = part.strip()
                if "::" in part:
                    name, typ = part.split("::", 1)
                    fields.append((name.strip(), typ.strip()))
        out[m.group(1)] = fields
    return out


def _eval_int(expr):
    for k, v in CONSTS.items():
        expr = re.sub(rf"\b{k}\b", str(v), expr)
    assert re.fullmatch(r"[0-9 *+]+", expr), expr
    return eval(expr)


def _layout(name, structs, cache):
    """(size, alignment, {field: offset}) of a Julia struct under C rules."""
    if name in cache:
        return cache[name]
    off, align, offsets = 0, 1, {}
    for fname, typ in structs[name]:
        m = re.fullmatch(r"NTuple\{(.+),\s*(\w+)\}", typ)
        if m:
            n = _eval_int(m.group(1))
            size1, al = _type(m.group(2), structs, cache)
            size = n * size1
        else:
            size, al = _type(typ, structs, cache)
        off = (off + al - 1) // al * al
        offsets[fname] = off
        off += size
        align = max(align, al)
    size = (off + align - 1) // align * align
    cache[name] = (size, align, offsets)
    return cache[name]


def _type(typ, structs, cache):
    if typ in PRIM:
        return PRIM[typ], PRIM[typ]
    size, align, _ = _layout(typ, structs, cache)
    return size, align


def test_julia_structs_match_the_c_layout(mg):
    from mavi_gb300 import abi
    structs = _structs(SHIM.read_text())
    cache = {}
    for jname, (cname, rename) in PAIRS.items():
        size, _, offsets = _layout(jname, structs, cache)
        ct = abi.STRUCTS[cname]
        assert size == C.sizeof(ct), (jname, size, C.sizeof(ct))
        for fname, off in offsets.items():
            cfield = (rename or {}).get(fname, fname)
            if hasattr(ct, cfield):
                assert getattr(ct, cfield).offset == off, (jname, fname, off, getattr(ct, cfield).offset)


def test_julia_shim_binds_declared_entry_points():
    text = SHIM.read_text()
    header = (ROOT / "include" / "mavi_cuda.h").read_text()
    for name in set(re.findall(r"ccall\(\(:(\w+), libmavi\)", text)):
        assert re.search(rf"\b{name}\s*\(", header), f"{name} is not declared in include/mavi_cuda.h"


def test_julia_ccalls_have_the_prototypes_arity():
    """Every ccall's argument-type tuple has as many entries as the C
    prototype has parameters (the shim is not executed here)."""
    from test_abi import header_arity
    arity = header_arity()
    text = SHIM.read_text()
    calls = re.findall(r"ccall\(\(:(\w+), libmavi\),\s*\w+,\s*\(([^()]*)\)", text)
    assert len(calls) >= 10
    for name, types in calls:
        n = len([x for x in types.split(",") if x.strip()])
        assert n == arity[name], (name, n, arity[name])


def test_julia_bulk_drivers_are_defined_for_cuda_systems():
    """run_system and run_experiment have methods for systems whose device is
    CUDADevice (one mavi_step per event instead of one call per step); the
    shim is not executed here, so the check is on its source."""
    text = SHIM.read_text()
    assert re.search(r"function Mavi\.RunSystem\.run_system\(system::CUDASystem;", text)
    assert re.search(r"function EXP\.run_experiment\(experiment::EXP\.Experiment\{<:CUDASystem\}", text)
    assert "gpu_run!(system, n)" in text and "gpu_run!(system, max(n, 1))" in text
