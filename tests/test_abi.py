"""The C ABI: the library loads, exports every entry point the header
declares, and the ctypes mirror matches the C struct layout. No GPU needed."""
import ctypes as C
import re

import pytest

from conftest import ROOT


def header_functions():
    text = (ROOT / "include" / "mavi_cuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mavi_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_entry_point(lib):
    names = header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), f"{n} declared in include/mavi_cuda.h but not exported"


def test_ctypes_signatures_cover_header(mg):
    from mavi_gb300 import abi
    assert set(header_functions()) == set(abi.SIGNATURES)


def header_arity():
    """{entry point: number of parameters} from the prototypes of the header."""
    text = (ROOT / "include" / "mavi_cuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(mavi_[a-z_]+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else len(params.split(","))
    return out


def test_ctypes_signatures_have_the_prototypes_arity(mg):
    from mavi_gb300 import abi
    arity = header_arity()
    assert set(arity) == set(abi.SIGNATURES)
    for name, (_, args) in abi.SIGNATURES.items():
        assert len(args) == arity[name], (name, len(args), arity[name])


def test_struct_layout_matches_c(mg, orc):
    from mavi_gb300 import abi
    sizes = orc.struct_sizes()
    for name, size in sizes.items():
        assert C.sizeof(abi.STRUCTS[name]) == size, name


def test_status_strings_and_version(lib):
    assert lib.mavi_abi_version() == 1
    for st in range(10):
        assert lib.mavi_status_string(st)
    assert lib.mavi_status_string(0) == b"ok"


def test_null_arguments_are_rejected_without_a_gpu(lib):
    from mavi_gb300 import abi
    h = C.c_void_p()
    assert lib.mavi_create(None, 1, None, None, None, None, None, C.byref(h)) == abi.MAVI_ERR_INVALID_ARG
    assert lib.mavi_step(None, 1) == abi.MAVI_ERR_INVALID_ARG
    assert lib.mavi_destroy(None) == abi.MAVI_OK


def test_missing_library_fails_loudly(mg, tmp_path):
    from mavi_gb300 import abi
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        abi.load_library(tmp_path / "libmavi_cuda.so")


def test_product_never_imports_the_oracle():
    pkg = ROOT / "mavi.jl_gb300"
    for p in list(pkg.rglob("*.py")) + list(pkg.rglob("*.cu")) + list(pkg.rglob("*.cuh")):
        assert "oracle" not in p.read_text().lower().replace("oracle/", ""), p


def test_ctypes_layer_binds_every_entry_point():
    """The Python host binds every entry point of the header with a signature."""
    from mavi_gb300 import abi
    missing = [n for n in header_functions() if n not in abi.SIGNATURES]
    assert not missing, missing
