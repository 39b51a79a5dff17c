"""The C-ABI library loads without a GPU and exports every entry point that
include/tealeaf_gb300.h declares; the oracle library exports its kernels."""
from __future__ import annotations

import ctypes as C
import subprocess

import exploringsycl_gb300 as tl


def test_library_exports_every_declared_symbol(backend_built):
    lib = C.CDLL(str(tl.LIB_PATH))
    declared = tl.declared_symbols()
    assert len(declared) >= 30
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    # and nothing exported under tl_ that the header does not declare
    out = subprocess.run(["nm", "-D", "--defined-only", str(tl.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T tl_" in ln}
    assert exported == set(declared), exported ^ set(declared)


def test_bindings_cover_header(backend_built):
    declared = set(tl.declared_symbols())
    bound = set(tl.SIGNATURES) | set(tl.CONTEXT_FREE) | set(tl.HANDLE_FIRST) | {"tl_last_error", "tl_launch_count",
                                                           "tl_net_num_params"}
    assert declared <= bound, declared - bound


def test_no_gpu_is_a_loud_error(backend_built):
    """Without a GPU the library refuses to create a context (no fallback)."""
    import torch
    if torch.cuda.is_available():
        return
    lib = tl.load_library()
    h = C.c_void_p()
    rc = lib.tl_context_create(0, None, C.byref(h))
    assert rc != 0
    assert lib.tl_last_error()


def test_oracle_exports(oracle_built):
    L = oracle_built.lib()
    for name in oracle_built.SIGNATURES:
        assert hasattr(L, name)


def test_grid_limit_matches_the_header_and_is_checked_before_any_allocation():
    """TL_MAX_CELLS (the deterministic reductions' largest grid, 131,072 tiles
    of 4096 cells) is one number in the header and the package, and a chunk
    above it is refused before a context or a field is made."""
    import re

    import pytest

    from exploringsycl_gb300 import deck as dk
    from exploringsycl_gb300.chunk import GpuChunk
    text = (tl.PKG.parent / "include" / "tealeaf_gb300.h").read_text()
    assert int(re.search(r"#define TL_MAX_CELLS (\d+)", text).group(1)) == tl.MAX_CELLS
    assert tl.MAX_CELLS == 131072 * 4096
    with pytest.raises(tl.TLError, match="TL_MAX_CELLS"):
        GpuChunk(dk.two_state(23168))  # 23172^2 cells with the halos


def test_bindings_match_the_header_prototypes():
    """Every ctypes binding passes as many arguments as its C prototype has,
    each of the same kind (int, size_t, float, double, pointer): a slip
    between the two would pass garbage without any error."""
    import re

    text = re.sub(r"/\*.*?\*/", "", (tl.PKG.parent / "include" / "tealeaf_gb300.h").read_text(),
                  flags=re.S)
    protos = {}
    for m in re.finditer(r"^\s*(?:int|const char\*|long long)\s+(tl_\w+)\(([^;]*?)\);", text,
                         re.M | re.S):
        body = m.group(2).strip()
        protos[m.group(1)] = [] if body in ("", "void") else [p.strip() for p in body.split(",")]

    def c_kind(param):
        param = re.sub(r"\s+", " ", param)
        if "*" in param:
            return "pointer"
        for kind in ("double", "float", "size_t", "int"):
            if re.match(rf"(const )?{kind}\b", param):
                return kind
        return param

    def py_kind(t):
        if t is C.c_void_p or (isinstance(t, type) and issubclass(t, C._Pointer)):
            return "pointer"
        return {C.c_double: "double", C.c_float: "float", C.c_size_t: "size_t",
                C.c_int: "int"}.get(t, repr(t))

    checked = 0
    for table, leading in ((tl.SIGNATURES, [C.c_void_p]), (tl.HANDLE_FIRST, [C.c_void_p]),
                           (tl.CONTEXT_FREE, [])):
        for name, args in table.items():
            assert [py_kind(t) for t in leading + list(args)] == \
                [c_kind(p) for p in protos[name]], name
            checked += 1
    assert checked >= 45
