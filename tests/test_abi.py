"""CPU-side checks of the C ABI: the library builds, loads and exports every
function that ``include/orthoroute_gb300.h`` declares (no GPU calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "orthoroute_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|size_t)\s+(ogr_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from orthoroute_gb300 import _build
    path = _build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "ogr_find_path" in names and "ogr_csr_build" in names
    assert len(names) >= 13


def test_library_exports_every_declared_function(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_python_binding_covers_header():
    from orthoroute_gb300 import _lib
    assert sorted(_lib.EXPORTED) == sorted(n for n in declared_functions() if n in _lib.EXPORTED)
    missing = [n for n in declared_functions() if n not in _lib.EXPORTED]
    assert not missing, missing


def test_edge_count_matches_oracle():
    """ogr_csr_num_edges is a host function: it runs without a GPU."""
    from orthoroute_gb300 import Lattice, _lib
    from oracle.lattice import LatticeSpec, build_csr
    lib = _lib.load()
    for nx, ny, nz, anyv in [(7, 5, 6, True), (9, 8, 12, False), (12, 10, 20, None), (5, 4, 2, None)]:
        L = Lattice(nx, ny, nz, allow_any_layer_via=anyv)
        d, keep = L.descriptor()
        E = ctypes.c_int64(0)
        assert lib.ogr_csr_num_edges(ctypes.byref(d), ctypes.byref(E)) == 0
        ref = build_csr(LatticeSpec(nx, ny, nz, allow_any_layer_via=anyv))
        assert E.value == len(ref.indices)


def test_fault_injection_hook_replaces_and_restores_an_entry_point():
    """The host-side failure hook used by the failure-handling tests: inside
    the block the entry point returns the injected status without running;
    afterwards the real entry point is back."""
    import ctypes as C
    from orthoroute_gb300 import _lib
    lib = _lib.load()
    real = lib.ogr_full_tile
    cur, d = C.c_int32(0), C.c_double(0.0)
    with _lib.inject_fault("ogr_full_tile", _lib.OGR_ERR_CUDA):
        assert lib.ogr_full_tile(-1, 0.0, 0, 0, C.byref(cur), C.byref(d)) == _lib.OGR_ERR_CUDA
    assert lib.ogr_full_tile is real
    assert lib.ogr_full_tile(-1, 0.0, 0, 0, C.byref(cur), C.byref(d)) == _lib.OGR_OK
    assert lib.ogr_debug_limits(-1, -1, None, None) == _lib.OGR_OK
