"""CPU tests of the boundary: the library loads without a GPU, exports every
symbol the header declares, and its struct layout matches ctypes and the
oracle build.  No compute calls."""
import ctypes as C
import os
import re

import pytest

from .conftest import ROOT

HEADER = os.path.join(ROOT, "include", "streamsculptor_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(ss_[a-z0-9_]+)\s*\(", text, flags=re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ["ss_potential_eval", "ss_orbit_f64", "ss_release_f64", "ss_stream_f64", "ss_stream_f32k",
              "ss_pert_response", "ss_binned_sums", "ss_last_error"]:
        assert s in syms


def test_library_loads_and_exports_every_declared_symbol():
    from streamsculptor_gb300 import _abi
    if not os.path.exists(_abi.LIB_PATH):
        pytest.skip("libssgb300.so not built")
    lib = _abi.load()
    for s in declared_symbols():
        assert hasattr(lib, s), s
        assert s in _abi.SIGNATURES, f"{s} missing from the ctypes signatures"
    assert lib.ss_abi_version() == _abi.SS_ABI_VERSION


def test_struct_layout_matches_oracle_build(oracle):
    from streamsculptor_gb300 import _abi
    L = oracle.lib()
    for i, st in enumerate(_abi.STRUCTS):
        assert L.or_abi_sizeof(i) == C.sizeof(st)


def test_error_path_without_gpu():
    # argument validation runs on the host before any CUDA call
    from streamsculptor_gb300 import _abi
    if not os.path.exists(_abi.LIB_PATH):
        pytest.skip("libssgb300.so not built")
    lib = _abi.load()
    P = _abi.ss_potential()
    P.G = 1.0
    P.n_components = 1
    P.comp[0].kind = 99
    rc = lib.ss_potential_eval(C.byref(P), None, 1, None, 0.0, None, None, None, None)
    assert rc == _abi.SS_ERR_INVALID_ARGUMENT
    assert b"unknown kind" in lib.ss_last_error()
    cfg = _abi.ss_stream_cfg()
    P.comp[0].kind = _abi.SS_PLUMMER
    P.comp[0].p[0], P.comp[0].p[1] = 1.0, 1.0
    cfg.dt = -1.0
    cfg.particles_per_release = 1
    rc = lib.ss_stream_f64(C.byref(P), C.byref(cfg), None, None, None, None, None)
    assert rc == _abi.SS_ERR_INVALID_ARGUMENT
