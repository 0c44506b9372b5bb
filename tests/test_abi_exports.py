"""The C ABI library loads and exports every function include/texo_gp.h
declares, and the ctypes mirror declares a signature for each of them (no
compute call: this runs without a GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "texo_gp.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(texo_gp_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_expected_surface():
    names = declared_functions()
    for n in ("texo_gp_place", "texo_gp_create", "texo_gp_evaluate", "texo_gp_scatter", "texo_gp_poisson",
              "texo_gp_run", "texo_gp_batch_advance", "texo_gp_server_submit", "texo_gp_scatter_static"):
        assert n in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    from texo_gb300 import abi, build
    build.build()
    lib = ctypes.CDLL(abi.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_mirror_covers_the_header():
    from texo_gb300 import abi
    assert sorted(abi.SIGNATURES) == declared_functions()


def test_status_names_round_trip_without_a_gpu():
    from texo_gb300 import abi
    lib = abi.load()
    for code, name in abi.STATUS.items():
        assert lib.texo_gp_status_name(code).decode() == name
    p = abi.Params()
    lib.texo_gp_default_params(ctypes.byref(p))
    ref = abi.default_params_py()
    for f, _ in abi.Params._fields_:
        if f != "reserved":
            assert getattr(p, f) == getattr(ref, f), f
