"""The C ABI library loads (no GPU needed) and exports every symbol that
include/mrmg_gb300.h declares, with a ctypes signature for each."""
import re
import subprocess
from pathlib import Path

from conftest import ROOT, pkg

HEADER = ROOT / "include" / "mrmg_gb300.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mrmg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "mrmg_is_edge_collision_free_batch" in syms
    assert len(syms) >= 15


def test_library_exports_every_declared_symbol(cuda_lib):
    lib_path = pkg("_lib").LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (mrmg_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    for s in declared_symbols():
        assert hasattr(cuda_lib, s)


def test_ctypes_signatures_cover_header():
    assert sorted(pkg("_lib").SIGNATURES) == declared_symbols()


def test_version_and_error_without_gpu(cuda_lib):
    assert b"sm_103a" in cuda_lib.mrmg_version()
    _lib = pkg("_lib")
    # argument validation happens before any device call
    assert cuda_lib.mrmg_scene_destroy(None) == 0
    rc = cuda_lib.mrmg_is_collision_free_batch(None, None, 0, 1, None, None, 0)
    assert rc == _lib.MRMG_ERR_ARG
    assert b"NULL" in cuda_lib.mrmg_last_error() or b"scene" in cuda_lib.mrmg_last_error()


def test_status_codes_match_header_and_map_to_exceptions(cuda_lib):
    """The header's status codes are the binding's, and each maps to the
    exception type the reference's callers expect."""
    import pytest

    _lib = pkg("_lib")
    text = HEADER.read_text()
    codes = dict((k, int(v)) for k, v in re.findall(r"\b(MRMG_(?:OK|ERR_[A-Z_]+))\s*=\s*(-?\d+)", text))
    assert codes == {k: getattr(_lib, k) for k in codes} and len(codes) == 7
    assert int(re.search(r"#define MRMG_MAX_STORE_MODES \(1 << (\d+)\)", text).group(1)) == 20
    assert _lib.MRMG_MAX_STORE_MODES == 1 << 20
    want = {"MRMG_ERR_ARG": ValueError, "MRMG_ERR_N_START": AssertionError,
            "MRMG_ERR_UNSUPPORTED": NotImplementedError, "MRMG_ERR_HOST": MemoryError,
            "MRMG_ERR_CUDA": _lib.Gb300Error, "MRMG_ERR_TIMEOUT": _lib.Gb300Error}
    for name, exc in want.items():
        with pytest.raises(exc):
            _lib.check(codes[name], name)
    assert _lib.check(0) == 0
    # store entry points validate their handle before any device call
    assert cuda_lib.mrmg_node_store_append(None, 0, None, 0, None) == _lib.MRMG_ERR_ARG
    assert cuda_lib.mrmg_near_fetch(None, None, None, 0, None) == _lib.MRMG_ERR_ARG


def test_every_entry_point_survives_null_arguments():
    """Every entry point called with NULL handles and pointers and zero
    sizes (no GPU here) returns a status instead of crashing: NULL handles
    and pointers are refused before anything is dereferenced.  Run in a
    child process, so that a crash names the entry point."""
    import sys

    code = (
        "import ctypes as C, importlib, sys\n"
        f"sys.path.insert(0, {str(ROOT)!r})\n"
        "L = importlib.import_module('multirobot-pathplanning-benchmark_gb300._lib')\n"
        "lib = L.load()\n"
        "for name, (res, args) in L.SIGNATURES.items():\n"
        "    print(name, flush=True)\n"
        "    vals = [0.0 if a in (C.c_double, C.c_float) else 0 if a in (C.c_int32, C.c_int64, C.c_uint32) else None"
        " for a in args]\n"
        "    rc = getattr(lib, name)(*vals)\n"
        "    if res is C.c_int32 and name not in ('mrmg_binary_search_indices', 'mrmg_status_from_error_bits',\n"
        "                                         'mrmg_scene_destroy', 'mrmg_node_store_destroy'):\n"
        "        assert rc == L.MRMG_ERR_ARG, (name, rc)\n"
        "print('done')\n")
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    last = (p.stdout.strip().splitlines() or ["(none)"])[-1]
    assert p.returncode == 0 and last == "done", f"stopped after {last}: {p.stderr[-500:]}"
