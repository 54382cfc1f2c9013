"""CPU-side checks of the C-ABI library: it loads, exports every entry point
the public headers declare, and its host-only parts (input generator,
argument validation) behave.  No kernel is launched here."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (REPO / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(wd_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(wd):
    names = declared_symbols()
    assert len(names) > 20
    lib = C.CDLL(str(wd.LIB_PATH))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(wd):
    for s in range(9):
        assert wd.lib.wd_status_string(s)
    assert wd.lib.wd_status_string(99) == b"unknown status"


def test_generator_is_deterministic_and_su3(wd):
    dims = (4, 2, 2, 4)
    g1 = wd.gen_gauge(dims, seed=3, eps=0.5)
    g2 = wd.gen_gauge(dims, seed=3, eps=0.5)
    g3 = wd.gen_gauge(dims, seed=4, eps=0.5)
    for a, b in zip(g1, g2):
        assert np.array_equal(a, b)
    assert not np.array_equal(g1[0], g3[0])
    for u in g1:
        m = u.reshape(-1, 3, 3)
        eye = np.einsum("sij,skj->sik", m, m.conj())
        assert np.abs(eye - np.eye(3)).max() < 1e-13
        assert np.abs(np.linalg.det(m) - 1).max() < 1e-13
    s1 = wd.gen_source(dims, seed=5)
    assert np.array_equal(s1, wd.gen_source(dims, seed=5))
    assert abs(np.linalg.norm(s1) - 1) < 1e-14


def test_generator_rejects_bad_dims(wd):
    g = [np.empty(9 * 30, np.complex128) for _ in range(4)]
    assert wd.lib.wd_gen_gauge(wd._dims((3, 2, 5, 1)), 1, 0.5, wd._gauge_ptrs(g)) == wd.BAD_DIMS
    s = np.empty(12 * 30, np.complex128)
    assert wd.lib.wd_gen_source(wd._dims((0, 2, 5, 3)), 1, wd._ptr(s)) == wd.BAD_DIMS


def test_context_without_matching_gpu_reports_no_device(wd):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert wd.lib.wd_context_create(0, C.byref(h)) == wd.NO_DEVICE


def test_null_arguments_are_rejected(wd):
    assert wd.lib.wd_context_create(0, None) == wd.BAD_ARG
    assert wd.lib.wd_solve(None, None, None, None, None, None) == wd.BAD_ARG


def test_reference_api_symbols_exported():
    """liblattice_gb300.so exports the reference's C++ entry points with its signatures."""
    import subprocess
    lib = REPO / "ipcc2021-final_gb300" / "wilson_gb300" / "liblattice_gb300.so"
    out = subprocess.run(["nm", "-DC", "--defined-only", str(lib)], capture_output=True, text=True).stdout
    for sig in ["DslashNew(lattice_fermion&, lattice_fermion&, lattice_gauge&, double, bool)",
                "Dslash(lattice_fermion&, lattice_fermion&, lattice_gauge&, double, bool)",
                "DslashoffdNew(lattice_fermion&, lattice_fermion&, lattice_gauge&, bool, int)",
                "Dslashoffd(lattice_fermion&, lattice_fermion&, lattice_gauge&, bool, int)",
                "DslashEEOONew(lattice_fermion&, lattice_fermion&, double)",
                "DslashEE(lattice_fermion&, lattice_fermion&, double)",
                "DslashOO(lattice_fermion&, lattice_fermion&, double)",
                "DslashEONew(lattice_fermion&, lattice_fermion&, lattice_gauge&, bool)",
                "DslashOENew(lattice_fermion&, lattice_fermion&, lattice_gauge&, bool)",
                "CGinvert(lattice_fermion&, lattice_fermion&, lattice_gauge&, double, int, double)",
                "CGinvert(std::complex<double>*, std::complex<double>*, std::complex<double>**, double, int, "
                "double, int*, int*)",
                "check(lattice_fermion&, lattice_fermion&, lattice_gauge&, double)",
                "load_gauge(std::complex<double>**, std::__cxx11::basic_string<char, std::char_traits<char>, "
                "std::allocator<char> >&, int*, int*)",
                "lattice_fermion::lattice_fermion(int*, int*)",
                "lattice_gauge::peeksite(int const*, int, int, int)"]:
        assert sig in out, sig


def test_driver_rejects_bad_arguments_before_touching_a_gpu():
    import subprocess
    exe = REPO / "ipcc2021-final_gb300" / "wilson_gb300" / "wilson_main"
    r = subprocess.run([str(exe), "0.1", "UNIT"], capture_output=True, text=True)
    assert r.returncode == 1 and "wilson_main Mass gaugefile" in r.stderr
    r = subprocess.run([str(exe), "0.1", "UNIT", "8", "8", "8", "8", "8", "8", "4", "8"], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "subgrid == lattice" in r.stderr


def test_tuner_pins_and_report(wd):
    """Pinning a launch variant needs no GPU; the report lists it (ms -1)."""
    wd.tune_pin("hop_f16", 12345, 1)
    try:
        rows = [r for r in wd.tune_report() if r[1] == "hop_f16" and r[2] == 12345]
        assert rows == [(0, "hop_f16", 12345, 1, -1.0)]
    finally:
        wd.tune_pin("hop_f16", 12345, -1)
    assert not [r for r in wd.tune_report() if r[2] == 12345]
    with pytest.raises(ValueError):
        wd.tune_pin("hop_f16", 0, 1)


def test_tuner_cache_file_is_read(tmp_path):
    """WD_TUNE_CACHE decisions are loaded before any timing (fresh process)."""
    import os
    import subprocess
    import sys

    cache = tmp_path / "tune.txt"
    cache.write_text("0 hop_df64 4096 3 0.125000\n0 hop_f32 4096 2 0.010000\n")
    code = ("import sys; sys.path.insert(0, %r); import wilson_gb300 as wd; "
            "wd.tune_pin('hop_f64', 1, -1); print(sorted(wd.tune_report()))") % str(REPO / "ipcc2021-final_gb300")
    env = dict(os.environ, WD_TUNE_CACHE=str(cache))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=120)
    assert out.returncode == 0, out.stderr
    assert "(0, 'hop_df64', 4096, 3, 0.125)" in out.stdout and "(0, 'hop_f32', 4096, 2, 0.01)" in out.stdout
