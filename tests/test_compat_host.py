"""The host-side parts of the reference-API C++ layer, with no GPU: the
fermion and gauge containers (borrow and own, alignment, zeroing, +=, +, -,
Minus, Plus, clean), gamma5, peeksite, and the index helpers of operator.h
(include/operator.h:11-75, src/lattice_fermion.cpp:15-95,
src/lattice_gauge.cpp:22-50 of the reference)."""
import subprocess
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent


def test_containers_and_index_helpers(tmp_path):
    import importlib.util
    spec = importlib.util.spec_from_file_location("wd_build", REPO / "ipcc2021-final_gb300/wilson_gb300/build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build_compat()
    exe = tmp_path / "compat_host"
    subprocess.run(b.compat_program_cmd(REPO / "tests/cpp/compat_host.cpp", exe), check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
