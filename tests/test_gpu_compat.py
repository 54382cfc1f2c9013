"""The reference-API C++ layer (liblattice_gb300.so) driven from C++ as the
reference's own callers use it: every operator on the golden inputs, the
CG with the reference's srand/rand initial guess, and the command-line driver
against the oracle."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import rel_l2

pytestmark = pytest.mark.gpu
REPO = Path(__file__).resolve().parent.parent
TOL = 1e-13


def _build_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("wd_build", REPO / "ipcc2021-final_gb300/wilson_gb300/build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build_compat()
    return mod


@pytest.fixture(scope="module")
def golden_prog(tmp_path_factory):
    b = _build_module()
    exe = tmp_path_factory.mktemp("cpp") / "compat_golden"
    subprocess.run(b.compat_program_cmd(REPO / "tests/cpp/compat_golden.cpp", exe), check=True)
    return exe


def test_reference_api_on_golden_vectors(wd, oracle, golden4, golden_prog, tmp_path):
    g = golden4
    V = int(np.prod(g["dims"]))
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array(g["dims"], np.int32).tofile(f)
        np.array([g["mass"]], np.float64).tofile(f)
        np.array([int(g["cg_seed"])], np.int32).tofile(f)
        for u in g["gauge"]:
            u.tofile(f)
        g["src"].tofile(f)
    r = subprocess.run([str(golden_prog), str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    data = np.fromfile(out, np.uint8)
    n = V * 12 * 16
    vecs = [data[i * n:(i + 1) * n].view(np.complex128) for i in range(12)]
    tail = data[12 * n:]
    norm2 = tail[:8].view(np.float64)[0]
    dot = tail[8:24].view(np.complex128)[0]
    x = tail[24:24 + n].view(np.complex128)
    x_ptr = tail[24 + n:24 + 2 * n].view(np.complex128)
    names = ["offd_new_dag0_cb0", "offd_new_dag0_cb1", "offd_new_dag1_cb0", "offd_new_dag1_cb1",
             "full_new_dag0", "full_new_dag1", "full_old_dag0", "eeoo_new", "offd_new_dag0_cb0",
             "offd_new_dag1_cb1"]
    for v, k in zip(vecs, names):
        assert rel_l2(v, g[k]) < TOL, k
    half = V * 6
    ee = g["eeoo_new"].copy()
    ee[half:] = 0
    oo = g["eeoo_new"].copy()
    oo[:half] = 0
    assert rel_l2(vecs[10], ee) == 0.0 and rel_l2(vecs[11], oo) == 0.0
    assert abs(norm2 - np.vdot(g["src"], g["src"]).real) < 1e-14
    ref_dot = np.vdot(g["src"], g["full_new_dag0"])
    assert abs(dot - ref_dot) < 1e-13 * abs(ref_dot)
    # CGinvert with srand(cg_seed), object overload then raw-pointer overload:
    # the reference's own run gave cg_iters / cg_x
    runs = re.findall(r"CG: (\d+) iterations, convergence residual \|r\| = ([0-9.eE+-]+)", r.stdout)
    assert len(runs) == 2, r.stdout
    for its, _ in runs:
        assert int(its) == int(g["cg_iters"]), r.stdout
    assert rel_l2(x, g["cg_x"]) < 1e-10
    assert rel_l2(x_ptr, g["cg_x"]) < 1e-10
    assert np.array_equal(x_ptr, x)


def test_command_line_driver_matches_oracle(wd, oracle):
    b = _build_module()
    dims, seed, mass = (4, 4, 4, 8), 3, 0.1
    r = subprocess.run([str(b.MAIN_BIN), str(mass), "RANDOM", *map(str, dims), *map(str, dims), str(seed)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = r.stdout
    src, x0 = oracle.main_inputs(dims, seed)
    gauge = wd.gen_gauge(dims, 1, 0.5)            # "RANDOM" with the default seed 1
    x, iters, rsd = oracle.cg_ref(src, gauge, dims, mass, 500, 1e-9, x0)
    m = re.search(r"CG: (\d+) iterations, convergence residual \|r\| = ([0-9.eE+-]+)", out)
    assert m, out
    assert abs(int(m.group(1)) - iters) <= 1
    chk = oracle.check(src, x, gauge, dims, mass)
    got_b = float(re.search(r"\|b\| = ([0-9.eE+-]+)", out).group(1))
    got_res = float(re.search(r"\|M x -b\| = ([0-9.eE+-]+)", out).group(1))
    assert abs(got_b - chk[0]) < 1e-5 * chk[0]
    assert got_res < 1e-6 * chk[0] and chk[10] < 1e-6 * chk[0]
    for line in ("Source and Gauge, time:", "CG invert, time:", "Total time:", "|M^dagger M x - Mdb| ="):
        assert line in out


def _write_gauge_file(path, gauge, dims, header=b"", trailer=b""):
    """Big-endian doubles, [site lex][mu][row][col][re, im] (src/load_gauge.cpp:110-161)."""
    Lx, Ly, Lz, Lt = dims
    V = Lx * Ly * Lz * Lt
    eo_of_lex = np.empty(V, np.int64)
    for lex in range(V):
        x, y, z, t = lex % Lx, (lex // Lx) % Ly, (lex // (Lx * Ly)) % Lz, lex // (Lx * Ly * Lz)
        eo_of_lex[lex] = lex // 2 + ((x + y + z + t) & 1) * (V // 2)
    data = np.stack([g.reshape(V, 9)[eo_of_lex] for g in gauge], axis=1)
    with open(path, "wb") as f:
        f.write(header)
        f.write(data.view(np.float64).astype(">f8").tobytes())
        f.write(trailer)


@pytest.mark.parametrize("framing", ["plain", "lime"])
def test_driver_reads_gauge_files(wd, oracle, golden4, tmp_path, framing):
    b = _build_module()
    g = golden4
    path = tmp_path / "conf.dat"
    if framing == "plain":
        _write_gauge_file(path, g["gauge"], g["dims"])
    else:
        _write_gauge_file(path, g["gauge"], g["dims"], header=b"L" * 1000, trailer=b"T" * 280)
    dims, seed, mass = g["dims"], 5, 0.1
    r = subprocess.run([str(b.MAIN_BIN), str(mass), str(path), *map(str, dims), *map(str, dims), str(seed)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    src, x0 = oracle.main_inputs(dims, seed)
    x, iters, rsd = oracle.cg_ref(src, g["gauge"], dims, mass, 500, 1e-9, x0)
    m = re.search(r"CG: (\d+) iterations", r.stdout)
    assert m and abs(int(m.group(1)) - iters) <= 1, r.stdout
    chk = oracle.check(src, x, g["gauge"], dims, mass)
    got = re.search(r"\(Mx, Mx\) = \(([0-9.eE+-]+),", r.stdout)
    assert abs(float(got.group(1)) - chk[6]) < 1e-5 * chk[6]   # the report prints 6 significant digits
