"""Write the golden vectors under tests/golden/ from the reference's own code.

The reference (CHN-ChenYi/IPCC2021-Final) ships no tests, fixtures or gauge
files, so these vectors are produced by running its unmodified sources,
compiled single-rank against oracle/mpi_shim/mpi.h (oracle/_ref/libref.so,
built by `make -C oracle`).  Inputs are generated here with numpy (seeded), so
the fixtures are self-contained: every array the check needs is stored.

The third fixture covers the 8^3x16 configuration (V = 8192, seed 1, mass 0.1,
links exp(i 0.5 H) and a unit Gaussian source from the package's own seeded
host generator, wd_gen_gauge / wd_gen_source).  Its vectors are too large to
store whole, so it keeps digests of the reference's outputs: the L2 norm of
each and its entries at every 37th index.

Run from the repository root, on an x86-64 host with the reference tree:
    python -c "import __graft_entry__ as g; g.build()" && python tests/golden/make_golden.py
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent / "oracle"))
sys.path.insert(0, str(HERE.parent.parent / "ipcc2021-final_gb300"))
from oracle import Reference  # noqa: E402

DIGEST_STRIDE = 37  # sampled entries of each stored 8^3x16 vector


def su3_links(rng: np.random.Generator, n: int, eps: float) -> np.ndarray:
    """n SU(3) matrices exp(i eps H), H Gaussian traceless hermitian (row-major, n*9)."""
    a = rng.normal(size=(n, 3, 3)) + 1j * rng.normal(size=(n, 3, 3))
    h = 0.5 * (a + np.conj(np.transpose(a, (0, 2, 1))))
    h -= np.trace(h, axis1=1, axis2=2)[:, None, None] * np.eye(3) / 3.0
    w, v = np.linalg.eigh(h)
    u = v @ (np.exp(1j * eps * w)[:, :, None] * np.conj(np.transpose(v, (0, 2, 1))))
    return np.ascontiguousarray(u.reshape(n * 9))


def inputs(dims, seed: int, eps: float = 0.5):
    rng = np.random.default_rng(seed)
    V = int(np.prod(dims))
    gauge = [su3_links(rng, V, eps) for _ in range(4)]
    src = rng.normal(size=V * 12) + 1j * rng.normal(size=V * 12)
    src /= np.linalg.norm(src)
    return gauge, np.ascontiguousarray(src)


def parse_check(text: str) -> dict:
    num = r"([-+0-9.eE]+)"
    cpl = r"\(" + num + "," + num + r"\)"
    out = {}
    m = re.search(r"\|b\| = " + num + r"\s+\|x\| = " + num, text)
    out["b"], out["x"] = float(m.group(1)), float(m.group(2))
    m = re.search(r"\(Mb, Mb\) = " + cpl + r"\s+\(b, MMb\) = " + cpl, text)
    out["MbMb"] = complex(float(m.group(1)), float(m.group(2)))
    out["bMMb"] = complex(float(m.group(3)), float(m.group(4)))
    m = re.search(r"\(Mx, Mx\) = " + cpl + r"\s+\(x, MMx\) = " + cpl, text)
    out["MxMx"] = complex(float(m.group(1)), float(m.group(2)))
    out["xMMx"] = complex(float(m.group(3)), float(m.group(4)))
    out["Mx_b"] = float(re.search(r"\|M x -b\| = " + num, text).group(1))
    out["MMx_Mdb"] = float(re.search(r"\|M\^dagger M x - Mdb\| = " + num, text).group(1))
    return out


def main() -> None:
    ref = Reference()

    # 1) 4^4, random links: every operator entry point
    dims = (4, 4, 4, 4)
    gauge, src = inputs(dims, seed=11)
    out = {"dims": np.array(dims), "gauge": np.stack(gauge), "src": src, "mass": 0.1}
    for dag in (0, 1):
        for cb in (0, 1):
            out[f"offd_new_dag{dag}_cb{cb}"] = ref.dslashoffd_new(src, gauge, dims, dag, cb)
        out[f"full_new_dag{dag}"] = ref.dslash_new(src, gauge, dims, 0.1, dag)
    out["full_old_dag0"] = ref.dslash_old(src, gauge, dims, 0.1, 0)
    out["eeoo_new"] = ref.dslash_eeoo_new(src, dims, 0.1)
    # CGinvert exactly as main.cpp calls it (srand seed, MaxCG 500, accuracy 1e-9)
    x, iters, rsd = ref.cginvert(src, gauge, dims, 0.1, 500, 1e-9, 7)
    out.update(cg_seed=7, cg_max=500, cg_acc=1e-9, cg_x=x, cg_iters=iters, cg_rsd=rsd)
    chk = parse_check(ref.check_text(src, x, gauge, dims, 0.1))
    out["check"] = np.array([chk["b"], chk["x"], chk["MbMb"].real, chk["MbMb"].imag, chk["bMMb"].real,
                             chk["bMMb"].imag, chk["MxMx"].real, chk["MxMx"].imag, chk["xMMx"].real,
                             chk["xMMx"].imag, chk["Mx_b"], chk["MMx_Mdb"]])
    np.savez_compressed(HERE / "wilson_4x4x4x4.npz", **out)

    # 2) 6x4x2x4: odd Lx/2, extent-2 direction (forward and backward neighbour coincide)
    dims = (6, 4, 2, 4)
    gauge, src = inputs(dims, seed=23)
    out = {"dims": np.array(dims), "gauge": np.stack(gauge), "src": src, "mass": 0.05}
    for dag in (0, 1):
        out[f"full_new_dag{dag}"] = ref.dslash_new(src, gauge, dims, 0.05, dag)
    out["offd_new_dag0_cb1"] = ref.dslashoffd_new(src, gauge, dims, 0, 1)
    np.savez_compressed(HERE / "wilson_6x4x2x4.npz", **out)
    print("golden vectors written; CG:", iters, "iterations, |r| =", rsd)

    # 3) 8^3x16 with the package's generator: digests of every entry point and of CGinvert
    import wilson_gb300 as wd
    dims, mass = (8, 8, 8, 16), 0.1
    gauge, src = wd.gen_gauge(dims, seed=1, eps=0.5), wd.gen_source(dims, seed=1)
    out = {"dims": np.array(dims), "mass": mass, "gauge_seed": 1, "source_seed": 1, "eps": 0.5,
           "stride": DIGEST_STRIDE}

    def digest(name, v):
        out[f"{name}_norm"] = np.linalg.norm(v)
        out[f"{name}_sample"] = np.ascontiguousarray(v[::DIGEST_STRIDE])

    for dag in (0, 1):
        for cb in (0, 1):
            digest(f"offd_new_dag{dag}_cb{cb}", ref.dslashoffd_new(src, gauge, dims, dag, cb))
        digest(f"full_new_dag{dag}", ref.dslash_new(src, gauge, dims, mass, dag))
    digest("full_old_dag1", ref.dslash_old(src, gauge, dims, mass, 1))
    x, iters, rsd = ref.cginvert(src, gauge, dims, mass, 1000, 1e-10, 7)
    out.update(cg_seed=7, cg_max=1000, cg_acc=1e-10, cg_iters=iters, cg_rsd=rsd)
    digest("cg_x", x)
    np.savez_compressed(HERE / "wilson_8x8x8x16_digest.npz", **out)
    print("8^3x16 digests written; CG:", iters, "iterations, |r| =", rsd)


if __name__ == "__main__":
    main()
