"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the CPU oracle.

`liboracle.so` is the plain-C restatement (wilson_oracle.c) of the reference
Wilson operator and CG; `_ref/libref.so` is the reference's own sources built
single-rank (x86-64 only, where the reference tree is present).  Tests, the
smoke check and the CPU-baseline leg of the benchmark use these to check or
time; the product never imports this module.

Arrays are numpy complex128 in the reference layout (fermion V*12, gauge 4 x V*9).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref.so"
REF_FAST_LIB = HERE / "_ref" / "libref_fast.so"


def build(reference_tree: str | None = None) -> None:
    """Compile the C restatement (and, where possible, the reference itself)."""
    cmd = ["make", "-C", str(HERE), "-s"]
    if reference_tree:
        cmd.append(f"REF={reference_tree}")
    subprocess.run(cmd, check=True)


def _p(a: np.ndarray):
    if a.dtype != np.complex128 or not a.flags.c_contiguous:
        raise TypeError("expected C-contiguous complex128")
    return C.c_void_p(a.ctypes.data)


def _g(gauge):
    return (C.c_void_p * 4)(*[_p(g).value for g in gauge])


def _d(dims):
    return (C.c_int * 4)(*[int(v) for v in dims])


class Oracle:
    """The C restatement."""

    def __init__(self, path: Path = ORACLE_LIB):
        if not path.exists():
            build()
        self.lib = C.CDLL(str(path))
        vp, d4, ip = C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_int)
        L = self.lib
        L.wo_num_threads.argtypes, L.wo_num_threads.restype = [C.c_int], C.c_int
        L.wo_dslash_offd.argtypes, L.wo_dslash_offd.restype = [vp, vp, d4, ip, C.c_int, C.c_int], None
        L.wo_dslash_eeoo.argtypes, L.wo_dslash_eeoo.restype = [vp, vp, ip, C.c_double], None
        L.wo_dslash_full.argtypes, L.wo_dslash_full.restype = [vp, vp, d4, ip, C.c_double, C.c_int], None
        L.wo_norm2.argtypes, L.wo_norm2.restype = [vp, C.c_long], C.c_double
        L.wo_dot.argtypes, L.wo_dot.restype = [vp, vp, C.c_long, C.POINTER(C.c_double)], None
        L.wo_srand.argtypes, L.wo_srand.restype = [C.c_uint], None
        L.wo_rand_guess.argtypes, L.wo_rand_guess.restype = [vp, C.c_long], None
        L.wo_rand_fill.argtypes, L.wo_rand_fill.restype = [vp, C.c_long], None
        L.wo_cg_ref.argtypes = [vp, vp, d4, ip, C.c_double, C.c_int, C.c_double, C.POINTER(C.c_double)]
        L.wo_cg_ref.restype = C.c_int
        L.wo_check.argtypes, L.wo_check.restype = [vp, vp, d4, ip, C.c_double, C.POINTER(C.c_double)], None
        L.wo_cg_eo.argtypes = [vp, vp, d4, ip, C.c_double, C.c_int, C.c_double, C.POINTER(C.c_double)]
        L.wo_cg_eo.restype = C.c_int
        L.wo_gen_gauge.argtypes, L.wo_gen_gauge.restype = [ip, C.c_uint64, C.c_double, d4], C.c_int
        L.wo_gen_source.argtypes, L.wo_gen_source.restype = [ip, C.c_uint64, vp], C.c_int

    def threads(self, n: int = 0) -> int:
        return self.lib.wo_num_threads(n)

    def gen_gauge(self, dims, seed: int, eps: float = 0.5) -> list[np.ndarray]:
        """Seeded SU(3) links exp(i eps H) in the reference layout: the package's
        generator (csrc/wd_gen.cpp) compiled into this library, so a CPU-only run
        gets the GPU path's input bytes without loading the CUDA library."""
        V = int(np.prod(dims))
        gauge = [np.empty(V * 9, np.complex128) for _ in range(4)]
        if self.lib.wo_gen_gauge(_d(dims), int(seed), float(eps), _g(gauge)) != 0:
            raise ValueError(f"bad lattice extents {tuple(dims)}")
        return gauge

    def gen_source(self, dims, seed: int) -> np.ndarray:
        """Seeded unit-norm Gaussian source (the package's generator)."""
        src = np.empty(int(np.prod(dims)) * 12, np.complex128)
        if self.lib.wo_gen_source(_d(dims), int(seed), _p(src)) != 0:
            raise ValueError(f"bad lattice extents {tuple(dims)}")
        return src

    def dslash_offd(self, src, gauge, dims, dag: bool, cb: int) -> np.ndarray:
        out = np.empty_like(src)
        self.lib.wo_dslash_offd(_p(src), _p(out), _g(gauge), _d(dims), int(dag), int(cb))
        return out

    def dslash_eeoo(self, src, dims, mass: float) -> np.ndarray:
        out = np.empty_like(src)
        self.lib.wo_dslash_eeoo(_p(src), _p(out), _d(dims), float(mass))
        return out

    def dslash_full(self, src, gauge, dims, mass: float, dag: bool) -> np.ndarray:
        out = np.empty_like(src)
        self.lib.wo_dslash_full(_p(src), _p(out), _g(gauge), _d(dims), float(mass), int(dag))
        return out

    def norm2(self, a) -> float:
        return self.lib.wo_norm2(_p(a), a.size)

    def dot(self, a, b) -> complex:
        o = (C.c_double * 2)()
        self.lib.wo_dot(_p(a), _p(b), a.size, o)
        return complex(o[0], o[1])

    def rand_guess(self, n: int, seed: int) -> np.ndarray:
        """The reference's CG initial guess: srand(seed), then rand()/RAND_MAX real parts."""
        x = np.empty(n, np.complex128)
        self.lib.wo_srand(seed)
        self.lib.wo_rand_guess(_p(x), n)
        return x

    def main_inputs(self, dims, seed: int) -> tuple[np.ndarray, np.ndarray]:
        """The source and CG initial guess the reference's main() draws from
        one rand() stream after srand(seed) (src/main.cpp:77-94, src/invert.cpp:42-44)."""
        V = int(np.prod(dims))
        raw = np.empty(V * 24, np.float64)
        self.lib.wo_srand(seed)
        self.lib.wo_rand_fill(C.c_void_p(raw.ctypes.data), raw.size)
        src = np.ascontiguousarray(raw[0::2] + 1j * raw[1::2])
        x0 = np.empty(V * 12, np.complex128)
        self.lib.wo_rand_guess(_p(x0), x0.size)
        return src, x0

    def cg_ref(self, src, gauge, dims, mass, max_iter, accuracy, x0) -> tuple[np.ndarray, int, float]:
        x = np.array(x0, dtype=np.complex128, copy=True)
        rsd = C.c_double()
        it = self.lib.wo_cg_ref(_p(src), _p(x), _g(gauge), _d(dims), float(mass), int(max_iter), float(accuracy),
                                C.byref(rsd))
        return x, it, rsd.value

    def cg_eo(self, src, gauge, dims, mass, tol: float = 1e-14, max_iter: int = 5000
              ) -> tuple[np.ndarray, int, float]:
        """Even-odd (Schur) CG from a zero guess until the normal residual is
        tol relative; returns (solution, iterations, FP64 true residual
        |b - Mx|/|b|).  Reference solutions at large volumes."""
        x = np.empty_like(src)
        res = C.c_double()
        it = self.lib.wo_cg_eo(_p(src), _p(x), _g(gauge), _d(dims), float(mass), int(max_iter), float(tol),
                               C.byref(res))
        return x, it, res.value

    def check(self, b, x, gauge, dims, mass) -> np.ndarray:
        o = (C.c_double * 12)()
        self.lib.wo_check(_p(b), _p(x), _g(gauge), _d(dims), float(mass), o)
        return np.array(o[:])


class Reference:
    """The reference's own sources, single rank (only where they were compiled)."""

    def __init__(self, path: Path = REF_LIB):
        if not path.exists():
            raise FileNotFoundError(f"{path} not built (needs the reference tree on x86-64)")
        self.lib = C.CDLL(str(path))
        vp, d4, ip = C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_int)
        L = self.lib
        for n in ("ref_dslash_new", "ref_dslash_old"):
            getattr(L, n).argtypes = [vp, vp, d4, ip, C.c_double, C.c_int]
            getattr(L, n).restype = None
        for n in ("ref_dslashoffd_new", "ref_dslashoffd_old"):
            getattr(L, n).argtypes = [vp, vp, d4, ip, C.c_int, C.c_int]
            getattr(L, n).restype = None
        L.ref_dslash_eeoo_new.argtypes, L.ref_dslash_eeoo_new.restype = [vp, vp, ip, C.c_double], None
        L.ref_cginvert.argtypes = [vp, vp, d4, ip, C.c_double, C.c_int, C.c_double, C.c_uint,
                                   C.POINTER(C.c_double)]
        L.ref_cginvert.restype = C.c_int
        L.ref_check.argtypes, L.ref_check.restype = [vp, vp, d4, ip, C.c_double, C.c_char_p, C.c_int], C.c_int

    def dslash_new(self, src, gauge, dims, mass, dag) -> np.ndarray:
        src, gauge, out = aligned(src), [aligned(g) for g in gauge], aligned(np.zeros_like(src))
        self.lib.ref_dslash_new(_p(src), _p(out), _g(gauge), _d(dims), float(mass), int(dag))
        return out

    def dslash_old(self, src, gauge, dims, mass, dag) -> np.ndarray:
        src, gauge, out = aligned(src), [aligned(g) for g in gauge], aligned(np.zeros_like(src))
        self.lib.ref_dslash_old(_p(src), _p(out), _g(gauge), _d(dims), float(mass), int(dag))
        return out

    def dslashoffd_new(self, src, gauge, dims, dag, cb) -> np.ndarray:
        src, gauge, out = aligned(src), [aligned(g) for g in gauge], aligned(np.zeros_like(src))
        self.lib.ref_dslashoffd_new(_p(src), _p(out), _g(gauge), _d(dims), int(dag), int(cb))
        return out

    def dslashoffd_old(self, src, gauge, dims, dag, cb) -> np.ndarray:
        src, gauge, out = aligned(src), [aligned(g) for g in gauge], aligned(np.zeros_like(src))
        self.lib.ref_dslashoffd_old(_p(src), _p(out), _g(gauge), _d(dims), int(dag), int(cb))
        return out

    def dslash_eeoo_new(self, src, dims, mass) -> np.ndarray:
        src, out = aligned(src), aligned(np.zeros_like(src))
        self.lib.ref_dslash_eeoo_new(_p(src), _p(out), _d(dims), float(mass))
        return out

    def cginvert(self, src, gauge, dims, mass, max_iter, accuracy, seed) -> tuple[np.ndarray, int, float]:
        src, gauge, x = aligned(src), [aligned(g) for g in gauge], aligned(np.zeros_like(src))
        rsd = C.c_double(-1.0)
        it = self.lib.ref_cginvert(_p(src), _p(x), _g(gauge), _d(dims), float(mass), int(max_iter),
                                   float(accuracy), int(seed), C.byref(rsd))
        return x, it, rsd.value

    def check_text(self, src, x, gauge, dims, mass) -> str:
        src, x, gauge = aligned(src), aligned(x), [aligned(g) for g in gauge]
        buf = C.create_string_buffer(8192)
        self.lib.ref_check(_p(src), _p(x), _g(gauge), _d(dims), float(mass), buf, 8192)
        return buf.value.decode()


def aligned(a: np.ndarray, align: int = 64) -> np.ndarray:
    """Copy into a complex128 buffer aligned to `align` bytes (the reference's
    AVX code uses aligned 32-byte loads on fermion arrays)."""
    a = np.asarray(a, dtype=np.complex128).ravel()
    raw = np.empty(a.size * 16 + align, np.uint8)
    off = (-raw.ctypes.data) % align
    out = raw[off:off + a.size * 16].view(np.complex128)
    out[:] = a
    return out


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
