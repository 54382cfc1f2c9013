"""Python binding of libwilson_gb300 (ctypes over the C ABI in include/wilson_gb300.h).

Fields cross the boundary as numpy complex128 arrays in the reference layout:
fermions have V*12 entries (eo*12 + spin*3 + colour), gauge fields are four
arrays of V*9 entries (eo*9 + row*3 + col), V = Lx*Ly*Lz*Lt with Lx even.

The compute path is the CUDA library only: if it is not built, importing
this module raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libwilson_gb300.so"

# wd_status
OK, BAD_DIMS, OOM, NOT_CONVERGED, TIMEOUT, CUDA_ERROR, BAD_ARG, NO_DEVICE, NAN = range(9)
# wd_precision
F64, DF64, F32, F16 = range(4)
# wd_solver_kind
CGNR_REF, CG_EO = range(2)


class WilsonError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


class SolverParams(C.Structure):
    _fields_ = [("kind", C.c_int), ("mass", C.c_double), ("tol", C.c_double), ("max_iter", C.c_int),
                ("prec", C.c_int), ("delta", C.c_double), ("use_initial_guess", C.c_int),
                ("prec_reliable", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("prec", C.c_int), ("prec_reliable", C.c_int), ("hbm_budget_bytes", C.c_double),
                ("max_systems", C.c_int), ("max_iter", C.c_int), ("delta", C.c_double)]


class SolverStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("reliable_updates", C.c_int), ("residual", C.c_double),
                ("true_residual", C.c_double), ("seconds", C.c_double), ("converged", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is not built; run __graft_entry__.build() first")
    lib = C.CDLL(str(LIB_PATH))
    vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    d4 = C.POINTER(C.c_void_p)
    sigs = {
        "wd_context_create": (C.c_int, [C.c_int, C.POINTER(vp)]),
        "wd_read_gauge_file": (C.c_int, [C.c_char_p, ip, C.c_int, d4, ip]),
        "wd_ctx_create": (C.c_int, [C.c_int, C.POINTER(vp)]),
        "wd_ctx_destroy": (None, [vp]),
        "wd_gauge_upload": (C.c_int, [vp, d4, ip, C.POINTER(vp)]),
        "wd_fermion_upload": (C.c_int, [vp, vp, vp]),
        "wd_fermion_download": (C.c_int, [vp, vp, vp]),
        "wd_M": (C.c_int, [vp, vp, vp, vp, C.c_double, C.c_int]),
        "wd_cg": (C.c_int, [vp, vp, vp, vp, C.c_double, C.c_double, C.c_int, C.c_int, C.POINTER(SolverStats)]),
        "wd_context_destroy": (None, [vp]),
        "wd_status_string": (C.c_char_p, [C.c_int]),
        "wd_last_error": (C.c_char_p, [vp]),
        "wd_context_sync": (C.c_int, [vp]),
        "wd_context_stream": (vp, [vp]),
        "wd_context_launches": (C.c_uint64, [vp]),
        "wd_context_device_check": (C.c_int, [vp]),
        "wd_debug_expire_wait": (C.c_int, [vp, C.POINTER(C.c_double)]),
        "wd_debug_fail_allocations_after": (C.c_int, [vp, C.c_int]),
        "wd_lattice_create": (C.c_int, [vp, ip, d4, C.POINTER(vp)]),
        "wd_lattice_update": (C.c_int, [vp, vp, d4]),
        "wd_lattice_destroy": (None, [vp]),
        "wd_lattice_volume": (C.c_int64, [vp]),
        "wd_field_create": (C.c_int, [vp, vp, C.POINTER(vp)]),
        "wd_field_create_prec": (C.c_int, [vp, vp, C.c_int, C.POINTER(vp)]),
        "wd_field_precision": (C.c_int, [vp]),
        "wd_field_destroy": (None, [vp]),
        "wd_field_upload": (C.c_int, [vp, vp, vp]),
        "wd_field_download": (C.c_int, [vp, vp, vp]),
        "wd_field_zero": (C.c_int, [vp, vp]),
        "wd_field_copy": (C.c_int, [vp, vp, vp]),
        "wd_dslash_offd": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int, C.c_int]),
        "wd_dslash_eo": (C.c_int, [vp, vp, vp, vp, C.c_int, C.c_int, C.c_int]),
        "wd_dslash_eeoo": (C.c_int, [vp, vp, vp, vp, C.c_double]),
        "wd_diag_fma_peak": (C.c_int, [vp, dp, dp]),
        "wd_dslash_full": (C.c_int, [vp, vp, vp, vp, C.c_double, C.c_int, C.c_int]),
        "wd_norm2": (C.c_int, [vp, vp, dp]),
        "wd_dot": (C.c_int, [vp, vp, vp, dp]),
        "wd_solver_params_default": (None, [C.POINTER(SolverParams)]),
        "wd_solve": (C.c_int, [vp, vp, vp, vp, C.POINTER(SolverParams), C.POINTER(SolverStats)]),
        "wd_check": (C.c_int, [vp, vp, vp, vp, C.c_double, dp]),
        "wd_solve_batch": (C.c_int, [vp, C.c_int, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), dp,
                                     C.POINTER(SolverParams), C.POINTER(SolverStats)]),
        "wd_host_dslash_offd": (C.c_int, [vp, ip, d4, vp, vp, C.c_int, C.c_int]),
        "wd_host_dslash_full": (C.c_int, [vp, ip, d4, vp, vp, C.c_double, C.c_int]),
        "wd_host_cg": (C.c_int, [vp, ip, d4, vp, vp, C.POINTER(SolverParams), C.POINTER(SolverStats)]),
        "wd_point_source": (C.c_int, [vp, vp, ip, C.c_int, C.c_int]),
        "wd_propagator": (C.c_int, [vp, vp, ip, C.POINTER(SolverParams), C.POINTER(vp), C.POINTER(SolverStats)]),
        "wd_pion_correlator": (C.c_int, [vp, vp, C.POINTER(vp), dp]),
        "wd_server_config_default": (None, [C.POINTER(ServerConfig)]),
        "wd_server_create": (C.c_int, [vp, C.POINTER(ServerConfig), C.POINTER(vp)]),
        "wd_server_destroy": (None, [vp]),
        "wd_server_add_lattice": (C.c_int, [vp, ip, d4, ip]),
        "wd_server_submit": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(vp), C.POINTER(C.c_uint64), C.c_double,
                                       C.c_double, C.POINTER(C.c_int64)]),
        "wd_server_step": (C.c_int, [vp, ip]),
        "wd_server_poll": (C.c_int, [vp, C.c_int64, ip, C.POINTER(vp), C.POINTER(SolverStats),
                                     C.POINTER(C.c_double)]),
        "wd_server_status": (C.c_int, [vp, ip, ip, dp]),
        "wd_tune_report": (C.c_int, [C.c_char_p, C.c_int]),
        "wd_tune_enable": (None, [C.c_int]),
        "wd_tune_pin": (C.c_int, [C.c_int, C.c_char_p, C.c_int, C.c_int]),
        "wd_tune_variants": (C.c_int, [C.c_char_p]),
        "wd_gen_gauge": (C.c_int, [ip, C.c_uint64, C.c_double, d4]),
        "wd_gen_source": (C.c_int, [ip, C.c_uint64, vp]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()

# every symbol the public header declares (checked by the CPU tests)
HEADER = _HERE.parent.parent / "include" / "wilson_gb300.h"


def _dims(dims) -> C.Array:
    d = [int(v) for v in dims]
    if len(d) != 4:
        raise ValueError("dims must have 4 entries (Lx, Ly, Lz, Lt)")
    return (C.c_int * 4)(*d)


def _ptr(a: np.ndarray) -> C.c_void_p:
    if a.dtype != np.complex128 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous complex128 array")
    return C.c_void_p(a.ctypes.data)


def _gauge_ptrs(gauge) -> C.Array:
    if len(gauge) != 4:
        raise ValueError("gauge must be four arrays (one per direction)")
    return (C.c_void_p * 4)(*[_ptr(g).value for g in gauge])


def volume(dims) -> int:
    return int(np.prod([int(v) for v in dims]))


def tune_report() -> list[tuple]:
    """Autotuner decisions: (device, kernel, half-volume, variant, ms)."""
    buf = C.create_string_buffer(65536)
    lib.wd_tune_report(buf, len(buf))
    out = []
    for line in buf.value.decode().splitlines():
        d, k, vh, v, ms = line.split()
        out.append((int(d), k, int(vh), int(v), float(ms)))
    return out


def tune_pin(kernel: str, half_volume: int, variant: int, device: int = 0) -> None:
    """Pin a hopping kernel's launch variant for one half-volume (variant < 0 unpins)."""
    if lib.wd_tune_pin(device, kernel.encode(), half_volume, variant) != 0:
        raise ValueError(f"cannot pin {kernel} variant {variant} at half-volume {half_volume}")


def tune_variants(kernel: str) -> int:
    """Launch variants of a hopping kernel (0 until it has launched once)."""
    return lib.wd_tune_variants(kernel.encode())


GAUGE_FILE_AUTO, GAUGE_FILE_REF, GAUGE_FILE_NERSC, GAUGE_FILE_ILDG = range(4)


def read_gauge_file(path: str, dims, fmt: int = GAUGE_FILE_AUTO) -> tuple[list[np.ndarray], int]:
    """A gauge-configuration file (reference / NERSC / ILDG) in the reference
    layout (4 arrays of V*9); returns (links, format read)."""
    V = volume(dims)
    g = [np.empty(V * 9, np.complex128) for _ in range(4)]
    found = C.c_int(-1)
    st = lib.wd_read_gauge_file(str(path).encode(), _dims(dims), fmt, _gauge_ptrs(g), C.byref(found))
    if st != OK:
        raise WilsonError(st, f"cannot read gauge file {path}: {lib.wd_status_string(st).decode()}")
    return g, found.value


def gen_gauge(dims, seed: int, eps: float = 0.5) -> list[np.ndarray]:
    """Seeded SU(3) links exp(i eps H) in the reference layout (4 arrays of V*9)."""
    V = volume(dims)
    g = [np.empty(V * 9, np.complex128) for _ in range(4)]
    _check(lib.wd_gen_gauge(_dims(dims), seed, eps, _gauge_ptrs(g)), None)
    return g


def gen_source(dims, seed: int) -> np.ndarray:
    """Seeded complex Gaussian source (V*12), unit L2 norm."""
    s = np.empty(volume(dims) * 12, np.complex128)
    _check(lib.wd_gen_source(_dims(dims), seed, _ptr(s)), None)
    return s


def _check(status: int, ctx) -> None:
    if status != OK:
        detail = lib.wd_last_error(ctx.handle).decode() if ctx is not None else ""
        raise WilsonError(status, f"{lib.wd_status_string(status).decode()}: {detail}")


class Context:
    """One device + one CUDA stream.  Owns lattices and fields created from it."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        st = lib.wd_context_create(device, C.byref(h))
        if st != OK:
            raise WilsonError(st, lib.wd_status_string(st).decode())
        self.handle = h

    def close(self) -> None:
        if self.handle:
            lib.wd_context_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, status: int) -> None:
        _check(status, self)

    def sync(self) -> None:
        self.check(lib.wd_context_sync(self.handle))

    @property
    def stream(self) -> int:
        return lib.wd_context_stream(self.handle) or 0

    @property
    def launches(self) -> int:
        return int(lib.wd_context_launches(self.handle))

    def device_check(self) -> None:
        """Wait for the stream and raise (TIMEOUT) if a kernel's bounded wait gave up."""
        self.check(lib.wd_context_device_check(self.handle))

    def debug_expire_wait(self) -> float:
        """Testing aid: run a device wait that can only give up (after its
        0.5 s bound); returns how long it waited, in seconds."""
        w = C.c_double()
        self.check(lib.wd_debug_expire_wait(self.handle, C.byref(w)))
        return w.value

    def fail_allocations_after(self, n: int) -> int:
        """Testing aid: the next allocations after n more successful ones fail
        with OOM (n < 0: off).  Returns the previous setting."""
        return int(lib.wd_debug_fail_allocations_after(self.handle, int(n)))

    def fma_peak(self) -> tuple[float, float]:
        """Measured (FP64, FP32) FMA throughput of the device in TFLOP/s."""
        a, b = C.c_double(), C.c_double()
        self.check(lib.wd_diag_fma_peak(self.handle, C.byref(a), C.byref(b)))
        return a.value, b.value

    def lattice(self, dims, gauge) -> "Lattice":
        return Lattice(self, dims, gauge)

    def solve_batch(self, systems, params: SolverParams, allow_unconverged: bool = False) -> list[SolverStats]:
        """systems: sequence of (lattice, src Field, dest Field, mass).  Returns per-system stats."""
        n = len(systems)
        lats = (C.c_void_p * n)(*[s[0].handle.value for s in systems])
        srcs = (C.c_void_p * n)(*[s[1].handle.value for s in systems])
        dsts = (C.c_void_p * n)(*[s[2].handle.value for s in systems])
        masses = (C.c_double * n)(*[float(s[3]) for s in systems])
        stats = (SolverStats * n)()
        st = lib.wd_solve_batch(self.handle, n, lats, srcs, dsts, masses, C.byref(params), stats)
        if not (allow_unconverged and st == NOT_CONVERGED):
            self.check(st)
        return list(stats)

    # host-buffer entry points (reference layout in and out)
    def host_dslash_offd(self, dims, gauge, src: np.ndarray, dag: bool, cb: int) -> np.ndarray:
        out = np.empty_like(src)
        self.check(lib.wd_host_dslash_offd(self.handle, _dims(dims), _gauge_ptrs(gauge), _ptr(src), _ptr(out),
                                           int(dag), int(cb)))
        return out

    def host_dslash_full(self, dims, gauge, src: np.ndarray, mass: float, dag: bool) -> np.ndarray:
        out = np.empty_like(src)
        self.check(lib.wd_host_dslash_full(self.handle, _dims(dims), _gauge_ptrs(gauge), _ptr(src), _ptr(out),
                                           float(mass), int(dag)))
        return out

    def host_cg(self, dims, gauge, src: np.ndarray, dest: np.ndarray, params: SolverParams,
                allow_unconverged: bool = False) -> SolverStats:
        stats = SolverStats()
        st = lib.wd_host_cg(self.handle, _dims(dims), _gauge_ptrs(gauge), _ptr(src), _ptr(dest), C.byref(params),
                            C.byref(stats))
        if not (allow_unconverged and st == NOT_CONVERGED):
            self.check(st)
        return stats


class Lattice:
    """Lattice extents plus the resident gauge field."""

    def __init__(self, ctx: Context, dims, gauge):
        self.ctx = ctx
        self.dims = tuple(int(v) for v in dims)
        self.V = volume(dims)
        h = C.c_void_p()
        ctx.check(lib.wd_lattice_create(ctx.handle, _dims(dims), _gauge_ptrs(gauge), C.byref(h)))
        self.handle = h

    def update(self, gauge) -> None:
        self.ctx.check(lib.wd_lattice_update(self.ctx.handle, self.handle, _gauge_ptrs(gauge)))

    def close(self) -> None:
        if self.handle:
            lib.wd_lattice_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field(self, host: np.ndarray | None = None, prec: int = F64) -> "Field":
        f = Field(self, prec)
        if host is not None:
            f.upload(host)
        return f

    # operators
    def dslash_offd(self, src: "Field", dest: "Field", dag: bool, cb: int, prec: int = F64) -> None:
        self.ctx.check(lib.wd_dslash_offd(self.ctx.handle, self.handle, src.handle, dest.handle, int(dag), int(cb),
                                          int(prec)))

    def dslash_eo(self, src: "Field", dest: "Field", dag: bool, cb: int, prec: int = F64) -> None:
        self.ctx.check(lib.wd_dslash_eo(self.ctx.handle, self.handle, src.handle, dest.handle, int(dag), int(cb),
                                        int(prec)))

    def dslash_eeoo(self, src: "Field", dest: "Field", mass: float) -> None:
        self.ctx.check(lib.wd_dslash_eeoo(self.ctx.handle, self.handle, src.handle, dest.handle, float(mass)))

    def dslash_full(self, src: "Field", dest: "Field", mass: float, dag: bool, prec: int = F64) -> None:
        self.ctx.check(lib.wd_dslash_full(self.ctx.handle, self.handle, src.handle, dest.handle, float(mass),
                                          int(dag), int(prec)))

    def solve(self, src: "Field", dest: "Field", params: SolverParams, allow_unconverged: bool = False) -> SolverStats:
        stats = SolverStats()
        st = lib.wd_solve(self.ctx.handle, self.handle, src.handle, dest.handle, C.byref(params), C.byref(stats))
        if not (allow_unconverged and st == NOT_CONVERGED):
            self.ctx.check(st)
        return stats

    def propagator(self, x_src, params: SolverParams):
        """12 FP64 fields M^-1 (point source at x_src, spin s, colour c), index s*3+c, and their stats."""
        props = [self.field() for _ in range(12)]
        arr = (C.c_void_p * 12)(*[f.handle.value for f in props])
        stats = (SolverStats * 12)()
        self.ctx.check(lib.wd_propagator(self.ctx.handle, self.handle, (C.c_int * 4)(*x_src), C.byref(params), arr,
                                         stats))
        return props, list(stats)

    def pion_correlator(self, props) -> np.ndarray:
        ct = np.zeros(self.dims[3], np.float64)
        arr = (C.c_void_p * 12)(*[f.handle.value for f in props])
        self.ctx.check(lib.wd_pion_correlator(self.ctx.handle, self.handle, arr,
                                              ct.ctypes.data_as(C.POINTER(C.c_double))))
        return ct

    def check(self, b: "Field", x: "Field", mass: float) -> np.ndarray:
        out = np.zeros(12, np.float64)
        self.ctx.check(lib.wd_check(self.ctx.handle, self.handle, b.handle, x.handle, float(mass),
                                    out.ctypes.data_as(C.POINTER(C.c_double))))
        return out


class Field:
    """Resident FP64 spinor field over the full lattice."""

    def __init__(self, lat: Lattice, prec: int = F64):
        self.lat = lat
        self.prec = prec
        h = C.c_void_p()
        lat.ctx.check(lib.wd_field_create_prec(lat.ctx.handle, lat.handle, int(prec), C.byref(h)))
        self.handle = h

    def upload(self, host: np.ndarray) -> None:
        if host.size != self.lat.V * 12:
            raise ValueError("field size mismatch")
        self.lat.ctx.check(lib.wd_field_upload(self.lat.ctx.handle, self.handle, _ptr(host)))

    def download(self) -> np.ndarray:
        out = np.empty(self.lat.V * 12, np.complex128)
        self.lat.ctx.check(lib.wd_field_download(self.lat.ctx.handle, self.handle, _ptr(out)))
        return out

    def zero(self) -> None:
        self.lat.ctx.check(lib.wd_field_zero(self.lat.ctx.handle, self.handle))

    def copy_from(self, other: "Field") -> None:
        self.lat.ctx.check(lib.wd_field_copy(self.lat.ctx.handle, self.handle, other.handle))

    def norm2(self) -> float:
        v = C.c_double()
        self.lat.ctx.check(lib.wd_norm2(self.lat.ctx.handle, self.handle, C.byref(v)))
        return v.value

    def dot(self, other: "Field") -> complex:
        v = (C.c_double * 2)()
        self.lat.ctx.check(lib.wd_dot(self.lat.ctx.handle, self.handle, other.handle, v))
        return complex(v[0], v[1])

    def close(self) -> None:
        if self.handle:
            lib.wd_field_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solver_params(kind: int = CG_EO, mass: float = 0.1, tol: float = 1e-10, max_iter: int = 1000,
                  prec: int = F64, delta: float = 0.1, use_initial_guess: bool = False,
                  prec_reliable: int = F64) -> SolverParams:
    p = SolverParams()
    lib.wd_solver_params_default(C.byref(p))
    p.kind, p.mass, p.tol, p.max_iter, p.prec, p.delta = kind, mass, tol, max_iter, prec, delta
    p.use_initial_guess = int(use_initial_guess)
    p.prec_reliable = prec_reliable
    return p


class Server:
    """Continuous-batching solve server on one context (see wd_server_* in the C header)."""

    def __init__(self, ctx: Context, prec: int = F32, prec_reliable: int = DF64, hbm_budget_bytes: float = 150e9,
                 max_systems: int = 256, max_iter: int = 5000, delta: float = 0.1):
        self.ctx = ctx
        cfg = ServerConfig()
        lib.wd_server_config_default(C.byref(cfg))
        cfg.prec, cfg.prec_reliable, cfg.hbm_budget_bytes = prec, prec_reliable, hbm_budget_bytes
        cfg.max_systems, cfg.max_iter, cfg.delta = max_systems, max_iter, delta
        h = C.c_void_p()
        ctx.check(lib.wd_server_create(ctx.handle, C.byref(cfg), C.byref(h)))
        self.handle = h
        self.dims = {}
        self.nsrc = {}

    def close(self) -> None:
        if self.handle:
            lib.wd_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_lattice(self, dims, gauge) -> int:
        i = C.c_int()
        self.ctx.check(lib.wd_server_add_lattice(self.handle, _dims(dims), _gauge_ptrs(gauge), C.byref(i)))
        self.dims[i.value] = tuple(int(v) for v in dims)
        return i.value

    def submit(self, lattice_id: int, nsrc: int, mass: float, tol: float, sources=None, seeds=None) -> int:
        rid = C.c_int64()
        src_arr = None
        seed_arr = None
        if sources is not None:
            src_arr = (C.c_void_p * nsrc)(*[_ptr(a).value for a in sources])
        else:
            seed_arr = (C.c_uint64 * nsrc)(*[int(v) for v in seeds])
        self.ctx.check(lib.wd_server_submit(self.handle, lattice_id, nsrc, src_arr, seed_arr, float(mass), float(tol),
                                            C.byref(rid)))
        self.nsrc[rid.value] = (lattice_id, nsrc)
        return rid.value

    def step(self) -> int:
        n = C.c_int()
        self.ctx.check(lib.wd_server_step(self.handle, C.byref(n)))
        return n.value

    def poll(self, rid: int, want_solutions: bool = False):
        """(done, solutions or None, stats list, latency seconds); collected requests are released."""
        lat, nsrc = self.nsrc[rid]
        done = C.c_int()
        stats = (SolverStats * nsrc)()
        lat_s = C.c_double()
        sols = None
        sol_ptrs = None
        if want_solutions:
            V = volume(self.dims[lat])
            sols = [np.empty(V * 12, np.complex128) for _ in range(nsrc)]
            sol_ptrs = (C.c_void_p * nsrc)(*[_ptr(a).value for a in sols])
        self.ctx.check(lib.wd_server_poll(self.handle, rid, C.byref(done), sol_ptrs, stats, C.byref(lat_s)))
        if not done.value:
            return False, None, None, None
        del self.nsrc[rid]
        return True, sols, list(stats), lat_s.value

    def status(self):
        q, a, b = C.c_int(), C.c_int(), C.c_double()
        self.ctx.check(lib.wd_server_status(self.handle, C.byref(q), C.byref(a), C.byref(b)))
        return q.value, a.value, b.value
