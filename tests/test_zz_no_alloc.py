"""wd_dot_noalloc: the dot product for callers that cannot allocate device
memory (codes that give all of HBM to their own pool, and loops that must not
call cudaMalloc/cudaFree because those synchronise the device).

It is checked through the C ABI against the context-based wd_dot on the same
data, on two calls in a row with different sizes (the second call must not
see the first one's partial sums).  This file sorts last so that a run that
stops at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-13


def noalloc(wd):
    f = wd.lib.wd_dot_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    return f


def _call(wd, f, a, b):
    import torch

    da = torch.from_numpy(a).to("cuda")
    db = torch.from_numpy(b).to("cuda")
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    st = f(da.data_ptr(), db.data_ptr(), a.size, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert st == wd.OK
    torch.cuda.synchronize()
    return complex(*out.cpu().numpy())


def test_dot_noalloc_matches_dot_on_two_calls(wd, ctx):
    """Lattice fields of 3 chunks, then 1 chunk, then 3 chunks again: each
    call against wd_dot on the same data."""
    f = noalloc(wd)
    for dims, seed in (((8, 4, 4, 8), 11), ((4, 4, 2, 4), 12), ((8, 4, 4, 8), 13)):
        a = wd.gen_source(dims, seed)
        b = wd.gen_source(dims, seed + 100) + 0.5j * a
        lat = ctx.lattice(dims, wd.gen_gauge(dims, seed))
        expected = lat.field(a).dot(lat.field(b))          # existing entry point
        got = _call(wd, f, a, b)
        assert abs(got - expected) <= TOL * abs(expected), (got, expected)


def test_dot_noalloc_partial_last_chunk(wd, ctx):
    """A small call, then n = 2*4096 + 17 (three chunks, the last one partial)
    from flat arrays, against numpy: a wrong chunk count or stale partial sums
    from the earlier calls would show."""
    f = noalloc(wd)
    rng = np.random.default_rng(21)
    for n in (100, 2 * 4096 + 17):
        a = rng.normal(size=n) + 1j * rng.normal(size=n)
        b = rng.normal(size=n) + 1j * rng.normal(size=n)
        expected = np.vdot(a, b)
        got = _call(wd, f, a, b)
        assert abs(got - expected) <= TOL * abs(expected), (n, got, expected)


def test_dot_noalloc_limits(wd, ctx):
    import torch

    f = noalloc(wd)
    d = torch.zeros(8, dtype=torch.complex128, device="cuda")
    out = torch.full((2,), 7.0, dtype=torch.float64, device="cuda")
    # beyond the fixed scratch capacity: rejected before anything is launched
    assert f(d.data_ptr(), d.data_ptr(), 32768 * 4096 + 1, out.data_ptr(), None) == wd.BAD_ARG
    assert f(d.data_ptr(), d.data_ptr(), -1, out.data_ptr(), None) == wd.BAD_ARG
    assert f(None, d.data_ptr(), 8, out.data_ptr(), None) == wd.BAD_ARG
    # empty input gives zero
    assert f(d.data_ptr(), d.data_ptr(), 0, out.data_ptr(), None) == wd.OK
    torch.cuda.synchronize()
    assert out.cpu().tolist() == [0.0, 0.0]
