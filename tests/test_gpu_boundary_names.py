"""The short entry-point names of the drop-in boundary (wd_ctx_create,
wd_gauge_upload, wd_fermion_upload/download, wd_M, wd_cg), called through the
C ABI: M against the oracle's DslashNew (relative L2 <= 1e-13) and wd_cg in
its flag combinations checked by the FP64 true residual."""
import ctypes as C

import numpy as np
import pytest

from oracle import rel_l2

pytestmark = pytest.mark.gpu


def test_short_names(wd, oracle):
    lib = wd.lib
    dims = (8, 4, 6, 8)
    gauge = wd.gen_gauge(dims, seed=21)
    src = wd.gen_source(dims, seed=21)
    ctx = C.c_void_p()
    assert lib.wd_ctx_create(0, C.byref(ctx)) == wd.OK
    try:
        lat = C.c_void_p()
        assert lib.wd_gauge_upload(ctx, wd._gauge_ptrs(gauge), wd._dims(dims), C.byref(lat)) == wd.OK
        fi, fo = C.c_void_p(), C.c_void_p()
        assert lib.wd_field_create(ctx, lat, C.byref(fi)) == wd.OK
        assert lib.wd_field_create(ctx, lat, C.byref(fo)) == wd.OK
        assert lib.wd_fermion_upload(ctx, fi, wd._ptr(src)) == wd.OK
        out = np.empty_like(src)
        for dag in (0, 1):
            assert lib.wd_M(ctx, lat, fi, fo, 0.07, dag) == wd.OK
            assert lib.wd_fermion_download(ctx, fo, wd._ptr(out)) == wd.OK
            assert rel_l2(out, oracle.dslash_full(src, gauge, dims, 0.07, dag)) < 1e-13
        flags_list = [0, 1, (wd.DF64 << 1), (wd.F32 << 1) | 8, (wd.F16 << 1) | 8]
        for flags in flags_list:
            st = wd.SolverStats()
            assert lib.wd_fermion_upload(ctx, fo, wd._ptr(np.zeros_like(src))) == wd.OK
            rc = lib.wd_cg(ctx, lat, fi, fo, 0.1, 1e-10, 2000, flags, C.byref(st))
            assert rc == wd.OK, flags
            assert st.converged and st.true_residual <= 1e-10, (flags, st.true_residual)
        lib.wd_field_destroy(fi)
        lib.wd_field_destroy(fo)
        lib.wd_lattice_destroy(lat)
    finally:
        lib.wd_ctx_destroy(ctx)
