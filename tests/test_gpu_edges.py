"""Edge cases on the GPU: a zero source (every solver returns the zero
solution at once, no NaN), a lattice larger than HBM (OOM, and the context
stays usable), a lattice above the site limit (BAD_DIMS)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_zero_source_every_solver(wd, ctx):
    dims = (8, 4, 4, 8)
    lat = ctx.lattice(dims, wd.gen_gauge(dims, seed=3))
    b = lat.field(np.zeros(int(np.prod(dims)) * 12, np.complex128))
    x = lat.field()
    plans = [(wd.CG_EO, wd.F64, wd.F64), (wd.CG_EO, wd.DF64, wd.F64), (wd.CG_EO, wd.F32, wd.F64),
             (wd.CG_EO, wd.F16, wd.DF64)]
    for kind, prec, rel in plans:
        st = lat.solve(b, x, wd.solver_params(kind=kind, mass=0.1, tol=1e-10, prec=prec, prec_reliable=rel))
        sol = x.download()
        assert st.converged and np.all(sol == 0), (kind, prec)
        assert np.isfinite(st.true_residual)
    # batched, with one zero and one Gaussian source
    x2 = lat.field()
    b2 = lat.field(wd.gen_source(dims, seed=3))
    stats = ctx.solve_batch([(lat, b, x, 0.1), (lat, b2, x2, 0.1)],
                            wd.solver_params(kind=wd.CG_EO, tol=1e-10, prec=wd.F32, prec_reliable=wd.DF64))
    assert all(s.converged for s in stats)
    assert np.all(x.download() == 0) and stats[1].true_residual <= 1e-10


def test_lattice_larger_than_hbm_is_oom(wd, ctx):
    dummy = [np.zeros(9, np.complex128) for _ in range(4)]  # never read: allocation fails first
    h = C.c_void_p()
    st = wd.lib.wd_lattice_create(ctx.handle, wd._dims((256, 256, 128, 128)), wd._gauge_ptrs(dummy), C.byref(h))
    assert st == wd.OOM and not h.value
    st = wd.lib.wd_lattice_create(ctx.handle, wd._dims((512, 256, 128, 128)), wd._gauge_ptrs(dummy), C.byref(h))
    assert st == wd.BAD_DIMS
    # the context still works
    dims = (4, 4, 4, 4)
    lat = ctx.lattice(dims, wd.gen_gauge(dims, seed=1))
    f = lat.field(wd.gen_source(dims, seed=1))
    assert abs(f.norm2() - 1.0) < 1e-12
