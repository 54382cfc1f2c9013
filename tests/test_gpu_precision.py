"""Hopping kernels in the other storage formats, and the solvers built on
them, against the FP64 oracle.

Bars: double-float (df64) output within 1e-13 relative L2 of the oracle (the
FP64 bar); FP32 with 12-real links within 2e-6; FP16 (per-site scale) within
5e-3.  Every solve is checked by its FP64 true residual |b - Mx|/|b| <= 1e-10
and its error against the oracle's 1e-13 solution <= 1e-9."""
import numpy as np
import pytest

from oracle import rel_l2

pytestmark = pytest.mark.gpu

BAR = {1: 1e-13, 2: 2e-6, 3: 5e-3}   # DF64, F32, F16


@pytest.fixture(scope="module")
def case(wd, ctx):
    dims = (8, 4, 6, 8)
    gauge = wd.gen_gauge(dims, seed=7)
    src = wd.gen_source(dims, seed=7)
    return dims, gauge, src, ctx.lattice(dims, gauge)


@pytest.mark.parametrize("prec", [1, 2, 3])
def test_roundtrip(wd, case, prec):
    dims, gauge, src, lat = case
    back = lat.field(src, prec=prec).download()
    tol = {1: 1e-14, 2: 1e-7, 3: 1e-3}[prec]
    assert rel_l2(back, src) < tol


@pytest.mark.parametrize("prec", [1, 2, 3])
def test_hopping_in_storage(wd, oracle, case, prec):
    dims, gauge, src, lat = case
    fi, fo = lat.field(src, prec=prec), lat.field(prec=prec)
    for dag in (0, 1):
        for cb in (0, 1):
            lat.dslash_offd(fi, fo, dag, cb, prec)
            assert rel_l2(fo.download(), oracle.dslash_offd(src, gauge, dims, dag, cb)) < BAR[prec]
        lat.dslash_full(fi, fo, 0.05, dag, prec)
        assert rel_l2(fo.download(), oracle.dslash_full(src, gauge, dims, 0.05, dag)) < BAR[prec]


def test_df64_arithmetic_on_fp64_fields(wd, oracle, case):
    dims, gauge, src, lat = case
    fi, fo = lat.field(src), lat.field()
    lat.dslash_full(fi, fo, 0.1, 1, wd.DF64)
    assert rel_l2(fo.download(), oracle.dslash_full(src, gauge, dims, 0.1, 1)) < 1e-13


def test_df64_reductions(wd, case):
    dims, gauge, src, lat = case
    a = lat.field(src, prec=wd.DF64)
    assert abs(a.norm2() - 1.0) < 1e-13
    b = lat.field(src * (0.5 - 0.25j), prec=wd.DF64)
    assert abs(a.dot(b) - (0.5 - 0.25j)) < 1e-13


def test_mismatched_storage_rejected(wd, case):
    dims, gauge, src, lat = case
    with pytest.raises(wd.WilsonError):
        lat.dslash_eo(lat.field(src, prec=wd.F32), lat.field(prec=wd.F16), 0, 0, wd.F32)
    with pytest.raises(wd.WilsonError):
        lat.dslash_eo(lat.field(src, prec=wd.F32), lat.field(prec=wd.F32), 0, 0, wd.F64)


@pytest.fixture(scope="module")
def solve_case(wd, oracle, ctx):
    dims = (8, 8, 8, 16)
    gauge = wd.gen_gauge(dims, seed=1)
    src = wd.gen_source(dims, seed=1)
    sols = {}
    for mass in (0.1, 0.01):
        sols[mass], _, _ = oracle.cg_ref(src, gauge, dims, mass, 5000, 1e-13, np.zeros_like(src))
    return dims, gauge, src, ctx.lattice(dims, gauge), sols


def _check_solution(wd, oracle, dims, gauge, src, x, mass, xo, st):
    assert st.converged, st.as_dict()
    assert st.true_residual <= 1e-10, st.as_dict()
    r = src - oracle.dslash_full(x, gauge, dims, mass, 0)
    assert np.linalg.norm(r) / np.linalg.norm(src) <= 1.05e-10
    assert rel_l2(x, xo) < 1e-9


@pytest.mark.parametrize("mass", [0.1, 0.01])
def test_cg_eo_df64(wd, oracle, solve_case, mass):
    dims, gauge, src, lat, sols = solve_case
    b, x = lat.field(src), lat.field()
    st = lat.solve(b, x, wd.solver_params(kind=wd.CG_EO, mass=mass, tol=1e-10, prec=wd.DF64))
    _check_solution(wd, oracle, dims, gauge, src, x.download(), mass, sols[mass], st)


def test_cgnr_ref_df64_matches_fp64(wd, oracle, solve_case):
    dims, gauge, src, lat, sols = solve_case
    x0 = oracle.rand_guess(src.size, 3)
    res = {}
    for prec in (wd.F64, wd.DF64):
        b, x = lat.field(src), lat.field(x0)
        st = lat.solve(b, x, wd.solver_params(kind=wd.CGNR_REF, mass=0.1, tol=1e-9, max_iter=1000, prec=prec))
        res[prec] = (st.iterations, x.download())
    assert abs(res[wd.F64][0] - res[wd.DF64][0]) <= 1
    assert rel_l2(res[wd.DF64][1], res[wd.F64][1]) < 1e-9


@pytest.mark.parametrize("inner", [2, 3])
@pytest.mark.parametrize("reliable", [0, 1])
@pytest.mark.parametrize("mass", [0.1, 0.01])
def test_mixed_cg(wd, oracle, solve_case, inner, reliable, mass):
    dims, gauge, src, lat, sols = solve_case
    b, x = lat.field(src), lat.field()
    st = lat.solve(b, x, wd.solver_params(kind=wd.CG_EO, mass=mass, tol=1e-10, max_iter=4000, prec=inner,
                                          prec_reliable=reliable))
    assert st.reliable_updates >= 1
    _check_solution(wd, oracle, dims, gauge, src, x.download(), mass, sols[mass], st)
