"""CG on the GPU: the reference algorithm step for step against the oracle,
and the even-odd solver checked by its FP64 true residual and its error
against the oracle's solution."""
import numpy as np
import pytest

from oracle import rel_l2

pytestmark = pytest.mark.gpu


def test_cgnr_ref_matches_reference_golden(wd, ctx, oracle, golden4):
    """CGinvert as main.cpp calls it: same iteration count, same solution."""
    g = golden4
    x0 = oracle.rand_guess(g["src"].size, int(g["cg_seed"]))
    p = wd.solver_params(kind=wd.CGNR_REF, mass=g["mass"], tol=float(g["cg_acc"]), max_iter=int(g["cg_max"]))
    x = x0.copy()
    st = ctx.host_cg(g["dims"], g["gauge"], g["src"], x, p)
    assert st.iterations == int(g["cg_iters"])
    assert abs(st.residual - float(g["cg_rsd"])) < 1e-3 * float(g["cg_rsd"])
    assert rel_l2(x, g["cg_x"]) < 1e-10


def test_cgnr_ref_vs_oracle_8c16(wd, ctx, oracle):
    dims = (8, 8, 8, 16)
    gauge = wd.gen_gauge(dims, seed=1)
    src = wd.gen_source(dims, seed=1)
    x0 = oracle.rand_guess(src.size, 1)
    xo, it_o, rsd_o = oracle.cg_ref(src, gauge, dims, 0.1, 1000, 1e-9, x0)
    x = x0.copy()
    st = ctx.host_cg(dims, gauge, src, x, wd.solver_params(kind=wd.CGNR_REF, mass=0.1, tol=1e-9, max_iter=1000))
    assert abs(st.iterations - it_o) <= 1
    assert rel_l2(x, xo) < 1e-9


@pytest.mark.parametrize("mass", [0.1, 0.01])
def test_cg_eo_true_residual_and_error(wd, ctx, oracle, mass):
    dims = (8, 8, 8, 16)
    gauge = wd.gen_gauge(dims, seed=1)
    src = wd.gen_source(dims, seed=1)
    # oracle solution to 1e-13 relative (reference CG, absolute stop scaled by |b| = 1)
    xo, _, _ = oracle.cg_ref(src, gauge, dims, mass, 5000, 1e-13, np.zeros_like(src))
    x = np.zeros_like(src)
    st = ctx.host_cg(dims, gauge, src, x, wd.solver_params(kind=wd.CG_EO, mass=mass, tol=1e-10, max_iter=2000))
    assert st.converged
    assert st.true_residual <= 1e-10
    # independent FP64 residual from the oracle
    r = src - oracle.dslash_full(x, gauge, dims, mass, 0)
    assert np.linalg.norm(r) / np.linalg.norm(src) <= 1.05e-10
    assert rel_l2(x, xo) < 1e-9


def test_check_report_matches_oracle(wd, ctx, oracle, golden4):
    g = golden4
    lat = ctx.lattice(g["dims"], g["gauge"])
    out = lat.check(lat.field(g["src"]), lat.field(g["cg_x"]), g["mass"])
    ref = oracle.check(g["src"], g["cg_x"], g["gauge"], g["dims"], g["mass"])
    for i in (0, 1, 2, 4, 6, 8):
        assert abs(out[i] - ref[i]) <= 1e-12 * abs(ref[i])
    for i in (10, 11):
        assert abs(out[i] - ref[i]) <= 1e-4 * ref[i] + 1e-15


def test_not_converged_is_reported(wd, ctx):
    dims = (4, 4, 4, 4)
    gauge = wd.gen_gauge(dims, seed=4)
    src = wd.gen_source(dims, seed=4)
    x = np.zeros_like(src)
    st = ctx.host_cg(dims, gauge, src, x, wd.solver_params(kind=wd.CG_EO, mass=0.1, tol=1e-12, max_iter=3),
                     allow_unconverged=True)
    assert not st.converged and st.iterations == 3
    with pytest.raises(wd.WilsonError) as e:
        ctx.host_cg(dims, gauge, src, np.zeros_like(src),
                    wd.solver_params(kind=wd.CG_EO, mass=0.1, tol=1e-12, max_iter=3))
    assert e.value.status == wd.NOT_CONVERGED


def test_cgnr_ref_matches_reference_digest_8c16(wd, ctx, oracle, digest8):
    """CGinvert at 8^3x16 (m = 0.1, srand(7) initial guess, 1e-10) against the
    reference's own iteration count, residual and solution digest."""
    from conftest import digest_error
    d = digest8
    x = oracle.rand_guess(d["src"].size, int(d["cg_seed"]))
    p = wd.solver_params(kind=wd.CGNR_REF, mass=d["mass"], tol=float(d["cg_acc"]), max_iter=int(d["cg_max"]))
    st = ctx.host_cg(d["dims"], d["gauge"], d["src"], x, p)
    assert abs(st.iterations - int(d["cg_iters"])) <= 1
    assert abs(st.residual - float(d["cg_rsd"])) < 0.05 * float(d["cg_rsd"])
    assert digest_error(d, "cg_x", x) < 1e-9
