"""Solves at the benchmark sizes against the oracle, on the benchmark's seeded
inputs (SU(3) links exp(i 0.5 H), unit Gaussian source):

* 32^3x64, seed 2, masses 0.05 and 0.01: every solver plan the benchmark
  times (FP64, double-float, mixed FP32 / FP16 inner with FP64 or
  double-float reliable updates) must reach FP64 true residual 1e-10 on the
  device, 1.05e-10 when the oracle recomputes |b - Mx|/|b| from the
  downloaded solution, and lie within 1e-9 relative of the oracle's even-odd
  solution driven to 1e-14;
* 32^3x64, mass 0.05: the reference's CG recurrences (CGinvert,
  src/invert.cpp:25-121) from the reference's rand() initial guess take the
  oracle's iteration count (+-1) and reach its solution to 1e-9;
* 48^3x96, seed 2, mass 0.01: the mixed plans, same bars;
* 24^3x48, seed 3, mass 0.05: 12 point + 12 Gaussian sources in one batched
  solve, each within 1e-9 of the oracle.

The oracle runs on all host cores (seconds to tens of seconds per solve at
these volumes)."""
import numpy as np
import pytest

from oracle import rel_l2

pytestmark = pytest.mark.gpu

PLANS = {"f64": (0, 0), "df64": (1, 0), "mixed_f32": (2, 0), "mixed_f16": (3, 0), "mixed_f16_df64": (3, 1)}


class Case:
    def __init__(self, wd, ctx, oracle, dims, seed):
        self.wd, self.oracle, self.dims = wd, oracle, dims
        self.gauge = wd.gen_gauge(dims, seed, 0.5)
        self.src = wd.gen_source(dims, seed)
        self.lat = ctx.lattice(dims, self.gauge)
        self.b = self.lat.field(self.src)
        self._sol = {}

    def oracle_solution(self, mass):
        if mass not in self._sol:
            x, it, res = self.oracle.cg_eo(self.src, self.gauge, self.dims, mass, tol=1e-14)
            assert res < 1e-12, (it, res)
            self._sol[mass] = x
        return self._sol[mass]

    def solve_and_check(self, plan, mass):
        wd = self.wd
        prec, rel = PLANS[plan]
        x = self.lat.field()
        st = self.lat.solve(self.b, x, wd.solver_params(kind=wd.CG_EO, mass=mass, tol=1e-10, max_iter=5000,
                                                        prec=prec, prec_reliable=rel))
        assert st.converged and st.true_residual <= 1e-10, st.as_dict()
        sol = x.download()
        x.close()
        r = self.src - self.oracle.dslash_full(sol, self.gauge, self.dims, mass, 0)
        assert np.linalg.norm(r) / np.linalg.norm(self.src) <= 1.05e-10
        err = rel_l2(sol, self.oracle_solution(mass))
        assert err < 1e-9, (plan, mass, err)
        return st

    def close(self):
        self.b.close()
        self.lat.close()


@pytest.fixture(scope="module")
def case32(wd, ctx, oracle):
    c = Case(wd, ctx, oracle, (32, 32, 32, 64), 2)
    yield c
    c.close()


@pytest.mark.parametrize("mass", [0.05, 0.01])
@pytest.mark.parametrize("plan", list(PLANS))
def test_solver_plans_32c64_against_oracle(case32, plan, mass):
    case32.solve_and_check(plan, mass)


def test_cginvert_recurrences_32c64_against_oracle(wd, case32, oracle):
    """WD_SOLVER_CGNR_REF: full-lattice normal equations, complex alpha and
    beta, absolute stop on |r_normal| < 1e-10, from the srand(7) guess."""
    c = case32
    x0 = oracle.rand_guess(c.src.size, 7)
    xo, it_o, rsd_o = oracle.cg_ref(c.src, c.gauge, c.dims, 0.05, 1000, 1e-10, x0)
    assert rsd_o < 1e-10
    x = c.lat.field(x0)
    st = c.lat.solve(c.b, x, wd.solver_params(kind=wd.CGNR_REF, mass=0.05, tol=1e-10, max_iter=1000))
    assert st.converged
    assert abs(st.iterations - it_o) <= 1, (st.iterations, it_o)
    assert rel_l2(x.download(), xo) < 1e-9
    x.close()


@pytest.fixture(scope="module")
def case48(wd, ctx, oracle, case32):
    case32.close()   # make room: one benchmark lattice resident at a time
    c = Case(wd, ctx, oracle, (48, 48, 48, 96), 2)
    yield c
    c.close()


@pytest.mark.parametrize("plan", ["mixed_f32", "mixed_f16", "mixed_f16_df64"])
def test_mixed_plans_48c96_against_oracle(case48, plan):
    case48.solve_and_check(plan, 0.01)


def test_batched_24c48_point_and_gaussian_sources_against_oracle(wd, ctx, oracle):
    dims, mass = (24, 24, 24, 48), 0.05
    V = int(np.prod(dims))
    gauge = wd.gen_gauge(dims, 3, 0.5)
    lat = ctx.lattice(dims, gauge)
    srcs = []
    for s in range(4):
        for col in range(3):
            b = np.zeros(V * 12, np.complex128)
            b[s * 3 + col] = 1.0          # site (0,0,0,0), even-odd index 0
            srcs.append(b)
    srcs += [wd.gen_source(dims, 1000 + k) for k in range(12)]
    systems = [(lat, lat.field(b), lat.field(), mass) for b in srcs]
    stats = ctx.solve_batch(systems, wd.solver_params(kind=wd.CG_EO, tol=1e-10, max_iter=5000, prec=wd.F32,
                                                      prec_reliable=wd.DF64))
    for (_, fb, fx, _), b, st in zip(systems, srcs, stats):
        assert st.converged and st.true_residual <= 1e-10, st.as_dict()
        x = fx.download()
        r = b - oracle.dslash_full(x, gauge, dims, mass, 0)
        assert np.linalg.norm(r) / np.linalg.norm(b) <= 1.05e-10
        xo, _, res = oracle.cg_eo(b, gauge, dims, mass, tol=1e-14)
        assert res < 1e-12
        assert rel_l2(x, xo) < 1e-9
        fb.close()
        fx.close()
    lat.close()
