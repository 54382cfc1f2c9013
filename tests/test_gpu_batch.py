"""Batched solves: many right-hand sides on one lattice, and lattices of
uneven volume, in one batched launch per operator application with CUDA-graph
iterations and per-system convergence masking.  Every system must reach FP64
true residual <= 1e-10, agree with the oracle's solution to 1e-9, and give the
same answer as when it is solved alone (to 1e-9 relative)."""
import numpy as np
import pytest

from oracle import rel_l2

pytestmark = pytest.mark.gpu


def point_source(V, spin, colour):
    b = np.zeros(V * 12, np.complex128)
    b[spin * 3 + colour] = 1.0      # site (0,0,0,0): even-odd index 0
    return b


def solve_alone(wd, lat, src, mass, prec, rel):
    b, x = lat.field(src), lat.field()
    lat.solve(b, x, wd.solver_params(kind=wd.CG_EO, mass=mass, tol=1e-10, max_iter=4000, prec=prec,
                                     prec_reliable=rel))
    return x.download()


@pytest.mark.parametrize("prec,rel", [(2, 0), (3, 1)])
def test_multi_rhs_one_lattice(wd, ctx, oracle, prec, rel):
    dims, mass = (8, 4, 4, 8), 0.05
    V = int(np.prod(dims))
    gauge = wd.gen_gauge(dims, seed=3)
    lat = ctx.lattice(dims, gauge)
    srcs = [point_source(V, s, c) for s, c in ((0, 0), (1, 2), (3, 1))]
    srcs += [wd.gen_source(dims, seed=100 + k) for k in range(3)]
    fields = [(lat, lat.field(b), lat.field(), mass) for b in srcs]
    stats = ctx.solve_batch(fields, wd.solver_params(kind=wd.CG_EO, mass=mass, tol=1e-10, max_iter=4000, prec=prec,
                                                     prec_reliable=rel))
    for (l, fb, fx, m), b, st in zip(fields, srcs, stats):
        assert st.converged and st.true_residual <= 1e-10, st.as_dict()
        x = fx.download()
        xo, _, _ = oracle.cg_ref(b, gauge, dims, mass, 5000, 1e-13 * np.linalg.norm(b), np.zeros_like(b))
        assert rel_l2(x, xo) < 1e-9
        assert rel_l2(x, solve_alone(wd, lat, b, mass, prec, rel)) < 1e-9


def test_uneven_lattices_and_masking(wd, ctx, oracle):
    # a heavy system (mass 2: a few iterations) next to light ones: it is
    # masked off while the others keep iterating
    cases = [((4, 4, 4, 8), 2.0), ((8, 8, 8, 16), 0.02), ((6, 4, 4, 8), 0.12), ((4, 4, 4, 4), 0.5),
             ((8, 4, 4, 8), 0.15)]
    systems, refs = [], []
    for k, (dims, mass) in enumerate(cases):
        gauge = wd.gen_gauge(dims, seed=10 + k)
        src = wd.gen_source(dims, seed=20 + k)
        lat = ctx.lattice(dims, gauge)
        systems.append((lat, lat.field(src), lat.field(), mass))
        refs.append((dims, gauge, src, mass))
    stats = ctx.solve_batch(systems, wd.solver_params(kind=wd.CG_EO, tol=1e-10, max_iter=4000, prec=wd.F32))
    iters = set()
    for (lat, fb, fx, mass), (dims, gauge, src, _), st in zip(systems, refs, stats):
        assert st.converged and st.true_residual <= 1e-10, st.as_dict()
        iters.add(st.iterations)
        x = fx.download()
        xo, _, _ = oracle.cg_ref(src, gauge, dims, mass, 5000, 1e-13, np.zeros_like(src))
        assert rel_l2(x, xo) < 1e-9
        assert rel_l2(x, solve_alone(wd, lat, src, mass, wd.F32, wd.F64)) < 1e-9
    assert len(iters) > 1   # systems converged at different iterations: masking kept them apart


def test_batch_rejects_fp64_inner(wd, ctx):
    dims = (4, 4, 4, 4)
    lat = ctx.lattice(dims, wd.gen_gauge(dims, 1))
    with pytest.raises(wd.WilsonError) as e:
        ctx.solve_batch([(lat, lat.field(wd.gen_source(dims, 1)), lat.field(), 0.1)],
                        wd.solver_params(kind=wd.CG_EO, prec=wd.F64))
    assert e.value.status == wd.BAD_ARG


@pytest.mark.parametrize("prec,kernel", [(2, "batch_hop_f32"), (3, "batch_hop_f16")])
def test_batch_hop_variants_bit_identical(wd, ctx, prec, kernel):
    """Every launch variant of the batched hop (the tuner picks one per batch
    size) gives the same solutions bit for bit."""
    dims, mass = (8, 4, 4, 8), 0.05
    gauge = wd.gen_gauge(dims, seed=5)
    lat = ctx.lattice(dims, gauge)
    srcs = [wd.gen_source(dims, seed=200 + k) for k in range(6)]
    fields = [(lat, lat.field(b), lat.field(), mass) for b in srcs]
    params = wd.solver_params(kind=wd.CG_EO, mass=mass, tol=1e-10, max_iter=4000, prec=prec)
    ctx.solve_batch(fields, params)  # registers the variant count
    n = wd.tune_variants(kernel)
    assert n >= 2
    bucket = 1
    while bucket < 6 * (int(np.prod(dims)) // 2):
        bucket *= 2
    ref = None
    try:
        for v in range(n):
            wd.tune_pin(kernel, bucket, v)
            for _, _, fx, _ in fields:
                fx.zero()
            stats = ctx.solve_batch(fields, params)
            got = [fx.download() for _, _, fx, _ in fields]
            its = [st.iterations for st in stats]
            if ref is None:
                ref = (got, its)
            else:
                assert its == ref[1], f"{kernel} variant {v}"
                for a, b in zip(got, ref[0]):
                    assert np.array_equal(a, b), f"{kernel} variant {v}"
    finally:
        wd.tune_pin(kernel, bucket, -1)
