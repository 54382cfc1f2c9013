"""Every launch variant the autotuner may pick computes the same result.

The tuner picks a launch shape per (kernel, half-volume) by timing, so which
variant runs differs between machines and runs; parity must not.  Each
variant is pinned in turn and its output compared bit for bit with variant
0's, and variant 0 against the oracle at the storage format's bar.  The
half-volume 1080 leaves a ragged last block for every block size."""
import numpy as np
import pytest

from oracle import rel_l2

pytestmark = pytest.mark.gpu

KERNELS = [(0, "hop_f64", 1e-13), (1, "hop_df64", 1e-13), (2, "hop_f32", 2e-6), (3, "hop_f16", 5e-3)]
DIMS = (10, 6, 6, 6)


@pytest.fixture(scope="module")
def case(wd, ctx):
    gauge = wd.gen_gauge(DIMS, seed=11)
    src = wd.gen_source(DIMS, seed=11)
    return gauge, src, ctx.lattice(DIMS, gauge)


@pytest.mark.parametrize("prec,kernel,bar", KERNELS)
def test_variants_bit_identical(wd, oracle, case, prec, kernel, bar):
    gauge, src, lat = case
    vh = int(np.prod(DIMS)) // 2
    fi = lat.field(src, prec=prec)
    lat.dslash_offd(fi, lat.field(prec=prec), 0, 0, prec)  # first launch registers the variant count
    n = wd.tune_variants(kernel)
    assert n >= 2
    outs = {}
    try:
        for v in range(n):
            wd.tune_pin(kernel, vh, v)
            for dag in (0, 1):
                for cb in (0, 1):
                    fo = lat.field(prec=prec)
                    lat.dslash_offd(fi, fo, dag, cb, prec)
                    got = fo.download()
                    if v == 0:
                        outs[dag, cb] = got
                        want = oracle.dslash_offd(src, gauge, DIMS, dag, cb)
                        assert rel_l2(got, want) < bar
                    else:
                        assert np.array_equal(got, outs[dag, cb]), f"{kernel} variant {v} dag {dag} cb {cb}"
        with pytest.raises(ValueError):
            wd.tune_pin(kernel, vh, n)
    finally:
        wd.tune_pin(kernel, vh, -1)


@pytest.mark.parametrize("dims", [(16, 8, 8, 8), (12, 6, 10, 4)])
def test_df64_grouped_split_in_solver(wd, oracle, ctx, dims):
    """The double-float hop's grouped colour split (variant 5: a colour per
    warp, half-spinors exchanged through shared memory) also drives the
    reliable update's fused residual kernel: the mixed FP16 solve with
    double-float reliable updates gives the same solution, bit for bit, with
    variant 5 pinned as with variant 0, and it matches the oracle.  The second
    lattice leaves a partial last group (Vh = 1440 = 22.5 x 64)."""
    gauge = wd.gen_gauge(dims, seed=12)
    src = wd.gen_source(dims, seed=12)
    lat = ctx.lattice(dims, gauge)
    vh = int(np.prod(dims)) // 2
    want, _, _ = oracle.cg_eo(src, gauge, dims, 0.05, tol=1e-12)
    sols = {}
    try:
        for v in (0, 5):
            wd.tune_pin("hop_df64", vh, v)
            b, x = lat.field(src), lat.field()
            p = wd.solver_params(kind=wd.CG_EO, mass=0.05, tol=1e-10, max_iter=5000, prec=wd.F16,
                                 prec_reliable=wd.DF64)
            st = lat.solve(b, x, p)
            assert st.reliable_updates >= 2
            sols[v] = x.download()
            assert rel_l2(sols[v], want) < 1e-8, v
            b.close()
            x.close()
        assert np.array_equal(sols[0], sols[5])
    finally:
        wd.tune_pin("hop_df64", vh, -1)
