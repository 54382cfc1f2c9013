"""The TMA-staged FP16 hopping kernel (tuner variant 2 of hop_f16).

A block stages the neighbour spinors of its tile of rows and of the six
one-row faces around it with bulk tensor copies and computes every site from
shared memory.  It must give the same bits as the cp.async-staged kernel
(variant 0) on lattices that exercise each tiling
rule: one tile spanning a whole y/z extent (faces wrapping onto the tile
itself), several tiles per direction, Lxh from 4 to 32 (4 x 4 and 4 x 2
tiles), several time extents, both parities, dagger, the x epilogue of the
full operator; and the device flag of the bounded copy wait must stay
clear.  Lattices the kernel does not take (Lxh not a multiple of 4, Ly or Lz
not a multiple of the tile) fall back to variant 0."""
import numpy as np
import pytest

from oracle import rel_l2

pytestmark = pytest.mark.gpu
BAR = 5e-3

DIMS = [(8, 4, 4, 2), (8, 8, 4, 6), (16, 4, 8, 6), (32, 8, 8, 4), (24, 4, 8, 2), (48, 8, 4, 2), (64, 4, 2, 2),
        (32, 12, 8, 10)]


def _run_all(wd, ctx, lat, fi, dims, variant):
    vh = int(np.prod(dims)) // 2
    wd.tune_pin("hop_f16", vh, variant)
    outs = {}
    for dag in (0, 1):
        for cb in (0, 1):
            fo = lat.field(prec=wd.F16)
            lat.dslash_offd(fi, fo, dag, cb, wd.F16)
            outs["offd", dag, cb] = fo.download()
            fo.close()
        fo = lat.field(prec=wd.F16)
        lat.dslash_full(fi, fo, 0.13, dag, wd.F16)
        outs["full", dag] = fo.download()
        fo.close()
    ctx.device_check()
    return outs


@pytest.mark.parametrize("dims", DIMS)
def test_tma_variants_bit_identical(wd, ctx, oracle, dims):
    gauge = wd.gen_gauge(dims, seed=21)
    src = wd.gen_source(dims, seed=21)
    lat = ctx.lattice(dims, gauge)
    fi = lat.field(src, prec=wd.F16)
    vh = int(np.prod(dims)) // 2
    lat.dslash_offd(fi, lat.field(prec=wd.F16), 0, 0, wd.F16)  # registers the variant count
    assert wd.tune_variants("hop_f16") >= 3  # variant 2 is the TMA-staged kernel
    try:
        base = _run_all(wd, ctx, lat, fi, dims, 0)
        for (kind, dag, *cb), got in base.items():
            want = (oracle.dslash_offd(src, gauge, dims, dag, cb[0]) if kind == "offd"
                    else oracle.dslash_full(src, gauge, dims, 0.13, dag))
            assert rel_l2(got, want) < BAR, (kind, dag, cb)
        outs = _run_all(wd, ctx, lat, fi, dims, 2)
        for k, got in outs.items():
            assert np.array_equal(got, base[k]), (dims, k)
    finally:
        wd.tune_pin("hop_f16", vh, -1)
    fi.close()
    lat.close()


def test_tma_fallback_shapes(wd, ctx, oracle):
    """Lxh = 5 and Ly = 6: not TMA shapes, variant 2 runs variant 0's kernel."""
    dims = (10, 6, 4, 4)
    gauge = wd.gen_gauge(dims, seed=22)
    src = wd.gen_source(dims, seed=22)
    lat = ctx.lattice(dims, gauge)
    fi = lat.field(src, prec=wd.F16)
    vh = int(np.prod(dims)) // 2
    lat.dslash_offd(fi, lat.field(prec=wd.F16), 0, 0, wd.F16)
    try:
        base = _run_all(wd, ctx, lat, fi, dims, 0)
        outs = _run_all(wd, ctx, lat, fi, dims, 2)
        for k in base:
            assert np.array_equal(outs[k], base[k]), k
    finally:
        wd.tune_pin("hop_f16", vh, -1)


def test_tma_in_mixed_solver(wd, ctx, oracle):
    """The mixed FP16 solver with the TMA kernel pinned for its plain hops
    converges to the oracle's solution (16^3 x 8) and gives the same
    iterate, bit for bit, as with the cp.async kernel."""
    dims = (16, 16, 16, 8)
    gauge = wd.gen_gauge(dims, seed=23)
    src = wd.gen_source(dims, seed=23)
    lat = ctx.lattice(dims, gauge)
    vh = int(np.prod(dims)) // 2
    want, _, _ = oracle.cg_eo(src, gauge, dims, 0.05, tol=1e-12)
    sols = {}
    try:
        for v in (0, 2):
            wd.tune_pin("hop_f16", vh, v)
            b, x = lat.field(src), lat.field()
            p = wd.solver_params(kind=wd.CG_EO, mass=0.05, tol=1e-10, max_iter=5000, prec=wd.F16,
                                 prec_reliable=wd.DF64)
            lat.solve(b, x, p)
            ctx.device_check()
            sols[v] = x.download()
            assert rel_l2(sols[v], want) < 1e-8, v
            b.close()
            x.close()
        assert np.array_equal(sols[0], sols[2])
    finally:
        wd.tune_pin("hop_f16", vh, -1)
