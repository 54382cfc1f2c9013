"""The oracle against the reference's own sources (oracle/_ref/libref.so,
compiled single-rank from the reference tree where it is present on x86-64)
on extra lattice shapes: extents of 2 (forward and backward neighbour
coincide), odd Lx/2, long and short directions.  Skipped where the reference
build is absent (the Arm GPU host)."""
import numpy as np
import pytest

from oracle import REF_LIB, rel_l2

pytestmark = pytest.mark.skipif(not REF_LIB.exists(), reason="reference build absent")

SHAPES = [(2, 2, 2, 2), (4, 2, 4, 6), (6, 6, 2, 2), (10, 2, 2, 4), (8, 4, 2, 4)]


@pytest.fixture(scope="module")
def ref():
    from oracle import Reference
    return Reference()


@pytest.mark.parametrize("dims", SHAPES)
def test_operators_match_reference(wd, oracle, ref, dims):
    gauge = wd.gen_gauge(dims, seed=17, eps=0.5)
    src = wd.gen_source(dims, seed=18)
    for dag in (0, 1):
        for cb in (0, 1):
            assert rel_l2(oracle.dslash_offd(src, gauge, dims, dag, cb),
                          ref.dslashoffd_new(src, gauge, dims, dag, cb)) < 1e-14
        full = oracle.dslash_full(src, gauge, dims, 0.07, dag)
        assert rel_l2(full, ref.dslash_new(src, gauge, dims, 0.07, dag)) < 1e-14
        assert rel_l2(full, ref.dslash_old(src, gauge, dims, 0.07, dag)) < 1e-14
    assert rel_l2(oracle.dslash_eeoo(src, dims, 0.07), ref.dslash_eeoo_new(src, dims, 0.07)) == 0.0


@pytest.mark.parametrize("dims", SHAPES[1:4])
def test_cg_matches_reference(wd, oracle, ref, dims):
    gauge = wd.gen_gauge(dims, seed=19, eps=0.5)
    src = wd.gen_source(dims, seed=20)
    x_ref, it_ref, rsd_ref = ref.cginvert(src, gauge, dims, 0.2, 500, 1e-11, 3)
    x, it, rsd = oracle.cg_ref(src, gauge, dims, 0.2, 500, 1e-11, oracle.rand_guess(src.size, 3))
    assert it == it_ref
    assert abs(rsd - rsd_ref) < 1e-3 * rsd_ref
    assert rel_l2(x, x_ref) < 1e-11
