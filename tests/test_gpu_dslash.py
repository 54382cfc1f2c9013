"""FP64 Dslash on the GPU against the CPU oracle (and the reference's golden
vectors).  Bar: relative L2 error <= 1e-13."""
import numpy as np
import pytest

from oracle import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-13


def test_golden_offd_and_full(wd, ctx, golden4, golden6):
    for g in (golden4, golden6):
        lat = ctx.lattice(g["dims"], g["gauge"])
        src = lat.field(g["src"])
        out = lat.field()
        for k in g:
            if k.startswith("offd_new"):
                dag, cb = int(k[12]), int(k[-1])
                lat.dslash_offd(src, out, dag, cb)
                assert rel_l2(out.download(), g[k]) < TOL, k
            elif k.startswith("full_"):
                lat.dslash_full(src, out, g["mass"], int(k[-1]))
                assert rel_l2(out.download(), g[k]) < TOL, k
        if "eeoo_new" in g:
            lat.dslash_eeoo(src, out, g["mass"])
            assert rel_l2(out.download(), g["eeoo_new"]) < TOL


@pytest.mark.parametrize("dims", [(8, 8, 8, 16), (4, 6, 2, 10), (2, 2, 2, 2), (12, 4, 6, 8)])
def test_generated_lattices_vs_oracle(wd, ctx, oracle, dims):
    gauge = wd.gen_gauge(dims, seed=1, eps=0.5)
    src = wd.gen_source(dims, seed=1)
    lat = ctx.lattice(dims, gauge)
    fs, fo = lat.field(src), lat.field()
    for dag in (0, 1):
        for cb in (0, 1):
            lat.dslash_offd(fs, fo, dag, cb)
            assert rel_l2(fo.download(), oracle.dslash_offd(src, gauge, dims, dag, cb)) < TOL
        lat.dslash_full(fs, fo, 0.1, dag)
        assert rel_l2(fo.download(), oracle.dslash_full(src, gauge, dims, 0.1, dag)) < TOL


def test_host_buffer_entry_points(wd, ctx, oracle, golden4):
    g = golden4
    out = ctx.host_dslash_offd(g["dims"], g["gauge"], g["src"], 1, 0)
    assert rel_l2(out, g["offd_new_dag1_cb0"]) < TOL
    out = ctx.host_dslash_full(g["dims"], g["gauge"], g["src"], g["mass"], 0)
    assert rel_l2(out, g["full_new_dag0"]) < TOL


def test_reductions(wd, ctx, golden4):
    g = golden4
    lat = ctx.lattice(g["dims"], g["gauge"])
    a = lat.field(g["src"])
    b = lat.field(g["full_new_dag0"])
    assert abs(a.norm2() - np.vdot(g["src"], g["src"]).real) < 1e-14
    d = a.dot(b)
    ref = np.vdot(g["src"], g["full_new_dag0"])
    assert abs(d - ref) < 1e-13 * abs(ref)
    # deterministic: same bits on repeat
    assert a.dot(b) == d


def test_upload_download_roundtrip(wd, ctx):
    dims = (6, 4, 4, 2)
    gauge = wd.gen_gauge(dims, seed=2)
    src = wd.gen_source(dims, seed=2)
    lat = ctx.lattice(dims, gauge)
    assert np.array_equal(lat.field(src).download(), src)


def test_bad_dims_and_mismatch(wd, ctx):
    g = [np.zeros(9 * 3 * 2 * 2 * 2, np.complex128) for _ in range(4)]
    with pytest.raises(wd.WilsonError) as e:
        ctx.lattice((3, 2, 2, 2), g)
    assert e.value.status == wd.BAD_DIMS
    dims_a, dims_b = (4, 2, 2, 2), (4, 2, 2, 4)
    la = ctx.lattice(dims_a, wd.gen_gauge(dims_a, 1))
    lb = ctx.lattice(dims_b, wd.gen_gauge(dims_b, 1))
    with pytest.raises(wd.WilsonError) as e:
        la.dslash_full(la.field(), lb.field(), 0.1, 0)
    assert e.value.status == wd.BAD_ARG


@pytest.mark.parametrize("dims,dag,cb", [((16, 16, 16, 16), 0, 0), ((24, 24, 24, 32), 1, 1),
                                         ((32, 32, 32, 32), 0, 1), ((32, 32, 32, 64), 1, 0)])
def test_host_offd_pipelined_large(wd, ctx, oracle, dims, dag, cb):
    """The host-buffer DslashoffdNew in one piece (16^4) and as overlapped
    time-slab chunks (3 chunks at 24^3x32, 8 at 32^4, 16 chunks and 32 upload
    units at 32^3x64); the untouched parity of dest must come back zero
    whatever it held before."""
    gauge = wd.gen_gauge(dims, seed=5)
    src = wd.gen_source(dims, seed=5)
    out = np.full_like(src, np.nan + 1j)
    from wilson_gb300 import _dims, _gauge_ptrs, _ptr, lib
    ctx.check(lib.wd_host_dslash_offd(ctx.handle, _dims(dims), _gauge_ptrs(gauge), _ptr(src), _ptr(out), dag, cb))
    ref = oracle.dslash_offd(src, gauge, dims, dag, cb)
    assert rel_l2(out, ref) < TOL
    half = src.size // 2
    assert np.all(out[(1 - cb) * half:(2 - cb) * half] == 0)


def test_volume_beyond_32bit_byte_offsets(wd, ctx, oracle):
    """32x32x32x128 (4.2M sites): the FP64 links (2.4 GB) and their double-float
    copy lie beyond 2^31 bytes, so every plane offset must be computed in 64
    bits.  Hopping terms in every storage against the oracle (bars: 1e-13 for
    FP64 and double-float, 2e-6 FP32, 5e-3 FP16), both parities and dagger."""
    dims = (32, 32, 32, 128)
    gauge = wd.gen_gauge(dims, seed=9)
    src = wd.gen_source(dims, seed=9)
    lat = ctx.lattice(dims, gauge)
    want = {(dag, cb): oracle.dslash_offd(src, gauge, dims, dag, cb) for dag, cb in ((0, 0), (1, 1))}
    for prec, bar in ((wd.F64, TOL), (wd.DF64, TOL), (wd.F32, 2e-6), (wd.F16, 5e-3)):
        fi, fo = lat.field(src, prec=prec), lat.field(prec=prec)
        for (dag, cb), ref in want.items():
            lat.dslash_offd(fi, fo, dag, cb, prec)
            assert rel_l2(fo.download(), ref) < bar, (prec, dag, cb)
        fi.close()
        fo.close()
    lat.close()


@pytest.mark.parametrize("dims,dag", [((16, 16, 16, 16), 0), ((24, 24, 24, 32), 1), ((32, 32, 32, 64), 0)])
def test_host_full_pipelined(wd, ctx, oracle, dims, dag):
    """The host-buffer DslashNew (both parities up and back) in one piece and
    as overlapped time-slab chunks, against the oracle."""
    gauge = wd.gen_gauge(dims, seed=6)
    src = wd.gen_source(dims, seed=6)
    out = np.full_like(src, np.nan + 1j)
    from wilson_gb300 import _dims, _gauge_ptrs, _ptr, lib
    ctx.check(lib.wd_host_dslash_full(ctx.handle, _dims(dims), _gauge_ptrs(gauge), _ptr(src), _ptr(out), 0.07, dag))
    assert rel_l2(out, oracle.dslash_full(src, gauge, dims, 0.07, dag)) < TOL


def test_host_paths_pinned_and_pageable_buffers(wd, ctx, oracle):
    """Pinned host buffers go through the copy engines, pageable ones
    through kernels that address host memory directly: both give the
    oracle's result (DslashoffdNew and DslashNew, 24^3x32, chunked)."""
    torch = pytest.importorskip("torch")
    dims = (24, 24, 24, 32)
    gauge = wd.gen_gauge(dims, seed=8)
    src = wd.gen_source(dims, seed=8)
    from wilson_gb300 import _dims, _gauge_ptrs, _ptr, lib
    want_offd = oracle.dslash_offd(src, gauge, dims, 1, 0)
    want_full = oracle.dslash_full(src, gauge, dims, 0.2, 0)
    pinned_src = torch.from_numpy(src).pin_memory().numpy()
    pinned_out = torch.empty(src.size, dtype=torch.complex128).pin_memory().numpy()
    for s, o in ((pinned_src, pinned_out), (src.copy(), np.empty_like(src))):
        o[:] = np.nan
        ctx.check(lib.wd_host_dslash_offd(ctx.handle, _dims(dims), _gauge_ptrs(gauge), _ptr(s), _ptr(o), 1, 0))
        assert rel_l2(o, want_offd) < TOL
        ctx.check(lib.wd_host_dslash_full(ctx.handle, _dims(dims), _gauge_ptrs(gauge), _ptr(s), _ptr(o), 0.2, 0))
        assert rel_l2(o, want_full) < TOL


def test_reference_digests_8c16(wd, ctx, digest8):
    """8^3x16, m = 0.1, seed 1 against the reference's own outputs (digests):
    host-buffer entry points and the resident lattice."""
    from conftest import digest_error
    d = digest8
    g, src, dims, m = d["gauge"], d["src"], d["dims"], d["mass"]
    lat = ctx.lattice(dims, g)
    fs, fo = lat.field(src), lat.field()
    for dag in (0, 1):
        for cb in (0, 1):
            name = f"offd_new_dag{dag}_cb{cb}"
            assert digest_error(d, name, ctx.host_dslash_offd(dims, g, src, dag, cb)) < TOL, name
            lat.dslash_offd(fs, fo, dag, cb)
            assert digest_error(d, name, fo.download()) < TOL, name
        name = f"full_new_dag{dag}"
        assert digest_error(d, name, ctx.host_dslash_full(dims, g, src, m, dag)) < TOL, name
        lat.dslash_full(fs, fo, m, dag)
        assert digest_error(d, name, fo.download()) < TOL, name
