"""The CPU oracle pinned against the reference's own outputs (golden vectors
written by tests/golden/make_golden.py from the reference sources) and
against analytic properties of the Wilson operator."""
import numpy as np
import pytest

from oracle import rel_l2


def test_offd_matches_reference(oracle, golden4):
    g = golden4
    for dag in (0, 1):
        for cb in (0, 1):
            out = oracle.dslash_offd(g["src"], g["gauge"], g["dims"], dag, cb)
            assert rel_l2(out, g[f"offd_new_dag{dag}_cb{cb}"]) < 1e-14


def test_full_matches_reference_new_and_old(oracle, golden4):
    g = golden4
    for dag in (0, 1):
        out = oracle.dslash_full(g["src"], g["gauge"], g["dims"], g["mass"], dag)
        assert rel_l2(out, g[f"full_new_dag{dag}"]) < 1e-14
    out = oracle.dslash_full(g["src"], g["gauge"], g["dims"], g["mass"], 0)
    assert rel_l2(out, g["full_old_dag0"]) < 1e-14


def test_eeoo_matches_reference(oracle, golden4):
    g = golden4
    assert rel_l2(oracle.dslash_eeoo(g["src"], g["dims"], g["mass"]), g["eeoo_new"]) == 0.0


def test_odd_half_x_and_extent_two(oracle, golden6):
    g = golden6
    for dag in (0, 1):
        out = oracle.dslash_full(g["src"], g["gauge"], g["dims"], g["mass"], dag)
        assert rel_l2(out, g[f"full_new_dag{dag}"]) < 1e-14
    out = oracle.dslash_offd(g["src"], g["gauge"], g["dims"], 0, 1)
    assert rel_l2(out, g["offd_new_dag0_cb1"]) < 1e-14


def test_cg_matches_reference(oracle, golden4):
    g = golden4
    x0 = oracle.rand_guess(g["src"].size, int(g["cg_seed"]))
    x, iters, rsd = oracle.cg_ref(g["src"], g["gauge"], g["dims"], g["mass"], int(g["cg_max"]),
                                  float(g["cg_acc"]), x0)
    assert iters == int(g["cg_iters"])
    assert abs(rsd - float(g["cg_rsd"])) < 1e-5 * float(g["cg_rsd"])
    assert rel_l2(x, g["cg_x"]) < 1e-12


def test_check_report_matches_reference(oracle, golden4):
    g = golden4
    out = oracle.check(g["src"], g["cg_x"], g["gauge"], g["dims"], g["mass"])
    ref = g["check"]
    for i in (0, 1, 2, 4, 6, 8):   # norms and real parts
        assert abs(out[i] - ref[i]) <= 1e-12 * abs(ref[i])
    for i in (3, 5, 7, 9):         # imaginary parts are rounding noise
        assert abs(out[i]) < 1e-12 and abs(ref[i]) < 1e-12
    for i in (10, 11):             # tiny residual norms
        assert abs(out[i] - ref[i]) < 1e-6 * abs(ref[i]) + 1e-15


def unit_gauge(V):
    u = np.zeros(V * 9, np.complex128)
    u[0::9] = u[4::9] = u[8::9] = 1.0
    return [u.copy() for _ in range(4)]


def test_free_field_constant_spinor(oracle):
    """Unit links, constant spinor: the hopping sum is 8 psi, so M psi = m psi."""
    dims = (4, 4, 4, 8)
    V = 4 * 4 * 4 * 8
    rng = np.random.default_rng(0)
    c = rng.normal(size=12) + 1j * rng.normal(size=12)
    psi = np.tile(c, V)
    for dag in (0, 1):
        out = oracle.dslash_full(psi, unit_gauge(V), dims, 0.3, dag)
        assert rel_l2(out, 0.3 * psi) < 1e-14


def test_adjointness_and_gamma5_hermiticity(oracle, golden4):
    g = golden4
    rng = np.random.default_rng(5)
    a = rng.normal(size=g["src"].size) + 1j * rng.normal(size=g["src"].size)
    b = g["src"]
    Mb = oracle.dslash_full(b, g["gauge"], g["dims"], g["mass"], 0)
    Mda = oracle.dslash_full(a, g["gauge"], g["dims"], g["mass"], 1)
    lhs, rhs = np.vdot(a, Mb), np.vdot(Mda, b)
    assert abs(lhs - rhs) < 1e-13 * abs(lhs)
    # gamma5 = diag(1,1,-1,-1) in this chiral basis: g5 M g5 = M^dag
    g5 = np.tile(np.repeat([1.0, 1.0, -1.0, -1.0], 3), b.size // 12)
    lhs = g5 * oracle.dslash_full(g5 * b, g["gauge"], g["dims"], g["mass"], 0)
    assert rel_l2(lhs, oracle.dslash_full(b, g["gauge"], g["dims"], g["mass"], 1)) < 1e-14


def test_gauge_covariance(oracle, golden6):
    """U_mu(x) -> W(x) U_mu(x) W(x+mu)^dag and psi -> W psi leaves |M psi| invariant."""
    g = golden6
    dims = g["dims"]
    Lx, Ly, Lz, Lt = dims
    V = Lx * Ly * Lz * Lt
    rng = np.random.default_rng(9)
    a = rng.normal(size=(V, 3, 3)) + 1j * rng.normal(size=(V, 3, 3))
    W, _ = np.linalg.qr(a)                       # random unitary per site (eo index)

    def eo(x, y, z, t):
        lex = x + Lx * (y + Ly * (z + Lz * t))
        return lex // 2 + ((x + y + z + t) & 1) * (V // 2)

    U = [u.reshape(V, 3, 3) for u in g["gauge"]]
    Un = [np.empty_like(u) for u in U]
    for t in range(Lt):
        for z in range(Lz):
            for y in range(Ly):
                for x in range(Lx):
                    e = eo(x, y, z, t)
                    c = [x, y, z, t]
                    for mu in range(4):
                        n = list(c)
                        n[mu] = (n[mu] + 1) % dims[mu]
                        Un[mu][e] = W[e] @ U[mu][e] @ W[eo(*n)].conj().T
    psi = g["src"].reshape(V, 4, 3)
    psin = np.einsum("sab,sib->sia", W, psi).reshape(-1)
    out = oracle.dslash_full(g["src"], g["gauge"], dims, 0.05, 0).reshape(V, 4, 3)
    outn = oracle.dslash_full(np.ascontiguousarray(psin), [np.ascontiguousarray(u.reshape(-1)) for u in Un],
                              dims, 0.05, 0)
    assert rel_l2(outn, np.einsum("sab,sib->sia", W, out).reshape(-1)) < 1e-13


def test_oracle_matches_reference_digests_8c16(oracle, digest8):
    """8^3x16, m = 0.1, seed 1: every entry point and CGinvert (srand(7)
    initial guess, 1e-10, 1000 iterations) against the reference's digests."""
    from conftest import digest_error
    d = digest8
    g, src, dims, m = d["gauge"], d["src"], d["dims"], d["mass"]
    for dag in (0, 1):
        for cb in (0, 1):
            assert digest_error(d, f"offd_new_dag{dag}_cb{cb}", oracle.dslash_offd(src, g, dims, dag, cb)) < 1e-14
        assert digest_error(d, f"full_new_dag{dag}", oracle.dslash_full(src, g, dims, m, dag)) < 1e-14
    assert digest_error(d, "full_old_dag1", oracle.dslash_full(src, g, dims, m, 1)) < 1e-14
    x0 = oracle.rand_guess(src.size, int(d["cg_seed"]))
    x, iters, rsd = oracle.cg_ref(src, g, dims, m, int(d["cg_max"]), float(d["cg_acc"]), x0)
    assert iters == int(d["cg_iters"])
    assert abs(rsd - float(d["cg_rsd"])) < 1e-6 * float(d["cg_rsd"])
    assert digest_error(d, "cg_x", x) < 1e-11


@pytest.mark.parametrize("which", ["golden4", "golden6"])
def test_schur_cg_agrees_with_cginvert(oracle, which, request):
    """The even-odd (Schur) CG that supplies reference solutions at large
    volumes solves the same M x = b as the reference's CGinvert: both driven
    to 1e-13 agree to 1e-12, and its recomputed true residual is tiny."""
    g = request.getfixturevalue(which)
    for mass in (g["mass"], 0.01):
        xe, it, res = oracle.cg_eo(g["src"], g["gauge"], g["dims"], mass, tol=1e-14)
        assert 0 < it < 5000 and res < 1e-12
        b = g["src"]
        r = b - oracle.dslash_full(xe, g["gauge"], g["dims"], mass, 0)
        assert np.linalg.norm(r) / np.linalg.norm(b) == pytest.approx(res, rel=1e-6, abs=1e-16)
        xr, _, _ = oracle.cg_ref(b, g["gauge"], g["dims"], mass, 5000, 1e-13 * np.linalg.norm(b),
                                 np.zeros_like(b))
        assert rel_l2(xe, xr) < 1e-12


def test_schur_cg_matches_reference_cginvert_solutions(oracle, golden4, digest8):
    """Against the reference's own CGinvert solutions: the 4^4 golden run
    (normal residual 1e-9) and the 8^3x16 digest (1e-10)."""
    from conftest import digest_error
    g = golden4
    xe, _, _ = oracle.cg_eo(g["src"], g["gauge"], g["dims"], g["mass"])
    assert rel_l2(g["cg_x"], xe) < 1e-8
    d = digest8
    xe, _, _ = oracle.cg_eo(d["src"], d["gauge"], d["dims"], d["mass"])
    assert digest_error(d, "cg_x", xe) < 1e-9


@pytest.mark.parametrize("dims,seed", [((8, 8, 8, 16), 1), ((6, 4, 2, 4), 3), ((4, 4, 4, 8), 2**62 + 5)])
def test_oracle_generator_bytes_equal_package_generator(wd, oracle, dims, seed):
    """The oracle library carries the package's input generator, so a
    CPU-only run (the reference arm of the benchmark) gets the same bytes
    without loading the CUDA library."""
    for a, b in zip(wd.gen_gauge(dims, seed, 0.5), oracle.gen_gauge(dims, seed, 0.5)):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    assert np.array_equal(wd.gen_source(dims, seed).view(np.uint64), oracle.gen_source(dims, seed).view(np.uint64))
