"""Point-source propagator (12 right-hand sides solved as one batch) and the
pion two-point function, against the oracle: each column within 1e-9 of the
oracle's solution, C(t) within 1e-9 relative."""
import numpy as np
import pytest

from oracle import rel_l2

pytestmark = pytest.mark.gpu


def oracle_ct(cols, dims):
    Lx, Ly, Lz, Lt = dims
    V = Lx * Ly * Lz * Lt
    ct = np.zeros(Lt)
    dens = sum(np.abs(c.reshape(V, 12)) ** 2 for c in cols).sum(axis=1)
    # site order: even-odd blocks of lexicographic order; t of eo index e
    for par in range(2):
        for s in range(V // 2):
            t = (s // (Lx // 2)) // (Ly * Lz)
            ct[t] += dens[par * (V // 2) + s]
    return ct


@pytest.mark.parametrize("prec", [2, 1])
def test_propagator_and_pion(wd, ctx, oracle, prec):
    dims, mass, x0 = (4, 4, 4, 8), 0.1, (1, 2, 0, 3)
    gauge = wd.gen_gauge(dims, seed=9)
    lat = ctx.lattice(dims, gauge)
    props, stats = lat.propagator(x0, wd.solver_params(kind=wd.CG_EO, mass=mass, tol=1e-10, max_iter=4000,
                                                        prec=prec, prec_reliable=wd.DF64))
    V = int(np.prod(dims))
    Lx, Ly, Lz, Lt = dims
    e0 = (x0[0] + Lx * (x0[1] + Ly * (x0[2] + Lz * x0[3]))) // 2 + (sum(x0) & 1) * (V // 2)
    cols = []
    for k, (f, st) in enumerate(zip(props, stats)):
        assert st.converged and st.true_residual <= 1e-10
        b = np.zeros(V * 12, np.complex128)
        b[e0 * 12 + k] = 1.0
        xo, _, _ = oracle.cg_ref(b, gauge, dims, mass, 5000, 1e-13, np.zeros_like(b))
        x = f.download()
        assert rel_l2(x, xo) < 1e-9
        cols.append(xo)
    ct = lat.pion_correlator(props)
    ref = oracle_ct(cols, dims)
    assert rel_l2(ct, ref) < 1e-9
    assert np.all(ct > 0) and np.argmax(ct) == x0[3]   # peaked on the source time slice
