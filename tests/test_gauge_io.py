"""Gauge-configuration files (host only, no GPU): the reference's load_gauge
format, NERSC (3x3 and two-row, double and single, big and little endian)
and ILDG (double and single), written here from seeded links and read back
into the reference layout."""
import numpy as np
import pytest

DIMS = (4, 2, 2, 4)


@pytest.fixture(scope="module")
def links(wd):
    """Seeded links in the reference layout and as [lex site][mu][3][3]."""
    g = wd.gen_gauge(DIMS, seed=13)
    V = int(np.prod(DIMS))
    lex = np.arange(V)
    x = lex % DIMS[0]
    y = (lex // DIMS[0]) % DIMS[1]
    z = (lex // (DIMS[0] * DIMS[1])) % DIMS[2]
    t = lex // (DIMS[0] * DIMS[1] * DIMS[2])
    eo = lex // 2 + ((x + y + z + t) & 1) * (V // 2)
    U = np.stack([g[mu].reshape(V, 3, 3)[eo] for mu in range(4)], axis=1)
    return g, U


def _pairs(U, rows):
    u = U[:, :, :rows, :]
    return np.stack([u.real, u.imag], axis=-1).reshape(-1)


def _header(kv):
    lines = ["BEGIN_HEADER"] + [f"{k} = {v}" for k, v in kv.items()] + ["END_HEADER"]
    return ("\n".join(lines) + "\n").encode()


def _check(wd, path, want, fmt, found_want, tol):
    got, found = wd.read_gauge_file(str(path), DIMS, fmt)
    assert found == found_want
    for mu in range(4):
        assert np.max(np.abs(got[mu] - want[mu])) <= tol, (path, mu)


def test_reference_format_plain_and_lime(wd, links, tmp_path):
    g, U = links
    payload = _pairs(U, 3).astype(">f8").tobytes()
    (tmp_path / "plain").write_bytes(payload)
    (tmp_path / "lime").write_bytes(b"\x45\x67\x89\xab" * 40 + payload + b"\0" * 280)
    for name in ("plain", "lime"):
        _check(wd, tmp_path / name, g, wd.GAUGE_FILE_AUTO, wd.GAUGE_FILE_REF, 0.0)
        _check(wd, tmp_path / name, g, wd.GAUGE_FILE_REF, wd.GAUGE_FILE_REF, 0.0)


@pytest.mark.parametrize("rows,fp,dtype,tol", [(3, "IEEE64BIG", ">f8", 0.0), (2, "IEEE64BIG", ">f8", 1e-14),
                                               (2, "IEEE64LITTLE", "<f8", 1e-14), (3, "IEEE32BIG", ">f4", 1e-6),
                                               (2, "IEEE32LITTLE", "<f4", 1e-6)])
def test_nersc(wd, links, tmp_path, rows, fp, dtype, tol):
    g, U = links
    kv = {"HDR_VERSION": "1.0", "DATATYPE": "4D_SU3_GAUGE_3x3" if rows == 3 else "4D_SU3_GAUGE",
          "FLOATING_POINT": fp}
    kv.update({f"DIMENSION_{i + 1}": d for i, d in enumerate(DIMS)})
    p = tmp_path / "cfg.nersc"
    p.write_bytes(_header(kv) + _pairs(U, rows).astype(dtype).tobytes())
    _check(wd, p, g, wd.GAUGE_FILE_AUTO, wd.GAUGE_FILE_NERSC, tol)


def test_nersc_dimension_mismatch(wd, links, tmp_path):
    g, U = links
    kv = {"DATATYPE": "4D_SU3_GAUGE_3x3", "DIMENSION_1": 8, "DIMENSION_2": 2, "DIMENSION_3": 2,
          "DIMENSION_4": 4, "FLOATING_POINT": "IEEE64BIG"}
    p = tmp_path / "bad.nersc"
    p.write_bytes(_header(kv) + _pairs(U, 3).astype(">f8").tobytes())
    with pytest.raises(wd.WilsonError) as e:
        wd.read_gauge_file(str(p), DIMS)
    assert e.value.status == wd.BAD_DIMS


@pytest.mark.parametrize("dtype,tol", [(">f8", 0.0), (">f4", 1e-6)])
def test_ildg(wd, links, tmp_path, dtype, tol):
    g, U = links
    p = tmp_path / "cfg.ildg"
    p.write_bytes(b"LIME-record-headers-and-xml" * 7 + _pairs(U, 3).astype(dtype).tobytes())
    _check(wd, p, g, wd.GAUGE_FILE_ILDG, wd.GAUGE_FILE_ILDG, tol)
    if dtype == ">f4":  # single precision is what AUTO takes for a file too small for doubles
        _check(wd, p, g, wd.GAUGE_FILE_AUTO, wd.GAUGE_FILE_ILDG, tol)


def test_missing_or_short_file(wd, tmp_path):
    with pytest.raises(wd.WilsonError) as e:
        wd.read_gauge_file(str(tmp_path / "nope"), DIMS)
    assert e.value.status == wd.BAD_ARG
    (tmp_path / "short").write_bytes(b"\0" * 100)
    with pytest.raises(wd.WilsonError) as e:
        wd.read_gauge_file(str(tmp_path / "short"), DIMS)
    assert e.value.status == wd.BAD_DIMS
