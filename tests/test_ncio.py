"""NetCDF classic I/O of libenkfg (host only, no GPU), checked against scipy's
independent reader and writer of the classic format (versions 1 and 2).

Files: transforms.nc (calc/transforms.c:54-131), enkf_diag.nc
(calc/transforms.c:380-470), member fields read as ncu_readfield does
(common/ncutils.c:102-530) and analysis layers written as ncu_writefield does
(common/ncutils.c:537-700).  The expected values of the attribute rules
(fill, missing, valid range, scale and offset) are restated here in numpy.
"""
import numpy as np
import pytest

scipy_io = pytest.importorskip("scipy.io")
netcdf_file = scipy_io.netcdf_file

FILL_F = np.float32(9.9692099683868690e+36)


@pytest.fixture(scope="module")
def nc():
    import build
    build.build()
    import enkfg
    return enkfg


def read_rules(raw, fill=None, missing=None, vmin=None, vmax=None, vrange=None, sf=None, ao=None,
               default_fill=None):
    """ncu_readfield's value rules on native values `raw`."""
    raw = np.asarray(raw)
    if raw.dtype == np.float64:
        with np.errstate(over="ignore"):
            v = raw.astype(np.float32)
        bad = ~np.isfinite(raw) | (np.abs(raw) > np.finfo(np.float32).max)
        v[bad] = np.nan
    else:
        v = raw.astype(np.float32)
    f = fill if fill is not None else default_fill
    mask = np.zeros(raw.shape, bool)
    if f is not None:
        mask |= raw == np.asarray(f, raw.dtype)
    if missing is not None:
        mask |= raw == np.asarray(missing, raw.dtype)
    if vmin is not None:
        mask |= raw < vmin
    if vmax is not None:
        mask |= raw > vmax
    if vrange is not None:
        mask |= (raw < vrange[0]) | (raw > vrange[1])
    v[mask] = np.nan
    if sf is not None:
        v = (v * np.float32(sf)).astype(np.float32)
    if ao is not None:
        v = (v + np.float32(ao)).astype(np.float32)
    return v


def same(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])


def test_transforms_file_read_by_scipy(nc, tmp_path):
    rng = np.random.default_rng(1)
    nj, ni, md, m = 7, 9, 5, 6
    T = rng.standard_normal((nj, ni, md, m)).astype(np.float32)
    w = rng.standard_normal((nj, ni, m)).astype(np.float32)
    p = tmp_path / "transforms.nc"
    nc.nc_write_transforms(p, T, w, stride=3, grid_name="t-grid")
    with netcdf_file(p, "r", mmap=False) as f:
        assert f.version_byte == 2
        assert f.dimensions == {"j": nj, "i": ni, "m_dyn": md, "m": m}
        assert f.variables["T"].dimensions == ("j", "i", "m_dyn", "m")
        assert f.variables["w"].dimensions == ("j", "i", "m")
        assert np.array_equal(f.variables["T"][:], T) and np.array_equal(f.variables["w"][:], w)
        assert int(f.stride) == 3 and f.grid_name == b"t-grid"
    # and through this library's own reader
    assert np.array_equal(nc.nc_get_vara_float(p, "T"), T)
    assert np.array_equal(nc.nc_get_vara_float(p, "w", [2, 3, 0], [4, 5, m]), w[2:6, 3:8])
    assert nc.nc_inq_var(p, "T") == ((nj, ni, md, m), 5, False)
    # EnOI: no T, no m_dyn
    p2 = tmp_path / "transforms-enoi.nc"
    nc.nc_write_transforms(p2, None, w, stride=1, grid_name="g")
    with netcdf_file(p2, "r", mmap=False) as f:
        assert f.dimensions == {"j": nj, "i": ni, "m": m} and "T" not in f.variables
        assert np.array_equal(f.variables["w"][:], w)


def test_diag_file_read_by_scipy(nc, tmp_path):
    rng = np.random.default_rng(2)
    nj, ni, nt = 5, 4, 3
    nlobs = rng.integers(0, 100, (nj, ni)).astype(np.int32)
    dfs = rng.random((nj, ni)).astype(np.float32)
    srf = rng.random((nj, ni)).astype(np.float32)
    pn = rng.integers(0, 50, (nt, nj, ni)).astype(np.int32)
    pd = rng.random((nt, nj, ni)).astype(np.float32)
    ps = rng.random((nt, nj, ni)).astype(np.float32)
    p = tmp_path / "enkf_diag.nc"
    nc.nc_write_diag(p, ["SST", "SLA", "TEM"], nlobs, dfs, srf, pn, pd, ps, stride=2)
    with netcdf_file(p, "r", mmap=False) as f:
        assert f.dimensions == {"nobstypes": nt, "j": nj, "i": ni}
        for name, a in (("nlobs", nlobs), ("dfs", dfs), ("srf", srf), ("pnlobs", pn), ("pdfs", pd), ("psrf", ps)):
            assert np.array_equal(f.variables[name][:], a), name
        assert f.variables["dfs"].long_name == b"local DFS (Degrees of Freedom for Signal)"
        assert int(f.stride) == 2 and int(f.SST) == 0 and int(f.SLA) == 1 and int(f.TEM) == 2


@pytest.mark.parametrize("version", [1, 2])
def test_read_layer_rules(nc, tmp_path, version):
    rng = np.random.default_rng(10 + version)
    nk, nj, ni = 4, 6, 8
    p = tmp_path / f"member_v{version}.nc"
    f3 = rng.normal(15, 2, (nk, nj, ni)).astype(np.float32)
    f3[0, 1, 2] = -999.0                                   # its _FillValue
    f3[1, 2, 3] = FILL_F                                   # the default fill: not the fill here
    d2 = rng.normal(0, 1, (nj, ni)).astype(np.float32)
    d2[3, 3] = FILL_F                                      # the default fill (no attribute)
    packed = rng.integers(-3000, 3000, (nk, nj, ni)).astype(np.int16)
    packed[2, 0, 0] = -32767                               # default short fill
    packed[2, 0, 1] = 7777                                 # missing_value
    packed[2, 0, 2] = 2999                                 # outside valid_range
    dbl = rng.normal(0, 1, (nj, ni))
    dbl[1, 1] = 1e300                                      # beyond the float range
    rec = rng.normal(0, 1, (2, nk, nj, ni)).astype(np.float32)
    with netcdf_file(p, "w", version=version) as f:
        f.createDimension("time", None)
        f.createDimension("k", nk)
        f.createDimension("j", nj)
        f.createDimension("i", ni)
        v = f.createVariable("temp", "f4", ("k", "j", "i"))
        v[:] = f3
        v._FillValue = np.float32(-999.0)
        v = f.createVariable("eta", "f4", ("j", "i"))
        v[:] = d2
        v = f.createVariable("salt", "i2", ("k", "j", "i"))
        v[:] = packed
        v.scale_factor = np.float32(0.01)
        v.add_offset = np.float32(35.0)
        v.missing_value = np.int16(7777)
        v.valid_range = np.array([-2999, 2998], np.int16)
        v = f.createVariable("dbl", "f8", ("j", "i"))
        v[:] = dbl
        v = f.createVariable("u", "f4", ("time", "k", "j", "i"))
        v[:] = rec
    for k in range(nk):
        got = nc.nc_read_layer(p, "temp", ni, nj, nk, k=k)
        assert same(got, read_rules(f3[k], fill=np.float32(-999.0))), k
        got = nc.nc_read_layer(p, "salt", ni, nj, nk, k=k)
        exp = read_rules(packed[k], missing=7777, vrange=(-2999, 2998), sf=0.01, ao=35.0, default_fill=-32767)
        assert same(got, exp), k
    assert same(nc.nc_read_layer(p, "eta", ni, nj, nk), read_rules(d2, default_fill=FILL_F))
    assert np.isnan(nc.nc_read_layer(p, "eta", ni, nj, nk)[3, 3])
    got = nc.nc_read_layer(p, "dbl", ni, nj, nk)
    assert np.isnan(got[1, 1]) and same(got, read_rules(dbl, default_fill=9.9692099683868690e+36))
    assert same(nc.nc_read_layer(p, "u", ni, nj, nk, k=2, r=1), rec[1, 2])
    with pytest.raises(Exception):                         # two records and no record given
        nc.nc_read_layer(p, "u", ni, nj, nk, k=0, r=-1)
    with pytest.raises(Exception):                         # grid mismatch
        nc.nc_read_layer(p, "temp", ni + 1, nj, nk)
    # hyperslabs of a record variable against numpy slicing
    for _ in range(20):
        st = [int(rng.integers(0, d)) for d in rec.shape]
        ct = [int(rng.integers(1, d - s + 1)) for d, s in zip(rec.shape, st)]
        sl = tuple(slice(s, s + c) for s, c in zip(st, ct))
        assert np.array_equal(nc.nc_get_vara_float(p, "u", st, ct), rec[sl])


def test_write_layer_rules(nc, tmp_path):
    rng = np.random.default_rng(3)
    nk, nj, ni = 3, 5, 7
    p = tmp_path / "analysis.nc"
    with netcdf_file(p, "w", version=2) as f:
        f.createDimension("time", None)
        f.createDimension("k", nk)
        f.createDimension("j", nj)
        f.createDimension("i", ni)
        v = f.createVariable("temp", "f4", ("k", "j", "i"))
        v[:] = np.zeros((nk, nj, ni), np.float32)
        v._FillValue = np.float32(-1.0e10)
        v.add_offset = np.float32(10.0)
        v.scale_factor = np.float32(0.5)
        v.valid_max = np.float32(30.0)
        v = f.createVariable("ssh", "f8", ("time", "j", "i"))
        v[:] = np.zeros((2, nj, ni))
    a = rng.normal(12, 5, (nj, ni)).astype(np.float32)
    a[0, 0] = np.nan
    nc.nc_write_layer(p, "temp", a, nk=nk, k=1)
    b = rng.normal(0, 1, (nj, ni)).astype(np.float32)
    nc.nc_write_layer(p, "ssh", b, nk=nk, k=0)
    exp = ((a - np.float32(10.0)) / np.float32(0.5)).astype(np.float32)
    exp = np.where(exp > np.float32(30.0), np.float32(30.0), exp)
    exp[0, 0] = np.float32(-1.0e10)
    with netcdf_file(p, "r", mmap=False) as f:
        got = f.variables["temp"][:].copy()
        assert np.array_equal(got[1], exp)
        assert np.array_equal(got[0], np.zeros((nj, ni), np.float32))
        ssh = f.variables["ssh"][:].copy()
        assert np.array_equal(ssh[1], b.astype(np.float64)) and np.array_equal(ssh[0], np.zeros((nj, ni)))


def test_errors(nc, tmp_path):
    p = tmp_path / "not.nc"
    p.write_bytes(b"HDF\x89 not classic")
    with pytest.raises(Exception) as ei:
        nc.nc_inq_var(p, "x")
    assert "not a NetCDF classic file" in str(ei.value)
    with pytest.raises(Exception):
        nc.nc_inq_var(tmp_path / "missing.nc", "x")
    q = tmp_path / "text.nc"
    with netcdf_file(q, "w", version=1) as f:
        f.createDimension("j", 2)
        f.createDimension("i", 3)
        v = f.createVariable("s", "c", ("j", "i"))
        v[:] = np.full((2, 3), b"a")
    with pytest.raises(Exception) as ei:
        nc.nc_write_layer(q, "s", np.zeros((2, 3), np.float32))
    assert getattr(ei.value, "status", None) == 8


def test_write_layer_packed(nc, tmp_path):
    """Packed short and byte variables: offset and scale undone in float,
    clamped, NaN to the fill value, then truncated toward zero."""
    rng = np.random.default_rng(13)
    nj, ni = 6, 7
    p = tmp_path / "packed.nc"
    with netcdf_file(p, "w", version=2) as f:
        f.createDimension("j", nj)
        f.createDimension("i", ni)
        v = f.createVariable("salt", "i2", ("j", "i"))
        v[:] = np.zeros((nj, ni), np.int16)
        v.scale_factor = np.float32(0.001)
        v.add_offset = np.float32(35.0)
        v._FillValue = np.int16(-32767)
        v.valid_range = np.array([-30000, 30000], np.int16)
        v = f.createVariable("flag", "i1", ("j", "i"))
        v[:] = np.zeros((nj, ni), np.int8)
    a = rng.normal(35.0, 5.0, (nj, ni)).astype(np.float32)
    a[0, 0] = np.nan
    a[1, 1] = 80.0                                          # beyond valid_range: clamped
    nc.nc_write_layer(p, "salt", a)
    x = ((a - np.float32(35.0)) / np.float32(0.001)).astype(np.float32)
    x = np.where(x < np.float32(-30000), np.float32(-30000), x)
    x = np.where(x > np.float32(30000), np.float32(30000), x)
    x[0, 0] = np.float32(-32767)
    b = rng.uniform(-100.0, 100.0, (nj, ni)).astype(np.float32)
    nc.nc_write_layer(p, "flag", b)
    with netcdf_file(p, "r", mmap=False) as f:
        assert np.array_equal(f.variables["salt"][:], np.trunc(x).astype(np.int16))
        assert np.array_equal(f.variables["flag"][:], np.trunc(b).astype(np.int8))
    # and back through the reader: the same values to the packing step
    back = nc.nc_read_layer(p, "salt", ni, nj)
    assert np.isnan(back[0, 0]) and np.abs(back[2:, :] - a[2:, :]).max() < 2e-3
    with pytest.raises(Exception):
        nc.nc_write_layer(p, "flag", np.full((nj, ni), 300.0, np.float32))


def _cdf5(path, dims, variables, numrecs=0):
    """A CDF-5 (64-bit data) file written here from the published format
    description, independently of the library: dims [(name, len)] (len 0:
    the record dimension), variables [(name, dimids, nc_type, data,
    atts)]; data big-endian, fixed variables first, then records."""
    import struct

    def name(s):
        b = s.encode()
        return struct.pack(">Q", len(b)) + b + b"\0" * (-len(b) % 4)

    def att_list(atts):
        if not atts:
            return b"\0" * 12
        out = struct.pack(">IQ", 0x0C, len(atts))
        for an, at, av in atts:
            raw = np.asarray(av).astype(at).tobytes()
            out += name(an) + struct.pack(">IQ", {">f4": 5, ">i2": 3, ">i4": 4}[at], np.asarray(av).size)
            out += raw + b"\0" * (-len(raw) % 4)
        return out

    def rec(v):
        return dims[v[1][0]][1] == 0 if v[1] else False

    codes = {">i1": 1, ">i2": 3, ">i4": 4, ">f4": 5, ">f8": 6, ">u1": 7, ">u2": 8, ">u4": 9, ">i8": 10, ">u8": 11}

    def vbytes(v):
        n = np.dtype(v[2]).itemsize
        for d in v[1][1:] if rec(v) else v[1]:
            n *= dims[d][1]
        return n

    def header(begins):
        h = b"CDF\x05" + struct.pack(">Q", numrecs)
        h += struct.pack(">IQ", 0x0A, len(dims)) + b"".join(name(n) + struct.pack(">Q", ln) for n, ln in dims)
        h += b"\0" * 12
        h += struct.pack(">IQ", 0x0B, len(variables))
        for v, b in zip(variables, begins):
            h += name(v[0]) + struct.pack(">Q", len(v[1])) + b"".join(struct.pack(">Q", d) for d in v[1])
            h += att_list(v[4]) + struct.pack(">I", codes[v[2]]) + struct.pack(">Q", vbytes(v) + (-vbytes(v) % 4))
            h += struct.pack(">Q", b)
        return h

    fixed = [v for v in variables if not rec(v)]
    recs = [v for v in variables if rec(v)]
    hlen = len(header([0] * len(variables)))
    begins, off = {}, hlen
    for v in fixed:
        begins[v[0]] = off
        off += vbytes(v) + (-vbytes(v) % 4)
    rsize = sum(vbytes(v) + (-vbytes(v) % 4) for v in recs) if len(recs) != 1 else (vbytes(recs[0]) if recs else 0)
    for v in recs:
        begins[v[0]] = off
        off += vbytes(v) + (-vbytes(v) % 4) if len(recs) != 1 else vbytes(v)
    body = bytearray()
    for v in fixed:
        raw = np.ascontiguousarray(v[3]).astype(v[2]).tobytes()
        body += raw + b"\0" * (-len(raw) % 4)
    for r in range(numrecs):
        for v in recs:
            raw = np.ascontiguousarray(v[3][r]).astype(v[2]).tobytes()
            body += raw + (b"\0" * (-len(raw) % 4) if len(recs) != 1 else b"")
    assert rsize >= 0
    with open(path, "wb") as f:
        f.write(header([begins[v[0]] for v in variables]) + bytes(body))


def test_read_cdf5(nc, tmp_path):
    rng = np.random.default_rng(4)
    nk, nj, ni = 3, 4, 5
    i8 = rng.integers(-2**40, 2**40, (nj, ni)).astype(np.int64)
    u2 = rng.integers(0, 60000, (nk, nj, ni)).astype(np.uint16)
    u2[1, 2, 3] = 65535                                     # the default ushort fill
    f3 = rng.normal(0, 1, (nk, nj, ni)).astype(np.float32)
    b1 = rng.integers(-100, 100, (nj, ni)).astype(np.int8)  # odd sizes: padding
    recs = rng.normal(0, 1, (3, nj, ni)).astype(np.float32)
    dims = [("time", 0), ("k", nk), ("j", nj), ("i", ni)]
    p = tmp_path / "cdf5.nc"
    _cdf5(p, dims, [("big", [2, 3], ">i8", i8, []),
                    ("u", [1, 2, 3], ">u2", u2, [("scale_factor", ">f4", np.float32(0.5))]),
                    ("temp", [1, 2, 3], ">f4", f3, []),
                    ("b", [2, 3], ">i1", b1, []),
                    ("eta", [0, 2, 3], ">f4", recs, []),
                    ("sal", [0, 2, 3], ">f4", recs + 1, [])], numrecs=3)
    assert nc.nc_inq_var(p, "eta") == ((3, nj, ni), 5, True)
    assert nc.nc_inq_var(p, "big") == ((nj, ni), 10, False)
    assert np.array_equal(nc.nc_get_vara_float(p, "big"), i8.astype(np.float32))
    assert np.array_equal(nc.nc_get_vara_float(p, "b"), b1.astype(np.float32))
    assert np.array_equal(nc.nc_get_vara_float(p, "temp"), f3)
    got = nc.nc_read_layer(p, "u", ni, nj, nk, k=1)
    assert same(got, read_rules(u2[1], sf=0.5, default_fill=65535))
    assert np.isnan(got[2, 3])
    for r in range(3):
        assert np.array_equal(nc.nc_read_layer(p, "eta", ni, nj, nk, r=r), recs[r])
        assert np.array_equal(nc.nc_read_layer(p, "sal", ni, nj, nk, r=r), recs[r] + 1)


def test_malformed_files_are_errors_not_crashes(nc, tmp_path):
    """Truncated and corrupted headers end in an error status (the process
    survives every case)."""
    rng = np.random.default_rng(6)
    good = tmp_path / "good.nc"
    T = rng.standard_normal((3, 4, 2, 5)).astype(np.float32)
    w = rng.standard_normal((3, 4, 5)).astype(np.float32)
    nc.nc_write_transforms(good, T, w, stride=2, grid_name="g")
    data = good.read_bytes()
    hdr = data.find(b"grid_name") + 64                      # well inside the header
    bad = tmp_path / "bad.nc"
    outcomes = {"error": 0, "ok": 0}
    for t in range(300):
        b = bytearray(data)
        if t % 3 == 0:
            b = b[: int(rng.integers(0, len(b)))]
        else:
            for _ in range(int(rng.integers(1, 4))):
                b[int(rng.integers(4, hdr))] = int(rng.integers(0, 256))
        bad.write_bytes(bytes(b))
        try:
            nc.nc_inq_var(bad, "T")
            nc.nc_get_vara_float(bad, "w", [0, 0, 0], [1, 1, 5])
            nc.nc_read_layer(bad, "w", 5, 4, 1)
            outcomes["ok"] += 1
        except Exception:
            outcomes["error"] += 1
    assert outcomes["error"] > 0


def test_read_field3d_rules(nc, tmp_path):
    rng = np.random.default_rng(7)
    nk, nj, ni = 3, 4, 6
    p = tmp_path / "member3d.nc"
    a = rng.normal(10, 1, (nk, nj, ni)).astype(np.float32)
    a[1, 1, 1] = FILL_F                     # default fill, but no masking attribute: kept
    b = rng.integers(-500, 500, (2, nk, nj, ni)).astype(np.int16)
    b[1, 2, 0, 0] = -32767                  # default short fill, masked because missing_value is present
    b[1, 0, 1, 1] = 99
    c = rng.normal(0, 1, (nk, nj, ni))
    with netcdf_file(p, "w", version=2) as f:
        f.createDimension("time", None)
        f.createDimension("k", nk)
        f.createDimension("j", nj)
        f.createDimension("i", ni)
        v = f.createVariable("a", "f4", ("k", "j", "i"))
        v[:] = a
        v = f.createVariable("b", "i2", ("time", "k", "j", "i"))
        v[:] = b
        v.missing_value = np.int16(99)
        v.scale_factor = np.float32(0.1)
        v = f.createVariable("c", "f8", ("k", "j", "i"))
        v[:] = c
    got = nc.nc_read_field3d(p, "a", ni, nj, nk)
    assert np.array_equal(got, a)                                   # FILL_F kept (no attributes)
    got = nc.nc_read_field3d(p, "b", ni, nj, nk, r=1)
    assert same(got, read_rules(b[1], missing=99, sf=0.1, default_fill=-32767))
    assert np.isnan(got[2, 0, 0]) and np.isnan(got[0, 1, 1])
    assert same(nc.nc_read_field3d(p, "c", ni, nj, nk), c.astype(np.float32))
    with pytest.raises(Exception):
        nc.nc_read_field3d(p, "b", ni, nj, nk)                      # two records, none named
    with pytest.raises(Exception):
        nc.nc_read_field3d(p, "a", ni, nj, nk + 1)                  # layer count mismatch


def test_transforms_row_by_row(nc, tmp_path):
    """nc_createtransforms then nc_writetransforms per strided row, in any
    row order, give the file the whole-array writer gives."""
    rng = np.random.default_rng(12)
    nj, ni, md, m = 6, 5, 3, 4
    T = rng.standard_normal((nj, ni, md, m)).astype(np.float32)
    w = rng.standard_normal((nj, ni, m)).astype(np.float32)
    p = tmp_path / "rows.nc"
    nc.nc_create_transforms(p, nj, ni, md, m, with_T=True, stride=2, grid_name="g1")
    for j in rng.permutation(nj):
        nc.nc_write_transforms_row(p, int(j), T[j], w[j])
    q = tmp_path / "whole.nc"
    nc.nc_write_transforms(q, T, w, stride=2, grid_name="g1")
    assert p.read_bytes() == q.read_bytes()
    with netcdf_file(p, "r", mmap=False) as f:
        assert np.array_equal(f.variables["T"][:], T) and np.array_equal(f.variables["w"][:], w)
    # EnOI (no T) and a row out of range
    e = tmp_path / "enoi.nc"
    nc.nc_create_transforms(e, nj, ni, 0, m, with_T=False)
    for j in range(nj):
        nc.nc_write_transforms_row(e, j, None, w[j])
    with netcdf_file(e, "r", mmap=False) as f:
        assert np.array_equal(f.variables["w"][:], w) and "T" not in f.variables
    with pytest.raises(Exception):
        nc.nc_write_transforms_row(e, nj, None, w[0])


def test_overflowing_sizes_are_errors(nc, tmp_path):
    """Sizes in a CDF-5 header that are negative as signed 64-bit numbers, or
    whose products with the type size overflow, are refused before any
    arithmetic on them (the reader returns an error status)."""
    import struct
    f3 = np.arange(20, dtype=np.float32).reshape(4, 5)
    p = tmp_path / "ok5.nc"
    _cdf5(p, [("j", 4), ("i", 5)], [("v", [0, 1], ">f4", f3, [("scale_factor", ">f4", np.float32(2.0))])])
    data = p.read_bytes()
    assert np.array_equal(nc.nc_get_vara_float(p, "v"), f3)
    bad = tmp_path / "bad5.nc"

    def refused(b):
        bad.write_bytes(bytes(b))
        with pytest.raises(Exception):
            nc.nc_get_vara_float(bad, "v")

    # the attribute's value count: 2^62 + 1 floats (x 4 bytes wraps to 4)
    at = data.find(b"scale_factor") + 12 + 4
    b = bytearray(data)
    b[at:at + 8] = struct.pack(">Q", (1 << 62) + 1)
    refused(b)
    # a dimension length with the top bit set (negative as a signed number)
    dj = data.find(b"j\0\0\0") + 4
    b = bytearray(data)
    b[dj:dj + 8] = struct.pack(">Q", 1 << 63)
    refused(b)
    # both lengths 2^32: 4 x 2^64 bytes overflows
    di = data.find(b"i\0\0\0", dj) + 4
    b = bytearray(data)
    b[dj:dj + 8] = struct.pack(">Q", 1 << 32)
    b[di:di + 8] = struct.pack(">Q", 1 << 32)
    refused(b)
