"""The netCDF classic-format reader/writer (wf_netcdf.cpp) on the CPU.

Files written by scipy's independent implementation of the classic format (CDF-1 and CDF-2)
are read back by the library, and files the library writes are read by scipy: types, fixed
and record variables (one and several record variables, whose record layout differs),
attributes, hyperslabs and the CF decoding (_FillValue, missing_value, scale_factor,
add_offset) that NCDatasets applies when Wflow reads a variable. CDF-5 (which scipy does not
read) is checked by round trip, including its 64-bit integer types.
"""

import numpy as np
import pytest

from wflow_gb300 import abi, build, ncio

netcdf = pytest.importorskip("scipy.io").netcdf_file


@pytest.fixture(scope="module", autouse=True)
def lib():
    build.build_all()
    return abi.load_library()


def test_header_symbols_exported(lib):
    names = abi.header_symbols("wflow_gb300_nc.h")
    assert "wf_nc_open" in names and "wf_nc_put" in names
    assert not [n for n in names if not hasattr(lib, n)]


@pytest.mark.parametrize("version", [1, 2])
@pytest.mark.parametrize("n_rec_vars", [1, 2])
def test_read_files_written_by_scipy(tmp_path, version, n_rec_vars):
    rng = np.random.default_rng(version * 10 + n_rec_vars)
    path = tmp_path / f"s{version}{n_rec_vars}.nc"
    f = netcdf(str(path), "w", version=version)
    f.title = "scipy written"
    f.createDimension("time", None)
    f.createDimension("layer", 3)
    f.createDimension("y", 5)
    f.createDimension("x", 7)
    dem = f.createVariable("dem", "d", ("y", "x"))
    dem[:] = rng.normal(100, 10, (5, 7))
    dem.units = "m"
    ldd = f.createVariable("ldd", "b", ("y", "x"))
    ldd[:] = rng.integers(1, 10, (5, 7)).astype(np.int8)
    ksat = f.createVariable("ksat", "h", ("layer", "y", "x"))
    raw = rng.integers(-1000, 1000, (3, 5, 7)).astype(np.int16)
    raw[0, 0, 0] = -9999
    ksat[:] = raw
    ksat._FillValue = np.int16(-9999)
    ksat.scale_factor = 0.5
    ksat.add_offset = 10.0
    p = f.createVariable("precip", "f", ("time", "y", "x"))
    pvals = rng.random((4, 5, 7)).astype(np.float32)
    p[:] = pvals
    if n_rec_vars == 2:
        t = f.createVariable("temp", "i", ("time", "x"))
        tvals = rng.integers(-50, 50, (4, 7)).astype(np.int32)
        t[:] = tvals
    f.close()

    nc = ncio.NcFile(path)
    assert nc.format == version and nc.numrecs == 4
    assert nc.dimensions["time"] == (4, True) and nc.dimensions["x"] == (7, False)
    assert nc.attrs()["title"] == "scipy written"
    assert nc.attrs("dem")["units"] == "m"
    with netcdf(str(path), "r", mmap=False) as ref:
        assert np.array_equal(nc.read("dem"), ref.variables["dem"][:])
        assert np.array_equal(nc.read("ldd"), ref.variables["ldd"][:].astype(float))
        assert np.array_equal(nc.read("precip"), ref.variables["precip"][:].astype(float))
        if n_rec_vars == 2:
            assert np.array_equal(nc.read("temp"), tvals.astype(float))
    # CF decoding: fill -> NaN, then raw * scale + offset
    dec = nc.read("ksat")
    assert np.isnan(dec[0, 0, 0])
    expect = raw.astype(float) * 0.5 + 10.0
    assert np.array_equal(dec.reshape(-1)[1:], expect.reshape(-1)[1:])
    assert np.array_equal(nc.read("ksat", decode=False), raw.astype(float))
    # hyperslabs (a record range, an inner box)
    assert np.array_equal(nc.read("precip", start=[1, 2, 3], count=[2, 2, 3]), pvals[1:3, 2:4, 3:6].astype(float))
    assert np.array_equal(nc.read("ksat", decode=False, start=[2, 0, 5], count=[1, 5, 2]),
                          raw[2:3, :, 5:7].astype(float))
    nc.close()


@pytest.mark.parametrize("version", [1, 2])
@pytest.mark.parametrize("n_rec_vars", [1, 3])
def test_scipy_reads_files_written_here(tmp_path, version, n_rec_vars):
    rng = np.random.default_rng(7 + version + n_rec_vars)
    path = tmp_path / f"w{version}{n_rec_vars}.nc"
    nc = ncio.NcFile(path, "w", format=version)
    nc.def_dim("time", 0)
    nc.def_dim("layer", 4)
    nc.def_dim("y", 6)
    nc.def_dim("x", 3)
    nc.def_var("sat", ncio.NC_DOUBLE, ("y", "x"), {"units": "mm"})
    nc.def_var("nl", ncio.NC_BYTE, ("y", "x"))
    nc.def_var("ustore", ncio.NC_FLOAT, ("layer", "y", "x"), {"_FillValue": -999.0})
    rec = ["q", "h", "code"][:n_rec_vars]
    types = {"q": ncio.NC_DOUBLE, "h": ncio.NC_FLOAT, "code": ncio.NC_SHORT}
    for r in rec:
        nc.def_var(r, types[r], ("time", "y", "x"))
    nc.put_att(None, "history", "written by wf_netcdf")
    sat = rng.random((6, 3))
    nl = rng.integers(1, 5, (6, 3))
    us = rng.random((4, 6, 3)).astype(np.float32).astype(float)
    us[3, 0, 0] = np.nan  # written as the fill value
    nc.write("sat", sat)
    nc.write("nl", nl)
    nc.write("ustore", us)
    vals = {}
    for k in range(3):  # three records, written one at a time
        for r in rec:
            v = rng.random((1, 6, 3)) * 100
            if r == "code":
                v = np.round(v)
            if r == "h":
                v = v.astype(np.float32).astype(float)
            vals.setdefault(r, []).append(v[0])
            nc.write(r, v, start=[k, 0, 0])
    nc.close()
    with netcdf(str(path), "r", mmap=False) as ref:
        assert ref.version_byte == version
        assert ref.history == b"written by wf_netcdf"
        assert ref.variables["sat"].units == b"mm"
        assert np.array_equal(ref.variables["sat"][:], sat)
        assert np.array_equal(ref.variables["nl"][:], nl)
        u = ref.variables["ustore"][:].astype(float)
        assert u[3, 0, 0] == -999.0
        assert np.array_equal(u.reshape(-1)[:-18], us.reshape(-1)[:-18])
        for r in rec:
            assert ref.variables[r].shape == (3, 6, 3)
            assert np.array_equal(ref.variables[r][:].astype(float), np.array(vals[r]))
    # and the library reads its own file back, NaN where the fill value was written
    back = ncio.NcFile(path)
    got = back.read("ustore")
    assert np.isnan(got[3, 0, 0])
    assert np.array_equal(got.reshape(-1)[:-18], us.reshape(-1)[:-18])


def test_cdf5_round_trip(tmp_path):
    path = tmp_path / "c5.nc"
    nc = ncio.NcFile(path, "w", format=5)
    nc.def_dim("n", 5)
    nc.def_dim("t", 0)
    data = {
        ncio.NC_INT64: np.array([-2.0**62, -1, 0, 1, 2.0**62]),
        ncio.NC_UINT64: np.array([0, 1, 2.0**40, 2.0**63, 3]),
        ncio.NC_UBYTE: np.array([0, 1, 128, 254, 255]),
        ncio.NC_USHORT: np.array([0, 1, 65535, 2, 3]),
        ncio.NC_UINT: np.array([0, 1, 4294967295, 2, 3]),
        ncio.NC_DOUBLE: np.array([np.pi, -np.e, 1e300, -1e-300, 0.0]),
    }
    for t in data:
        nc.def_var(f"v{t}", t, ("n",))
    nc.def_var("series", ncio.NC_INT64, ("t", "n"))
    for t, v in data.items():
        nc.write(f"v{t}", v)
    s = np.arange(15, dtype=float).reshape(3, 5) - 7
    nc.write("series", s)
    nc.close()
    back = ncio.NcFile(path)
    assert back.format == 5 and back.numrecs == 3
    for t, v in data.items():
        assert np.array_equal(back.read(f"v{t}"), v), t
    assert np.array_equal(back.read("series"), s)


def test_rejections(tmp_path):
    hdf = tmp_path / "x.nc"
    hdf.write_bytes(b"\x89HDF\r\n\x1a\n" + b"\0" * 64)
    with pytest.raises(OSError, match="netCDF-4"):
        ncio.NcFile(hdf)
    nc = ncio.NcFile(tmp_path / "r.nc", "w", format=1)
    nc.def_dim("n", 3)
    with pytest.raises(ValueError):
        nc.def_var("bad", ncio.NC_INT64, ("n",))  # 64-bit integers need CDF-5
    nc.def_var("b", ncio.NC_BYTE, ("n",))
    with pytest.raises(ValueError, match="out of range"):
        nc.write("b", np.array([1.0, 300.0, 2.0]))
    nc.close()
    # a truncated file
    good = tmp_path / "g.nc"
    w = ncio.NcFile(good, "w", format=2)
    w.def_dim("n", 1000)
    w.def_var("v", ncio.NC_DOUBLE, ("n",))
    w.write("v", np.arange(1000.0))
    w.close()
    cut = tmp_path / "cut.nc"
    cut.write_bytes(good.read_bytes()[:2000])
    f = ncio.NcFile(cut)
    with pytest.raises(ValueError, match="past the end"):
        f.read("v")


@pytest.mark.parametrize("code,nctype", [("b", ncio.NC_BYTE), ("h", ncio.NC_SHORT)])
@pytest.mark.parametrize("n_rec_vars", [1, 2])
def test_record_padding_matches_scipy(tmp_path, code, nctype, n_rec_vars):
    # records of byte and short variables whose size is not a multiple of 4: padded when there
    # are several record variables, unpadded for a lone one
    vals = (np.arange(3 * 35).reshape(3, 5, 7) % 100).astype(np.int8 if code == "b" else np.int16)
    w_vals = np.arange(21).reshape(3, 7).astype(np.int8)
    p = tmp_path / "s.nc"
    f = netcdf(str(p), "w", version=2)
    f.createDimension("time", None)
    f.createDimension("y", 5)
    f.createDimension("x", 7)
    f.createVariable("v", code, ("time", "y", "x"))[:] = vals
    if n_rec_vars == 2:
        f.createVariable("w", "b", ("time", "x"))[:] = w_vals
    f.close()
    nc = ncio.NcFile(p)
    assert np.array_equal(nc.read("v"), vals.astype(float))
    if n_rec_vars == 2:
        assert np.array_equal(nc.read("w"), w_vals.astype(float))
    q = tmp_path / "o.nc"
    o = ncio.NcFile(q, "w", format=2)
    o.def_dim("time", 0)
    o.def_dim("y", 5)
    o.def_dim("x", 7)
    o.def_var("v", nctype, ("time", "y", "x"))
    if n_rec_vars == 2:
        o.def_var("w", ncio.NC_BYTE, ("time", "x"))
    o.write("v", vals.astype(float))
    if n_rec_vars == 2:
        o.write("w", w_vals.astype(float))
    o.close()
    with netcdf(str(q), "r", mmap=False) as r:
        assert np.array_equal(r.variables["v"][:], vals)
        if n_rec_vars == 2:
            assert np.array_equal(r.variables["w"][:], w_vals)


def test_one_dimensional_record_variable(tmp_path):
    # a time coordinate (one value per record) beside a gridded record variable: its values are
    # a record size apart in the file, not contiguous
    p = tmp_path / "t.nc"
    f = netcdf(str(p), "w", version=2)
    f.createDimension("time", None)
    f.createDimension("x", 3)
    f.createVariable("time", "d", ("time",))[:] = [1.5, 2.5, 3.5, 4.5]
    f.createVariable("v", "f", ("time", "x"))[:] = np.arange(12, dtype=np.float32).reshape(4, 3)
    f.close()
    r = ncio.NcFile(p)
    assert np.array_equal(r.read("time"), [1.5, 2.5, 3.5, 4.5])
    assert np.array_equal(r.read("time", start=[1], count=[2]), [2.5, 3.5])
    q = tmp_path / "o.nc"
    w = ncio.NcFile(q, "w", format=1)
    w.def_dim("time", 0)
    w.def_dim("x", 3)
    w.def_var("time", ncio.NC_DOUBLE, ("time",))
    w.def_var("v", ncio.NC_DOUBLE, ("time", "x"))
    w.write("time", np.array([10.0, 20.0, 30.0]))
    for k in range(3):
        w.write("v", np.full((1, 3), float(k)), start=[k, 0])
    w.close()
    with netcdf(str(q), "r", mmap=False) as g:
        assert np.array_equal(g.variables["time"][:], [10.0, 20.0, 30.0])
        assert np.array_equal(g.variables["v"][:], np.repeat(np.arange(3.0)[:, None], 3, axis=1))


def test_corrupted_files_are_rejected_or_read_without_crashing(tmp_path):
    # bytes of a valid file's header flipped at random, or the file cut short: the reader either
    # rejects the file with an error or reads it; it never reads out of bounds
    p = tmp_path / "base.nc"
    w = ncio.NcFile(p, "w", format=2)
    w.def_dim("time", 0)
    w.def_dim("y", 4)
    w.def_dim("x", 5)
    w.def_var("a", ncio.NC_DOUBLE, ("y", "x"), {"units": "mm", "_FillValue": -9.0})
    w.def_var("t", ncio.NC_DOUBLE, ("time",))
    w.def_var("r", ncio.NC_SHORT, ("time", "y", "x"))
    w.write("a", np.arange(20.0).reshape(4, 5))
    w.write("t", np.arange(3.0))
    w.write("r", np.ones((3, 4, 5)))
    w.close()
    base = p.read_bytes()
    rng = np.random.default_rng(0)
    q = tmp_path / "fz.nc"
    for _ in range(400):
        b = bytearray(base)
        for _ in range(int(rng.integers(1, 4))):
            b[int(rng.integers(0, min(len(b), 300)))] = int(rng.integers(0, 256))
        if rng.random() < 0.2:
            b = b[: int(rng.integers(4, len(b)))]
        q.write_bytes(bytes(b))
        try:
            f = ncio.NcFile(q)
        except (OSError, ValueError):
            continue
        for name in list(f.variables):
            try:
                if np.prod(f.shape(name), dtype=float) <= 1e6:  # a corrupted length may claim gigabytes
                    f.read(name)
                f.attrs(name)
            except (ValueError, KeyError, MemoryError):
                pass
        f.close()
