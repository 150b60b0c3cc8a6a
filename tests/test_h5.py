"""HDF5 restart files without libhdf5 (host only, no GPU).

The files are checked two ways: read back through the library's own reader,
and walked byte by byte by the small parser below, written from the HDF5
file format specification (superblock version 0, symbol-table groups,
version-1 object headers, contiguous storage), so that a writer and reader
that agreed on a private format would not pass."""
import math
import os
import struct

import numpy as np
import pytest

from conftest import make_bou, tc

SIG = b"\x89HDF\r\n\x1a\n"


def u(b, off, n):
    return int.from_bytes(b[off:off + n], "little")


def walk(path):
    """name -> (dims, dtype, values) of every dataset in the root group."""
    b = open(path, "rb").read()
    assert b[:8] == SIG
    assert b[8] == 0 and b[13] == 8 and b[14] == 8          # superblock 0, 8-byte offsets/lengths
    leaf_k, node_k = u(b, 16, 2), u(b, 18, 2)
    assert u(b, 40, 8) == len(b)                            # end-of-file address
    root = 56                                               # root symbol table entry
    root_oh = u(b, root + 8, 8)
    assert u(b, root + 16, 4) == 1                          # scratch pad: cached group tables
    btree, heap = u(b, root + 24, 8), u(b, root + 32, 8)
    # root object header: version 1, the symbol table message
    assert b[root_oh] == 1
    nmsg = u(b, root_oh + 2, 2)
    p = root_oh + 16
    found = False
    for _ in range(nmsg):
        t, sz = u(b, p, 2), u(b, p + 2, 2)
        if t == 0x11:
            assert (u(b, p + 8, 8), u(b, p + 16, 8)) == (btree, heap)
            found = True
        p += 8 + sz
    assert found
    assert b[heap:heap + 4] == b"HEAP"
    hsize, hdata = u(b, heap + 8, 8), u(b, heap + 24, 8)
    assert b[hdata] == 0                                    # offset 0: the empty name
    assert b[btree:btree + 4] == b"TREE" and b[btree + 4] == 0 and b[btree + 5] == 0
    nchild = u(b, btree + 6, 2)
    out = {}
    for c in range(nchild):
        snod = u(b, btree + 32 + 16 * c, 8)
        assert b[snod:snod + 4] == b"SNOD" and b[snod + 4] == 1
        nsym = u(b, snod + 6, 2)
        assert nsym <= 2 * leaf_k
        names = []
        for e in range(nsym):
            ent = snod + 8 + 40 * e
            off, oh = u(b, ent, 8), u(b, ent + 8, 8)
            name = b[hdata + off:b.index(b"\0", hdata + off)].decode()
            names.append(name)
            out[name] = dataset(b, oh)
        assert names == sorted(names)
        last_key = u(b, btree + 24 + 16 * (c + 1), 8)
        assert b[hdata + last_key:b.index(b"\0", hdata + last_key)].decode() == names[-1]
    return out


def dataset(b, oh):
    assert b[oh] == 1
    nmsg, p = u(b, oh + 2, 2), oh + 16
    dims = dtype = addr = size = None
    for _ in range(nmsg):
        t, sz = u(b, p, 2), u(b, p + 2, 2)
        d = p + 8
        if t == 0x01:
            assert b[d] == 1
            dims = [u(b, d + 8 + 8 * r, 8) for r in range(b[d + 1])]
        elif t == 0x03:
            cls, size_t = b[d] & 0x0F, u(b, d + 4, 4)
            if cls == 1:
                assert size_t == 8 and b[d + 1] == 0x20 and b[d + 2] == 63
                assert (b[d + 12], b[d + 13], b[d + 14], b[d + 15], u(b, d + 16, 4)) == (52, 11, 0, 52, 1023)
                dtype = "<f8"
            else:
                assert cls == 0 and size_t == 4 and b[d + 1] & 0x08
                dtype = "<i4"
        elif t == 0x08:
            assert b[d] == 3 and b[d + 1] == 1
            addr, size = u(b, d + 2, 8), u(b, d + 10, 8)
        p = d + sz
    n = math.prod(dims)
    vals = np.frombuffer(b[addr:addr + size], dtype=dtype, count=n).reshape(dims)
    assert size == n * np.dtype(dtype).itemsize
    return dims, dtype, vals


def test_dataset_round_trip_and_format(tmp_path):
    rng = np.random.default_rng(3)
    a = rng.standard_normal((5, 7, 9))
    path = str(tmp_path / "x.h5")
    tc.h5_write(path, "var", a)
    assert np.array_equal(tc.h5_read(path, "var"), a)
    ds = walk(path)
    assert list(ds) == ["var"]
    dims, dtype, vals = ds["var"]
    assert dims == [5, 7, 9] and dtype == "<f8" and np.array_equal(vals, a)


def test_grid_info_file(tmp_path):
    bou = make_bou(nthm=24, nzm=20, nrm=16, istr=6, str=3.0)
    tc.h5_write_grid_info(bou, str(tmp_path))
    path = str(tmp_path / "cordin_info.h5")
    ds = walk(path)
    assert sorted(ds) == ["rc", "rm", "tm", "zm"]
    rc, rm = tc.grid_array(bou, "rc"), tc.grid_array(bou, "rm")
    assert np.array_equal(ds["rc"][2], rc[:17]) and np.array_equal(ds["rm"][2], rm[:16])
    dxt = 24 * bou["lamb"] / (2 * math.pi)
    dxz = 20 / bou["alx3"]
    assert np.allclose(ds["tm"][2], (np.arange(24) + 0.5) / dxt, rtol=0, atol=1e-15)
    assert np.allclose(ds["zm"][2], (np.arange(20) + 0.5) / dxz, rtol=0, atol=1e-15)
    assert np.array_equal(tc.h5_read(path, "zm"), ds["zm"][2])


def test_reader_rejects_bad_files(tmp_path):
    p = tmp_path / "bad.h5"
    p.write_bytes(b"not an hdf5 file at all" * 4)
    with pytest.raises(tc.TCError) as e:
        tc.h5_read(str(p), "var")
    assert e.value.code == 2022
    good = str(tmp_path / "g.h5")
    tc.h5_write(good, "var", np.ones((3, 4)))
    raw = open(good, "rb").read()
    (tmp_path / "t.h5").write_bytes(raw[:300])
    with pytest.raises(tc.TCError):
        tc.h5_read(str(tmp_path / "t.h5"), "var")
    with pytest.raises(tc.TCError) as e:
        tc.h5_read(good, "missing")
    assert "missing" in str(e.value)


def test_reader_follows_multi_node_group_trees(tmp_path):
    """A file laid out as the HDF5 library lays out a group with more names
    than one symbol table node holds (leaf K = 4: 8 entries per node): two
    symbol table nodes under one B-tree node, and a continuation block in a
    dataset header."""
    names = [f"s{i:02d}" for i in range(11)]
    vals = {n: float(i) * 1.5 for i, n in enumerate(names)}
    blob = bytearray(b"\0" * 4096)

    def put(off, fmt, *v):
        struct.pack_into(fmt, blob, off, *v)

    heap_names = b"\0" * 8
    offs = {}
    for n in names:
        offs[n] = len(heap_names)
        heap_names += n.encode() + b"\0" * (8 - len(n) % 8)
    root_oh, heap, heapdata = 96, 200, 232
    btree = heapdata + len(heap_names)
    btree += (-btree) % 8
    snods = [btree + 544, btree + 544 + 328]
    oh0 = snods[1] + 328
    blob[0:8] = SIG
    put(8, "<8B", 0, 0, 0, 0, 0, 8, 8, 0)
    put(16, "<HHI", 4, 16, 0)
    put(24, "<QQQQ", 0, 2**64 - 1, 0, 2**64 - 1)
    put(56, "<QQII QQ", 0, root_oh, 1, 0, btree, heap)
    put(root_oh, "<BBHII", 1, 0, 1, 1, 24)
    put(root_oh + 16, "<HHB3x QQ", 0x11, 16, 0, btree, heap)
    blob[heap:heap + 4] = b"HEAP"
    put(heap + 8, "<QQQ", len(heap_names), 2**64 - 1, heapdata)
    blob[heapdata:heapdata + len(heap_names)] = heap_names
    groups = [names[:8], names[8:]]
    blob[btree:btree + 4] = b"TREE"
    put(btree + 4, "<BBH QQ", 0, 0, 2, 2**64 - 1, 2**64 - 1)
    put(btree + 24, "<Q", 0)
    p = oh0
    for c, grp in enumerate(groups):
        put(btree + 32 + 16 * c, "<QQ", snods[c], offs[grp[-1]])
        blob[snods[c]:snods[c] + 4] = b"SNOD"
        put(snods[c] + 4, "<BBH", 1, 0, len(grp))
        for e, n in enumerate(grp):
            # header: dataspace + a continuation to a block with datatype and layout
            cont = p + 16 + 24 + 24
            data = cont + 64
            put(snods[c] + 8 + 40 * e, "<QQII", offs[n], p, 0, 0)
            put(p, "<BBHII", 1, 0, 4, 1, 48)
            put(p + 16, "<HHB3x BBB5x Q", 0x01, 16, 0, 1, 1, 0, 1)
            put(p + 40, "<HHB3x QQ", 0x10, 16, 0, cont, 64)
            put(cont, "<HHB3x B3B I HH BBBB I 4x", 0x03, 24, 1, 0x11, 0x20, 63, 0, 8, 0, 64, 52, 11, 0, 52, 1023)
            put(cont + 32, "<HHB3x BB QQ 6x", 0x08, 24, 0, 3, 1, data, 8)
            put(data, "<d", vals[n])
            p = data + 8
    put(40, "<Q", p)
    path = tmp_path / "master_like.h5"
    path.write_bytes(bytes(blob[:p]))
    for n in names:
        assert tc.h5_read(str(path), n)[0] == vals[n]


def _write_continua(d, nthm, nzm, nrm, fields, time=0.25, istr=0, str_=1.0):
    nr = nrm + 1
    tc.h5_write_scalars(str(d / "continua_master.h5"),
                        dict(nr=nr, nth=nthm + 1, nz=nzm + 1, time=time, rint=1.0, rext=1.4, istr=istr, str=str_,
                             alx3=2 * math.pi, lamb=1.0), ints=("nr", "nth", "nz", "istr"))
    for name, f in zip(("qt", "qr", "qz"), fields):
        tc.h5_write(str(d / f"continua_{name}.h5"), "var", f)


def _gridnew(n, rint, rext):
    # interp.F90 gridnew for istr = 0: rc = rext x + rint (kept as in the reference)
    rc = np.array([rext * (i / (n - 1)) + rint for i in range(n)])
    rm = np.empty(n)
    rm[:-1] = 0.5 * (rc[:-1] + rc[1:])
    rm[-1] = 2 * rc[-1] - rm[-2]
    return rc, rm


def test_continua_load_same_grid(tmp_path):
    from conftest import make_bou
    bou = make_bou(nthm=8, nzm=6, nrm=5)
    rng = np.random.default_rng(0)
    f = [rng.standard_normal((8, 6, 6)) for _ in range(3)]
    _write_continua(tmp_path, 8, 6, 5, f, time=0.75, istr=bou["istr"], str_=bou["str"])
    qt, qr, qz, t = tc.h5_load_continua(bou, str(tmp_path))
    assert t == 0.75
    for a, b in zip((qt, qr, qz), f):
        assert np.array_equal(a[1:-1, 1:-1, :], b)
    # IRESET = 1 starts the clock again (ReadFlowField.F90:144)
    assert tc.h5_load_continua(dict(bou, ireset=1), str(tmp_path))[3] == 0.0


def test_continua_interpolated_onto_a_finer_grid(tmp_path):
    """interp.F90: bilinear in theta and z between the old points (a field
    linear in theta and z comes back exactly away from the corners), no
    interpolation in r, qt placed at (tc, zm), qz at (tm, zm)."""
    from conftest import make_bou
    old = dict(nthm=8, nzm=6, nrm=6)
    new = make_bou(nthm=12, nzm=10, nrm=6, istr=0)
    thmax, alx3 = 2 * math.pi, 2 * math.pi
    tco, tmo = _gridnew(old["nthm"] + 1, 0.0, thmax)
    zco, zmo = _gridnew(old["nzm"] + 1, 0.0, alx3)
    tcn, tmn = _gridnew(13, 0.0, thmax)
    zcn, zmn = _gridnew(11, 0.0, alx3)
    a, b, c = 0.3, -0.7, 1.25

    def field(xs, ys, nth, nz, nr):
        f = np.empty((nth, nz, nr))
        for i in range(nth):
            for j in range(nz):
                f[i, j, :] = a * xs[i] + b * ys[j] + c
        return f

    f_qt = field(tco, zmo, 8, 6, 7)
    f_qz = field(tmo, zmo, 8, 6, 7)
    _write_continua(tmp_path, 8, 6, 6, [f_qt, f_qt * 0, f_qz])
    qt, qr, qz, t = tc.h5_load_continua(new, str(tmp_path))
    want_qt = field(tcn, zmn, 12, 10, 7)
    want_qz = field(tmn, zmn, 12, 10, 7)
    # away from the old field's unset corner halos (first and last new points)
    sl = (slice(2, 11), slice(2, 9), slice(1, 6))
    got_qt = qt[1:-1, 1:-1, :][sl]
    got_qz = qz[1:-1, 1:-1, :][sl]
    assert np.allclose(got_qt, want_qt[sl], rtol=0, atol=1e-12)
    assert np.allclose(got_qz, want_qz[sl], rtol=0, atol=1e-12)
    # more than twice as fine is refused
    with pytest.raises(tc.TCError) as e:
        tc.h5_load_continua(make_bou(nthm=24, nzm=10, nrm=6), str(tmp_path))
    assert e.value.code == 2024
