"""Acquisition files without h5py: the Dataset layout and the UDSP v4.0 Set.

The round trips restate the reference's own tests (simulation/tests/
test_dataset.py: 2D and 3D, ground truth kept; simulation/tests/
test_uarp_format.py: data, geometry, timing and transmit map kept, and the
UDSP group layout present).  No HDF5 implementation exists here to read the
files written here, so the format tests pin the structures themselves: the
superblock, variable-length strings in a global heap, B-trees of several
levels (small node ranks) and sibling links, chunked gzip data with an edge
chunk, a user block before the superblock, a hand-built file of the
structures newer writers use, and one file the HDF5 library itself wrote
(read back, and its messages compared byte for byte with the writer's).
"""

import os
import struct

import numpy as np
import pytest

from openusct_gb300 import dataset_io, hdf5
from openusct_gb300.acquire import ArrayGeometry, Dataset


def _ring_dataset(n_tx=3, nt=300, n_el=8, truth=True, seed=0):
    rng = np.random.default_rng(seed)
    ang = np.linspace(0, 2 * np.pi, n_el, endpoint=False)
    pos = 0.024 * np.column_stack([np.cos(ang), np.sin(ang)])
    c = 1480.0 + 20.0 * rng.standard_normal((61, 61))
    return Dataset(geometry=ArrayGeometry(pos, 0.024, 0.4e6, "ring"),
                   data=rng.standard_normal((n_tx, nt, n_el)) * 1e-3, sample_rate_hz=1 / 1.2e-7,
                   tx_wavelet=rng.standard_normal(nt), tx_centre_freq_hz=0.41e6,
                   nominal_speed_m_s=1480.0, tx_elements=[0, 2, 4][:n_tx],
                   ground_truth={"c": c, "h_m": 1e-3} if truth else None,
                   metadata={"description": "roundtrip test", "created_by": "tests"})


def _cylinder_dataset(src=(0, 6), nt=120):
    rng = np.random.default_rng(1)
    zs = np.linspace(-0.005, 0.005, 2)
    ang = np.linspace(0, 2 * np.pi, 6, endpoint=False)
    pos = np.array([[0.012 * np.cos(a), 0.012 * np.sin(a), z] for z in zs for a in ang])
    c = 1480.0 + rng.standard_normal((16, 16, 16))
    return Dataset(geometry=ArrayGeometry(pos, 0.012, 0.3e6, "cylinder"),
                   data=rng.standard_normal((len(src), nt, 12)), sample_rate_hz=5e6,
                   tx_wavelet=rng.standard_normal(nt), tx_centre_freq_hz=0.3e6,
                   nominal_speed_m_s=1480.0, tx_elements=list(src),
                   ground_truth={"c": c, "h_m": 2e-3})


def test_dataset_roundtrip_2d(tmp_path):
    ds = _ring_dataset()
    path = str(tmp_path / "ds.h5")
    ds.save(path)
    got = Dataset.load(path)
    assert got.data.dtype == np.float32 and got.data.shape == (3, 300, 8)
    assert np.array_equal(got.data, ds.data.astype(np.float32))
    assert np.array_equal(got.geometry.element_pos, ds.geometry.element_pos)
    assert got.geometry.dim == 2 and got.geometry.n_elements == 8
    assert got.geometry.array_type == "ring" and got.geometry.radius_m == 0.024
    assert got.geometry.centre_freq_hz == 0.4e6
    assert got.sample_rate_hz == ds.sample_rate_hz and got.nominal_speed_m_s == 1480.0
    assert got.tx_centre_freq_hz == 0.41e6
    assert np.array_equal(got.tx_wavelet, ds.tx_wavelet)
    assert list(got.tx_elements) == [0, 2, 4]
    assert np.array_equal(got.ground_truth["c"], ds.ground_truth["c"])
    assert got.ground_truth["h_m"] == 1e-3
    assert got.metadata == {"description": "roundtrip test", "created_by": "tests",
                            "format_version": "1.0"}


def test_dataset_roundtrip_3d_and_without_truth(tmp_path):
    ds = _cylinder_dataset()
    path = str(tmp_path / "ds3d.h5")
    dataset_io.save(ds, path)
    got = dataset_io.load(path)
    assert got.geometry.dim == 3 and got.geometry.element_pos.shape == (12, 3)
    assert np.array_equal(got.data, ds.data.astype(np.float32))
    assert got.ground_truth["c"].shape == (16, 16, 16)
    assert np.array_equal(got.ground_truth["c"], ds.ground_truth["c"])
    bare = _ring_dataset(truth=False)
    dataset_io.save(bare, path, compression=None)
    got = dataset_io.load(path)
    assert got.ground_truth is None and np.array_equal(got.data, bare.data.astype(np.float32))
    with hdf5.File(path, "r") as f:
        assert "ground_truth" not in f and f["acquisition/data"].compression is None


def test_dataset_layout_is_the_schema(tmp_path):
    path = str(tmp_path / "ds.h5")
    dataset_io.save(_ring_dataset(), path)
    with hdf5.File(path, "r") as f:
        assert sorted(f.keys()) == ["acquisition", "geometry", "ground_truth"]
        assert f.attrs["format_version"] == "1.0" and isinstance(f.attrs["description"], str)
        g = f["geometry"]
        assert sorted(g.attrs.keys()) == ["array_type", "centre_freq_hz", "n_elements", "radius_m"]
        assert g.attrs["n_elements"] == 8 and g.attrs["n_elements"].dtype == np.int64
        assert g["element_pos"].dtype == np.float64 and g["element_pos"].shape == (8, 2)
        a = f["acquisition"]
        assert sorted(a.keys()) == ["data", "tx_elements", "tx_wavelet"]
        assert a["data"].dtype == np.float32 and a["data"].compression == "gzip"
        assert a["tx_elements"].dtype == np.int64
        assert f["ground_truth"]["c"].compression == "gzip"


def test_unknown_major_version_is_refused(tmp_path):
    path = str(tmp_path / "v2.h5")
    with hdf5.File(path, "w") as f:
        f.attrs["format_version"] = "2.0"
    with pytest.raises(ValueError, match="format_version"):
        dataset_io.load(path)


def test_uarp_roundtrip_and_layout(tmp_path):
    ds = _cylinder_dataset(src=(0, 4, 8, 11), nt=120)
    path = str(tmp_path / "acq_udsp.h5")
    dataset_io.to_uarp_set(ds, path)
    with hdf5.File(path, "r") as f:
        assert f.attrs["Version"] == "4.0"
        s0 = f["Series/Series000"]
        assert "Dimensions/Value" in s0
        assert float(s0["Dimensions/Dimension1"].attrs["Uniform.Stride"]) == 1 / 5e6
        assert "Dimensions/Dimension2/Sparse.Points" in s0
        assert int(s0["Frames"].attrs["Size"]) == 4
        assert "Frames/Frame000000" in s0
        assert s0["Frames/Frame000003"].attrs["Description"] == "tx_element=11"
        assert s0.attrs["State"] == "Analytical"
    got = dataset_io.from_uarp_set(path)
    assert got.n_tx == 4 and got.n_samples == 120 and got.geometry.dim == 3
    assert np.array_equal(got.data, ds.data.astype(np.float32))
    assert np.array_equal(got.geometry.element_pos, ds.geometry.element_pos)
    assert abs(got.dt - 1 / 5e6) < 1e-15
    assert list(got.tx_elements) == [0, 4, 8, 11]
    assert got.geometry.array_type == "cylinder"
    assert np.isclose(got.geometry.radius_m, np.linalg.norm(ds.geometry.element_pos, axis=1).max())


def test_superblock_and_strings_are_the_earliest_format(tmp_path):
    path = str(tmp_path / "s.h5")
    with hdf5.File(path, "w") as f:
        f.attrs["text"] = "ring"
        f.attrs["empty"] = ""
        f.attrs["fixed"] = b"abc"
        f.attrs["labels"] = np.array(["a", "bc"])
        f.attrs["ints"] = np.arange(3, dtype=np.int32)
        f.create_group("g")
        f.create_dataset("scalar", data=np.float64(3.5))
        f.create_dataset("empty", data=np.zeros((0, 3)))
        f.create_dataset("strided", data=np.arange(12, dtype=np.int16).reshape(3, 4)[:, ::2])
    raw = open(path, "rb").read()
    assert raw[:8] == hdf5.SIGNATURE
    assert raw[8:16] == bytes([0, 0, 0, 0, 0, 8, 8, 0])          # version 0, 8-byte offsets
    leaf_k, internal_k = struct.unpack("<HH", raw[16:20])
    assert leaf_k >= 4 and internal_k == 16
    assert struct.unpack("<Q", raw[40:48])[0] == len(raw)        # end of file
    assert b"GCOL" in raw and b"TREE" in raw and b"HEAP" in raw and b"SNOD" in raw
    oh = struct.unpack("<Q", raw[64:72])[0]                       # the root entry's header
    assert raw[oh] == 1                                           # version-1 object header
    with hdf5.File(path, "r") as f:
        assert f.attrs["text"] == "ring" and isinstance(f.attrs["text"], str)
        assert f.attrs["empty"] == ""
        assert f.attrs["fixed"] == b"abc" and isinstance(f.attrs["fixed"], np.bytes_)
        assert list(f.attrs["labels"]) == ["a", "bc"]
        assert f.attrs["ints"].dtype == np.int32 and list(f.attrs["ints"]) == [0, 1, 2]
        assert f.keys() == ["empty", "g", "scalar", "strided"] and f["g"].keys() == []
        assert f["scalar"].shape == () and f["scalar"][()] == 3.5
        assert f["empty"][()].shape == (0, 3)
        assert f["strided"][()].tolist() == [[0, 2], [4, 6], [8, 10]]


def test_deep_btrees_and_edge_chunks(tmp_path, monkeypatch):
    """Small node ranks force several symbol-table nodes and B-tree levels;
    small chunks force a chunk B-tree of several levels and a partial last
    chunk: everything reads back in order and unchanged."""
    monkeypatch.setattr(hdf5, "_CHUNK_BYTES", 4 * 7 * 5)       # 5 rows of 7 FP32 per chunk
    path = str(tmp_path / "deep.h5")
    rng = np.random.default_rng(2)
    big = rng.standard_normal((333, 7)).astype(np.float32)      # 67 chunks, the last partial
    arrays = {f"Frame{i:06d}": rng.standard_normal((3, 2)) for i in range(41)}
    with hdf5.File(path, "w", leaf_k=2, internal_k=2) as f:
        fr = f.create_group("Frames")
        for k, v in arrays.items():
            fr.create_dataset(k, data=v)
        f.create_dataset("big", data=big, compression="gzip")
    with hdf5.File(path, "r") as f:
        assert f["Frames"].keys() == sorted(arrays)
        for k, v in arrays.items():
            assert np.array_equal(f["Frames"][k][()], v)
        assert f["big"].chunks == (5, 7)
        assert np.array_equal(f["big"][()], big)


def test_btree_leaves_are_linked_by_siblings(tmp_path):
    """Readers that walk a B-tree's leaf level through right-sibling links
    (instead of descending every child) find the same symbol-table nodes."""
    path = str(tmp_path / "sib.h5")
    with hdf5.File(path, "w", leaf_k=1, internal_k=2) as f:
        for i in range(37):
            f.create_group(f"g{i:03d}")
    raw = open(path, "rb").read()
    bt = struct.unpack("<Q", raw[80:88])[0]            # root entry scratch: B-tree
    q = lambda a: struct.unpack("<Q", raw[a:a + 8])[0]  # noqa: E731

    def node(a):
        assert raw[a:a + 4] == b"TREE" and raw[a + 4] == 0
        level, n = raw[a + 5], struct.unpack("<H", raw[a + 6:a + 8])[0]
        left, right = q(a + 8), q(a + 16)
        kids = [q(a + 24 + 8 + 16 * i) for i in range(n)]
        return level, left, right, kids

    def descend(a):
        level, _, _, kids = node(a)
        return [a] if level == 0 else [x for k in kids for x in descend(k)]

    leaves = descend(bt)
    assert len(leaves) > 2
    level, left, right, _ = node(bt)
    a = bt
    while node(a)[0] > 0:
        a = node(a)[3][0]
    walked = []
    while a != hdf5.UNDEF:
        walked.append(a)
        a = node(a)[2]
    assert walked == leaves
    assert node(leaves[0])[1] == hdf5.UNDEF
    assert all(node(leaves[i])[1] == leaves[i - 1] for i in range(1, len(leaves)))
    names = []
    for leaf in leaves:
        for snod in node(leaf)[3]:
            assert raw[snod:snod + 4] == b"SNOD"
            names.append(struct.unpack("<H", raw[snod + 6:snod + 8])[0])
    assert sum(names) == 37
    with hdf5.File(path, "r") as f:
        assert f.keys() == [f"g{i:03d}" for i in range(37)]


def test_user_block_before_the_superblock(tmp_path):
    path = str(tmp_path / "plain.h5")
    dataset_io.save(_ring_dataset(), path)
    shifted = str(tmp_path / "shifted.h5")
    with open(shifted, "wb") as out:
        out.write(b"\0" * 512 + open(path, "rb").read())
    got = dataset_io.load(shifted)
    assert np.array_equal(got.data, _ring_dataset().data.astype(np.float32))


def test_errors_are_reported(tmp_path):
    with pytest.raises(ValueError, match="not an HDF5 file"):
        p = tmp_path / "x.h5"
        p.write_bytes(b"nope" * 100)
        hdf5.File(str(p), "r")
    with hdf5.File(str(tmp_path / "e.h5"), "w") as f:
        with pytest.raises(NotImplementedError):
            f.create_dataset("s", data=np.array(["a"]))
        with pytest.raises(NotImplementedError):
            f.create_dataset("z", data=np.zeros(3), compression="lzf")
    # a failed write leaves no file behind
    with pytest.raises(RuntimeError):
        with hdf5.File(str(tmp_path / "never.h5"), "w") as f:
            f.attrs["a"] = 1
            raise RuntimeError("stop")
    assert not os.path.exists(tmp_path / "never.h5")


REF = os.path.join(os.environ.get("USCT_REFERENCE", ""), "simulation") \
    if os.environ.get("USCT_REFERENCE") else ""


@pytest.mark.skipif(not REF or not os.path.isdir(REF),
                    reason="USCT_REFERENCE does not name the reference checkout")
def test_reference_dataset_objects_round_trip(tmp_path):
    """The reference's own Dataset and ArrayGeometry (built by its
    constructors) go through both file layouts, and the readers hand back the
    reference's classes."""
    import sys
    sys.path.insert(0, REF)
    from ringfwi.dataset import ArrayGeometry as RG, Dataset as RD
    rng = np.random.default_rng(4)
    geom = RG.cylinder(2, 6, 0.012, 0.010, 0.3e6)
    ds = RD(geometry=geom, data=rng.standard_normal((4, 50, 12)), sample_rate_hz=5e6,
            tx_wavelet=rng.standard_normal(50), tx_centre_freq_hz=0.3e6, nominal_speed_m_s=1480.0,
            tx_elements=[0, 4, 8, 11], ground_truth={"c": rng.standard_normal((9, 9, 9)),
                                                     "h_m": 2e-3},
            metadata={"description": "ref objects"})
    p = str(tmp_path / "ref.h5")
    dataset_io.save(ds, p)
    got = dataset_io.load(p)
    assert type(got) is RD and type(got.geometry) is RG
    assert np.array_equal(got.data, ds.data.astype(np.float32))
    assert np.array_equal(got.geometry.element_pos, geom.element_pos)
    assert got.geometry.array_type == "cylinder" and got.geometry.dim == 3
    assert list(got.tx_elements) == [0, 4, 8, 11]
    assert got.metadata["description"] == "ref objects" and got.metadata["created_by"] == "OpenUSCT"
    q = str(tmp_path / "ref_udsp.h5")
    dataset_io.to_uarp_set(ds, q)
    back = dataset_io.from_uarp_set(q)
    assert type(back) is RD and list(back.tx_elements) == [0, 4, 8, 11]
    assert np.array_equal(back.data, ds.data.astype(np.float32))


def test_reader_takes_structures_the_writer_does_not_emit(tmp_path):
    """A file built byte by byte from the format's structures that newer
    writers use: superblock version 2; version-2 object headers whose link
    messages make a compact group; a compact layout; version-3 attribute and
    version-2 dataspace messages; a version-1 header continued in a second
    block; a chunked dataset through shuffle + deflate (version-2 filter
    pipeline) with a partial last chunk."""
    import zlib
    buf = bytearray(48)

    def put(data):
        while len(buf) % 8:
            buf.append(0)
        a = len(buf)
        buf.extend(data)
        return a

    class Sink:                  # hdf5._btree's allocator over this buffer
        alloc = staticmethod(put)

        @staticmethod
        def patch(a, d):
            buf[a:a + len(d)] = d

    def ohdr2(msgs):
        body = b"".join(struct.pack("<BHB", t, len(m), 0) + m for t, m in msgs)
        return b"OHDR" + bytes([2, 0x02]) + struct.pack("<I", len(body)) + body + b"\0" * 4

    def ohdr1(msgs, n_total):
        body = b"".join(struct.pack("<HHB3x", t, len(hdf5._pad8(m)), 0) + hdf5._pad8(m)
                        for t, m in msgs)
        return struct.pack("<BBHII4x", 1, 0, n_total, 1, len(body)) + body, body

    def space2(shape):
        return struct.pack("<BBBB", 2, len(shape), 0, 1) + b"".join(struct.pack("<Q", s)
                                                                      for s in shape)

    def attr3(name, dt, sp, data):
        nm = name.encode() + b"\0"
        return struct.pack("<BBHHHB", 3, 0, len(nm), len(dt), len(sp), 0) + nm + dt + sp + data

    f4, f8, i2, i8 = (hdf5._dtype_message(np.dtype(t)) for t in ("<f4", "<f8", "<i2", "<i8"))
    a = np.arange(6, dtype=np.float32).reshape(2, 3) / 7
    compact = put(ohdr2([
        (0x01, space2(a.shape)), (0x03, f4),
        (0x08, struct.pack("<BBH", 3, 0, a.nbytes) + a.tobytes()),
        (0x0C, attr3("units", hdf5._dtype_message(np.dtype("S3")), space2(()), b"m/s")),
        (0x0C, attr3("n", i8, space2(()), struct.pack("<q", 7)))]))
    b = np.linspace(0, 1, 4)
    data_b = put(b.tobytes())
    cont_msgs = [(0x03, f8), (0x08, struct.pack("<BBQQ", 3, 1, data_b, b.nbytes)),
                 (0x0C, hdf5._attr_message("scale", 2.5, None))]
    _, cont_body = ohdr1(cont_msgs, 0)
    cont = put(cont_body)
    continued, _ = ohdr1([(0x01, hdf5._space_message(b.shape)),
                          (0x10, struct.pack("<QQ", cont, len(cont_body)))], 5)
    continued = put(continued)
    c = (np.arange(10, dtype=np.int16) * 1000 - 4321)
    children, keys = [], []
    for i in range(3):
        part = np.zeros(4, np.int16)
        seg = c[4 * i:4 * i + 4]
        part[:len(seg)] = seg
        shuffled = np.frombuffer(part.tobytes(), np.uint8).reshape(-1, 2).T.tobytes()
        blob = zlib.compress(shuffled, 6)
        children.append(put(blob))
        keys.append(struct.pack("<II", len(blob), 0) + struct.pack("<QQ", 4 * i, 0))
    keys.append(struct.pack("<II", 0, 0) + struct.pack("<QQ", 12, 2))
    bt = hdf5._btree(Sink, 1, children, keys, 24, 32)
    pipeline = (struct.pack("<BB", 2, 2) + struct.pack("<HHH", 2, 0, 1) + struct.pack("<I", 2) +
                struct.pack("<HHH", 1, 0, 1) + struct.pack("<I", 6))
    chunked = put(ohdr2([(0x01, space2(c.shape)), (0x03, i2),
                         (0x08, struct.pack("<BBBQ", 3, 2, 2, bt) + struct.pack("<2I", 4, 2)),
                         (0x0B, pipeline)]))

    def link(name, addr):
        nm = name.encode()
        return struct.pack("<BBB", 1, 0, len(nm)) + nm + struct.pack("<Q", addr)

    root = put(ohdr2([(0x06, link("compact", compact)), (0x06, link("continued", continued)),
                      (0x06, link("chunked", chunked)),
                      (0x0C, attr3("title", hdf5._dtype_message(np.dtype("S4")), space2(()),
                                   b"demo"))]))
    while len(buf) % 8:
        buf.append(0)
    buf[:48] = (hdf5.SIGNATURE + struct.pack("<BBBB", 2, 8, 8, 0) +
                struct.pack("<QQQQ", 0, hdf5.UNDEF, len(buf), root) + b"\0" * 4)
    path = tmp_path / "newer.h5"
    path.write_bytes(bytes(buf))
    with hdf5.File(str(path), "r") as f:
        assert f.keys() == ["chunked", "compact", "continued"]
        assert f.attrs["title"] == b"demo"
        assert np.array_equal(f["compact"][()], a)
        assert f["compact"].attrs["units"] == b"m/s" and f["compact"].attrs["n"] == 7
        assert np.array_equal(f["continued"][()], b)
        assert f["continued"].attrs["scale"] == 2.5
        got = f["chunked"][()]
        assert got.dtype == np.int16 and np.array_equal(got, c)
        assert f["chunked"].chunks == (4,) and f["chunked"].compression == "gzip"


def _library_file():
    """A file the HDF5 library itself wrote: scipy's MATLAB 7.4 v7.3-format
    test file (an HDF5 file behind a 512-byte user block)."""
    try:
        import scipy.io.matlab as sm
    except ImportError:
        return None
    p = os.path.join(os.path.dirname(sm.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
    return p if os.path.exists(p) else None


@pytest.mark.skipif(_library_file() is None, reason="no HDF5 file written by the HDF5 library here")
def test_a_file_the_hdf5_library_wrote():
    """The reader takes a file written by the HDF5 library (user block,
    superblock 0, symbol-table root, version-2 layout, fill-value,
    modification-time and NIL messages), and the writer's FP64 datatype and
    dataspace messages are byte-identical to the library's; its version-1
    attribute message differs only in the fixed-length string padding
    (null-padded, as h5py writes NumPy bytes, where the file is
    null-terminated)."""
    path = _library_file()
    with hdf5.File(path, "r") as f:
        assert f.keys() == ["testdouble"]
        ds = f["testdouble"]
        assert ds.shape == (9, 1) and ds.dtype == np.float64
        assert np.allclose(ds[()][:, 0], np.arange(9) * np.pi / 4, rtol=1e-15, atol=0)
        assert ds.attrs["MATLAB_class"] == b"double"
    r = hdf5._Reader(path)
    try:
        msgs = {t: bytes(b) for t, b, _ in r.messages(r.links(r.root)["testdouble"])}
        assert msgs[0x03] == hdf5._pad8(hdf5._dtype_message(np.dtype("<f8")))
        assert msgs[0x01] == hdf5._space_message((9, 1))
        ours = hdf5._pad8(hdf5._attr_message("MATLAB_class", b"double", None))
        assert len(ours) == len(msgs[0x0C])
        diff = [i for i in range(len(ours)) if ours[i] != msgs[0x0C][i]]
        assert diff == [25]                  # the string datatype's padding-type bits
        assert msgs[0x0C][25] == 0x00 and ours[25] == 0x01
        # the group structures follow the conventions the writer uses: B-tree
        # key 0 is the empty name (heap offset 0) and key 1 the child's last
        # name; the heap starts with the empty string, names are 8-byte padded,
        # and a free list ends with the offset the writer stores for "none"
        stab = {t: bytes(b) for t, b, _ in r.messages(r.root)}[0x11]
        bt, heap = (int.from_bytes(stab[i:i + 8], "little") + r.sb_base for i in (0, 8))
        key0, child, key1 = struct.unpack("<QQQ", bytes(r.b[bt + 24:bt + 48]))
        child += r.sb_base                    # file addresses are relative to the superblock
        assert bytes(r.b[bt:bt + 4]) == b"TREE" and key0 == 0
        assert bytes(r.b[child:child + 4]) == b"SNOD"
        seg = r.addr(heap + 24)
        assert bytes(r.b[seg:seg + 8]) == b"\0" * 8 and r._heap_name(heap, key1) == "testdouble"
        assert key1 == 8 and r._heap_name(heap, 8) == "testdouble"
        free = int.from_bytes(bytes(r.b[heap + 16:heap + 24]), "little")
        assert int.from_bytes(bytes(r.b[seg + free:seg + free + 8]), "little") == \
            hdf5._HEAP_FREE_NULL
    finally:
        r.close()
