"""hdf5lite: the HDF5 subset of the PSF .mat files, without h5py.

No HDF5 library exists on either machine, so these tests check the reader on
files laid out by hand from the published file-format specification (chunked
storage with deflate and shuffle, a user block, version-2 object headers with
link messages) and on files of the module's own writer, and the PSF .mat round
trip SaveRawMatrixData -> LoadRawMatrixData (the reference's key names, its
transposed CAindex and its [Z][nh][nh][L][L] arrays)."""

import os
import struct
import zlib

import numpy as np
import pytest

import hdf5lite

UNDEF = 0xFFFFFFFFFFFFFFFF


def _pad8(b):
    return b + bytes((-len(b)) % 8)


class _Builder:
    """Append-only byte buffer with 8-byte aligned allocations."""

    def __init__(self):
        self.b = bytearray()

    def put(self, data):
        while len(self.b) % 8:
            self.b.append(0)
        a = len(self.b)
        self.b += data
        return a


def _msg_v1(t, data, flags=0):
    data = _pad8(data)
    return struct.pack("<HHB3x", t, len(data), flags) + data


def _ohdr_v1(msgs):
    body = b"".join(msgs)
    return struct.pack("<BBHII", 1, 0, len(msgs), 1, len(body)) + bytes(4) + body


def _f32_type():
    return bytes([0x11, 0x20, 31, 0]) + struct.pack("<I", 4) + struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)


def _old_style_file(dsets, prefix=b""):
    """Superblock v0 + root group (symbol table) over the given {name: object header bytes
    builder(f)} entries; each builder gets the buffer and returns its header address."""
    f = _Builder()
    f.put(bytes(96))
    names = sorted(dsets)
    heap = bytearray(bytes(8))
    off = {}
    for n in names:
        off[n] = len(heap)
        heap += _pad8(n.encode() + b"\x00")
    seg = f.put(bytes(heap))
    hh = f.put(struct.pack("<4sB3xQQQ", b"HEAP", 0, len(heap), UNDEF, seg))
    addr = {n: dsets[n](f) for n in names}
    snod = f.put(struct.pack("<4sBBH", b"SNOD", 1, 0, len(names)) +
                 b"".join(struct.pack("<QQII16x", off[n], addr[n], 0, 0) for n in names) + bytes(40 * 8))
    tree = f.put(struct.pack("<4sBBHQQ", b"TREE", 0, 0, 1, UNDEF, UNDEF) + struct.pack("<QQQ", 0, snod, off[names[-1]])
                 + bytes(8 * 64))
    root = f.put(_ohdr_v1([_msg_v1(0x11, struct.pack("<QQ", tree, hh))]))
    sb = bytearray(b"\x89HDF\r\n\x1a\n" + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 16, 16, 0))
    sb += struct.pack("<QQQQ", 0, UNDEF, len(f.b), UNDEF) + struct.pack("<QQII", 0, root, 1, 0) + struct.pack("<QQ", tree, hh)
    f.b[0:96] = sb
    return prefix + bytes(f.b)


def test_round_trip_of_own_writer(tmp_path):
    d = {"Nnum": np.int64(15), "M": 40.0, "lambda": 5.2e-7, "ReducedMatrix": True,
         "CAindex": np.array([[1, 5], [3, 9], [2, 8]], np.int64),
         "H": np.random.default_rng(0).random((2, 3, 4, 5, 6)).astype(np.float32),
         "x3objspace": np.array([-1e-5, 0.0, 1e-5]), "i8": np.arange(-3, 4, dtype=np.int8),
         "u16": np.arange(7, dtype=">u2"), "empty": np.zeros((0, 3), np.float32)}
    p = str(tmp_path / "t.mat")
    hdf5lite.write(p, d)
    with hdf5lite.File(p) as f:
        assert sorted(f.keys()) == sorted(d)
        for k, v in d.items():
            r = f[k]
            v = np.asarray(v)
            assert r.shape == v.shape and r.dtype == v.dtype.newbyteorder("=") and np.array_equal(r, v), k
        with pytest.raises(KeyError):
            f.read("missing")


def test_user_block_and_chunked_deflate_shuffle(tmp_path):
    rng = np.random.default_rng(1)
    a = rng.random((5, 7)).astype(np.float32)
    chunk = (2, 3)

    def chunked(f):
        # chunks of 2 x 3 (edge chunks padded), each shuffled then deflated
        entries = []
        for i in range(0, 5, 2):
            for j in range(0, 7, 3):
                c = np.zeros(chunk, np.float32)
                blk = a[i:i + 2, j:j + 3]
                c[:blk.shape[0], :blk.shape[1]] = blk
                raw = np.frombuffer(c.tobytes(), np.uint8).reshape(-1, 4).T.tobytes()   # shuffle
                comp = zlib.compress(raw)
                entries.append(((i, j), f.put(comp), len(comp)))
        keys = b""
        for (i, j), addr, n in entries:
            keys += struct.pack("<II", n, 0) + struct.pack("<QQQ", i, j, 0) + struct.pack("<Q", addr)
        keys += struct.pack("<II", 0, 0) + struct.pack("<QQQ", 5, 7, 0)
        tree = f.put(struct.pack("<4sBBHQQ", b"TREE", 1, 0, len(entries), UNDEF, UNDEF) + keys)
        space = bytes([1, 2, 0, 0, 0, 0, 0, 0]) + struct.pack("<QQ", 5, 7)
        # filter pipeline v1: shuffle (2, element size), deflate (1, level 4)
        filt = bytes([1, 2, 0, 0, 0, 0, 0, 0])
        filt += struct.pack("<HHHH", 2, 0, 1, 1) + struct.pack("<I", 4) + bytes(4)
        filt += struct.pack("<HHHH", 1, 0, 1, 1) + struct.pack("<I", 4) + bytes(4)
        layout = bytes([3, 2, 3]) + struct.pack("<Q", tree) + struct.pack("<III", 2, 3, 4)
        return f.put(_ohdr_v1([_msg_v1(1, space), _msg_v1(3, _f32_type(), 1), _msg_v1(0x0B, filt),
                               _msg_v1(8, layout)]))

    def compact(f):
        v = np.arange(4, dtype=np.float32)
        layout = bytes([3, 0]) + struct.pack("<H", v.nbytes) + v.tobytes()
        space = bytes([1, 1, 0, 0, 0, 0, 0, 0]) + struct.pack("<Q", 4)
        return f.put(_ohdr_v1([_msg_v1(1, space), _msg_v1(3, _f32_type(), 1), _msg_v1(8, layout)]))

    p = str(tmp_path / "c.mat")
    with open(p, "wb") as fh:
        fh.write(_old_style_file({"A": chunked, "B": compact}, prefix=b"MATLAB 7.3 MAT-file".ljust(512, b" ")))
    with hdf5lite.File(p) as f:
        assert np.array_equal(f["A"], a)
        assert np.array_equal(f["B"], np.arange(4, dtype=np.float32))


def test_version2_object_headers_and_link_messages(tmp_path):
    f = _Builder()
    f.put(bytes(48))
    v = np.array([[1.5, -2.0]], np.float64)
    data = f.put(v.tobytes())

    def ohdr2(msgs):
        body = b"".join(bytes([t]) + struct.pack("<H", len(m)) + bytes([0]) + m for t, m in msgs)
        return b"OHDR" + bytes([2, 0x02]) + struct.pack("<I", len(body)) + body + bytes(4)

    f64 = bytes([0x11, 0x20, 63, 0]) + struct.pack("<I", 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
    space = bytes([2, 2, 0, 1]) + struct.pack("<QQ", 1, 2)
    layout = bytes([3, 1]) + struct.pack("<QQ", data, v.nbytes)
    ds = f.put(ohdr2([(1, space), (3, f64), (8, layout)]))
    name = b"zspacing"
    link = bytes([1, 0x00, len(name)]) + name + struct.pack("<Q", ds)
    root = f.put(ohdr2([(6, link)]))
    sb = b"\x89HDF\r\n\x1a\n" + bytes([2, 8, 8, 0]) + struct.pack("<QQQQ", 0, UNDEF, len(f.b), root) + bytes(4)
    f.b[0:len(sb)] = sb
    p = str(tmp_path / "v2.h5")
    with open(p, "wb") as fh:
        fh.write(bytes(f.b))
    with hdf5lite.File(p) as h:
        assert h.keys() == ["zspacing"]
        assert np.array_equal(h["zspacing"], v)


def test_not_hdf5(tmp_path):
    p = str(tmp_path / "x.mat")
    with open(p, "wb") as fh:
        fh.write(b"MATLAB 5.0 MAT-file" + bytes(2000))
    with pytest.raises(hdf5lite.HDF5Error):
        hdf5lite.File(p)


def test_psf_mat_round_trip(tmp_path):
    """SaveRawMatrixData writes the reference's .mat layout; LoadRawMatrixData (the
    reference's reading code path, psfmatrix.py:100-167) gives back the quadrants."""
    import psfmatrix
    import synthetic
    N = 5
    H, Ht = synthetic.synthetic_psf(N, [-10, 0, 10], 2)
    hs = [h.shape[-1] for h in H]
    L = max(hs)
    c = (L + 1) // 2
    CA = np.array([[c - (h - 1) // 2 for h in hs], [c + (h - 1) // 2 for h in hs]])
    mat = str(tmp_path / "fdnormPSFmatrix_test.mat")
    psfmatrix.SaveRawMatrixData(mat, H, Ht, CA, {"Nnum": N, "M": 40.0, "lambda": 5.2e-7})
    with hdf5lite.File(mat) as f:
        assert f["CAindex"].shape == (3, 2) and bool(f["ReducedMatrix"]) and int(f["Nnum"]) == N
        assert f["H"].shape == (3, (N + 1) // 2, (N + 1) // 2, L, L)
    Hq, Htq, CA2, _, _, hshape, _ = psfmatrix.LoadRawMatrixData(mat, expectedNnum=N, createPSF=False)
    assert np.array_equal(CA2, CA)
    for a, b in zip(Hq + Htq, list(H) + list(Ht)):
        assert np.array_equal(a, b)
    hm = psfmatrix.LoadMatrix(mat)
    assert hm.numZ == 3 and os.path.isdir(os.path.splitext(mat)[0])
