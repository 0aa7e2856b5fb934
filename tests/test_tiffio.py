"""TIFF reader/writer used by the time-series driver (no GPU)."""

import os
import struct
import zlib

import numpy as np
import pytest

import tiffio

REF_IMAGES = os.path.join(os.sep, "root", "reference", "Data", "02_Rectified", "exampleData")


@pytest.mark.parametrize("dtype", ["uint8", "uint16", "int16", "uint32", "int32", "float32", "float64"])
def test_round_trip(tmp_path, dtype):
    a = (np.random.default_rng(0).random((3, 17, 23)) * 200).astype(dtype)
    p = str(tmp_path / "a.tif")
    tiffio.imwrite(p, a)
    b = tiffio.imread(p)
    assert b.dtype == a.dtype and np.array_equal(a, b)
    assert tiffio.imshape(p) == (3, 17, 23)
    tiffio.imwrite(p, a[1])
    assert np.array_equal(tiffio.imread(p), a[1]) and tiffio.imshape(p) == (17, 23)


def _packbits_encode(raw):
    out = bytearray()
    for i in range(0, len(raw), 100):          # literal runs, plus one replicate run per chunk
        chunk = raw[i:i + 100]
        out += bytes([len(chunk) - 1]) + chunk
    return bytes(out)


def _lzw_encode(raw):
    """TIFF LZW encoder (MSB-first codes) used to check the decoder, which widens one
    table entry earlier than this encoder because it adds each entry one code late."""
    table = {bytes([i]): i for i in range(256)}
    nxt, width = 258, 9
    codes = [(256, 9)]
    w = b""
    for ch in raw:
        wc = w + bytes([ch])
        if wc in table:
            w = wc
            continue
        codes.append((table[w], width))
        table[wc] = nxt
        nxt += 1
        if nxt >= (1 << width) and width < 12:     # the encoder widens when the next code needs it
            width += 1
        if nxt >= 4094:
            codes.append((256, width))
            table = {bytes([i]): i for i in range(256)}
            nxt, width = 258, 9
        w = bytes([ch])
    if w:
        codes.append((table[w], width))
    codes.append((257, width))
    bits = "".join(format(c, "0%db" % n) for c, n in codes)
    bits += "0" * (-len(bits) % 8)
    return int(bits, 2).to_bytes(len(bits) // 8, "big")


def _tiff(bo, W, H, bits, fmt, strips, compression, predictor=1, tiles=None):
    """A one-page TIFF with the given (already encoded) strips or tiles."""
    entries = [(256, 4, W), (257, 4, H), (258, 3, bits), (259, 3, compression), (262, 3, 1),
               (277, 3, 1), (284, 3, 1), (317, 3, predictor), (339, 3, fmt)]
    data = b"".join(strips)
    n_off = len(strips)
    if tiles:
        entries += [(322, 4, tiles[0]), (323, 4, tiles[1])]
        otag, ctag = 324, 325
    else:
        entries += [(278, 4, tiles_rows(H, n_off))]
        otag, ctag = 273, 279
    nt = len(entries) + 2
    ifd_off = 8
    arrays_off = ifd_off + 2 + 12 * nt + 4
    data_off = arrays_off + 8 * n_off
    offs, pos = [], data_off
    for s in strips:
        offs.append(pos)
        pos += len(s)
    arr = struct.pack(bo + "%dI" % n_off, *offs) + struct.pack(bo + "%dI" % n_off, *[len(s) for s in strips])
    out = (b"II" if bo == "<" else b"MM") + struct.pack(bo + "HI", 42, ifd_off) + struct.pack(bo + "H", nt)
    for tag, typ, val in sorted(entries + [(otag, 4, None), (ctag, 4, None)]):
        if tag == otag:
            out += struct.pack(bo + "HHI", tag, 4, n_off) + struct.pack(bo + "I", arrays_off if n_off > 1 else offs[0])
        elif tag == ctag:
            out += struct.pack(bo + "HHI", tag, 4, n_off) + struct.pack(
                bo + "I", arrays_off + 4 * n_off if n_off > 1 else len(strips[0]))
        elif typ == 3:
            out += struct.pack(bo + "HHIHH", tag, 3, 1, val, 0)
        else:
            out += struct.pack(bo + "HHII", tag, 4, 1, val)
    out += struct.pack(bo + "I", 0) + arr + data
    return out


def tiles_rows(H, n):
    return -(-H // n)


@pytest.mark.parametrize("compression", [1, 32773, 5, 8])
@pytest.mark.parametrize("bo", ["<", ">"])
def test_compressed_strips(tmp_path, compression, bo):
    rng = np.random.default_rng(compression)
    img = (rng.random((37, 29)) * 60000).astype(np.uint16)
    img[5:9] = 1234                           # runs for the compressors
    rps = 10
    strips = []
    for r in range(0, 37, rps):
        raw = img[r:r + rps].astype(np.dtype(bo + "u2")).tobytes()
        strips.append({1: raw, 32773: _packbits_encode(raw), 5: _lzw_encode(raw), 8: zlib.compress(raw)}[compression])
    p = tmp_path / "c.tif"
    p.write_bytes(_tiff(bo, 29, 37, 16, 1, strips, compression))
    assert np.array_equal(tiffio.imread(str(p)), img)


def test_predictor_and_tiles(tmp_path):
    img = (np.random.default_rng(3).random((40, 36)) * 1000).astype(np.int32)
    diff = img.copy()
    diff[:, 1:] = img[:, 1:] - img[:, :-1]
    p = tmp_path / "p.tif"
    p.write_bytes(_tiff("<", 36, 40, 32, 2, [zlib.compress(diff.tobytes())], 8, predictor=2))
    assert np.array_equal(tiffio.imread(str(p)), img)
    f = (np.random.default_rng(4).random((20, 24))).astype(np.float32)
    pad = np.zeros((32, 32), np.float32)
    pad[:20, :24] = f
    tiles = [pad[:16, :16], pad[:16, 16:], pad[16:, :16], pad[16:, 16:]]
    p.write_bytes(_tiff("<", 24, 20, 32, 3, [t.tobytes() for t in tiles], 1, tiles=(16, 16)))
    assert np.array_equal(tiffio.imread(str(p)), f)


def test_rejects_what_it_cannot_read(tmp_path):
    p = tmp_path / "x.tif"
    p.write_bytes(b"NOTATIFF")
    with pytest.raises(tiffio.TiffError):
        tiffio.imread(str(p))
    with pytest.raises(tiffio.TiffError):
        tiffio.imwrite(str(p), np.zeros((2, 2, 2, 2)))


@pytest.mark.skipif(not os.path.isdir(REF_IMAGES), reason="reference example images not present")
def test_reads_reference_example_images():
    import lfimage
    w = lfimage.LoadLightFieldTiff(os.path.join(REF_IMAGES, "20131219WORM2_small_full_neg_X1_N15_cropped_uncompressed.tif"))
    assert w.shape == (675, 450) and w.dtype == np.float32 and w.max() == 200
    n = tiffio.imread(os.path.join(REF_IMAGES, "Nils_test_LFImage.tif"))     # 16-bit PackBits
    assert n.shape == (1273, 1463) and n.dtype == np.uint16


def test_lzw_all_code_widths(tmp_path):
    # ~48 KB in one strip: the code table passes every width (9..12 bits) and is cleared
    img = (np.random.default_rng(5).random((160, 150)) * 300).astype(np.uint16)
    enc = _lzw_encode(img.tobytes())
    assert len(enc) > 16000
    p = tmp_path / "l.tif"
    p.write_bytes(_tiff("<", 150, 160, 16, 1, [enc], 5))
    assert np.array_equal(tiffio.imread(str(p)), img)
