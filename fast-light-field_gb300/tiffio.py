"""Minimal baseline-TIFF reader and writer for light-field images and volumes.

The reference reads camera images with ``tifffile.imread`` and writes
deconvolved stacks with ``tifffile.imsave`` (lfimage.py:4-20,
deconvolve_time_series.py:36).  tifffile is not available here, so this
module reads the TIFF 6.0 features light-field microscopy images use and
writes plain stacks that any TIFF reader opens:

* read: little/big endian, one or more pages (stacked into [pages, Y, X]
  when they share a shape), 1 sample per pixel, 8/16/32/64-bit unsigned,
  signed or float samples, strips or tiles, compression none, PackBits,
  LZW or Deflate, with or without the horizontal-differencing predictor;
* write: little endian, one page per leading index of a 2-D or 3-D array,
  one uncompressed strip per page, any of the sample types above.
"""

import struct
import zlib

import numpy as np

_TYPES = {1: ("B", 1), 2: ("s", 1), 3: ("H", 2), 4: ("I", 4), 5: ("II", 8), 6: ("b", 1), 7: ("B", 1),
          8: ("h", 2), 9: ("i", 4), 10: ("ii", 8), 11: ("f", 4), 12: ("d", 8), 16: ("Q", 8)}


class TiffError(ValueError):
    """The file is not a TIFF this reader supports."""


def _read_ifd(buf, bo, off):
    (n,) = struct.unpack_from(bo + "H", buf, off)
    tags = {}
    for i in range(n):
        tag, typ, cnt = struct.unpack_from(bo + "HHI", buf, off + 2 + 12 * i)
        if typ not in _TYPES:
            continue
        code, size = _TYPES[typ]
        nbytes = size * cnt
        voff = off + 2 + 12 * i + 8
        if nbytes > 4:
            (voff,) = struct.unpack_from(bo + "I", buf, voff)
        if typ == 2:
            tags[tag] = buf[voff:voff + cnt].split(b"\0", 1)[0].decode("latin-1")
        else:
            vals = struct.unpack_from(bo + code[0] * (cnt * len(code)), buf, voff)
            tags[tag] = vals
    (nxt,) = struct.unpack_from(bo + "I", buf, off + 2 + 12 * n)
    return tags, nxt


def _packbits(data):
    out = bytearray()
    i, n = 0, len(data)
    while i < n:
        h = data[i]
        i += 1
        if h < 128:
            out += data[i:i + h + 1]
            i += h + 1
        elif h > 128:
            out += bytes([data[i]]) * (257 - h)
            i += 1
    return bytes(out)


def _lzw(data):
    """TIFF LZW (MSB-first codes, 9..12 bits, 256 = clear, 257 = end)."""
    out = bytearray()
    table = [bytes([i]) for i in range(256)] + [b"", b""]
    width, pos, prev = 9, 0, None
    nbits = len(data) * 8
    while pos + width <= nbits:
        byte = pos >> 3
        chunk = int.from_bytes(data[byte:byte + 3].ljust(3, b"\0"), "big")
        code = (chunk >> (24 - width - (pos & 7))) & ((1 << width) - 1)
        pos += width
        if code == 257:
            break
        if code == 256:
            table = table[:258]
            width, prev = 9, None
            continue
        if prev is None:
            entry = table[code]
        elif code < len(table):
            entry = table[code]
            table.append(prev + entry[:1])
        else:
            entry = prev + prev[:1]
            table.append(entry)
        out += entry
        prev = entry
        # the writer switches one code early (TIFF 6.0 LZW)
        if len(table) + 1 >= (1 << width) and width < 12:
            width += 1
    return bytes(out)


def _decode(data, compression):
    if compression == 1:
        return data
    if compression == 32773:
        return _packbits(data)
    if compression == 5:
        return _lzw(data)
    if compression in (8, 32946):
        return zlib.decompress(data)
    raise TiffError("unsupported TIFF compression %d" % compression)


def _page(buf, bo, tags):
    def one(tag, default=None):
        v = tags.get(tag)
        if v is None:
            if default is None:
                raise TiffError("TIFF tag %d missing" % tag)
            return default
        return v[0]

    W, H = one(256), one(257)
    bits = tags.get(258, (1,))[0]
    spp = one(277, 1)
    if spp != 1:
        raise TiffError("only single-sample (greyscale) TIFF images are supported")
    fmt = one(339, 1)
    kind = {1: "u", 2: "i", 3: "f"}.get(fmt)
    if kind is None or bits not in (8, 16, 32, 64) or (kind == "f" and bits < 32):
        raise TiffError("unsupported TIFF sample format %d / %d bits" % (fmt, bits))
    dt = np.dtype(("<" if bo == "<" else ">") + kind + str(bits // 8))
    comp = one(259, 1)
    pred = one(317, 1)
    if 322 in tags:   # tiles
        tw, th = one(322), one(323)
        offs, cnts = tags[324], tags[325]
        img = np.zeros((-(-H // th) * th, -(-W // tw) * tw), dt)
        per_row = -(-W // tw)
        for k, (o, c) in enumerate(zip(offs, cnts)):
            t = np.frombuffer(_decode(buf[o:o + c], comp), dt, count=tw * th).reshape(th, tw)
            if pred == 2:
                t = np.cumsum(t, axis=1, dtype=dt)
            r, q = divmod(k, per_row)
            img[r * th:(r + 1) * th, q * tw:(q + 1) * tw] = t
        img = img[:H, :W]
    else:
        rps = min(one(278, H), H)
        offs, cnts = tags[273], tags[279] if 279 in tags else (W * H * dt.itemsize,)
        rows = []
        for k, (o, c) in enumerate(zip(offs, cnts)):
            nr = min(rps, H - k * rps)
            s = np.frombuffer(_decode(buf[o:o + c], comp), dt, count=nr * W).reshape(nr, W)
            if pred == 2:
                s = np.cumsum(s, axis=1, dtype=dt)
            rows.append(s)
        img = np.concatenate(rows, axis=0)
    return np.ascontiguousarray(img.astype(dt.newbyteorder("=")))


def imread(path):
    """Read a TIFF file: [Y, X] for one page, [pages, Y, X] for several of one shape."""
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:2] == b"II":
        bo = "<"
    elif buf[:2] == b"MM":
        bo = ">"
    else:
        raise TiffError("%s is not a TIFF file" % path)
    (magic,) = struct.unpack_from(bo + "H", buf, 2)
    if magic != 42:
        raise TiffError("%s: unsupported TIFF variant (magic %d)" % (path, magic))
    (off,) = struct.unpack_from(bo + "I", buf, 4)
    pages = []
    while off:
        tags, off = _read_ifd(buf, bo, off)
        if tags.get(254, (0,))[0] & 1:   # reduced-resolution thumbnail
            continue
        pages.append(_page(buf, bo, tags))
    if not pages:
        raise TiffError("%s holds no image" % path)
    if len(pages) == 1:
        return pages[0]
    if any(p.shape != pages[0].shape for p in pages):
        raise TiffError("%s: pages differ in shape" % path)
    return np.stack(pages)


def imshape(path):
    """Shape imread would return, from the first page's header only ([Y, X] or [pages, Y, X])."""
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:2] not in (b"II", b"MM"):
        raise TiffError("%s is not a TIFF file" % path)
    bo = "<" if buf[:2] == b"II" else ">"
    (off,) = struct.unpack_from(bo + "I", buf, 4)
    shape, pages = None, 0
    while off:
        tags, off = _read_ifd(buf, bo, off)
        if tags.get(254, (0,))[0] & 1:
            continue
        shape = shape or (tags[257][0], tags[256][0])
        pages += 1
    if shape is None:
        raise TiffError("%s holds no image" % path)
    return shape if pages == 1 else (pages,) + shape


def imwrite(path, data):
    """Write a 2-D array as one page or a 3-D array [pages, Y, X] as a multi-page TIFF."""
    a = np.asarray(data)
    if a.ndim == 2:
        a = a[np.newaxis]
    if a.ndim != 3:
        raise TiffError("imwrite takes a 2-D image or a 3-D stack, got shape %s" % (a.shape,))
    a = np.ascontiguousarray(a, dtype=a.dtype.newbyteorder("<"))
    kind = {"u": 1, "i": 2, "f": 3}.get(a.dtype.kind)
    if kind is None or a.dtype.itemsize not in (1, 2, 4, 8):
        raise TiffError("unsupported sample type %s" % a.dtype)
    P, H, W = a.shape
    page_bytes = H * W * a.itemsize
    ntags = 11
    ifd_size = 2 + 12 * ntags + 4
    if 8 + P * (ifd_size + page_bytes) >= 1 << 32:
        raise TiffError("stack too large for a classic TIFF (4 GiB)")
    out = bytearray(b"II" + struct.pack("<HI", 42, 8))
    pos = 8
    for p in range(P):
        data_off = pos + ifd_size
        nxt = data_off + page_bytes if p + 1 < P else 0
        entries = [(256, 4, 1, W), (257, 4, 1, H), (258, 3, 1, a.itemsize * 8), (259, 3, 1, 1),
                   (262, 3, 1, 1), (273, 4, 1, data_off), (277, 3, 1, 1), (278, 4, 1, H),
                   (279, 4, 1, page_bytes), (284, 3, 1, 1), (339, 3, 1, kind)]
        out += struct.pack("<H", ntags)
        for tag, typ, cnt, val in entries:
            out += struct.pack("<HHI", tag, typ, cnt)
            out += struct.pack("<HH", val, 0) if typ == 3 else struct.pack("<I", val)
        out += struct.pack("<I", nxt)
        out += a[p].tobytes()
        pos = nxt
    with open(path, "wb") as f:
        f.write(bytes(out))
