"""A small HDF5 reader and writer for the PSF ``.mat`` files (MATLAB 7.3 / h5py).

The reference keeps its PSF matrices in HDF5 files written by h5py
(generate_psf.py:739-785, ``SaveMatrices``) or by MATLAB, and reads them with
h5py (psfmatrix.py:100-167, ``LoadRawMatrixData``).  h5py is not installed on
these machines, so this module reads and writes the subset of the format those
files use, from the published HDF5 file-format specification:

reading
  * superblock versions 0-3, at offset 0 or after a user block (MATLAB writes
    512 bytes of text first);
  * object headers version 1 and 2, with continuation blocks;
  * groups in the old style (symbol table: v1 B-tree of symbol-table nodes over
    a local heap) and the compact new style (link messages in the header);
  * datasets with a simple or scalar dataspace, fixed-point, floating-point or
    enum (h5py's bool) element types in either byte order, and compact,
    contiguous or chunked storage (v1 B-tree chunk index) with the deflate,
    shuffle and Fletcher-32 filters;

writing
  * superblock version 0, one root group of the old style, and contiguous
    datasets (scalars as scalar dataspaces, bool as h5py's enum), which is how
    h5py lays out ``f[name] = value`` with its default settings.

``File(path).read(name)`` returns a numpy array in the file's (C) dimension
order, as ``h5py.File(path)[name][()]`` does; ``write(path, {name: value})``
creates a file.
"""

import struct
import zlib

import numpy as np

__all__ = ["File", "write", "HDF5Error"]

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF


class HDF5Error(ValueError):
    """The file is not HDF5, or uses a part of the format this module does not read."""


# --------------------------------------------------------------------------- reading

class File:
    """Read-only view of an HDF5 file: ``keys()``, ``read(name)``, ``file[name]``."""

    def __init__(self, path, mode="r"):
        if mode != "r":
            raise ValueError("hdf5lite.File reads only; write() creates files")
        with open(path, "rb") as f:
            self._b = f.read()
        self._base = self._find_superblock()
        self._root = self._parse_superblock()
        self._links = self._group_links(self._root)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def keys(self):
        return list(self._links)

    def __contains__(self, name):
        return name in self._links

    def __getitem__(self, name):
        return self.read(name)

    def read(self, name):
        if name not in self._links:
            raise KeyError(name)
        return self._read_dataset(self._links[name])

    # -- low level
    def _u(self, off, n):
        return int.from_bytes(self._b[off:off + n], "little")

    def _find_superblock(self):
        off = 0
        while off + 8 <= len(self._b):
            if self._b[off:off + 8] == _SIG:
                return off
            off = 512 if off == 0 else off * 2
        raise HDF5Error("no HDF5 superblock found")

    def _addr(self, a):
        """A file address -> an offset into the bytes.  Addresses are relative to the
        base address, which is the superblock's own position (after any user block)."""
        return None if a == _UNDEF or a == (1 << (8 * self._so)) - 1 else self._base + a

    def _parse_superblock(self):
        b, o = self._b, self._base + 8
        ver = b[o]
        if ver in (0, 1):
            self._so, self._sl = b[o + 5], b[o + 6]
            p = o + 16 + (4 if ver == 1 else 0)
            p += 4 * self._so                     # base, free space, end of file, driver info
            # root group symbol table entry: link name offset, object header address
            return self._addr(self._u(p + self._so, self._so))
        if ver in (2, 3):
            self._so, self._sl = b[o + 1], b[o + 2]
            p = o + 4
            return self._addr(self._u(p + 3 * self._so, self._so))
        raise HDF5Error("superblock version %d is not supported" % ver)

    # object headers -> list of (type, bytes)
    def _messages(self, off):
        b = self._b
        if b[off:off + 4] == b"OHDR":
            return self._messages_v2(off)
        if b[off] != 1:
            raise HDF5Error("object header version %d at %d is not supported" % (b[off], off))
        nmsg = self._u(off + 2, 2)
        size = self._u(off + 8, 4)
        blocks = [(off + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            p, n = blocks.pop(0)
            end = p + n
            while p + 8 <= end and len(out) < nmsg:
                mtype, msize = self._u(p, 2), self._u(p + 2, 2)
                data = b[p + 8:p + 8 + msize]
                p += 8 + msize
                if mtype == 0x10:   # continuation
                    blocks.append((self._addr(int.from_bytes(data[:self._so], "little")),
                                   int.from_bytes(data[self._so:self._so + self._sl], "little")))
                out.append((mtype, data))
        return out

    def _messages_v2(self, off):
        b = self._b
        flags = b[off + 5]
        p = off + 6
        if flags & 0x20:
            p += 16
        if flags & 0x10:
            p += 4
        sz_bytes = 1 << (flags & 3)
        size = self._u(p, sz_bytes)
        p += sz_bytes
        blocks = [(p, size)]
        out = []
        tracked = bool(flags & 0x04)
        while blocks:
            p, n = blocks.pop(0)
            end = p + n
            while p + 4 <= end:
                mtype, msize, mflags = b[p], self._u(p + 1, 2), b[p + 3]
                p += 4 + (2 if tracked else 0)
                if p + msize > end:
                    break
                data = b[p:p + msize]
                p += msize
                if mtype == 0x10:
                    a = self._addr(int.from_bytes(data[:self._so], "little"))
                    ln = int.from_bytes(data[self._so:self._so + self._sl], "little")
                    if b[a:a + 4] != b"OCHK":
                        raise HDF5Error("bad object header continuation block")
                    blocks.append((a + 4, ln - 8))
                elif mtype != 0:
                    out.append((mtype, data))
        return out

    # groups
    def _group_links(self, off):
        links = {}
        for mtype, data in self._messages(off):
            if mtype == 0x11:       # symbol table: v1 B-tree of symbol-table nodes, local heap
                btree = self._addr(int.from_bytes(data[:self._so], "little"))
                heap = self._addr(int.from_bytes(data[self._so:2 * self._so], "little"))
                names = self._local_heap(heap)
                self._walk_group_btree(btree, names, links)
            elif mtype == 0x06:     # link message (compact new-style group)
                name, addr = self._link_message(data)
                if addr is not None:
                    links[name] = addr
            elif mtype == 0x02:     # link info: dense storage is not read
                fheap = int.from_bytes(data[2 + (8 if data[1] & 1 else 0):][:self._so], "little")
                if fheap != _UNDEF and fheap != (1 << (8 * self._so)) - 1:
                    raise HDF5Error("groups with dense link storage are not supported")
        return links

    def _local_heap(self, off):
        b = self._b
        if b[off:off + 4] != b"HEAP":
            raise HDF5Error("bad local heap signature")
        p = off + 8 + 2 * self._sl
        data = self._addr(self._u(p, self._so))

        def name(o):
            s = data + o
            e = b.index(b"\x00", s)
            return b[s:e].decode("utf-8")
        return name

    def _walk_group_btree(self, off, names, links):
        b = self._b
        if b[off:off + 4] != b"TREE":
            raise HDF5Error("bad group B-tree signature")
        level, used = b[off + 5], self._u(off + 6, 2)
        p = off + 8 + 2 * self._so
        for i in range(used):
            p += self._sl                                     # key: heap offset
            child = self._addr(self._u(p, self._so))
            p += self._so
            if level > 0:
                self._walk_group_btree(child, names, links)
            else:
                self._symbol_node(child, names, links)

    def _symbol_node(self, off, names, links):
        b = self._b
        if b[off:off + 4] != b"SNOD":
            raise HDF5Error("bad symbol table node signature")
        n = self._u(off + 6, 2)
        p = off + 8
        esize = 2 * self._so + 24
        for i in range(n):
            nm = names(self._u(p, self._so))
            links[nm] = self._addr(self._u(p + self._so, self._so))
            p += esize

    def _link_message(self, data):
        flags = data[1]
        p = 2
        ltype = 0
        if flags & 0x08:
            ltype = data[p]
            p += 1
        if flags & 0x04:
            p += 8
        if flags & 0x10:
            p += 1
        nlen_bytes = 1 << (flags & 3)
        nlen = int.from_bytes(data[p:p + nlen_bytes], "little")
        p += nlen_bytes
        name = data[p:p + nlen].decode("utf-8")
        p += nlen
        if ltype != 0:
            return name, None        # soft / external links are not followed
        return name, self._addr(int.from_bytes(data[p:p + self._so], "little"))

    # datasets
    def _read_dataset(self, off):
        shape = dtype = layout = enum = None
        filters = []
        for mtype, data in self._messages(off):
            if mtype == 0x01:
                shape = self._dataspace(data)
            elif mtype == 0x03:
                dtype, enum = self._datatype(data)
            elif mtype == 0x08:
                layout = data
            elif mtype == 0x0B:
                filters = self._filters(data)
        if shape is None or dtype is None or layout is None:
            raise HDF5Error("object is not a dataset")
        n = int(np.prod(shape)) if shape else 1
        raw = self._layout_data(layout, shape, dtype.itemsize, filters)
        arr = np.frombuffer(raw[:n * dtype.itemsize], dtype=dtype).reshape(shape).copy()
        if enum == "bool":
            arr = arr != 0
        return arr.astype(arr.dtype.newbyteorder("=")) if arr.dtype.byteorder not in "=|" else arr

    def _dataspace(self, d):
        ver, rank, flags = d[0], d[1], d[2]
        p = 8 if ver == 1 else 4
        if ver == 2 and d[3] == 0:     # scalar
            return ()
        return tuple(int.from_bytes(d[p + self._sl * i:p + self._sl * (i + 1)], "little") for i in range(rank))

    def _datatype(self, d):
        cls, bits0 = d[0] & 0x0F, d[1]
        size = int.from_bytes(d[4:8], "little")
        order = ">" if bits0 & 1 else "<"
        if cls == 0:
            return np.dtype("%s%s%d" % (order, "i" if bits0 & 0x08 else "u", size)), None
        if cls == 1:
            if size not in (2, 4, 8):
                raise HDF5Error("floating-point size %d is not supported" % size)
            return np.dtype("%sf%d" % (order, size)), None
        if cls == 8:                   # enum: read its base type (h5py's bool is an int8 enum)
            base, _ = self._datatype(d[8:])
            return base, "bool"
        raise HDF5Error("datatype class %d is not supported" % cls)

    def _filters(self, d):
        ver, n = d[0], d[1]
        p = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = int.from_bytes(d[p:p + 2], "little")
            if ver == 1 or fid >= 256:
                nlen = int.from_bytes(d[p + 2:p + 4], "little")
                ncv = int.from_bytes(d[p + 6:p + 8], "little")
                p += 8 + ((nlen + 7) // 8 * 8 if ver == 1 else nlen)
            else:
                ncv = int.from_bytes(d[p + 4:p + 6], "little")
                p += 6
            cv = [int.from_bytes(d[p + 4 * i:p + 4 * i + 4], "little") for i in range(ncv)]
            p += 4 * ncv + (4 if ver == 1 and ncv % 2 else 0)
            out.append((fid, cv))
        return out

    def _layout_data(self, d, shape, esize, filters):
        ver = d[0]
        if ver == 3 or ver == 4:
            cls = d[1]
            if cls == 0:
                n = int.from_bytes(d[2:4], "little")
                return d[4:4 + n]
            if cls == 1:
                a = self._addr(int.from_bytes(d[2:2 + self._so], "little"))
                n = int.from_bytes(d[2 + self._so:2 + self._so + self._sl], "little")
                if a is None:
                    return bytes(n)
                return self._b[a:a + n]
            if cls == 2 and ver == 3:
                rank = d[2]
                btree = int.from_bytes(d[3:3 + self._so], "little")
                cdims = [int.from_bytes(d[3 + self._so + 4 * i:3 + self._so + 4 * i + 4], "little")
                         for i in range(rank)]
                return self._chunked(self._addr(btree), shape, cdims[:-1], esize, filters)
        raise HDF5Error("data layout version %d class %d is not supported" % (ver, d[1] if len(d) > 1 else -1))

    def _chunked(self, btree, shape, cdims, esize, filters):
        out = np.zeros(tuple(shape) + (esize,), np.uint8)
        if btree is None:
            return out.tobytes()
        rank = len(shape)
        for offs, raw in self._chunks(btree, rank):
            for fid, cv in reversed(filters):
                if fid == 1:
                    raw = zlib.decompress(raw)
                elif fid == 2:
                    raw = np.frombuffer(raw, np.uint8).reshape(esize, -1).T.tobytes()
                elif fid == 3:
                    raw = raw[:-4]
                else:
                    raise HDF5Error("filter %d is not supported" % fid)
            chunk = np.frombuffer(raw, np.uint8)[:int(np.prod(cdims)) * esize].reshape(tuple(cdims) + (esize,))
            dst = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, shape))
            src = tuple(slice(0, sl.stop - sl.start) for sl in dst)
            out[dst] = chunk[src]
        return out.tobytes()

    def _chunks(self, off, rank):
        b = self._b
        if b[off:off + 4] != b"TREE" or b[off + 4] != 1:
            raise HDF5Error("bad chunk B-tree")
        level, used = b[off + 5], self._u(off + 6, 2)
        p = off + 8 + 2 * self._so
        ksize = 8 + 8 * (rank + 1)
        for i in range(used):
            csize = self._u(p, 4)
            offs = [self._u(p + 8 + 8 * k, 8) for k in range(rank)]
            child = self._addr(self._u(p + ksize, self._so))
            p += ksize + self._so
            if level > 0:
                yield from self._chunks(child, rank)
            else:
                yield offs, self._b[child:child + csize]


# --------------------------------------------------------------------------- writing

def _pad8(b):
    return b + bytes((-len(b)) % 8)


def _dtype_message(a):
    dt = a.dtype
    if dt == np.bool_:
        # h5py's bool: an enum of int8 with FALSE = 0, TRUE = 1
        base = _dtype_message(np.zeros((), np.int8))
        names = b"".join(_pad8(n + b"\x00") for n in (b"FALSE", b"TRUE"))
        head = bytes([0x18, 2, 0, 0]) + struct.pack("<I", 1)     # class 8, version 1, 2 members
        return head + base + names + bytes([0, 1])
    size = dt.itemsize
    if dt.kind == "f":
        prec = size * 8
        exp_size, mant_size, bias = {4: (8, 23, 127), 8: (11, 52, 1023), 2: (5, 10, 15)}[size]
        b0 = 0x20                           # little endian, mantissa normalisation: implied msb
        b1 = prec - 1                        # sign bit position
        props = struct.pack("<HHBBBBI", 0, prec, mant_size, exp_size, 0, mant_size, bias)
        return bytes([0x11, b0, b1, 0]) + struct.pack("<I", size) + props
    if dt.kind in "iu":
        b0 = 0x08 if dt.kind == "i" else 0
        return bytes([0x10, b0, 0, 0]) + struct.pack("<I", size) + struct.pack("<HH", 0, size * 8)
    raise TypeError("dtype %s is not supported" % dt)


def write(path, items):
    """Write an HDF5 file holding the numpy-convertible values of ``items`` (a
    dict name -> value) as contiguous datasets in the root group."""
    arrays = {}
    for k, v in items.items():
        a = np.asarray(v)
        if a.dtype.kind == "f" and a.dtype.itemsize not in (4, 8):
            a = a.astype(np.float64)
        if a.dtype.kind in "iu" and a.dtype.byteorder == ">":
            a = a.astype(a.dtype.newbyteorder("<"))
        arrays[k.encode("utf-8") if isinstance(k, str) else k] = a.copy(order="C")   # keeps 0-d arrays 0-d
    names = sorted(arrays)
    out = bytearray()

    def alloc(n, align=8):
        while len(out) % align:
            out.append(0)
        a = len(out)
        out.extend(bytes(n))
        return a

    so = 8
    sb = alloc(56 + 40)                       # superblock v0 with the root symbol table entry
    # local heap: "" at 0, then the names
    heap_data = bytearray(b"\x00" * 8)
    name_off = {}
    for nm in names:
        name_off[nm] = len(heap_data)
        heap_data += _pad8(nm + b"\x00")
    heap_hdr = alloc(32)
    heap_seg = alloc(len(heap_data))
    out[heap_seg:heap_seg + len(heap_data)] = heap_data
    struct.pack_into("<4sB3xQQQ", out, heap_hdr, b"HEAP", 0, len(heap_data), _UNDEF, heap_seg)   # no free list
    # datasets
    obj = {}
    for nm in names:
        a = arrays[nm]
        data_addr = alloc(max(a.nbytes, 1)) if a.nbytes else _UNDEF
        if a.nbytes:
            out[data_addr:data_addr + a.nbytes] = a.tobytes()
        if a.ndim == 0:
            space = bytes([1, 0, 0, 0, 0, 0, 0, 0])            # version 1, rank 0: scalar
        else:
            space = bytes([1, a.ndim, 0, 0, 0, 0, 0, 0]) + b"".join(struct.pack("<Q", s) for s in a.shape)
        dtype = _dtype_message(a)
        fill = bytes([2, 2, 2, 0])                             # fill value v2: late, on allocation, undefined
        layout = bytes([3, 1]) + struct.pack("<QQ", data_addr, a.nbytes)
        msgs = [(0x01, space), (0x03, dtype), (0x05, fill), (0x08, layout)]
        body = b"".join(struct.pack("<HHB3x", t, len(_pad8(m)), 1 if t == 0x03 else 0) + _pad8(m) for t, m in msgs)
        hdr = struct.pack("<BBHII", 1, 0, len(msgs), 1, len(body)) + bytes(4)
        oh = alloc(len(hdr) + len(body))
        out[oh:oh + len(hdr) + len(body)] = hdr + body
        obj[nm] = oh
    # symbol table node (all entries, sorted) and the group B-tree with one child
    K = max(4, (len(names) + 1) // 2)
    snod = alloc(8 + 2 * K * 40)
    struct.pack_into("<4sBBH", out, snod, b"SNOD", 1, 0, len(names))
    for i, nm in enumerate(names):
        struct.pack_into("<QQII16x", out, snod + 8 + 40 * i, name_off[nm], obj[nm], 0, 0)
    KI = 16                                   # group internal node K: the node's allocated size
    tree = alloc(24 + 8 * (2 * KI + 1) + 8 * 2 * KI)
    struct.pack_into("<4sBBHQQ", out, tree, b"TREE", 0, 0, 1 if names else 0, _UNDEF, _UNDEF)
    p = tree + 24
    struct.pack_into("<QQQ", out, p, 0, snod, name_off[names[-1]] if names else 0)
    # root group object header: symbol table message
    stab = struct.pack("<QQ", tree, heap_hdr)
    body = struct.pack("<HHB3x", 0x11, len(stab), 0) + stab
    root = alloc(16 + len(body))
    out[root:root + 16 + len(body)] = struct.pack("<BBHII", 1, 0, 1, 1, len(body)) + bytes(4) + body
    # superblock v0
    sbb = bytearray()
    sbb += _SIG + bytes([0, 0, 0, 0, 0, so, 8, 0])
    sbb += struct.pack("<HHI", K, KI, 0)
    sbb += struct.pack("<QQQQ", 0, _UNDEF, len(out), _UNDEF)
    sbb += struct.pack("<QQII", 0, root, 1, 0) + struct.pack("<QQ", tree, heap_hdr)
    out[sb:sb + len(sbb)] = sbb
    with open(path, "wb") as f:
        f.write(bytes(out))
