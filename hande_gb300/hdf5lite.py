"""A small reader and writer for the part of the HDF5 file format that HANDE's
restart files use, with no HDF5 library.

HANDE writes its restart files (src/restart_hdf5.F90) through the HDF5
library's defaults: a version-0 superblock, groups as symbol tables (a v1
B-tree of group nodes, symbol-table nodes and a local heap of names), version-1
object headers, and datasets of fixed-point, floating-point or fixed-length
string elements in contiguous (or compact) storage with a simple or scalar
dataspace.  This module reads exactly that subset -- enough to open every
restart file in HANDE's test suite -- and writes files of the same shape:

    read(path) -> {"/qmc/psips/determinants": numpy array, ...}
    write(path, {"/qmc/psips/determinants": array, "/metadata/date": b"...", ...})

Structures follow the published HDF5 File Format Specification (version 2.0
for the version-0 superblock, version-1 object headers, v1 B-trees, local
heaps and symbol-table nodes; message encodings for dataspace v1/v2, datatype
classes 0/1/3, fill value v1-v3 and data layout v1-v3).  Array order: HDF5
stores dimensions slowest first; HANDE's Fortran arrays appear transposed, so
a Fortran states(W, n) dataset is read as an (n, W) array, which is also the
layout of hgpu_upload_walkers' column-major input.
"""

import mmap
import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class FormatError(ValueError):
    pass


# ---------------------------------------------------------------------------
# Reading
# ---------------------------------------------------------------------------

class _Reader:
    def __init__(self, data: bytes):
        self.d = data
        if data[:8] != SIGNATURE:
            raise FormatError("not an HDF5 file")
        ver = data[8]
        if ver not in (0, 1):
            raise FormatError("superblock version %d is not supported" % ver)
        self.so, self.sl = data[13], data[14]
        if self.so != 8 or self.sl != 8:
            raise FormatError("only 8-byte offsets and lengths are supported")
        p = 24 + (4 if ver == 1 else 0)
        self.base, _free, self.eof, _drv = struct.unpack_from("<4Q", data, p)
        self.root_entry = p + 32

    def u(self, fmt, p):
        return struct.unpack_from("<" + fmt, self.d, p)

    # -- symbol table entries, groups ------------------------------------
    def entry(self, p):
        name_off, hdr = self.u("QQ", p)
        cache, = self.u("I", p + 16)
        btree = heap = None
        if cache == 1:
            btree, heap = self.u("QQ", p + 24)
        return name_off, hdr, btree, heap

    def heap_name(self, heap, off):
        sig = self.d[heap:heap + 4]
        if sig != b"HEAP":
            raise FormatError("local heap expected at %d" % heap)
        seg, = self.u("Q", heap + 24)
        s = seg + off
        e = self.d.find(b"\0", s)
        if e < 0:
            raise FormatError("unterminated name in the local heap at %d" % heap)
        return bytes(self.d[s:e]).decode()

    def group_members(self, btree, heap):
        """(name, object header address) of every link of a symbol-table group."""
        out = []
        self._walk_btree(btree, heap, out, set())
        return out

    def _walk_btree(self, node, heap, out, seen):
        if node in seen or len(seen) > 4096:
            raise FormatError("group B-tree revisits node %d" % node)
        seen.add(node)
        if self.d[node:node + 4] != b"TREE":
            raise FormatError("v1 B-tree node expected at %d" % node)
        ntype, level, used = self.d[node + 4], self.d[node + 5], self.u("H", node + 6)[0]
        if ntype != 0:
            raise FormatError("group B-tree expected (node type %d)" % ntype)
        p = node + 24
        children = []
        for i in range(used):
            p += 8  # key i (heap offset of the largest name to its left)
            children.append(self.u("Q", p)[0])
            p += 8
        for c in children:
            if level > 0:
                self._walk_btree(c, heap, out, seen)
            else:
                self._snod(c, heap, out)

    def _snod(self, p, heap, out):
        if self.d[p:p + 4] != b"SNOD":
            raise FormatError("symbol-table node expected at %d" % p)
        n, = self.u("H", p + 6)
        q = p + 8
        for _ in range(n):
            name_off, hdr, _, _ = self.entry(q)
            out.append((self.heap_name(heap, name_off), hdr))
            q += 40

    # -- object headers -----------------------------------------------------
    def messages(self, addr):
        """[(type, flags, payload bytes)] of a version-1 object header,
        continuation blocks followed."""
        if self.d[addr] != 1:
            raise FormatError("object header version %d at %d is not supported" % (self.d[addr], addr))
        nmsg, _refc, size = self.u("HII", addr + 2)
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            p, size = blocks.pop(0)
            end = p + size
            while p + 8 <= end and len(out) < nmsg:
                mtype, msize, flags = self.u("HHB", p)
                payload = self.d[p + 8:p + 8 + msize]
                out.append((mtype, flags, payload))
                if mtype == 0x10:  # continuation
                    blocks.append(self.u("QQ", p + 8))
                p += 8 + msize
        return out

    # -- datasets ------------------------------------------------------------
    def dataset(self, msgs):
        shape = dtype = layout = None
        for mtype, _flags, m in msgs:
            if mtype == 0x01:
                shape = _dataspace(m)
            elif mtype == 0x03:
                dtype = _datatype(m)
            elif mtype == 0x08:
                layout = _layout(m)
        if shape is None or dtype is None or layout is None:
            raise FormatError("dataset without dataspace, datatype or layout")
        kind, where, nbytes = layout
        count = int(np.prod(shape)) if shape else 1
        if kind == "compact":
            arr = np.frombuffer(where, dtype=dtype, count=count).copy()
        elif where == UNDEF:
            arr = np.zeros(count, dtype=dtype)
        else:
            off = self.base + where
            if off + count * dtype.itemsize > len(self.d):
                raise FormatError("dataset data past the end of the file")
            arr = np.frombuffer(self.d, dtype=dtype, count=count, offset=off).copy()
        return arr.reshape(shape) if shape else arr.reshape(())


def _dataspace(m):
    ver, ndim, flags = m[0], m[1], m[2]
    if ver == 1:
        p = 8
    elif ver == 2:
        if m[3] == 0:  # scalar
            return ()
        p = 4
    else:
        raise FormatError("dataspace version %d" % ver)
    return tuple(struct.unpack_from("<%dQ" % ndim, m, p))


def _datatype(m):
    cls, ver = m[0] & 0x0F, m[0] >> 4
    bits = m[1] | (m[2] << 8) | (m[3] << 16)
    size, = struct.unpack_from("<I", m, 4)
    order = ">" if bits & 1 else "<"
    if cls == 0:  # fixed point
        signed = bool(bits & 0x08)
        return np.dtype("%s%s%d" % (order, "i" if signed else "u", size))
    if cls == 1:  # floating point
        return np.dtype("%sf%d" % (order, size))
    if cls == 3:  # fixed-length string
        return np.dtype("S%d" % size)
    raise FormatError("datatype class %d (version %d) is not supported" % (cls, ver))


def _layout(m):
    ver = m[0]
    if ver == 3:
        cls = m[1]
        if cls == 0:
            n, = struct.unpack_from("<H", m, 2)
            return "compact", bytes(m[4:4 + n]), n
        if cls == 1:
            addr, n = struct.unpack_from("<QQ", m, 2)
            return "contiguous", addr, n
        raise FormatError("chunked storage is not supported")
    if ver in (1, 2):
        ndim, cls = m[1], m[2]
        if cls == 1:
            addr, = struct.unpack_from("<Q", m, 8)
            return "contiguous", addr, None
        if cls == 0:
            p = 8 + 4 * ndim
            n, = struct.unpack_from("<I", m, p)
            return "compact", bytes(m[p + 4:p + 4 + n]), n
        raise FormatError("chunked storage is not supported")
    raise FormatError("data layout version %d" % ver)


def _mapped(path):
    """The file mapped read-only (datasets are copied out of it, so a list of
    many GB is not read into memory twice)."""
    with open(path, "rb") as f:
        return mmap.mmap(f.fileno(), 0, access=mmap.ACCESS_READ)


def read(path):
    """Every dataset of the file by its path ('/group/name'); strings come back
    as numpy bytes arrays (scalars as 0-d arrays)."""
    mm = _mapped(path)
    try:
        r = _Reader(mm)
        out = {}
        _, hdr, btree, heap = r.entry(r.root_entry)
        _read_group(r, hdr, btree, heap, "", out)
        return out
    finally:
        mm.close()


def _read_group(r, hdr, btree, heap, prefix, out, depth=0):
    if depth > 64:
        raise FormatError("groups nested deeper than 64 levels")
    if btree is None:
        for mtype, _f, m in r.messages(hdr):
            if mtype == 0x11:
                btree, heap = struct.unpack_from("<QQ", m, 0)
    for name, child in r.group_members(btree, heap):
        msgs = r.messages(child)
        stab = [m for t, _f, m in msgs if t == 0x11]
        path = prefix + "/" + name
        if stab:
            b, h = struct.unpack_from("<QQ", stab[0], 0)
            _read_group(r, child, b, h, path, out, depth + 1)
        else:
            out[path] = r.dataset(msgs)


def _msg_sig(t, f, m):
    """(type, flags, version or datatype class/version) of a header message."""
    if t == 0x03:
        return (t, f, m[0] & 0x0F, m[0] >> 4)
    if t in (0x01, 0x05, 0x08, 0x12, 0x0C) and m:
        return (t, f, m[0])
    return (t, f)


def structure(path):
    """Every object of the file with the signature of its header messages
    (type, flags, version; datatype class and version), NIL padding left out,
    for comparing the shape of two files."""
    with open(path, "rb") as f:
        r = _Reader(f.read())
    out = {}
    _, hdr, _btree, _heap = r.entry(r.root_entry)

    def walk(addr, path):
        msgs = r.messages(addr)
        out[path or "/"] = [_msg_sig(t, fl, m) for t, fl, m in msgs if t != 0]
        for t, _fl, m in msgs:
            if t == 0x11:
                b, h = struct.unpack_from("<QQ", m, 0)
                for name, child in r.group_members(b, h):
                    walk(child, path + "/" + name)

    walk(hdr, "")
    return out


# ---------------------------------------------------------------------------
# Writing
# ---------------------------------------------------------------------------

LEAF_K, INTERNAL_K = 4, 16                      # the library's defaults
SNOD_SIZE = 8 + 2 * LEAF_K * 40                 # symbol-table node with 2K entries
BTREE_SIZE = 24 + (2 * INTERNAL_K + 1) * 8 + 2 * INTERNAL_K * 8
DATASET_HEADER = 256                            # message space of a dataset's object header
FREE_NULL = 1                                   # "no next free block" in a local heap


def _pad8(n):
    return (n + 7) & ~7


def _msg(mtype, flags, payload):
    payload = bytes(payload)
    payload += b"\0" * (_pad8(len(payload)) - len(payload))
    return struct.pack("<HHB3x", mtype, len(payload), flags) + payload


def _dtype_msg(dt):
    """Datatype message (version 1) of a numpy dtype: signed or unsigned
    little-endian integers, IEEE doubles, fixed-length space-padded strings."""
    if dt.kind in "iu":
        bits = 0x08 if dt.kind == "i" else 0x00
        return struct.pack("<B3BI HH", 0x10, bits, 0, 0, dt.itemsize, 0, 8 * dt.itemsize)
    if dt.kind == "f" and dt.itemsize == 8:
        return struct.pack("<B3BI HHBBBBI", 0x11, 0x20, 0x3F, 0x00, 8, 0, 64, 52, 11, 0, 52, 1023)
    if dt.kind == "S":
        return struct.pack("<B3BI", 0x13, 0x02, 0, 0, dt.itemsize)
    raise FormatError("no HDF5 type for %s" % dt)


def _dataspace_msg(shape):
    if not shape:
        return struct.pack("<BBBB4x", 1, 0, 0, 0)
    n = len(shape)
    return struct.pack("<BBBB4x%dQ%dQ" % (n, n), 1, n, 1, 0, *shape, *shape)


class _Writer:
    """Lays the file out in address order: metadata blocks are kept in memory,
    dataset contents are written straight from their arrays at the end."""

    def __init__(self, mtime):
        self.size = 0
        self.blocks = {}  # address -> bytearray (metadata)
        self.arrays = []  # (address, contiguous little-endian array)
        self.mtime = int(mtime) & 0xFFFFFFFF
        self.alloc(96)    # superblock and root entry, filled last

    def alloc(self, n):
        addr = self.size
        self.size += _pad8(n)
        self.blocks[addr] = bytearray(_pad8(n))
        return addr

    def alloc_array(self, arr):
        addr = self.size
        self.size += _pad8(arr.nbytes)
        self.arrays.append((addr, arr))
        return addr

    def put(self, addr, data):
        blk = self.blocks[addr]
        blk[:len(data)] = data

    def flush(self, f):
        for addr, blk in self.blocks.items():
            f.seek(addr)
            f.write(blk)
        for addr, arr in self.arrays:
            f.seek(addr)
            arr.tofile(f)
        f.truncate(self.size)

    def dataset(self, arr):
        arr = np.asarray(arr)
        if arr.dtype.kind in "iuf":
            arr = arr.astype(arr.dtype.newbyteorder("<"), copy=False)
        if not arr.flags.c_contiguous:
            arr = arr.copy(order="C")  # (np.ascontiguousarray would turn a scalar into a vector)
        nbytes = arr.nbytes
        hdr = self.alloc(16 + DATASET_HEADER)
        addr = self.alloc_array(arr) if nbytes else UNDEF
        raw_len = nbytes
        msgs = [
            _msg(0x01, 0, _dataspace_msg(arr.shape)),
            _msg(0x03, 1, _dtype_msg(arr.dtype)),
            _msg(0x05, 1, struct.pack("<BBBBI", 2, 2, 2, 1, 0)),
            _msg(0x08, 1, struct.pack("<BBQQ", 3, 1, addr, raw_len)),
            _msg(0x12, 0, struct.pack("<B3xI", 1, self.mtime)),
        ]
        body = b"".join(msgs)
        if len(body) + 8 > DATASET_HEADER:
            raise FormatError("dataset header overflow")
        body += struct.pack("<HHB3x", 0, DATASET_HEADER - len(body) - 8, 0) + b"\0" * (DATASET_HEADER - len(body) - 8)
        self.put(hdr, struct.pack("<BBHII4x", 1, 0, len(msgs) + 1, 1, DATASET_HEADER) + body)
        return hdr, None, None

    def group(self, members):
        """A symbol-table group; returns (object header, B-tree, local heap)."""
        hdr = self.alloc(16 + 24)
        btree = self.alloc(BTREE_SIZE)
        names = sorted(members, key=lambda n: n.encode())
        heap_data = bytearray(8)  # offset 0: the empty name
        offs = {}
        for n in names:
            offs[n] = len(heap_data)
            b = n.encode() + b"\0"
            heap_data += b + b"\0" * (_pad8(len(b)) - len(b))
        free_at = len(heap_data)
        free_size = max(16, 88 - free_at)
        heap_data += struct.pack("<QQ", FREE_NULL, free_size) + b"\0" * (free_size - 16)
        heap = self.alloc(32)
        seg = self.alloc(len(heap_data))
        self.put(heap, b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap_data), free_at, seg))
        self.put(seg, bytes(heap_data))
        entries = []
        for n in names:
            child = members[n]
            if isinstance(child, dict):
                ch, cb, chp = self.group(child)
                entries.append(struct.pack("<QQI4xQQ", offs[n], ch, 1, cb, chp))
            else:
                ch, _, _ = self.dataset(child)
                entries.append(struct.pack("<QQI4x16x", offs[n], ch, 0))
        chunks = [entries[i:i + 2 * LEAF_K] for i in range(0, len(entries), 2 * LEAF_K)]
        name_chunks = [names[i:i + 2 * LEAF_K] for i in range(0, len(names), 2 * LEAF_K)]
        if len(chunks) > 2 * INTERNAL_K:
            raise FormatError("group with more than %d members" % (4 * INTERNAL_K * LEAF_K))
        tree = bytearray(b"TREE" + struct.pack("<BBHQQ", 0, 0, len(chunks), UNDEF, UNDEF))
        tree += struct.pack("<Q", 0)
        for ch, nc in zip(chunks, name_chunks):
            snod = self.alloc(SNOD_SIZE)
            self.put(snod, b"SNOD" + struct.pack("<BBH", 1, 0, len(ch)) + b"".join(ch))
            tree += struct.pack("<QQ", snod, offs[nc[-1]])
        self.put(btree, bytes(tree))
        self.put(hdr, struct.pack("<BBHII4x", 1, 0, 1, 1, 24) + _msg(0x11, 0, struct.pack("<QQ", btree, heap)))
        return hdr, btree, heap


def _tree(datasets, groups=()):
    root = {}
    for path in list(datasets) + list(groups):
        parts = [p for p in path.split("/") if p]
        node = root
        for p in parts[:-1]:
            node = node.setdefault(p, {})
        if path in datasets:
            node[parts[-1]] = datasets[path]
        else:
            node.setdefault(parts[-1], {})
    return root


def write(path, datasets, groups=(), mtime=0):
    """Write datasets ({'/group/name': array or bytes}) and empty groups
    (['/rng']) as an HDF5 file in the layout the HDF5 library gives HANDE's
    restart files.  bytes values become fixed-length string scalars."""
    conv = {}
    for k, v in datasets.items():
        if isinstance(v, (bytes, str)):
            b = v.encode() if isinstance(v, str) else v
            conv[k] = np.array(b, dtype="S%d" % max(1, len(b)))
        else:
            conv[k] = np.asarray(v)
    w = _Writer(mtime)
    hdr, btree, heap = w.group(_tree(conv, groups))
    sb = SIGNATURE + struct.pack("<8BHHI", 0, 0, 0, 0, 0, 8, 8, 0, LEAF_K, INTERNAL_K, 0)
    sb += struct.pack("<4Q", 0, UNDEF, w.size, UNDEF)
    sb += struct.pack("<QQI4xQQ", 0, hdr, 1, btree, heap)
    w.put(0, sb)
    with open(path, "wb") as f:
        w.flush(f)
