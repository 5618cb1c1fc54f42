"""HDF5 files without h5py or libhdf5: the subset acquisition files use.

Neither h5py nor the HDF5 library exists on the machines this package runs
on, so the Dataset file (simulation/ringfwi/dataset.py:112-174) and the
UARP/UDSP v4.0 Set (simulation/ringfwi/uarp_format.py:37-116) are read and
written here, in pure Python + NumPy + zlib, after the HDF5 File Format
Specification (the structures the HDF5 library writes with its default,
earliest-compatible format).

Written: superblock version 0; version-1 object headers; groups as symbol
tables (version-1 B-tree, local heap for the link names, symbol-table nodes);
attributes as version-1 attribute messages -- scalars and arrays of IEEE
floats and signed/unsigned integers, and strings as variable-length UTF-8
strings in a global heap collection (what h5py stores for a Python ``str``, so
h5py hands them back as ``str``); datasets contiguous, or chunked (version-1
B-tree of chunks) through the deflate filter.

Read: the same, plus what other writers of that format produce -- B-trees
of any depth, object-header continuation blocks, version-2 object headers and
superblocks 1-3, compact groups (link messages), version-2/3 attribute and
dataspace messages, layout messages 1-3 (compact, contiguous, chunked), the
shuffle and Fletcher-32 filters, fixed-length strings (returned as bytes, as
h5py does).  Not read: dense (fractal-heap) link or attribute storage, shared
messages, version-4 layouts and compound, enum, array, reference or
variable-length sequence types -- each raises NotImplementedError.

The API is the part of h5py's the file layouts need: ``File(path, "w"|"r")``
as a context manager, ``attrs`` mappings, ``create_group``,
``create_dataset(name, data=, compression="gzip", compression_opts=)``,
``group[name]`` (also "a/b" paths), ``name in group``, ``group.keys()`` and
``dataset[()]``.
"""

from __future__ import annotations

import mmap
import os
import struct
import zlib
from concurrent.futures import ThreadPoolExecutor

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF            # the undefined address (8-byte offsets)
_HEAP_FREE_NULL = 1                   # local heap: no free block
_CHUNK_BYTES = 4 << 20                # target size of a written chunk
_GCOL_MIN = 4096                      # smallest global heap collection

# object header message types
_M_NIL, _M_SPACE, _M_LINFO, _M_DTYPE, _M_FILL_OLD, _M_FILL = 0x00, 0x01, 0x02, 0x03, 0x04, 0x05
_M_LINK, _M_LAYOUT, _M_FILTER, _M_ATTR, _M_CONT, _M_STAB = 0x06, 0x08, 0x0B, 0x0C, 0x10, 0x11
_M_AINFO = 0x15

_F_DEFLATE, _F_SHUFFLE, _F_FLETCHER = 1, 2, 3


def _pad8(b: bytes) -> bytes:
    return bytes(b) + b"\0" * (-len(b) % 8)


def _up8(n: int) -> int:
    return (n + 7) & ~7


# ---------------------------------------------------------------------------
# datatype and dataspace messages
# ---------------------------------------------------------------------------
# IEEE layouts: itemsize -> (sign bit, exponent location, exponent size,
# mantissa size, exponent bias)
_IEEE = {2: (15, 10, 5, 10, 15), 4: (31, 23, 8, 23, 127), 8: (63, 52, 11, 52, 1023)}


def _dtype_message(dt: np.dtype) -> bytes:
    """The datatype message of a little-endian NumPy number or bytes type."""
    dt = np.dtype(dt)
    size = dt.itemsize
    if dt.kind == "f" and size in _IEEE:
        sign, eloc, esz, msz, bias = _IEEE[size]
        # class 1, version 1; bit field: little endian, no padding, the
        # mantissa's leading bit implied (normalization 2), sign location
        head = struct.pack("<BBBBI", 0x11, 0x20, sign, 0, size)
        return head + struct.pack("<HHBBBBI", 0, 8 * size, eloc, esz, 0, msz, bias)
    if dt.kind in "iu" and size in (1, 2, 4, 8):
        head = struct.pack("<BBBBI", 0x10, 0x08 if dt.kind == "i" else 0x00, 0, 0, size)
        return head + struct.pack("<HH", 0, 8 * size)
    if dt.kind == "S":
        return struct.pack("<BBBBI", 0x13, 0x01, 0, 0, size)   # null-padded ASCII
    raise NotImplementedError(f"no HDF5 datatype written for {dt}")


def _vlen_string_message() -> bytes:
    """Variable-length UTF-8 string (class 9, null-terminated padding); its
    base type is the unsigned 8-bit integer; 16 bytes per element on disk."""
    base = struct.pack("<BBBBI", 0x10, 0, 0, 0, 1) + struct.pack("<HH", 0, 8)
    return struct.pack("<BBBBI", 0x19, 0x01, 0x01, 0, 16) + base


def _space_message(shape) -> bytes:
    shape = tuple(int(s) for s in shape)
    return struct.pack("<BBBB4x", 1, len(shape), 0, 0) + b"".join(
        struct.pack("<Q", s) for s in shape)


# ---------------------------------------------------------------------------
# writing
# ---------------------------------------------------------------------------
class _Buffer:
    """The file being written: 8-byte aligned allocations appended in order
    (so raw data goes straight to the file), and patches of what was
    allocated as a placeholder."""

    def __init__(self, f, reserve: int):
        self.f = f
        self.end = reserve
        f.write(b"\0" * reserve)

    def alloc(self, data) -> int:
        pad = -self.end % 8
        if pad:
            self.f.write(b"\0" * pad)
            self.end += pad
        addr = self.end
        self.f.write(data)
        self.end += len(data)
        return addr

    def patch(self, addr: int, data: bytes):
        self.f.seek(addr)
        self.f.write(data)
        self.f.seek(self.end)


class _WAttrs(dict):
    """Attributes of an object being written (name -> value)."""

    def __setitem__(self, name, value):
        if not isinstance(name, str) or not name:
            raise ValueError("attribute names are non-empty strings")
        super().__setitem__(name, value)


class _WDataset:
    def __init__(self, data, compression, level):
        arr = np.asarray(data)
        if arr.dtype.kind == "U":
            raise NotImplementedError("string datasets are not written")
        if arr.dtype.kind == "b":
            raise NotImplementedError("boolean datasets are not written")
        if arr.dtype.kind == "f" and arr.dtype.itemsize not in _IEEE:
            raise NotImplementedError(f"no HDF5 datatype written for {arr.dtype}")
        data = arr.astype(arr.dtype.newbyteorder("<"), copy=False)
        self.data = data if data.flags.c_contiguous else data.copy(order="C")   # keeps 0-d
        if compression not in (None, "gzip"):
            raise NotImplementedError(f"compression {compression!r} (only 'gzip')")
        self.compression = compression if self.data.ndim > 0 and self.data.size else None
        self.level = 4 if level is None else int(level)
        self.attrs = _WAttrs()
        self.shape = self.data.shape
        self.dtype = self.data.dtype


class _WGroup:
    def __init__(self):
        self.attrs = _WAttrs()
        self.children = {}

    def _parent_of(self, path):
        parts = [p for p in path.split("/") if p]
        if not parts:
            raise ValueError("empty name")
        g = self
        for p in parts[:-1]:
            g = g.children.get(p) or g.create_group(p)
            if not isinstance(g, _WGroup):
                raise ValueError(f"{p} is a dataset")
        return g, parts[-1]

    def create_group(self, name):
        g, leaf = self._parent_of(name)
        if leaf in g.children:
            raise ValueError(f"{name} exists")
        new = _WGroup()
        g.children[leaf] = new
        return new

    def require_group(self, name):
        return self[name] if name in self else self.create_group(name)

    def create_dataset(self, name, data=None, compression=None, compression_opts=None):
        g, leaf = self._parent_of(name)
        if leaf in g.children:
            raise ValueError(f"{name} exists")
        ds = _WDataset(data, compression, compression_opts)
        g.children[leaf] = ds
        return ds

    def __getitem__(self, name):
        g = self
        for p in [p for p in name.split("/") if p]:
            g = g.children[p]
        return g

    def __contains__(self, name):
        try:
            self[name]
            return True
        except (KeyError, AttributeError):
            return False

    def keys(self):
        return list(self.children)


def _strings_of(node, out):
    for v in node.attrs.values():
        if isinstance(v, str):
            out.append(v)
        elif isinstance(v, np.ndarray) and v.dtype.kind in "UO":
            out.extend(str(s) for s in v.ravel())
    if isinstance(node, _WGroup):
        for c in node.children.values():
            _strings_of(c, out)


class _GlobalHeap:
    """One global heap collection holding every variable-length string."""

    def __init__(self, strings):
        self.index = {}
        objs = []
        for s in strings:
            if s not in self.index:
                self.index[s] = len(objs) + 1
                objs.append(s.encode("utf-8"))
        body = bytearray()
        for i, b in enumerate(objs, 1):
            body += struct.pack("<HH4xQ", i, 0, len(b)) + _pad8(b)
        used = 16 + len(body)
        size = max(_GCOL_MIN, used + 16)
        free = size - used                       # the free-space object (index 0)
        self.image = (b"GCOL" + struct.pack("<B3xQ", 1, size) + bytes(body) +
                      struct.pack("<HH4xQ", 0, 0, free) + b"\0" * (free - 16))
        self.addr = None
        self.lengths = {s: len(s.encode("utf-8")) for s in self.index}

    def ref(self, s: str) -> bytes:
        """The 16-byte on-disk element of string s: length, collection, index."""
        return struct.pack("<IQI", self.lengths[s], self.addr, self.index[s])


def _attr_value(value, gheap):
    """(datatype message, dataspace message, data) of an attribute value."""
    if isinstance(value, str):
        return _vlen_string_message(), _space_message(()), gheap.ref(value)
    if isinstance(value, bytes):
        arr = np.array(value)
        return _dtype_message(arr.dtype), _space_message(()), arr.tobytes()
    arr = np.asarray(value)
    if arr.dtype.kind in "UO":
        flat = [str(s) for s in arr.ravel()]
        return (_vlen_string_message(), _space_message(arr.shape),
                b"".join(gheap.ref(s) for s in flat))
    if arr.dtype.kind == "b":
        arr = arr.astype(np.int8)
    arr = arr.astype(arr.dtype.newbyteorder("<"), copy=False)
    return _dtype_message(arr.dtype), _space_message(arr.shape), np.ascontiguousarray(arr).tobytes()


def _attr_message(name, value, gheap) -> bytes:
    dt, sp, data = _attr_value(value, gheap)
    nm = name.encode("utf-8") + b"\0"
    return (struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(sp)) + _pad8(nm) + _pad8(dt) +
            _pad8(sp) + data)


def _object_header(messages) -> bytes:
    """Version-1 object header: messages (type, body, flags), each body padded
    to 8 bytes; the prefix is 16 bytes (12 + 4 of alignment)."""
    chunk = bytearray()
    for mtype, body, flags in messages:
        body = _pad8(body)
        if len(body) > 0xFFFF:
            raise ValueError("an object header message above 64 KiB (an attribute too large)")
        chunk += struct.pack("<HHB3x", mtype, len(body), flags) + body
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(chunk)) + bytes(chunk)


def _btree(buf, node_type, children, keys, key_size, k):
    """Version-1 B-tree over ``children`` (addresses, in key order) with
    ``keys`` (len(children) + 1 encoded keys: key i bounds child i on the left,
    key i + 1 on the right); nodes of at most 2k children, sibling-linked on
    every level.  Returns the root's address."""
    level = 0
    node_size = 24 + 2 * k * 8 + (2 * k + 1) * key_size
    while True:
        n = len(children)
        groups = [(lo, min(lo + 2 * k, n)) for lo in range(0, max(n, 1), 2 * k)]
        addrs = [buf.alloc(b"\0" * node_size) for _ in groups]
        for gi, (lo, hi) in enumerate(groups):
            left = addrs[gi - 1] if gi > 0 else UNDEF
            right = addrs[gi + 1] if gi + 1 < len(groups) else UNDEF
            node = bytearray(b"TREE" + struct.pack("<BBHQQ", node_type, level, hi - lo, left, right))
            for i in range(lo, hi):
                node += keys[i] + struct.pack("<Q", children[i])
            node += keys[hi]
            buf.patch(addrs[gi], bytes(node))
        if len(groups) == 1:
            return addrs[0]
        keys = [keys[lo] for lo, _ in groups] + [keys[groups[-1][1]]]
        children = addrs
        level += 1


def _chunk_shape(shape, itemsize):
    """Chunks along the slowest axis of about _CHUNK_BYTES (whole rows)."""
    row = itemsize * int(np.prod(shape[1:], dtype=np.int64)) if len(shape) > 1 else itemsize
    c0 = max(1, min(int(shape[0]), _CHUNK_BYTES // max(row, 1)))
    chunk = (c0,) + tuple(int(s) for s in shape[1:])
    if itemsize * int(np.prod(chunk, dtype=np.int64)) >= 1 << 32:
        raise ValueError("a row of this dataset is too large for one HDF5 chunk")
    return chunk


def _write_dataset(buf, ds, gheap, workers):
    arr = ds.data
    msgs = [(_M_SPACE, _space_message(arr.shape), 0), (_M_DTYPE, _dtype_message(arr.dtype), 1)]
    if ds.compression is None:
        addr = buf.alloc(arr.reshape(-1).view(np.uint8)) if arr.nbytes else UNDEF
        msgs.append((_M_LAYOUT, struct.pack("<BBQQ", 3, 1, addr, arr.nbytes), 0))
    else:
        rank = arr.ndim
        chunk = _chunk_shape(arr.shape, arr.itemsize)
        n0 = -(-arr.shape[0] // chunk[0])

        def encode(i):
            part = arr[i * chunk[0]:(i + 1) * chunk[0]]
            if part.shape[0] < chunk[0]:        # edge chunks are stored full size
                full = np.zeros(chunk, arr.dtype)
                full[:part.shape[0]] = part
                part = full
            return zlib.compress(np.ascontiguousarray(part).tobytes(), ds.level)

        with ThreadPoolExecutor(max_workers=workers) as pool:   # zlib drops the GIL
            blobs = list(pool.map(encode, range(n0)))
        key_size = 8 + 8 * (rank + 1)
        children, keys = [], []
        for i, blob in enumerate(blobs):
            children.append(buf.alloc(blob))
            off = (i * chunk[0],) + (0,) * rank
            keys.append(struct.pack("<II", len(blob), 0) + struct.pack(f"<{rank + 1}Q", *off))
        # the right-most key: one chunk beyond the last in every dimension
        last = ((n0 - 1) + 1) * chunk[0]
        end = (last,) + tuple(chunk[1:]) + (arr.itemsize,)
        keys.append(struct.pack("<II", 0, 0) + struct.pack(f"<{rank + 1}Q", *end))
        root = _btree(buf, 1, children, keys, key_size, 32)
        dims = tuple(chunk) + (arr.itemsize,)
        msgs.append((_M_LAYOUT, struct.pack("<BBBQ", 3, 2, rank + 1, root) +
                     struct.pack(f"<{rank + 1}I", *dims), 0))
        name = b"deflate\0"
        msgs.append((_M_FILTER, struct.pack("<BB6x", 1, 1) +
                     struct.pack("<HHHH", _F_DEFLATE, len(name), 1, 1) + name +
                     struct.pack("<I4x", ds.level), 0))
    msgs += [(_M_ATTR, _attr_message(n, v, gheap), 0) for n, v in ds.attrs.items()]
    return buf.alloc(_object_header(msgs))


def _write_group(buf, grp, gheap, leaf_k, internal_k, workers):
    """Post-order: children, then the name heap, symbol-table nodes, B-tree and
    the group's own object header.  Returns (header, B-tree, heap) addresses."""
    names = sorted(grp.children, key=lambda s: s.encode("utf-8"))
    entries = {}
    for nm in names:
        c = grp.children[nm]
        if isinstance(c, _WGroup):
            oh, bt, hp = _write_group(buf, c, gheap, leaf_k, internal_k, workers)
            entries[nm] = (oh, 1, struct.pack("<QQ", bt, hp))
        else:
            entries[nm] = (_write_dataset(buf, c, gheap, workers), 0, b"\0" * 16)
    # local heap: the empty string at offset 0, then each name
    data = bytearray(8)
    offset = {}
    for nm in names:
        offset[nm] = len(data)
        data += _pad8(nm.encode("utf-8") + b"\0")
    heap = buf.alloc(b"\0" * 32)
    seg = buf.alloc(bytes(data))
    buf.patch(heap, b"HEAP" + struct.pack("<B3xQQQ", 0, len(data), _HEAP_FREE_NULL, seg))
    # symbol-table nodes of at most 2 leaf_k entries, names in byte order
    snods, keys = [], [struct.pack("<Q", 0)]
    for lo in range(0, len(names), 2 * leaf_k):
        part = names[lo:lo + 2 * leaf_k]
        node = bytearray(b"SNOD" + struct.pack("<BBH", 1, 0, len(part)))
        for nm in part:
            oh, cache, scratch = entries[nm]
            node += struct.pack("<QQI4x", offset[nm], oh, cache) + scratch
        node += b"\0" * (40 * (2 * leaf_k - len(part)))
        snods.append(buf.alloc(bytes(node)))
        keys.append(struct.pack("<Q", offset[part[-1]]))
    bt = _btree(buf, 0, snods, keys, 8, internal_k)
    msgs = [(_M_STAB, struct.pack("<QQ", bt, heap), 0)]
    msgs += [(_M_ATTR, _attr_message(n, v, gheap), 0) for n, v in grp.attrs.items()]
    return buf.alloc(_object_header(msgs)), bt, heap


def _max_entries(grp):
    n = len(grp.children)
    for c in grp.children.values():
        if isinstance(c, _WGroup):
            n = max(n, _max_entries(c))
    return n


def _serialize(root, path, leaf_k=None, internal_k=16, workers=None):
    if leaf_k is None:   # one symbol-table node per group
        leaf_k = max(4, -(-_max_entries(root) // 2))
    if not (1 <= leaf_k <= 0xFFFF and 1 <= internal_k <= 0xFFFF):
        raise ValueError("B-tree ranks must be 1..65535")
    workers = workers or min(32, os.cpu_count() or 1)
    tmp = path + ".tmp"
    try:
        with open(tmp, "wb") as f:
            buf = _Buffer(f, 96)
            strings = []
            _strings_of(root, strings)
            gheap = _GlobalHeap(strings)
            if gheap.index:
                gheap.addr = buf.alloc(gheap.image)
            oh, bt, hp = _write_group(buf, root, gheap, leaf_k, internal_k, workers)
            buf.alloc(b"")                       # the end of file, 8-byte aligned
            sb = (SIGNATURE + struct.pack("<BBBBBBBB", 0, 0, 0, 0, 0, 8, 8, 0) +
                  struct.pack("<HHI", leaf_k, internal_k, 0) +
                  struct.pack("<QQQQ", 0, UNDEF, buf.end, UNDEF) +
                  struct.pack("<QQI4x", 0, oh, 1) + struct.pack("<QQ", bt, hp))
            assert len(sb) == 96
            buf.patch(0, sb)
        os.replace(tmp, path)
    except BaseException:
        if os.path.exists(tmp):
            os.remove(tmp)
        raise


# ---------------------------------------------------------------------------
# reading
# ---------------------------------------------------------------------------
class _Reader:
    def __init__(self, path):
        self.f = open(path, "rb")
        try:
            self._open(path)
        except BaseException:
            self.f.close()
            raise

    def _open(self, path):
        size = os.fstat(self.f.fileno()).st_size
        self.mm = mmap.mmap(self.f.fileno(), 0, access=mmap.ACCESS_READ) if size else b""
        self.b = memoryview(self.mm) if size else memoryview(b"")
        self.base = None
        for at in [0] + [512 << i for i in range(20)]:       # user blocks of 512 * 2^i bytes
            if at + 8 > size:
                break
            if bytes(self.b[at:at + 8]) == SIGNATURE:
                self.base = at
                break
        if self.base is None:
            raise ValueError(f"{path}: not an HDF5 file")
        self._superblock()
        self._gheaps = {}

    def close(self):
        try:
            self.b.release()
            if self.mm:
                self.mm.close()
        except BufferError:      # a view is still alive: the map closes when it goes
            pass
        self.f.close()

    # -- primitives
    def u(self, at, n):
        return int.from_bytes(self.b[at:at + n], "little")

    def addr(self, at):
        v = self.u(at, self.O)
        return None if v == (1 << (8 * self.O)) - 1 else v + self.sb_base

    def _superblock(self):
        b0 = self.base
        v = self.b[b0 + 8]
        if v in (0, 1):
            self.O, self.L = self.b[b0 + 13], self.b[b0 + 14]
            p = b0 + 24 + (4 if v == 1 else 0)
            self.sb_base = b0                        # addresses are relative to the superblock
            p += 4 * self.O                          # base, free space, end of file, driver
            self.root = self.addr(p + self.O)        # the root entry's object header
        elif v in (2, 3):
            self.O, self.L = self.b[b0 + 9], self.b[b0 + 10]
            p = b0 + 12
            self.sb_base = b0
            self.root = self.addr(p + 3 * self.O)
        else:
            raise NotImplementedError(f"superblock version {v}")

    # -- object headers
    def messages(self, at):
        """[(type, body memoryview, flags)] of the object header at ``at``."""
        b = self.b
        out = []
        chunks = []
        if bytes(b[at:at + 4]) == b"OHDR":
            flags = b[at + 5]
            p = at + 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
            w = 1 << (flags & 3)
            size = self.u(p, w)
            p += w
            chunks.append((p, p + size, 2, flags))
        else:
            if b[at] != 1:
                raise NotImplementedError(f"object header version {b[at]}")
            chunks.append((at + 16, at + 16 + self.u(at + 8, 4), 1, 0))
        while chunks:
            p, end, ver, oflags = chunks.pop(0)
            while True:
                if ver == 1:
                    if p + 8 > end:
                        break
                    mtype, size, mflags = self.u(p, 2), self.u(p + 2, 2), b[p + 4]
                    p += 8
                else:
                    hdr = 4 + (2 if oflags & 0x04 else 0)
                    if p + hdr > end:                    # a gap shorter than a header
                        break
                    mtype, size, mflags = b[p], self.u(p + 1, 2), b[p + 3]
                    p += hdr
                body = b[p:p + size]
                p += size
                if mflags & 0x02:
                    raise NotImplementedError("shared object header messages")
                if mtype == _M_CONT:
                    ca = self.u_addr_body(body, 0)
                    cl = int.from_bytes(body[self.O:self.O + self.L], "little")
                    if ver == 1:
                        chunks.append((ca, ca + cl, 1, 0))
                    else:                                # "OCHK", messages, checksum
                        chunks.append((ca + 4, ca + cl - 4, 2, oflags))
                    continue
                out.append((mtype, body, mflags))
        return out

    def u_addr_body(self, body, off):
        v = int.from_bytes(body[off:off + self.O], "little")
        return None if v == (1 << (8 * self.O)) - 1 else v + self.sb_base

    # -- groups
    def links(self, at):
        """{name: object header address} of the group at ``at``."""
        out = {}
        for mtype, body, _ in self.messages(at):
            if mtype == _M_STAB:
                bt = self.u_addr_body(body, 0)
                heap = self.u_addr_body(body, self.O)
                self._stab(bt, heap, out)
            elif mtype == _M_LINK:
                name, target = self._link(body)
                if target is not None:
                    out[name] = target
            elif mtype == _M_LINFO:
                fheap = self.u_addr_body(body, 2 + (8 if body[1] & 1 else 0))
                if fheap is not None:
                    raise NotImplementedError("dense link storage (fractal heap)")
        return out

    def _heap_name(self, heap, off):
        b = self.b
        if bytes(b[heap:heap + 4]) != b"HEAP":
            raise ValueError("bad local heap")
        seg = self.addr(heap + 8 + 2 * self.L)
        p = seg + off
        q = p
        while b[q] != 0:
            q += 1
        return bytes(b[p:q]).decode("utf-8")

    def _btree_children(self, at, node_type, key_size):
        """[(left key position, child address)] of the leaves of a version-1
        B-tree, in key order (every child descended, so sibling links are not
        needed)."""
        b = self.b
        if bytes(b[at:at + 4]) != b"TREE" or b[at + 4] != node_type:
            raise ValueError("bad B-tree node")
        level, n = b[at + 5], self.u(at + 6, 2)
        p = at + 8 + 2 * self.O
        out = []
        for _ in range(n):
            child = self.addr(p + key_size)
            if level > 0:
                out.extend(self._btree_children(child, node_type, key_size))
            else:
                out.append((p, child))
            p += key_size + self.O
        return out

    def _stab(self, bt, heap, out):
        b = self.b
        for _, snod in self._btree_children(bt, 0, self.L):
            if bytes(b[snod:snod + 4]) != b"SNOD":
                raise ValueError("bad symbol table node")
            n = self.u(snod + 6, 2)
            p = snod + 8
            for _ in range(n):
                name = self._heap_name(heap, self.u(p, self.O))
                out[name] = self.addr(p + self.O)
                p += 2 * self.O + 8 + 16

    def _link(self, body):
        ver, flags = body[0], body[1]
        if ver != 1:
            raise NotImplementedError(f"link message version {ver}")
        p = 2
        ltype = 0
        if flags & 0x08:
            ltype = body[p]
            p += 1
        if flags & 0x04:
            p += 8
        if flags & 0x10:
            p += 1
        w = 1 << (flags & 3)
        n = int.from_bytes(body[p:p + w], "little")
        p += w
        name = bytes(body[p:p + n]).decode("utf-8")
        p += n
        if ltype != 0:            # soft / external links are not followed
            return name, None
        return name, self.u_addr_body(body, p)

    # -- types and spaces
    def dtype(self, body):
        """NumPy dtype, or "vlen-str", of a datatype message body."""
        cls, bits, size = body[0] & 0x0F, int.from_bytes(body[1:4], "little"), \
            int.from_bytes(body[4:8], "little")
        if cls == 0:
            return np.dtype((">" if bits & 1 else "<") + ("i" if bits & 0x08 else "u") + str(size))
        if cls == 1:
            if bits & 0x40:
                raise NotImplementedError("VAX floating point")
            return np.dtype((">" if bits & 1 else "<") + "f" + str(size))
        if cls == 3:
            return np.dtype(f"S{size}")
        if cls == 9 and (bits & 0x0F) == 1:
            return "vlen-str"
        raise NotImplementedError(f"HDF5 datatype class {cls}")

    def space(self, body):
        """Shape of a dataspace message body (() for a scalar)."""
        ver, rank, flags = body[0], body[1], body[2]
        if ver == 1:
            p = 8
        elif ver == 2:
            if body[3] == 2:
                return None                     # the null dataspace
            p = 4
        else:
            raise NotImplementedError(f"dataspace version {ver}")
        return tuple(int.from_bytes(body[p + i * self.L:p + (i + 1) * self.L], "little")
                     for i in range(rank))

    def vlen_string(self, elem):
        n, coll, idx = (int.from_bytes(elem[:4], "little"), self.u_addr_body(elem, 4),
                        int.from_bytes(elem[4 + self.O:8 + self.O], "little"))
        if n == 0 or coll is None:
            return ""
        objs = self._gheaps.get(coll)
        if objs is None:
            objs = self._gheaps[coll] = self._global_heap(coll)
        return bytes(objs[idx][:n]).decode("utf-8")

    def _global_heap(self, at):
        b = self.b
        if bytes(b[at:at + 4]) != b"GCOL":
            raise ValueError("bad global heap collection")
        size = self.u(at + 8, self.L)
        end = at + size
        p = at + 8 + self.L
        hdr = 8 + self.L
        objs = {}
        while p + hdr <= end:
            idx, osize = self.u(p, 2), self.u(p + 8, self.L)
            if idx == 0:
                break
            objs[idx] = bytes(b[p + hdr:p + hdr + osize])
            p += hdr + _up8(osize)
        return objs

    # -- attributes
    def attributes(self, msgs):
        out = {}
        for mtype, body, _ in msgs:
            if mtype == _M_AINFO:
                fheap = self.u_addr_body(body, 2 + (2 if body[1] & 1 else 0))
                if fheap is not None:
                    raise NotImplementedError("dense attribute storage (fractal heap)")
            if mtype != _M_ATTR:
                continue
            ver = body[0]
            nlen, dlen, slen = (int.from_bytes(body[2 + 2 * i:4 + 2 * i], "little") for i in range(3))
            if ver == 1:
                p = 8
                al = _up8
            elif ver in (2, 3):
                if body[1] & 0x03:
                    raise NotImplementedError("shared attribute datatype or dataspace")
                p = 8 if ver == 2 else 9
                al = int
            else:
                raise NotImplementedError(f"attribute message version {ver}")
            name = bytes(body[p:p + nlen]).rstrip(b"\0").decode("utf-8")
            p += al(nlen)
            dt = self.dtype(body[p:p + dlen])
            p += al(dlen)
            shape = self.space(body[p:p + slen])
            p += al(slen)
            out[name] = self._value(dt, shape, body[p:])
        return out

    def _value(self, dt, shape, data):
        if shape is None:
            return None
        count = int(np.prod(shape, dtype=np.int64)) if shape else 1
        if dt == "vlen-str":
            esz = 8 + self.O
            vals = [self.vlen_string(data[i * esz:(i + 1) * esz]) for i in range(count)]
            return vals[0] if shape == () else np.array(vals, dtype=object).reshape(shape)
        arr = np.frombuffer(bytes(data[:count * dt.itemsize]), dt, count=count)
        if dt.kind == "S":
            arr = arr.astype(dt)
            return arr[0] if shape == () else arr.reshape(shape)
        arr = arr.astype(dt.newbyteorder("="))
        return arr[0] if shape == () else arr.reshape(shape)

    # -- datasets
    def dataset_info(self, msgs):
        info = {"filters": []}
        for mtype, body, _ in msgs:
            if mtype == _M_SPACE:
                info["shape"] = self.space(body)
            elif mtype == _M_DTYPE:
                info["dtype"] = self.dtype(body)
            elif mtype == _M_LAYOUT:
                info["layout"] = self._layout(body)
            elif mtype == _M_FILTER:
                info["filters"] = self._filters(body)
        return info

    def _layout(self, body):
        ver = body[0]
        if ver == 3:
            cls = body[1]
            if cls == 0:
                n = int.from_bytes(body[2:4], "little")
                return ("compact", bytes(body[4:4 + n]))
            if cls == 1:
                return ("contiguous", self.u_addr_body(body, 2),
                        int.from_bytes(body[2 + self.O:2 + self.O + self.L], "little"))
            if cls == 2:
                nd = body[2]
                bt = self.u_addr_body(body, 3)
                p = 3 + self.O
                dims = tuple(int.from_bytes(body[p + 4 * i:p + 4 * i + 4], "little")
                             for i in range(nd))
                return ("chunked", bt, dims)
        elif ver in (1, 2):
            nd, cls = body[1], body[2]
            p = 8
            a = None
            if cls != 0:
                a = self.u_addr_body(body, p)
                p += self.O
            dims = tuple(int.from_bytes(body[p + 4 * i:p + 4 * i + 4], "little") for i in range(nd))
            p += 4 * nd
            if cls == 0:
                n = int.from_bytes(body[p:p + 4], "little")
                return ("compact", bytes(body[p + 4:p + 4 + n]))
            if cls == 1:
                return ("contiguous", a, None)
            return ("chunked", a, dims)
        raise NotImplementedError(f"data layout message version {ver}")

    def _filters(self, body):
        ver, n = body[0], body[1]
        p = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = int.from_bytes(body[p:p + 2], "little")
            p += 2
            nlen = 0
            if ver == 1 or fid >= 256:
                nlen = int.from_bytes(body[p:p + 2], "little")
                p += 2
            p += 2                                       # flags
            ncd = int.from_bytes(body[p:p + 2], "little")
            p += 2
            p += _up8(nlen) if ver == 1 else nlen
            cd = [int.from_bytes(body[p + 4 * i:p + 4 * i + 4], "little") for i in range(ncd)]
            p += 4 * ncd + (4 if ver == 1 and ncd % 2 else 0)
            out.append((fid, cd))
        return out

    def read(self, info):
        shape, dt = info["shape"], info["dtype"]
        if dt == "vlen-str":
            raise NotImplementedError("variable-length string datasets")
        if shape is None:
            return None
        count = int(np.prod(shape, dtype=np.int64)) if shape else 1
        kind = info["layout"][0]
        if kind == "compact":
            arr = np.frombuffer(info["layout"][1][:count * dt.itemsize], dt, count=count)
        elif kind == "contiguous":
            a = info["layout"][1]
            if a is None:
                arr = np.zeros(count, dt)
            else:
                arr = np.frombuffer(self.b[a:a + count * dt.itemsize], dt, count=count)
        else:
            return self._read_chunked(info, shape, dt)
        return np.array(arr.astype(dt.newbyteorder("="), copy=True).reshape(shape))

    def _read_chunked(self, info, shape, dt):
        _, bt, dims = info["layout"]
        rank = len(shape)
        cdims = dims[:rank]
        out = np.zeros(shape, dt.newbyteorder("="))
        if bt is None:
            return out
        filters = info["filters"]
        leaves = self._btree_children(bt, 1, 8 + 8 * (rank + 1))

        def one(leaf):
            kp, child = leaf
            nbytes, mask = self.u(kp, 4), self.u(kp + 4, 4)
            off = tuple(self.u(kp + 8 + 8 * i, 8) for i in range(rank))
            raw = bytes(self.b[child:child + nbytes])
            for i in range(len(filters) - 1, -1, -1):
                if mask & (1 << i):
                    continue
                fid, cd = filters[i]
                if fid == _F_DEFLATE:
                    raw = zlib.decompress(raw)
                elif fid == _F_SHUFFLE:
                    es = cd[0] if cd else dt.itemsize
                    raw = np.frombuffer(raw, np.uint8).reshape(es, -1).T.tobytes()
                elif fid == _F_FLETCHER:
                    raw = raw[:-4]
                else:
                    raise NotImplementedError(f"HDF5 filter {fid}")
            blk = np.frombuffer(raw, dt, count=int(np.prod(cdims))).reshape(cdims)
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(off, cdims, shape))
            out[sl] = blk[tuple(slice(0, x.stop - x.start) for x in sl)]

        with ThreadPoolExecutor(max_workers=min(32, os.cpu_count() or 1)) as pool:
            list(pool.map(one, leaves))
        return out


# ---------------------------------------------------------------------------
# the h5py-shaped API
# ---------------------------------------------------------------------------
class _RAttrs:
    def __init__(self, values):
        self._v = values

    def __getitem__(self, k):
        return self._v[k]

    def get(self, k, default=None):
        return self._v.get(k, default)

    def __contains__(self, k):
        return k in self._v

    def keys(self):
        return list(self._v)

    def items(self):
        return list(self._v.items())

    def __len__(self):
        return len(self._v)


class Dataset:
    """A dataset of a file open for reading; ``ds[()]`` reads it whole."""

    def __init__(self, reader, addr, msgs):
        self._r = reader
        self._info = reader.dataset_info(msgs)
        self.attrs = _RAttrs(reader.attributes(msgs))
        self.shape = self._info.get("shape")
        self.dtype = self._info.get("dtype")
        self.chunks = (self._info["layout"][2][:-1] if self._info["layout"][0] == "chunked"
                       else None)
        self.compression = ("gzip" if any(f == _F_DEFLATE for f, _ in self._info["filters"])
                            else None)

    def __getitem__(self, key):
        data = self._r.read(self._info)
        return data if key == () or key is Ellipsis else data[key]


class Group:
    """A group of a file open for reading."""

    def __init__(self, reader, addr):
        self._r = reader
        self._addr = addr
        msgs = reader.messages(addr)
        self.attrs = _RAttrs(reader.attributes(msgs))
        self._links = None

    def _children(self):
        if self._links is None:
            self._links = self._r.links(self._addr)
        return self._links

    def __getitem__(self, name):
        obj = self
        for part in [p for p in name.split("/") if p]:
            if not isinstance(obj, Group):
                raise KeyError(name)
            addr = obj._children()[part]
            msgs = self._r.messages(addr)
            if any(t in (_M_STAB, _M_LINK, _M_LINFO) for t, _, _ in msgs) or \
                    not any(t == _M_LAYOUT for t, _, _ in msgs):
                obj = Group(self._r, addr)
            else:
                obj = Dataset(self._r, addr, msgs)
        return obj

    def __contains__(self, name):
        try:
            self[name]
            return True
        except KeyError:
            return False

    def keys(self):
        return sorted(self._children())

    def __iter__(self):
        return iter(self.keys())


class File:
    """``File(path, "w")`` builds the file in memory and writes it on close;
    ``File(path, "r")`` maps it and reads objects on access."""

    def __init__(self, path, mode="r", *, leaf_k=None, internal_k=16):
        self.path = os.fspath(path)
        self.mode = mode
        if mode == "w":
            self._w = _WGroup()
            self.attrs = self._w.attrs
            self._opts = (leaf_k, internal_k)
        elif mode == "r":
            self._r = _Reader(self.path)
            self._root = Group(self._r, self._r.root)
            self.attrs = self._root.attrs
        else:
            raise ValueError("mode must be 'r' or 'w'")

    def __getattr__(self, name):
        if name in ("create_group", "create_dataset", "require_group"):
            if self.mode != "w":
                raise ValueError("file opened read-only")
            return getattr(self._w, name)
        raise AttributeError(name)

    def __getitem__(self, name):
        return self._w[name] if self.mode == "w" else self._root[name]

    def __contains__(self, name):
        return name in (self._w if self.mode == "w" else self._root)

    def keys(self):
        return self._w.keys() if self.mode == "w" else self._root.keys()

    def close(self):
        if self.mode == "w" and self._w is not None:
            _serialize(self._w, self.path, *self._opts)
            self._w = None
        elif self.mode == "r" and self._r is not None:
            self._root = None
            self._r.close()
            self._r = None

    def __enter__(self):
        return self

    def __exit__(self, exc_type, *exc):
        if exc_type is not None and self.mode == "w":
            self._w = None          # nothing is written after an error
        self.close()
