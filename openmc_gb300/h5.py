"""A small HDF5 reader and writer for the files this path exchanges with the
reference's tools: incident-neutron nuclide files (``docs/source/io_formats/
nuclear_data.rst``) and statepoints (``statepoint.rst``).

libhdf5 and h5py are not available here, so the subset of the HDF5 file
format (version 2 specification) that these files use is implemented from
the format specification:

* superblock version 0 (written) and 0/1/2/3 (read), 8-byte offsets and
  lengths;
* groups in the original "symbol table" form (a version-1 B-tree of group
  nodes, symbol-table nodes and a local heap of names), as h5py writes by
  default; compact "link message" groups are read too;
* object headers version 1 (written) and 1/2 (read), with continuation
  blocks;
* datasets with contiguous or compact storage (no chunking or filters);
* datatypes: little-endian IEEE floats, signed and unsigned integers, and
  fixed-length strings (enumerations are read as their base integers);
  attributes with the same datatypes.

Reading returns a tree of :class:`Group` objects whose ``attrs`` and
children (sub-groups or numpy arrays) can be indexed like h5py's.  Writing
takes a nested dict (see :func:`write`).
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF

# object header message types
MSG_NIL, MSG_DATASPACE, MSG_LINK_INFO, MSG_DATATYPE, MSG_FILL_OLD, MSG_FILL = 0, 1, 2, 3, 4, 5
MSG_LINK, MSG_LAYOUT, MSG_GROUP_INFO, MSG_ATTRIBUTE, MSG_CONTINUATION, MSG_SYMBOL_TABLE = 6, 8, 10, 12, 16, 17


class H5Error(ValueError):
    pass


class Group(dict):
    """A group: child name -> Group or numpy array, plus ``attrs``."""

    def __init__(self):
        super().__init__()
        self.attrs = {}

    def __getitem__(self, path):
        node = self
        for part in str(path).strip("/").split("/"):
            if part:
                node = dict.__getitem__(node, part)
        return node


# ---------------------------------------------------------------- reading
class _Reader:
    def __init__(self, buf: bytes):
        self.b = buf

    def u(self, off, n):
        return int.from_bytes(self.b[off:off + n], "little")

    # -- superblock
    def root(self):
        b = self.b
        base = b.find(SIGNATURE)
        if base != 0:
            raise H5Error("not an HDF5 file (signature not at offset 0)")
        ver = b[8]
        if ver in (0, 1):
            so, sl = b[13], b[14]
            if so != 8 or sl != 8:
                raise H5Error("only 8-byte offsets and lengths are supported")
            off = 24 + (4 if ver == 1 else 0)
            off += 8 * 4  # base, free space, EOF, driver addresses
            # root symbol table entry: name offset, object header address
            return self.u(off + 8, 8)
        if ver in (2, 3):
            so, sl = b[9], b[10]
            if so != 8 or sl != 8:
                raise H5Error("only 8-byte offsets and lengths are supported")
            return self.u(12 + 8 * 3, 8)
        raise H5Error(f"superblock version {ver} is not supported")

    # -- object headers
    def messages(self, addr):
        b = self.b
        out = []
        if b[addr:addr + 4] == b"OHDR":
            ver, flags = b[addr + 4], b[addr + 5]
            off = addr + 6
            if flags & 0x20:
                off += 16
            if flags & 0x10:
                off += 4
            size_len = 1 << (flags & 3)
            chunk = self.u(off, size_len)
            off += size_len
            blocks = [(off, chunk)]  # the checksum follows the chunk
            while blocks:
                start, length = blocks.pop(0)
                p, end = start, start + length
                while p + 4 <= end:
                    mtype, msize, mflags = b[p], self.u(p + 1, 2), b[p + 3]
                    p += 4
                    if flags & 0x04:
                        p += 2
                    if mtype == MSG_CONTINUATION:
                        caddr, clen = self.u(p, 8), self.u(p + 8, 8)
                        if b[caddr:caddr + 4] != b"OCHK":
                            raise H5Error("bad continuation block")
                        blocks.append((caddr + 4, clen - 8))
                    else:
                        out.append((mtype, mflags, p, msize))
                    p += msize
            return out
        ver = b[addr]
        if ver != 1:
            raise H5Error(f"object header version {ver} is not supported")
        nmsg, hsize = self.u(addr + 2, 2), self.u(addr + 8, 4)
        blocks = [(addr + 16, hsize)]
        count = 0
        while blocks and count < nmsg:
            start, length = blocks.pop(0)
            p, end = start, start + length
            while p + 8 <= end and count < nmsg:
                mtype, msize, mflags = self.u(p, 2), self.u(p + 2, 2), b[p + 4]
                p += 8
                count += 1
                if mtype == MSG_CONTINUATION:
                    blocks.append((self.u(p, 8), self.u(p + 8, 8)))
                else:
                    out.append((mtype, mflags, p, msize))
                p += msize
        return out

    # -- datatypes, dataspaces, data
    def datatype(self, p):
        b = self.b
        cls, ver = b[p] & 0x0F, b[p] >> 4
        bits0 = b[p + 1]
        size = self.u(p + 4, 4)
        if cls == 0:  # fixed point
            if bits0 & 1:
                raise H5Error("big-endian integers are not supported")
            signed = bool(bits0 & 0x08)
            return np.dtype(f"<{'i' if signed else 'u'}{size}")
        if cls == 1:  # floating point
            if bits0 & 1 or size not in (4, 8):
                raise H5Error("only little-endian IEEE floats are supported")
            return np.dtype(f"<f{size}")
        if cls == 3:  # fixed-length string
            return np.dtype(f"S{size}")
        if cls == 8:  # enumeration (h5py's booleans): read as its base integer type
            return self.datatype(p + 8)
        raise H5Error(f"datatype class {cls} is not supported")

    def dataspace(self, p):
        b = self.b
        ver, ndim = b[p], b[p + 1]
        if ver == 1:
            q = p + 8
        elif ver == 2:
            if b[p + 3] == 2:  # null dataspace
                return None
            q = p + 4
        else:
            raise H5Error(f"dataspace version {ver} is not supported")
        return tuple(self.u(q + 8 * k, 8) for k in range(ndim))

    def read_values(self, dtype, shape, addr_or_bytes):
        n = int(np.prod(shape)) if shape else 1
        if isinstance(addr_or_bytes, int):
            if addr_or_bytes == UNDEF:
                data = np.zeros(n, dtype)
            else:
                data = np.frombuffer(self.b, dtype, n, addr_or_bytes).copy()
        else:
            data = np.frombuffer(addr_or_bytes, dtype, n).copy()
        return data.reshape(shape) if shape else data[0]

    def attribute(self, p):
        b = self.b
        ver = b[p]
        name_size, dt_size, ds_size = self.u(p + 2, 2), self.u(p + 4, 2), self.u(p + 6, 2)
        if ver == 1:
            pad = lambda n: (n + 7) & ~7
            q = p + 8
            name = b[q:q + name_size].split(b"\0")[0].decode()
            q += pad(name_size)
            dtype = self.datatype(q)
            q += pad(dt_size)
            shape = self.dataspace(q)
            q += pad(ds_size)
        elif ver in (2, 3):
            q = p + 8 + (1 if ver == 3 else 0)
            name = b[q:q + name_size].split(b"\0")[0].decode()
            q += name_size
            dtype = self.datatype(q)
            q += dt_size
            shape = self.dataspace(q)
            q += ds_size
        else:
            raise H5Error(f"attribute version {ver} is not supported")
        n = int(np.prod(shape)) if shape else 1
        return name, self.read_values(dtype, shape, self.b[q:q + n * dtype.itemsize])

    def layout(self, p):
        b = self.b
        ver, cls = b[p], b[p + 1]
        if ver != 3:
            raise H5Error(f"data layout version {ver} is not supported")
        if cls == 0:
            size = self.u(p + 2, 2)
            return bytes(b[p + 4:p + 4 + size])
        if cls == 1:
            return self.u(p + 2, 8)
        raise H5Error("chunked or virtual datasets are not supported")

    # -- objects
    def obj(self, addr):
        msgs = self.messages(addr)
        types = {m[0] for m in msgs}
        if MSG_LAYOUT in types:
            return self.dataset(msgs)
        g = Group()
        for mtype, _, p, _ in msgs:
            if mtype == MSG_ATTRIBUTE:
                k, v = self.attribute(p)
                g.attrs[k] = v
            elif mtype == MSG_SYMBOL_TABLE:
                for name, child in self.symbol_table(self.u(p, 8), self.u(p + 8, 8)):
                    dict.__setitem__(g, name, self.obj(child))
            elif mtype == MSG_LINK:
                name, child = self.link(p)
                if child is not None:
                    dict.__setitem__(g, name, self.obj(child))
            elif mtype == MSG_LINK_INFO:
                if self.u(p + 2 + (8 if self.b[p + 1] & 1 else 0), 8) != UNDEF:
                    raise H5Error("groups with dense link storage are not supported")
        return g

    def dataset(self, msgs):
        dtype = shape = where = None
        attrs = {}
        for mtype, _, p, _ in msgs:
            if mtype == MSG_DATATYPE:
                dtype = self.datatype(p)
            elif mtype == MSG_DATASPACE:
                shape = self.dataspace(p)
            elif mtype == MSG_LAYOUT:
                where = self.layout(p)
            elif mtype == MSG_ATTRIBUTE:
                k, v = self.attribute(p)
                attrs[k] = v
        value = np.asarray(self.read_values(dtype, shape, where))
        if attrs:
            value = _Dataset(value, attrs)
        return value

    def link(self, p):
        b = self.b
        flags = b[p + 1]
        q = p + 2
        ltype = 0
        if flags & 0x08:
            ltype = b[q]
            q += 1
        if flags & 0x04:
            q += 8
        if flags & 0x10:
            q += 1
        nlen_size = 1 << (flags & 3)
        nlen = self.u(q, nlen_size)
        q += nlen_size
        name = b[q:q + nlen].decode()
        q += nlen
        if ltype != 0:
            return name, None  # soft / external links are not followed
        return name, self.u(q, 8)

    def symbol_table(self, btree, heap):
        b = self.b
        if b[heap:heap + 4] != b"HEAP":
            raise H5Error("bad local heap")
        data = self.u(heap + 24, 8)

        def name_at(off):
            end = b.index(b"\0", data + off)
            return b[data + off:end].decode()

        out = []

        def walk(node):
            if b[node:node + 4] != b"TREE":
                raise H5Error("bad B-tree node")
            level, used = b[node + 5], self.u(node + 6, 2)
            p = node + 24 + 8  # past the header and key 0
            for _ in range(used):
                child = self.u(p, 8)
                p += 16
                if level > 0:
                    walk(child)
                else:
                    if b[child:child + 4] != b"SNOD":
                        raise H5Error("bad symbol table node")
                    n = self.u(child + 6, 2)
                    for k in range(n):
                        e = child + 8 + 40 * k
                        out.append((name_at(self.u(e, 8)), self.u(e + 8, 8)))

        walk(btree)
        return out


class _Dataset(np.ndarray):
    """A numpy array that also carries the dataset's attributes."""

    def __new__(cls, value, attrs):
        obj = np.asarray(value).view(cls)
        obj.attrs = attrs
        return obj

    def __array_finalize__(self, obj):
        self.attrs = getattr(obj, "attrs", {})


def read(path) -> Group:
    """The whole file as a tree of :class:`Group` and numpy arrays."""
    buf = Path(path).read_bytes()
    r = _Reader(buf)
    return r.obj(r.root())


# ---------------------------------------------------------------- writing
class Dataset:
    """A dataset to write: a value with attributes."""

    def __init__(self, value, attrs=None):
        self.value = value
        self.attrs = dict(attrs or {})


def _as_array(v):
    if isinstance(v, (bytes, np.bytes_)):
        return np.array(v, dtype=f"S{max(len(v), 1)}")
    if isinstance(v, str):
        b = v.encode()
        return np.array(b, dtype=f"S{max(len(b), 1)}")
    a = np.asarray(v)
    if a.dtype.kind == "U":
        a = a.astype("S")
    if a.dtype.kind == "b":
        a = a.astype(np.int8)
    if a.dtype.kind in "iu" and a.dtype.itemsize < 4:
        a = a.astype(np.int32 if a.dtype.kind == "i" else np.uint32)
    if a.dtype.kind == "f" and a.dtype.itemsize not in (4, 8):
        a = a.astype(np.float64)
    return a.astype(a.dtype.newbyteorder("<"), order="C")  # keeps 0-d arrays scalar


def _datatype_msg(dt: np.dtype) -> bytes:
    if dt.kind in "iu":
        bits = 0x08 if dt.kind == "i" else 0
        return bytes([0x10 | 0, bits, 0, 0]) + struct.pack("<IHH", dt.itemsize, 0, dt.itemsize * 8)
    if dt.kind == "f":
        if dt.itemsize == 8:
            return (bytes([0x10 | 1, 0x20, 63, 0]) + struct.pack("<IHHBBBBI", 8, 0, 64, 52, 11, 0, 52, 1023))
        return (bytes([0x10 | 1, 0x20, 31, 0]) + struct.pack("<IHHBBBBI", 4, 0, 32, 23, 8, 0, 23, 127))
    if dt.kind == "S":
        return bytes([0x10 | 3, 0x00, 0, 0]) + struct.pack("<I", dt.itemsize)  # null-terminated ASCII
    raise H5Error(f"cannot write dtype {dt}")


def _dataspace_msg(shape) -> bytes:
    out = bytes([1, len(shape), 0, 0]) + b"\0" * 4
    return out + b"".join(struct.pack("<Q", n) for n in shape)


def _pad8(b: bytes) -> bytes:
    return b + b"\0" * (-len(b) % 8)


class _Writer:
    LEAF_K = 64      # symbols per symbol-table node: 2 K
    INTERNAL_K = 16  # children per B-tree node: 2 K

    def __init__(self):
        self.buf = bytearray(b"\0" * 96)  # superblock, filled in last

    def alloc(self, data: bytes) -> int:
        addr = len(self.buf)
        self.buf += data
        self.buf += b"\0" * (-len(self.buf) % 8)
        return addr

    def header(self, msgs) -> int:
        """Version-1 object header holding (type, payload) messages."""
        body = b""
        for mtype, payload in msgs:
            payload = _pad8(payload)
            body += struct.pack("<HHB3x", mtype, len(payload), 0) + payload
        if not msgs:
            body = struct.pack("<HHB3x", MSG_NIL, 8, 0) + b"\0" * 8
            msgs = [(MSG_NIL, b"")]
        prefix = struct.pack("<BxHII", 1, len(msgs), 1, len(body)) + b"\0" * 4
        return self.alloc(prefix + body)

    def attr_msg(self, name, value) -> bytes:
        a = _as_array(value)
        nb = name.encode() + b"\0"
        dt, ds = _datatype_msg(a.dtype), _dataspace_msg(a.shape)
        head = struct.pack("<BxHHH", 1, len(nb), len(dt), len(ds))
        return head + _pad8(nb) + _pad8(dt) + _pad8(ds) + a.tobytes()

    def dataset(self, value, attrs) -> int:
        a = _as_array(value)
        addr = self.alloc(a.tobytes()) if a.nbytes else UNDEF
        layout = struct.pack("<BBQQ", 3, 1, addr, a.nbytes)
        fill = bytes([2, 2, 2, 0])  # version 2: allocation late, write if set, no fill value defined
        msgs = [(MSG_DATASPACE, _dataspace_msg(a.shape)), (MSG_DATATYPE, _datatype_msg(a.dtype)),
                (MSG_FILL, fill), (MSG_LAYOUT, layout)]
        msgs += [(MSG_ATTRIBUTE, self.attr_msg(k, v)) for k, v in attrs.items()]
        return self.header(msgs)

    def group(self, names, children, attrs):
        """A symbol-table group of the given (sorted) member names and their
        object header addresses; returns (header, B-tree, local heap)."""
        cap = 2 * self.LEAF_K
        if len(names) > cap * 2 * self.INTERNAL_K:
            raise H5Error(f"groups of more than {cap * 2 * self.INTERNAL_K} members are not supported")
        # local heap: "" at offset 0, then the names
        heap_data = b"\0" * 8
        offs = []
        for name in names:
            offs.append(len(heap_data))
            heap_data += _pad8(name.encode() + b"\0")
        heap_data += b"\0" * 8
        data_addr = self.alloc(heap_data)
        heap = self.alloc(b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap_data), UNDEF, data_addr))
        # symbol-table nodes of up to 2 LEAF_K members each, in name order
        snods, last = [], []
        for k0 in range(0, max(len(names), 1), cap):
            part = list(zip(offs, children))[k0:k0 + cap]
            snod = b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(part))
            for off, child in part:
                snod += struct.pack("<QQII16x", off, child, 0, 0)
            snod += b"\0" * (40 * (cap - len(part)))
            snods.append(self.alloc(snod))
            last.append(part[-1][0] if part else 0)
        # a one-level B-tree over them (keys: the heap offsets of "" and of
        # each node's last name)
        tree = b"TREE" + bytes([0, 0]) + struct.pack("<H", len(snods)) + struct.pack("<QQ", UNDEF, UNDEF)
        tree += struct.pack("<Q", 0)
        for a, key in zip(snods, last):
            tree += struct.pack("<QQ", a, key)
        tree += b"\0" * (16 * (2 * self.INTERNAL_K - len(snods)))
        tree_addr = self.alloc(tree)
        msgs = [(MSG_SYMBOL_TABLE, struct.pack("<QQ", tree_addr, heap))]
        msgs += [(MSG_ATTRIBUTE, self.attr_msg(k, v)) for k, v in attrs.items()]
        return self.header(msgs), tree_addr, heap

    def finish(self, root_addr, root_tree, root_heap) -> bytes:
        sb = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0])
        sb += struct.pack("<HHI", self.LEAF_K, self.INTERNAL_K, 0)
        sb += struct.pack("<QQQQ", 0, UNDEF, len(self.buf), UNDEF)
        sb += struct.pack("<QQII", 0, root_addr, 1, 0) + struct.pack("<QQ", root_tree, root_heap)
        assert len(sb) == 96
        self.buf[:96] = sb
        return bytes(self.buf)


class Node(dict):
    """A group to write: child name -> Node, Dataset or array-like, plus
    ``attrs``."""

    def __init__(self, children=None, attrs=None):
        super().__init__(children or {})
        self.attrs = dict(attrs or {})


def write(path, root: Node) -> None:
    """Write a tree of :class:`Node` (groups), :class:`Dataset` and
    array-likes (datasets without attributes) as an HDF5 file."""
    w = _Writer()

    def group(node):
        names = sorted(node)
        children = []
        for name in names:
            v = node[name]
            if isinstance(v, Node):
                children.append(group(v)[0])
            elif isinstance(v, Dataset):
                children.append(w.dataset(v.value, v.attrs))
            else:
                children.append(w.dataset(v, {}))
        return w.group(names, children, node.attrs)

    root_addr, tree, heap = group(root)
    Path(path).write_bytes(w.finish(root_addr, tree, heap))
