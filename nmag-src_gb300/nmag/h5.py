"""A small HDF5 reader and writer for the files nmag exchanges: the
``.nmesh.h5`` mesh (nmeshlib/lib1.py:805-863, written by
nfem/hdf5_v01.py:1370-1545 through PyTables) and other plain datasets.

Written from the HDF5 file format specification (the structures of the
HDF5 1.6/1.8 library's default output, which PyTables writes):

* superblock versions 0 and 1 (read and write) and 2/3 (read);
* object headers version 1 (read and write) and 2 (read), with
  continuation blocks;
* groups as symbol tables (version 1 B-tree of symbol-table nodes and a
  local heap; read and write) and compact link messages (read);
* datasets with contiguous, compact and chunked layout (layout message
  versions 1-3; chunks indexed by a version 1 B-tree) and the deflate,
  shuffle and Fletcher-32 filters;
* fixed-point, floating-point, fixed-length string, compound and array
  datatypes; attributes (message versions 1-3).

Variable-length data, references, the version 4 layout's chunk indices,
dense (fractal-heap) link and attribute storage and external storage are
outside this subset and raise ``NotImplementedError``.

Reading::

    f = File("bar.nmesh.h5")
    pts = f["/mesh/points"].read()

Writing::

    w = Writer()
    w.create_dataset("/mesh/points", pts, chunks=(1024, 3), compression=5,
                     attrs={"CLASS": "CARRAY", "VERSION": "1.0", "TITLE": "..."})
    w.save("bar.nmesh.h5")
"""
from __future__ import annotations

import os
import struct
import zlib

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class HDF5Error(Exception):
    pass


# ---------------------------------------------------------------- reading --

class _Buf(object):
    """The file's bytes and its address size."""

    def __init__(self, data, so=8, sl=8, base=0):
        self.d = data
        self.so, self.sl, self.base = so, sl, base

    def u(self, pos, n):
        return int.from_bytes(self.d[pos:pos + n], "little")

    def addr(self, pos):
        a = self.u(pos, self.so)
        return UNDEF if a == (1 << (8 * self.so)) - 1 else a + self.base

    def length(self, pos):
        return self.u(pos, self.sl)

    def cstr(self, pos):
        end = self.d.index(b"\0", pos)
        return self.d[pos:end].decode("latin-1")


def _round8(n):
    return (n + 7) & ~7


def _dtype(b, pos):
    """The numpy dtype of the datatype message at pos, and its encoded size."""
    cls, ver = b.d[pos] & 0x0F, b.d[pos] >> 4
    bits = b.u(pos + 1, 3)
    size = b.u(pos + 4, 4)
    p = pos + 8
    if cls == 0:   # fixed point
        order = ">" if bits & 1 else "<"
        kind = "i" if bits & 8 else "u"
        return np.dtype("%s%s%d" % (order, kind, size)), 8 + 4
    if cls == 1:   # floating point
        order = ">" if bits & 1 else "<"
        if size not in (2, 4, 8):
            raise NotImplementedError("HDF5: floating point of %d bytes" % size)
        return np.dtype("%sf%d" % (order, size)), 8 + 12
    if cls == 3:   # fixed-length string
        return np.dtype("S%d" % size), 8
    if cls == 6:   # compound
        nmemb = bits & 0xFFFF
        names, formats, offsets = [], [], []
        for _ in range(nmemb):
            name = b.cstr(p)
            if ver < 3:
                p += _round8(len(name) + 1)
                off = b.u(p, 4)
                p += 4
                shape = ()
                if ver == 1:
                    ndim = b.d[p]
                    dims = [b.u(p + 12 + 4 * k, 4) for k in range(ndim)]
                    shape = tuple(dims)
                    p += 28
            else:
                p += len(name) + 1
                nb = 1 if size < 256 else (2 if size < 65536 else (3 if size < (1 << 24) else 4))
                off = b.u(p, nb)
                p += nb
                shape = ()
            mdt, mlen = _dtype(b, p)
            p += mlen
            names.append(name)
            formats.append((mdt, shape) if shape else mdt)
            offsets.append(off)
        return np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": size}), p - pos
    if cls == 4:   # bitfield: unsigned integers of its size
        order = ">" if bits & 1 else "<"
        return np.dtype("%su%d" % (order, size)), 8 + 4
    if cls == 5:   # opaque: raw bytes, then its tag (padded to 8)
        taglen = bits & 0xFF
        return np.dtype("V%d" % size), 8 + taglen
    if cls == 8:   # enumeration: its base integer type, then names and values
        nmemb = bits & 0xFFFF
        base, blen = _dtype(b, p)
        q = p + blen
        for _ in range(nmemb):
            name = b.cstr(q)
            q += _round8(len(name) + 1) if ver < 3 else len(name) + 1
        q += nmemb * base.itemsize
        return base, q - pos
    if cls == 10:  # array
        ndim = b.d[p]
        if ver < 3:
            dims = tuple(b.u(p + 4 + 4 * k, 4) for k in range(ndim))
            q = p + 4 + 8 * ndim
        else:
            dims = tuple(b.u(p + 1 + 4 * k, 4) for k in range(ndim))
            q = p + 1 + 4 * ndim
        base, blen = _dtype(b, q)
        return np.dtype((base, dims)), q + blen - pos
    raise NotImplementedError("HDF5: datatype class %d" % cls)


def _dataspace(b, pos):
    ver, rank, flags = b.d[pos], b.d[pos + 1], b.d[pos + 2]
    if ver == 1:
        p = pos + 8
    elif ver == 2:
        if b.d[pos + 3] == 2:   # null dataspace
            return None
        p = pos + 4
    else:
        raise NotImplementedError("HDF5: dataspace version %d" % ver)
    return tuple(b.length(p + b.sl * k) for k in range(rank))


def _messages(b, addr):
    """The (type, data offset, size) of every message of the object header at addr."""
    out = []
    if b.d[addr:addr + 4] == b"OHDR":   # version 2 header
        flags = b.d[addr + 5]
        p = addr + 6
        if flags & 0x20:
            p += 16
        if flags & 0x10:
            p += 4
        nsz = 1 << (flags & 3)
        chunk = b.u(p, nsz)
        p += nsz
        blocks = [(p, p + chunk)]   # the chunk's checksum follows it
        cre = bool(flags & 0x04)
        hsz = 6 if cre else 4
        seen = 0
        while blocks:
            seen += 1
            if seen > 4096:
                raise HDF5Error("HDF5: object header at %d does not end" % addr)
            start, end = blocks.pop(0)
            q = start
            while q + hsz <= end:
                mtype, msize = b.d[q], b.u(q + 1, 2)
                q += hsz
                if mtype == 0x10:
                    ca, cl = b.addr(q), b.length(q + b.so)
                    blocks.append((ca + 4, ca + cl - 4))   # "OCHK" ... checksum
                elif mtype:
                    out.append((mtype, q, msize))
                q += msize
        return out
    if b.d[addr] != 1:
        raise HDF5Error("HDF5: object header version %d at %d" % (b.d[addr], addr))
    nmsg = b.u(addr + 2, 2)
    size = b.u(addr + 8, 4)
    blocks = [(addr + 16, addr + 16 + size)]
    seen = 0
    while blocks and len(out) < nmsg:
        seen += 1
        if seen > 4096:   # continuation blocks that loop: a damaged file
            raise HDF5Error("HDF5: object header at %d does not end" % addr)
        start, end = blocks.pop(0)
        q = start
        while q + 8 <= end:
            mtype, msize = b.u(q, 2), b.u(q + 2, 2)
            if mtype == 0x10:
                blocks.append((b.addr(q + 8), b.addr(q + 8) + b.length(q + 8 + b.so)))
            elif mtype:
                out.append((mtype, q + 8, msize))
            q += 8 + msize
    return out


def _attributes(b, msgs):
    attrs = {}
    for mtype, p, _ in msgs:
        if mtype != 0x0C:
            continue
        try:
            name, value = _attribute(b, p)
        except (NotImplementedError, ValueError, IndexError):
            continue   # an attribute outside the subset (e.g. variable-length): not read
        attrs[name] = value
    return attrs


def _attribute(b, p):
    """(name, value) of the attribute message at p."""
    ver = b.d[p]
    nlen, tlen, slen = b.u(p + 2, 2), b.u(p + 4, 2), b.u(p + 6, 2)
    if ver == 1:
        q = p + 8
        name = b.d[q:q + nlen].split(b"\0")[0].decode("latin-1")
        q += _round8(nlen)
        dt, _ = _dtype(b, q)
        q += _round8(tlen)
        shape = _dataspace(b, q)
        q += _round8(slen)
    else:
        q = p + 8 + (1 if ver == 3 else 0)
        name = b.d[q:q + nlen].split(b"\0")[0].decode("latin-1")
        q += nlen
        dt, _ = _dtype(b, q)
        q += tlen
        shape = _dataspace(b, q)
        q += slen
    if shape is None:
        return name, None
    n = int(np.prod(shape)) if shape else 1
    val = np.frombuffer(b.d, dtype=dt, count=n, offset=q).reshape(shape)
    if dt.kind == "S":
        val = val.astype(str)
    return name, (val[()] if shape == () else val)


class Node(object):
    def __init__(self, f, addr, name):
        self.file, self.addr, self.name = f, addr, name
        self._msgs = _messages(f.b, addr)
        self.attrs = _attributes(f.b, self._msgs)

    def _msg(self, mtype):
        for t, p, s in self._msgs:
            if t == mtype:
                return p, s
        return None


class Group(Node):
    """A group: its members by name (symbol table or compact links)."""

    def _links(self):
        b = self.file.b
        links = {}
        st = self._msg(0x11)
        if st is not None:
            p, _ = st
            _group_btree(b, b.addr(p), b.addr(p + b.so), links)
        for t, p, _ in self._msgs:
            if t == 0x06:
                flags = b.d[p + 1]
                q = p + 2
                ltype = 0
                if flags & 0x08:
                    ltype = b.d[q]
                    q += 1
                if flags & 0x04:
                    q += 8
                if flags & 0x10:
                    q += 1
                nsz = 1 << (flags & 3)
                nlen = b.u(q, nsz)
                q += nsz
                name = b.d[q:q + nlen].decode("utf-8")
                q += nlen
                if ltype == 0:
                    links[name] = b.addr(q)
            elif t == 0x02:
                fh = b.addr(p + 2 + (8 if b.d[p + 1] & 1 else 0))
                if fh != UNDEF:
                    raise NotImplementedError("HDF5: dense link storage (fractal heap)")
        return links

    def keys(self):
        return sorted(self._links())

    def __contains__(self, name):
        return name in self._links()

    def __getitem__(self, path):
        node = self.file if path.startswith("/") else self   # absolute paths start at the root
        for part in [s for s in path.split("/") if s]:
            links = node._links()
            if part not in links:
                raise KeyError("HDF5: no member '%s' in '%s'" % (part, node.name))
            node = node.file._node(links[part], (node.name.rstrip("/") + "/" + part))
        return node


def _group_btree(b, addr, heap, links):
    """Walk a group's version 1 B-tree; names come from the local heap."""
    if b.d[addr:addr + 4] != b"TREE":
        raise HDF5Error("HDF5: no group B-tree at %d" % addr)
    level, used = b.d[addr + 5], b.u(addr + 6, 2)
    hdata = b.addr(heap + 8 + 2 * b.sl)   # the heap's data segment
    p = addr + 8 + 2 * b.so + b.sl        # after the first key
    for _ in range(used):
        child = b.addr(p)
        p += b.so + b.sl
        if level > 0:
            _group_btree(b, child, heap, links)
            continue
        if b.d[child:child + 4] != b"SNOD":
            raise HDF5Error("HDF5: no symbol table node at %d" % child)
        n = b.u(child + 6, 2)
        e = child + 8
        esize = 2 * b.so + 24
        for k in range(n):
            q = e + k * esize
            links[b.cstr(hdata + b.u(q, b.so))] = b.addr(q + b.so)


class Dataset(Node):
    """A dataset: shape, dtype, attributes and read()."""

    @property
    def shape(self):
        m = self._msg(0x01)
        return _dataspace(self.file.b, m[0]) if m else None

    @property
    def dtype(self):
        return _dtype(self.file.b, self._msg(0x03)[0])[0]

    def _filters(self):
        m = self._msg(0x0B)
        if m is None:
            return []
        b = self.file.b
        p, _ = m
        ver, n = b.d[p], b.d[p + 1]
        q = p + (8 if ver == 1 else 2)
        out = []
        for _ in range(n):
            fid = b.u(q, 2)
            if ver == 1 or fid >= 256:
                nlen = b.u(q + 2, 2)
                flags, nval = b.u(q + 4, 2), b.u(q + 6, 2)
                q += 8
                q += _round8(nlen) if ver == 1 else nlen
            else:
                flags, nval = b.u(q + 2, 2), b.u(q + 4, 2)
                q += 6
            vals = [b.u(q + 4 * k, 4) for k in range(nval)]
            q += 4 * nval
            if ver == 1 and nval % 2:
                q += 4
            out.append((fid, vals))
        return out

    def read(self):
        b = self.file.b
        shape, dt = self.shape, self.dtype
        if shape is None:
            return None
        n = int(np.prod(shape)) if shape else 1
        p, _ = self._msg(0x08)
        ver = b.d[p]
        if ver in (1, 2):
            ndim, cls = b.d[p + 1], b.d[p + 2]
            q = p + 8
            if cls == 1:
                raw = b.addr(q)
                out = np.frombuffer(b.d, dtype=dt, count=n, offset=raw) if raw != UNDEF else np.zeros(n, dt)
                return out.reshape(shape).copy()
            if cls == 0:
                q += 4 * ndim
                return np.frombuffer(b.d, dtype=dt, count=n, offset=q + 4).reshape(shape).copy()
            bt = b.addr(q)
            cdims = tuple(b.u(q + b.so + 4 * k, 4) for k in range(ndim))
            return self._chunked(bt, cdims[:-1], shape, dt)
        if ver == 3:
            cls = b.d[p + 1]
            if cls == 0:
                return np.frombuffer(b.d, dtype=dt, count=n, offset=p + 4).reshape(shape).copy()
            if cls == 1:
                raw = b.addr(p + 2)
                if raw == UNDEF:
                    return np.zeros(shape, dt)
                return np.frombuffer(b.d, dtype=dt, count=n, offset=raw).reshape(shape).copy()
            if cls == 2:
                ndim = b.d[p + 2]
                bt = b.addr(p + 3)
                cdims = tuple(b.u(p + 3 + b.so + 4 * k, 4) for k in range(ndim))
                return self._chunked(bt, cdims[:-1], shape, dt)
        raise NotImplementedError("HDF5: data layout version %d" % ver)

    def _chunked(self, bt, cdims, shape, dt):
        b = self.file.b
        out = np.zeros(shape, dt)
        filters = self._filters()
        rank = len(shape)

        def walk(addr):
            if b.d[addr:addr + 4] != b"TREE" or b.d[addr + 4] != 1:
                raise HDF5Error("HDF5: no chunk B-tree at %d" % addr)
            level, used = b.d[addr + 5], b.u(addr + 6, 2)
            ksize = 8 + 8 * (rank + 1)
            p = addr + 8 + 2 * b.so
            for _ in range(used):
                csize, mask = b.u(p, 4), b.u(p + 4, 4)
                offs = [b.u(p + 8 + 8 * k, 8) for k in range(rank)]
                child = b.addr(p + ksize)
                p += ksize + b.so
                if level > 0:
                    walk(child)
                    continue
                data = bytes(b.d[child:child + csize])
                for k in range(len(filters) - 1, -1, -1):
                    if mask & (1 << k):
                        continue
                    data = _unfilter(filters[k], data, dt.itemsize)
                chunk = np.frombuffer(data, dtype=dt, count=int(np.prod(cdims))).reshape(cdims)
                sl_out = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, shape))
                sl_in = tuple(slice(0, x.stop - x.start) for x in sl_out)
                out[sl_out] = chunk[sl_in]

        if bt != UNDEF:
            walk(bt)
        return out


def _unfilter(flt, data, itemsize):
    fid, vals = flt
    if fid == 1:   # deflate
        return zlib.decompress(data)
    if fid == 2:   # shuffle: byte planes back to elements
        n = len(data) // itemsize
        head = np.frombuffer(data[:n * itemsize], dtype=np.uint8).reshape(itemsize, n)
        return head.T.tobytes() + data[n * itemsize:]
    if fid == 3:   # Fletcher-32: the checksum is the last 4 bytes
        return data[:-4]
    raise NotImplementedError("HDF5: filter %d" % fid)


class File(Group):
    """An HDF5 file opened for reading (the whole file is held in memory)."""

    def __init__(self, path_or_bytes):
        if isinstance(path_or_bytes, (bytes, bytearray)):
            data = bytes(path_or_bytes)
        else:
            with open(path_or_bytes, "rb") as fh:
                data = fh.read()
        start = _superblock_offset(data)
        if start is None:
            raise HDF5Error("not an HDF5 file")
        ver = data[start + 8]
        if ver in (0, 1):
            so, sl = data[start + 13], data[start + 14]
            p = start + 24 + (4 if ver == 1 else 0)
            b = _Buf(data, so, sl)
            base = b.u(p, so)
            b.base = base
            root_entry = p + 4 * so
            root = b.addr(root_entry + so)
        elif ver in (2, 3):
            so, sl = data[start + 9], data[start + 10]
            b = _Buf(data, so, sl)
            p = start + 12
            b.base = b.u(p, so)
            root = b.addr(p + 3 * so)
        else:
            raise NotImplementedError("HDF5: superblock version %d" % ver)
        self.b = b
        Node.__init__(self, self, root, "/")

    def _node(self, addr, name):
        msgs = _messages(self.b, addr)
        if any(t in (0x11, 0x06, 0x02) for t, _, _ in msgs) and not any(t == 0x08 for t, _, _ in msgs):
            return Group(self, addr, name)
        return Dataset(self, addr, name)


def _superblock_offset(data):
    """Where the superblock starts: byte 0, or after a user block of 512,
    1024, 2048, ... bytes (files whose first bytes belong to another
    application, e.g. MATLAB's 512-byte header)."""
    for off in [0] + [512 << k for k in range(20)]:
        if off + 8 > len(data):
            break
        if data[off:off + 8] == SIGNATURE:
            return off
    return None


def is_hdf5(path):
    try:
        with open(path, "rb") as fh:
            head = fh.read(8)
            if head == SIGNATURE:
                return True
            size = os.fstat(fh.fileno()).st_size
            for off in [512 << k for k in range(20)]:
                if off + 8 > size:
                    break
                fh.seek(off)
                if fh.read(8) == SIGNATURE:
                    return True
    except IOError:
        return False
    return False


# ---------------------------------------------------------------- writing --

def _dt_msg(dt):
    """Datatype message bytes of a numpy dtype."""
    dt = np.dtype(dt)
    if dt.kind in "iu":
        bits = (1 if dt.byteorder == ">" else 0) | (8 if dt.kind == "i" else 0)
        return bytes([0x10]) + bits.to_bytes(3, "little") + struct.pack("<I", dt.itemsize) + \
            struct.pack("<HH", 0, 8 * dt.itemsize)
    if dt.kind == "f":
        n = dt.itemsize
        sign, eloc, esize, msize, bias = {4: (31, 23, 8, 23, 127), 8: (63, 52, 11, 52, 1023)}[n]
        bits = (1 if dt.byteorder == ">" else 0) | (2 << 4) | (sign << 8)
        return bytes([0x11]) + bits.to_bytes(3, "little") + struct.pack("<I", n) + \
            struct.pack("<HHBBBBI", 0, 8 * n, eloc, esize, 0, msize, bias)
    if dt.kind == "S":
        return bytes([0x13, 0, 0, 0]) + struct.pack("<I", dt.itemsize)
    if dt.kind == "V" and dt.names:   # compound, version 1 (sub-array members by their dimensions)
        body = b""
        for name in dt.names:
            mdt, off = dt.fields[name][0], dt.fields[name][1]
            shape = mdt.shape
            if len(shape) > 4:
                raise NotImplementedError("HDF5 writer: compound member of rank %d" % len(shape))
            base = mdt.base if shape else mdt
            dims = list(shape) + [0] * (4 - len(shape))
            body += _pad8(name.encode("latin-1") + b"\0") + struct.pack("<IB3xI4x", off, len(shape), 0)
            body += struct.pack("<4I", *dims) + _dt_msg(base)
        return bytes([0x16]) + len(dt.names).to_bytes(3, "little") + struct.pack("<I", dt.itemsize) + body
    raise NotImplementedError("HDF5 writer: dtype %s" % dt)


def _space_msg(shape):
    out = struct.pack("<BBBB", 1, len(shape), 0, 0) + b"\0" * 4
    for d in shape:
        out += struct.pack("<Q", d)
    return out


def _pad8(b):
    return b + b"\0" * (_round8(len(b)) - len(b))


def _msg(mtype, data, flags=0):
    data = _pad8(data)
    return struct.pack("<HHB3x", mtype, len(data), flags) + data


def _attr_msg(name, value):
    if isinstance(value, str):
        raw = value.encode("latin-1") + b"\0"
        dt, shape, data = np.dtype("S%d" % len(raw)), (), raw
    else:
        arr = np.asarray(value)
        if arr.dtype.kind == "U":
            arr = arr.astype("S")
        dt, shape, data = arr.dtype, arr.shape, arr.tobytes()
    nm = name.encode("latin-1") + b"\0"
    t, s = _dt_msg(dt), _space_msg(shape)
    body = struct.pack("<BBHHH", 1, 0, len(nm), len(t), len(s)) + _pad8(nm) + _pad8(t) + _pad8(s) + data
    return _msg(0x0C, body)


class _WGroup(object):
    def __init__(self):
        self.members = {}
        self.attrs = {}


class _WDataset(object):
    def __init__(self, data, chunks, compression, shuffle, attrs):
        self.data = np.array(data, order="C")   # keeps 0-d (scalar) data 0-d
        if self.data.dtype.kind == "U":
            self.data = self.data.astype("S")
        if self.data.dtype.byteorder == ">":
            self.data = self.data.astype(self.data.dtype.newbyteorder("<"))
        self.chunks, self.compression, self.shuffle = chunks, compression, shuffle
        self.attrs = dict(attrs or {})


class Writer(object):
    """Build groups and datasets, then save() them as an HDF5 file
    (version 0 superblock, version 1 object headers, symbol-table groups)."""

    LEAF_K, NODE_K, CHUNK_K = 4, 16, 32

    def __init__(self):
        self.root = _WGroup()

    def _parent(self, path, create=True):
        parts = [s for s in path.split("/") if s]
        g = self.root
        for part in parts[:-1]:
            if part not in g.members:
                if not create:
                    raise KeyError(path)
                g.members[part] = _WGroup()
            g = g.members[part]
        return g, parts[-1]

    def create_group(self, path, attrs=None):
        g, name = self._parent(path)
        node = g.members.setdefault(name, _WGroup())
        node.attrs.update(attrs or {})
        return node

    def create_dataset(self, path, data, chunks=None, compression=None, shuffle=False, attrs=None):
        """compression: a deflate level (0-9) or None; chunks: the chunk shape
        (required with compression or shuffle)."""
        if (compression is not None or shuffle) and chunks is None:
            raise ValueError("HDF5 writer: filters need a chunk shape")
        g, name = self._parent(path)
        g.members[name] = _WDataset(data, chunks, compression, shuffle, attrs)

    def set_attrs(self, path, attrs):
        node = self.root if path.strip("/") == "" else self._get(path)
        node.attrs.update(attrs)

    def _get(self, path):
        g, name = self._parent(path, create=False)
        return g.members[name]

    # -- serialisation: objects appended after the superblock; children first --
    def save(self, path):
        self.out = bytearray(96)   # the version 0 superblock (8-byte offsets and lengths)
        root_hdr, bt, heap = self._group(self.root)
        sb = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", self.LEAF_K, self.NODE_K, 0)
        sb += struct.pack("<QQQQ", 0, UNDEF, len(self.out), UNDEF)
        sb += struct.pack("<QQII", 0, root_hdr, 1, 0) + struct.pack("<QQ", bt, heap)
        assert len(sb) == 96
        self.out[0:96] = sb
        with open(path, "wb") as fh:
            fh.write(bytes(self.out))

    def _put(self, data, align=8):
        while len(self.out) % align:
            self.out.append(0)
        at = len(self.out)
        self.out += data
        return at

    def _header(self, msgs):
        body = b"".join(msgs)
        hdr = struct.pack("<BBHII", 1, 0, len(msgs), 1, len(body)) + b"\0" * 4 + body
        return self._put(hdr)

    def _attr_msgs(self, attrs):
        return [_attr_msg(k, v) for k, v in attrs.items()]

    def _group(self, g):
        names = sorted(g.members)
        addrs = {}
        for name in names:
            m = g.members[name]
            addrs[name] = self._group(m)[0] if isinstance(m, _WGroup) else self._dataset(m)
        # local heap: "" at offset 0, then the names
        heapdata = bytearray(8)
        offs = {}
        for name in names:
            offs[name] = len(heapdata)
            heapdata += _pad8(name.encode("latin-1") + b"\0")
        heapdata += b"\0" * 8
        hdata = self._put(bytes(heapdata))
        heap = self._put(b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heapdata), UNDEF, hdata))
        # symbol-table nodes of 2 LEAF_K entries, one level-0 B-tree over them
        cap = 2 * self.LEAF_K
        groups = [names[i:i + cap] for i in range(0, len(names), cap)] or [[]]
        if len(groups) > 2 * self.NODE_K:
            raise NotImplementedError("HDF5 writer: more than %d members in a group" % (cap * 2 * self.NODE_K))
        snods = []
        for part in groups:
            ent = b""
            for name in part:
                ent += struct.pack("<QQII", offs[name], addrs[name], 0, 0) + b"\0" * 16
            ent += b"\0" * (40 * (cap - len(part)))
            snods.append(self._put(b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(part)) + ent))
        tree = b"TREE" + bytes([0, 0]) + struct.pack("<H", len(snods)) + struct.pack("<QQ", UNDEF, UNDEF)
        tree += struct.pack("<Q", 0)
        for part, sn in zip(groups, snods):
            tree += struct.pack("<QQ", sn, offs[part[-1]] if part else 0)
        tree += b"\0" * ((2 * self.NODE_K - len(snods)) * 16)
        bt = self._put(tree)
        msgs = [_msg(0x11, struct.pack("<QQ", bt, heap))] + self._attr_msgs(g.attrs)
        return self._header(msgs), bt, heap

    def _dataset(self, d):
        arr = d.data
        shape = arr.shape
        msgs = [_msg(0x01, _space_msg(shape)), _msg(0x03, _dt_msg(arr.dtype))]
        if d.chunks is None:
            raw = self._put(arr.tobytes()) if arr.nbytes else UNDEF
            msgs.append(_msg(0x08, struct.pack("<BBQQ", 3, 1, raw, arr.nbytes)))
        else:
            msgs.extend(self._chunked(d))
        msgs += self._attr_msgs(d.attrs)
        return self._header(msgs)

    def _chunked(self, d):
        arr = d.data
        shape, cdims = arr.shape, tuple(int(c) for c in d.chunks)
        if len(cdims) != len(shape) or any(c < 1 for c in cdims):
            raise ValueError("HDF5 writer: chunk shape %s for data shape %s" % (cdims, shape))
        grid = [range(0, max(s, 1), c) for s, c in zip(shape, cdims)]
        starts = [()]
        for g in grid:
            starts = [s + (o,) for s in starts for o in g]
        if len(starts) > 2 * self.CHUNK_K:
            raise NotImplementedError("HDF5 writer: more than %d chunks" % (2 * self.CHUNK_K))
        isz = arr.dtype.itemsize
        filters = []
        if d.shuffle:
            filters.append((2, [isz]))
        if d.compression is not None:
            filters.append((1, [int(d.compression)]))
        entries = []
        for st in starts:
            chunk = np.zeros(cdims, arr.dtype)
            src = tuple(slice(o, min(o + c, s)) for o, c, s in zip(st, cdims, shape))
            chunk[tuple(slice(0, x.stop - x.start) for x in src)] = arr[src]
            data = chunk.tobytes()
            for fid, vals in filters:
                if fid == 2:
                    n = len(data) // isz
                    data = np.frombuffer(data, dtype=np.uint8).reshape(n, isz).T.tobytes()
                else:
                    data = zlib.compress(data, vals[0])
            entries.append((st, self._put(data), len(data)))
        rank = len(shape)
        tree = b"TREE" + bytes([1, 0]) + struct.pack("<H", len(entries)) + struct.pack("<QQ", UNDEF, UNDEF)
        for st, at, n in entries:
            tree += struct.pack("<II", n, 0) + b"".join(struct.pack("<Q", o) for o in st + (0,)) + struct.pack("<Q", at)
        tree += struct.pack("<II", 0, 0) + b"".join(struct.pack("<Q", s) for s in shape + (0,))
        ksize = 8 + 8 * (rank + 1)
        tree += b"\0" * ((2 * self.CHUNK_K - len(entries)) * (ksize + 8))
        bt = self._put(tree)
        layout = struct.pack("<BBBQ", 3, 2, rank + 1, bt) + b"".join(struct.pack("<I", c) for c in cdims + (isz,))
        msgs = [_msg(0x08, layout)]
        if filters:
            body = struct.pack("<BB6x", 1, len(filters))
            for fid, vals in filters:
                body += struct.pack("<HHHH", fid, 0, 0 if fid == 2 else 1, len(vals))
                body += b"".join(struct.pack("<I", v) for v in vals) + (b"\0" * 4 if len(vals) % 2 else b"")
            msgs.append(_msg(0x0B, body))
        return msgs
