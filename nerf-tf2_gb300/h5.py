"""Read-only HDF5 for Keras weight files (nerf/core/model.py:278-287 loads
them with Keras's load_weights; nerf/core/ops.py:142-143 writes them).

h5py is not available, so this restates the published HDF5 file format
(The HDF Group, "HDF5 File Format Specification") for the structures the
HDF5 library writes by default, which is what h5py (and so Keras's
save_weights) produces:

* superblock versions 0 and 1 (8-byte offsets and lengths), with a user
  block before it;
* groups stored as symbol tables: a version-1 B-tree of group nodes whose
  leaves are symbol table nodes (SNOD), link names in a local heap;
* version-1 object headers, with continuation blocks;
* messages: dataspace (versions 1, 2), datatype (fixed-point, IEEE
  floating-point, fixed-length strings), data layout (versions 1-3;
  contiguous or compact), attributes (versions 1-3), symbol table.

Anything else (version-2 object headers and superblocks, new-style link
groups, chunked or filtered data, variable-length or shared types, soft
links) raises NotImplementedError rather than being misread.
"""
import struct

import numpy as np

_SIGNATURE = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(ValueError):
    """The file is not HDF5 or is damaged."""


def _pad8(n):
    return (n + 7) & ~7


class _Reader:
    def __init__(self, data):
        self.d = data
        self.base = self._find_superblock()
        sv = self.d[self.base + 8]
        if sv not in (0, 1):
            raise NotImplementedError(f"HDF5 superblock version {sv} (only 0 and 1)")
        so, sl = self.d[self.base + 13], self.d[self.base + 14]
        if (so, sl) != (8, 8):
            raise NotImplementedError(f"HDF5 offsets/lengths of {so}/{sl} bytes (only 8/8)")
        off = self.base + 24 + (4 if sv == 1 else 0)
        base_addr, _, eof, _ = struct.unpack_from("<4Q", self.d, off)
        # addresses in the file are relative to the base address (the
        # superblock's position when a user block precedes it)
        self.addr0 = base_addr
        self.root_entry = struct.unpack_from("<QQII16s", self.d, off + 32)

    def _find_superblock(self):
        pos = 0
        while pos + 8 <= len(self.d):
            if self.d[pos:pos + 8] == _SIGNATURE:
                return pos
            pos = 512 if pos == 0 else pos * 2  # 0, 512, 1024, 2048, ...
        raise H5Error("no HDF5 signature")

    def at(self, addr):
        if addr == _UNDEF:
            raise H5Error("undefined address")
        a = self.addr0 + addr
        if a >= len(self.d):
            raise H5Error(f"address {addr} beyond the end of the file")
        return a

    def u(self, fmt, addr):
        return struct.unpack_from("<" + fmt, self.d, self.at(addr))

    # -- local heap, B-tree, symbol table nodes --
    def heap_string(self, heap_addr, offset):
        a = self.at(heap_addr)
        if self.d[a:a + 4] != b"HEAP":
            raise H5Error("bad local heap")
        seg_size, _, seg_addr = struct.unpack_from("<QQQ", self.d, a + 8)
        if offset >= seg_size:
            raise H5Error("heap offset out of range")
        s = self.at(seg_addr) + offset
        end = self.d.index(b"\0", s)
        return self.d[s:end].decode("utf-8")

    def group_entries(self, btree_addr, heap_addr):
        a = self.at(btree_addr)
        if self.d[a:a + 4] != b"TREE":
            raise H5Error("bad B-tree node")
        node_type, level, used = self.d[a + 4], self.d[a + 5], struct.unpack_from("<H", self.d, a + 6)[0]
        if node_type != 0:
            raise H5Error("not a group B-tree")
        out = []
        pos = a + 24  # after the signature, type, level, entries, siblings
        for _ in range(used):
            _key, child = struct.unpack_from("<QQ", self.d, pos)
            pos += 16
            if level > 0:
                out += self.group_entries(child, heap_addr)
            else:
                out += self.snod_entries(child, heap_addr)
        return out

    def snod_entries(self, addr, heap_addr):
        a = self.at(addr)
        if self.d[a:a + 4] != b"SNOD":
            raise H5Error("bad symbol table node")
        n = struct.unpack_from("<H", self.d, a + 6)[0]
        out = []
        for i in range(n):
            name_off, obj_addr, cache, _, _scratch = struct.unpack_from("<QQII16s", self.d, a + 8 + 40 * i)
            if cache == 2:
                raise NotImplementedError("HDF5 soft links")
            out.append((self.heap_string(heap_addr, name_off), obj_addr))
        return out

    # -- object headers --
    def messages(self, addr):
        a = self.at(addr)
        if self.d[a:a + 4] == b"OHDR":
            raise NotImplementedError("HDF5 version-2 object headers")
        version, _, nmsg, _, size = struct.unpack_from("<BBHII", self.d, a)
        if version != 1:
            raise H5Error(f"object header version {version}")
        blocks, msgs = [(a + 16, size)], []
        while blocks and len(msgs) < nmsg:
            start, length = blocks.pop(0)
            pos = start
            while pos + 8 <= start + length and len(msgs) < nmsg:
                mtype, msize, flags = struct.unpack_from("<HHB", self.d, pos)
                body = self.d[pos + 8:pos + 8 + msize]
                if flags & 0x02:
                    raise NotImplementedError("HDF5 shared object header messages")
                if mtype == 0x0010:  # continuation
                    coff, clen = struct.unpack_from("<QQ", body)
                    blocks.append((self.at(coff), clen))
                msgs.append((mtype, body))
                pos += 8 + msize
        return msgs


def _dataspace(body):
    version, rank, flags = body[0], body[1], body[2]
    if version == 1:
        pos = 8
    elif version == 2:
        if body[3] == 2:  # null dataspace
            return None
        pos = 4
    else:
        raise NotImplementedError(f"HDF5 dataspace version {version}")
    return tuple(struct.unpack_from("<" + "Q" * rank, body, pos)) if rank else ()


def _datatype(body):
    cls, version = body[0] & 0x0F, body[0] >> 4
    bits = body[1] | (body[2] << 8) | (body[3] << 16)
    size = struct.unpack_from("<I", body, 4)[0]
    if cls == 0:  # fixed-point
        order = ">" if bits & 1 else "<"
        kind = "i" if bits & 0x08 else "u"
        if size not in (1, 2, 4, 8):
            raise NotImplementedError(f"HDF5 integer of {size} bytes")
        return np.dtype(order + kind + str(size))
    if cls == 1:  # IEEE floating point
        if bits & 0x40:
            raise NotImplementedError("VAX-order floats")
        order = ">" if bits & 1 else "<"
        _, prec, eloc, esize, mloc, msize, bias = struct.unpack_from("<HHBBBBI", body, 8)
        std = {4: (32, 23, 8, 0, 23, 127), 2: (16, 10, 5, 0, 10, 15), 8: (64, 52, 11, 0, 52, 1023)}
        if std.get(size) != (prec, eloc, esize, mloc, msize, bias):
            raise NotImplementedError("non-IEEE floating-point layout")
        return np.dtype(order + "f" + str(size))
    if cls == 3:  # fixed-length string
        return np.dtype("S" + str(size))
    raise NotImplementedError(f"HDF5 datatype class {cls} (version {version})")


def _read_values(raw, dtype, shape):
    n = int(np.prod(shape)) if shape else 1
    need = n * dtype.itemsize
    if len(raw) < need:
        raise H5Error("data shorter than its dataspace")
    a = np.frombuffer(raw[:need], dtype=dtype).copy()
    return a.reshape(shape) if shape else a.reshape(())


def _attribute(body):
    version = body[0]
    if version == 1:
        name_size, dt_size, ds_size = struct.unpack_from("<HHH", body, 2)
        pos = 8
        name = body[pos:pos + name_size].split(b"\0")[0].decode("utf-8")
        pos += _pad8(name_size)
        dt = body[pos:pos + dt_size]
        pos += _pad8(dt_size)
        ds = body[pos:pos + ds_size]
        pos += _pad8(ds_size)
    elif version in (2, 3):
        flags = body[1]
        if flags & 0x03:
            raise NotImplementedError("HDF5 shared attribute datatype/dataspace")
        name_size, dt_size, ds_size = struct.unpack_from("<HHH", body, 2)
        pos = 8 if version == 2 else 9
        name = body[pos:pos + name_size].split(b"\0")[0].decode("utf-8")
        pos += name_size
        dt = body[pos:pos + dt_size]
        pos += dt_size
        ds = body[pos:pos + ds_size]
        pos += ds_size
    else:
        raise NotImplementedError(f"HDF5 attribute version {version}")
    dtype, shape = _datatype(dt), _dataspace(ds)
    if shape is None:
        return name, None
    return name, _read_values(body[pos:], dtype, shape)


class Dataset:
    """A dataset: .shape, .dtype, .attrs, and read() / numpy conversion."""

    def __init__(self, r, msgs, name):
        self._r, self.name = r, name
        self.attrs = {}
        self.shape, self.dtype, self._layout = None, None, None
        for t, body in msgs:
            if t == 0x0001:
                self.shape = _dataspace(body)
            elif t == 0x0003:
                self.dtype = _datatype(body)
            elif t == 0x0008:
                self._layout = body
            elif t == 0x000B:
                raise NotImplementedError("HDF5 filters (compressed data)")
            elif t == 0x000C:
                k, v = _attribute(body)
                self.attrs[k] = v

    def read(self):
        if self.shape is None:
            return None
        n = int(np.prod(self.shape)) * self.dtype.itemsize
        b = self._layout
        version = b[0]
        if version in (1, 2):
            rank, cls = b[1], b[2]
            if cls == 1:  # contiguous
                addr = struct.unpack_from("<Q", b, 8)[0]
                raw = None if addr == _UNDEF else self._r.d[self._r.at(addr):self._r.at(addr) + n]
            elif cls == 0:  # compact: dimension sizes, then size and data
                pos = 8 + 4 * rank
                size = struct.unpack_from("<I", b, pos)[0]
                raw = b[pos + 4:pos + 4 + size]
            else:
                raise NotImplementedError("HDF5 chunked storage")
        elif version == 3:
            cls = b[1]
            if cls == 1:
                addr, _size = struct.unpack_from("<QQ", b, 2)
                raw = None if addr == _UNDEF else self._r.d[self._r.at(addr):self._r.at(addr) + n]
            elif cls == 0:
                size = struct.unpack_from("<H", b, 2)[0]
                raw = b[4:4 + size]
            else:
                raise NotImplementedError("HDF5 chunked storage")
        else:
            raise NotImplementedError(f"HDF5 data layout version {version}")
        if raw is None:  # never written: the fill value, zero by default
            return np.zeros(self.shape, self.dtype)
        return _read_values(raw, self.dtype, self.shape)

    def __array__(self, dtype=None, copy=None):
        a = self.read()
        return a if dtype is None else a.astype(dtype)


class Group:
    """A group: .attrs, members(), and g["a/b/c"] for nested paths."""

    def __init__(self, r, msgs, name):
        self._r, self.name = r, name
        self.attrs = {}
        self._table = None
        for t, body in msgs:
            if t == 0x0011:
                self._table = struct.unpack_from("<QQ", body)
            elif t in (0x0002, 0x0006):
                raise NotImplementedError("HDF5 new-style (link message) groups")
            elif t == 0x000C:
                k, v = _attribute(body)
                self.attrs[k] = v

    def members(self):
        if self._table is None:
            return {}
        return dict(self._r.group_entries(*self._table))

    def __contains__(self, path):
        try:
            self[path]
            return True
        except KeyError:
            return False

    def __getitem__(self, path):
        node = self
        for part in [p for p in path.split("/") if p]:
            if not isinstance(node, Group):
                raise KeyError(path)
            m = node.members()
            if part not in m:
                raise KeyError(path)
            node = _object(node._r, m[part], node.name.rstrip("/") + "/" + part)
        return node


def _object(r, addr, name):
    msgs = r.messages(addr)
    if any(t == 0x0011 for t, _ in msgs):
        return Group(r, msgs, name)
    if any(t == 0x0008 for t, _ in msgs):
        return Dataset(r, msgs, name)
    if any(t in (0x0002, 0x0006) for t, _ in msgs):
        raise NotImplementedError("HDF5 new-style (link message) groups")
    return Group(r, msgs, name)


def open_file(path):
    """The root group of an HDF5 file."""
    with open(path, "rb") as f:
        r = _Reader(f.read())
    return _object(r, r.root_entry[1], "/")


# ---------------------------------------------------------------------------
# Keras weight files
# ---------------------------------------------------------------------------
def _str_list(values):
    if values is None:
        return []
    return [v.decode("utf-8") if isinstance(v, (bytes, np.bytes_)) else str(v) for v in np.asarray(values).ravel()]


def keras_attribute(group, name):
    """Keras's load_attributes_from_hdf5_group: the attribute `name`, or,
    when Keras split a long list, name0, name1, ... concatenated."""
    if name in group.attrs:
        return _str_list(group.attrs[name])
    out, k = [], 0
    while f"{name}{k}" in group.attrs:
        out += _str_list(group.attrs[f"{name}{k}"])
        k += 1
    return out


def keras_layer_weights(path):
    """The weights of a Keras save_weights file, as Keras's
    load_weights_from_hdf5_group reads them: the root's layer_names, and
    for each layer that has weights its weight_names and the arrays stored
    under them. Returns [(layer name, [(weight name, array), ...]), ...] in
    the file's layer order."""
    f = open_file(path)
    if "layer_names" not in f.attrs and "layer_names0" not in f.attrs and "model_weights" in f:
        f = f["model_weights"]  # a whole-model file keeps its weights here
    out = []
    for lname in keras_attribute(f, "layer_names"):
        g = f[lname]
        wnames = keras_attribute(g, "weight_names")
        if wnames:
            out.append((lname, [(w, np.asarray(g[w])) for w in wnames]))
    return out
