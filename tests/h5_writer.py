"""Test infrastructure: writes HDF5 files with the structures the HDF5
library uses by default (and so h5py and Keras's save_weights): superblock
version 0, version-1 object headers, groups as symbol tables (a version-1
B-tree leaf over symbol table nodes of at most 2K = 8 entries, names in a
local heap), contiguous datasets and version-1 attributes. Follows the
published HDF5 file format specification; used to check the reader in
nerf-tf2_gb300/h5.py on the Keras weight-file layout."""
import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
LEAF_K = 4  # group leaf node K: 2K = 8 entries per symbol table node


def _pad8(b):
    return b + b"\0" * (-len(b) % 8)


def _datatype(dt):
    dt = np.dtype(dt)
    if dt.kind == "f":
        if dt.itemsize == 4:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
        else:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
        bits = bytes([0x20 | (1 if dt.byteorder == ">" else 0), dt.itemsize * 8 - 1, 0])
        return bytes([0x11]) + bits + struct.pack("<I", dt.itemsize) + props
    if dt.kind == "S":
        return bytes([0x13, 0x01, 0, 0]) + struct.pack("<I", dt.itemsize)  # null-padded ASCII
    if dt.kind in "iu":
        bits = bytes([0x08 if dt.kind == "i" else 0, 0, 0])
        return bytes([0x10]) + bits + struct.pack("<I", dt.itemsize) + struct.pack("<HH", 0, dt.itemsize * 8)
    raise ValueError(dt)


def _dataspace(shape):
    return struct.pack("<BBBB4x", 1, len(shape), 0, 0) + b"".join(struct.pack("<Q", n) for n in shape)


def _attribute(name, value):
    a = np.asarray(value)
    if a.dtype.kind == "U":
        a = np.char.encode(a, "utf-8")
    nm = name.encode() + b"\0"
    dt, ds = _datatype(a.dtype), _dataspace(a.shape)
    head = struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(ds))
    return head + _pad8(nm) + _pad8(dt) + _pad8(ds) + np.ascontiguousarray(a).tobytes()


class Writer:
    def __init__(self, userblock=0):
        self.userblock = userblock
        self.buf = bytearray(96)  # the superblock, filled in by close()

    def _alloc(self, data):
        self.buf += b"\0" * (-len(self.buf) % 8)
        addr = len(self.buf)
        self.buf += data
        return addr

    def _header(self, messages):
        body = b""
        for mtype, data in messages:
            data = _pad8(data)
            body += struct.pack("<HHB3x", mtype, len(data), 0) + data
        return self._alloc(struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body)

    def dataset(self, value, attrs=None):
        a = np.ascontiguousarray(value)
        raw = self._alloc(a.tobytes())
        msgs = [(0x0001, _dataspace(a.shape)), (0x0003, _datatype(a.dtype)),
                (0x0008, struct.pack("<BBQQ", 3, 1, raw, a.nbytes))]
        msgs += [(0x000C, _attribute(k, v)) for k, v in (attrs or {}).items()]
        return ("dataset", self._header(msgs))

    def group(self, members, attrs=None):
        """members: {name: ("dataset"|"group", header address[, (btree, heap)])}."""
        names = sorted(members)
        seg = b"\0" * 8  # offset 0: the empty name
        offs = {}
        for nm in names:
            offs[nm] = len(seg)
            seg += _pad8(nm.encode() + b"\0")
        seg_addr = self._alloc(seg)
        heap = self._alloc(b"HEAP" + struct.pack("<B3xQQQ", 0, len(seg), UNDEF, seg_addr))
        nodes, keys = [], [0]
        for i in range(0, max(len(names), 1), 2 * LEAF_K):
            chunk = names[i:i + 2 * LEAF_K]
            entries = b""
            for nm in chunk:
                m = members[nm]
                cache, scratch = (1, struct.pack("<QQ", *m[2])) if m[0] == "group" else (0, b"\0" * 16)
                entries += struct.pack("<QQII", offs[nm], m[1], cache, 0) + scratch
            entries += b"\0" * (40 * (2 * LEAF_K - len(chunk)))
            nodes.append(self._alloc(b"SNOD" + struct.pack("<BBH", 1, 0, len(chunk)) + entries))
            keys.append(offs[chunk[-1]] if chunk else 0)
        tree = b"TREE" + struct.pack("<BBHQQ", 0, 0, len(nodes), UNDEF, UNDEF)
        for k in range(len(nodes)):
            tree += struct.pack("<QQ", keys[k], nodes[k])
        tree += struct.pack("<Q", keys[-1])
        btree = self._alloc(tree)
        msgs = [(0x0011, struct.pack("<QQ", btree, heap))]
        msgs += [(0x000C, _attribute(k, v)) for k, v in (attrs or {}).items()]
        return ("group", self._header(msgs), (btree, heap))

    def close(self, path, root):
        sb = b"\x89HDF\r\n\x1a\n" + struct.pack("<BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, LEAF_K, 16, 0)
        sb += struct.pack("<QQQQ", self.userblock, UNDEF, len(self.buf), UNDEF)
        sb += struct.pack("<QQII", 0, root[1], 1, 0) + struct.pack("<QQ", *root[2])
        assert len(sb) == 96
        self.buf[:96] = sb
        with open(path, "wb") as f:
            f.write(b"\0" * self.userblock + bytes(self.buf))


def write_nested(w, tree, attrs_of=None, prefix=""):
    """tree: {name: ndarray or subtree}; attrs_of(path) -> attribute dict."""
    members = {}
    for name, v in tree.items():
        path = prefix + "/" + name
        if isinstance(v, dict):
            members[name] = write_nested(w, v, attrs_of, path)
        else:
            members[name] = w.dataset(v)
    return w.group(members, attrs_of(prefix or "/") if attrs_of else None)


def write_keras_weights(path, layers, split_layer_names=False, userblock=0):
    """A Keras save_weights file (hdf5_format.save_weights_to_hdf5_group):
    root attributes layer_names, backend, keras_version; one group per layer
    (a "/" in a layer name nests groups) with the attribute weight_names and
    one dataset per weight under its full name (nested again).
    layers: [(layer name, [(weight name, array), ...]), ...], layers without
    weights included (empty list)."""
    tree, wnames = {}, {}
    for lname, ws in layers:
        node = tree
        for part in lname.split("/"):
            node = node.setdefault(part, {})
        wnames["/" + lname] = [w for w, _ in ws]
        for wname, arr in ws:
            sub = node
            parts = wname.split("/")
            for part in parts[:-1]:
                sub = sub.setdefault(part, {})
            sub[parts[-1]] = arr
    names = np.array([ln.encode() for ln, _ in layers])

    def attrs_of(p):
        if p == "/":
            a = {"backend": np.bytes_(b"tensorflow"), "keras_version": np.bytes_(b"2.6.0")}
            if split_layer_names:
                h = len(names) // 2
                a["layer_names0"], a["layer_names1"] = names[:h], names[h:]
            else:
                a["layer_names"] = names
            return a
        if p in wnames:
            w = wnames[p]
            return {"weight_names": np.array([x.encode() for x in w]) if w else np.asarray([])}
        return {}

    w = Writer(userblock)
    root = write_nested(w, tree, attrs_of)
    w.close(path, root)
