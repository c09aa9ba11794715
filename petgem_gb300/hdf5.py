"""Minimal HDF5 writer and reader for petgem's result files, with no HDF5 library.

petgem writes its receiver responses with h5py (petgem/postprocessing.py:
341-461): groups ``machine`` and ``model`` (and sub-groups such as
``model/E-fields``) holding scalar and 1-D datasets of strings, integers,
booleans, floats and complex numbers.  This module writes the same layout in
the classic HDF5 file format that h5py produces with its default settings, so
a petgem user's h5py / HDF5 tools read the file unchanged:

* superblock version 0 (8-byte offsets and lengths, group leaf K 4, group
  internal K 16);
* groups as symbol tables: a version-1 B-tree (group nodes), symbol-table
  nodes of up to 8 entries sorted by name, and a local heap of names;
* version-1 object headers; datasets carry a dataspace (version 1, with
  maximum dimensions), a datatype (version 1), a fill-value message
  (version 2), a contiguous layout (version 3) and a modification time;
* datatypes: IEEE f64 / signed i64 little-endian, fixed-length UTF-8
  strings (null padded), h5py's boolean enum (FALSE = 0, TRUE = 1 over int8)
  and h5py's complex compound {"r": f64, "i": f64}.

``read`` parses the same subset (and the files h5py writes in it, such as
petgem's ``tests/data/receiver_pos.h5``) into {path: numpy array}.
"""
import struct
import time

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"
LEAF_K = 4            # symbol-table node: up to 2 * LEAF_K entries
INTERNAL_K = 16       # group B-tree node: up to 2 * INTERNAL_K children


def _pad8(b):
    return b + b"\0" * (-len(b) % 8)


# ------------------------------------------------------------------ datatypes
def _dt_float64():
    return bytes([0x11, 0x20, 0x3F, 0x00]) + struct.pack("<I", 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)


def _dt_int(size, signed=True):
    return bytes([0x10, 0x08 if signed else 0x00, 0, 0]) + struct.pack("<I", size) + struct.pack("<HH", 0, 8 * size)


def _dt_string(n):
    return bytes([0x13, 0x11, 0, 0]) + struct.pack("<I", n)          # null padded, UTF-8


def _dt_bool():
    names = _pad8(b"FALSE\0") + _pad8(b"TRUE\0")
    return bytes([0x18, 2, 0, 0]) + struct.pack("<I", 1) + _dt_int(1) + names + bytes([0, 1])


def _dt_complex128():
    out = bytes([0x16, 2, 0, 0]) + struct.pack("<I", 16)
    for name, off in ((b"r", 0), (b"i", 8)):
        out += _pad8(name + b"\0") + struct.pack("<IB3xI4x4I", off, 0, 0, 0, 0, 0, 0) + _dt_float64()
    return out


def _encode(value):
    """(datatype message, shape, raw little-endian bytes) for a value."""
    if isinstance(value, (str, bytes)):
        b = value.encode("utf-8") if isinstance(value, str) else value
        b = b or b"\0"
        return _dt_string(len(b)), (), b
    a = np.asarray(value)
    if a.dtype.kind in "US":
        items = [s.encode("utf-8") if isinstance(s, str) else bytes(s) for s in a.reshape(-1).tolist()]
        n = max(1, max((len(s) for s in items), default=1))
        raw = b"".join(s + b"\0" * (n - len(s)) for s in items)
        return _dt_string(n), a.shape, raw
    if a.dtype == np.bool_:
        return _dt_bool(), a.shape, a.astype(np.int8).tobytes()
    if a.dtype.kind == "c":
        c = np.ascontiguousarray(a.astype(np.complex128))
        return _dt_complex128(), a.shape, c.view(np.float64).astype("<f8").tobytes()
    if a.dtype.kind in "iu":
        return _dt_int(8), a.shape, np.ascontiguousarray(a.astype("<i8")).tobytes()
    if a.dtype.kind == "f":
        return _dt_float64(), a.shape, np.ascontiguousarray(a.astype("<f8")).tobytes()
    raise TypeError(f"unsupported dataset type {a.dtype}")


# ------------------------------------------------------------------ writer
class _File:
    def __init__(self):
        self.buf = bytearray()

    def alloc(self, n, align=8):
        self.buf += b"\0" * (-len(self.buf) % align)
        at = len(self.buf)
        self.buf += b"\0" * n
        return at

    def put(self, at, data):
        self.buf[at:at + len(data)] = data


def _message(mtype, data, flags=0):
    data = _pad8(data)
    return struct.pack("<HHB3x", mtype, len(data), flags) + data


def _object_header(f, messages):
    body = b"".join(messages)
    at = f.alloc(16 + len(body))
    f.put(at, struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body)
    return at


def _write_dataset(f, value):
    dtype, shape, raw = _encode(value)
    rank = len(shape)
    space = struct.pack("<BBBB4x", 1, rank, 1 if rank else 0, 0)
    if rank:
        space += struct.pack(f"<{rank}Q", *shape) + struct.pack(f"<{rank}Q", *shape)
    data_at = f.alloc(len(raw))
    f.put(data_at, raw)
    msgs = [_message(0x0001, space),
            _message(0x0003, dtype, flags=1),
            _message(0x0005, bytes([2, 2, 2, 1]) + struct.pack("<I", 0), flags=1),
            _message(0x0008, struct.pack("<BBQQ", 3, 1, data_at, len(raw))),
            _message(0x0012, struct.pack("<B3xI", 1, int(time.time())))]
    return _object_header(f, msgs)


def _write_group(f, tree):
    """Write a group (dict name -> subtree or value); returns (object header,
    B-tree, heap) addresses."""
    names = sorted(tree, key=lambda s: s.encode("utf-8"))
    children = {}
    for name in names:
        v = tree[name]
        if isinstance(v, dict):
            children[name] = (1,) + _write_group(f, v)
        else:
            children[name] = (0, _write_dataset(f, v), 0, 0)
    # local heap: "" at offset 0, the names, then one free block (next-free
    # offset 1 = none, size) as h5py leaves it
    heap = bytearray(8)
    offs = {}
    for name in names:
        offs[name] = len(heap)
        heap += _pad8(name.encode("utf-8") + b"\0")
    free_at = len(heap)
    heap += struct.pack("<QQ", 1, 16)
    heap_data = f.alloc(len(heap))
    f.put(heap_data, bytes(heap))
    heap_at = f.alloc(32)
    f.put(heap_at, b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap), free_at, heap_data))
    # symbol-table nodes of up to 2 * LEAF_K sorted entries (none for an empty group)
    chunks = [names[i:i + 2 * LEAF_K] for i in range(0, len(names), 2 * LEAF_K)]
    if len(chunks) > 2 * INTERNAL_K:
        raise ValueError(f"a group of more than {2 * LEAF_K * 2 * INTERNAL_K} entries is not supported")
    snods = []
    for ch in chunks:
        node = bytearray(b"SNOD" + struct.pack("<BBH", 1, 0, len(ch)))
        for name in ch:
            kind, hdr, bt, hp = children[name]
            node += struct.pack("<QQI4x", offs[name], hdr, kind) + struct.pack("<QQ", bt, hp)
        node += b"\0" * (8 + 2 * LEAF_K * 40 - len(node))
        at = f.alloc(len(node))
        f.put(at, bytes(node))
        snods.append((at, offs[ch[-1]]))
    # one B-tree node (level 0) over the symbol-table nodes
    tree_node = bytearray(b"TREE" + struct.pack("<BBHQQ", 0, 0, len(snods), UNDEF, UNDEF))
    tree_node += struct.pack("<Q", 0)
    for at, last in snods:
        tree_node += struct.pack("<QQ", at, last)
    tree_node += b"\0" * (24 + (2 * INTERNAL_K + 1) * 8 + 2 * INTERNAL_K * 8 - len(tree_node))
    bt_at = f.alloc(len(tree_node))
    f.put(bt_at, bytes(tree_node))
    hdr_at = _object_header(f, [_message(0x0011, struct.pack("<QQ", bt_at, heap_at))])
    return hdr_at, bt_at, heap_at


def write(path, datasets):
    """Write {"group/sub/name": value} (str, bool, int, float, complex, or a
    1-D array of them) as an HDF5 file in petgem's layout."""
    tree = {}
    for key, v in datasets.items():
        parts = [p for p in key.split("/") if p]
        node = tree
        for g in parts[:-1]:
            node = node.setdefault(g, {})
            if not isinstance(node, dict):
                raise ValueError(f"{key}: {g} is a dataset, not a group")
        node[parts[-1]] = v
    f = _File()
    f.alloc(96)                                       # superblock, written last
    root_hdr, root_bt, root_heap = _write_group(f, tree)
    f.buf += b"\0" * (-len(f.buf) % 8)
    sb = SIGNATURE + struct.pack("<BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, LEAF_K, INTERNAL_K, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, len(f.buf), UNDEF)
    sb += struct.pack("<QQI4xQQ", 0, root_hdr, 1, root_bt, root_heap)
    f.put(0, sb)
    with open(path, "wb") as fh:
        fh.write(bytes(f.buf))
    return path


# ------------------------------------------------------------------ reader
def _u(b, at, fmt):
    return struct.unpack_from("<" + fmt, b, at)


def _decode_dtype(b, at):
    """(numpy dtype or "bool"/"str:n"/"complex", size) from a datatype encoding."""
    cls, v = b[at] & 0x0F, b[at] >> 4
    bits = b[at + 1] | (b[at + 2] << 8) | (b[at + 3] << 16)
    size = _u(b, at + 4, "I")[0]
    if cls == 0:
        return np.dtype(("<" if not bits & 1 else ">") + ("i" if bits & 8 else "u") + str(size)), 8 + 4
    if cls == 1:
        return np.dtype(("<" if not bits & 1 else ">") + "f" + str(size)), 8 + 12
    if cls == 3:
        return f"str:{size}", 8
    if cls == 8:
        return "bool", None
    if cls == 6:
        nm = bits & 0xFFFF
        p = at + 8
        fields = []
        for _ in range(nm):
            e = b.index(b"\0", p)
            name = b[p:e].decode()
            if v == 1:
                p += (e - p + 8) // 8 * 8
                off = _u(b, p, "I")[0]
                p += 32            # offset, rank, reserved, permutation, reserved, 4 sizes
            else:
                p = e + 1
                off = int.from_bytes(b[p:p + 4], "little")
                p += 4
            dt, n = _decode_dtype(b, p)
            fields.append((name, dt, off))
            p += n
        if [f[0] for f in fields] == ["r", "i"] and size == 16:
            return "complex", p - at
        return np.dtype({"names": [f[0] for f in fields], "formats": [f[1] for f in fields],
                         "offsets": [f[2] for f in fields], "itemsize": size}), p - at
    raise ValueError(f"unsupported HDF5 datatype class {cls}")


def _read_object(b, at):
    ver, nmsg, _, hsize = _u(b, at, "BxHII")
    if ver != 1:
        raise ValueError("only version-1 object headers are supported")
    p, end = at + 16, at + 16 + hsize
    msgs = {}
    while p + 8 <= end and len(msgs) < nmsg + 1:
        mtype, msize, _ = _u(b, p, "HHB")
        msgs.setdefault(mtype, p + 8)
        p += 8 + msize
    return msgs


def _group_entries(b, bt_at, heap_at):
    heap_data = _u(b, heap_at + 24, "Q")[0]
    out = []

    def node(at):
        assert b[at:at + 4] == b"TREE", "B-tree node expected"
        _, level, used = _u(b, at + 4, "BBH")
        for i in range(used):
            child = _u(b, at + 24 + 8 + 16 * i, "Q")[0]
            if level > 0:
                node(child)
            else:
                assert b[child:child + 4] == b"SNOD", "symbol-table node expected"
                n = _u(b, child + 6, "H")[0]
                for j in range(n):
                    e = child + 8 + 40 * j
                    name_off, hdr = _u(b, e, "QQ")
                    s = heap_data + name_off
                    out.append((b[s:b.index(b"\0", s)].decode(), hdr))
    node(bt_at)
    return out


def _read_dataset(b, msgs):
    sp = msgs[0x0001]
    ver, rank = b[sp], b[sp + 1]
    shape = tuple(_u(b, sp + (8 if ver == 1 else 4), f"{rank}Q")) if rank else ()
    dt, _ = _decode_dtype(b, msgs[0x0003])
    lay = msgs[0x0008]
    if b[lay] != 3:
        raise ValueError("only version-3 layout messages are supported")
    if b[lay + 1] == 1:
        addr, size = _u(b, lay + 2, "QQ")
        raw = b[addr:addr + size] if addr != UNDEF else b""
    elif b[lay + 1] == 0:
        size = _u(b, lay + 2, "H")[0]
        raw = b[lay + 4:lay + 4 + size]
    else:
        raise ValueError("chunked datasets are not supported")
    if dt == "complex":
        a = np.frombuffer(raw, dtype="<f8").copy().view(np.complex128)
    elif dt == "bool":
        a = np.frombuffer(raw, dtype=np.int8).astype(bool)
    elif isinstance(dt, str) and dt.startswith("str:"):
        n = int(dt[4:])
        items = [raw[i:i + n].rstrip(b"\0").decode("utf-8") for i in range(0, len(raw), n)]
        return items[0] if not shape else np.array(items).reshape(shape)
    else:
        a = np.frombuffer(raw, dtype=dt).copy()
    a = a.reshape(shape)
    return a[()] if not shape else a


def read(path):
    """{"group/name": value} of every dataset in a classic-format HDF5 file."""
    with open(path, "rb") as fh:
        b = fh.read()
    if b[:8] != SIGNATURE or b[8] != 0:
        raise ValueError("not an HDF5 file with a version-0 superblock")
    root_hdr = _u(b, 0x38 + 8, "Q")[0]
    out = {}

    def walk(hdr, prefix):
        msgs = _read_object(b, hdr)
        if 0x0011 in msgs:
            bt, hp = _u(b, msgs[0x0011], "QQ")
            for name, child in _group_entries(b, bt, hp):
                walk(child, prefix + name + "/")
        else:
            out[prefix[:-1]] = _read_dataset(b, msgs)
    walk(root_hdr, "")
    return out
