"""Minimal reader for the HDF5 files elpasoC reads and writes.

elpasoC's model files (``ESC/misc/parser/femparserhdf5.cpp:202-499``, group
and dataset names in ``ESC/misc/hdf5/rulesh5.h:31-157``) and its solution
files (``ESC/analysis/frequency/analysisfrequencybasic.cpp:184-262``) are
written by HDF5 1.8-era libraries with the default file format: superblock
version 0, version-1 object headers, groups as symbol tables (v1 B-tree +
local heap), contiguous or compact dataset storage, no filters. This module
reads exactly that subset, in pure Python + numpy, following the published
HDF5 File Format Specification (version 2.0 document, sections II-IV):

* superblock v0/v1, symbol table entries, v1 group B-trees (``TREE``),
  symbol table nodes (``SNOD``) and local heaps (``HEAP``);
* object header v1 messages: dataspace (0x1), datatype (0x3), data layout
  (0x8, versions 1-3, contiguous/compact), attribute (0xC), continuation
  (0x10), symbol table (0x11);
* datatypes: fixed-point, floating-point, fixed- and variable-length strings
  (the latter in global heap collections, ``GCOL``), enumerations (read as
  their base integer type, the members in the dtype's metadata; booleans
  are the ``{FALSE, TRUE}`` enum of a byte) and compounds of those (the
  elpasoC complex type is the compound ``{real, imag}``).

Anything else (chunked or filtered storage, v2 object headers, dense
attribute storage, variable-length types) raises ``NotImplementedError``.

``Writer`` produces files in the same subset (superblock 0, v1 object
headers, symbol-table groups with full-size v1 B-tree nodes of K = 16 and
symbol nodes of K = 4 -- up to 8,192 links per group --, contiguous datasets
of float64 / int32 / int64 / complex128 stored as the compound {real, imag}
/ structured arrays of those (compounds, e.g. elpasoC's node table),
scalar int64 / float64 / fixed-length string attributes). The image this was
built in has no HDF5 library, so files are checked by a round trip through
``File`` only.
"""
from __future__ import annotations

import struct

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF


class Dataset:
    """A dataset: ``shape``, numpy ``dtype``, ``attrs`` and lazy ``read()``."""

    def __init__(self, f: "File", addr: int, msgs):
        self._f = f
        self.addr = addr
        self.attrs = {}
        self.shape = ()
        self.dtype = None
        self._layout = None
        for mtype, data in msgs:
            if mtype == 0x1:
                self.shape = f._dataspace(data)
            elif mtype == 0x3:
                self.dtype = f._datatype(data, 0)[0]
            elif mtype == 0x8:
                self._layout = data
            elif mtype == 0xC:
                k, v = f._attribute(data)
                self.attrs[k] = v

    def read(self) -> np.ndarray:
        count = int(np.prod(self.shape)) if self.shape else 1
        nbytes = count * self.dtype.itemsize
        raw = self._f._layout_bytes(self._layout, nbytes)
        if raw is None:
            return np.zeros(self.shape, self.dtype)
        arr = np.frombuffer(raw, self.dtype, count)
        if self.dtype.metadata and self.dtype.metadata.get("vlen_str"):
            arr = np.array([self._f._vlen_str(r) for r in arr], dtype=object)
        return arr.reshape(self.shape).copy()


class Group:
    """A group: ``keys()``, ``[name]`` (nested paths allowed) and ``attrs``."""

    def __init__(self, f: "File", addr: int, msgs):
        self._f = f
        self.addr = addr
        self.attrs = {}
        self._links = {}
        for mtype, data in msgs:
            if mtype == 0x11:
                btree, heap = struct.unpack_from("<QQ", data, 0)
                self._links = f._group_links(btree, heap)
            elif mtype == 0xC:
                k, v = f._attribute(data)
                self.attrs[k] = v

    def keys(self):
        return list(self._links)

    def __contains__(self, name):
        try:
            self[name]
            return True
        except KeyError:
            return False

    def __getitem__(self, path: str):
        node = self
        for part in [p for p in path.split("/") if p]:
            if not isinstance(node, Group) or part not in node._links:
                raise KeyError(path)
            node = node._f._object(node._links[part])
        return node


class File(Group):
    """Opens an HDF5 file held in memory; the root group of the file."""

    def __init__(self, path: str):
        with open(path, "rb") as fh:
            self._b = fh.read()
        b = self._b
        if b[:8] != _SIG:
            raise ValueError(f"{path}: not an HDF5 file")
        ver = b[8]
        if ver not in (0, 1):
            raise NotImplementedError(f"superblock version {ver}")
        self._so, self._sl = b[13], b[14]
        if (self._so, self._sl) != (8, 8):
            raise NotImplementedError("offsets/lengths other than 8 bytes")
        pos = 24 + (4 if ver == 1 else 0)
        self._base = struct.unpack_from("<Q", b, pos)[0]
        root_entry = pos + 32
        _, root_ohdr = struct.unpack_from("<QQ", b, root_entry)
        Group.__init__(self, self, root_ohdr, self._messages(root_ohdr))

    # ------------------------------------------------------------ structure
    def _object(self, addr: int):
        msgs = self._messages(addr)
        if any(t == 0x11 for t, _ in msgs):
            return Group(self, addr, msgs)
        return Dataset(self, addr, msgs)

    def _messages(self, addr: int):
        b = self._b
        a = self._base + addr
        version, _, nmsgs, _, hsize = struct.unpack_from("<BBHII", b, a)
        if version != 1:
            raise NotImplementedError(f"object header version {version}")
        blocks = [(a + 16, hsize)]
        out = []
        while blocks and len(out) < nmsgs:
            start, size = blocks.pop(0)
            p = start
            while p + 8 <= start + size and len(out) < nmsgs:
                mtype, msize, _flags = struct.unpack_from("<HHB", b, p)
                data = b[p + 8:p + 8 + msize]
                p += 8 + msize
                if mtype == 0x10:
                    caddr, clen = struct.unpack_from("<QQ", data, 0)
                    blocks.append((self._base + caddr, clen))
                out.append((mtype, data))
        return out

    def _group_links(self, btree: int, heap: int):
        b = self._b
        h = self._base + heap
        if b[h:h + 4] != b"HEAP":
            raise ValueError("bad local heap")
        heap_data = struct.unpack_from("<Q", b, h + 24)[0] + self._base
        links = {}

        def name_at(off):
            e = b.index(b"\0", heap_data + off)
            return b[heap_data + off:e].decode()

        def walk(node):
            n = self._base + node
            sig = b[n:n + 4]
            if sig == b"TREE":
                _ntype, level, used = struct.unpack_from("<BBH", b, n + 4)
                p = n + 8 + 16 + 8  # siblings, then key 0
                for _ in range(used):
                    child = struct.unpack_from("<Q", b, p)[0]
                    walk(child)
                    p += 16  # child + next key
            elif sig == b"SNOD":
                nsym = struct.unpack_from("<H", b, n + 6)[0]
                p = n + 8
                for _ in range(nsym):
                    name_off, ohdr = struct.unpack_from("<QQ", b, p)
                    links[name_at(name_off)] = ohdr
                    p += 40
            else:
                raise ValueError("bad group node")

        walk(btree)
        return links

    # ------------------------------------------------------------ messages
    @staticmethod
    def _dataspace(d: bytes):
        version, rank = d[0], d[1]
        if version == 1:
            p = 8
        elif version == 2:
            p = 4
        else:
            raise NotImplementedError(f"dataspace version {version}")
        return tuple(struct.unpack_from("<Q", d, p + 8 * i)[0] for i in range(rank))

    def _datatype(self, d: bytes, p: int):
        """Returns (numpy dtype, bytes consumed)."""
        cls_ver = d[p]
        cls, ver = cls_ver & 0x0F, cls_ver >> 4
        bits = d[p + 1] | (d[p + 2] << 8) | (d[p + 3] << 16)
        size = struct.unpack_from("<I", d, p + 4)[0]
        q = p + 8
        if cls == 0:  # fixed point: byte order bit 0, signed bit 3
            if bits & 1:
                raise NotImplementedError("big-endian integer")
            kind = "i" if bits & 0x8 else "u"
            return np.dtype(f"<{kind}{size}"), 8 + 4
        if cls == 1:  # floating point
            if bits & 1:
                raise NotImplementedError("big-endian float")
            return np.dtype(f"<f{size}"), 8 + 12
        if cls == 3:  # fixed-length string
            return np.dtype(f"S{size}"), 8
        if cls == 9:  # variable length; strings only (type bits 0-3 == 1)
            if bits & 0xF != 1:
                raise NotImplementedError("variable-length sequence")
            _, used = self._datatype(d, q)  # base type (characters)
            dt = np.dtype([("len", "<u4"), ("heap", "<u8"), ("index", "<u4")], metadata={"vlen_str": True})
            return dt, 8 + used
        if cls == 6:  # compound
            nmem = bits & 0xFFFF
            names, formats, offsets = [], [], []
            for _ in range(nmem):
                e = d.index(b"\0", q)
                name = d[q:e].decode()
                if ver < 3:
                    q += ((e - q) // 8 + 1) * 8
                else:
                    q = e + 1
                if ver == 1:
                    off = struct.unpack_from("<I", d, q)[0]
                    q += 4 + 1 + 3 + 4 + 4 + 16
                elif ver == 2:
                    off = struct.unpack_from("<I", d, q)[0]
                    q += 4
                else:
                    nb = max(1, (size.bit_length() + 7) // 8)
                    off = int.from_bytes(d[q:q + nb], "little")
                    q += nb
                mt, used = self._datatype(d, q)
                q += used
                names.append(name)
                formats.append(mt)
                offsets.append(off)
            dt = np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": size})
            return dt, q - p
        if cls == 8:  # enumeration (booleans are the {FALSE, TRUE} enum of an 8-bit integer)
            nmem = bits & 0xFFFF
            base, used = self._datatype(d, q)
            q += used
            names = []
            for _ in range(nmem):
                e = d.index(b"\0", q)
                names.append(d[q:e].decode())
                q = q + ((e - q) // 8 + 1) * 8 if ver < 3 else e + 1
            values = np.frombuffer(d, base, nmem, q)
            q += nmem * base.itemsize
            members = {nm: int(v) for nm, v in zip(names, values)}
            return np.dtype(base, metadata={"enum": members}), q - p
        raise NotImplementedError(f"datatype class {cls}")

    def _attribute(self, d: bytes):
        version = d[0]
        if version != 1:
            raise NotImplementedError(f"attribute message version {version}")
        name_sz, type_sz, space_sz = struct.unpack_from("<HHH", d, 2)
        pad = lambda x: (x + 7) // 8 * 8
        p = 8
        name = d[p:p + name_sz].split(b"\0")[0].decode()
        p += pad(name_sz)
        dt, _ = self._datatype(d, p)
        p += pad(type_sz)
        shape = self._dataspace(d[p:p + space_sz]) if space_sz else ()
        p += pad(space_sz)
        count = int(np.prod(shape)) if shape else 1
        arr = np.frombuffer(d, dt, count, p)
        if dt.metadata and dt.metadata.get("vlen_str"):
            arr = np.array([self._vlen_str(r) for r in arr], dtype=object)
        val = arr.reshape(shape).copy() if shape else arr[0]
        if isinstance(val, bytes):
            val = val.split(b"\0")[0].decode(errors="replace")
        return name, val

    def _vlen_str(self, rec) -> str:
        """String of a variable-length element: an object of a global heap."""
        b = self._b
        g = self._base + int(rec["heap"])
        if b[g:g + 4] != b"GCOL":
            raise ValueError("bad global heap collection")
        end = g + struct.unpack_from("<Q", b, g + 8)[0]
        q = g + 16
        while q + 16 <= end:
            idx, _refs, _res, size = struct.unpack_from("<HHIQ", b, q)
            if idx == int(rec["index"]):
                return b[q + 16:q + 16 + int(rec["len"])].decode(errors="replace")
            if idx == 0:
                break
            q += 16 + (size + 7) // 8 * 8
        raise KeyError("global heap object not found")

    def _layout_bytes(self, d: bytes, nbytes: int):
        version = d[0]
        if version in (1, 2):
            cls = d[2]
            if cls == 1:
                addr = struct.unpack_from("<Q", d, 8)[0]
            elif cls == 0:
                rank = d[1]
                size = struct.unpack_from("<I", d, 8 + 4 * rank)[0]
                return d[12 + 4 * rank:12 + 4 * rank + size][:nbytes]
            else:
                raise NotImplementedError("chunked storage")
        elif version == 3:
            cls = d[1]
            if cls == 1:
                addr = struct.unpack_from("<Q", d, 2)[0]
            elif cls == 0:
                size = struct.unpack_from("<H", d, 2)[0]
                return d[4:4 + size][:nbytes]
            else:
                raise NotImplementedError("chunked storage")
        else:
            raise NotImplementedError(f"layout version {version}")
        if addr == _UNDEF:
            return None
        a = self._base + addr
        return self._b[a:a + nbytes]


def walk(node, prefix=""):
    """Yields (path, object) for every group and dataset under `node`."""
    if isinstance(node, Group):
        for k in sorted(node.keys()):
            child = node[k]
            path = f"{prefix}/{k}"
            yield path, child
            yield from walk(child, path)


# ============================================================================ writer
_GROUP_LEAF_K = 4        # symbol table node: up to 2K = 8 links
_GROUP_INTERNAL_K = 16   # v1 B-tree node: up to 2K = 32 children


def _pad8(b: bytes) -> bytes:
    return b + b"\0" * ((-len(b)) % 8)


def _dt_float64() -> bytes:
    # class 1 (floating point), version 1; little endian, IEEE: sign bit 63,
    # exponent 52..62 (bias 1023), mantissa 0..51, implied msb (normalisation 2)
    return bytes([0x11, 0x20, 63, 0]) + struct.pack("<I", 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)


def _dt_int(size: int) -> bytes:
    # class 0 (fixed point), version 1, little endian, signed
    return bytes([0x10, 0x08, 0, 0]) + struct.pack("<I", size) + struct.pack("<HH", 0, 8 * size)


def _dt_string(size: int) -> bytes:
    # class 3 (string), version 1, null terminated, ASCII
    return bytes([0x13, 0x00, 0, 0]) + struct.pack("<I", size)


def _dt_complex() -> bytes:
    # class 6 (compound), version 1, two float64 members "real" and "imag"
    out = bytes([0x16, 2, 0, 0]) + struct.pack("<I", 16)
    for name, off in (("real", 0), ("imag", 8)):
        out += _pad8(name.encode() + b"\0") + struct.pack("<I", off) + bytes(4) + bytes(4) + bytes(4) + bytes(16)
        out += _dt_float64()
    return out


def _dt_struct(dt: np.dtype) -> bytes:
    # class 6 (compound), version 1, one member per field of a structured dtype
    out = bytes([0x16, len(dt.names) & 0xFF, len(dt.names) >> 8, 0]) + struct.pack("<I", dt.itemsize)
    for name in dt.names:
        sub, off = dt.fields[name][:2]
        out += _pad8(name.encode() + b"\0") + struct.pack("<I", off) + bytes(4) + bytes(4) + bytes(4) + bytes(16)
        out += _dtype_message(sub)
    return out


def _dtype_message(dt: np.dtype) -> bytes:
    if dt.names is not None:
        return _dt_struct(dt)
    if dt == np.float64:
        return _dt_float64()
    if dt == np.complex128:
        return _dt_complex()
    if dt == np.int32:
        return _dt_int(4)
    if dt == np.int64:
        return _dt_int(8)
    raise NotImplementedError(f"dataset type {dt}")


def _dataspace(shape) -> bytes:
    return bytes([1, len(shape), 0, 0]) + bytes(4) + b"".join(struct.pack("<Q", d) for d in shape)


class Writer:
    """Builds an HDF5 file in memory; ``close()`` writes it.

        w = Writer(path)
        w.dataset("/Solution/State/vecFemStep1", x)        # groups made on the way
        w.attr("/Solution/State", "FreqStep1", "10.000000")
        w.close()
    """

    def __init__(self, path: str):
        self.path = path
        self.root = {"children": {}, "attrs": []}

    def _group(self, path: str):
        node = self.root
        for part in [p for p in path.split("/") if p]:
            ch = node["children"]
            if part not in ch:
                ch[part] = {"children": {}, "attrs": []}
            node = ch[part]
            if "data" in node:
                raise ValueError(f"{path}: {part} is a dataset")
        return node

    def group(self, path: str):
        self._group(path)
        return self

    def dataset(self, path: str, data):
        parts = [p for p in path.split("/") if p]
        parent = self._group("/".join(parts[:-1]))
        arr = np.ascontiguousarray(data)
        plain = (np.float64, np.complex128, np.int32, np.int64)
        if arr.dtype.names is not None:  # compound of plain members (e.g. the node table)
            if any(arr.dtype.fields[n][0] not in plain for n in arr.dtype.names):
                raise NotImplementedError(f"compound member type in {arr.dtype}")
        elif arr.dtype not in plain:
            raise NotImplementedError(f"dataset type {arr.dtype}")
        parent["children"][parts[-1]] = {"data": arr, "attrs": []}
        return self

    def attr(self, path: str, name: str, value):
        parts = [p for p in path.split("/") if p]
        node = self.root
        for part in parts:
            node = node["children"][part]
        node["attrs"].append((name, value))
        return self

    # ------------------------------------------------------------ layout
    def close(self):
        self._buf = bytearray(96)  # superblock placeholder
        root_ohdr, root_btree, root_heap = self._write_group(self.root)
        eof = len(self._buf)
        sb = bytearray(_SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]))
        sb += struct.pack("<HHI", _GROUP_LEAF_K, _GROUP_INTERNAL_K, 0)
        sb += struct.pack("<QQQQ", 0, _UNDEF, eof, _UNDEF)
        sb += struct.pack("<QQII", 0, root_ohdr, 1, 0) + struct.pack("<QQ", root_btree, root_heap)
        assert len(sb) == 96
        self._buf[0:96] = sb
        with open(self.path, "wb") as fh:
            fh.write(bytes(self._buf))

    def _alloc(self, data: bytes) -> int:
        while len(self._buf) % 8:
            self._buf += b"\0"
        addr = len(self._buf)
        self._buf += data
        return addr

    def _object_header(self, messages) -> int:
        body = b""
        for mtype, data in messages:
            data = _pad8(data)
            body += struct.pack("<HHB3x", mtype, len(data), 0) + data
        head = struct.pack("<BBHII", 1, 0, len(messages), 1, len(body)) + bytes(4)
        return self._alloc(head + body)

    def _attr_message(self, name: str, value) -> bytes:
        if isinstance(value, str):
            raw = value.encode() + b"\0"
            dt, data = _dt_string(len(raw)), raw
        elif isinstance(value, (bool, int, np.integer)):
            dt, data = _dt_int(8), struct.pack("<q", int(value))
        elif isinstance(value, (float, np.floating)):
            dt, data = _dt_float64(), struct.pack("<d", float(value))
        else:
            raise NotImplementedError(f"attribute type {type(value)}")
        nm = name.encode() + b"\0"
        sp = bytes([1, 0, 0, 0]) + bytes(4)  # scalar dataspace
        return (struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(sp)) + _pad8(nm) + _pad8(dt) + _pad8(sp) + data)

    def _write_dataset(self, node) -> int:
        arr = node["data"]
        raw = arr.astype(arr.dtype.newbyteorder("<"), copy=False).tobytes()
        data_addr = self._alloc(raw) if raw else _UNDEF
        layout = bytes([3, 1]) + struct.pack("<QQ", data_addr, len(raw))
        fill = bytes([2, 2, 2, 0])  # version 2: late allocation, never write fill, fill undefined
        msgs = [(0x1, _dataspace(arr.shape)), (0x3, _dtype_message(arr.dtype)), (0x5, fill), (0x8, layout)]
        msgs += [(0xC, self._attr_message(n, v)) for n, v in node["attrs"]]
        return self._object_header(msgs)

    def _write_group(self, node):
        # children first (their object header addresses go into the symbol table)
        entries = []
        for name in sorted(node["children"], key=lambda s: s.encode()):
            ch = node["children"][name]
            if "data" in ch:
                entries.append((name, self._write_dataset(ch), None))
            else:
                ohdr, bt, hp = self._write_group(ch)
                entries.append((name, ohdr, (bt, hp)))
        # local heap: "" at offset 0, then the names (8-byte padded)
        heap_data = bytearray(8)
        name_off = {}
        for name, _, _ in entries:
            name_off[name] = len(heap_data)
            heap_data += _pad8(name.encode() + b"\0")
        heap_data += bytes(8)  # a little free space, as libraries leave
        seg = self._alloc(bytes(heap_data))
        heap = self._alloc(b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap_data), _UNDEF, seg))
        # symbol table nodes of up to 2 * leaf K entries
        cap = 2 * _GROUP_LEAF_K
        snods = []
        for i in range(0, max(1, len(entries)), cap):
            chunk = entries[i:i + cap]
            body = b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(chunk))
            for name, addr, grp in chunk:
                if grp is None:
                    body += struct.pack("<QQII", name_off[name], addr, 0, 0) + bytes(16)
                else:
                    body += struct.pack("<QQII", name_off[name], addr, 1, 0) + struct.pack("<QQ", *grp)
            body += bytes(40 * (cap - len(chunk)))
            last = name_off[chunk[-1][0]] if chunk else 0
            snods.append((self._alloc(body), last))
        btree = self._btree(snods, 0)
        msgs = [(0x11, struct.pack("<QQ", btree, heap))]
        msgs += [(0xC, self._attr_message(n, v)) for n, v in node["attrs"]]
        return self._object_header(msgs), btree, heap

    def _btree(self, children, level) -> int:
        """v1 group B-tree over (child address, key = heap offset of its largest
        name) pairs; adds levels while a node would exceed 2K children."""
        k2 = 2 * _GROUP_INTERNAL_K
        if len(children) > k2:
            parents = []
            for i in range(0, len(children), k2):
                grp = children[i:i + k2]
                parents.append((self._btree_node(grp, level), grp[-1][1]))
            return self._btree(parents, level + 1)
        return self._btree_node(children, level)

    def _btree_node(self, children, level) -> int:
        k2 = 2 * _GROUP_INTERNAL_K
        body = b"TREE" + bytes([0, level]) + struct.pack("<H", len(children)) + struct.pack("<QQ", _UNDEF, _UNDEF)
        body += struct.pack("<Q", 0)  # key 0: the empty name
        for addr, key in children:
            body += struct.pack("<QQ", addr, key)
        body += bytes(16 * (k2 - len(children)))  # the node is allocated at full size
        return self._alloc(body)
