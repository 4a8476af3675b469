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
  (the latter in global heap collections, ``GCOL``) and compounds of those
  (the elpasoC complex type is the compound ``{real, imag}``).

Anything else (chunked or filtered storage, v2 object headers, dense
attribute storage, variable-length types) raises ``NotImplementedError``.
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
