"""Minimal HDF5 reader for the reference's data files, written from the public
HDF5 file-format specification (no libhdf5 is available).

Supported: superblock versions 0 and 1, groups stored as symbol tables
(version-1 B-trees of SNOD nodes with a local heap), version-1 object
headers with continuation blocks, simple dataspaces, IEEE float / integer /
compound datatypes, contiguous and compact layouts.  That covers the
reference's force-constant file (dataset `force_constants` of shape
(N,N,3,3), read at force_read.F90:89-164) and its output files
(write_output.F90:91-484: one group per q named '%012d' holding `q_vec`,
`eigenvalues`, optional compound `evec` {r, i} and `vel`).
"""
from __future__ import annotations

import struct

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"


class HDF5Error(ValueError):
    pass


class _File:
    def __init__(self, data: bytes):
        self.d = data
        base = data.find(SIG)
        if base != 0:
            raise HDF5Error("not an HDF5 file (superblock signature missing at offset 0)")
        ver = data[8]
        if ver not in (0, 1):
            raise HDF5Error(f"superblock version {ver} not supported")
        self.so, self.sl = data[13], data[14]
        if self.so != 8 or self.sl != 8:
            raise HDF5Error("only 8-byte offsets/lengths supported")
        p = 16 + 4 + 4
        if ver == 1:
            p += 4
        self.base, _, self.eof, _ = struct.unpack_from("<4Q", data, p)
        p += 32
        # root symbol table entry
        self.root_header = struct.unpack_from("<Q", data, p + 8)[0]

    def u(self, fmt, off):
        return struct.unpack_from("<" + fmt, self.d, off)

    # -- object headers -----------------------------------------------------
    def messages(self, addr):
        d = self.d
        ver = d[addr]
        if ver != 1:
            raise HDF5Error(f"object header version {ver} not supported")
        nmsg = self.u("H", addr + 2)[0]
        size = self.u("I", addr + 8)[0]
        blocks = [(addr + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            p = start
            while p + 8 <= start + length and len(out) < nmsg:
                mtype, msize, mflags = self.u("HHB", p)
                body = p + 8
                if mtype == 0x10:
                    caddr, clen = self.u("QQ", body)
                    blocks.append((caddr, clen))
                out.append((mtype, body, msize))
                p = body + msize
        return out

    def group_links(self, header_addr):
        for mtype, body, _ in self.messages(header_addr):
            if mtype == 0x11:
                btree, heap = self.u("QQ", body)
                return self._walk_btree(btree, self._heap_data(heap))
        raise HDF5Error("object is not a symbol-table group")

    def _heap_data(self, addr):
        if self.d[addr:addr + 4] != b"HEAP":
            raise HDF5Error("bad local heap")
        size, _, data_addr = self.u("QQQ", addr + 8)
        return data_addr

    def _name(self, heap_data, off):
        s = heap_data + off
        e = self.d.index(b"\x00", s)
        return self.d[s:e].decode()

    def _walk_btree(self, addr, heap_data):
        d = self.d
        if d[addr:addr + 4] != b"TREE":
            raise HDF5Error("bad B-tree node")
        ntype, level, used = d[addr + 4], d[addr + 5], self.u("H", addr + 6)[0]
        if ntype != 0:
            raise HDF5Error("not a group B-tree")
        p = addr + 24
        links = {}
        p += 8  # key 0
        for _ in range(used):
            child = self.u("Q", p)[0]
            p += 16  # child + next key
            if level > 0:
                links.update(self._walk_btree(child, heap_data))
            else:
                links.update(self._snod(child, heap_data))
        return links

    def _snod(self, addr, heap_data):
        d = self.d
        if d[addr:addr + 4] != b"SNOD":
            raise HDF5Error("bad symbol table node")
        nsym = self.u("H", addr + 6)[0]
        out = {}
        p = addr + 8
        for _ in range(nsym):
            name_off, hdr = self.u("QQ", p)
            out[self._name(heap_data, name_off)] = hdr
            p += 40
        return out

    # -- datasets -----------------------------------------------------------
    def dataset(self, header_addr):
        shape = dtype = None
        data_addr = data_size = None
        compact = None
        for mtype, body, msize in self.messages(header_addr):
            if mtype == 0x01:
                shape = self._dataspace(body)
            elif mtype == 0x03:
                dtype = self._datatype(body)
            elif mtype == 0x08:
                ver = self.d[body]
                if ver == 3:
                    cls = self.d[body + 1]
                    if cls == 1:
                        data_addr, data_size = self.u("QQ", body + 2)
                    elif cls == 0:
                        sz = self.u("H", body + 2)[0]
                        compact = self.d[body + 4:body + 4 + sz]
                    else:
                        raise HDF5Error("chunked layout not supported")
                elif ver in (1, 2):
                    ndim, cls = self.d[body + 1], self.d[body + 2]
                    if cls != 1:
                        raise HDF5Error("only contiguous layout supported for layout v1/v2")
                    data_addr = self.u("Q", body + 8)[0]
                else:
                    raise HDF5Error(f"layout version {ver} not supported")
        if shape is None or dtype is None:
            raise HDF5Error("dataset without dataspace/datatype")
        count = int(np.prod(shape)) if shape else 1
        if compact is not None:
            raw = compact
        else:
            nbytes = count * dtype.itemsize
            if data_addr == 0xFFFFFFFFFFFFFFFF:
                raw = b"\x00" * nbytes
            else:
                raw = self.d[data_addr:data_addr + nbytes]
                if len(raw) != nbytes:
                    raise HDF5Error("truncated dataset")
        return np.frombuffer(raw, dtype=dtype, count=count).reshape(shape).copy()

    def _dataspace(self, p):
        ver, ndim, flags = self.d[p], self.d[p + 1], self.d[p + 2]
        off = p + 8 if ver == 1 else p + 4
        return tuple(self.u(f"{ndim}Q", off)) if ndim else ()

    def _datatype(self, p):
        cv = self.d[p]
        cls = cv & 0x0F
        bits0 = self.d[p + 1]
        size = self.u("I", p + 4)[0]
        order = ">" if bits0 & 1 else "<"
        if cls == 1:
            return np.dtype(f"{order}f{size}")
        if cls == 0:
            signed = (bits0 >> 3) & 1
            return np.dtype(f"{order}{'i' if signed else 'u'}{size}")
        if cls == 6:
            nmemb = self.u("H", p + 1)[0]
            ver = cv >> 4
            q = p + 8
            names, fmts, offs = [], [], []
            for _ in range(nmemb):
                e = self.d.index(b"\x00", q)
                name = self.d[q:e].decode()
                nlen = e - q + 1
                if ver < 3:
                    q += (nlen + 7) // 8 * 8
                    moff = self.u("I", q)[0]
                    q += 4 + 1 + 3 + 4 + 4 + 16
                else:
                    q += nlen
                    nb = 1 if size < 256 else 2 if size < 65536 else 4
                    moff = int.from_bytes(self.d[q:q + nb], "little")
                    q += nb
                mt = self._datatype(q)
                q += 8 + self._dt_props_len(q)
                names.append(name)
                fmts.append(mt)
                offs.append(moff)
            return np.dtype({"names": names, "formats": fmts, "offsets": offs, "itemsize": size})
        raise HDF5Error(f"datatype class {cls} not supported")

    def _dt_props_len(self, p):
        cls = self.d[p] & 0x0F
        if cls == 1:
            return 12
        if cls == 0:
            return 4
        raise HDF5Error("nested compound members not supported")


class File:
    """Read-only view: `File(path)['group/dset']` -> numpy array."""

    def __init__(self, path: str):
        with open(path, "rb") as f:
            self._f = _File(f.read())

    def _resolve(self, path: str):
        addr = self._f.root_header
        for part in [p for p in path.split("/") if p]:
            links = self._f.group_links(addr)
            if part not in links:
                raise KeyError(path)
            addr = links[part]
        return addr

    def keys(self, group: str = "/"):
        return sorted(self._f.group_links(self._resolve(group)))

    def __getitem__(self, path: str) -> np.ndarray:
        return self._f.dataset(self._resolve(path))


def read_dataset(path: str, name: str) -> np.ndarray:
    return File(path)[name]


# ---------------------------------------------------------------------------
# Writer (superblock 0, symbol-table groups, version-1 object headers,
# contiguous datasets) for the reference's output layout.
UNDEF = 0xFFFFFFFFFFFFFFFF
LEAF_K = 64         # a symbol-table node holds up to 2K entries
INTERNAL_K = 64     # a group B-tree node holds up to 2K children (one level: <= 16384 members)


def _pad8(b: bytes) -> bytes:
    return b + b"\x00" * ((-len(b)) % 8)


def _msg(mtype: int, body: bytes, flags: int = 0) -> bytes:
    body = _pad8(body)
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _dt_f64() -> bytes:
    # class 1 (floating point), version 1; little endian, implied MSB, sign at bit 63
    return struct.pack("<B3BI", 0x11, 0x20, 0x3F, 0x00, 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)


def _dt_i64() -> bytes:
    # class 0 (fixed point), version 1, little endian, signed
    return struct.pack("<B3BI", 0x10, 0x08, 0x00, 0x00, 8) + struct.pack("<HH", 0, 64)


def _dt_compound(members) -> bytes:
    """members: [(name, offset)] of float64 fields, version-1 compound."""
    size = 8 * len(members)
    out = struct.pack("<BHBI", 0x16, len(members), 0, size)
    for name, off in members:
        out += _pad8(name.encode() + b"\x00")
        out += struct.pack("<IB3xI4x4I", off, 0, 0, 0, 0, 0, 0)
        out += _dt_f64()
    return out


class _Writer:
    """Appends objects to a file; the superblock is written last."""

    def __init__(self, f):
        self.f = f
        self.pos = 96
        f.write(b"\x00" * 96)

    def alloc(self, data) -> int:
        pad = (-self.pos) % 8
        if pad:
            self.f.write(b"\x00" * pad)
            self.pos += pad
        addr = self.pos
        self.f.write(data)
        self.pos += len(data)
        return addr

    def object_header(self, messages) -> int:
        body = b"".join(messages)
        hdr = struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body))
        return self.alloc(hdr + body)

    def dataset(self, arr: np.ndarray, dtype_msg: bytes) -> int:
        raw = memoryview(np.ascontiguousarray(arr)).cast("B")
        data_addr = self.alloc(raw) if len(raw) else UNDEF
        shape = arr.shape
        space = struct.pack("<BBBx4x", 1, len(shape), 0) + b"".join(struct.pack("<Q", d) for d in shape)
        layout = struct.pack("<BBQQ", 3, 1, data_addr, len(raw))
        return self.object_header([_msg(0x0001, space), _msg(0x0003, dtype_msg, flags=1), _msg(0x0008, layout)])

    def group(self, entries) -> int:
        """entries: sorted list of (name, header_addr, is_group, (btree, heap) or None)."""
        btree, heap = self.symbol_table(entries)
        return self.object_header([_msg(0x0011, struct.pack("<QQ", btree, heap))]), btree, heap

    def symbol_table(self, entries):
        entries = sorted(entries, key=lambda e: e[0].encode())
        heapdata = bytearray(b"\x00" * 8)     # offset 0: the empty name
        offs = []
        for e in entries:
            offs.append(len(heapdata))
            heapdata += _pad8(e[0].encode() + b"\x00")
        data_addr = self.alloc(bytes(heapdata))
        heap_addr = self.alloc(b"HEAP" + struct.pack("<B3xQQQ", 0, len(heapdata), UNDEF, data_addr))
        # symbol-table nodes of at most 2*LEAF_K entries each
        cap = 2 * LEAF_K
        chunks = [list(range(i, min(i + cap, len(entries)))) for i in range(0, max(len(entries), 1), cap)]
        if not entries:
            chunks = [[]]
        snods = []
        for ch in chunks:
            node = bytearray(b"SNOD" + struct.pack("<BBH", 1, 0, len(ch)))
            for k in ch:
                name, hdr, is_grp, scratch = entries[k]
                if is_grp:
                    node += struct.pack("<QQI4xQQ", offs[k], hdr, 1, scratch[0], scratch[1])
                else:
                    node += struct.pack("<QQI4x16x", offs[k], hdr, 0)
            node += b"\x00" * (40 * (cap - len(ch)))
            snods.append(self.alloc(bytes(node)))
        if len(snods) > 2 * INTERNAL_K:
            raise HDF5Error("too many group members for a one-level group B-tree")
        tree = bytearray(b"TREE" + struct.pack("<BBHQQ", 0, 0, len(snods), UNDEF, UNDEF))
        tree += struct.pack("<Q", 0)
        for i, (s, ch) in enumerate(zip(snods, chunks)):
            last = offs[ch[-1]] if ch else 0
            tree += struct.pack("<QQ", s, last)
        tree += b"\x00" * (16 * (2 * INTERNAL_K - len(snods)))
        btree_addr = self.alloc(bytes(tree))
        return btree_addr, heap_addr

    def close(self, root_entries) -> None:
        root_hdr, btree, heap = self.group(root_entries)
        sb = bytearray(SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", LEAF_K, INTERNAL_K, 0))
        sb += struct.pack("<QQQQ", 0, UNDEF, self.pos, UNDEF)
        sb += struct.pack("<QQI4xQQ", 0, root_hdr, 1, btree, heap)
        assert len(sb) == 96
        self.f.seek(0)
        self.f.write(bytes(sb))


class Writer:
    """Streaming writer: `add_group(name, datasets)` writes one group and its
    datasets immediately; `close()` writes the root group and superblock.
    Used for the per-q output groups, which can be large (eigenvectors)."""

    def __init__(self, path: str):
        self._f = open(path, "wb")
        self._w = _Writer(self._f)
        self._root = []

    def add_group(self, name: str, datasets: dict) -> None:
        ents = []
        for k, v in datasets.items():
            ents.append((k, _write_dataset(self._w, v), False, None))
        hdr, bt, hp = self._w.group(ents)
        self._root.append((name, hdr, True, (bt, hp)))

    def add_dataset(self, name: str, value) -> None:
        self._root.append((name, _write_dataset(self._w, value), False, None))

    def close(self) -> None:
        if self._f is None:
            return
        try:
            self._w.close(self._root)
        finally:
            self._f.close()
            self._f = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def _write_dataset(w: _Writer, v) -> int:
    a = np.asarray(v)
    if np.iscomplexobj(a):
        rec = np.empty(a.shape, dtype=[("r", "<f8"), ("i", "<f8")])
        rec["r"], rec["i"] = a.real, a.imag
        return w.dataset(rec, _dt_compound([("r", 0), ("i", 8)]))
    if a.dtype.kind in "iu":
        return w.dataset(a.astype("<i8"), _dt_i64())
    return w.dataset(a.astype("<f8"), _dt_f64())


def write_file(path: str, tree: dict) -> None:
    """Write nested dict {group: {name: ndarray | dict}} as HDF5.  float64
    arrays become IEEE F64LE datasets, int64 arrays I64LE, complex128 arrays
    the reference's compound {r: f64, i: f64} type."""
    f = open(path, "wb")
    w = _Writer(f)

    def build(d):
        ents = []
        for name, v in d.items():
            if isinstance(v, dict):
                hdr, bt, hp = build_group(v)
                ents.append((name, hdr, True, (bt, hp)))
            else:
                a = np.asarray(v)
                if np.iscomplexobj(a):
                    rec = np.empty(a.shape, dtype=[("r", "<f8"), ("i", "<f8")])
                    rec["r"], rec["i"] = a.real, a.imag
                    hdr = w.dataset(rec, _dt_compound([("r", 0), ("i", 8)]))
                elif a.dtype.kind in "iu":
                    hdr = w.dataset(a.astype("<i8"), _dt_i64())
                else:
                    hdr = w.dataset(a.astype("<f8"), _dt_f64())
                ents.append((name, hdr, False, None))
        return ents

    def build_group(d):
        return w.group(build(d))

    try:
        w.close(build(tree))
    finally:
        f.close()
