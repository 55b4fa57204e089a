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
