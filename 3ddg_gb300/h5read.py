"""Minimal pure-Python HDF5 reader for snapshot files.

Reads files whose root group is an old-style symbol-table group (superblock
version 0 or 1, version-1 object headers, v1 group B-tree, local heap,
symbol-table nodes) holding contiguous, uncompressed numeric datasets: the
layout of the reference's output files (cppsrc/HDF5Functions.cpp:249-397, one
float64 dataset plus "time" per file) and of this package's writer.  For
environments without h5py.
"""
from __future__ import annotations

import struct

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5FormatError(ValueError):
    pass


class _File:
    def __init__(self, buf: bytes):
        self.b = buf
        if buf[:8] != SIG:
            raise H5FormatError("not an HDF5 file (signature)")
        ver = buf[8]
        if ver not in (0, 1):
            raise H5FormatError("superblock version %d not supported" % ver)
        self.so, self.sl = buf[13], buf[14]
        if (self.so, self.sl) != (8, 8):
            raise H5FormatError("only 8-byte offsets/lengths supported")
        off = 24 + (4 if ver == 1 else 0)
        base, _fs, eof, _drv = struct.unpack_from("<4Q", buf, off)
        self.eof = eof
        ent = off + 32
        _name, self.root_oh = struct.unpack_from("<2Q", buf, ent)

    def u(self, fmt, off):
        return struct.unpack_from("<" + fmt, self.b, off)

    def messages(self, addr):
        b = self.b
        if b[addr] != 1:
            raise H5FormatError("object header version %d not supported" % b[addr])
        nmsg, _ref, size = struct.unpack_from("<HII", b, addr + 2)
        p, end, out = addr + 16, addr + 16 + size, []
        while p + 8 <= end and len(out) < nmsg:
            mtype, msize, _flags = struct.unpack_from("<HHB", b, p)
            out.append((mtype, p + 8, msize))
            p += 8 + msize
        return out

    def group_entries(self, oh_addr):
        st = [m for m in self.messages(oh_addr) if m[0] == 0x11]
        if not st:
            raise H5FormatError("root is not a symbol-table group")
        btree, heap = self.u("2Q", st[0][1])
        if self.b[heap:heap + 4] != b"HEAP":
            raise H5FormatError("bad local heap")
        _dsize, _free, hdata = self.u("3Q", heap + 8)
        entries = []
        self._walk(btree, hdata, entries)
        return entries

    def _walk(self, node, hdata, out):
        b = self.b
        if b[node:node + 4] != b"TREE":
            raise H5FormatError("bad B-tree node")
        ntype, level, used = b[node + 4], b[node + 5], struct.unpack_from("<H", b, node + 6)[0]
        if ntype != 0:
            raise H5FormatError("not a group B-tree")
        p = node + 24 + 8  # skip key 0
        for _ in range(used):
            child = struct.unpack_from("<Q", b, p)[0]
            p += 16
            if level > 0:
                self._walk(child, hdata, out)
                continue
            if b[child:child + 4] != b"SNOD":
                raise H5FormatError("bad symbol table node")
            nsym = struct.unpack_from("<H", b, child + 6)[0]
            for i in range(nsym):
                e = child + 8 + 40 * i
                noff, oh = struct.unpack_from("<2Q", b, e)
                s = hdata + noff
                name = b[s:b.index(b"\0", s)].decode()
                out.append((name, oh))

    def dataset(self, oh):
        dims, dtype, layout = None, None, None
        for mtype, p, _size in self.messages(oh):
            if mtype == 0x0001:
                ver, nd, flags = self.b[p], self.b[p + 1], self.b[p + 2]
                q = p + (8 if ver == 1 else 4)
                dims = list(struct.unpack_from("<%dQ" % nd, self.b, q))
            elif mtype == 0x0003:
                cls = self.b[p] & 0x0F
                size = self.u("I", p + 4)[0]
                le = (self.b[p + 1] & 1) == 0
                if cls == 1:
                    dtype = np.dtype(("<" if le else ">") + "f%d" % size)
                elif cls == 0:
                    signed = (self.b[p + 1] >> 3) & 1
                    dtype = np.dtype(("<" if le else ">") + ("i" if signed else "u") + "%d" % size)
                else:
                    raise H5FormatError("datatype class %d not supported" % cls)
            elif mtype == 0x0008:
                ver, cls = self.b[p], self.b[p + 1]
                if ver != 3 or cls != 1:
                    raise H5FormatError("only contiguous layout (message v3) supported")
                layout = self.u("2Q", p + 2)
        if dims is None or dtype is None or layout is None:
            raise H5FormatError("incomplete dataset header")
        addr, size = layout
        n = int(np.prod(dims)) if dims else 1
        if size != n * dtype.itemsize or addr == UNDEF:
            raise H5FormatError("dataset size mismatch")
        return np.frombuffer(self.b, dtype=dtype, count=n, offset=addr).reshape(dims).copy()


def read(path: str) -> dict:
    """All datasets of the root group: {name: numpy array}."""
    with open(path, "rb") as f:
        buf = f.read()
    f5 = _File(buf)
    return {name: f5.dataset(oh) for name, oh in f5.group_entries(f5.root_oh)}
