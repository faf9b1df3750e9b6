"""Minimal pure-Python HDF5 reader for snapshot files.

Reads files whose root group is an old-style symbol-table group (superblock
version 0 or 1 at offset 0 or after a user block of 512, 1024, ... bytes,
version-1 object headers with continuation blocks, v1 group B-tree, local
heap, symbol-table nodes) holding contiguous or compact, uncompressed numeric
datasets (data layout message versions 1, 2 and 3): the layout of the
reference's output files (cppsrc/HDF5Functions.cpp:249-397, one float64
dataset plus "time" per file), of this package's writer and of the HDF5
library's default format.  For environments without h5py.
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
        sb = 0  # the superblock sits at 0, 512, 1024, 2048, ...
        while sb + 8 <= len(buf) and buf[sb:sb + 8] != SIG:
            sb = 2 * sb if sb else 512
        if sb + 8 > len(buf):
            raise H5FormatError("not an HDF5 file (signature)")
        ver = buf[sb + 8]
        if ver not in (0, 1):
            raise H5FormatError("superblock version %d not supported" % ver)
        self.so, self.sl = buf[sb + 13], buf[sb + 14]
        if (self.so, self.sl) != (8, 8):
            raise H5FormatError("only 8-byte offsets/lengths supported")
        off = sb + 24 + (4 if ver == 1 else 0)
        base, _fs, eof, _drv = struct.unpack_from("<4Q", buf, off)
        self.eof = eof
        ent = off + 32
        _name, self.root_oh = struct.unpack_from("<2Q", buf, ent)
        # every address in the file is relative to the base address
        self.b = buf[base:]

    def u(self, fmt, off):
        return struct.unpack_from("<" + fmt, self.b, off)

    def messages(self, addr):
        b = self.b
        if b[addr] != 1:
            raise H5FormatError("object header version %d not supported" % b[addr])
        nmsg, _ref, size = struct.unpack_from("<HII", b, addr + 2)
        blocks, out = [(addr + 16, size)], []
        while blocks and len(out) < nmsg:
            p, n = blocks.pop(0)
            end = p + n
            while p + 8 <= end and len(out) < nmsg:
                mtype, msize, _flags = struct.unpack_from("<HHB", b, p)
                if mtype == 0x10:  # continuation: another block of messages
                    blocks.append(struct.unpack_from("<2Q", b, p + 8))
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
                ver = self.b[p]
                if ver == 3:
                    cls = self.b[p + 1]
                    if cls == 1:  # contiguous: address, size
                        layout = self.u("2Q", p + 2)
                    elif cls == 0:  # compact: size, data in the message
                        layout = (("compact", p + 4), self.u("H", p + 2)[0])
                    else:
                        raise H5FormatError("chunked or virtual layout not supported")
                elif ver in (1, 2):
                    nd, cls = self.b[p + 1], self.b[p + 2]
                    if cls == 1:  # contiguous: address, then nd dimension sizes
                        layout = (self.u("Q", p + 8)[0], None)
                    elif cls == 0:  # compact: nd dimension sizes, size, data
                        q = p + 8 + 4 * nd
                        layout = (("compact", q + 4), self.u("I", q)[0])
                    else:
                        raise H5FormatError("chunked layout not supported")
                else:
                    raise H5FormatError("layout message version %d not supported" % ver)
            elif mtype == 0x000B:
                raise H5FormatError("filtered (compressed) datasets not supported")
        if dims is None or dtype is None or layout is None:
            raise H5FormatError("incomplete dataset header")
        addr, size = layout
        n = int(np.prod(dims)) if dims else 1
        if size is not None and size != n * dtype.itemsize:
            raise H5FormatError("dataset size mismatch")
        if isinstance(addr, tuple):
            addr = addr[1]
        elif addr == UNDEF:
            return np.zeros(dims, dtype=dtype)  # unallocated: the default fill value
        return np.frombuffer(self.b, dtype=dtype, count=n, offset=addr).reshape(dims).copy()


def read(path: str) -> dict:
    """All datasets of the root group: {name: numpy array}."""
    with open(path, "rb") as f:
        buf = f.read()
    f5 = _File(buf)
    return {name: f5.dataset(oh) for name, oh in f5.group_entries(f5.root_oh)}
