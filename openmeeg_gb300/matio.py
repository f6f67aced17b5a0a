"""MATLAB v7.3 matrix files (HDF5 with a 512-byte MATLAB header), read
without libhdf5: the subset the reference's MatlabIO writes
(OpenMEEGMaths/include/MatlabIO.H:269-389, through matio with zlib
compression) --

* a Matrix as the double dataset ``linop`` (MATLAB column-major, so HDF5
  dims are [ncol, nlin]),
* a SymMatrix as the struct ``symmatrix`` with fields ``size`` (uint32) and
  ``data`` (the packed upper triangle, OpenMEEGMaths/include/symmatrix.h),
* a SparseMatrix as the MATLAB sparse ``matrix`` (a group with ``data``,
  ``ir``, ``jc`` in compressed-column form and the row count in its
  ``MATLAB_sparse`` attribute),
* a Vector as a one-column ``linop``.

HDF5 structures handled (HDF5 File Format Specification, version 0
superblock): v1 object headers with continuation blocks; dataspace,
datatype (IEEE floats, integers), data layout v1-v3 (compact, contiguous,
chunked), filter pipeline v1/v2 (deflate), attribute and symbol-table
messages; v1 B-trees of group and raw-data-chunk nodes, symbol-table nodes
and local heaps.  Anything else raises ValueError.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"


class _File:
    def __init__(self, data: bytes):
        self.d = data
        base = -1
        for off in (0, 512, 1024, 2048, 4096):
            if data[off:off + 8] == _SIG:
                base = off
                break
        if base < 0:
            raise ValueError("not an HDF5 (MATLAB v7.3) file")
        p = base + 8
        sb_ver = data[p]
        if sb_ver not in (0, 1):
            raise ValueError(f"HDF5 superblock version {sb_ver} not supported")
        self.so, self.sl = data[p + 5], data[p + 6]
        if self.so != 8 or self.sl != 8:
            raise ValueError("HDF5 offsets/lengths other than 8 bytes not supported")
        p += 16 + (4 if sb_ver == 1 else 0)
        self.base = self.u(p)
        p += 32                                   # base, free-space, end-of-file, driver addresses
        self.root = self._entry(p)

    # --- primitives -------------------------------------------------------
    def u(self, p, n=8):
        return int.from_bytes(self.d[p:p + n], "little")

    def a(self, addr):                            # file address -> byte position
        return self.base + addr

    def _entry(self, p):
        """Symbol table entry: (name offset, object header address, cache type, scratch)."""
        return self.u(p), self.u(p + 8), self.u(p + 16, 4), self.d[p + 24:p + 40]

    # --- object headers -----------------------------------------------------
    def messages(self, addr):
        p = self.a(addr)
        if self.d[p] != 1:
            raise ValueError(f"HDF5 object header version {self.d[p]} not supported")
        nmsg = self.u(p + 2, 2)
        size = self.u(p + 8, 4)
        blocks = [(p + 16, size)]
        out = []
        while blocks and len(out) < nmsg:
            q, n = blocks.pop(0)
            end = q + n
            while q + 8 <= end and len(out) < nmsg:
                mtype, msize = self.u(q, 2), self.u(q + 2, 2)
                body = self.d[q + 8:q + 8 + msize]
                if mtype == 0x10:                 # continuation
                    blocks.append((self.a(self.u(q + 8)), self.u(q + 16)))
                out.append((mtype, body))
                q += 8 + msize
        return out

    # --- groups -------------------------------------------------------------
    def group(self, addr):
        """name -> object header address of the links of a symbol-table group."""
        for mtype, body in self.messages(addr):
            if mtype == 0x11:
                return self._symtab(self.u_b(body, 0), self.u_b(body, 8))
        raise ValueError("HDF5 group without a symbol table")

    @staticmethod
    def u_b(body, p, n=8):
        return int.from_bytes(body[p:p + n], "little")

    def _heap(self, addr):
        p = self.a(addr)
        if self.d[p:p + 4] != b"HEAP":
            raise ValueError("bad HDF5 local heap")
        return self.a(self.u(p + 24))

    def _name(self, heap, off):
        p = heap + off
        return self.d[p:self.d.index(b"\0", p)].decode()

    def _symtab(self, btree, heap_addr):
        heap = self._heap(heap_addr)
        out = {}

        def walk(addr):
            p = self.a(addr)
            if self.d[p:p + 4] != b"TREE" or self.d[p + 4] != 0:
                raise ValueError("bad HDF5 group B-tree")
            level, used = self.d[p + 5], self.u(p + 6, 2)
            q = p + 24 + 8                        # header, then key 0
            for _ in range(used):
                child = self.u(q)
                if level > 0:
                    walk(child)
                else:
                    s = self.a(child)
                    if self.d[s:s + 4] != b"SNOD":
                        raise ValueError("bad HDF5 symbol table node")
                    for k in range(self.u(s + 6, 2)):
                        e = self._entry(s + 8 + 40 * k)
                        out[self._name(heap, e[0])] = e[1]
                q += 16                           # child, next key
        walk(btree)
        return out

    # --- datasets -----------------------------------------------------------
    def dataset(self, addr):
        shape = dtype = layout = None
        filters = []
        attrs = {}
        for mtype, b in self.messages(addr):
            if mtype == 0x01:
                shape = self._dataspace(b)
            elif mtype == 0x03:
                dtype = self._datatype(b)
            elif mtype == 0x08:
                layout = b
            elif mtype == 0x0B:
                filters = self._filters(b)
            elif mtype == 0x0C:
                n, v = self._attribute(b)
                attrs[n] = v
        if shape is None or dtype is None or layout is None:
            raise ValueError("HDF5 dataset without dataspace, datatype or layout")
        return self._read(layout, shape, dtype, filters), attrs

    def attributes(self, addr):
        return dict(self._attribute(b) for t, b in self.messages(addr) if t == 0x0C)

    def _dataspace(self, b):
        ver, rank, flags = b[0], b[1], b[2]
        p = 8 if ver == 1 else 4
        return tuple(self.u_b(b, p + 8 * i) for i in range(rank))

    @staticmethod
    def _datatype(b):
        cls, size = b[0] & 0x0F, int.from_bytes(b[4:8], "little")
        if b[1] & 1:
            raise ValueError("big-endian HDF5 data not supported")
        if cls == 1 and size in (4, 8):
            return np.dtype(f"<f{size}")
        if cls == 0 and size in (1, 2, 4, 8):
            return np.dtype(f"<{'i' if b[1] & 0x08 else 'u'}{size}")
        if cls == 3:                              # fixed-length string
            return np.dtype(f"S{size}")
        raise ValueError(f"HDF5 datatype class {cls} not supported")

    def _filters(self, b):
        ver, n = b[0], b[1]
        p = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = self.u_b(b, p, 2)
            if ver == 1 or fid >= 256:
                nlen = self.u_b(b, p + 2, 2)
                ncd = self.u_b(b, p + 6, 2)
                p += 8 + ((nlen + 7) // 8 * 8 if ver == 1 else nlen)
            else:
                ncd = self.u_b(b, p + 4, 2)
                p += 6
            p += 4 * ncd + (4 if ver == 1 and ncd % 2 else 0)
            out.append(fid)
        for f in out:
            if f != 1:
                raise ValueError(f"HDF5 filter {f} not supported (deflate only)")
        return out

    def _attribute(self, b):
        ver = b[0]
        nlen, tlen, slen = self.u_b(b, 2, 2), self.u_b(b, 4, 2), self.u_b(b, 6, 2)
        pad = (lambda x: (x + 7) // 8 * 8) if ver == 1 else (lambda x: x)
        p = 8 + (1 if ver >= 3 else 0)
        name = b[p:p + nlen].split(b"\0")[0].decode()
        p += pad(nlen)
        try:
            dt = self._datatype(b[p:p + tlen])
        except ValueError:
            return name, None
        p += pad(tlen)
        shape = self._dataspace(b[p:p + slen])
        p += pad(slen)
        count = int(np.prod(shape)) if shape else 1
        val = np.frombuffer(b[p:p + count * dt.itemsize], dt).reshape(shape)
        return name, val

    def _read(self, lay, shape, dtype, filters):
        ver = lay[0]
        count = int(np.prod(shape)) if shape else 1
        if ver == 3:
            cls = lay[1]
            if cls == 0:
                n = self.u_b(lay, 2, 2)
                return np.frombuffer(lay[4:4 + n], dtype).reshape(shape)
            if cls == 1:
                p = self.a(self.u_b(lay, 2))
                return np.frombuffer(self.d[p:p + count * dtype.itemsize], dtype).reshape(shape)
            if cls == 2:
                rank = lay[2] - 1
                btree = self.u_b(lay, 3)
                cdims = tuple(self.u_b(lay, 11 + 4 * i, 4) for i in range(rank))
                return self._chunked(btree, shape, cdims, dtype, filters)
        elif ver in (1, 2):
            rank, cls = lay[1], lay[2]
            if cls == 1:
                p = self.a(self.u_b(lay, 8))
                return np.frombuffer(self.d[p:p + count * dtype.itemsize], dtype).reshape(shape)
            if cls == 2:
                btree = self.u_b(lay, 8)
                cdims = tuple(self.u_b(lay, 16 + 4 * i, 4) for i in range(rank - 1))
                return self._chunked(btree, shape, cdims, dtype, filters)
        raise ValueError(f"HDF5 data layout version {ver} not supported")

    def _chunked(self, btree, shape, cdims, dtype, filters):
        out = np.zeros(shape, dtype)
        rank = len(shape)
        if btree == (1 << 64) - 1:                # never written: fill value (zeros)
            return out

        def walk(addr):
            p = self.a(addr)
            if self.d[p:p + 4] != b"TREE" or self.d[p + 4] != 1:
                raise ValueError("bad HDF5 chunk B-tree")
            level, used = self.d[p + 5], self.u(p + 6, 2)
            ksize = 8 + 8 * (rank + 1)
            q = p + 24
            for _ in range(used):
                csize, fmask = self.u(q, 4), self.u(q + 4, 4)
                offs = [self.u(q + 8 + 8 * i) for i in range(rank)]
                child = self.u(q + ksize)
                if level > 0:
                    walk(child)
                else:
                    c = self.a(child)
                    raw = self.d[c:c + csize]
                    if filters and not (fmask & 1):
                        raw = zlib.decompress(raw)
                    blk = np.frombuffer(raw[:int(np.prod(cdims)) * dtype.itemsize], dtype).reshape(cdims)
                    sl = tuple(slice(o, min(o + cd, s)) for o, cd, s in zip(offs, cdims, shape))
                    out[sl] = blk[tuple(slice(0, x.stop - x.start) for x in sl)]
                q += ksize + 8
        walk(btree)
        return out


def read_mat(path: str):
    """Reads a MATLAB v7.3 file written by the reference's MatlabIO: returns
    ("full", A) for a Matrix or Vector (A n x m, or n), ("sym", A) for a
    SymMatrix (dense symmetric), ("sparse", A) for a SparseMatrix (dense)."""
    f = _File(open(path, "rb").read())
    links = f.group(f.root[1])
    if "linop" in links:
        A, _ = f.dataset(links["linop"])
        A = np.ascontiguousarray(np.asarray(A, np.float64).T)   # MATLAB column-major: HDF5 dims [ncol, nlin]
        return "full", (A[:, 0].copy() if A.ndim == 2 and A.shape[1] == 1 else A)
    if "symmatrix" in links:
        fields = f.group(links["symmatrix"])
        size, _ = f.dataset(fields["size"])
        data, _ = f.dataset(fields["data"])
        n = int(np.asarray(size).ravel()[0])
        p = np.asarray(data, np.float64).ravel()
        if p.size != n * (n + 1) // 2:
            raise ValueError("symmatrix: data does not hold a packed triangle")
        from .io import unpack_upper
        return "sym", unpack_upper(p, n)
    if "matrix" in links:
        g = links["matrix"]
        attrs = f.attributes(g)
        parts = f.group(g)
        jc = np.asarray(f.dataset(parts["jc"])[0], np.int64).ravel()
        nrow = int(np.asarray(attrs["MATLAB_sparse"]).ravel()[0])
        A = np.zeros((nrow, jc.size - 1))
        if "ir" in parts:
            ir = np.asarray(f.dataset(parts["ir"])[0], np.int64).ravel()
            data = np.asarray(f.dataset(parts["data"])[0], np.float64).ravel()
            for j in range(jc.size - 1):
                A[ir[jc[j]:jc[j + 1]], j] = data[jc[j]:jc[j + 1]]
        return "sparse", A
    raise ValueError(f"{path}: no linop, symmatrix or matrix variable ({sorted(links)})")
