"""Minimal reader for WABBIT's HDF5 field files.

WABBIT writes one HDF5 file per field (LIB/MESH/InputOutput.f90:1-309,
saveHDF5_tree): a dataset ``blocks`` of shape (Nb, [Bs+1,] Bs+1, Bs+1) with
the block interiors plus one redundant point per direction, the datasets
``coords_origin``, ``coords_spacing``, ``block_treecode_num``, ``level``,
``refinement_status``, ``procs``, ``lgt_ids`` and a set of attributes on
``blocks`` (time, iteration, domain-size, block-size, max_level, dim, ...).
The files are written by the HDF5 1.x library with the classic layout:
superblock v0, version-1 object headers, symbol-table groups with v1 B-trees
and local heaps, and contiguous or chunked (v1 B-tree indexed, unfiltered)
datasets (LIB/MODULE/module_hdf5_wrapper.f90:87,261-337).

This module implements exactly that subset in pure numpy so that the
reference's committed regression files can be read without libhdf5. It raises
``ValueError`` on anything outside the subset (filters, v2 B-trees, ...).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF


@dataclass
class _Dataset:
    name: str
    shape: tuple = ()
    dtype: np.dtype | None = None
    layout: int = -1
    address: int = _UNDEF
    size: int = 0
    chunk: tuple = ()
    compact: bytes = b""
    attrs: dict = field(default_factory=dict)


class H5File:
    """Read-only view of a classic-layout HDF5 file (see module docstring)."""

    def __init__(self, path: str):
        with open(path, "rb") as f:
            self.buf = f.read()
        b = self.buf
        if b[:8] != _SIG:
            raise ValueError(f"{path}: not an HDF5 file")
        if b[8] != 0:
            raise ValueError(f"{path}: superblock version {b[8]} not supported")
        if b[13] != 8 or b[14] != 8:
            raise ValueError("only 8-byte offsets/lengths supported")
        root_ohdr = struct.unpack_from("<Q", b, 64)[0]
        self.datasets: dict[str, _Dataset] = {}
        self._read_group(root_ohdr, prefix="")

    # ------------------------------------------------------------------ utils
    def _u(self, fmt, off):
        return struct.unpack_from(fmt, self.buf, off)

    def _messages(self, addr):
        """Yield (type, data_offset, size) for a version-1 object header."""
        b = self.buf
        if b[addr] != 1:
            raise ValueError(f"object header version {b[addr]} at {addr} not supported")
        nmsg = self._u("<H", addr + 2)[0]
        hsize = self._u("<I", addr + 8)[0]
        blocks = [(addr + 16, hsize)]
        seen = 0
        while blocks and seen < nmsg:
            start, length = blocks.pop(0)
            off = start
            while off + 8 <= start + length and seen < nmsg:
                mtype, msize, _flags = self._u("<HHB", off)
                data = off + 8
                seen += 1
                if mtype == 0x10:  # continuation
                    caddr, clen = self._u("<QQ", data)
                    blocks.append((caddr, clen))
                else:
                    yield mtype, data, msize
                off = data + msize
                off = (off + 7) & ~7 if ((off - start) % 8) else off

    def _heap_string(self, heap_addr, offset):
        b = self.buf
        if b[heap_addr:heap_addr + 4] != b"HEAP":
            raise ValueError("bad local heap")
        data_addr = self._u("<Q", heap_addr + 24)[0]
        s = data_addr + offset
        e = b.index(b"\x00", s)
        return b[s:e].decode()

    # ----------------------------------------------------------------- groups
    def _read_group(self, ohdr, prefix):
        for mtype, off, _ in self._messages(ohdr):
            if mtype == 0x11:  # symbol table
                btree, heap = self._u("<QQ", off)
                self._walk_group_btree(btree, heap, prefix)

    def _walk_group_btree(self, addr, heap, prefix):
        b = self.buf
        if b[addr:addr + 4] != b"TREE" or b[addr + 4] != 0:
            raise ValueError("bad group B-tree")
        level = b[addr + 5]
        nent = self._u("<H", addr + 6)[0]
        p = addr + 24 + 8  # skip key 0
        for _ in range(nent):
            child = self._u("<Q", p)[0]
            p += 16  # child + next key
            if level > 0:
                self._walk_group_btree(child, heap, prefix)
            else:
                self._read_snod(child, heap, prefix)

    def _read_snod(self, addr, heap, prefix):
        b = self.buf
        if b[addr:addr + 4] != b"SNOD":
            raise ValueError("bad symbol table node")
        nsym = self._u("<H", addr + 6)[0]
        p = addr + 8
        for _ in range(nsym):
            name_off, ohdr, cache = self._u("<QQI", p)
            name = self._heap_string(heap, name_off)
            full = prefix + name
            if cache == 1:  # cached group
                self._read_group(ohdr, full + "/")
            else:
                ds = self._read_object(ohdr, full)
                if ds is None:
                    self._read_group(ohdr, full + "/")
            p += 40

    # --------------------------------------------------------------- datasets
    def _datatype(self, off):
        b = self.buf
        cls = b[off] & 0x0F
        bits0 = b[off + 1]
        size = self._u("<I", off + 4)[0]
        if bits0 & 1:
            raise ValueError("big-endian data not supported")
        if cls == 0:
            signed = bool(bits0 & 0x08)
            return np.dtype(f"<{'i' if signed else 'u'}{size}")
        if cls == 1:
            return np.dtype(f"<f{size}")
        if cls == 3:
            return np.dtype(f"S{size}")
        raise ValueError(f"datatype class {cls} not supported")

    def _dataspace(self, off):
        b = self.buf
        ver = b[off]
        rank = b[off + 1]
        if ver == 1:
            dims = self._u(f"<{rank}Q", off + 8) if rank else ()
        elif ver == 2:
            dims = self._u(f"<{rank}Q", off + 4) if rank else ()
        else:
            raise ValueError(f"dataspace version {ver} not supported")
        return tuple(int(d) for d in dims)

    def _read_object(self, ohdr, name):
        ds = _Dataset(name)
        is_ds = False
        for mtype, off, msize in self._messages(ohdr):
            if mtype == 0x01:
                ds.shape = self._dataspace(off)
                is_ds = True
            elif mtype == 0x03:
                ds.dtype = self._datatype(off)
            elif mtype == 0x08:
                ver = self.buf[off]
                if ver != 3:
                    raise ValueError(f"layout version {ver} not supported")
                ds.layout = self.buf[off + 1]
                if ds.layout == 0:
                    n = self._u("<H", off + 2)[0]
                    ds.compact = self.buf[off + 4:off + 4 + n]
                elif ds.layout == 1:
                    ds.address, ds.size = self._u("<QQ", off + 2)
                elif ds.layout == 2:
                    nd = self.buf[off + 2]
                    ds.address = self._u("<Q", off + 3)[0]
                    ds.chunk = self._u(f"<{nd}I", off + 11)
            elif mtype == 0x0B:
                raise ValueError(f"{name}: filtered datasets not supported")
            elif mtype == 0x0C:
                self._attribute(off, ds.attrs)
        if not is_ds:
            return None
        self.datasets[name] = ds
        return ds

    def _attribute(self, off, attrs):
        b = self.buf
        ver = b[off]
        if ver != 1:
            raise ValueError(f"attribute version {ver} not supported")
        nlen, tlen, slen = self._u("<HHH", off + 2)
        p = off + 8
        name = b[p:p + nlen].split(b"\x00")[0].decode()
        p += (nlen + 7) & ~7
        dt = self._datatype(p)
        p += (tlen + 7) & ~7
        shape = self._dataspace(p)
        p += (slen + 7) & ~7
        n = int(np.prod(shape)) if shape else 1
        val = np.frombuffer(b, dtype=dt, count=n, offset=p).copy()
        attrs[name] = val.reshape(shape) if shape else val[0]

    # ------------------------------------------------------------------ read
    def read(self, name: str) -> np.ndarray:
        ds = self.datasets[name]
        n = int(np.prod(ds.shape)) if ds.shape else 1
        if ds.layout == 1:
            if ds.address == _UNDEF:
                return np.zeros(ds.shape, ds.dtype)
            return np.frombuffer(self.buf, ds.dtype, n, ds.address).reshape(ds.shape).copy()
        if ds.layout == 0:
            return np.frombuffer(ds.compact, ds.dtype, n).reshape(ds.shape).copy()
        if ds.layout == 2:
            out = np.zeros(ds.shape, ds.dtype)
            if ds.address != _UNDEF:
                self._read_chunks(ds.address, ds, out)
            return out
        raise ValueError(f"{name}: unknown layout {ds.layout}")

    def _read_chunks(self, addr, ds, out):
        b = self.buf
        if b[addr:addr + 4] != b"TREE" or b[addr + 4] != 1:
            raise ValueError("bad chunk B-tree")
        level = b[addr + 5]
        nent = self._u("<H", addr + 6)[0]
        rank = len(ds.shape)
        ksize = 8 + 8 * (rank + 1)
        p = addr + 24
        cshape = tuple(int(c) for c in ds.chunk[:rank])
        for _ in range(nent):
            csize, _mask = self._u("<II", p)
            offs = self._u(f"<{rank}Q", p + 8)
            child = self._u("<Q", p + ksize)[0]
            p += ksize + 8
            if level > 0:
                self._read_chunks(child, ds, out)
                continue
            n = int(np.prod(cshape))
            chunk = np.frombuffer(b, ds.dtype, n, child).reshape(cshape)
            sl_out = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cshape, ds.shape))
            sl_in = tuple(slice(0, s.stop - s.start) for s in sl_out)
            out[sl_out] = chunk[sl_in]

    def attrs(self, name: str) -> dict:
        return self.datasets[name].attrs


def read_wabbit(path: str) -> dict:
    """Read one WABBIT field file.

    Returns a dict with ``blocks`` (Nb, [nz,] ny, nx) float64 in the file's
    C order (x fastest), ``level`` (Nb,), ``coords`` (Nb, dim) integer block
    coordinates on that level, ``origin``/``spacing`` (Nb, dim) in x,y[,z]
    order and the attributes ``time``, ``iteration``, ``domain`` and ``Bs``.
    """
    h = H5File(path)
    blocks = h.read("blocks").astype(np.float64)
    a = h.attrs("blocks")
    dim = int(np.ravel(a["dim"])[0]) if "dim" in a else blocks.ndim - 1
    bs = np.ravel(a["block-size"]).astype(np.int64)[:dim]
    domain = np.ravel(a["domain-size"]).astype(np.float64)[:dim]
    # origin/spacing are stored in reversed axis order (z,y,x) / (y,x)
    origin = h.read("coords_origin").astype(np.float64)[:, ::-1]
    spacing = h.read("coords_spacing").astype(np.float64)[:, ::-1]
    level = np.rint(np.log2(domain[0] / (spacing[:, 0] * bs[0]))).astype(np.int64)
    coords = np.rint(origin / (spacing * bs)).astype(np.int64)
    out = {
        "blocks": blocks,
        "level": level,
        "coords": coords,
        "origin": origin,
        "spacing": spacing,
        "time": float(np.ravel(a["time"])[0]),
        "iteration": int(np.ravel(a["iteration"])[0]),
        "domain": domain,
        "Bs": bs,
        "dim": dim,
        "version": int(np.ravel(a["version"])[0]) if "version" in a else 0,
    }
    if "level" in h.datasets:
        lv = h.read("level").astype(np.int64).ravel()
        if not np.array_equal(lv, level):
            raise ValueError(f"{path}: level dataset disagrees with block spacing")
    if "max_level" in a:
        out["max_level"] = int(np.ravel(a["max_level"])[0])
    return out
