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

``write_h5`` / ``save_wabbit`` write the same subset: a v0 superblock, a root
symbol-table group, and datasets chunked as module_hdf5_wrapper.f90:261-293
chunks them on one process (each dimension's chunk extent is the dataset's
extent, at most 128), with the attributes saveHDF5_tree puts on ``blocks``.
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


# ============================================================================
# writer
# ============================================================================
_GROUP_K = 16      # group internal node K (superblock v0 default)
_LEAF_K = 4        # group leaf node K: a symbol-table node holds 2K entries
_ISTORE_K = 32     # chunk B-tree K of v0 superblocks: 2K entries per node
_MAX_CHUNK = 128   # module_hdf5_wrapper.f90:30 (max_chunk)


def _pad8(n):
    return (n + 7) & ~7


def _dtype_msg(dt: np.dtype) -> bytes:
    """Datatype message (version 1): little-endian IEEE float or integer."""
    dt = np.dtype(dt)
    if dt.kind == "f":
        if dt.itemsize != 8:
            raise ValueError("only float64 is written")
        # class 1, bit field: little endian, implied mantissa MSB, sign at 63;
        # offset 0, precision 64, exponent at 52 (11 bits), mantissa at 0 (52
        # bits), bias 1023
        return struct.pack("<BBBBIHHBBBBI", 0x11, 0x20, 0x3F, 0x00, 8, 0, 64, 52, 11, 0, 52, 1023)
    if dt.kind in "iu":
        bits0 = 0x08 if dt.kind == "i" else 0x00
        return struct.pack("<BBBBIHH", 0x10, bits0, 0, 0, dt.itemsize, 0, 8 * dt.itemsize)
    raise ValueError(f"dtype {dt} is not written")


def _space_msg(shape) -> bytes:
    """Dataspace message (version 1) with maximum dimensions equal to the
    dimensions."""
    rank = len(shape)
    return struct.pack("<BBBB4x", 1, rank, 1, 0) + struct.pack(f"<{2 * rank}Q", *shape, *shape)


def _attr_msg(name: str, value) -> bytes:
    """Attribute message (version 1) of a 1-D array value."""
    arr = np.ascontiguousarray(np.atleast_1d(value))
    nb = name.encode() + b"\x00"
    dtm = _dtype_msg(arr.dtype)
    spm = _space_msg(arr.shape)
    head = struct.pack("<BBHHH", 1, 0, len(nb), len(dtm), len(spm))
    body = nb.ljust(_pad8(len(nb)), b"\x00") + dtm.ljust(_pad8(len(dtm)), b"\x00") + \
        spm.ljust(_pad8(len(spm)), b"\x00") + arr.astype(arr.dtype.newbyteorder("<")).tobytes()
    return head + body


def _object_header(messages) -> bytes:
    """Version-1 object header holding the (type, payload) messages in one
    chunk, each payload padded to 8 bytes."""
    chunk = b""
    for mtype, payload in messages:
        payload = payload.ljust(_pad8(len(payload)), b"\x00")
        chunk += struct.pack("<HHB3x", mtype, len(payload), 0) + payload
    return struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(chunk)) + chunk


class _Writer:
    """Appends objects to a byte image; addresses are offsets in the file."""

    def __init__(self):
        self.buf = bytearray(96)   # superblock, written last

    def alloc(self, n: int) -> int:
        addr = len(self.buf)
        self.buf += b"\x00" * _pad8(n)
        return addr

    def put(self, addr: int, data: bytes):
        self.buf[addr:addr + len(data)] = data

    def add(self, data: bytes) -> int:
        addr = self.alloc(len(data))
        self.put(addr, data)
        return addr


def _chunk_btree(w: _Writer, entries, rank: int) -> int:
    """v1 B-tree (node type 1) over the chunks: entries are (offsets,
    nbytes, address) in row-major chunk order, the final key one chunk past
    the last. Nodes hold up to 2K entries; more chunks get internal levels."""
    ksize = 8 + 8 * (rank + 1)
    node_size = 24 + 2 * _ISTORE_K * (8 + ksize) + ksize

    def key(offs, nbytes):
        return struct.pack("<II", nbytes, 0) + struct.pack(f"<{rank + 1}Q", *offs, 0)

    def write_node(level, children):
        # children: (first key offsets, first nbytes, address, last key offsets, last nbytes)
        addr = w.alloc(node_size)
        out = b"TREE" + struct.pack("<BBHQQ", 1, level, len(children), _UNDEF, _UNDEF)
        for c in children:
            out += key(c[0], c[1]) + struct.pack("<Q", c[2])
        out += key(children[-1][3], 0)
        w.put(addr, out)
        return addr

    level = 0
    nodes = [(e[0], e[1], e[2], e[3], e[1]) for e in entries]
    cap = 2 * _ISTORE_K
    while True:
        groups = [nodes[i:i + cap] for i in range(0, len(nodes), cap)]
        made = [(g[0][0], g[0][1], write_node(level, g), g[-1][3], g[-1][4]) for g in groups]
        if len(made) == 1:
            return made[0][2]
        nodes = made
        level += 1


def _chunked_dataset(w: _Writer, name: str, data: np.ndarray, attrs: dict) -> int:
    data = np.ascontiguousarray(data)
    data = data.astype(data.dtype.newbyteorder("<"))
    shape = data.shape
    rank = len(shape)
    chunk = tuple(min(n, _MAX_CHUNK) for n in shape)
    nbytes = int(np.prod(chunk)) * data.itemsize
    counts = [-(-n // c) for n, c in zip(shape, chunk)]
    entries = []
    for idx in np.ndindex(*counts):
        offs = tuple(i * c for i, c in zip(idx, chunk))
        block = np.zeros(chunk, data.dtype)
        sl = tuple(slice(o, min(o + c, n)) for o, c, n in zip(offs, chunk, shape))
        block[tuple(slice(0, s.stop - s.start) for s in sl)] = data[sl]
        addr = w.add(block.tobytes())
        past = tuple(o + c for o, c in zip(offs, chunk))
        entries.append((offs, nbytes, addr, past))
    btree = _chunk_btree(w, entries, rank)
    layout = struct.pack("<BBBQ", 3, 2, rank + 1, btree) + struct.pack(f"<{rank + 1}I", *chunk, data.itemsize)
    # fill value (version 2): allocated early, written if set, defined, none
    msgs = [(0x01, _space_msg(shape)), (0x03, _dtype_msg(data.dtype)), (0x05, struct.pack("<BBBBI", 2, 1, 2, 1, 0)),
            (0x08, layout)]
    msgs += [(0x0C, _attr_msg(k, v)) for k, v in attrs.items()]
    return w.add(_object_header(msgs))


def write_h5(path: str, datasets: dict, attrs: dict | None = None):
    """Write the named arrays as chunked datasets of the root group of a new
    HDF5 file; attrs maps a dataset name to its {attribute: 1-D array}."""
    attrs = attrs or {}
    names = sorted(datasets, key=lambda n: n.encode())
    if len(names) > 2 * _LEAF_K:
        raise ValueError(f"at most {2 * _LEAF_K} datasets per file")
    w = _Writer()
    # local heap of the names: the empty name at 0, then each name, padded
    # to 8 bytes, then one free block (next = 1: none, size 16)
    heap_data = b"\x00" * 8
    offsets = {}
    for n in names:
        offsets[n] = len(heap_data)
        nb = n.encode() + b"\x00"
        heap_data += nb.ljust(_pad8(len(nb)), b"\x00")
    free = len(heap_data)
    heap_data += struct.pack("<QQ", 1, 16)
    heap_data_addr = w.add(heap_data)
    heap_addr = w.add(b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap_data), free, heap_data_addr))
    ohdrs = {n: _chunked_dataset(w, n, datasets[n], attrs.get(n, {})) for n in names}
    # one symbol-table node with every dataset, sorted by name
    snod = w.alloc(8 + 2 * _LEAF_K * 40)
    out = b"SNOD" + struct.pack("<BBH", 1, 0, len(names))
    for n in names:
        out += struct.pack("<QQII16x", offsets[n], ohdrs[n], 0, 0)
    w.put(snod, out)
    # group B-tree (node type 0): keys are heap offsets, the last the largest name
    gnode = w.alloc(24 + 2 * _GROUP_K * 16 + 8)
    w.put(gnode, b"TREE" + struct.pack("<BBHQQ", 0, 0, 1, _UNDEF, _UNDEF) +
          struct.pack("<QQQ", 0, snod, offsets[names[-1]] if names else 0))
    root = w.add(_object_header([(0x11, struct.pack("<QQ", gnode, heap_addr))]))
    eof = len(w.buf)
    sb = _SIG + struct.pack("<BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, _LEAF_K, _GROUP_K, 0)
    sb += struct.pack("<QQQQ", 0, _UNDEF, eof, _UNDEF)
    sb += struct.pack("<QQII", 0, root, 1, 0) + struct.pack("<QQ", gnode, heap_addr)
    assert len(sb) == 96
    w.put(0, sb)
    with open(path, "wb") as f:
        f.write(bytes(w.buf))


def treecode(level: int, coords, dim: int, max_level: int) -> int:
    """The block's 64-bit treecode as lgt_block stores it (encoding_b,
    LIB/TREE/module_treelib.f90:837-871 with max_level = Jmax): bit i of the
    0-based block index along y, x, z goes to bit (i + Jmax - level) * dim +
    (0, 1, 2)."""
    ix = [int(coords[1]), int(coords[0])] + ([int(coords[2])] if dim == 3 else [])
    tc = 0
    for d in range(dim):
        v, i = ix[d], 0
        while v >> i:
            tc |= ((v >> i) & 1) << ((i + max_level - level) * dim + d)
            i += 1
    return tc


def timestr(time: float) -> str:
    """The 12-digit time stamp of the reference's file names (timestr,
    LIB/HELPER/module_helpers.f90:765-771): integer part, then micro units."""
    ip = int(time + 1.0e-12)
    frac = int(np.rint(max((time - np.floor(time + 1.0e-12)) * 1.0e6, 0.0)))
    return f"{ip:06d}{frac:06d}"


def save_wabbit(path: str, blocks, level, coords, time: float, iteration: int, domain, Bs, max_level: int,
                refinement_status=None, lgt_ids=None, procs=None):
    """One field file in saveHDF5_tree's layout (LIB/MESH/InputOutput.f90:
    1-309) without ghost nodes: blocks (Nb, [Bs+1,] Bs+1, Bs+1) holding the
    interior and the first ghost layer on the upper side, coords_origin /
    coords_spacing in reversed axis order (z, y, x), the treecodes, levels,
    refinement status, process ranks and light ids, and the attributes of
    ``blocks`` (domain-size, periodic_BC, symmetry_BC, version, block-size,
    time, iteration, total_number_blocks, max_level, dim)."""
    blocks = np.ascontiguousarray(blocks, np.float64)
    level = np.asarray(level, np.int64).ravel()
    nb = len(level)
    dim = blocks.ndim - 1
    coords = np.asarray(coords, np.int64).reshape(nb, -1)[:, :dim]
    domain = np.asarray(domain, np.float64).ravel()[:dim]
    Bs = np.asarray(Bs, np.int64).ravel()[:dim]
    if blocks.shape[0] != nb or tuple(blocks.shape[1:]) != tuple(int(b) + 1 for b in Bs[::-1]):
        raise ValueError("blocks must be (Nb, [Bs+1,] Bs+1, Bs+1)")
    # get_block_spacing_origin_b (module_treelib.f90:96-101)
    dx = np.stack([2.0 ** (-level.astype(np.float64)) * domain[d] / float(Bs[d]) for d in range(dim)], axis=1)
    x0 = np.stack([(coords[:, d] * Bs[d]).astype(np.float64) * dx[:, d] for d in range(dim)], axis=1)
    bsz = np.ones(3, np.int32)
    bsz[:dim] = Bs
    ds = {
        "blocks": blocks,
        "coords_origin": np.ascontiguousarray(x0[:, ::-1]),
        "coords_spacing": np.ascontiguousarray(dx[:, ::-1]),
        "block_treecode_num": np.array([treecode(l, c, dim, max_level) for l, c in zip(level, coords)], np.int64),
        "procs": np.zeros(nb, np.int32) if procs is None else np.asarray(procs, np.int32),
        "refinement_status": np.zeros(nb, np.int32) if refinement_status is None
        else np.asarray(refinement_status, np.int32),
        "level": level.astype(np.int32),
        "lgt_ids": np.arange(1, nb + 1, dtype=np.int32) if lgt_ids is None else np.asarray(lgt_ids, np.int32),
    }
    at = {"domain-size": domain, "periodic_BC": np.ones(3, np.int32), "symmetry_BC": np.zeros(3, np.int32),
          "version": np.array([20240410], np.int32), "block-size": bsz, "time": np.array([time], np.float64),
          "iteration": np.array([iteration], np.int32), "total_number_blocks": np.array([nb], np.int32),
          "max_level": np.array([max_level], np.int32), "dim": np.array([dim], np.int32)}
    write_h5(path, ds, {"blocks": at})
