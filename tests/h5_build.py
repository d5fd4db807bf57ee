"""Test helper: builds HDF5 files with chunked datasets (shuffle, LZF, deflate
filters; several chunks, edge chunks, unfiltered chunks flagged in the filter
mask), following the public HDF5 file format specification, to exercise the
library's reader on the layouts libhdf5 / h5py write. Also a greedy LZF
encoder (the liblzf stream format: literal runs and back references)."""
from __future__ import annotations

import struct
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


def lzf_compress(data: bytes) -> bytes:
    out = bytearray()
    lit = bytearray()
    table = {}
    n = len(data)
    i = 0

    def flush():
        while lit:
            chunk = lit[:32]
            out.append(len(chunk) - 1)
            out.extend(chunk)
            del lit[:32]

    while i < n:
        if i + 2 < n:
            key = bytes(data[i:i + 3])
            ref = table.get(key)
            table[key] = i
            if ref is not None and i - ref - 1 < 8192:
                l, maxl = 3, min(264, n - i)
                while l < maxl and data[ref + l] == data[i + l]:
                    l += 1
                flush()
                dist, L = i - ref - 1, l - 2
                if L < 7:
                    out.append((L << 5) | (dist >> 8))
                else:
                    out.append((7 << 5) | (dist >> 8))
                    out.append(L - 7)
                out.append(dist & 0xFF)
                i += l
                continue
        lit.append(data[i])
        i += 1
    flush()
    return bytes(out)


def shuffle(raw: bytes, es: int) -> bytes:
    a = np.frombuffer(raw, np.uint8).reshape(-1, es)
    return a.T.tobytes()


class _W:
    def __init__(self):
        self.b = bytearray()

    def put(self, v, n):
        self.b += int(v).to_bytes(n, "little")

    def pos(self):
        return len(self.b)

    def patch(self, at, v, n=8):
        self.b[at:at + n] = int(v).to_bytes(n, "little")

    def align8(self):
        while len(self.b) % 8:
            self.b.append(0)


def _msg(w, typ, body: bytes, flags=0):
    n = (len(body) + 7) & ~7
    w.put(typ, 2)
    w.put(n, 2)
    w.put(flags, 1)
    w.b += bytes(3)
    w.b += body
    w.b += bytes(n - len(body))


def build_chunked(name: str, data: np.ndarray, chunk, filters=("shuffle", "lzf"), dtype="<f8") -> bytes:
    """A version-0 file with one chunked dataset. filters: sequence of
    'shuffle', 'lzf', 'deflate' (applied in order when writing)."""
    a = np.ascontiguousarray(data, dtype=dtype)
    if a.ndim == 1:
        a = a.reshape(-1)
    rank = a.ndim
    es = a.dtype.itemsize
    dims = a.shape
    chunk = tuple(chunk)
    w = _W()
    w.b += b"\x89HDF\r\n\x1a\n"
    w.b += bytes([0, 0, 0, 0, 0, 8, 8, 0])
    w.put(4, 2)
    w.put(16, 2)
    w.put(0, 4)
    w.put(0, 8)
    w.put(UNDEF, 8)
    eof = w.pos()
    w.put(0, 8)
    w.put(UNDEF, 8)
    w.put(0, 8)
    root_oh_at = w.pos()
    w.put(0, 8)
    w.put(1, 4)
    w.put(0, 4)
    scratch = w.pos()
    w.put(0, 8)
    w.put(0, 8)
    # root object header with a symbol table message
    root_oh = w.pos()
    w.put(1, 1); w.put(0, 1); w.put(1, 2); w.put(1, 4); w.put(24, 4); w.put(0, 4)
    stab_at = w.pos() + 8
    _msg(w, 0x11, bytes(16))
    w.patch(root_oh_at, root_oh)
    # group B-tree
    btree = w.pos()
    w.b += b"TREE"
    w.put(0, 1); w.put(0, 1); w.put(1, 2); w.put(UNDEF, 8); w.put(UNDEF, 8)
    w.put(0, 8)
    child_at = w.pos()
    w.put(0, 8)
    key1_at = w.pos()
    w.put(0, 8)
    w.b += bytes(31 * 16)
    # local heap
    heap_data = bytearray(8) + name.encode() + b"\0"
    while len(heap_data) % 8:
        heap_data.append(0)
    heap = w.pos()
    w.b += b"HEAP"
    w.put(0, 4)
    w.put(len(heap_data), 8)
    w.put(UNDEF, 8)
    w.put(w.pos() + 8, 8)
    w.b += heap_data
    w.patch(key1_at, 8)
    # symbol table node
    snod = w.pos()
    w.b += b"SNOD"
    w.put(1, 1); w.put(0, 1); w.put(1, 2)
    w.put(8, 8)
    ds_oh_at = w.pos()
    w.put(0, 8)
    w.b += bytes(24)
    w.b += bytes(7 * 40)
    w.patch(child_at, snod)
    # chunks
    grid = [range(0, d, c) for d, c in zip(dims, chunk)]
    offsets = [(o,) for o in grid[0]] if rank == 1 else [(o0, o1) for o0 in grid[0] for o1 in grid[1]]
    chunk_recs = []
    for off in offsets:
        blk = np.zeros(chunk, dtype=a.dtype)
        sl = tuple(slice(o, min(o + c, d)) for o, c, d in zip(off, chunk, dims))
        part = a[sl]
        blk[tuple(slice(0, s) for s in part.shape)] = part
        raw = blk.tobytes()
        mask = 0
        for fi, f in enumerate(filters):
            if f == "shuffle":
                raw = shuffle(raw, es)
            elif f == "deflate":
                raw = zlib.compress(raw, 6)
            elif f == "lzf":
                c = lzf_compress(raw)
                if len(c) >= len(raw):
                    mask |= 1 << fi   # optional filter skipped, as h5py's LZF filter does
                else:
                    raw = c
        w.align8()
        chunk_recs.append((off, len(raw), mask, w.pos()))
        w.b += raw
    # chunk B-tree (one leaf)
    w.align8()
    cbt = w.pos()
    w.b += b"TREE"
    w.put(1, 1); w.put(0, 1); w.put(len(chunk_recs), 2); w.put(UNDEF, 8); w.put(UNDEF, 8)
    for off, size, mask, at in chunk_recs:
        w.put(size, 4); w.put(mask, 4)
        for o in off:
            w.put(o, 8)
        w.put(0, 8)
        w.put(at, 8)
    w.put(0, 4); w.put(0, 4)
    for d in dims:
        w.put(d, 8)
    w.put(0, 8)
    # dataset object header
    w.align8()
    ds_oh = w.pos()
    space = bytes([1, rank, 0, 0]) + bytes(4) + b"".join(struct.pack("<Q", d) for d in dims)
    if es == 8:
        typ = bytes([0x11, 0x20, 63, 0]) + struct.pack("<I", 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
    else:
        typ = bytes([0x11, 0x20, 31, 0]) + struct.pack("<I", 4) + struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
    pipe = bytearray([1, len(filters)]) + bytes(6)
    for f in filters:
        fid, cd = {"shuffle": (2, [es]), "deflate": (1, [6]), "lzf": (32000, [4, 261, len(bytes(np.zeros(chunk, a.dtype)))])}[f]
        pipe += struct.pack("<HHHH", fid, 0, 1 if f == "lzf" else 0, len(cd))
        pipe += b"".join(struct.pack("<I", v) for v in cd)
        if len(cd) % 2:
            pipe += bytes(4)
    layout = bytes([3, 2, rank + 1]) + struct.pack("<Q", cbt) + b"".join(struct.pack("<I", c) for c in chunk) + \
        struct.pack("<I", es)
    bodies = [(0x01, space, 0), (0x03, typ, 1), (0x0B, bytes(pipe), 0), (0x08, layout, 0)]
    size = sum(8 + ((len(b) + 7) & ~7) for _, b, _ in bodies)
    w.put(1, 1); w.put(0, 1); w.put(len(bodies), 2); w.put(1, 4); w.put(size, 4); w.put(0, 4)
    for t, b, fl in bodies:
        _msg(w, t, b, fl)
    w.patch(ds_oh_at, ds_oh)
    w.patch(stab_at, btree)
    w.patch(stab_at + 8, heap)
    w.patch(scratch, btree)
    w.patch(scratch + 8, heap)
    w.patch(eof, len(w.b))
    return bytes(w.b)
