"""Test-side HDF5 writer (HDF5 File Format Specification 3.0): files in the
two styles the HDF5 library writes, for the reader in
``fastlisaresponse_gb300.h5lite`` when h5py is absent.

* ``style="v0"``: superblock version 0, version-1 object headers, groups as
  symbol tables (version-1 B-tree, symbol table node, local heap) -- h5py's
  default ("earliest") format.  Attributes after the first go into a
  continuation block, as the library does once an object header fills up.
* ``style="v2"``: superblock version 2, version-2 object headers ("OHDR") with
  lookup3 checksums, groups as link messages -- h5py with
  ``libver="latest"``, continuation blocks ("OCHK") likewise.

Datasets are contiguous, chunked with a version-1 B-tree chunk index (two
levels beyond four chunks) and the shuffle + deflate filters, or compact
(the data inside the layout message).  Attributes: numeric scalars and
arrays, fixed-length strings, variable-length UTF-8 strings (global heap).
Only what the tests need; no free-space management.
"""

from __future__ import annotations

import zlib

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = b"\xff" * 8


def lookup3(data: bytes, initval: int = 0) -> int:
    """Bob Jenkins' lookup3 ``hashlittle`` (the HDF5 metadata checksum)."""
    m = 0xFFFFFFFF

    def rot(x, k):
        return ((x << k) | (x >> (32 - k))) & m

    n = len(data)
    a = b = c = (0xDEADBEEF + n + initval) & m
    i = 0
    while n > 12:
        a = (a + int.from_bytes(data[i:i + 4], "little")) & m
        b = (b + int.from_bytes(data[i + 4:i + 8], "little")) & m
        c = (c + int.from_bytes(data[i + 8:i + 12], "little")) & m
        a = (a - c) & m; a ^= rot(c, 4); c = (c + b) & m
        b = (b - a) & m; b ^= rot(a, 6); a = (a + c) & m
        c = (c - b) & m; c ^= rot(b, 8); b = (b + a) & m
        a = (a - c) & m; a ^= rot(c, 16); c = (c + b) & m
        b = (b - a) & m; b ^= rot(a, 19); a = (a + c) & m
        c = (c - b) & m; c ^= rot(b, 4); b = (b + a) & m
        n -= 12
        i += 12
    if n == 0:
        return c
    tail = data[i:] + bytes(12 - n)
    a = (a + int.from_bytes(tail[0:4], "little")) & m
    b = (b + int.from_bytes(tail[4:8], "little")) & m
    c = (c + int.from_bytes(tail[8:12], "little")) & m
    c ^= b; c = (c - rot(b, 14)) & m
    a ^= c; a = (a - rot(c, 11)) & m
    b ^= a; b = (b - rot(a, 25)) & m
    c ^= b; c = (c - rot(b, 16)) & m
    a ^= c; a = (a - rot(c, 4)) & m
    b ^= a; b = (b - rot(a, 14)) & m
    c ^= b; c = (c - rot(b, 24)) & m
    return c


def _u(v: int, n: int) -> bytes:
    return int(v).to_bytes(n, "little")


def _pad8(b: bytes) -> bytes:
    return b + bytes(-len(b) % 8)


def _dtype_msg(dt: np.dtype) -> bytes:
    dt = np.dtype(dt)
    order = 1 if dt.byteorder == ">" else 0
    if dt.kind == "f":
        exp = {2: (10, 5, 10, 15), 4: (23, 8, 23, 127), 8: (52, 11, 52, 1023)}[dt.itemsize]
        bits = order | 0x20  # implied leading mantissa bit
        return (bytes([0x11, bits, dt.itemsize * 8 - 1, 0]) + _u(dt.itemsize, 4) +
                _u(0, 2) + _u(dt.itemsize * 8, 2) + bytes([exp[0], exp[1], 0, exp[2]]) +
                _u(exp[3], 4))
    if dt.kind in "iu":
        bits = order | (0x08 if dt.kind == "i" else 0)
        return bytes([0x10, bits, 0, 0]) + _u(dt.itemsize, 4) + _u(0, 2) + _u(dt.itemsize * 8, 2)
    if dt.kind == "S":  # fixed-length, null-padded ASCII
        return bytes([0x13, 0x01, 0, 0]) + _u(dt.itemsize, 4)
    raise TypeError(dt)


def _vlen_str_msg() -> bytes:
    base = bytes([0x10, 0, 0, 0]) + _u(1, 4) + _u(0, 2) + _u(8, 2)
    return bytes([0x19, 0x01, 0x01, 0x00]) + _u(16, 4) + base  # string, UTF-8


def _space_msg(shape, v2: bool) -> bytes:
    if v2:
        return bytes([2, len(shape), 0, 0 if not shape else 1]) + b"".join(_u(d, 8) for d in shape)
    return bytes([1, len(shape), 0, 0]) + bytes(4) + b"".join(_u(d, 8) for d in shape)


class Writer:
    def __init__(self, style: str = "v0", user_block: int = 0):
        assert style in ("v0", "v2")
        self.style = style
        self.user_block = user_block
        self.sb_size = 96 if style == "v0" else 48
        self.buf = bytearray(self.sb_size)
        self.root = {"attrs": {}, "members": {}}

    # -- building the tree ----------------------------------------------------------
    def group(self, path: str) -> dict:
        node = self.root
        for part in [p for p in path.split("/") if p]:
            node = node["members"].setdefault(part, {"attrs": {}, "members": {}})
        return node

    def dataset(self, path: str, data, chunks=None, attrs=None, compact=False) -> None:
        parent, _, name = path.rpartition("/")
        self.group(parent)["members"][name] = {"data": np.asarray(data), "chunks": chunks,
                                               "attrs": dict(attrs or {}), "compact": compact}

    # -- file space ---------------------------------------------------------------------
    def alloc(self, data: bytes) -> int:
        self.buf += bytes(-len(self.buf) % 8)
        a = len(self.buf)
        self.buf += data
        return a

    def _gheap_string(self, s: str) -> bytes:
        raw = s.encode("utf-8")
        obj = _u(1, 2) + _u(1, 2) + bytes(4) + _u(len(raw), 8) + _pad8(raw)
        size = max(4096, 16 + len(obj) + 16)
        free = size - 16 - len(obj)
        body = b"GCOL" + bytes([1, 0, 0, 0]) + _u(size, 8) + obj + _u(0, 2) + bytes(6) + _u(free, 8)
        a = self.alloc(body + bytes(size - len(body)))
        return _u(len(raw), 4) + _u(a, 8) + _u(1, 4)

    def _attr_msg(self, name: str, value) -> bytes:
        v2 = self.style == "v2"
        if isinstance(value, str):
            tmsg, smsg, data = _vlen_str_msg(), _space_msg((), v2), self._gheap_string(value)
        else:
            arr = np.asarray(value)
            tmsg, smsg, data = _dtype_msg(arr.dtype), _space_msg(arr.shape, v2), arr.tobytes()
        nm = name.encode() + b"\x00"
        if v2:
            return (bytes([3, 0]) + _u(len(nm), 2) + _u(len(tmsg), 2) + _u(len(smsg), 2) +
                    b"\x01" + nm + tmsg + smsg + data)
        return (bytes([1, 0]) + _u(len(nm), 2) + _u(len(tmsg), 2) + _u(len(smsg), 2) +
                _pad8(nm) + _pad8(tmsg) + _pad8(smsg) + data)

    def _header(self, msgs) -> int:
        """Object header with ``msgs`` [(type, data)]; every message after the
        first attribute goes into a continuation block."""
        first, rest, seen_attr = [], [], False
        for t, d in msgs:
            (rest if seen_attr else first).append((t, d))
            seen_attr = seen_attr or t == 0x0C
        if self.style == "v2":
            def block2(ms):
                return b"".join(bytes([t]) + _u(len(d), 2) + b"\x00" + d for t, d in ms)

            if rest:
                chk = b"OCHK" + block2(rest)
                chk += _u(lookup3(chk), 4)
                first.append((0x10, _u(self.alloc(chk), 8) + _u(len(chk), 8)))
            body = block2(first)
            head = b"OHDR" + bytes([2, 0x02]) + _u(len(body), 4) + body
            return self.alloc(head + _u(lookup3(head), 4))

        def block(ms):
            return b"".join(_u(t, 2) + _u(len(_pad8(d)), 2) + bytes(4) + _pad8(d) for t, d in ms)

        if rest:
            cont = self.alloc(block(rest))
            first.append((0x10, _u(cont, 8) + _u(len(block(rest)), 8)))
        body = block(first)
        head = bytes([1, 0]) + _u(len(first) + len(rest), 2) + _u(1, 4) + _u(len(body), 4) + bytes(4)
        return self.alloc(head + body)

    def _write_dataset(self, node) -> int:
        data, chunks = node["data"], node["chunks"]
        v2 = self.style == "v2"
        msgs = [(0x03, _dtype_msg(data.dtype)), (0x01, _space_msg(data.shape, v2))]
        if node.get("compact"):  # the raw data inside the layout message
            msgs.append((0x08, bytes([3, 0]) + _u(data.nbytes, 2) + data.tobytes()))
        elif chunks is None:
            a = self.alloc(data.tobytes())
            msgs.append((0x08, bytes([3, 1]) + _u(a, 8) + _u(data.nbytes, 8)))
        else:
            item = data.dtype.itemsize
            msgs.append((0x0B, bytes([1, 2]) + bytes(6) +
                         _u(2, 2) + _u(0, 2) + _u(1, 2) + _u(1, 2) + _u(item, 4) + bytes(4) +
                         _u(1, 2) + _u(0, 2) + _u(1, 2) + _u(1, 2) + _u(6, 4) + bytes(4)))
            grid = [range(0, s, c) for s, c in zip(data.shape, chunks)]
            entries = []
            for offs in np.array(np.meshgrid(*grid, indexing="ij")).reshape(len(chunks), -1).T:
                block = np.zeros(chunks, dtype=data.dtype)
                src = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, chunks, data.shape))
                block[tuple(slice(0, x.stop - x.start) for x in src)] = data[src]
                raw = block.tobytes()
                n = len(raw) // item
                raw = np.frombuffer(raw, np.uint8).reshape(n, item).T.tobytes()  # shuffle
                raw = zlib.compress(raw, 6)
                entries.append((tuple(int(o) for o in offs), len(raw), self.alloc(raw)))
            rank = data.ndim

            def key(size, offs):
                return _u(size, 4) + _u(0, 4) + b"".join(_u(o, 8) for o in offs) + _u(0, 8)

            def tree_node(level, items, end):
                tree = b"TREE" + bytes([1, level]) + _u(len(items), 2) + UNDEF + UNDEF
                for offs, size, a in items:
                    tree += key(size, offs) + _u(a, 8)
                return self.alloc(tree + key(0, end))

            # leaves of at most 4 chunks; more than one leaf: a level-1 root
            leaves = [entries[i:i + 4] for i in range(0, len(entries), 4)]
            bounds = [lf[0][0] for lf in leaves[1:]] + [tuple(data.shape)]
            kids = [(lf[0][0], lf[0][1], tree_node(0, lf, end)) for lf, end in zip(leaves, bounds)]
            t = kids[0][2] if len(kids) == 1 else tree_node(1, kids, tuple(data.shape))
            msgs.append((0x08, bytes([3, 2, rank + 1]) + _u(t, 8) +
                         b"".join(_u(c, 4) for c in chunks) + _u(item, 4)))
        msgs += [(0x0C, self._attr_msg(k, v)) for k, v in node["attrs"].items()]
        return self._header(msgs)

    def _write_group(self, node) -> int:
        addrs = {}
        for name, child in node["members"].items():
            addrs[name] = self._write_dataset(child) if "data" in child else self._write_group(child)
        msgs = []
        if self.style == "v2":
            msgs.append((0x02, bytes([0, 0]) + UNDEF + UNDEF))  # link info: compact
            msgs.append((0x0A, bytes([0, 0])))  # group info
            for name, a in addrs.items():
                nm = name.encode()
                msgs.append((0x06, bytes([1, 0x10, 1]) + bytes([len(nm)]) + nm + _u(a, 8)))
        else:
            names = sorted(addrs)
            heap = b"\x00" * 8
            offsets = {}
            for name in names:
                offsets[name] = len(heap)
                heap += _pad8(name.encode() + b"\x00")
            heap_data = self.alloc(heap)
            heap_hdr = self.alloc(b"HEAP" + bytes(4) + _u(len(heap), 8) + UNDEF + _u(heap_data, 8))
            snod = b"SNOD" + bytes([1, 0]) + _u(len(names), 2)
            for name in names:
                snod += _u(offsets[name], 8) + _u(addrs[name], 8) + bytes(8) + bytes(16)
            snod_a = self.alloc(snod)
            last = offsets[names[-1]] if names else 0
            tree = (b"TREE" + bytes([0, 0]) + _u(1, 2) + UNDEF + UNDEF + _u(0, 8) + _u(snod_a, 8) +
                    _u(last, 8))
            tree_a = self.alloc(tree)
            msgs.append((0x11, _u(tree_a, 8) + _u(heap_hdr, 8)))
            node["_symtab"] = (tree_a, heap_hdr)
        msgs += [(0x0C, self._attr_msg(k, v)) for k, v in node["attrs"].items()]
        return self._header(msgs)

    def save(self, path) -> None:
        root = self._write_group(self.root)
        eof = len(self.buf)
        if self.style == "v0":
            tree_a, heap_a = self.root["_symtab"]
            sb = (SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + _u(4, 2) + _u(16, 2) + bytes(4) +
                  _u(0, 8) + UNDEF + _u(eof, 8) + UNDEF +
                  _u(0, 8) + _u(root, 8) + _u(1, 4) + bytes(4) + _u(tree_a, 8) + _u(heap_a, 8))
        else:
            sb = SIG + bytes([2, 8, 8, 0]) + _u(0, 8) + UNDEF + _u(eof, 8) + _u(root, 8)
            sb += _u(lookup3(sb), 4)
        assert len(sb) == self.sb_size
        self.buf[:len(sb)] = sb
        with open(path, "wb") as f:
            f.write(bytes(self.user_block) + bytes(self.buf))
