"""A small read-only HDF5 reader: the parts of the format that the HDF5
library and h5py write with their default, most compatible settings, which
is how LISA Orbits files (the orbit tables lisaanalysistools' ``Orbits``
reads for the reference, ``response.py:13,119``) are written.  It is used by
:func:`orbits.read_lisa_orbits` when h5py is not installed.

Following the HDF5 File Format Specification (version 3.0), it reads:

* superblocks of versions 0 to 3, with or without a user block;
* object headers of versions 1 and 2, with continuation blocks;
* groups stored as symbol tables (version-1 B-tree, symbol table nodes,
  local heap) or as link messages (compact groups);
* datasets with compact, contiguous or chunked (version-1 B-tree index)
  storage; chunk filters deflate, shuffle and Fletcher-32;
* fixed-point and IEEE floating-point data of either byte order, fixed-length
  strings and variable-length strings (global heap), in datasets and in
  attributes stored in the object header.

Dense (fractal-heap) link or attribute storage, the version-4 chunk indexes,
compound, enum, array, reference and opaque types raise
``NotImplementedError`` when reached.  The interface is the subset of h5py's
``File`` / ``Group`` / ``Dataset`` that reading tables needs: ``f["a/b"]``,
``keys()``, ``attrs``, ``shape``, ``dtype``, ``np.asarray(dataset)`` and
slicing a dataset.
"""

from __future__ import annotations

import mmap
import zlib
from typing import Dict, Iterator, List, Optional, Tuple

import numpy as np

_SIGNATURE = b"\x89HDF\r\n\x1a\n"

# header message types
_MSG_NIL = 0x0
_MSG_DATASPACE = 0x1
_MSG_LINK_INFO = 0x2
_MSG_DATATYPE = 0x3
_MSG_LINK = 0x6
_MSG_LAYOUT = 0x8
_MSG_FILTERS = 0xB
_MSG_ATTRIBUTE = 0xC
_MSG_CONTINUATION = 0x10
_MSG_SYMBOL_TABLE = 0x11
_MSG_ATTRIBUTE_INFO = 0x15


class HDF5FormatError(ValueError):
    """The file is not HDF5, or a structure in it is malformed."""


def _u(buf, pos: int, n: int) -> int:
    return int.from_bytes(buf[pos:pos + n], "little")


def _pad8(n: int) -> int:
    return (n + 7) & ~7


class _VlenString:
    """Datatype marker: variable-length string (global heap references)."""

    def __init__(self, size: int, utf8: bool):
        self.itemsize = size
        self.utf8 = utf8


class _FixedString:
    def __init__(self, size: int, utf8: bool, pad: int):
        self.itemsize = size
        self.utf8 = utf8
        self.pad = pad  # 0: null-terminated, 1: null-padded, 2: space-padded


class _File:
    """The mapped file, its offset and length sizes, and the structure parsers."""

    def __init__(self, path: str):
        self._fh = open(path, "rb")
        try:
            self.buf = mmap.mmap(self._fh.fileno(), 0, access=mmap.ACCESS_READ)
        except ValueError:  # an empty file cannot be mapped
            self._fh.close()
            raise HDF5FormatError(f"{path}: not an HDF5 file (empty)")
        self.path = path
        # the superblock sits at 0 or after a user block of 512 * 2^k bytes
        pos = 0
        while pos + 8 <= len(self.buf):
            if self.buf[pos:pos + 8] == _SIGNATURE:
                break
            pos = 512 if pos == 0 else pos * 2
        else:
            self.close()
            raise HDF5FormatError(f"{path}: no HDF5 signature")
        self.base = pos  # file addresses count from the superblock
        b = self.buf
        version = b[pos + 8]
        if version in (0, 1):
            self.so, self.sl = b[pos + 13], b[pos + 14]
            # after the base, free-space, end-of-file and driver addresses, the
            # root group's symbol table entry: name offset, object header address
            root = pos + 24 + (4 if version == 1 else 0) + 5 * self.so
        elif version in (2, 3):
            self.so, self.sl = b[pos + 9], b[pos + 10]
            root = pos + 12 + 3 * self.so  # after base, extension, end-of-file
        else:
            self.close()
            raise HDF5FormatError(f"{path}: superblock version {version} is not supported")
        if self.so not in (2, 4, 8) or self.sl not in (2, 4, 8):
            self.close()
            raise HDF5FormatError(f"{path}: offset/length sizes {self.so}/{self.sl}")
        self._undef = (1 << (8 * self.so)) - 1
        self.root = self.addr(root)
        self._headers: Dict[int, List[Tuple[int, int, int]]] = {}

    def close(self) -> None:
        if getattr(self, "buf", None) is not None:
            self.buf.close()
            self.buf = None
        if not self._fh.closed:
            self._fh.close()

    # -- primitive reads ---------------------------------------------------------
    def addr(self, pos: int) -> Optional[int]:
        """A file address at absolute position ``pos`` (None when undefined)."""
        a = _u(self.buf, pos, self.so)
        return None if a == self._undef else a

    def at(self, a: int) -> int:
        """Absolute position of file address ``a``."""
        p = self.base + a
        if p >= len(self.buf):
            raise HDF5FormatError(f"{self.path}: address {a} beyond the end of the file")
        return p

    def length(self, pos: int) -> int:
        return _u(self.buf, pos, self.sl)

    def expect(self, pos: int, sig: bytes) -> None:
        if self.buf[pos:pos + 4] != sig:
            raise HDF5FormatError(f"{self.path}: expected {sig!r} at {pos - self.base}")

    # -- object headers -------------------------------------------------------------
    def messages(self, a: int) -> List[Tuple[int, int, int]]:
        """(type, absolute position of the data, data size) of each message of
        the object header at address ``a``, continuation blocks followed."""
        if a in self._headers:
            return self._headers[a]
        b = self.buf
        p = self.at(a)
        out: List[Tuple[int, int, int]] = []
        blocks: List[Tuple[int, int, int]] = []  # (start, end, header version)
        if b[p:p + 4] == b"OHDR":
            if b[p + 4] != 2:
                raise HDF5FormatError(f"{self.path}: object header version {b[p + 4]}")
            flags = b[p + 5]
            q = p + 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
            n = 1 << (flags & 3)
            size0 = _u(b, q, n)  # message bytes; the checksum follows them
            blocks.append((q + n, q + n + size0, 2))
            order = bool(flags & 0x04)
        else:
            if b[p] != 1:
                raise HDF5FormatError(f"{self.path}: object header version {b[p]} at {a}")
            size0 = _u(b, p + 8, 4)
            blocks.append((p + 16, p + 16 + size0, 1))
            order = False
        i = 0
        while i < len(blocks):
            start, end, v = blocks[i]
            i += 1
            q = start
            if v == 1:
                while q + 8 <= end:
                    mtype, msize = _u(b, q, 2), _u(b, q + 2, 2)
                    data = q + 8
                    if data + msize > end:
                        raise HDF5FormatError(f"{self.path}: message overruns its header")
                    out.append((mtype, data, msize))
                    if mtype == _MSG_CONTINUATION:
                        c = self.at(self.addr(data))
                        blocks.append((c, c + self.length(data + self.so), 1))
                    q = data + msize
            else:
                hdr = 6 if order else 4
                while q + hdr <= end:
                    mtype, msize = b[q], _u(b, q + 1, 2)
                    data = q + hdr
                    if data + msize > end:
                        raise HDF5FormatError(f"{self.path}: message overruns its header")
                    out.append((mtype, data, msize))
                    if mtype == _MSG_CONTINUATION:
                        c = self.at(self.addr(data))
                        self.expect(c, b"OCHK")
                        # the block's length counts its signature and checksum
                        blocks.append((c + 4, c + self.length(data + self.so) - 4, 2))
                    q = data + msize
        self._headers[a] = out
        return out

    def find(self, a: int, mtype: int) -> Optional[Tuple[int, int]]:
        for t, pos, size in self.messages(a):
            if t == mtype:
                return pos, size
        return None

    # -- datatypes and dataspaces -----------------------------------------------------
    def datatype(self, pos: int):
        """numpy dtype, or a string marker, of the datatype message at ``pos``."""
        b = self.buf
        cls = b[pos] & 0x0F
        bits = _u(b, pos + 1, 3)
        size = _u(b, pos + 4, 4)
        if cls == 0:  # fixed-point
            order = ">" if bits & 1 else "<"
            if size not in (1, 2, 4, 8):
                raise NotImplementedError(f"{size}-byte integers")
            return np.dtype(f"{order}{'i' if bits & 8 else 'u'}{size}")
        if cls == 1:  # floating-point
            if bits & 0x40:
                raise NotImplementedError("VAX floating-point order")
            order = ">" if bits & 1 else "<"
            exp_loc, exp_size, man_loc, man_size = b[pos + 12], b[pos + 13], b[pos + 14], b[pos + 15]
            ieee = {2: (10, 5, 0, 10), 4: (23, 8, 0, 23), 8: (52, 11, 0, 52)}
            if ieee.get(size) != (exp_loc, exp_size, man_loc, man_size):
                raise NotImplementedError(f"non-IEEE {size}-byte floating point")
            return np.dtype(f"{order}f{size}")
        if cls == 3:  # fixed-length string
            return _FixedString(size, (bits >> 4) & 0xF == 1, bits & 0xF)
        if cls == 9 and bits & 0xF == 1:  # variable-length string
            return _VlenString(size, (bits >> 8) & 0xF == 1)
        raise NotImplementedError(f"HDF5 datatype class {cls}")

    def dataspace(self, pos: int) -> Optional[Tuple[int, ...]]:
        """Shape of the dataspace message at ``pos`` (None: the null space)."""
        b = self.buf
        version, ndim = b[pos], b[pos + 1]
        if version == 1:
            q = pos + 8
        elif version == 2:
            if b[pos + 3] == 2:
                return None
            q = pos + 4
        else:
            raise HDF5FormatError(f"{self.path}: dataspace version {version}")
        return tuple(self.length(q + i * self.sl) for i in range(ndim))

    # -- data ---------------------------------------------------------------------------
    def decode(self, raw: bytes, dtype, shape: Tuple[int, ...]):
        """Elements of ``dtype`` in ``raw`` as an array of ``shape``."""
        count = int(np.prod(shape, dtype=np.int64)) if shape else 1
        if isinstance(dtype, np.dtype):
            arr = np.frombuffer(raw, dtype=dtype, count=count).copy()
            return arr.astype(dtype.newbyteorder("="), copy=False).reshape(shape)
        if isinstance(dtype, _FixedString):
            arr = np.frombuffer(raw, dtype=f"S{dtype.itemsize}", count=count).copy()
            return arr.reshape(shape)
        out = np.empty(count, dtype=object)
        for i in range(count):
            q = i * dtype.itemsize
            n = _u(raw, q, 4)
            coll = _u(raw, q + 4, self.so)
            index = _u(raw, q + 4 + self.so, 4)
            data = self.global_heap_object(coll, index)[:n]
            out[i] = data.decode("utf-8" if dtype.utf8 else "ascii", errors="replace")
        return out.reshape(shape)

    def global_heap_object(self, a: int, index: int) -> bytes:
        b = self.buf
        p = self.at(a)
        self.expect(p, b"GCOL")
        end = p + self.length(p + 8)
        q = p + 8 + self.sl
        while q + 8 + self.sl <= end:
            idx = _u(b, q, 2)
            size = self.length(q + 8)
            if idx == 0:
                break
            if idx == index:
                return bytes(b[q + 8 + self.sl:q + 8 + self.sl + size])
            q += 8 + self.sl + _pad8(size)
        raise HDF5FormatError(f"{self.path}: global heap object {index} not found")

    def filters(self, a: int) -> List[Tuple[int, Tuple[int, ...]]]:
        """(filter id, client values) of the object's filter pipeline."""
        m = self.find(a, _MSG_FILTERS)
        if m is None:
            return []
        b = self.buf
        pos = m[0]
        version, count = b[pos], b[pos + 1]
        q = pos + (8 if version == 1 else 2)
        out = []
        for _ in range(count):
            fid = _u(b, q, 2)
            q += 2
            name_len = 0
            if version == 1 or fid >= 256:
                name_len = _u(b, q, 2)
                q += 2
            nvals = _u(b, q + 2, 2)
            q += 4
            q += _pad8(name_len) if version == 1 else name_len
            vals = tuple(_u(b, q + 4 * i, 4) for i in range(nvals))
            q += 4 * nvals
            if version == 1 and nvals % 2:
                q += 4
            out.append((fid, vals))
        return out

    def unfilter(self, raw: bytes, pipeline, mask: int, itemsize: int) -> bytes:
        for i in range(len(pipeline) - 1, -1, -1):
            if mask & (1 << i):
                continue
            fid, vals = pipeline[i]
            if fid == 1:
                raw = zlib.decompress(raw)
            elif fid == 2:
                size = vals[0] if vals else itemsize
                n = len(raw) // size
                body = np.frombuffer(raw[:n * size], dtype=np.uint8).reshape(size, n)
                raw = body.T.tobytes() + raw[n * size:]
            elif fid == 3:
                raw = raw[:-4]
            else:
                raise NotImplementedError(f"HDF5 filter {fid}")
        return raw

    def read_dataset(self, a: int, dtype, shape: Tuple[int, ...]):
        b = self.buf
        m = self.find(a, _MSG_LAYOUT)
        if m is None:
            raise HDF5FormatError(f"{self.path}: dataset without a layout message")
        pos = m[0]
        version = b[pos]
        itemsize = dtype.itemsize
        count = int(np.prod(shape, dtype=np.int64)) if shape else 1
        nbytes = count * itemsize
        if version in (1, 2):
            ndim, cls = b[pos + 1], b[pos + 2]
            q = pos + 8
            if cls == 0:
                q += 4 * ndim
                size = _u(b, q, 4)
                return self.decode(bytes(b[q + 4:q + 4 + size]), dtype, shape)
            data_addr = self.addr(q)
            q += self.so
            dims = tuple(_u(b, q + 4 * i, 4) for i in range(ndim))
            if cls == 1:
                return self._contiguous(data_addr, nbytes, dtype, shape)
            return self._chunked(a, data_addr, dims[:len(shape)], dtype, shape)
        if version in (3, 4):
            cls = b[pos + 1]
            if cls == 0:
                size = _u(b, pos + 2, 2)
                return self.decode(bytes(b[pos + 4:pos + 4 + size]), dtype, shape)
            if cls == 1:
                return self._contiguous(self.addr(pos + 2), nbytes, dtype, shape)
            if cls == 2 and version == 3:
                ndim = b[pos + 2]
                data_addr = self.addr(pos + 3)
                q = pos + 3 + self.so
                dims = tuple(_u(b, q + 4 * i, 4) for i in range(ndim))
                return self._chunked(a, data_addr, dims[:-1], dtype, shape)
            raise NotImplementedError(f"layout version {version} class {cls}")
        raise HDF5FormatError(f"{self.path}: layout version {version}")

    def _contiguous(self, data_addr, nbytes, dtype, shape):
        if data_addr is None:  # never written: the default fill value
            return self.decode(bytes(nbytes), dtype, shape)
        p = self.at(data_addr)
        if p + nbytes > len(self.buf):
            raise HDF5FormatError(f"{self.path}: dataset runs past the end of the file")
        return self.decode(bytes(self.buf[p:p + nbytes]), dtype, shape)

    def _chunked(self, a, btree, chunk, dtype, shape):
        if not isinstance(dtype, np.dtype):
            raise NotImplementedError("chunked string datasets")
        out = np.zeros(shape, dtype=dtype.newbyteorder("="))
        if btree is None:
            return out
        pipeline = self.filters(a)
        rank = len(shape)
        chunk_bytes = int(np.prod(chunk, dtype=np.int64)) * dtype.itemsize
        for offsets, size, mask, addr in self._chunk_entries(btree, rank):
            raw = bytes(self.buf[self.at(addr):self.at(addr) + size])
            raw = self.unfilter(raw, pipeline, mask, dtype.itemsize)
            if len(raw) < chunk_bytes:
                raise HDF5FormatError(f"{self.path}: short chunk at {offsets}")
            block = np.frombuffer(raw[:chunk_bytes], dtype=dtype).reshape(chunk)
            dst = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offsets, chunk, shape))
            src = tuple(slice(0, d.stop - d.start) for d in dst)
            out[dst] = block[src]
        return out

    def _chunk_entries(self, a: int, rank: int) -> Iterator[Tuple[Tuple[int, ...], int, int, int]]:
        b = self.buf
        p = self.at(a)
        self.expect(p, b"TREE")
        if b[p + 4] != 1:
            raise HDF5FormatError(f"{self.path}: B-tree at {a} is not a chunk index")
        level, used = b[p + 5], _u(b, p + 6, 2)
        key = 8 + 8 * (rank + 1)
        q = p + 8 + 2 * self.so
        for i in range(used):
            k = q + i * (key + self.so)
            child = self.addr(k + key)
            if level > 0:
                yield from self._chunk_entries(child, rank)
            else:
                offsets = tuple(_u(b, k + 8 + 8 * d, 8) for d in range(rank))
                yield offsets, _u(b, k, 4), _u(b, k + 4, 4), child

    # -- groups ---------------------------------------------------------------------------
    def links(self, a: int) -> Dict[str, int]:
        """Name -> object header address of each hard link of the group at ``a``."""
        out: Dict[str, int] = {}
        st = self.find(a, _MSG_SYMBOL_TABLE)
        if st is not None:
            btree = self.addr(st[0])
            heap = self.at(self.addr(st[0] + self.so))
            self.expect(heap, b"HEAP")
            names = self.at(self.addr(heap + 8 + 2 * self.sl))
            self._symbol_nodes(btree, names, out)
            return out
        dense = False
        for t, pos, size in self.messages(a):
            if t == _MSG_LINK:
                self._link(pos, out)
            elif t == _MSG_LINK_INFO:
                flags = self.buf[pos + 1]
                q = pos + 2 + (8 if flags & 1 else 0)
                dense = dense or self.addr(q) is not None
        if dense:
            raise NotImplementedError("groups with dense (fractal heap) link storage")
        return out

    def _symbol_nodes(self, a: int, names: int, out: Dict[str, int]) -> None:
        b = self.buf
        p = self.at(a)
        self.expect(p, b"TREE")
        level, used = b[p + 5], _u(b, p + 6, 2)
        q = p + 8 + 2 * self.so
        for i in range(used):
            child = self.addr(q + self.sl + i * (self.sl + self.so))
            if level > 0:
                self._symbol_nodes(child, names, out)
                continue
            s = self.at(child)
            self.expect(s, b"SNOD")
            for j in range(_u(b, s + 6, 2)):
                e = s + 8 + j * (2 * self.so + 24)
                name_off = _u(b, e, self.so)
                start = names + name_off
                stop = b.find(b"\x00", start)
                out[b[start:stop].decode("utf-8")] = self.addr(e + self.so)

    def _link(self, pos: int, out: Dict[str, int]) -> None:
        b = self.buf
        flags = b[pos + 1]
        q = pos + 2
        ltype = 0
        if flags & 0x08:
            ltype = b[q]
            q += 1
        if flags & 0x04:
            q += 8
        if flags & 0x10:
            q += 1
        n = 1 << (flags & 3)
        name_len = _u(b, q, n)
        q += n
        name = bytes(b[q:q + name_len]).decode("utf-8")
        q += name_len
        if ltype == 0:
            out[name] = self.addr(q)

    def attributes(self, a: int) -> Dict[str, Tuple[int, int]]:
        """Name -> (position, size) of each attribute message of the object."""
        out: Dict[str, Tuple[int, int]] = {}
        dense = False
        for t, pos, size in self.messages(a):
            if t == _MSG_ATTRIBUTE:
                out[self._attribute_fields(pos)[0]] = (pos, size)
            elif t == _MSG_ATTRIBUTE_INFO:
                flags = self.buf[pos + 1]
                q = pos + 2 + (2 if flags & 1 else 0)
                dense = dense or self.addr(q) is not None
        if dense:
            out["\x00dense"] = (0, 0)
        return out

    def _attribute_fields(self, pos: int):
        """(name, datatype position, dataspace position, data position)."""
        b = self.buf
        version = b[pos]
        name_size, type_size, space_size = _u(b, pos + 2, 2), _u(b, pos + 4, 2), _u(b, pos + 6, 2)
        if version == 1:
            q = pos + 8
            name = bytes(b[q:q + name_size]).split(b"\x00")[0].decode("utf-8")
            q += _pad8(name_size)
            tpos = q
            q += _pad8(type_size)
            spos = q
            q += _pad8(space_size)
        elif version in (2, 3):
            if b[pos + 1] & 3:
                raise NotImplementedError("attributes with shared datatypes or dataspaces")
            q = pos + 8 + (1 if version == 3 else 0)
            name = bytes(b[q:q + name_size]).split(b"\x00")[0].decode("utf-8")
            q += name_size
            tpos = q
            q += type_size
            spos = q
            q += space_size
        else:
            raise HDF5FormatError(f"{self.path}: attribute message version {version}")
        return name, tpos, spos, q

    def attribute_value(self, pos: int):
        _, tpos, spos, dpos = self._attribute_fields(pos)
        dtype = self.datatype(tpos)
        shape = self.dataspace(spos)
        if shape is None:
            return None
        count = int(np.prod(shape, dtype=np.int64)) if shape else 1
        raw = bytes(self.buf[dpos:dpos + count * dtype.itemsize])
        value = self.decode(raw, dtype, shape)
        return value[()] if shape == () else value


class AttributeManager:
    """Read-only mapping of an object's attributes (h5py's ``obj.attrs``)."""

    def __init__(self, f: _File, a: int):
        self._f = f
        self._a = a
        self._index = f.attributes(a)
        self._dense = self._index.pop("\x00dense", None) is not None

    def __getitem__(self, name: str):
        if name not in self._index:
            if self._dense:
                raise NotImplementedError("objects with dense (fractal heap) attribute storage")
            raise KeyError(name)
        return self._f.attribute_value(self._index[name][0])

    def __contains__(self, name) -> bool:
        return name in self._index

    def __iter__(self):
        return iter(self._index)

    def __len__(self) -> int:
        return len(self._index)

    def keys(self):
        return self._index.keys()

    def get(self, name, default=None):
        return self[name] if name in self._index else default


class Dataset:
    """A dataset; read it with ``np.asarray(ds)``, ``ds[()]`` or ``ds[slices]``."""

    def __init__(self, f: _File, a: int, name: str):
        self._f, self._a, self.name = f, a, name
        t = f.find(a, _MSG_DATATYPE)
        s = f.find(a, _MSG_DATASPACE)
        if t is None or s is None:
            raise HDF5FormatError(f"{f.path}: {name} has no datatype or dataspace")
        self._dtype = f.datatype(t[0])
        shape = f.dataspace(s[0])
        self.shape = () if shape is None else shape
        self._null = shape is None
        self.attrs = AttributeManager(f, a)

    @property
    def dtype(self):
        d = self._dtype
        return d.newbyteorder("=") if isinstance(d, np.dtype) else np.dtype(object)

    @property
    def ndim(self) -> int:
        return len(self.shape)

    @property
    def size(self) -> int:
        return int(np.prod(self.shape, dtype=np.int64))

    def read(self):
        if self._null:
            return np.empty((0,), dtype=self.dtype)
        return self._f.read_dataset(self._a, self._dtype, self.shape)

    def __getitem__(self, key):
        return self.read()[key]

    def __array__(self, dtype=None, copy=None):
        arr = self.read()
        return arr if dtype is None else arr.astype(dtype, copy=False)

    def __len__(self) -> int:
        if not self.shape:
            raise TypeError("len() of a scalar dataset")
        return self.shape[0]

    def __repr__(self) -> str:
        return f"<HDF5 dataset {self.name!r}: shape {self.shape}, type {self.dtype}>"


class Group:
    """A group: ``g["name"]`` or ``g["a/b"]``, ``keys()``, ``attrs``."""

    def __init__(self, f: _File, a: int, name: str):
        self._f, self._a, self.name = f, a, name
        self._links = None
        self.attrs = AttributeManager(f, a)

    def _names(self) -> Dict[str, int]:
        if self._links is None:
            self._links = self._f.links(self._a)
        return self._links

    def keys(self):
        return self._names().keys()

    def __iter__(self):
        return iter(self._names())

    def __len__(self) -> int:
        return len(self._names())

    def __contains__(self, path) -> bool:
        try:
            self[path]
        except KeyError:
            return False
        return True

    def __getitem__(self, path: str):
        node = self
        parts = [p for p in path.split("/") if p]
        for i, part in enumerate(parts):
            if not isinstance(node, Group):
                raise KeyError(path)
            links = node._names()
            if part not in links:
                raise KeyError(path)
            a = links[part]
            full = (node.name.rstrip("/") + "/" + part)
            node = Group(self._f, a, full) if self._f.find(a, _MSG_LAYOUT) is None \
                else Dataset(self._f, a, full)
        return node

    def __repr__(self) -> str:
        return f"<HDF5 group {self.name!r} ({len(self)} members)>"


class File(Group):
    """An HDF5 file opened for reading (``mode`` must be "r")."""

    def __init__(self, path, mode: str = "r"):
        if mode != "r":
            raise ValueError("h5lite reads files only (mode 'r')")
        self._file = _File(str(path))
        super().__init__(self._file, self._file.root, "/")
        self.filename = str(path)

    def close(self) -> None:
        self._file.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False
