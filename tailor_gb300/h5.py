"""Minimal HDF5 reader for the reference's case, rule and result files.

No HDF5 library exists in this environment, so the files the reference
exchanges -- structured source samples (read by interpolate.py:170-215),
prepared FD-q cases (written by PETSc's HDF5 viewer and h5py,
interpolate.py:355-437; read by Prepare.cpp:443-687) and FD-q rule caches
(fdq_nodes.py:470-565) -- are parsed here directly from the published HDF5
file format.  Supported: superblock versions 0 and 1, version-1 object
headers with continuation blocks, old-style groups (symbol table, v1 B-tree
and local heap), contiguous, compact and chunked (v1 B-tree, unfiltered)
dataset layouts, fixed-point and IEEE floating-point element types,
fixed-length and variable-length strings (global heap) and compact
attributes.  Anything else raises ``H5Error``, never a silent misread.

    with h5.File(path) as f:
        f.attrs["Ny"], f["grid"][...]      # numpy arrays
        f["discretization/y"].attrs, list(f["discretization"])
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(ValueError):
    pass


def _guard(fn):
    """Report a damaged or truncated file as H5Error, never as an index or
    decoding error from deep inside the parser."""
    def wrapped(*a, **k):
        try:
            return fn(*a, **k)
        except H5Error:
            raise
        except KeyError:
            raise
        except (IndexError, ValueError, OverflowError, RecursionError, UnicodeDecodeError,
                TypeError, MemoryError) as e:
            raise H5Error(f"damaged or truncated HDF5 file ({type(e).__name__}: {e})") from e
    wrapped.__name__, wrapped.__doc__ = fn.__name__, fn.__doc__
    return wrapped


class _Reader:
    def __init__(self, data: bytes):
        self.d = data
        if data[:8] != _SIG:
            raise H5Error("not an HDF5 file (no superblock signature at offset 0)")
        ver = data[8]
        if ver not in (0, 1):
            raise H5Error(f"superblock version {ver} is not supported")
        self.so, self.sl = data[13], data[14]
        if self.so != 8 or self.sl != 8:
            raise H5Error("only 8-byte offsets and lengths are supported")
        p = 24 + (4 if ver == 1 else 0)
        self.base = self.u(p, 8)
        p += 32  # base, free-space, end-of-file and driver addresses
        self.root_entry = p
        self._gheaps: dict[int, dict[int, bytes]] = {}

    def u(self, p: int, n: int) -> int:
        return int.from_bytes(self.d[p:p + n], "little")

    def addr(self, a: int) -> int:
        return self.base + a

    # ---- object headers -------------------------------------------------
    def messages(self, oh: int) -> list[tuple[int, bytes]]:
        p = self.addr(oh)
        if self.d[p] != 1:
            raise H5Error(f"object header version {self.d[p]} is not supported")
        nmsg = self.u(p + 2, 2)
        size = self.u(p + 8, 4)
        blocks = [(p + 16, size)]
        out: list[tuple[int, bytes]] = []
        while blocks and len(out) < nmsg:
            q, n = blocks.pop(0)
            end = q + n
            while q + 8 <= end and len(out) < nmsg:
                mtype, msize = self.u(q, 2), self.u(q + 2, 2)
                body = self.d[q + 8:q + 8 + msize]
                out.append((mtype, body))
                if mtype == 0x10:  # continuation
                    blocks.append((self.addr(int.from_bytes(body[:8], "little")),
                                   int.from_bytes(body[8:16], "little")))
                q += 8 + msize
        return out

    # ---- groups -----------------------------------------------------------
    def heap_data(self, heap: int) -> int:
        p = self.addr(heap)
        if self.d[p:p + 4] != b"HEAP":
            raise H5Error("bad local heap signature")
        return self.addr(self.u(p + 24, 8))

    def cstr(self, p: int) -> str:
        e = self.d.index(b"\x00", p)
        return self.d[p:e].decode("utf-8")

    def group_links(self, btree: int, heap: int) -> dict[str, int]:
        hd = self.heap_data(heap)
        links: dict[str, int] = {}

        def walk(node: int) -> None:
            p = self.addr(node)
            if self.d[p:p + 4] != b"TREE" or self.d[p + 4] != 0:
                raise H5Error("bad group B-tree node")
            level, used = self.d[p + 5], self.u(p + 6, 2)
            q = p + 24 + 8  # after header and key 0
            for _ in range(used):
                child = self.u(q, 8)
                q += 16  # child address and the next key
                if level > 0:
                    walk(child)
                    continue
                s = self.addr(child)
                if self.d[s:s + 4] != b"SNOD":
                    raise H5Error("bad symbol table node")
                for k in range(self.u(s + 6, 2)):
                    e = s + 8 + 40 * k
                    links[self.cstr(hd + self.u(e, 8))] = self.u(e + 8, 8)

        walk(btree)
        return links

    # ---- global heap (variable-length data) --------------------------------
    def gheap_object(self, coll: int, index: int) -> bytes:
        if coll not in self._gheaps:
            p = self.addr(coll)
            if self.d[p:p + 4] != b"GCOL":
                raise H5Error("bad global heap signature")
            size = self.u(p + 8, 8)
            end, q, objs = p + size, p + 16, {}
            while q + 16 <= end:
                idx, osize = self.u(q, 2), self.u(q + 8, 8)
                if idx == 0:
                    break
                objs[idx] = self.d[q + 16:q + 16 + osize]
                q += 16 + ((osize + 7) & ~7)
            self._gheaps[coll] = objs
        return self._gheaps[coll][index]


def _link(b: bytes) -> tuple[str, int | None]:
    """Name and object header address of a hard link (None: soft/external)."""
    if b[0] != 1:
        raise H5Error(f"link message version {b[0]} is not supported")
    flags, p = b[1], 2
    ltype = 0
    if flags & 0x08:
        ltype = b[p]
        p += 1
    if flags & 0x04:
        p += 8
    if flags & 0x10:
        p += 1
    nl = 1 << (flags & 0x03)
    n = int.from_bytes(b[p:p + nl], "little")
    p += nl
    name = b[p:p + n].decode("utf-8")
    p += n
    if ltype != 0:
        return name, None
    return name, int.from_bytes(b[p:p + 8], "little")


def _dataspace(b: bytes) -> tuple[int, ...] | None:
    ver, rank, flags = b[0], b[1], b[2]
    if ver == 1:
        p = 8
    elif ver == 2:
        if b[3] == 2:
            return None  # null dataspace
        p = 4
    else:
        raise H5Error(f"dataspace version {ver} is not supported")
    return tuple(int.from_bytes(b[p + 8 * i:p + 8 * i + 8], "little") for i in range(rank))


class _Type:
    """An element type: numpy dtype, or a string kind."""

    def __init__(self, b: bytes):
        cls, bits, size = b[0] & 0x0F, b[1:4], int.from_bytes(b[4:8], "little")
        self.size, self.kind, self.dtype = size, None, None
        order = ">" if bits[0] & 1 else "<"
        if cls == 0:  # fixed point
            signed = bool(bits[0] & 0x08)
            self.dtype = np.dtype(f"{order}{'i' if signed else 'u'}{size}")
        elif cls == 1:  # IEEE floating point
            if size not in (4, 8):
                raise H5Error(f"floating-point size {size} is not supported")
            self.dtype = np.dtype(f"{order}f{size}")
        elif cls == 3:  # fixed-length string
            self.kind = "fstring"
        elif cls == 9:  # variable length: string or sequence
            if (bits[0] & 0x0F) != 1:
                raise H5Error("variable-length sequences are not supported")
            self.kind = "vstring"
        else:
            raise H5Error(f"datatype class {cls} is not supported")


def _split_attr(b: bytes) -> tuple[str, bytes, bytes, bytes]:
    ver = b[0]
    nsz, tsz, ssz = (int.from_bytes(b[i:i + 2], "little") for i in (2, 4, 6))
    pad = (lambda n: (n + 7) & ~7) if ver == 1 else (lambda n: n)
    p = 8 if ver in (1, 2) else 9
    if ver not in (1, 2, 3):
        raise H5Error(f"attribute message version {ver} is not supported")
    name = b[p:p + nsz].split(b"\x00")[0].decode("utf-8")
    p += pad(nsz)
    t = b[p:p + tsz]
    p += pad(tsz)
    s = b[p:p + ssz]
    p += pad(ssz)
    return name, t, s, b[p:]


def _decode(r: _Reader, t: _Type, shape: tuple[int, ...], raw: bytes):
    count = int(np.prod(shape)) if shape else 1
    if t.dtype is not None:
        a = np.frombuffer(raw[:count * t.size], dtype=t.dtype).astype(t.dtype.newbyteorder("="))
        return a.reshape(shape) if shape else a[0]
    if t.kind == "fstring":
        vals = [raw[i * t.size:(i + 1) * t.size].split(b"\x00")[0].decode("utf-8")
                for i in range(count)]
    else:  # variable-length string: length, collection address, object index
        vals = []
        for i in range(count):
            q = i * 16
            n = int.from_bytes(raw[q:q + 4], "little")
            coll = int.from_bytes(raw[q + 4:q + 12], "little")
            idx = int.from_bytes(raw[q + 12:q + 16], "little")
            vals.append(r.gheap_object(coll, idx)[:n].decode("utf-8") if n else "")
    return vals[0] if not shape else np.array(vals, dtype=object).reshape(shape)


class Dataset:
    def __init__(self, r: _Reader, msgs):
        self._r = r
        self.attrs: dict = {}
        self.shape: tuple[int, ...] | None = None
        self._type = None
        self._layout = None
        for mtype, b in msgs:
            if mtype == 0x1:
                self.shape = _dataspace(b)
            elif mtype == 0x3:
                self._type = _Type(b)
            elif mtype == 0x8:
                self._layout = b
            elif mtype == 0xB:
                raise H5Error("filtered (compressed) datasets are not supported")
            elif mtype == 0xC:
                name, t, s, data = _split_attr(b)
                self.attrs[name] = _decode(r, _Type(t), _dataspace(s) or (), data)
        if self._type is None or self._layout is None:
            raise H5Error("dataset without datatype or layout message")

    @property
    def dtype(self):
        return self._type.dtype

    def _raw(self) -> bytes:
        r, b = self._r, self._layout
        shape = self.shape or ()
        nbytes = (int(np.prod(shape)) if shape else 1) * self._type.size
        ver = b[0]
        if ver == 3:
            cls = b[1]
            if cls == 0:  # compact
                n = int.from_bytes(b[2:4], "little")
                return b[4:4 + n]
            if cls == 1:  # contiguous
                a = int.from_bytes(b[2:10], "little")
                if a == _UNDEF:
                    return bytes(nbytes)
                if r.addr(a) + nbytes > len(r.d):
                    raise H5Error("dataset extends past the end of the file")
                return r.d[r.addr(a):r.addr(a) + nbytes]
            if cls == 2:  # chunked
                rank = b[2] - 1
                bt = int.from_bytes(b[3:11], "little")
                cdims = [int.from_bytes(b[11 + 4 * i:15 + 4 * i], "little") for i in range(rank)]
                return self._chunked(bt, cdims, shape, nbytes)
        elif ver in (1, 2):
            rank, cls = b[1], b[2]
            if cls == 1:
                a = int.from_bytes(b[8:16], "little")
                return r.d[r.addr(a):r.addr(a) + nbytes]
            if cls == 2:
                bt = int.from_bytes(b[8:16], "little")
                cdims = [int.from_bytes(b[16 + 4 * i:20 + 4 * i], "little")
                         for i in range(rank - 1)]
                return self._chunked(bt, cdims, shape, nbytes)
        raise H5Error(f"data layout version {ver} class is not supported")

    def _chunked(self, bt: int, cdims, shape, nbytes: int) -> bytes:
        r, es = self._r, self._type.size
        if nbytes > 64 * len(r.d) + (1 << 20):
            raise H5Error("chunked dataset far larger than the file")
        rank = len(cdims)
        out = np.zeros(nbytes, dtype=np.uint8)
        view = out.reshape(tuple(shape) + (es,)) if shape else out

        def walk(node: int) -> None:
            p = r.addr(node)
            if r.d[p:p + 4] != b"TREE" or r.d[p + 4] != 1:
                raise H5Error("bad chunk B-tree node")
            level, used = r.d[p + 5], r.u(p + 6, 2)
            ksz = 8 + 8 * (rank + 1)
            q = p + 24
            for _ in range(used):
                csize, mask = r.u(q, 4), r.u(q + 4, 4)
                offs = [r.u(q + 8 + 8 * i, 8) for i in range(rank)]
                child = r.u(q + ksz, 8)
                q += ksz + 8
                if level > 0:
                    walk(child)
                    continue
                if mask:
                    raise H5Error("filtered chunks are not supported")
                buf = np.frombuffer(r.d[r.addr(child):r.addr(child) + csize], dtype=np.uint8)
                chunk = buf[:int(np.prod(cdims)) * es].reshape(tuple(cdims) + (es,))
                sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cdims, shape))
                view[sl] = chunk[tuple(slice(0, x.stop - x.start) for x in sl)]

        walk(bt)
        return out.tobytes()

    @_guard
    def __getitem__(self, key):
        a = _decode(self._r, self._type, self.shape or (), self._raw())
        return a if key is Ellipsis or key == () else a[key]


class Group:
    def __init__(self, r: _Reader, msgs):
        self._r = r
        self.attrs: dict = {}
        self._links: dict[str, int] = {}
        for mtype, b in msgs:
            if mtype == 0x11:
                self._links = r.group_links(int.from_bytes(b[:8], "little"),
                                            int.from_bytes(b[8:16], "little"))
            elif mtype == 0xC:
                name, t, s, data = _split_attr(b)
                self.attrs[name] = _decode(r, _Type(t), _dataspace(s) or (), data)
            elif mtype == 0x6:  # link message (compact new-style group)
                name, target = _link(b)
                if target is not None:
                    self._links[name] = target
            elif mtype == 0x2:  # link info: dense link storage is not supported
                flags = b[1]
                q = 2 + (8 if flags & 1 else 0)
                if int.from_bytes(b[q:q + 8], "little") != _UNDEF:
                    raise H5Error("groups with dense link storage are not supported")

    def __iter__(self):
        return iter(sorted(self._links))

    def __contains__(self, name: str) -> bool:
        try:
            self[name]
        except KeyError:
            return False
        return True

    def keys(self):
        return sorted(self._links)

    @_guard
    def __getitem__(self, path: str):
        node = self
        for part in [x for x in path.split("/") if x]:
            if not isinstance(node, Group) or part not in node._links:
                raise KeyError(path)
            msgs = node._r.messages(node._links[part])
            kinds = {m for m, _ in msgs}
            node = (Group(node._r, msgs) if kinds & {0x11, 0x2, 0x6} and 0x8 not in kinds
                    else Dataset(node._r, msgs))
        return node


class File(Group):
    @_guard
    def __init__(self, path: str | Path):
        r = _Reader(Path(path).read_bytes())
        oh = r.u(r.root_entry + 8, 8)
        super().__init__(r, r.messages(oh))

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False


# ---- writer -----------------------------------------------------------------
# The writer emits the classic layout every HDF5 reader accepts: superblock
# version 0 (group leaf K 4, internal K 16), version-1 object headers,
# old-style groups (v1 B-tree, symbol table nodes of at most 2K = 8 entries,
# local heap whose free list ends with the library's null offset 1),
# contiguous datasets and compact attributes (64-bit integers, doubles,
# unsigned bytes, fixed-length null-terminated ASCII strings).  Encodings
# follow files written by the HDF5 library itself (B-tree nodes and symbol
# table nodes are allocated at their full capacity, since readers load them
# whole).

_LEAF_K, _INTERNAL_K = 4, 16


def _pad8(b: bytes) -> bytes:
    return b + bytes((-len(b)) % 8)


def _dtype_msg(a: np.ndarray | np.generic | str) -> tuple[bytes, int]:
    """Datatype message body and element size."""
    if isinstance(a, str):
        n = len(a.encode("ascii")) + 1
        return bytes([0x13, 0x00, 0x00, 0x00]) + n.to_bytes(4, "little"), n
    dt = np.asarray(a).dtype
    if dt == np.float64:
        return (bytes([0x11, 0x20, 0x3F, 0x00]) + (8).to_bytes(4, "little")
                + (0).to_bytes(2, "little") + (64).to_bytes(2, "little")
                + bytes([52, 11, 0, 52]) + (1023).to_bytes(4, "little")), 8
    if dt.kind in "iu":
        signed = 0x08 if dt.kind == "i" else 0x00
        n = dt.itemsize
        return (bytes([0x10, signed, 0x00, 0x00]) + n.to_bytes(4, "little")
                + (0).to_bytes(2, "little") + (8 * n).to_bytes(2, "little")), n
    raise H5Error(f"cannot write element type {dt}")


def _space_msg(shape: tuple[int, ...]) -> bytes:
    b = bytes([1, len(shape), 0, 0]) + bytes(4)
    for s in shape:
        b += int(s).to_bytes(8, "little")
    return b


def _value_bytes(a) -> bytes:
    if isinstance(a, str):
        return a.encode("ascii") + b"\x00"
    arr = np.asarray(a)
    if arr.dtype == np.float64 or arr.dtype.kind in "iu":
        return np.ascontiguousarray(arr, dtype=arr.dtype.newbyteorder("<")).tobytes()
    raise H5Error(f"cannot write element type {arr.dtype}")


def _attr_msg(name: str, value) -> bytes:
    if isinstance(value, (bool, np.bool_)):
        value = np.int64(int(value))
    elif isinstance(value, int) and not isinstance(value, np.generic):
        value = np.int64(value)
    elif isinstance(value, float):
        value = np.float64(value)
    t, _ = _dtype_msg(value)
    shape = () if isinstance(value, str) else np.shape(value)
    s = _space_msg(shape)
    nm = name.encode("ascii") + b"\x00"
    return (bytes([1, 0]) + len(nm).to_bytes(2, "little") + len(t).to_bytes(2, "little")
            + len(s).to_bytes(2, "little") + _pad8(nm) + _pad8(t) + _pad8(s)
            + _value_bytes(value))


class _Node:
    def __init__(self):
        self.attrs: dict = {}


class WGroup(_Node):
    def __init__(self):
        super().__init__()
        self.children: dict[str, _Node] = {}

    def group(self, name: str) -> "WGroup":
        node = self
        for part in [x for x in name.split("/") if x]:
            if part not in node.children:
                node.children[part] = WGroup()
            node = node.children[part]
            if not isinstance(node, WGroup):
                raise H5Error(f"{name} is a dataset")
        return node

    def dataset(self, name: str, data, attrs: dict | None = None) -> None:
        *parents, leaf = [x for x in name.split("/") if x]
        g = self.group("/".join(parents)) if parents else self
        arr = np.asarray(data)
        if arr.dtype not in (np.float64,) and arr.dtype.kind not in "iu":
            raise H5Error(f"cannot write element type {arr.dtype}")
        d = _WData(np.array(arr, order="C"))  # keeps 0-d arrays scalar
        d.attrs.update(attrs or {})
        g.children[leaf] = d


class _WData(_Node):
    def __init__(self, arr: np.ndarray):
        super().__init__()
        self.arr = arr


class Writer(WGroup):
    """An HDF5 file built in memory and written at once: ``w.attrs[...]``,
    ``w.dataset("a/b", array, attrs)``, ``w.group("g")``, ``w.write(path)``."""

    def write(self, path: str | Path) -> None:
        buf = bytearray(96)  # superblock + root symbol table entry, patched last

        def alloc(b: bytes) -> int:
            a = len(buf)
            buf.extend(b)
            buf.extend(bytes((-len(buf)) % 8))
            return a

        def header(msgs: list[tuple[int, bytes, int]]) -> int:
            body = b""
            for mtype, data, flags in msgs:
                data = _pad8(data)
                body += (mtype.to_bytes(2, "little") + len(data).to_bytes(2, "little")
                         + bytes([flags, 0, 0, 0]) + data)
            hdr = (bytes([1, 0]) + len(msgs).to_bytes(2, "little") + (1).to_bytes(4, "little")
                   + len(body).to_bytes(4, "little") + bytes(4))
            return alloc(hdr + body)

        def emit(node: _Node) -> tuple[int, int, int]:
            """Object header address and, for groups, (B-tree, heap) addresses."""
            attrs = [(0xC, _attr_msg(k, v), 0) for k, v in node.attrs.items()]
            if isinstance(node, _WData):
                raw = _value_bytes(node.arr)
                daddr = alloc(raw) if raw else _UNDEF
                t, _ = _dtype_msg(node.arr)
                layout = (bytes([3, 1]) + daddr.to_bytes(8, "little")
                          + len(raw).to_bytes(8, "little"))
                fill = bytes([2, 1, 2, 1, 0, 0, 0, 0])
                return header([(0x1, _space_msg(node.arr.shape), 0), (0x3, t, 1),
                               (0x5, fill, 1), (0x8, layout, 0)] + attrs), 0, 0
            names = sorted(node.children)
            addrs = {n: emit(node.children[n]) for n in names}
            # local heap: "" at 0, the names, then one free block
            heap, offs = bytearray(8), {}
            for n in names:
                offs[n] = len(heap)
                heap += _pad8(n.encode("ascii") + b"\x00")
            free = len(heap)
            heap += (1).to_bytes(8, "little") + (16).to_bytes(8, "little")
            data_addr = alloc(bytes(heap))
            heap_addr = alloc(b"HEAP" + bytes([0, 0, 0, 0]) + len(heap).to_bytes(8, "little")
                              + free.to_bytes(8, "little") + data_addr.to_bytes(8, "little"))
            # symbol table nodes of at most 2 * leaf K entries
            cap = 2 * _LEAF_K
            chunks = [names[i:i + cap] for i in range(0, len(names), cap)] or [[]]
            if len(chunks) > 2 * _INTERNAL_K:
                raise H5Error("too many links in one group for a single B-tree node")
            snods = []
            for ch in chunks:
                b = b"SNOD" + bytes([1, 0]) + len(ch).to_bytes(2, "little")
                for n in ch:
                    oh, bt, hp = addrs[n]
                    cache = 1 if isinstance(node.children[n], WGroup) else 0
                    b += (offs[n].to_bytes(8, "little") + oh.to_bytes(8, "little")
                          + cache.to_bytes(4, "little") + bytes(4)
                          + (bt.to_bytes(8, "little") + hp.to_bytes(8, "little")
                             if cache else bytes(16)))
                b += bytes(8 + 40 * cap - len(b))
                snods.append(alloc(b))
            keys = [0] + [offs[ch[-1]] if ch else 0 for ch in chunks]
            b = (b"TREE" + bytes([0, 0]) + len(snods).to_bytes(2, "little")
                 + _UNDEF.to_bytes(8, "little") + _UNDEF.to_bytes(8, "little"))
            for i, s in enumerate(snods):
                b += keys[i].to_bytes(8, "little") + s.to_bytes(8, "little")
            b += keys[-1].to_bytes(8, "little")
            b += bytes(24 + 8 * (2 * _INTERNAL_K + 1) + 8 * 2 * _INTERNAL_K - len(b))
            btree = alloc(b)
            sym = btree.to_bytes(8, "little") + heap_addr.to_bytes(8, "little")
            return header([(0x11, sym, 0)] + attrs), btree, heap_addr

        root_oh, root_bt, root_hp = emit(self)
        sb = (_SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + _LEAF_K.to_bytes(2, "little")
              + _INTERNAL_K.to_bytes(2, "little") + bytes(4)
              + (0).to_bytes(8, "little") + _UNDEF.to_bytes(8, "little")
              + len(buf).to_bytes(8, "little") + _UNDEF.to_bytes(8, "little")
              + (0).to_bytes(8, "little") + root_oh.to_bytes(8, "little")
              + (1).to_bytes(4, "little") + bytes(4)
              + root_bt.to_bytes(8, "little") + root_hp.to_bytes(8, "little"))
        buf[:96] = sb
        tmp = Path(str(path) + ".tmp")
        tmp.write_bytes(bytes(buf))
        tmp.replace(path)
