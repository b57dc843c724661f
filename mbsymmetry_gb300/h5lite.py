"""Minimal read-only HDF5 reader for the reference's input files.

The reference reads its inputs through ALPSCore/HDF5-HL
(``SymmetryMBPT/src/common/symmetry_utils.cpp:113-159``,
``SymmetryMBPT/include/common/df_integral_block_t.h:21-59``,
``SymmetryMBPT/src/scmbpt/sc_loop_block_t.cpp:64-76``,
``SymmetryMBPT/src/common/transformer_t.cpp:17-33``).  Neither libhdf5 nor
h5py exist on the target machines, so this module parses the subset of the
HDF5 file format those files use:

* superblock version 0/1 (8-byte offsets and lengths),
* version-1 object headers with continuation blocks,
* old-style groups (symbol-table message -> v1 B-tree -> SNOD nodes,
  link names in a local heap),
* contiguous, compact and (unfiltered) chunked data layouts,
* fixed-point and IEEE floating point element types.

Complex arrays follow the ALPSCore convention (a trailing dimension of 2 for
real/imag, ``scripts/common/blk_utils.py:56-61``); :func:`as_complex` folds it.
"""
from __future__ import annotations

import struct
from typing import Dict, List, Optional, Tuple

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5Error(RuntimeError):
    pass


class _Obj:
    """Parsed object header: its messages keyed by type id."""

    def __init__(self):
        self.msgs: List[Tuple[int, bytes]] = []

    def get(self, mtype: int) -> Optional[bytes]:
        for t, d in self.msgs:
            if t == mtype:
                return d
        return None


class H5File:
    """Read-only view of one HDF5 file; ``f["a/b"]`` returns a numpy array."""

    def __init__(self, path: str):
        with open(path, "rb") as fh:
            self.buf = fh.read()
        self.path = path
        base = self.buf.find(_SIG)
        if base != 0:
            raise H5Error(f"{path}: HDF5 signature not at offset 0")
        ver = self.buf[8]
        if ver not in (0, 1):
            raise H5Error(f"{path}: superblock version {ver} not supported")
        so, sl = self.buf[13], self.buf[14]
        if so != 8 or sl != 8:
            raise H5Error(f"{path}: offset/length size {so}/{sl} not supported")
        p = 24 if ver == 0 else 28
        # base, free-space, eof, driver addresses
        p += 32
        # root group symbol table entry: link name offset, object header address
        _, root_oh = struct.unpack_from("<QQ", self.buf, p)
        self.root = root_oh
        self._cache: Dict[int, _Obj] = {}

    # ------------------------------------------------------------------ #
    def _u(self, fmt: str, off: int):
        return struct.unpack_from(fmt, self.buf, off)

    def _object(self, addr: int) -> _Obj:
        if addr in self._cache:
            return self._cache[addr]
        ver = self.buf[addr]
        if ver != 1:
            raise H5Error(f"object header version {ver} at {addr:#x} not supported")
        nmsg, = self._u("<H", addr + 2)
        hsize, = self._u("<I", addr + 8)
        obj = _Obj()
        blocks = [(addr + 16, hsize)]
        count = 0
        while blocks and count < nmsg:
            start, size = blocks.pop(0)
            p = start
            end = start + size
            while p + 8 <= end and count < nmsg:
                mtype, msize, _flags = self._u("<HHB", p)
                data = self.buf[p + 8:p + 8 + msize]
                p += 8 + msize
                count += 1
                if mtype == 0x10:  # continuation
                    caddr, clen = struct.unpack_from("<QQ", data, 0)
                    blocks.append((caddr, clen))
                else:
                    obj.msgs.append((mtype, data))
        self._cache[addr] = obj
        return obj

    def _heap_name(self, heap_addr: int, off: int) -> str:
        if self.buf[heap_addr:heap_addr + 4] != b"HEAP":
            raise H5Error("bad local heap signature")
        data_addr, = self._u("<Q", heap_addr + 24)
        s = data_addr + off
        e = self.buf.index(b"\x00", s)
        return self.buf[s:e].decode()

    def _group_entries(self, addr: int) -> Dict[str, int]:
        obj = self._object(addr)
        st = obj.get(0x11)
        if st is None:
            link_msgs = [d for t, d in obj.msgs if t == 0x06]
            if link_msgs:
                raise H5Error("new-style (link message) groups are not supported")
            raise H5Error(f"object at {addr:#x} is not a group")
        btree, heap = struct.unpack_from("<QQ", st, 0)
        out: Dict[str, int] = {}
        self._walk_btree(btree, heap, out)
        return out

    def _walk_btree(self, node: int, heap: int, out: Dict[str, int]):
        if self.buf[node:node + 4] != b"TREE":
            raise H5Error("bad v1 B-tree signature")
        ntype, level, nent = self._u("<BBH", node + 4)
        if ntype != 0:
            raise H5Error("expected group B-tree")
        p = node + 24  # after left/right sibling addresses
        p += 8  # key 0
        for _ in range(nent):
            child, = self._u("<Q", p)
            p += 8 + 8  # child + next key
            if level > 0:
                self._walk_btree(child, heap, out)
            else:
                self._read_snod(child, heap, out)

    def _read_snod(self, addr: int, heap: int, out: Dict[str, int]):
        if self.buf[addr:addr + 4] != b"SNOD":
            raise H5Error("bad symbol table node signature")
        nsym, = self._u("<H", addr + 6)
        p = addr + 8
        for _ in range(nsym):
            name_off, oh = self._u("<QQ", p)
            out[self._heap_name(heap, name_off)] = oh
            p += 40

    def _resolve(self, path: str) -> int:
        addr = self.root
        for part in [x for x in path.strip("/").split("/") if x]:
            ents = self._group_entries(addr)
            if part not in ents:
                raise KeyError(f"{self.path}: '{path}' not found (missing '{part}')")
            addr = ents[part]
        return addr

    # ------------------------------------------------------------------ #
    def keys(self, path: str = "/") -> List[str]:
        return sorted(self._group_entries(self._resolve(path)).keys())

    def is_group(self, path: str) -> bool:
        return self._object(self._resolve(path)).get(0x11) is not None

    def __contains__(self, path: str) -> bool:
        try:
            self._resolve(path)
            return True
        except KeyError:
            return False

    def __getitem__(self, path: str) -> np.ndarray:
        return self._read_dataset(self._resolve(path), path)

    def _dtype(self, d: bytes) -> np.dtype:
        return self._dtype_at(d, 0)[0]

    def _dtype_at(self, d: bytes, p0: int) -> Tuple[np.dtype, int]:
        """Decode a datatype message starting at ``p0``; returns (dtype, end)."""
        cls_ver = d[p0]
        cls = cls_ver & 0x0F
        ver = cls_ver >> 4
        flags = d[p0 + 1] | (d[p0 + 2] << 8) | (d[p0 + 3] << 16)
        size, = struct.unpack_from("<I", d, p0 + 4)
        order = ">" if (flags & 1) else "<"
        p = p0 + 8
        if cls == 0:
            signed = bool(flags & 0x08)
            return np.dtype(f"{order}{'i' if signed else 'u'}{size}"), p + 4
        if cls == 1:
            return np.dtype(f"{order}f{size}"), p + 12
        if cls == 3:
            return np.dtype(f"S{size}"), p
        if cls == 6:  # compound (h5py writes complex as {r, i})
            nmemb = flags & 0xFFFF
            names, formats, offsets = [], [], []
            for _ in range(nmemb):
                e = d.index(b"\x00", p)
                name = d[p:e].decode()
                if ver < 3:
                    p = p + ((e - p) // 8 + 1) * 8
                else:
                    p = e + 1
                if ver < 3:
                    off, = struct.unpack_from("<I", d, p)
                    p += 4
                else:
                    nb = max(1, (size.bit_length() + 7) // 8)
                    off = int.from_bytes(d[p:p + nb], "little")
                    p += nb
                if ver == 1:
                    p += 1 + 3 + 4 + 4 + 16  # dimensionality, reserved, perm, reserved, dims
                mdt, p = self._dtype_at(d, p)
                names.append(name)
                formats.append(mdt)
                offsets.append(off)
            return np.dtype({"names": names, "formats": formats, "offsets": offsets,
                             "itemsize": size}), p
        raise H5Error(f"datatype class {cls} not supported")

    def _shape(self, d: bytes) -> Tuple[int, ...]:
        ver = d[0]
        ndim = d[1]
        if ver == 1:
            p = 8
        elif ver == 2:
            if d[3] == 2:  # null dataspace
                return (0,)
            p = 4
        else:
            raise H5Error(f"dataspace version {ver}")
        dims = struct.unpack_from(f"<{ndim}Q", d, p)
        return tuple(int(x) for x in dims)

    def _read_dataset(self, addr: int, path: str) -> np.ndarray:
        obj = self._object(addr)
        ds, dt, ly = obj.get(0x01), obj.get(0x03), obj.get(0x08)
        if ds is None or dt is None or ly is None:
            raise H5Error(f"{path} is not a dataset")
        if obj.get(0x0B) is not None:
            raise H5Error(f"{path}: filtered (compressed) datasets are not supported")
        shape = self._shape(ds)
        dtype = self._dtype(dt)
        n = int(np.prod(shape)) if shape else 1
        nbytes = n * dtype.itemsize
        ver = ly[0]
        if ver != 3:
            raise H5Error(f"{path}: layout message version {ver} not supported")
        cls = ly[1]
        if cls == 0:  # compact
            size, = struct.unpack_from("<H", ly, 2)
            raw = ly[4:4 + size]
        elif cls == 1:  # contiguous
            daddr, size = struct.unpack_from("<QQ", ly, 2)
            if daddr == UNDEF:
                raw = bytes(nbytes)
            else:
                raw = self.buf[daddr:daddr + nbytes]
        elif cls == 2:  # chunked, no filters
            raw = self._read_chunked(ly, shape, dtype)
        else:
            raise H5Error(f"{path}: layout class {cls}")
        arr = np.frombuffer(raw[:nbytes], dtype=dtype).copy()
        return arr.reshape(shape) if shape else arr.reshape(())

    def _read_chunked(self, ly: bytes, shape, dtype) -> bytes:
        ndim_p1 = ly[2]
        btree, = struct.unpack_from("<Q", ly, 3)
        cdims = struct.unpack_from(f"<{ndim_p1}I", ly, 11)
        cshape = tuple(int(x) for x in cdims[:-1])
        out = np.zeros(shape, dtype=dtype)
        self._walk_chunks(btree, ndim_p1, cshape, out)
        return out.tobytes()

    def _walk_chunks(self, node, ndim_p1, cshape, out):
        if self.buf[node:node + 4] != b"TREE":
            raise H5Error("bad chunk B-tree signature")
        ntype, level, nent = self._u("<BBH", node + 4)
        p = node + 24
        keysz = 8 + 8 * ndim_p1
        for _ in range(nent):
            csize, = self._u("<I", p)
            offs = self._u(f"<{ndim_p1}Q", p + 8)
            child, = self._u("<Q", p + keysz)
            p += keysz + 8
            if level > 0:
                self._walk_chunks(child, ndim_p1, cshape, out)
                continue
            raw = np.frombuffer(self.buf[child:child + int(np.prod(cshape)) * out.dtype.itemsize],
                                dtype=out.dtype).reshape(cshape)
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs[:-1], cshape, out.shape))
            sub = tuple(slice(0, s.stop - s.start) for s in sl)
            out[sl] = raw[sub]


def as_complex(a: np.ndarray) -> np.ndarray:
    """Return complex128 data from either complex convention.

    h5py writes complex numbers as a compound ``{r, i}``; ALPSCore writes a
    trailing dimension of 2 (``scripts/common/blk_utils.py:56-61``).
    """
    if a.dtype.names is not None and len(a.dtype.names) == 2:
        re, im = a.dtype.names
        return np.ascontiguousarray(a[re].astype(np.float64) + 1j * a[im].astype(np.float64))
    if a.shape and a.shape[-1] == 2 and a.dtype.kind == "f":
        return np.ascontiguousarray(a[..., 0] + 1j * a[..., 1])
    return a.astype(np.complex128)
