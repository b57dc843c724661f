"""Minimal HDF5 writer: the reference's input files for our synthetic crystals.

The reference reads its inputs through ALPSCore/HDF5-HL
(``SymmetryMBPT/src/common/symmetry_utils.cpp:113-159``,
``SymmetryMBPT/include/common/df_integral_block_t.h:21-59``,
``SymmetryMBPT/src/scmbpt/sc_loop_block_t.cpp:64-76``).  No HDF5 library
exists here, so this module writes the file-format subset the reference's
files use (the same subset :mod:`h5lite` reads):

* superblock version 0, 8-byte offsets and lengths;
* version-1 object headers;
* old-style groups: symbol-table message -> one v1 B-tree node (group
  leaf and internal K = 64, so a group holds up to 64 x 128 links in a
  single-level tree) -> symbol-table nodes, names in a local heap;
* contiguous datasets of little-endian int32, int64 and IEEE float64, with
  version-1 dataspaces (rank 0 = scalar), a fill-value message and a
  version-3 layout message.

Complex arrays follow the ALPSCore convention (trailing dimension 2).
:func:`export_reference_inputs` writes a crystal as the reference's
``block`` directory (``symmetry_info.h5``, ``df_int/meta.h5``,
``df_int/VQ_flat_0.h5``, ``input_flat.h5``), for layouts without rotations
(ink = nk; the rotation file ``symmetry_rot.h5`` is not in the reference
tree, so its format is not known here).
"""
from __future__ import annotations

import os
import struct
from typing import Dict, Union

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
K_LEAF = 64       # symbol-table node holds 2 K_LEAF links
K_INTERNAL = 64   # B-tree node holds 2 K_INTERNAL children
_SNOD_CAP = 2 * K_LEAF
_BTREE_CAP = 2 * K_INTERNAL

Tree = Dict[str, Union["Tree", np.ndarray]]


def _pad8(n: int) -> int:
    return (n + 7) & ~7


class _Buf:
    def __init__(self):
        self.b = bytearray()

    def alloc(self, size: int) -> int:
        off = _pad8(len(self.b))
        self.b.extend(b"\0" * (off - len(self.b) + size))
        return off

    def put(self, off: int, fmt: str, *vals):
        struct.pack_into("<" + fmt, self.b, off, *vals)


def _datatype(dt: np.dtype) -> bytes:
    if dt == np.float64:
        # class 1 version 1; LE, mantissa normalisation "implied", sign bit 63
        head = struct.pack("<BBBBI", 0x11, 0x20, 63, 0, 8)
        props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
        return head + props
    if dt in (np.int64, np.int32):
        size = dt.itemsize
        head = struct.pack("<BBBBI", 0x10, 0x08, 0, 0, size)   # class 0 version 1, LE, signed
        return head + struct.pack("<HH", 0, 8 * size)
    raise TypeError(f"unsupported dtype {dt}")


def _message(mtype: int, data: bytes, flags: int = 0) -> bytes:
    data = data + b"\0" * (_pad8(len(data)) - len(data))
    return struct.pack("<HHB3x", mtype, len(data), flags) + data


def _object_header(buf: _Buf, msgs) -> int:
    body = b"".join(msgs)
    off = buf.alloc(16 + len(body))
    buf.put(off, "BBHII", 1, 0, len(msgs), 1, len(body))
    buf.b[off + 16:off + 16 + len(body)] = body
    return off


def _write_dataset(buf: _Buf, a: np.ndarray) -> int:
    a = np.asarray(a, order="C")  # keeps 0-d arrays 0-d (scalar dataspace)
    if a.dtype not in (np.float64, np.int64, np.int32):
        a = a.astype(np.int64 if np.issubdtype(a.dtype, np.integer) else np.float64)
    raw = a.astype(a.dtype.newbyteorder("<"), copy=False).tobytes()
    daddr = UNDEF
    if raw:
        daddr = buf.alloc(len(raw))
        buf.b[daddr:daddr + len(raw)] = raw
    space = struct.pack("<BBBB4x", 1, a.ndim, 0, 0) + b"".join(struct.pack("<Q", d) for d in a.shape)
    fill = struct.pack("<BBBB", 2, 1, 2, 0)       # early allocation, fill value undefined
    layout = struct.pack("<BBQQ", 3, 1, daddr, len(raw))
    return _object_header(buf, [_message(0x01, space), _message(0x03, _datatype(a.dtype), 1),
                                _message(0x05, fill), _message(0x08, layout)])


def _write_group(buf: _Buf, tree: Tree):
    """Children first; returns (object header, B-tree, local heap) addresses."""
    names = sorted(tree.keys(), key=lambda s: s.encode())
    children = {}
    for n in names:
        v = tree[n]
        if isinstance(v, dict):
            oh, bt, hp = _write_group(buf, v)
            children[n] = (oh, 1, bt, hp)
        else:
            children[n] = (_write_dataset(buf, v), 0, 0, 0)
    # local heap: "" at offset 0, then the names
    seg = bytearray(b"\0" * 8)
    name_off = {}
    for n in names:
        name_off[n] = len(seg)
        e = n.encode() + b"\0"
        seg += e + b"\0" * (_pad8(len(e)) - len(e))
    seg_addr = buf.alloc(len(seg))
    buf.b[seg_addr:seg_addr + len(seg)] = seg
    heap = buf.alloc(32)
    buf.b[heap:heap + 4] = b"HEAP"
    buf.put(heap + 4, "B3xQQQ", 0, len(seg), UNDEF, seg_addr)
    # symbol-table nodes of at most _SNOD_CAP sorted links
    chunks = [names[i:i + _SNOD_CAP] for i in range(0, len(names), _SNOD_CAP)] or [[]]
    if len(chunks) > _BTREE_CAP:
        raise ValueError(f"group with {len(names)} links exceeds {_BTREE_CAP * _SNOD_CAP}")
    snods = []
    for ch in chunks:
        sn = buf.alloc(8 + _SNOD_CAP * 40)
        buf.b[sn:sn + 4] = b"SNOD"
        buf.put(sn + 4, "BBH", 1, 0, len(ch))
        for i, n in enumerate(ch):
            oh, ctype, bt, hp = children[n]
            e = sn + 8 + 40 * i
            buf.put(e, "QQI4xQQ", name_off[n], oh, ctype, bt, hp)
        snods.append(sn)
    # one leaf B-tree node (type 0: group); key i+1 = the last name of child i
    bt = buf.alloc(24 + (2 * K_INTERNAL + 1) * 8 + 2 * K_INTERNAL * 8)
    buf.b[bt:bt + 4] = b"TREE"
    buf.put(bt + 4, "BBHQQ", 0, 0, len(snods), UNDEF, UNDEF)
    p = bt + 24
    buf.put(p, "Q", 0)
    for ch, sn in zip(chunks, snods):
        buf.put(p + 8, "QQ", sn, name_off[ch[-1]] if ch else 0)
        p += 16
    oh = _object_header(buf, [_message(0x11, struct.pack("<QQ", bt, heap))])
    return oh, bt, heap


def write(path: str, tree: Tree) -> None:
    """Write a nested dict {name: subtree | array} as an HDF5 file."""
    buf = _Buf()
    buf.alloc(96)  # superblock and root symbol-table entry at offset 0
    oh, bt, hp = _write_group(buf, tree)
    eof = len(buf.b)
    buf.b[0:8] = _SIG
    buf.put(8, "BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, K_LEAF, K_INTERNAL, 0)
    buf.put(24, "QQQQ", 0, UNDEF, eof, UNDEF)
    buf.put(56, "QQI4xQQ", 0, oh, 1, bt, hp)
    with open(path, "wb") as f:
        f.write(bytes(buf.b))


def _nest(flat: Dict[str, np.ndarray]) -> Tree:
    root: Tree = {}
    for path, a in flat.items():
        parts = [p for p in path.split("/") if p]
        node = root
        for p in parts[:-1]:
            node = node.setdefault(p, {})
        node[parts[-1]] = a
    return root


def _ri(z: np.ndarray) -> np.ndarray:
    z = np.asarray(z, dtype=np.complex128)
    return np.stack([z.real, z.imag], axis=-1)


def export_reference_inputs(block_dir: str, layout, V, F, S, H, ns: int) -> None:
    """Write a layout without rotations and its V, F, S, H as the reference's
    ``block`` directory: ``symmetry_info.h5`` (block/*, dataset names and
    integer widths as in the reference's LiH fixture), ``df_int/meta.h5``,
    ``df_int/VQ_flat_0.h5`` (one chunk, dataset "0", real/imag interleaved)
    and ``input_flat.h5`` (HF/Fock-k, S-k, H-k as [s][flat_ao][2]; the energies
    and the Madelung constant as 0).  F, S, H are [s][flat_ao] flat blocks."""
    L = layout
    nk = L.nk
    if L.ink != nk:
        raise ValueError("export needs a layout without rotations (ink = nk)")
    i32 = lambda x: np.asarray(x, dtype=np.int32)
    i64 = lambda x: np.asarray(x, dtype=np.int64)
    blk = {}
    for k in range(nk):
        blk[f"block/ao_sizes/{k}"] = i32(L.ao_sizes[k])
        blk[f"block/aux_sizes/{k}"] = i32(L.aux_sizes[k])
        blk[f"block/ao_block_offsets/{k}"] = i32(L.ao_block_offsets[k])
        blk[f"block/aux_block_offsets/{k}"] = i32(L.aux_block_offsets[k])
        blk[f"block/ao_offsets/{k}"] = i64(L.ao_offsets[k])
        blk[f"block/aux_offsets/{k}"] = i64(L.aux_offsets[k])
    for p in range(nk * nk):
        blk[f"block/tensor_irreps/{p}"] = i64(L.tensor_irreps[p]).reshape(-1, 3)
        blk[f"block/tensor_offsets/{p}"] = i64(L.tensor_offsets[p])
    blk["block/kao_nblocks"] = i64([len(a) for a in L.ao_sizes])
    blk["block/qaux_nblocks"] = i64([len(a) for a in L.aux_sizes])
    blk["block/kpair_nblocks"] = i64([len(t) for t in L.tensor_irreps])
    blk["block/kao_slice_offsets"] = i64(L.kao_slice_offsets)
    blk["block/kao_slice_sizes"] = i64(L.kao_slice_sizes)
    blk["block/qaux_slice_offsets"] = i64(L.qaux_slice_offsets)
    blk["block/qaux_slice_sizes"] = i64(L.qaux_slice_sizes)
    blk["block/kpair_slice_offsets"] = i64(L.kpair_slice_offsets)
    blk["block/kpair_slice_sizes"] = i64(L.kpair_slice_sizes)
    os.makedirs(os.path.join(block_dir, "df_int"), exist_ok=True)
    write(os.path.join(block_dir, "symmetry_info.h5"), _nest(blk))
    npair = nk * nk
    pairs = np.array([(p // nk, p % nk) for p in range(npair)], dtype=np.int64)
    Vf = np.asarray(V, dtype=np.complex128).ravel()
    meta = {"chunk_size": np.array(npair, dtype=np.int64), "chunk_indices": i64([0]),
            "total_size": np.array(Vf.size, dtype=np.int64),
            "grid/k_mesh_scaled": np.asarray(L.kmesh, dtype=np.float64),
            "grid/kpair_idx": pairs, "grid/kpair_irre_list": np.arange(npair, dtype=np.int64),
            "grid/conj_pairs_list": np.arange(npair, dtype=np.int64),
            "grid/trans_pairs_list": np.arange(npair, dtype=np.int64),
            "grid/num_kpair_stored": np.array(npair, dtype=np.int64)}
    write(os.path.join(block_dir, "df_int", "meta.h5"), _nest(meta))
    write(os.path.join(block_dir, "df_int", "VQ_flat_0.h5"), {"0": _ri(Vf).ravel()})
    sh = (ns, -1)
    hf = {"HF/Fock-k": _ri(np.reshape(F, sh)), "HF/S-k": _ri(np.reshape(S, sh)), "HF/H-k": _ri(np.reshape(H, sh)),
          "HF/Energy": np.array(0.0), "HF/Energy_nuc": np.array(0.0), "HF/madelung": np.array(0.0)}
    write(os.path.join(block_dir, "input_flat.h5"), _nest(hf))
