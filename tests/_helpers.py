"""Shared fixture loaders for the tests (LiH reference fixture, crystals)."""
import os
from functools import lru_cache

import numpy as np

from mbsymmetry_gb300.layout import BlockLayout
from mbsymmetry_gb300.transformer import build_transforms

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _split(flat, ptr):
    return [flat[ptr[i]:ptr[i + 1]] for i in range(len(ptr) - 1)]


@lru_cache(maxsize=1)
def lih():
    """LiH nk=2x2x2 (the reference's fixture): layout, V, F, S, IR transforms, golden."""
    z = np.load(os.path.join(GOLDEN, "lih_inputs.npz"))
    nk = int(z["nk"])
    ao = _split(z["ao_sizes"], z["ao_ptr"])
    aux = _split(z["aux_sizes"], z["aux_ptr"])
    aob = _split(z["ao_block_offsets"], z["ao_ptr"])
    auxb = _split(z["aux_block_offsets"], z["aux_ptr"])
    ti = [t.reshape(-1, 3) for t in _split(z["tensor_irreps"], z["tensor_ptr"])]
    lay = BlockLayout(nk=nk, kmesh=z["kmesh"], ao_sizes=ao, aux_sizes=aux, tensor_irreps=ti,
                      irre_list=np.arange(nk), index=np.arange(nk), irre_index=np.arange(nk),
                      conj_index=np.arange(nk), ao_block_offsets=aob, aux_block_offsets=auxb)
    ir = {k[3:].replace("_", "/", 1): z[k] for k in z.files if k.startswith("ir_")}
    tr = build_transforms(ir, float(z["beta"]))
    g = dict(np.load(os.path.join(GOLDEN, "lih_golden.npz")))
    return dict(layout=lay, V=z["V"], F=z["F"], S=z["S"], ns=int(z["ns"]), mu=float(z["mu"]),
                tr=tr, ir=ir, golden=g)


def p_slices(layout, nts, P, t_list):
    """Rows t of a [ink][nts][qslice] buffer, concatenated over q (flat_aux each)."""
    out = []
    for t in t_list:
        row = np.concatenate([
            P[nts * layout.qaux_slice_offsets_irre[iq] + t * layout.qaux_slice_sizes_irre[iq]:
              nts * layout.qaux_slice_offsets_irre[iq] + (t + 1) * layout.qaux_slice_sizes_irre[iq]]
            for iq in range(layout.ink)])
        out.append(row)
    return np.concatenate(out)


@lru_cache(maxsize=8)
def crystal(name, rotate=True, ns=None, physical=False):
    from mbsymmetry_gb300.crystal import CONFIGS, load_ir, make_crystal
    import dataclasses
    spec = CONFIGS[name]
    if ns is not None:
        spec = dataclasses.replace(spec, ns=ns)
    cr = make_crystal(spec, rotate=rotate, physical=physical)
    tr = build_transforms(load_ir(spec.nts), spec.beta)
    return cr, tr
