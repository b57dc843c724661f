"""HDF5 writer: files it writes read back exactly through the HDF5 reader, and
a crystal exported as the reference's ``block`` directory loads through the
reference-input loader unchanged (on-disk format compatibility)."""
import os

import numpy as np
import pytest

from _helpers import GOLDEN, crystal, lih
from mbsymmetry_gb300 import h5write
from mbsymmetry_gb300.h5lite import H5File
from mbsymmetry_gb300.inputs import load_reference_inputs


def test_write_read_roundtrip(tmp_path):
    rng = np.random.default_rng(7)
    tree = {"a": np.arange(5, dtype=np.int32), "b": rng.standard_normal((3, 4, 2)),
            "s": np.array(12, dtype=np.int64), "x": np.array(2.5), "e": np.zeros(0),
            "g": {f"{i}": np.full(i % 5 + 1, i, dtype=np.int64) for i in range(300)},   # 3 symbol-table nodes
            "h": {"deep": {"z": rng.standard_normal(7)}}}
    p = str(tmp_path / "t.h5")
    h5write.write(p, tree)
    f = H5File(p)
    assert sorted(f.keys("/")) == sorted(tree)
    assert np.array_equal(f["a"], tree["a"]) and f["a"].dtype == np.int32
    assert np.array_equal(f["b"], tree["b"]) and f["b"].dtype == np.float64
    assert int(f["s"]) == 12 and float(f["x"]) == 2.5 and f["e"].size == 0
    assert len(f.keys("/g")) == 300
    for i in (0, 127, 128, 255, 299):
        assert np.array_equal(f[f"g/{i}"], tree["g"][f"{i}"])
    assert np.array_equal(f["h/deep/z"], tree["h"]["deep"]["z"])


def test_export_reference_block_dir_lih(tmp_path):
    d = lih()
    z = np.load(os.path.join(GOLDEN, "lih_inputs.npz"))
    out = str(tmp_path / "block")
    h5write.export_reference_inputs(out, d["layout"], d["V"], z["F"], z["S"], z["H"], d["ns"])
    ri = load_reference_inputs(out)
    L0, L1 = d["layout"], ri.layout
    assert ri.ns == d["ns"]
    for k in range(L0.nk):
        assert np.array_equal(L0.ao_sizes[k], L1.ao_sizes[k]) and np.array_equal(L0.aux_sizes[k], L1.aux_sizes[k])
    for p in range(L0.nk * L0.nk):
        assert np.array_equal(L0.tensor_irreps[p], L1.tensor_irreps[p])
    assert np.array_equal(ri.V, d["V"])
    assert np.allclose(ri.onebody.F, d["F"], rtol=0, atol=1e-14)
    assert np.allclose(ri.onebody.S, d["S"], rtol=0, atol=1e-14)


@pytest.mark.parametrize("kind", ["labelled", "orbital", "orbital-wurtzite"])
def test_export_reference_block_dir_crystal(tmp_path, kind):
    if kind == "labelled":
        cr, _ = crystal("C1", rotate=False)
    else:   # Slater-Koster / Gaussian-orbital data with the group's selection rule
        import dataclasses
        from mbsymmetry_gb300.crystal import CONFIGS
        from mbsymmetry_gb300.orbitals import make_orbital_crystal
        spec = CONFIGS["C1"] if kind == "orbital" else dataclasses.replace(
            CONFIGS["C4"], name="wurtzite", mesh=(2, 2, 3), nao=16, naux=40, nts=62, beta=50.0)
        cr = make_orbital_crystal(spec, rotate=False)
    out = str(tmp_path / "block")
    h5write.export_reference_inputs(out, cr.layout, cr.V, cr.F, cr.S, cr.H, cr.ns)
    ri = load_reference_inputs(out)
    assert np.array_equal(ri.V, cr.V)
    assert ri.layout.flat_V_size == cr.layout.flat_V_size
    assert np.array_equal(ri.layout.kpair_slice_offsets, cr.layout.kpair_slice_offsets)
    assert np.allclose(ri.onebody.F, cr.F.reshape(ri.onebody.F.shape), rtol=0, atol=1e-14)
