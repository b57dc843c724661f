"""Autotuner host logic: the fingerprint sees what the tile rules see, and a
cached result is returned without building any handle."""
import json

import pytest

from _helpers import crystal


def test_fingerprint_and_cache(tmp_path, monkeypatch):
    from mbsymmetry_gb300 import autotune
    cr, tr = crystal("C1")
    f1 = autotune.fingerprint(cr.layout, tr.nts, "tf32x3")
    assert f1 == autotune.fingerprint(cr.layout, tr.nts, "tf32x3")
    assert f1 != autotune.fingerprint(cr.layout, tr.nts + 2, "tf32x3")
    assert f1 != autotune.fingerprint(cr.layout, tr.nts, "bf16x3")
    cr2, _ = crystal("C1", rotate=False)
    assert f1 != autotune.fingerprint(cr2.layout, tr.nts, "tf32x3")
    stored = {"fingerprint": f1, "precision": "tf32x3", "best": {"uvt_smem_kb": 72, "sw_npk_max": 64, "uv_waves": 4},
              "trials": []}
    path = tmp_path / "tune.json"
    path.write_text(json.dumps({f1: stored}))

    def no_solver(*a, **k):
        raise AssertionError("a cached result must not build a handle")
    monkeypatch.setattr(autotune, "GWSolver", no_solver)
    out = autotune.autotune(cr.layout, cr.ns, tr, cr.V, cr.F, cr.S, cr.mu, cache=str(path))
    assert out["best"]["uvt_smem_kb"] == 72
