"""Any cfg-string loads (ncrystal_create_scatter accepts every cfg-string
NCrystal does, ncrystal.cc:1510-1516): a cfg-string without a material bundle
gets one exported on demand through NCrystal's own material loading
(libncgb_export.so, run in-process), and the exported material is the
reference's to the bit.  Without an exporter a missing bundle stays a loud
FileNotFound.  CPU only; needs the NCrystal sources (reference build)."""
import os

import numpy as np
import pytest

import ncrystal_gb300 as NC
import ncrystal_gb300._build as B
import ncrystal_gb300.workloads as W
from oracle import pyoracle

pytestmark = pytest.mark.skipif(not os.path.exists(B.exporter_path()) or pyoracle.refpin_lib() is None,
                                reason="needs the NCrystal sources (exporter and reference build)")

CFG = "Polyethylene_CH2.ncmat;temp=301K"


def test_any_cfg_exported_on_demand_equals_reference(tmp_path, monkeypatch):
    monkeypatch.setenv("NCGB_BUNDLE_CACHE", str(tmp_path))
    if os.path.exists(os.path.join(B.BUNDLES, B.bundle_file_name(CFG))):
        pytest.skip("a bundle for %s was exported ahead of time" % CFG)
    p = NC.bundle_path(CFG)
    assert p == os.path.join(str(tmp_path), B.bundle_file_name(CFG))
    m = pyoracle.HostMaterial(p)
    e = np.concatenate([W.loguniform_energies(20000, 1e-6, 3.0, 31), W.al_wavelength_energies(2000, 32)])
    seed = 24680
    r = pyoracle.reference_run(CFG, e, seed, callseq=2, stream=5)
    np.testing.assert_array_equal(m.xs(e), r["xs"])
    ef, mu, st, nd = m.scatter(e, seed, callseq=2, stream=5)
    assert np.all(st == 0) and np.all(r["status"] == 0)
    np.testing.assert_array_equal(nd, r["ndraws"])
    np.testing.assert_array_equal(ef, r["ekin_final"])
    np.testing.assert_array_equal(mu, r["mu"])
    # found again without a second export
    t = os.path.getmtime(p)
    assert NC.bundle_path(CFG) == p and os.path.getmtime(p) == t


def test_missing_bundle_without_exporter_is_file_not_found(tmp_path, monkeypatch):
    monkeypatch.setenv("NCGB_BUNDLE_CACHE", str(tmp_path))
    monkeypatch.setenv("NCGB_EXPORT_LIB", str(tmp_path / "no_such_exporter.so"))
    with pytest.raises(NC.NCFileNotFound, match="no bundle exporter"):
        NC.bundle_path("Polyethylene_CH2.ncmat;temp=302K")
    assert not os.listdir(str(tmp_path))


def test_cfg_rejected_by_ncrystal_gives_its_error(tmp_path, monkeypatch):
    monkeypatch.setenv("NCGB_BUNDLE_CACHE", str(tmp_path))
    with pytest.raises(NC.NCFileNotFound, match="NoSuchMaterial"):
        NC.bundle_path("NoSuchMaterial.ncmat;temp=300K")
    with pytest.raises(NC.NCBadInput):
        NC.bundle_path("Al_sg225.ncmat;temp=-5K")
    assert not [f for f in os.listdir(str(tmp_path)) if f.endswith(".ncgb")]
