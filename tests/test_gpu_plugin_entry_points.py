"""The device entry points the NCrystal plugin calls (ncgb_plugin.cc): a
material created from an explicit bundle file, and one scatter on the random
stream of a caller's 64-bit key (the plugin draws the key from NCrystal's
RNG).  Checked against the oracle on the same streams.  A cfg-string with no
bundle on a host without an exporter fails loudly."""
import numpy as np
import pytest

import ncrystal_gb300 as NC
import ncrystal_gb300.workloads as W
from conftest import bundle_path
from oracle.pyoracle import HostMaterial

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg", [W.PE293, W.AL2O3, W.WATER])
def test_bundle_material_and_keyed_scatters_match_oracle(cfg):
    path = bundle_path(cfg)
    by_path = NC.createScatterFromBundle(path)
    by_cfg = NC.createScatter(cfg)
    e = W.loguniform_energies(5000, 1e-5, 3.0, 91)
    np.testing.assert_array_equal(by_path.crossSectionIsotropic(e), by_cfg.crossSectionIsotropic(e))
    m = HostMaterial(path)
    r = np.random.default_rng(92)
    keys = r.integers(0, 2 ** 63, 150, dtype=np.uint64)
    for k, e0 in zip(keys, W.loguniform_energies(150, 1e-4, 1.0, 93)):
        ef, mu = by_path.sample_keyed(e0, int(k))
        oef, omu, ost, _ = m.scatter(np.array([e0]), int(k))
        assert ost[0] == 0
        assert ef == pytest.approx(oef[0], rel=1e-9, abs=0) and mu == pytest.approx(omu[0], abs=1e-9)


def test_missing_bundle_without_exporter_fails_loudly(tmp_path, monkeypatch):
    monkeypatch.setenv("NCGB_BUNDLE_CACHE", str(tmp_path))
    monkeypatch.setenv("NCGB_EXPORT_LIB", str(tmp_path / "no_such_exporter.so"))
    with pytest.raises(NC.NCFileNotFound):
        NC.createScatter("Polyethylene_CH2.ncmat;temp=303K")
