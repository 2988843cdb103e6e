"""The library's table builder against the reference's own derived SAB tables
and samplers, and the oracle against the live reference library on the same
random streams.  Needs the NCrystal sources (skipped elsewhere)."""
import os

import numpy as np
import pytest

import ncrystal_gb300._build as B
import ncrystal_gb300.workloads as W
from ncrystal_gb300.bundle.reader import read_bundle
from oracle import pyoracle

pytestmark = pytest.mark.skipif(not B.reference_available() or pyoracle.refpin_lib() is None,
                                reason="needs the NCrystal sources (reference build)")

INFO = np.dtype([("d", "<f8", (8,)), ("u", "<u4", (2,)), ("inv", "<f8", (3,))])
CFGS = [W.AL, W.AL2O3, W.PE293, W.WATER]


@pytest.mark.parametrize("cfg", CFGS)
def test_derived_sab_tables_bit_identical(cfg, tmp_path):
    path = B.export_bundles([cfg], outdir=str(tmp_path), with_derived=True)[cfg]
    b = read_bundle(path)
    m = pyoracle.HostMaterial(path)
    nsab = 0
    for ic in range(int(b["ncomp"][0])):
        p = "c%d." % ic
        if b[p + "type"] != "SABScatter":
            continue
        nsab += 1
        pairs = [("xs", "f8", "ref.xs"), ("logsab", "f8", "ref.logsab"), ("cumul", "f8", "ref.cumul"),
                 ("smp_ibetaoffset", "i4", "ref.smp_ibetaoffset"), ("smp_nbeta", "i4", "ref.smp_nbeta"),
                 ("smp_offset", "i8", "ref.smp_offset"), ("smp_fbkep", "f8", "ref.smp_fbkep"),
                 ("bx", "f8", "ref.smp_beta_x"), ("by", "f8", "ref.smp_beta_y"),
                 ("bcdf", "f8", "ref.smp_beta_cdf")]
        for name, dt, ref in pairs:
            a = m.array(ic, name, dt)
            np.testing.assert_array_equal(a.astype(b[p + ref].dtype), b[p + ref], err_msg=name)
        info = m.array(ic, "info", INFO)
        nb = m.array(ic, "smp_nbeta", "i4")
        off = m.array(ic, "smp_offset", "i8")
        keep = np.concatenate([np.arange(o, o + n - 1) for o, n in zip(off, nb) if n > 0])
        np.testing.assert_array_equal(info["d"][keep].ravel(), b[p + "ref.smp_info_d"])
        np.testing.assert_array_equal(info["u"][keep].ravel(), b[p + "ref.smp_info_u"])
        assert m.scalar(ic, "kext") == b[p + "ref.kExtension"][0]
        assert m.scalar(ic, "k1") == b[p + "ref.k1"][0]
        assert m.scalar(ic, "k2") == b[p + "ref.k2"][0]
    assert nsab >= 1


@pytest.mark.parametrize("cfg", [W.AL, W.AL2O3, W.PE293, "Polyethylene_CH2.ncmat;temp=280K"])
def test_oracle_equals_live_reference(cfg):
    m = pyoracle.HostMaterial(os.path.join(B.BUNDLES, B.bundle_file_name(cfg)))
    e = np.concatenate([W.loguniform_energies(20000, 1e-6, 3.0, 11),
                        W.al_wavelength_energies(5000, 12)])
    seed = 987654321
    r = pyoracle.reference_run(cfg, e, seed, callseq=7, stream=3)
    np.testing.assert_array_equal(m.xs(e), r["xs"])
    ef, mu, st, nd = m.scatter(e, seed, callseq=7, stream=3)
    assert np.all(st == 0) and np.all(r["status"] == 0)
    np.testing.assert_array_equal(nd, r["ndraws"])
    np.testing.assert_array_equal(ef, r["ekin_final"])
    np.testing.assert_array_equal(mu, r["mu"])


@pytest.mark.parametrize("cfg", [W.AL, W.PE293, W.WATER])
def test_oracle_directions_equal_live_reference(cfg):
    """ncrystal_samplescatter of the reference, driven with the same streams,
    against the oracle: identical E' and outgoing directions."""
    m = pyoracle.HostMaterial(B.export_bundles([cfg])[cfg])
    r = np.random.default_rng(17)
    e = np.concatenate([W.loguniform_energies(5000, 1e-5, 20.0, 18), [-1.0, 0.0, 1e-300]])
    d = r.normal(size=(len(e), 3))
    ef, do, st = m.scatter_dir(e, d, 4321)
    ref = pyoracle.reference_run_dir(cfg, e, d, 4321)
    # the reference raises CalcError exactly where the oracle fails (E = 0 for
    # S(alpha,beta) materials: beta = -E/kT)
    np.testing.assert_array_equal(st != 0, ref["status"] != 0)
    np.testing.assert_array_equal(ef, ref["ekin_final"])
    np.testing.assert_array_equal(do, ref["direction"])


@pytest.mark.parametrize("cfg", [W.AL, W.PE293, W.WATER, W.AL2O3])
def test_oracle_absorption_equals_live_reference(cfg):
    m = pyoracle.HostMaterial(B.export_bundles([cfg])[cfg])
    e = np.concatenate([W.loguniform_energies(3000, 1e-7, 1e3, 5), [0.0, -1.0, np.inf]])
    np.testing.assert_array_equal(m.abs_xs(e), pyoracle.reference_abs_xs(cfg, e))
