"""The CPU oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py with the reference library) and against the
reference's known-answer tests."""
import glob
import os

import numpy as np
import pytest

from conftest import KAT_AL_BRAGG, KAT_NI, bundle_path
from oracle.pyoracle import HostMaterial

GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                if not os.path.basename(p).startswith(("dir_", "abs_", "mmc_")))
WL2EKIN = 0.081804209605330899


def flteq(a, b, rtol=1e-6, atol=1e-6):
    # NCrystal's floateq (NCMath.hh:538-547), as used by _testimpl.py:70-71
    return abs(a - b) <= 0.5 * rtol * (abs(a) + abs(b)) + atol


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference_golden(path):
    g = np.load(path)
    cfg = str(g["cfg"])
    m = HostMaterial(bundle_path(cfg))
    e = g["ekin"]
    xs = m.xs(e)
    # cross-sections: the reference's FP64 values (bit-identical on x86-64;
    # allow 1 ulp-level differences of another libm)
    np.testing.assert_allclose(xs, g["xs"], rtol=1e-14, atol=0)
    ef, mu, st, nd = m.scatter(e, int(g["seed"]))
    # the reference raised no error on these inputs, and neither may the oracle
    assert np.all(g["status"] == 0)
    assert np.all(st == 0)
    # same number of random numbers consumed, same (E', mu)
    np.testing.assert_array_equal(nd, g["ndraws"])
    np.testing.assert_allclose(ef, g["ekin_final"], rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(mu, g["mu"], rtol=0, atol=1e-13)


def test_kat_al_powderbragg():
    """_testimpl.py:118-133: Al PowderBragg-only xs at 4 and 5 Aa."""
    m = HostMaterial(bundle_path(KAT_AL_BRAGG))
    xs = m.xs(np.array([WL2EKIN / 16.0, WL2EKIN / 25.0]))
    assert flteq(1.632435821586171, xs[0])
    assert xs[1] == 0.0


def test_kat_ni_total():
    """_testimpl.py:146-158: Ni (dcutoff=0.6, vdoslux=2) total xs at 1.2 and 5 Aa."""
    m = HostMaterial(bundle_path(KAT_NI))
    xs = m.xs(np.array([WL2EKIN / 1.44, WL2EKIN / 25.0]))
    assert flteq(16.76474410391571, xs[0])
    assert flteq(5.958467463288343, xs[1])


def test_basic_log_al_bragg_curve():
    """tests/scripts/basic.log:32-33: Al PowderBragg xs at 1,2,3,4 Aa (%g format)."""
    m = HostMaterial(bundle_path(KAT_AL_BRAGG.replace("dcutoff=1.4;", "")))
    wl = np.array([1.0, 2.0, 3.0, 4.0])
    xs = m.xs(WL2EKIN / wl ** 2)
    assert ["%g" % v for v in xs] == ["0.72722", "1.09644", "0.918245", "1.63244"]


DIR_GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "dir_*.npz")))


@pytest.mark.parametrize("path", DIR_GOLDEN, ids=[os.path.basename(p)[:-4] for p in DIR_GOLDEN])
def test_oracle_directions_match_reference_golden(path):
    """Scatters with directions (ncrystal_samplescatter): the oracle against the
    reference's outputs on the same streams, bit for bit on x86-64 (to rounding
    of another libm elsewhere); out-of-domain and non-normalised inputs
    included."""
    g = np.load(path)
    m = HostMaterial(bundle_path(str(g["cfg"])))
    ef, d, st = m.scatter_dir(g["ekin"], g["direction"], int(g["seed"]))
    assert np.all(g["status"] == 0) and np.all(st == 0)
    np.testing.assert_allclose(ef, g["ekin_final"], rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(d, g["direction_final"], rtol=0, atol=1e-13)
    inside = g["ekin"] > 0
    np.testing.assert_allclose(np.linalg.norm(d[inside], axis=1), 1.0, atol=1e-12)


def test_oracle_absorption_matches_reference_golden():
    """AbsOOV cross-sections c/sqrt(E) against the reference's
    (ncrystal_create_absorption), bit for bit."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "abs_xs.npz"))
    for k, cfg in enumerate(g["cfgs"]):
        m = HostMaterial(bundle_path(str(cfg)))
        np.testing.assert_array_equal(m.abs_xs(g["ekin"]), g["xs"][k])
