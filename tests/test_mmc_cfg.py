"""MiniMC configuration handling of the device engine (no GPU needed): the
cfg-string decoding behind ["mmc","inspectcfg",...] queries, its errors, the
Python entry point's argument rules, and the consistency of the reference
fixtures the GPU tests compare against."""
import glob
import os

import numpy as np
import pytest

import ncrystal_gb300 as NC
import ncrystal_gb300.minimc as M

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_geometry_cfg_decoding():
    d = M.decode_cfgstr("sphere;r=0.05", "geom")
    assert d["cfgstr"] == "sphere;r=0.05" and d["decoded"]["r"] == 0.05
    assert M.decode_cfgstr("sphere", "geom")["decoded"]["r"] == 0.01          # default radius 1 cm
    d = M.decode_cfgstr("box;dx=0.1;dy=0.2;dz=0.3", "geom")["decoded"]
    assert (d["dx"], d["dy"], d["dz"]) == (0.1, 0.2, 0.3)
    d = M.decode_cfgstr("cyl;r=0.007;dy=0.03", "geom")["decoded"]
    assert (d["name"], d["r"], d["dy"]) == ("cyl", 0.007, 0.03)
    assert M.decode_cfgstr("slab", "geom")["decoded"]["dz"] == 0.01
    # repeated keys: the last value wins (NCMMC_ParseCfg.hh:45-75)
    assert M.decode_cfgstr("sphere;r=1;r=2", "geom")["decoded"]["r"] == 2.0


@pytest.mark.parametrize("cfg,msg", [
    ("foo", "Unknown geometry type"),
    ("sphere;q=1", "Invalid parameter for chosen geometry"),
    ("sphere;r=-1", "Invalid value for parameter"),
    ("box;dx=abc", "Invalid value for parameter"),
])
def test_geometry_cfg_errors(cfg, msg):
    with pytest.raises(NC.NCBadInput, match=msg):
        M.decode_cfgstr(cfg, "geom")


def test_source_cfg_decoding():
    d = M.decode_cfgstr("constant;ekin=0.025;z=-0.01;n=1e5", "src")
    assert d["decoded"]["n"] == 100000 and d["decoded"]["z"] == -0.01 and d["decoded"]["uz"] == 1
    assert "ekin=0.025" in d["cfgstr"]
    d = M.decode_cfgstr("circular;wl=1.8-5;r=0.01", "src")
    assert "wl=1.8-5" in d["cfgstr"] and d["decoded"]["r"] == 0.01
    assert "thermal:300K" in M.decode_cfgstr("isotropic;ekin=thermal:300K", "src")["cfgstr"]
    assert "wl=1.8+-0.01" in M.decode_cfgstr("constant;wl=1.8+-0.01", "src")["cfgstr"]
    # a '-' after an exponent is not a range (NCMMC_ParseCfg.hh:268-276)
    assert "ekin=1e-05" in M.decode_cfgstr("constant;ekin=1e-5", "src")["cfgstr"]
    d = M.decode_cfgstr("constant;ux=0;uy=3;uz=4", "src")["decoded"]
    assert abs(d["uy"] - 0.6) < 1e-15 and abs(d["uz"] - 0.8) < 1e-15


@pytest.mark.parametrize("cfg,msg", [
    ("constant;ekin=1;wl=2", "Do not set both"),
    ("constant;ekin=0.5-0.1", "Invalid value"),
    ("constant;wl=thermal:300K", "do not use"),
    ("isotropic;ekin=thermal:300", "Maxwell"),
    ("constant;n=1.5", "Invalid value for parameter \"n\""),
    ("circular;q=2", "Invalid parameter for chosen source"),
    ("beam;ekin=1", "Unknown source type"),
])
def test_source_cfg_errors(cfg, msg):
    with pytest.raises(NC.NCBadInput, match=msg):
        M.decode_cfgstr(cfg, "src")


def test_engine_cfg_decoding():
    d = M.decode_cfgstr("", "engine")
    assert d["cfgstr"] == ""
    dd = d["decoded"]
    assert dd["tally"] == ["theta"] and dd["absorption"] and dd["tallybreakdown"]
    assert dd["roulette"] == {"psurvival": 0.1, "weight_threshold": 0.01, "nscat_threshold": 2}
    d = M.decode_cfgstr("seed=7;tally=mu,q,e,l;roulette=0.5,1e-4,5;nscatlimit=1;absorption=0", "engine")
    dd = d["decoded"]
    assert dd["seed"] == 7 and dd["tally"] == ["e", "l", "mu", "q"] and dd["nscatlimit"] == 1
    assert not dd["absorption"] and dd["roulette"]["nscat_threshold"] == 5


@pytest.mark.parametrize("cfg,msg", [
    ("bad=1", "Invalid parameter for chosen engine"),
    ("tally=lowres", "tallybins=-"),
    ("tally=nobreakdown", "tallybreakdown=0"),
    ("tally=foo", "Invalid tally"),
    ("roulette=0.5,1", "Invalid roulette options"),
    ("roulette=1.5,0.1,2", "must be <1.0"),
    ("tallybins=q:10:1", "Invalid enginecfg tallybins entry"),
    ("tallyref=other", "tallyref must be"),
    ("seed=-3", "Invalid seed"),
    ("absorption=2", "Invalid value for parameter"),
    ("nscatlimit=40000", "at most 32000"),
    ("foo", "Invalid MiniMC engine"),
])
def test_engine_cfg_errors(cfg, msg):
    with pytest.raises(NC.NCBadInput, match=msg):
        M.decode_cfgstr(cfg, "engine")


def test_run_argument_rules():
    with pytest.raises(NC.NCBadInput, match="Missing required parameter"):
        M.run(None)
    with pytest.raises(NC.NCBadInput, match="Inconsistent parameters"):
        M.run("Al_sg225.ncmat", geomcfg="sphere", srccfg="constant", scenario="1Aa")
    with pytest.raises(NC.NCBadInput, match="Missing srccfg"):
        M.run("Al_sg225.ncmat", geomcfg="sphere")
    with pytest.raises(NC.NCBadInput, match="callbacks"):
        M.run("Al_sg225.ncmat", callback=lambda *a: 0)


def test_non_minimc_queries_are_refused():
    with pytest.raises(NC.NCBadInput, match="only MiniMC"):
        M._query("nc", "info")


def test_reference_fixtures_are_consistent():
    """The reference's breakdowns add up to its totals, and its metadata
    counts are those of the queries (guards the fixture files)."""
    from mmc_stats import GROUPS
    files = sorted(glob.glob(os.path.join(GOLDEN, "mmc_*.npz")))
    files = [f for f in files if not f.endswith("mmc_scenarios.npz")]
    assert len(files) >= 5
    for f in files:
        g = np.load(f)
        assert g["meta.provided"][0] == 1e7
        tallies = sorted({k.split(".")[0] for k in g.files if k.endswith(".total.content")})
        for t in tallies:
            tot = g["%s.total.content" % t]
            parts = [g["%s.%s.content" % (t, p)] for p in GROUPS if "%s.%s.content" % (t, p) in g.files]
            if parts:
                np.testing.assert_allclose(np.sum(parts, axis=0), tot, rtol=1e-9, atol=1e-9 * tot.max())
    sc = np.load(os.path.join(GOLDEN, "mmc_scenarios.npz"))["rows"]
    assert sc.shape[1] == 4 and len(sc) >= 8
