"""Device-side derivation of the S(alpha,beta) sampling tables
(ncrystal_gb300/csrc/ncgb_sabderive.cu) against the host builder, which the
CPU tests pin bit for bit to the reference's own tables: identical integer
structure, doubles equal up to the last-place differences of CUDA's log/exp;
and materials built with the device builder scatter like host-built ones."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import ncrystal_gb300 as NC
import ncrystal_gb300.workloads as W
from conftest import bundle_path
from ncrystal_gb300.bundle.reader import read_bundle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _sab_components(path):
    b = read_bundle(path)
    return [i for i in range(int(b["ncomp"][0])) if "c%d.sab" % i in b]


@pytest.mark.parametrize("cfg", [W.PE293, W.WATER, W.AL2O3, W.AL, "Polyethylene_CH2.ncmat;temp=320K"])
def test_device_derivation_matches_host(cfg):
    path = bundle_path(cfg)
    comps = _sab_components(path)
    assert comps
    for c in comps:
        r = NC.core.sab_derive_compare(path, c)
        print(cfg, c, json.dumps(r))
        assert r["n_int_mismatch"] == 0, r
        assert r["max_rel_diff"] < 1e-9, r


_CHILD = r"""
import json, sys, numpy as np
import ncrystal_gb300 as NC, ncrystal_gb300.workloads as W
e = W.loguniform_energies(200000, 1e-4, 2.0, 5)
sc = NC.createScatter(sys.argv[1], seed=77)
xs = sc.crossSectionIsotropic(e)
ef, mu = sc.sampleScatterIsotropic(e)
np.savez(sys.argv[2], xs=xs, ef=ef, mu=mu)
"""


def test_device_built_material_scatters_like_host_built(tmp_path):
    cfg = W.PE293
    bundle_path(cfg)
    out = {}
    for mode in ("host", "device"):
        env = dict(os.environ, NCGB_TABLES_BUILD=mode, PYTHONPATH=ROOT)
        f = str(tmp_path / (mode + ".npz"))
        subprocess.run([sys.executable, "-c", _CHILD, cfg, f], env=env, check=True, cwd=ROOT)
        out[mode] = np.load(f)
    h, d = out["host"], out["device"]
    np.testing.assert_allclose(d["xs"], h["xs"], rtol=1e-10, atol=0)
    same = np.isclose(d["ef"], h["ef"], rtol=1e-6, atol=1e-300) & np.isclose(d["mu"], h["mu"], rtol=0, atol=1e-6)
    assert same.mean() > 0.999, same.mean()


def test_batched_device_derivation_matches_host():
    """Every S(alpha,beta) component of every material bundle, derived in one
    batched device derivation, against the host builder."""
    import ncrystal_gb300._build as B
    paths = sorted(os.path.join(B.BUNDLES, f) for f in os.listdir(B.BUNDLES) if f.endswith(".ncgb"))
    assert paths
    r = NC.core.sab_derive_compare_many(paths)
    print(len(paths), "bundles", json.dumps(r))
    assert r["ncomp"] >= len(W.PE_TRAIN_TEMPS)
    assert r["n_int_mismatch"] == 0, r
    assert r["max_rel_diff"] < 1e-9, r


_CHILD_MANY = r"""
import json, sys, numpy as np
import ncrystal_gb300 as NC, ncrystal_gb300.workloads as W
cfgs = json.loads(sys.argv[1])
e = W.loguniform_energies(50000, 1e-4, 2.0, 9)
if sys.argv[3] == "batched":
    scs = NC.core.createScatters(cfgs + cfgs[:2], seed=41)[:len(cfgs)]
else:
    scs = [NC.createScatter(c, seed=41) for c in cfgs]
out = {}
for i, sc in enumerate(scs):
    out["xs%d" % i] = sc.crossSectionIsotropic(e)
    out["ef%d" % i], out["mu%d" % i] = sc.sampleScatterIsotropic(e)
np.savez(sys.argv[2], **out)
"""


def test_create_scatters_batched_matches_single(tmp_path):
    """ncgb_create_scatters (one batched device derivation for a temperature
    grid, duplicates included) gives the handles that one-by-one host-built
    creation gives: same cross sections, same sampled scatterings."""
    cfgs = [W.pe_cfg(T) for T in W.PE_TRAIN_TEMPS[:4]] + [W.WATER]
    for c in cfgs:
        bundle_path(c)
    out = {}
    for mode, build in (("batched", "device"), ("single", "host")):
        env = dict(os.environ, NCGB_TABLES_BUILD=build, PYTHONPATH=ROOT)
        f = str(tmp_path / (mode + ".npz"))
        subprocess.run([sys.executable, "-c", _CHILD_MANY, json.dumps(cfgs), f, mode], env=env, check=True,
                       cwd=ROOT)
        out[mode] = np.load(f)
    b, s = out["batched"], out["single"]
    for i in range(len(cfgs)):
        np.testing.assert_allclose(b["xs%d" % i], s["xs%d" % i], rtol=1e-10, atol=0)
        same = (np.isclose(b["ef%d" % i], s["ef%d" % i], rtol=1e-6, atol=1e-300)
                & np.isclose(b["mu%d" % i], s["mu%d" % i], rtol=0, atol=1e-6))
        assert same.mean() > 0.999, (cfgs[i], same.mean())


def test_create_scatters_errors():
    with pytest.raises(NC.NCException):
        NC.core.createScatters([W.PE293, "NoSuchMaterial_sg1.ncmat"])
    assert NC.core.createScatters([]) == []


_CHILD_GROUPS = r"""
import json, sys
import ncrystal_gb300 as NC
print(json.dumps(NC.core.sab_derive_compare_many(json.loads(sys.argv[1]))))
"""


def test_batched_derivation_in_memory_bounded_groups():
    """A device budget below one allocation for all components
    (NCGB_TABLES_DEVICE_MB) splits the derivation into groups with the same
    results: the same doubles differ from the host builder, by the same
    largest amount."""
    cfgs = [W.pe_cfg(T) for T in W.PE_TRAIN_TEMPS] + [W.WATER, W.AL2O3]
    paths = [bundle_path(c) for c in cfgs]
    out = {}
    for mb in ("200", "16384"):
        env = dict(os.environ, NCGB_TABLES_DEVICE_MB=mb, PYTHONPATH=ROOT)
        r = subprocess.run([sys.executable, "-c", _CHILD_GROUPS, json.dumps(paths)], env=env, check=True,
                           cwd=ROOT, capture_output=True, text=True)
        out[mb] = json.loads(r.stdout.strip().splitlines()[-1])
        print(mb, "MB", out[mb])
    a, b = out["200"], out["16384"]
    assert a["n_int_mismatch"] == 0 and b["n_int_mismatch"] == 0
    for k in ("ncomp", "n_double_diff", "max_rel_diff"):
        assert a[k] == b[k], (k, a, b)
