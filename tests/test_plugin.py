"""The NCrystal plugin (libNCrystalPlugin_GB300.so) loaded into NCrystal itself
through NCRYSTAL_PLUGIN_LIST, as NCrystal loads any dynamic plugin
(NCPluginMgmt.cc:475-507), driven through NCrystal's own C interface in a
child process:

* its factory wins NCrystal's factory selection for non-oriented materials
  (priority 150 over stdscat's 100): here, without a GPU, the request fails
  loudly with the plugin's error instead of falling back to a CPU model, after
  the plugin has written the material's bundle;
* that bundle holds the same tables as the bundle exporter's for the same
  cfg-string;
* an explicit scatfactory=stdscat, a single-crystal cfg-string (which the
  GPU path does not implement) and NCGB_PLUGIN_DISABLE=1 all leave the request
  to NCrystal's own factories.

The GPU host has no NCrystal, so the plugin's device calls are covered there
through the entry points it uses (test_gpu_plugin_entry_points.py).  CPU only;
needs the NCrystal sources (reference build)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import ncrystal_gb300._build as B
from ncrystal_gb300.bundle.reader import read_bundle

REFLIB = os.path.join(B.REF_OUT, "libNCrystal.so")
pytestmark = pytest.mark.skipif(not (os.path.exists(B.plugin_path()) and os.path.exists(REFLIB)),
                                reason="needs the NCrystal sources (plugin and reference build)")

CFG = "Al_sg225.ncmat;temp=350K"
SINGLE_CRYSTAL = "Al_sg225.ncmat;mos=0.3deg;dir1=@crys_hkl:1,0,0@lab:0,0,1;dir2=@crys_hkl:0,1,0@lab:0,1,0"

# NCrystal's C interface, in a child process (plugins are read once per process)
CHILD = r"""
import ctypes as C, json, sys
class H(C.Structure):
    _fields_ = [("internal", C.c_void_p)]
L = C.CDLL(sys.argv[1])
L.ncrystal_create_scatter.restype = H
L.ncrystal_create_scatter.argtypes = [C.c_char_p]
L.ncrystal_cast_scat2proc.restype = H
L.ncrystal_cast_scat2proc.argtypes = [H]
L.ncrystal_name.restype = C.c_char_p
L.ncrystal_name.argtypes = [H]
L.ncrystal_lasterror.restype = C.c_char_p
L.ncrystal_lasterrortype.restype = C.c_char_p
L.ncrystal_sethaltonerror(0)
L.ncrystal_setquietonerror(1)
out = []
for cfg in sys.argv[2:]:
    h = L.ncrystal_create_scatter(cfg.encode())
    if L.ncrystal_error():
        out.append({"cfg": cfg, "ok": False, "type": L.ncrystal_lasterrortype().decode(),
                    "error": L.ncrystal_lasterror().decode()})
        L.ncrystal_clearerror()
    else:
        out.append({"cfg": cfg, "ok": True, "name": L.ncrystal_name(L.ncrystal_cast_scat2proc(h)).decode()})
print(json.dumps(out))
"""


def run_ncrystal(cfgs, cache, **env_extra):
    env = dict(os.environ)
    env.update({"NCRYSTAL_PLUGIN_LIST": B.plugin_path(), "NCGB_BUNDLE_CACHE": str(cache),
                "CUDA_VISIBLE_DEVICES": ""})
    env.update(env_extra)
    r = subprocess.run([sys.executable, "-c", CHILD, REFLIB] + list(cfgs), env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_plugin_wins_factory_selection_and_fails_loudly_without_gpu(tmp_path):
    res = run_ncrystal([CFG], tmp_path)[0]
    assert not res["ok"]
    assert "GB300 plugin" in res["error"], res
    # the bundle of the request was written before the device upload failed
    assert [f for f in os.listdir(str(tmp_path)) if f.startswith("plugin_") and f.endswith(".ncgb")]


def test_plugin_bundle_equals_exporter_bundle(tmp_path):
    run_ncrystal([CFG], tmp_path)
    plug = [f for f in os.listdir(str(tmp_path)) if f.startswith("plugin_") and f.endswith(".ncgb")]
    assert len(plug) == 1
    a = read_bundle(os.path.join(str(tmp_path), plug[0]))
    b = read_bundle(B.export_bundles([CFG], outdir=str(tmp_path / "tool"))[CFG])
    # the plugin records NCrystal's request description as its key and no
    # absorption constant; everything the tables are built from is identical
    skip = {"cfg", "abs_c", "ncrystal_version"}
    assert set(a) - skip == set(b) - skip
    for k in sorted(set(a) - skip):
        if isinstance(a[k], str):
            assert a[k] == b[k], k
        else:
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_requests_the_plugin_leaves_to_ncrystal(tmp_path):
    res = run_ncrystal([CFG + ";scatfactory=stdscat", SINGLE_CRYSTAL], tmp_path)
    assert all(r["ok"] for r in res), res
    assert res[0]["name"] != "GB300Scatter"
    res = run_ncrystal([CFG], tmp_path, NCGB_PLUGIN_DISABLE="1")
    assert res[0]["ok"] and res[0]["name"] != "GB300Scatter", res
