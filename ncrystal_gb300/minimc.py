"""MiniMC on the device, with the reference's Python entry points
(ncrystal_python/src/NCrystal/minimc.py:46-115, _mmc_impl.py:42-110):

    import ncrystal_gb300.minimc as M
    res = M.run("Polyethylene_CH2.ncmat;temp=293K", scenario="1.8Aa on 1mfp sphere",
                enginecfg="seed=1;tally=theta,mu")
    res["output"]["tally"]["theta"]["total"]["bindata"]["content"]

The query goes to ncrystal_jsonquery of this library, which runs the engine
with the neutron population resident on the GPU.  Results are returned as the
reference's JSON document (NCrystalMiniMCResults_v1), as a dictionary (or the
raw JSON text with unpack='json').  Callbacks over all tallied neutrons
(ncrystal_flexmmcrun) are not offered.
"""
import json as _json
import ctypes as _C

from .core import NCBadInput, _check, lib


def _take_json(raw):
    if not raw:
        _check()
        raise NCBadInput("MiniMC query failed")
    try:
        txt = _C.cast(raw, _C.c_char_p).value.decode()
    finally:
        lib().ncrystal_dealloc_string(raw)
    return _json.loads(txt)


def _query(*entries, unpack="dict"):
    for e in entries:
        if "\x07" in e:
            raise NCBadInput("query entries may not contain the BEL character")
    raw = lib().ncrystal_jsonquery("\x07".join(entries).encode())
    if not raw:
        _check()
        raise NCBadInput("MiniMC query failed")
    try:
        txt = _C.cast(raw, _C.c_char_p).value.decode()
    finally:
        lib().ncrystal_dealloc_string(raw)
    return txt if unpack == "json" else _json.loads(txt)


def run(cfgstr, *, geomcfg=None, srccfg=None, scenario=None, enginecfg=None, callback=None,
        callback_options=None, unpack="dict"):
    """Run MiniMC (same parameter rules as the reference's minimc.run)."""
    for v, n in ((cfgstr, "cfgstr"), (geomcfg, "geomcfg"), (srccfg, "srccfg"), (scenario, "scenario"),
                 (enginecfg, "enginecfg")):
        if v is not None and not isinstance(v, str):
            raise NCBadInput(f"The {n} parameter must be a string.")
    if cfgstr is None:
        raise NCBadInput("Missing required parameter: cfgstr.")
    if callback is not None or callback_options is not None:
        raise NCBadInput("MiniMC callbacks are not supported by the device engine.")
    if unpack not in ("dict", "json", "dict_jsoncompat"):
        raise NCBadInput('Invalid value of unpack (must be "dict", "json", or "dict_jsoncompat"): %r' % (unpack,))
    enginecfg = "" if enginecfg is None else enginecfg
    n_geomsrc = (geomcfg is not None) + (srccfg is not None)
    if n_geomsrc == 0 and scenario is None:
        scenario = ""
    if n_geomsrc and scenario is not None:
        raise NCBadInput("Inconsistent parameters. Do not supply geomcfg or srccfg when also supplying a "
                         "scenario string.")
    if n_geomsrc == 1:
        raise NCBadInput("Missing %scfg parameter." % ("geom" if srccfg is not None else "src"))
    q = ["mmc", "run", cfgstr] + ([geomcfg, srccfg] if n_geomsrc else [scenario]) + [enginecfg]
    return _query(*q, unpack="json" if unpack == "json" else "dict")


def decode_scenario(cfgstr, scenario):
    """{'geomcfg': ..., 'srccfg': ...} of a scenario string (NCMMC_Utils.cc:244-490)."""
    return _query("mmc", "scenario", cfgstr, scenario)


def decode_cfgstr(cfgstr, cfgtype):
    """Decoded MiniMC cfg-string of type "src", "geom" or "engine"."""
    if cfgtype not in ("src", "geom", "engine"):
        raise NCBadInput('cfgtype parameter must be "src", "geom", or "engine"')
    return _query("mmc", "inspectcfg", cfgtype, cfgstr)


def hist_arrays(res, tally="theta", part="total"):
    """(edges, content, errorsq) of one tally histogram of a results dict;
    part is "total" or a breakdown name (NOSCAT, SINGLESCAT_ELAS, ...)."""
    import numpy as np
    t = res["output"]["tally"][tally]
    h = t["total"] if part == "total" else t["breakdown"][part]
    b = h["bindata"]
    edges = np.linspace(b["xmin"], b["xmax"], b["nbins"] + 1)
    return edges, np.asarray(b["content"], dtype=float), np.asarray(b["errorsq"], dtype=float)
