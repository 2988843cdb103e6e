"""Synthetic neutron workloads (seeded) of the batched scattering benchmarks.

The reference publishes no benchmark suite for this path; these are the five
workload shapes the path is measured on, with their material cfg-strings,
neutron counts and energy distributions.  Energies are generated with numpy's
PCG64 from fixed seeds, so every run and every machine sees the same arrays.
"""
import math

import numpy as np

WL2EKIN = 0.081804209605330899  # eV*Aa^2, NCDefs.hh:823-838

# Materials of the ragged crystal batch (16 crystals x 4 temperatures).
CRYSTALS16 = [
    "Al_sg225.ncmat", "Cu_sg225.ncmat", "Ni_sg225.ncmat", "Si_sg227.ncmat",
    "Ge_sg227.ncmat", "Fe_sg229_Iron-alpha.ncmat", "Mg_sg194.ncmat",
    "MgO_sg225_Periclase.ncmat", "Al2O3_sg167_Corundum.ncmat",
    "LiF_sg225_LithiumFlouride.ncmat", "NaCl_sg225_SodiumChloride.ncmat",
    "CaF2_sg225_CalciumFlouride.ncmat", "SiC-beta_sg216_BetaSiliconCarbide.ncmat",
    "TiO2_sg136_Rutile.ncmat", "ZnO_sg186_ZincOxide.ncmat", "Nb_sg229.ncmat",
]
CRYSTAL_TEMPS = [77, 150, 293, 400]

AL = "Al_sg225.ncmat;temp=293K"
AL2O3 = "Al2O3_sg167_Corundum.ncmat;temp=293K;dcutoff=0.2"
PE293 = "Polyethylene_CH2.ncmat;temp=293K"
WATER = "LiquidWaterH2O_T293.6K.ncmat"


def al_wavelength_energies(n, seed=0x5EED0001):
    """Wavelengths uniform in [0.5, 5] Aa, converted to energies (eV)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    wl = rng.uniform(0.5, 5.0, n)
    return WL2EKIN / (wl * wl)


def loguniform_energies(n, emin, emax, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.exp(rng.uniform(math.log(emin), math.log(emax), n))


def crystal_batch_cfgs():
    return ["%s;temp=%dK" % (m, t) for m in CRYSTALS16 for t in CRYSTAL_TEMPS]


def mixed_batch_cfgs():
    """32 instances: liquid water (its one temperature), polyethylene at 280,
    293 and 320 K, the 16 crystals at 293 K and the first 12 at 400 K."""
    return ([WATER] + ["Polyethylene_CH2.ncmat;temp=%dK" % t for t in (280, 293, 320)]
            + ["%s;temp=293K" % m for m in CRYSTALS16] + ["%s;temp=400K" % m for m in CRYSTALS16[:12]])


def ragged_counts(ninst, lo, hi, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.exp(rng.uniform(math.log(lo), math.log(hi), ninst)).astype(np.int64)


def config(name):
    """Return a dict describing one workload: cfgs, per-instance counts and an
    energy generator."""
    if name == "al_small":
        return dict(name=name, cfgs=[AL], counts=[1 << 20],
                    energies=lambda n, k=0: al_wavelength_energies(n, 0x5EED0001 + k),
                    io="f64")
    if name == "al2o3_large":
        return dict(name=name, cfgs=[AL2O3], counts=[1 << 24],
                    energies=lambda n, k=0: loguniform_energies(n, 1e-4, 1.0, 0x5EED0002 + k),
                    io="f32")
    if name == "crystal_batch":
        cfgs = crystal_batch_cfgs()
        return dict(name=name, cfgs=cfgs, counts=list(ragged_counts(len(cfgs), 1e3, 1e6, 0x5EED0003)),
                    energies=lambda n, k=0: loguniform_energies(n, 1e-4, 1.0, 0x5EED0003 + 17 * (k + 1)),
                    io="f64")
    if name == "mixed_batch":
        cfgs = mixed_batch_cfgs()
        return dict(name=name, cfgs=cfgs, counts=list(ragged_counts(len(cfgs), 1e4, 2e6, 0x5EED0005)),
                    energies=lambda n, k=0: loguniform_energies(n, 1e-5, 2.0, 0x5EED0005 + 31 * (k + 1)),
                    io="f64")
    if name == "pe_learned":
        return dict(name=name, cfgs=[PE293], counts=[1 << 24],
                    energies=lambda n, k=0: loguniform_energies(n, 1e-4, 1.0, 0x5EED0004 + k),
                    io="f64")
    raise KeyError(name)


# Polyethylene instances the learned beta proposal is trained on (K).
PE_TRAIN_TEMPS = [250.0, 265.0, 280.0, 293.0, 305.0, 320.0, 335.0, 350.0]


def pe_cfg(T):
    return "Polyethylene_CH2.ncmat;temp=%gK" % T


# cfg-strings whose bundles the default build exports (the single-material
# workloads and the proposal's training instances).
DEFAULT_BUNDLE_CFGS = [AL, AL2O3, WATER] + [pe_cfg(T) for T in PE_TRAIN_TEMPS]
