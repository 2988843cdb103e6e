"""ncrystal_gb300 -- NCrystal's batched non-oriented scattering path on one
GB300 GPU (sm_103a), behind NCrystal's own C and Python interfaces.

    import ncrystal_gb300 as NC
    sc = NC.createScatter("Al_sg225.ncmat;temp=293K")
    xs = sc.crossSectionIsotropic(ekin_array)
    ekin_final, mu = sc.sampleScatterIsotropic(ekin_array)
"""
from .core import (NCBadInput, NCCalcError, NCException, NCFileNotFound,  # noqa: F401
                   MLP, Absorption, Batch, NCLogicError, Process, Scatter, createAbsorption, createProcess,
                   createScatter, createScatterFromBundle, bundle_path, lib, phase_times,
                   phase_timing)

__version__ = "0.1.0"
