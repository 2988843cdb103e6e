"""Test configuration.

Markers: tests that need a CUDA GPU are marked ``gpu``; everything else runs
on the CPU.  A session fixture builds the library and the oracle (quick, and
a no-op when up to date) and, where the NCrystal sources are present, the
reference harness and the material bundles.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


# Known-answer-test materials of the reference (ncrystal_python/src/NCrystal/_testimpl.py:118-158)
KAT_AL_BRAGG = "Al_sg225.ncmat;dcutoff=1.4;incoh_elas=0;inelas=0"
KAT_NI = "Ni_sg225.ncmat;dcutoff=0.6;vdoslux=2"


def bundle_path(cfg):
    import ncrystal_gb300._build as B
    p = os.path.join(B.BUNDLES, B.bundle_file_name(cfg))
    if not os.path.exists(p):
        pytest.skip("no material bundle for %r (bundles are exported where the NCrystal sources exist)" % cfg)
    return p


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
