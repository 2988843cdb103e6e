"""The S(alpha,beta) pass's phase-clock copy (ncgb_sab_phase_profile): it must
sample exactly what the product pass samples (same random streams, same
results) and return a cycle count for every phase and the number of Alg.1
attempts."""
import numpy as np
import pytest

import ncrystal_gb300 as NC
import ncrystal_gb300.workloads as W
from conftest import bundle_path

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["exact", "mixed"])
def test_phase_profile_samples_like_the_product_pass(mode):
    import torch
    bundle_path(W.PE293)
    n = 200000
    e = torch.as_tensor(W.loguniform_energies(n, 1e-4, 1.0, 81), dtype=torch.float64, device="cuda")
    ref = NC.createScatter(W.PE293, seed=4242).set_mode(mode)
    prof = NC.createScatter(W.PE293, seed=4242).set_mode(mode)
    out_r = [torch.empty_like(e) for _ in range(3)]
    out_p = [torch.empty_like(e) for _ in range(3)]
    ref.scatter_device(e, *out_r)
    torch.cuda.synchronize()
    cyc, attempts = prof.sab_phase_profile(e, *out_p)
    for a, b in zip(out_r, out_p):
        assert torch.equal(a, b)
    assert set(cyc) == set(NC.Scatter.SAB_PHASES)
    assert all(v > 0 for k, v in cyc.items() if k != "idle")
    # polyethylene: most neutrons pick an S(alpha,beta) component, each needs
    # at least one Alg.1 attempt
    assert attempts >= 0.5 * n
    shares = np.array(list(cyc.values()), dtype=float) / sum(cyc.values())
    print({k: round(float(v), 3) for k, v in zip(cyc, shares)}, attempts)
