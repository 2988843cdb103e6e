"""Learned beta proposal on the GPU: the network's kernels against the CPU
restatement (oracle/mlp_ref.py), training, the gain of the trained network
over the same envelope without it, per-stream parity of the learned sampler
with the CPU oracle, and 1e8-event distribution tests against the plain
sampler."""

import numpy as np
import pytest

import ncrystal_gb300 as NC
import ncrystal_gb300.learn as LR
import ncrystal_gb300.workloads as W
from conftest import bundle_path
from oracle import mlp_ref
from oracle.pyoracle import HostMaterial

pytestmark = pytest.mark.gpu

RANGES = (LR.TRAIN_EMIN, LR.TRAIN_EMAX, 250.0, 350.0)


def _log_ranges(r):
    return (float(np.float32(np.log(r[0]))), float(np.float32(np.log(r[1]))), r[2], r[3])


def _cuda(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float32), device="cuda")


@pytest.fixture(scope="module")
def nets():
    for T in LR.TRAIN_TEMPS:
        bundle_path(W.pe_cfg(T))
    n, info = LR.train_proposals(n_total=1 << 24, steps=4000, batch=8192, lr=2e-3, seed=3)
    return n, info


def test_mlp_gradients_match_cpu_restatement():
    net = NC.MLP(seed=5, emin=RANGES[0], emax=RANGES[1], tmin=RANGES[2], tmax=RANGES[3])
    r = np.random.default_rng(1)
    n = 4096
    loge = r.uniform(np.log(1e-5), np.log(2.0), n).astype(np.float32)
    temp = r.uniform(250, 350, n).astype(np.float32)
    tgt = np.arcsinh(r.normal(0, 5, n)).astype(np.float32)
    loss, g = net.gradients(_cuda(loge), _cuda(temp), _cuda(tgt))
    p = net.params()
    rl, rg = mlp_ref.loss_and_gradients(p, loge, temp, tgt, _log_ranges(RANGES))
    assert abs(loss - rl) <= 2e-3 * abs(rl)
    w, b, _ = mlp_ref.layout()
    for l in range(5):
        for off, size in ((w[l], mlp_ref.DIN[l] * mlp_ref.DOUT[l]), (b[l], mlp_ref.DOUT[l])):
            gg, rr = g[off:off + size].astype(np.float64), rg[off:off + size]
            nrm = np.linalg.norm(rr)
            if nrm == 0:
                assert np.all(gg == 0)
                continue
            # BF16 operands: the GPU and the restatement round the same values;
            # accumulation order differs, which may flip a BF16 rounding
            assert np.linalg.norm(gg - rr) <= 2e-2 * nrm, (l, off)
            assert np.dot(gg, rr) / (np.linalg.norm(gg) * nrm) > 0.999


def test_mlp_knots_match_fp32_reference():
    """Inference (BF16 GEMMs, FP32 accumulation) against a plain FP64
    evaluation of the same network without BF16 rounding."""
    import torch
    net = NC.MLP(seed=9, emin=RANGES[0], emax=RANGES[1], tmin=RANGES[2], tmax=RANGES[3])
    r = np.random.default_rng(2)
    n = 1000
    loge = r.uniform(np.log(1e-5), np.log(2.0), n).astype(np.float32)
    temp = r.uniform(250, 350, n).astype(np.float32)
    k = net.knots(_cuda(loge), _cuda(temp)).cpu().numpy()
    ref = mlp_ref.knots(net.params(), loge, temp, _log_ranges(RANGES), emulate_bf16=False)
    assert np.all(np.diff(k, axis=1) >= 0)
    assert np.all(np.abs(k - ref) <= 0.05 + 0.02 * np.abs(ref))
    ref16 = mlp_ref.knots(net.params(), loge, temp, _log_ranges(RANGES), emulate_bf16=True)
    assert np.all(np.abs(k - ref16) <= 5e-3 + 5e-3 * np.abs(ref16))
    del torch


def test_training_reduces_loss(nets):
    """Pinball loss on fresh samples (Polyethylene at 293 K): the trained
    network against an untrained one; the quantile loss has an irreducible
    part, so the trained loss is compared, not required to vanish."""
    n, info = nets
    for comp, net in n.items():
        tr = info[comp]["loss_trace"]
        assert len(tr) >= 4 and tr[-1] <= tr[0], tr
        loge, temp, tgt = LR.training_set([W.PE293], comp, 1 << 16, seed=99)
        trained, _ = net.gradients(loge, temp, tgt)
        fresh, _ = NC.MLP(seed=123, emin=RANGES[0], emax=RANGES[1]).gradients(loge, temp, tgt)
        print("comp %d pinball loss: trained %.4f untrained %.4f" % (comp, trained, fresh))
        assert trained < 0.8 * fresh


def test_trained_network_gain(nets):
    """Envelope acceptance on Polyethylene at 293 K (inside the trained
    range) with the trained network's knots, against the same envelope
    built from an untrained network and from equal-width knots."""
    n, _ = nets
    sc = NC.createScatter(W.PE293, seed=1)
    for comp, net in n.items():
        trained = sc.attach_proposal(comp, net, min_accept=0.0)
        untrained = sc.attach_proposal(comp, NC.MLP(seed=77, emin=RANGES[0], emax=RANGES[1]), min_accept=0.0)
        uniform = sc.attach_proposal_knots(comp, LR.reference_knots(W.PE293, comp, "uniform"), min_accept=0.0)
        exact = sc.attach_proposal_knots(comp, LR.reference_knots(W.PE293, comp, "quantile"), min_accept=0.0)
        print("comp %d acceptance: trained %.3f untrained %.3f uniform %.3f exact-quantile %.3f"
              % (comp, trained, untrained, uniform, exact))
        # the trained knots do as well as the exact quantiles of the table,
        # better than an untrained network's and much better than equal widths
        assert trained > 0.9 and abs(trained - exact) < 0.01
        assert trained > untrained + 0.02
        assert trained > uniform + 0.1
        sc.detach_proposal(comp)


def _attached(nets, cfg, seed):
    n, _ = nets
    sc = NC.createScatter(cfg, seed=seed)
    for comp, net in n.items():
        sc.attach_proposal(comp, net, min_accept=0.5)
    return sc.set_sampler("learned")


def test_learned_sampler_matches_oracle_per_stream(nets):
    """The CUDA learned sampler and the oracle's restatement of it, same knots
    and tables, same random streams."""
    import torch
    n, _ = nets
    cfg = W.PE293
    sc = _attached(nets, cfg, 31)
    m = HostMaterial(bundle_path(cfg))
    T = sc.material_info()[1]
    for comp, net in n.items():
        eg = sc.sab_egrid(comp)
        kn = net.knots(_cuda(np.log(eg)), _cuda(np.full(len(eg), T))).cpu().numpy()
        lo, hi = np.float32(np.log(RANGES[0])), np.float32(np.log(RANGES[1]))
        allowed = ((np.log(eg).astype(np.float32) >= lo) & (np.log(eg).astype(np.float32) <= hi)).astype(np.uint8)
        tables = m.build_proposal(comp, kn, allowed=allowed, min_accept=0.5)
        acc, en = sc.proposal_acceptance(comp)
        np.testing.assert_array_equal(en, tables[0]["enabled"].astype(bool))
        np.testing.assert_array_equal(acc, tables[0]["accept"])
        m.set_proposal(comp, tables)
    e = np.concatenate([W.loguniform_energies(150000, 1e-5, 3.0, 41), np.full(20000, 0.0253)])
    ef, mu = sc.sampleScatterIsotropic(e)
    oef, omu, ost, _ = m.scatter(e, 31)
    assert np.all(ost == 0)
    ok = np.isclose(ef, oef, rtol=1e-9, atol=1e-300) & np.isclose(mu, omu, rtol=0, atol=1e-9)
    assert ok.mean() >= 0.999, ok.mean()
    del torch


def test_learned_alpha_beta_vs_plain(nets):
    """(alpha, beta) of the hydrogen component alone, learned vs plain, at
    fixed energies: KS on beta and alpha, 4e6 samples each."""
    import torch
    from scipy.stats import ks_2samp
    n, _ = nets
    learned = _attached(nets, W.PE293, 51)
    plain = NC.createScatter(W.PE293, seed=52)
    comp = min(n)
    for e0 in (1e-3, 0.0253, 0.5):
        e = torch.full((4_000_000,), e0, dtype=torch.float64, device="cuda")
        out = []
        for sc in (learned, plain):
            a, b = torch.empty_like(e), torch.empty_like(e)
            st = torch.empty(e.shape, dtype=torch.int32, device="cuda")
            sc.sab_sample_device(comp, e, a, b, st)
            torch.cuda.synchronize()
            assert int((st != 0).sum()) == 0
            out.append((a.cpu().numpy(), b.cpu().numpy()))
        assert ks_2samp(out[0][1], out[1][1]).pvalue > 1e-3
        assert ks_2samp(out[0][0], out[1][0]).pvalue > 1e-3


LEARNED_1E8 = [(0.001, "exact"), (0.0253, "exact"), (0.5, "exact"), (None, "mixed")]
# comparisons of the module's 1e8-event tests (chi-square, KS on E', KS on mu each)
ALPHA_1E8 = 0.01 / (3 * len(LEARNED_1E8))


@pytest.mark.parametrize("e0,mode", LEARNED_1E8,
                         ids=["%s-%s" % ("loguniform" if e is None else "%g" % e, m) for e, m in LEARNED_1E8])
def test_learned_1e8_distributions_vs_plain_oracle(nets, e0, mode):
    """1e8 events: the learned GPU sampler against the plain sampler (the CPU
    oracle, pinned to the reference), binned chi-square + exact KS, p > 0.01
    with a Bonferroni correction over the module's comparisons.  e0 None: the
    benchmark's own configuration (energies log-uniform in [1e-4, 1] eV, the
    mixed-precision mode with the learned proposal), the GPU and the oracle
    each on their own draw of 1e8 energies."""
    pytest.importorskip("scipy")
    from test_gpu_statistics import LOGU, check_same_distribution, oracle_samples, scatter_device
    import torch
    N = 10 ** 8
    sc = _attached(nets, W.PE293, 1001).set_mode(mode)
    if e0 is None:
        ge = W.loguniform_energies(N, LOGU[0], LOGU[1], 0x57A7011)
        oe = W.loguniform_energies(N, LOGU[0], LOGU[1], 0x57A7012)
        e = torch.as_tensor(ge, device="cuda")
    else:
        ge = oe = None
        e = torch.full((N,), e0, dtype=torch.float64, device="cuda")
    gef, gmu = scatter_device(sc, e)
    gef, gmu = gef.cpu().numpy(), gmu.cpu().numpy()
    del e
    oef, omu = oracle_samples(W.PE293, e0, N, seed=2002, energies=oe)
    print(check_same_distribution(gef, gmu, oef, omu, e0, ALPHA_1E8, ge=ge, oe=oe))
