"""Learned beta proposal, CPU side: the envelope tables the library builds
(ncgb_tables_build_proposal) bound the sampler's beta density everywhere, the
alias tables reproduce the interval masses, and the oracle sampling through
them gives the plain sampler's distribution (whatever the knots)."""
import os

import numpy as np
import pytest

import ncrystal_gb300._build as B
import ncrystal_gb300.learn as LR
import ncrystal_gb300.workloads as W
from conftest import bundle_path
from oracle.pyoracle import HostMaterial

K = HostMaterial.LP_K


@pytest.fixture(scope="module")
def pe():
    return HostMaterial(bundle_path(W.PE293))


def _sab_comps(m):
    n = int(m.scalar(0, "ncomp"))
    return [c for c in range(n) if m.scalar(c, "type") == 3]


def _sampler(m, comp, ie):
    off = m.array(comp, "smp_offset", np.int64)[ie]
    nb = m.array(comp, "smp_nbeta", np.int32)[ie]
    fb = m.array(comp, "smp_fbkep", np.float64)[ie]
    bx = m.array(comp, "bx", np.float64)[off:off + nb]
    by = m.array(comp, "by", np.float64)[off:off + nb]
    bc = m.array(comp, "bcdf", np.float64)[off:off + nb]
    return bx, by, bc, (1 if fb <= 0 else 0)


def _random_knots(ne, seed):
    r = np.random.default_rng(seed)
    return np.sort(r.normal(0.0, 3.0, (ne, 62)), axis=1).astype(np.float32)


@pytest.mark.parametrize("kind", ["quantile", "uniform", "random"])
def test_envelope_bounds_density_and_alias_masses(pe, kind):
    for comp in _sab_comps(pe):
        ne = len(pe.array(comp, "egrid", np.float64))
        kn = _random_knots(ne, comp) if kind == "random" else LR.reference_knots(W.PE293, comp, kind)
        hdr, slot, cell, seg = pe.build_proposal(comp, kn, min_accept=0.0)
        r = np.random.default_rng(7)
        for ie in list(range(0, ne, 23)) + [ne - 1]:
            if not hdr["enabled"][ie]:
                continue
            bx, by, bc, fr = _sampler(pe, comp, ie)
            c, sl = cell[ie], slot[ie]
            q = c["q"]
            width = c["h"] * 2.0 ** 33
            assert q[0] == bx[fr] and np.isclose(q[-1] + width[-1], bx[-1], rtol=1e-14, atol=1e-14)
            assert np.all(width >= 0) and np.all(np.diff(q) >= 0)
            assert hdr["c1"][ie] == (bc[1] if fr else 0.0)
            assert abs(hdr["c1_thr"][ie] / 2.0 ** 32 - hdr["c1"][ie]) <= 2.0 ** -32
            for k in range(K):
                lo, hi = q[k], q[k] + width[k]
                # the envelope is above y at the interval ends, at every bx
                # point inside and at random points
                if hi > lo:
                    pts = np.concatenate([[lo, hi], bx[(bx > lo) & (bx < hi)], r.uniform(lo, hi, 16)])
                    assert np.all(np.interp(pts, bx, by) <= c["env"][k]), (comp, ie, k)
                # linear pieces in the draw coordinate: the FP32 density and the
                # bin of beta(w) = q + (2w+1) h at random draws (and the piece starts)
                g = seg[c["seg_lo"][k]:c["seg_lo"][k] + c["seg_n"][k]]
                assert len(g) >= 1 and g["w0"][0] == 0 and np.all(np.diff(g["w0"].astype(np.int64)) > 0)
                if hi <= lo:
                    continue
                w = np.concatenate([g["w0"], r.integers(0, 2 ** 32, 64)]).astype(np.uint64)
                beta = (2 * w + 1).astype(np.float64) * c["h"][k] + q[k]
                ip = np.searchsorted(g["w0"], w, side="right") - 1
                gi = g[ip]
                yf = gi["y0"].astype(np.float64) + gi["slope"].astype(np.float64) * (w - gi["w0"]).astype(np.float64)
                ye = np.interp(beta, bx, by)
                assert np.all(np.abs(yf - ye) <= 1e-5 * np.maximum(ye, 1e-300) + 1e-12 * by.max()), (comp, ie, k)
                bins = gi["bin"]
                tol = 1e-14 * np.abs(beta) + 1e-300   # numpy forms beta without the FMA
                assert np.all(bx[bins] <= beta + tol)
                assert np.all((bins == len(bx) - 2) | (beta < bx[np.minimum(bins + 1, len(bx) - 1)] + tol))
            # alias table: slot probabilities add up to the interval masses
            wm = np.where(width > 0, c["env"].astype(np.float64) * width, 0.0)
            p = sl["aprob"].astype(np.float64) / K
            np.add.at(p, sl["alias"], (1.0 - sl["aprob"].astype(np.float64)) / K)
            np.testing.assert_allclose(p, wm / wm.sum(), atol=2e-7)
            # acceptance = (integral of y over the regular range) / (envelope area)
            np.testing.assert_allclose(hdr["accept"][ie], (bc[-1] - bc[fr]) / wm.sum(), rtol=1e-6)


def test_partition_from_quantiles_beats_uniform(pe):
    """The sqrt-density partition from good quantiles gives a higher envelope
    acceptance than one from equal-width knots."""
    for comp in _sab_comps(pe):
        hq = pe.build_proposal(comp, LR.reference_knots(W.PE293, comp, "quantile"), min_accept=0.0)[0]
        hu = pe.build_proposal(comp, LR.reference_knots(W.PE293, comp, "uniform"), min_accept=0.0)[0]
        eq, eu = hq["enabled"].astype(bool), hu["enabled"].astype(bool)
        assert hq["accept"][eq].mean() > 0.9
        assert hq["accept"][eq].mean() > hu["accept"][eu].mean() + 0.05


def test_disabled_points_and_thresholds(pe):
    comp = _sab_comps(pe)[0]
    ne = len(pe.array(comp, "egrid", np.float64))
    kn = LR.reference_knots(W.PE293, comp, "quantile")
    allowed = np.zeros(ne, dtype=np.uint8)
    allowed[::2] = 1
    hdr = pe.build_proposal(comp, kn, allowed=allowed, min_accept=0.0)[0]
    assert not np.any(hdr["enabled"][1::2])
    hdr2 = pe.build_proposal(comp, kn, min_accept=1.01)[0]
    assert not np.any(hdr2["enabled"])


def test_oracle_disabled_proposal_is_the_plain_sampler(pe):
    """With every egrid point disabled the learned branch is never taken: the
    oracle reproduces the plain sampler draw for draw."""
    m = HostMaterial(bundle_path(W.PE293))
    e = W.loguniform_energies(20000, 1e-4, 1.0, 3)
    ef0, mu0, _, nd0 = m.scatter(e, 5)
    for comp in _sab_comps(m):
        kn = LR.reference_knots(W.PE293, comp, "quantile")
        m.set_proposal(comp, m.build_proposal(comp, kn, min_accept=2.0))
    ef1, mu1, _, nd1 = m.scatter(e, 5)
    np.testing.assert_array_equal(ef0, ef1)
    np.testing.assert_array_equal(mu0, mu1)
    np.testing.assert_array_equal(nd0, nd1)


@pytest.mark.parametrize("kind", ["quantile", "random"])
@pytest.mark.parametrize("e0", [0.001, 0.0253, 0.3])
def test_oracle_learned_distribution_matches_plain(kind, e0):
    """Oracle with the learned proposal vs oracle plain, independent streams:
    two-sample chi-square on (log E'/E, mu) and KS on E' and mu."""
    from scipy.stats import chi2, ks_2samp
    m = HostMaterial(bundle_path(W.PE293))
    n = 300000
    e = np.full(n, e0)
    ef0, mu0, st0, _ = m.scatter(e, 11)
    for comp in _sab_comps(m):
        ne = len(m.array(comp, "egrid", np.float64))
        kn = _random_knots(ne, 5 + comp) if kind == "random" else LR.reference_knots(W.PE293, comp, kind)
        m.set_proposal(comp, m.build_proposal(comp, kn, min_accept=0.0))
    ef1, mu1, st1, _ = m.scatter(e, 12)
    assert np.all(st0 == 0) and np.all(st1 == 0)
    la, lb = np.log(np.maximum(ef0, 1e-30) / e0), np.log(np.maximum(ef1, 1e-30) / e0)
    edges = np.unique(np.quantile(np.concatenate([la, lb]), np.linspace(0, 1, 31)))
    ha, _, _ = np.histogram2d(la, mu0, bins=[edges, np.linspace(-1, 1, 21)])
    hb, _, _ = np.histogram2d(lb, mu1, bins=[edges, np.linspace(-1, 1, 21)])
    ha, hb = ha.ravel(), hb.ravel()
    keep = (ha + hb) > 0
    stat = np.sum((ha[keep] - hb[keep]) ** 2 / (ha[keep] + hb[keep]))
    p = chi2.sf(stat, int(keep.sum()) - 1)
    alpha = 1e-3
    assert p > alpha, (stat, p)
    assert ks_2samp(ef0, ef1).pvalue > alpha
    assert ks_2samp(mu0, mu1).pvalue > alpha


def test_energy_grid_bucket_index_equals_binary_search(pe):
    """The GPU's energy-grid search (bucket of E's bit pattern, then a short
    scan; ncgb_device.cuh egridUpper / egridUpperF) gives std::upper_bound's
    index for every energy, in FP64 and FP32."""
    r = np.random.default_rng(3)
    for comp in _sab_comps(pe):
        eg = pe.array(comp, "egrid", np.float64)
        egf = pe.array(comp, "egrid_f", np.float32)
        bk = pe.array(comp, "ebkt", np.int32)
        bkf = pe.array(comp, "ebkt_f", np.int32)
        k0 = int(pe.scalar(comp, "ebkt_kmin"))
        k0f = int(pe.scalar(comp, "ebkt_f_kmin"))
        e = np.concatenate([np.exp(r.uniform(np.log(1e-9), np.log(1e3), 200000)), eg, np.nextafter(eg, 0),
                            np.nextafter(eg, np.inf), [0.0, np.inf]])

        def upper64(x):
            b = np.array([x]).view(np.int64)[0]
            k = (b >> 49) - k0
            if k < 0:
                return 0
            if k >= len(bk) - 1:
                return len(eg)
            i, hi = bk[k], bk[k + 1]
            while i < hi and not (b < eg[i:i + 1].view(np.int64)[0]):
                i += 1
            return i

        def upper32(x):
            b = np.array([x], dtype=np.float32).view(np.int32)[0]
            k = (b >> 20) - k0f
            if k < 0:
                return 0
            if k >= len(bkf) - 1:
                return len(egf)
            i, hi = bkf[k], bkf[k + 1]
            while i < hi and not (b < egf[i:i + 1].view(np.int32)[0]):
                i += 1
            return i
        sub = e[::50]
        got = np.array([upper64(x) for x in sub])
        np.testing.assert_array_equal(got, np.searchsorted(eg, sub, side="right"))
        subf = sub.astype(np.float32)
        gotf = np.array([upper32(x) for x in subf])
        np.testing.assert_array_equal(gotf, np.searchsorted(egf, subf, side="right"))
