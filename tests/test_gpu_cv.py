"""What the trained network gains: the learned control variate against the
same estimators without it, on a flake whose twist is not in the training set.

Training: site-resolved moments (first 256, exact unit-vector recursions) of
the bulk orbitals (more than 40 A inside the edge) of three flakes at 1.2, 2.0
and 3.0 degrees; the target flake is at 1.6 degrees. All four share one
spectral scale, so their moments are comparable. Exact moments of every
orbital of the target are the truth. Orbitals near the edge are not a function
of the stacking features (their moments vary 1000x more), so the site
estimator is compared on the bulk stratum, where the network applies.

(a) site sampling of the bulk stratum, S orbitals: N_b mean_s mu(s) vs
    sum_b f + N_b mean_s (mu(s) - f(s)); for moments 16..127 the network must
    cut the error variance at least 3x, and the estimate stays unbiased;
(b) the reference's Gaussian-vector trace (real N(0,1) vectors): <r|T|r> vs
    sum_i f(i) + <r|T|r> - sum_i r_i^2 f(i); the diagonal part of the variance
    (2 sum_i T_ii^2 of 2 ||T||_F^2) goes. mu_0 is all diagonal (T_0 = I): its
    variance must drop at least 100x; mu_2 (about half diagonal): by 20 %;
(c) leo2d_kpm_dos_cv reproduces (a)'s estimator for its own site draw.
"""
import numpy as np
import pytest

import leo2d_gb300 as L

pytestmark = pytest.mark.gpu
PC = 256  # moments the network predicts


EDGE = 40.0  # A


def _flake(ctx, twist, radius):
    size = int(radius / 2.46 * 1.6) + 4
    g = L.make_geom(model=L.MODEL_SIMPLE, size=size, max_R=radius, angles_deg=(0.0, twist), energy_rescale=1.0)
    return ctx.build_csr(ctx.prepare(g)), radius


def _bulk(csr, radius):
    _, pos = csr.geometry()
    p = pos.reshape(-1, 3)
    return np.hypot(p[:, 0], p[:, 1]) < radius - EDGE


@pytest.fixture(scope="module")
def setup():
    ctx = L.Context(0)
    train = [(_flake(ctx, t, 120.0), t) for t in (1.2, 2.0, 3.0)]
    target_twist = 1.6
    target, t_radius = _flake(ctx, target_twist, 140.0)
    a = 1.01 * max(max(abs(lo), abs(hi)) for lo, hi in (c.bounds() for (c, _), _ in train + [((target, 0), 0)]))
    for (c, _), _ in train + [((target, 0), 0)]:
        c.rescale(a, 0.0)
    cfg = L.kpm_cfg(PC, R=1)
    xs, ts = [], []
    for (c, radius), t in train:
        sel = np.nonzero(_bulk(c, radius))[0]
        xs.append(c.site_features(t)[sel])
        ts.append(c.kpm_ldos(cfg, sel))
    x = np.concatenate(xs)
    t = np.concatenate(ts).astype(np.float32)
    mlp = L.Mlp(ctx, seed=0)
    mlp.train(x, t, steps=2000, batch=4096, lr=2e-3, seed=3)
    mu_sites = target.kpm_ldos(cfg, np.arange(target.n))  # exact, every orbital
    f = mlp.predict(target.site_features(target_twist)).astype(np.float64)
    target.bulk = _bulk(target, t_radius)
    yield ctx, mlp, target, target_twist, mu_sites, f
    mlp.close()
    ctx.close()


def test_site_sampling_gain(setup):
    ctx, mlp, target, twist, mu, f = setup
    idx = np.nonzero(target.bulk)[0]
    nb = len(idx)
    truth = mu[idx].sum(axis=0)
    F = f[idx].sum(axis=0)
    rng = np.random.default_rng(0)
    S, trials = 128, 300
    e_plain, e_cv = [], []
    for _ in range(trials):
        s = idx[rng.integers(0, nb, S)]
        e_plain.append(nb * mu[s].mean(axis=0) - truth)
        e_cv.append(F + nb * (mu[s] - f[s]).mean(axis=0) - truth)
    e_plain, e_cv = np.array(e_plain), np.array(e_cv)
    band = slice(16, 128)
    v_plain = (e_plain[:, band] ** 2).mean()
    v_cv = (e_cv[:, band] ** 2).mean()
    assert v_cv < v_plain / 3, (v_plain, v_cv)
    # unbiased: the mean error is within 4 standard errors for every moment
    se = e_cv.std(axis=0) / np.sqrt(trials)
    assert np.all(np.abs(e_cv.mean(axis=0)) <= 4 * se + 1e-9 * np.abs(truth).max())


def test_gaussian_trace_gain(setup):
    ctx, mlp, target, twist, mu, f = setup
    n = target.n
    truth = mu.sum(axis=0)
    F = f.sum(axis=0)
    rng = np.random.default_rng(1)
    R = 64
    r = rng.normal(size=(R, n))
    per_vec = target.kpm_dos(L.kpm_cfg(PC, R=R, kind=L.VEC_HOST), r)
    diag = (r ** 2) @ f  # sum_i r_i^2 f(i) per vector
    e_plain = per_vec - truth
    e_cv = F + (per_vec - diag) - truth
    v_plain = (e_plain ** 2).mean(axis=0)
    v_cv = (e_cv ** 2).mean(axis=0)
    assert v_cv[0] < v_plain[0] / 100, (v_plain[0], v_cv[0])
    assert v_cv[2] < 0.8 * v_plain[2], (v_plain[2], v_cv[2])


def test_cv_entry_point_matches_formula(setup):
    ctx, mlp, target, twist, mu, f = setup
    cfg = L.kpm_cfg(PC, R=2, seed=9)
    got, parts = target.kpm_dos_cv(mlp, cfg, twist, num_sites=64, site_seed=5, parts=True)
    F, corr, phase = parts
    np.testing.assert_allclose(F, f.sum(axis=0), rtol=1e-5, atol=1e-5 * np.abs(F).max())
    ph = target.kpm_dos(cfg).mean(axis=0)
    np.testing.assert_allclose(phase[:PC], ph, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(got, F + corr, rtol=1e-12, atol=1e-12)
    w = np.full(PC, 0.25)
    mixed = target.kpm_dos_cv(mlp, cfg, twist, num_sites=64, site_seed=5, weights=w)
    np.testing.assert_allclose(mixed, 0.25 * (F + corr) + 0.75 * ph, rtol=1e-9, atol=1e-9 * np.abs(ph).max())
