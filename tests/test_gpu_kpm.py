"""GPU KPM recursion against the reference's moments and the FP64 oracle.

FP64 mode reproduces the reference's moments (golden fixtures, same Gaussian
vectors) to 1e-10 relative. The FP32 recursion (FP64 moment sums) is held to a
relative tolerance of 1e-4 of the largest moment against the FP64 oracle of the
same recursion on the same vectors, at these sizes and orders.
"""
import numpy as np
import pytest

import leo2d_gb300 as L
from oracle import oracle
from tests._golden import CASES, load, parse_in

pytestmark = pytest.mark.gpu
FP64_RTOL = 1e-10
FP32_RTOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    with L.Context(0) as c:
        yield c


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("name", [c for c in CASES if "cond" not in c])
def test_golden_moments(ctx, name):
    gold = load(name)
    g, kv = parse_in(name)
    meta = gold["meta"]
    P, trace = int(meta[5]), int(meta[6])
    csr = ctx.build_csr(ctx.prepare(g), keep_zeros=True)
    if trace:
        R = int(meta[4])
        vec = oracle.reference_gaussian(R, csr.n)
        ref = gold["moments"].reshape(R, P)
        mu = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_HOST, precision=L.FP64), vec)
        assert _rel(mu, ref) < FP64_RTOL
        mu32 = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_HOST, precision=L.FP32), vec)
        assert _rel(mu32, ref) < FP32_RTOL
        dos, E = ctx.dos_transform(mu, P, g.energy_rescale, g.energy_shift, 1.0 / csr.n)
        np.testing.assert_allclose(dos, gold["dos"], rtol=1e-8, atol=1e-10 * np.abs(gold["dos"]).max())
    else:
        tg = gold["targets"].astype(np.int64)
        ref = gold["moments"].reshape(len(tg), P)
        mu = csr.kpm_ldos(L.kpm_cfg(P, precision=L.FP64), tg)
        np.testing.assert_allclose(mu, ref, rtol=0, atol=1e-11)
        mu32 = csr.kpm_ldos(L.kpm_cfg(P, precision=L.FP32), tg)
        np.testing.assert_allclose(mu32, ref, rtol=0, atol=1e-5)
        dos = np.stack([ctx.dos_transform(m, P, g.energy_rescale, g.energy_shift)[0] for m in mu])
        np.testing.assert_allclose(dos.ravel(), gold["dos"], rtol=1e-8,
                                   atol=1e-10 * np.abs(gold["dos"]).max())


@pytest.fixture(scope="module")
def flake(ctx):
    g = L.make_geom(model=L.MODEL_SIMPLE, size=22, angles_deg=(0.0, 3.0), energy_rescale=1.0)
    gp = ctx.prepare(g)
    csr = ctx.build_csr(gp)
    lo, hi = csr.bounds()
    a, b = 1.01 * (hi - lo) / 2, (hi + lo) / 2
    csr.rescale(a, -b)
    rp, col, val = csr.download()
    return csr, rp, col, val


def _with_options(ctx, opts, fn):
    for k, v in opts.items():
        ctx.set_option(k, v)
    try:
        return fn()
    finally:
        for k, v in {"step_kernel": -1, "reorder": -1, "tile_warps": 0, "tile_chunk": 4,
                     "tile_stages": 2, "reorder_patch_dA": 0}.items():
            ctx.set_option(k, v)


@pytest.mark.parametrize("opts", [{"step_kernel": 0}, {"step_kernel": 1},
                                  {"step_kernel": 0, "reorder": 1},
                                  {"step_kernel": 0, "reorder": 1, "tile_warps": 24},
                                  {"step_kernel": 1, "reorder": 1},
                                  {"step_kernel": 0, "tile_stages": 4, "tile_chunk": 1}])
@pytest.mark.parametrize("cols", [8, 16, 32, 64, 128])
@pytest.mark.parametrize("rows", [1, 3, 8])
def test_block_shapes_fp32(ctx, flake, opts, cols, rows):
    csr, rp, col, val = flake
    P, R = 128, 6
    vec = np.random.default_rng(cols * 10 + rows).standard_normal((R, csr.n))
    ref = oracle.kpm_trace(rp, col, val, vec, P, literal=False)
    mu = _with_options(ctx, opts, lambda: csr.kpm_dos(
        L.kpm_cfg(P, R=R, kind=L.VEC_HOST, block=cols, rows_per_warp=rows), vec))
    assert _rel(mu, ref) < FP32_RTOL


@pytest.mark.parametrize("opts", [{"step_kernel": 0}, {"step_kernel": 1},
                                  {"step_kernel": 0, "reorder": 1, "tile_warps": 24}])
@pytest.mark.parametrize("cols", [8, 16, 32, 64])
def test_block_shapes_fp64(ctx, flake, opts, cols):
    csr, rp, col, val = flake
    P, R = 96, 5
    vec = np.random.default_rng(cols).standard_normal((R, csr.n))
    ref = oracle.kpm_trace(rp, col, val, vec, P, literal=False)
    mu = _with_options(ctx, opts, lambda: csr.kpm_dos(
        L.kpm_cfg(P, R=R, kind=L.VEC_HOST, precision=L.FP64, block=cols), vec))
    assert _rel(mu, ref) < 1e-12


@pytest.mark.parametrize("patch_dA", [60, 160, 400])
def test_reordered_phase_and_ldos(ctx, flake, patch_dA):
    csr, rp, col, val = flake
    P, R, seed = 64, 3, 77
    ref = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_PHASE, precision=L.FP64, seed=seed))
    opts = {"reorder": 1, "reorder_patch_dA": patch_dA}
    mu = _with_options(ctx, opts, lambda: csr.kpm_dos(
        L.kpm_cfg(P, R=R, kind=L.VEC_PHASE, precision=L.FP64, seed=seed)))
    assert _rel(mu, ref) < 1e-12
    tg = [0, 5, csr.n // 2, csr.n - 1]
    lref = oracle.kpm_ldos(rp, col, val, tg, P)
    ld = _with_options(ctx, opts, lambda: csr.kpm_ldos(L.kpm_cfg(P, precision=L.FP64), tg))
    np.testing.assert_allclose(ld, lref, rtol=0, atol=1e-11)


def test_phase_vectors_match_oracle_generator(flake):
    csr, rp, col, val = flake
    P, R, seed = 64, 5, 1234
    mu = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_PHASE, precision=L.FP64, seed=seed, first_vector=7))
    re, im = oracle.phase_vectors(seed, 7, R, csr.n)
    ref = (oracle.kpm_trace(rp, col, val, re, P, literal=False) +
           oracle.kpm_trace(rp, col, val, im, P, literal=False))
    assert _rel(mu, ref) < 1e-9
    # |r_i| = 1 for every random-phase vector: mu_0 = n (to FP32 rounding of cos/sin)
    assert np.allclose(mu[:, 0], csr.n, rtol=1e-6)
    # extending a run reproduces the same vectors
    mu2 = csr.kpm_dos(L.kpm_cfg(P, R=2, kind=L.VEC_PHASE, precision=L.FP64, seed=seed, first_vector=10))
    np.testing.assert_allclose(mu2, mu[3:5], rtol=1e-13, atol=1e-9)


def test_fp32_phase_against_fp64(flake):
    csr, rp, col, val = flake
    P, R = 512, 32
    mu64 = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_PHASE, precision=L.FP64, seed=3))
    mu32 = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_PHASE, precision=L.FP32, seed=3))
    assert _rel(mu32, mu64) < FP32_RTOL


def test_gaussian_device_vectors(flake):
    csr, rp, col, val = flake
    mu = csr.kpm_dos(L.kpm_cfg(32, R=64, kind=L.VEC_GAUSSIAN, precision=L.FP64, seed=5))
    # E[mu_0] = n for N(0,1) entries
    assert abs(mu[:, 0].mean() / csr.n - 1.0) < 0.05


def test_reconstruct_matches_oracle(ctx, flake):
    csr, rp, col, val = flake
    P = 256
    mu = csr.kpm_dos(L.kpm_cfg(P, R=4, kind=L.VEC_PHASE, precision=L.FP64, seed=9)).mean(axis=0)
    E = np.linspace(-1.2, 1.2, 4001)
    d = ctx.dos_reconstruct(mu, E, 1.0, 0.0, 1.0 / csr.n)
    r = oracle.dos_reconstruct(mu, E, 1.0, 0.0, 1.0 / csr.n)
    np.testing.assert_allclose(d, r, rtol=1e-9, atol=1e-12)
    assert d[0] == 0.0 and d[-1] == 0.0


def test_bad_arguments(flake):
    csr = flake[0]
    with pytest.raises(L.Leo2dError, match="multiple of 4"):
        csr.kpm_dos(L.kpm_cfg(30, R=1))
    with pytest.raises(L.Leo2dError, match="out of range"):
        csr.kpm_ldos(L.kpm_cfg(32), [csr.n])
    with pytest.raises(L.Leo2dError, match="block width"):
        csr.kpm_dos(L.kpm_cfg(32, R=1, block=48))


def test_autotune_picks_a_supported_shape(ctx, flake):
    csr, rp, col, val = flake
    cfg = L.kpm_cfg(64, R=10, kind=L.VEC_PHASE, seed=2)
    block, rows = csr.autotune(cfg)
    assert block in (8, 16, 32, 64, 128) and rows in (0, 2)
    ref = csr.kpm_dos(L.kpm_cfg(64, R=10, kind=L.VEC_PHASE, precision=L.FP64, seed=2))
    mu = csr.kpm_dos(cfg)  # block = 0 -> the tuned width
    assert _rel(mu, ref) < FP32_RTOL
