"""Vacancies: the matrix of the reference's vacancy solvers, built on the device
from the full matrix (leo2d_csr_remove_orbitals), against fixtures generated
from the reference's own generateRealH with a vacancy list and against the
oracle's restatement of its relabelling.

Row pointers and columns must be identical to the reference's; values carry
the full matrix's tolerance (1e-12: CUDA's and glibc's transcendental
functions). Moments: FP64 recursion to 1e-10 of the reference's, the FP32
Kubo recursion at the FP32 bar (1e-4 of the largest moment).
"""
import numpy as np
import pytest

import leo2d_gb300 as L
from oracle import oracle
from tests._golden import VAC_CASES, load, parse_in, vac_base

pytestmark = pytest.mark.gpu
VAL_TOL = 1e-12


@pytest.fixture(scope="module")
def ctx():
    with L.Context(0) as c:
        yield c


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def _reduced(ctx, name):
    gold = load(name)
    g, kv = parse_in(vac_base(name))
    full = ctx.build_csr(ctx.prepare(g), keep_zeros=True, with_dx=True)
    vac = gold["vacancies"].astype(np.int64)
    return gold, full, full.remove_orbitals(vac), vac


@pytest.mark.parametrize("name", VAC_CASES)
def test_vacancy_csr_matches_reference(ctx, name):
    gold, full, csr, vac = _reduced(ctx, name)
    assert csr.n == int(gold["n_kept"][0]) and csr.nnz == int(gold["meta"][1])
    rp, col, val, dx, dy = csr.download(dx=True)
    assert np.array_equal(rp, gold["rowptr"].astype(np.int64))
    assert np.array_equal(col, gold["col"])
    np.testing.assert_allclose(val, gold["val"], rtol=0, atol=VAL_TOL)
    if "val_dx" in gold:
        np.testing.assert_allclose(dx, gold["val_dx"], rtol=0, atol=VAL_TOL * 100)
        np.testing.assert_allclose(dy, gold["val_dy"], rtol=0, atol=VAL_TOL * 100)
    # the device compaction equals the oracle's on the device's own full matrix, bit for bit
    frp, fcol, fval, fdx, fdy = full.download(dx=True)
    orp, ocol, (oval, odx, ody) = oracle.remove_orbitals(frp, fcol, [fval, fdx, fdy], vac)
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    assert np.array_equal(val, oval) and np.array_equal(dx, odx) and np.array_equal(dy, ody)
    # positions and grid indices of the kept orbitals
    grid, pos = csr.geometry()
    fgrid, fpos = full.geometry()
    keep = np.ones(full.n, bool)
    keep[vac[(vac >= 0) & (vac < full.n)]] = False
    assert np.array_equal(grid.reshape(-1, 4), fgrid.reshape(-1, 4)[keep])
    assert np.array_equal(pos.reshape(-1, 3), fpos.reshape(-1, 3)[keep])


@pytest.mark.parametrize("name", VAC_CASES)
def test_vacancy_moments_match_reference(ctx, name):
    gold, full, csr, vac = _reduced(ctx, name)
    meta = gold["meta"]
    P, trace, observable = int(meta[5]), int(meta[6]), int(meta[7])
    tg = gold["targets"].astype(np.int64)
    rows = L.vacancy_rows(full.n, vac, tg)
    if observable == 1:
        C = csr.kpm_cond(L.kpm_cfg(P), rows)
        ref = gold["cond_moments"].reshape(len(tg), P, P)
        assert _rel(C[0, :, :P - 1], ref[0, :, :P - 1]) < 1e-4
    elif trace == 1:
        R = int(meta[4])
        vec = oracle.reference_gaussian(R, csr.n)
        mu = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_HOST, precision=L.FP64), vec)
        assert _rel(mu, gold["moments"].reshape(R, P)) < 1e-10
    else:
        mu = csr.kpm_ldos(L.kpm_cfg(P, precision=L.FP64), rows)
        np.testing.assert_allclose(mu, gold["moments"].reshape(len(tg), P), rtol=0, atol=1e-11)


def test_vacancy_edge_lists(ctx):
    """No vacancies gives the same matrix; duplicates and out-of-range entries
    remove nothing more; removing every orbital is an error."""
    g = L.make_geom(size=7, angles_deg=(0.0, 6.0), energy_rescale=13.0)
    full = ctx.build_csr(ctx.prepare(g))
    rp, col, val = full.download()
    same = full.remove_orbitals([])
    for a, b in zip(same.download(), (rp, col, val)):
        assert np.array_equal(a, b)
    a = full.remove_orbitals([3, 3, -1, full.n, 10 ** 9, full.n - 1])
    b = full.remove_orbitals([full.n - 1, 3])
    assert a.n == full.n - 2
    for x, y in zip(a.download(), b.download()):
        assert np.array_equal(x, y)
    assert list(L.vacancy_rows(full.n, [3, 3, -1, full.n - 1], [0, 2, 4, full.n - 2])) == [0, 2, 3, full.n - 3]
    with pytest.raises(L.Leo2dError, match="every orbital"):
        full.remove_orbitals(np.arange(full.n))


def test_vacancies_in_a_field(ctx):
    """A complex (magnetic-field) matrix keeps its imaginary parts through the compaction."""
    g = L.make_geom(size=9, angles_deg=(0.0, 4.0), energy_rescale=13.0, b_field=200.0)
    full = ctx.build_csr(ctx.prepare(g), keep_zeros=True)
    vac = np.array([0, 5, 6, 77, full.n - 1])
    red = full.remove_orbitals(vac)
    frp, fcol, fval = full.download()
    orp, ocol, (ore, oim) = oracle.remove_orbitals(frp, fcol, [fval, full.download_imag()], vac)
    rp, col, val = red.download()
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    assert np.array_equal(val, ore) and np.array_equal(red.download_imag(), oim)
    P = 64
    rows = L.vacancy_rows(full.n, vac, [10, 40])
    mu = red.kpm_ldos(L.kpm_cfg(P, precision=L.FP32), rows)
    ref = oracle.kpm_ldos_cpx(orp, ocol, ore, oim, rows, P)
    assert _rel(mu, ref) < 1e-4


def test_vacancy_flake_on_the_row_block_paths(ctx):
    """A larger flake with 2 % vacancies: the locality ordering and the 8-row
    blocks take the kept orbitals' positions; DOS moments against the FP64 oracle
    and the Kubo trace against the stored-dxH path."""
    g = L.make_geom(model=L.MODEL_SIMPLE, size=30, angles_deg=(0.0, 2.5), energy_rescale=1.0)
    full = ctx.build_csr(ctx.prepare(g), with_dx=True)
    rng = np.random.default_rng(5)
    vac = rng.choice(full.n, size=full.n // 50, replace=False)
    csr = full.remove_orbitals(vac)
    lo, hi = csr.bounds()
    csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
    ctx.set_option("reorder", 1)
    try:
        cfg = L.kpm_cfg(64, R=16, seed=4, block=32)
        mu = csr.kpm_dos(cfg)
        assert csr.rt_info()[0] == (csr.n + 7) // 8  # the 8-row tensor-core step ran
        rp, col, val, dx, dy = csr.download(dx=True)
        re, im = oracle.phase_vectors(4, 0, 16, csr.n)
        ref = (oracle.kpm_trace(rp, col, val, re, 64, literal=False) +
               oracle.kpm_trace(rp, col, val, im, 64, literal=False))
        assert _rel(mu, ref) < 1e-4
        kcfg = L.kpm_cfg(24, R=16, kind=L.VEC_PHASE, seed=2)
        fly = csr.kpm_cond(kcfg)
        ctx.set_option("kubo_velocity", 0)
        stored = csr.kpm_cond(kcfg)
    finally:
        ctx.set_option("kubo_velocity", -1)
        ctx.set_option("reorder", -1)
    assert _rel(fly, stored) < 2e-5
