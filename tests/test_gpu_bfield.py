"""A perpendicular magnetic field: the complex Hamiltonian (generateCpxH with
Peierls phases) against fixtures generated by the reference's own code, and
against the oracle.

The complex matrix must equal the reference's to rounding (CUDA's cos/sin
against glibc's: 1e-15 of the largest entry). Moments come from the FP32
complex row-block recursion and are compared at the FP32 bar, 1e-4 of the
largest moment.
"""
import os

import numpy as np
import pytest

import leo2d_gb300 as L
from oracle import oracle
from tests._golden import BFIELD_CASES, GOLDEN, e2e_text, load, parse_in

pytestmark = pytest.mark.gpu
FP32_RTOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    with L.Context(0) as c:
        yield c


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("name", BFIELD_CASES)
def test_complex_csr_matches_reference(ctx, name):
    gold = load(name)
    g, kv = parse_in(name)
    csr = ctx.build_csr(ctx.prepare(g), keep_zeros=True)
    rp, col, val = csr.download()
    im = csr.download_imag()
    assert np.array_equal(rp, gold["rowptr"].astype(np.int64))
    assert np.array_equal(col, gold["col"])
    scale = np.abs(gold["val"]).max()
    np.testing.assert_allclose(val, gold["val"], rtol=0, atol=1e-15 * scale)
    np.testing.assert_allclose(im, gold["val_im"], rtol=0, atol=1e-15 * scale)


@pytest.mark.parametrize("name", BFIELD_CASES)
def test_complex_moments_match_reference(ctx, name):
    gold = load(name)
    g, kv = parse_in(name)
    meta = gold["meta"]
    P, trace = int(meta[5]), int(meta[6])
    csr = ctx.build_csr(ctx.prepare(g), keep_zeros=True)
    if trace == 1:
        R = int(meta[4])
        vec = oracle.reference_gaussian(R, csr.n)
        mu = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_HOST, precision=L.FP32), vec)
    else:
        tg = gold["targets"].astype(np.int64)
        mu = csr.kpm_ldos(L.kpm_cfg(P, precision=L.FP32), tg)
    ref = gold["moments"].reshape(mu.shape)
    assert _rel(mu, ref) < FP32_RTOL


def test_phase_vectors_and_rescale(ctx):
    """Random-phase (complex) start vectors on a larger flake after a
    Gershgorin rescale, against the oracle's complex recursion."""
    g = L.make_geom(model=L.MODEL_SIMPLE, size=40, max_R=70.0, angles_deg=(0.0, 2.0), energy_rescale=1.0,
                    b_field=300.0)
    csr = ctx.build_csr(ctx.prepare(g))
    lo, hi = csr.bounds()
    a, b = 1.01 * (hi - lo) / 2, (hi + lo) / 2
    csr.rescale(a, -b)
    rp, col, val = csr.download()
    im = csr.download_imag()
    # the rescale divides the imaginary parts too; |H_ij| bounds the spectrum
    assert np.abs(im).max() > 0.05 * np.abs(val).max()
    P, R, seed = 96, 16, 11
    mu = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_PHASE, precision=L.FP32, seed=seed))
    re_v, im_v = oracle.phase_vectors(seed, 0, R, csr.n)
    ref = oracle.kpm_trace_cpx_doubling(rp, col, val, im, re_v, im_v, P)
    assert _rel(mu, ref) < FP32_RTOL
    # the same flake without the field gives other moments
    g0 = L.make_geom(model=L.MODEL_SIMPLE, size=40, max_R=70.0, angles_deg=(0.0, 2.0), energy_rescale=1.0)
    c0 = ctx.build_csr(ctx.prepare(g0))
    c0.rescale(a, -b)
    mu0 = c0.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_PHASE, precision=L.FP32, seed=seed))
    assert _rel(mu0, mu) > 1e-3


def test_complex_limits(ctx):
    g = L.make_geom(size=8, angles_deg=(0.0, 5.0), energy_rescale=13.0, b_field=100.0)
    gp = ctx.prepare(g)
    csr = ctx.build_csr(gp)
    with pytest.raises(L.Leo2dError, match="FP32"):
        csr.kpm_dos(L.kpm_cfg(16, R=2, precision=L.FP64))
    with pytest.raises(L.Leo2dError, match="complex"):
        ctx.build_csr(gp, with_dx=True)
    with pytest.raises(L.Leo2dError, match="real"):
        L.Batch(ctx, [csr], L.kpm_cfg(16, R=2))
    gr = L.make_geom(size=8, angles_deg=(0.0, 5.0), energy_rescale=13.0)
    with pytest.raises(L.Leo2dError, match="real"):
        ctx.build_csr(ctx.prepare(gr)).download_imag()


def _numbers(text):
    out = []
    for tok in text.replace(",", " ").split():
        try:
            out.append(float(tok))
        except ValueError:
            out.append(tok)
    return out


@pytest.mark.parametrize("name", BFIELD_CASES)
def test_driver_files(tmp_path, name):
    """`leo2d` on the field inputs: the .cheb (FP32 recursion: 1e-4 of the
    largest DOS value) and the complex _matrix.dat (re, im per entry)."""
    L.run_input(os.path.join(GOLDEN, "inputs", name + ".in"), tmp_path)
    ours = _numbers((tmp_path / (name + ".cheb")).read_text())
    ref = _numbers(e2e_text(name, ".cheb"))
    assert len(ours) == len(ref)
    fo = np.array([x for x in ours if isinstance(x, float)])
    fr = np.array([x for x in ref if isinstance(x, float)])
    assert [x for x in ours if not isinstance(x, float)] == [x for x in ref if not isinstance(x, float)]
    assert np.abs(fo - fr).max() <= 1e-4 * np.abs(fr).max() + 2e-6
    mo = _numbers((tmp_path / (name + "_matrix.dat")).read_text())
    mr = _numbers(e2e_text(name, "_matrix.dat"))
    assert len(mo) == len(mr)
    np.testing.assert_allclose(np.array(mo, float), np.array(mr, float), rtol=1e-5, atol=1e-6)
