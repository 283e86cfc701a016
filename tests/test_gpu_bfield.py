"""Complex Hamiltonians (generateCpxH): a perpendicular magnetic field (Peierls
phases on a flake) and k-sampled periodic supercells (Bloch phases per image),
against fixtures generated by the reference's own code, and against the oracle.

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
from tests._golden import BFIELD_CASES, COMPLEX_CASES, GOLDEN, e2e_text, load, parse_in

pytestmark = pytest.mark.gpu
FP32_RTOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    with L.Context(0) as c:
        yield c


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("name", COMPLEX_CASES)
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


@pytest.mark.parametrize("kernel", [-1, 5])
@pytest.mark.parametrize("name", COMPLEX_CASES)
def test_complex_moments_match_reference(ctx, name, kernel):
    """The reference's complex moments (fields on flakes and supercells, k points),
    with the default step and with the complex 8-row tensor-core step."""
    gold = load(name)
    g, kv = parse_in(name)
    meta = gold["meta"]
    P, trace = int(meta[5]), int(meta[6])
    csr = ctx.build_csr(ctx.prepare(g), keep_zeros=True)
    ctx.set_option("step_kernel", kernel)
    try:
        if trace == 1:
            R = int(meta[4])
            vec = oracle.reference_gaussian(R, csr.n)
            mu = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_HOST, precision=L.FP32), vec)
        else:
            tg = gold["targets"].astype(np.int64)
            mu = csr.kpm_ldos(L.kpm_cfg(P, precision=L.FP32), tg)
        if kernel == 5:
            assert csr.rt_info()[0] == (csr.n + 7) // 8
    finally:
        ctx.set_option("step_kernel", -1)
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


def test_bloch_supercell_on_a_k_grid(ctx):
    """A (4,5) twisted supercell at the points of a 2 x 3 k grid: the device's
    image-resolved Bloch sums against the oracle's, and the complex recursion
    (random-phase vectors) against the oracle's; k = 0 gives the real matrix."""
    g = ctx.prepare(L.make_geom(boundary_condition=1, supercell_mn=(4, 5), size=16, energy_rescale=13.0))
    ks = L.k_grid(g, 2, 3)
    assert ks.shape == (6, 2) and np.all(ks[0] == 0.0)
    b1 = ks[3]  # k1 = 1: half of the first reciprocal vector
    a = np.array(g.supercell)
    assert abs(2 * b1 @ a[0] - 2 * np.pi) < 1e-9 and abs(b1 @ a[1]) < 1e-9
    real = ctx.build_csr(g)
    assert np.abs(real.download()[2]).max() > 0
    with pytest.raises(L.Leo2dError, match="real"):
        real.download_imag()
    for k in ks[1:3]:
        gk = L.make_geom(boundary_condition=1, supercell_mn=(4, 5), size=16, energy_rescale=13.0, k_vec=k)
        gk = ctx.prepare(gk)
        csr = ctx.build_csr(gk, keep_zeros=True)
        rp, col, re = csr.download()
        im = csr.download_imag()
        b = oracle.Built(gk)
        ore, oim = b.bloch(*k)
        assert np.array_equal(rp, b.rowptr) and np.array_equal(col, b.col)
        scale = np.abs(ore).max()
        np.testing.assert_allclose(re, ore, rtol=0, atol=4e-15 * scale)
        np.testing.assert_allclose(im, oim, rtol=0, atol=4e-15 * scale)
        P, R, seed = 64, 16, 3
        mu = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_PHASE, precision=L.FP32, seed=seed))
        vre, vim = oracle.phase_vectors(seed, 0, R, csr.n)
        ref = oracle.kpm_trace_cpx_doubling(rp, col, ore, oim, vre, vim, P)
        assert _rel(mu, ref) < FP32_RTOL


def test_bloch_phase_on_a_flake_is_a_gauge(ctx):
    """On a flake, k.(r_col - r_row) phases are a diagonal unitary change of basis:
    local DOS moments are unchanged (to FP32 rounding) and the matrix entries keep
    their moduli."""
    g0 = L.make_geom(model=L.MODEL_SIMPLE, size=20, angles_deg=(0.0, 3.0), energy_rescale=13.0)
    gk = L.make_geom(model=L.MODEL_SIMPLE, size=20, angles_deg=(0.0, 3.0), energy_rescale=13.0, k_vec=(0.31, -0.17))
    c0 = ctx.build_csr(ctx.prepare(g0), keep_zeros=True)
    ck = ctx.build_csr(ctx.prepare(gk), keep_zeros=True)
    rp0, col0, v0 = c0.download()
    rpk, colk, vk = ck.download()
    imk = ck.download_imag()
    assert np.array_equal(rp0, rpk) and np.array_equal(col0, colk)
    np.testing.assert_allclose(np.hypot(vk, imk), np.abs(v0), rtol=1e-14, atol=1e-16)
    assert np.abs(imk).max() > 0.1 * np.abs(v0).max()
    targets = np.array([5, 100, 333])
    cfg = L.kpm_cfg(64, precision=L.FP32)
    assert _rel(ck.kpm_ldos(cfg, targets), c0.kpm_ldos(cfg, targets)) < FP32_RTOL


@pytest.mark.parametrize("warps", [16, 12])
def test_complex_eight_row_step(ctx, warps):
    """The complex 8-row tensor-core step (step_kernel 5): real and imaginary value
    panels of each 8-row block, the complex product combined per column pair at
    the block's end. Against the 4-row complex step to 2e-5 and the oracle's
    complex recursion to the FP32 bar, with random-phase and host start vectors,
    on a flake whose row count leaves a partial last block."""
    g = L.make_geom(model=L.MODEL_SIMPLE, size=40, max_R=69.0, angles_deg=(0.0, 2.0), energy_rescale=1.0,
                    b_field=300.0)
    csr = ctx.build_csr(ctx.prepare(g))
    assert csr.n % 8 != 0  # 11,438 orbitals
    lo, hi = csr.bounds()
    csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
    rp, col, val = csr.download()
    im = csr.download_imag()
    P, R, seed = 96, 16, 11
    cfg = L.kpm_cfg(P, R=R, kind=L.VEC_PHASE, precision=L.FP32, seed=seed)
    rb = csr.kpm_dos(cfg)  # the 4-row complex step (the default)
    ctx.set_option("step_kernel", 5)
    ctx.set_option("rt_warps", warps)
    try:
        mu = csr.kpm_dos(cfg)
        assert csr.rt_info()[0] == (csr.n + 7) // 8
        vec = np.random.default_rng(3).normal(size=(5, csr.n))
        host = csr.kpm_dos(L.kpm_cfg(P, R=5, kind=L.VEC_HOST, precision=L.FP32), vec)
    finally:
        ctx.set_option("step_kernel", -1)
        ctx.set_option("rt_warps", 0)
    assert _rel(mu, rb) < 2e-5
    re_v, im_v = oracle.phase_vectors(seed, 0, R, csr.n)
    assert _rel(mu, oracle.kpm_trace_cpx_doubling(rp, col, val, im, re_v, im_v, P)) < FP32_RTOL
    assert _rel(host, oracle.kpm_trace_cpx(rp, col, val, im, vec, P)) < FP32_RTOL
