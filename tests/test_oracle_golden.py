"""The CPU oracle against fixtures generated from the reference's own code.

These pin the restatement in oracle/leo2d_oracle.cpp: geometry, pair lists and
CSR must be identical to the reference's; moments and transforms agree to
rounding.
"""
import numpy as np
import pytest

import leo2d_gb300 as L
from oracle import oracle
from tests._golden import CASES, VAC_CASES, load, parse_in, vac_base


@pytest.fixture(scope="module", params=CASES)
def case(request):
    name = request.param
    gold = load(name)
    g, kv = parse_in(name)
    built = oracle.Built(g)
    return name, gold, built, kv


def test_geometry_and_pairs_bit_exact(case):
    name, gold, b, kv = case
    meta = gold["meta"]
    assert b.n == meta[0] and b.n_intra == meta[2] and b.n_inter == meta[3]
    assert np.array_equal(b.index_to_grid, gold["index_to_grid"])
    assert np.array_equal(b.pos, gold["i2pos"])
    assert np.array_equal(b.intra_pairs, gold["intra_pairs"])
    assert np.array_equal(b.intra_t, gold["intra_t"])
    assert np.array_equal(b.inter_pairs, gold["inter_pairs"])
    if b.geom.boundary_condition == 1:
        assert np.array_equal(b.intra_sc, gold["intra_sc"])
        assert np.array_equal(b.inter_sc, gold["inter_sc"])


def test_csr_bit_exact(case):
    name, gold, b, kv = case
    assert np.array_equal(b.rowptr, gold["rowptr"].astype(np.int64))
    assert np.array_equal(b.col, gold["col"])
    # the same glibc transcendental calls in the same order: values are identical
    assert np.array_equal(b.val, gold["val"])
    if "val_dx" in gold:
        assert np.array_equal(b.val_dx, gold["val_dx"])
        assert np.array_equal(b.val_dy, gold["val_dy"])


def test_shift_configs_bit_exact(case):
    name, gold, b, kv = case
    if "shift_configs" not in gold:
        with pytest.raises(ValueError):
            b.shift_configs()
        return
    np.testing.assert_array_equal(b.shift_configs().ravel(), gold["shift_configs"])


def test_targets(case):
    name, gold, b, kv = case
    t = b.targets(kv["target_sheets"])
    assert np.array_equal(t, gold["targets"].astype(np.int64))


def test_moments(case):
    name, gold, b, kv = case
    meta = gold["meta"]
    P, trace, observable = int(meta[5]), int(meta[6]), int(meta[7])
    if observable == 1:
        pytest.skip("conductivity case: see test_cond_moments")
    if trace == 1:
        R = int(meta[4])
        vec = oracle.reference_gaussian(R, b.n)
        mu = oracle.kpm_trace(b.rowptr, b.col, b.val, vec, P)
        ref = gold["moments"].reshape(R, P)
        np.testing.assert_array_equal(mu, ref)
        mu2 = oracle.kpm_trace(b.rowptr, b.col, b.val, vec, P, literal=False)
        np.testing.assert_allclose(mu2, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
        dos, E = oracle.dos_transform(ref, P, b.geom.energy_rescale, b.geom.energy_shift,
                                      1.0 / b.n)
    else:
        tg = gold["targets"].astype(np.int64)
        mu = oracle.kpm_ldos(b.rowptr, b.col, b.val, tg, P)
        ref = gold["moments"].reshape(len(tg), P)
        np.testing.assert_array_equal(mu, ref)
        dos = np.stack([oracle.dos_transform(m, P, b.geom.energy_rescale,
                                             b.geom.energy_shift)[0] for m in ref])
    np.testing.assert_allclose(dos.ravel(), gold["dos"], rtol=1e-12,
                               atol=1e-13 * np.abs(gold["dos"]).max())


def test_cond_moments(case):
    name, gold, b, kv = case
    meta = gold["meta"]
    P, observable = int(meta[5]), int(meta[7])
    if observable != 1:
        pytest.skip("DOS case")
    tg = gold["targets"].astype(np.int64)
    C = oracle.kpm_cond(b.rowptr, b.col, b.val, b.val_dx, tg, P)
    ref = gold["cond_moments"].reshape(len(tg), P, P)
    # Column P-1 reads beta_{P-1}, which the reference never writes
    # (locality.cpp:6600-6621), and from the second target on the reference's
    # uninitialised stack vectors (temp_vec, locality.cpp:6641) enter as
    # 0 * garbage, which is NaN when the garbage is. The defined part is the
    # first target, columns 0..P-2; the oracle zero-initialises both.
    np.testing.assert_array_equal(C[0, :, :P - 1], ref[0, :, :P - 1])
    assert np.isfinite(C).all()
    # the 2-D transform, compared on a matrix whose last column is defined
    M = ref[0].copy()
    M[:, P - 1] = 0.0
    out = oracle.cond_transform(M)
    assert np.isfinite(out).all()


def test_dct_matches_scipy():
    scipy = pytest.importorskip("scipy.fft")
    rng = np.random.default_rng(0)
    P = 48
    mu = rng.standard_normal(P)
    dos, E = oracle.dos_transform(mu, P, 1.0, 0.0)
    g = np.array([((P - i) * np.cos(np.pi * i / P) + np.sin(np.pi * i / P) / np.tan(np.pi / P)) / P
                  for i in range(P)])
    # FFTW REDFT01 == scipy DCT-III (unnormalised) : out_k = x_0 + 2 sum x_j cos(pi j (k+1/2)/P)
    ref = scipy.dct(g * mu, type=3)
    ref = ref / (np.pi * np.sqrt(1.0 - np.cos((np.arange(P) + 0.5) * np.pi / P) ** 2))
    np.testing.assert_allclose(dos, ref, rtol=1e-11, atol=1e-12)


# ---------------------------------------------------------------- magnetic field (generateCpxH)

from tests._golden import COMPLEX_CASES  # noqa: E402


@pytest.fixture(scope="module", params=COMPLEX_CASES)
def bcase(request):
    name = request.param
    gold = load(name)
    g, kv = parse_in(name)
    return name, gold, oracle.Built(g), kv


def _complex_values(b, kv):
    """A flake in a field: std::polar(t, Peierls phase) per entry of the real H;
    a periodic job (k-sampled, in a field or both): the image-resolved sums of
    std::polar(t, Peierls phase + k.(r2 - r1))."""
    if "k_vec" in kv or kv.get("periodic"):
        return b.bloch(*kv.get("k_vec", (0.0, 0.0)))
    return oracle.peierls(b.rowptr, b.col, b.val, b.pos, kv["b_field"])


def _hermitian(b, re, im):
    import scipy.sparse as sp
    n = len(b.rowptr) - 1
    h = sp.csr_matrix((re + 1j * im, b.col.copy(), b.rowptr.copy()), shape=(n, n))  # scipy may sort in place
    return abs(h - h.conj().T).max() <= 1e-14 * abs(h).max()


def test_periodic_field_breaks_hermiticity(bcase):
    """The reference's Peierls phase on periodic images (the row's orbital shifted
    by the image, locality.cpp:4718-4738, 7157-7161) is not periodic in the
    Landau gauge, so H~ of a supercell in a field is not Hermitian; flakes in a
    field and k-sampled supercells are."""
    name, gold, b, kv = bcase
    herm = _hermitian(b, gold["val"], gold["val_im"])
    assert herm == (not (kv.get("periodic") and kv.get("use_b"))), name


def test_bfield_csr(bcase):
    """Structure of the real H; the complex values as generateCpxH builds them."""
    name, gold, b, kv = bcase
    assert np.array_equal(b.rowptr, gold["rowptr"].astype(np.int64))
    assert np.array_equal(b.col, gold["col"])
    re, im = _complex_values(b, kv)
    np.testing.assert_array_equal(re, gold["val"])
    np.testing.assert_array_equal(im, gold["val_im"])
    assert np.abs(im).max() > 0.05 * np.abs(re).max()  # the phases really twist the hoppings


def test_bfield_moments(bcase):
    name, gold, b, kv = bcase
    meta = gold["meta"]
    P, trace = int(meta[5]), int(meta[6])
    re, im = _complex_values(b, kv)
    if trace == 1:
        R = int(meta[4])
        vec = oracle.reference_gaussian(R, b.n)
        ref = gold["moments"].reshape(R, P)
        mu = oracle.kpm_trace_cpx(b.rowptr, b.col, re, im, vec, P)
        np.testing.assert_allclose(mu, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
        mu2 = oracle.kpm_trace_cpx_doubling(b.rowptr, b.col, re, im, vec, np.zeros_like(vec), P)
        if _hermitian(b, re, im):
            np.testing.assert_allclose(mu2, ref, rtol=0, atol=1e-11 * np.abs(ref).max())
        else:
            # a field on a periodic supercell: the moments below P/2 are direct
            # dots, and every-moment doubling is not the same estimate
            assert np.abs(mu2 - ref).max() > 1e-6 * np.abs(ref).max()
        # the field changes the moments
        mu0 = oracle.kpm_trace(b.rowptr, b.col, b.val, vec, P)
        assert np.abs(mu0 - ref).max() > 1e-4 * np.abs(ref).max()
    else:
        tg = gold["targets"].astype(np.int64)
        ref = gold["moments"].reshape(len(tg), P)
        mu = oracle.kpm_ldos_cpx(b.rowptr, b.col, re, im, tg, P)
        np.testing.assert_allclose(mu, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


# ------------------------------------------------------------- vacancies

@pytest.fixture(scope="module", params=VAC_CASES)
def vcase(request):
    name = request.param
    gold = load(name)
    g, kv = parse_in(vac_base(name))
    built = oracle.Built(g)
    return name, gold, built, kv


def test_vacancy_csr_bit_exact(vcase):
    """generateRealH's vacancy skips restated on the full matrix: rows, columns and
    values of the reference's reduced matrix (duplicates and out-of-range list
    entries change nothing)."""
    name, gold, b, kv = vcase
    vac = gold["vacancies"].astype(np.int64)
    vals = [b.val] + ([b.val_dx, b.val_dy] if "val_dx" in gold else [])
    rp, col, out = oracle.remove_orbitals(b.rowptr, b.col, vals, vac)
    red, kept = oracle.vacancy_reduction(b.n, vac)
    assert kept == int(gold["n_kept"][0]) == len(rp) - 1
    assert np.array_equal(rp, gold["rowptr"].astype(np.int64))
    assert np.array_equal(col, gold["col"])
    assert np.array_equal(out[0], gold["val"])
    if "val_dx" in gold:
        assert np.array_equal(out[1], gold["val_dx"])
        assert np.array_equal(out[2], gold["val_dy"])


def test_vacancy_moments(vcase):
    """Moments on the reduced matrix: targets renumbered as computeDosKPM does
    (t - reduction[t]), trace vectors of the reduced length."""
    name, gold, b, kv = vcase
    meta = gold["meta"]
    P, trace, observable = int(meta[5]), int(meta[6]), int(meta[7])
    vac = gold["vacancies"].astype(np.int64)
    vals = [b.val] + ([b.val_dx] if observable == 1 else [])
    rp, col, out = oracle.remove_orbitals(b.rowptr, b.col, vals, vac)
    red, kept = oracle.vacancy_reduction(b.n, vac)
    tg = gold["targets"].astype(np.int64)
    tl = tg - red[tg]
    # the library's host-side mapping of reference orbitals to reduced rows
    assert np.array_equal(L.vacancy_rows(b.n, vac, tg), tl)
    if observable == 1:
        C = oracle.kpm_cond(rp, col, out[0], out[1], tl, P)
        ref = gold["cond_moments"].reshape(len(tg), P, P)
        np.testing.assert_array_equal(C[0, :, :P - 1], ref[0, :, :P - 1])
    elif trace == 1:
        R = int(meta[4])
        mu = oracle.kpm_trace(rp, col, out[0], oracle.reference_gaussian(R, kept), P)
        np.testing.assert_array_equal(mu, gold["moments"].reshape(R, P))
        # the worker's DOS scale subtracts the list length once more (locality.cpp:3124-3128)
        dos, E = oracle.dos_transform(mu, P, b.geom.energy_rescale, b.geom.energy_shift,
                                      1.0 / (kept - len(vac)))
        np.testing.assert_allclose(dos.ravel(), gold["dos"], rtol=1e-12, atol=1e-13 * np.abs(gold["dos"]).max())
    else:
        mu = oracle.kpm_ldos(rp, col, out[0], tl, P)
        np.testing.assert_array_equal(mu, gold["moments"].reshape(len(tg), P))
