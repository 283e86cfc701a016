"""The GPU path at the full sizes of the two smallest workloads, against
digests of the reference's own output (tests/golden/configs).

cfg0_flake: the 5.09 deg twisted-bilayer flake of radius 147.6 A, 51,560
orbitals, 15,145,954 stored entries (reference hoppings, every in-window pair
kept), P = 1000. cfg1_sc3132: the (31,32) supercell at 1.05 deg, periodic,
11,908 orbitals, P = 4096. Each with the reference's two Gaussian trace
vectors. The device assembly must reproduce the reference's row pointers and
columns bit for bit (SHA-256) and its FP64 values to 1e-12 (every 997th entry,
and every row's sums); FP64 moments match the reference's to 1e-10 of the
largest, FP32 moments to 1e-4, and the DOS to 1e-8.
"""
import hashlib

import numpy as np
import pytest

import leo2d_gb300 as L
from oracle import oracle
from tests._golden import load_config, parse_in

pytestmark = pytest.mark.gpu
CONFIGS = ["cfg0_flake", "cfg1_sc3132"]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.fixture(scope="module")
def ctx():
    with L.Context(0) as c:
        yield c


@pytest.mark.parametrize("name", CONFIGS)
def test_full_size_csr_and_moments(ctx, name):
    gold = load_config(name)
    g, _ = parse_in(name, folder="configs")
    meta = gold["meta"]
    P, R = int(meta[5]), gold["moments"].shape[0]
    csr = ctx.build_csr(ctx.prepare(g), keep_zeros=True)
    assert (csr.n, csr.nnz) == (meta[0], meta[1])
    rp, col, val = csr.download()
    d = gold["digests"]
    assert _sha(rp.astype(np.int32)) == d[0]
    assert _sha(col) == d[1]
    # values: the device's FP64 exp / cos / atan2 may differ from the host libm's
    # in the last bit, so they are held to 1e-12, entry by entry on the sample
    # and row by row on the sums
    idx = gold["sample_idx"]
    np.testing.assert_array_equal(col[idx], gold["sample_col"])
    assert np.max(np.abs(val[idx] - gold["sample_val"])) <= 1e-12
    starts = rp[:-1].astype(np.int64)
    assert np.max(np.abs(np.add.reduceat(val, starts) - gold["row_sum"])) <= 1e-12
    assert np.max(np.abs(np.add.reduceat(np.abs(val), starts) - gold["row_abs"])) <= 1e-12
    vec = oracle.reference_gaussian(R, csr.n)
    ref = gold["moments"]
    mu = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_HOST, precision=L.FP64), vec)
    assert _rel(mu, ref) < 1e-10
    mu32 = csr.kpm_dos(L.kpm_cfg(P, R=R, kind=L.VEC_HOST, precision=L.FP32), vec)
    assert _rel(mu32, ref) < 1e-4
    dos, E = ctx.dos_transform(mu, P, g.energy_rescale, g.energy_shift, 1.0 / csr.n)
    # the DOS divides the Jackson-weighted DCT by pi sqrt(a^2 - (E - b)^2), which
    # is about 1e-3 a at the outermost Chebyshev nodes of P = 4096: compare the
    # sums before that division
    w = np.sqrt(np.maximum(g.energy_rescale ** 2 - (E - g.energy_shift) ** 2, 0.0))
    np.testing.assert_allclose(dos * w, gold["dos"] * w, rtol=1e-8, atol=1e-10 * np.abs(gold["dos"] * w).max())
    csr.close()


def test_cfg0_phase_vectors_against_oracle(ctx):
    """The timed form of the flake workload (random-phase vectors, FP32 and FP64
    recursions, the simple model's parameters kept aside): the GPU FP64 moments
    of two Philox phase vectors equal the FP64 oracle's on the same vectors."""
    g, _ = parse_in("cfg0_flake", folder="configs")
    csr = ctx.build_csr(ctx.prepare(g))
    P = 256
    mu = csr.kpm_dos(L.kpm_cfg(P, R=2, seed=17, precision=L.FP64))
    mu32 = csr.kpm_dos(L.kpm_cfg(P, R=2, seed=17))
    rp, col, val = csr.download()
    re, im = oracle.phase_vectors(17, 0, 2, csr.n)
    o = (oracle.kpm_trace(rp, col, val, re, P, literal=False) +
         oracle.kpm_trace(rp, col, val, im, P, literal=False))
    assert _rel(mu, o) < 1e-10
    assert _rel(mu32, o) < 1e-4
    csr.close()
