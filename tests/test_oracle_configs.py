"""The oracle at the full sizes of the two smallest workloads, against digests
of the reference's own output (tests/golden/configs, made by
make_config_golden.py from oracle/_ref/ref_dump).

cfg0_flake: the 5.09 deg twisted-bilayer flake of radius 147.6 A (51,560
orbitals, 15,145,954 stored entries, reference hoppings). cfg1_sc3132: the
commensurate (31,32) supercell at 1.05 deg with periodic boundaries (11,908
orbitals). The CSR must match bit for bit (SHA-256 of row pointers, columns
and FP64 values). The moments of the reference's two Gaussian vectors are
checked on their first 32 entries, which the recursion computes directly for
any P >= 64 (locality.cpp:6195-6221), with a P = 64 run.
"""
import hashlib

import numpy as np
import pytest

from oracle import oracle
from tests._golden import load_config, parse_in

CONFIGS = ["cfg0_flake", "cfg1_sc3132"]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module", params=CONFIGS)
def built(request):
    name = request.param
    g, _ = parse_in(name, folder="configs")
    return name, load_config(name), oracle.Built(g)


def test_csr_bit_exact_at_full_size(built):
    name, gold, b = built
    meta = gold["meta"]
    assert b.n == meta[0] and b.nnz == meta[1], name
    assert (b.n_intra, b.n_inter) == (meta[2], meta[3])
    rp = b.rowptr.astype(np.int32)
    np.testing.assert_array_equal(rp, gold["rowptr"])
    d = gold["digests"]
    assert _sha(rp) == d[0]
    assert _sha(b.col) == d[1]
    assert _sha(b.val) == d[2]
    idx = gold["sample_idx"]
    np.testing.assert_array_equal(b.col[idx], gold["sample_col"])
    np.testing.assert_array_equal(b.val[idx], gold["sample_val"])
    starts = b.rowptr[:-1].astype(np.int64)
    np.testing.assert_array_equal(np.add.reduceat(b.val, starts), gold["row_sum"])


def test_trace_vectors_and_first_moments(built):
    name, gold, b = built
    R = gold["moments"].shape[0]
    vec = oracle.reference_gaussian(R, b.n)
    assert _sha(vec.ravel()) == gold["digests"][3]
    mu = oracle.kpm_trace(b.rowptr, b.col, b.val, vec, 64, literal=True)
    ref = gold["moments"][:, :32]
    assert np.max(np.abs(mu[:, :32] - ref)) <= 1e-11 * np.max(np.abs(ref)), name
