"""Host-side helpers of the Python API (no GPU): the k grid of K_TYPE = 0 and the
row numbering of a matrix with vacancies."""
import numpy as np

import leo2d_gb300 as L
from oracle import oracle


def test_k_grid_is_the_reciprocal_grid():
    """k = (k1/n1) b1 + (k2/n2) b2 with b_i . a_j = 2 pi delta_ij of the prepared
    supercell, in the reference's job order (k1 outer)."""
    g = L.make_geom(boundary_condition=1, supercell_mn=(4, 5), size=16, energy_rescale=13.0)
    g = oracle.geom_prepare(g)
    a = np.array(g.supercell)
    ks = L.k_grid(g, 3, 2)
    assert ks.shape == (6, 2) and np.all(ks[0] == 0.0)
    b1, b2 = 3 * ks[2], 2 * ks[1]  # (k1 = 1, k2 = 0) and (k1 = 0, k2 = 1)
    np.testing.assert_allclose([b1 @ a[0], b1 @ a[1], b2 @ a[0], b2 @ a[1]], [2 * np.pi, 0, 0, 2 * np.pi],
                               atol=1e-12)
    np.testing.assert_allclose(ks[5], (2 / 3) * b1 + (1 / 2) * b2, atol=1e-15)


def test_vacancy_rows_match_the_relabelling():
    n = 40
    vac = [0, 3, 3, 17, 39, -5, 100]
    red, kept = oracle.vacancy_reduction(n, vac)
    assert kept == n - 4
    orbitals = np.arange(n)
    np.testing.assert_array_equal(L.vacancy_rows(n, vac, orbitals), orbitals - red[:n])
