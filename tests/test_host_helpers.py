"""Host-side helpers of the Python API (no GPU): the k grid of K_TYPE = 0 and the
row numbering of a matrix with vacancies."""
import numpy as np
import pytest

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


def _kpts_text(ks):
    """Param_tools::saveKpts (param_tools.cpp:579-602): 10 decimals, a space before
    a non-negative value, two tabs between the components."""
    out = []
    for kx, ky in ks:
        out.append((" " if kx >= 0 else "") + f"{kx:.10f}\t\t" + (" " if ky >= 0 else "") + f"{ky:.10f} \n")
    return "".join(out)


def test_k_lists_match_the_reference_kpts_files():
    """The k points the reference's own main() wrote for a K_TYPE = 0 grid (2 x 2),
    a K_TYPE = 1 path (6 points, every leg of K -> Gamma -> M -> K), a K_TYPE = 2
    path (5 points of sheet 0's zone, Gamma -> M -> K -> Gamma), a K_TYPE = 3
    path (7 points, Gamma -> M -> K -> K' -> Gamma) and K_TYPE = 4 paths
    (Gamma -> K -> M -> Gamma, 3 and 2 points a leg, on (3,2) and (2,3) cells:
    both orderings of the cell's basis) and a K_TYPE = 5 path (the (2,1) helical
    trilayer's three K points joined, 2 points a leg)."""
    from tests._golden import e2e_text, parse_in
    for name, ks in (("sc32_ksamp_ldos", lambda g: L.k_grid(g, 2, 2)),
                     ("sc32_ksamp_path_ldos", lambda g: L.k_path(g, 6)),
                     ("sc32_ksamp_mono_ldos", lambda g: L.k_path(g, 5, k_type=2)),
                     ("sc32_ksamp_loop_ldos", lambda g: L.k_path(g, 7, k_type=3)),
                     ("sc32_ksamp_gkm_ldos", lambda g: L.k_path(g, 3, k_type=4)),
                     ("sc23_ksamp_gkm_ldos", lambda g: L.k_path(g, 2, k_type=4)),
                     ("tri21_ksamp_dirac_ldos", lambda g: L.k_path(g, 2, k_type=5))):
        g, _ = parse_in(name)
        g = oracle.geom_prepare(g)
        assert _kpts_text(ks(g)) == e2e_text(name, ".kpts"), name


def test_k_path_corners():
    """Gamma at a third of the way, M at two thirds; |K| = |b2| / (2 cos 30) = |b2| / sqrt 3."""
    g = oracle.geom_prepare(L.make_geom(boundary_condition=1, supercell_mn=(4, 5), size=16, energy_rescale=13.0))
    ks = L.k_path(g, 9)
    b2 = 2 * L.k_grid(g, 1, 2)[1]
    np.testing.assert_allclose(ks[3], [0.0, 0.0], atol=1e-15)
    np.testing.assert_allclose(ks[6], b2 / 2, atol=1e-15)
    np.testing.assert_allclose(np.linalg.norm(ks[0]), np.linalg.norm(b2) / np.sqrt(3), rtol=1e-14)


def test_k_path_twisted_zone_needs_two_sheets():
    """K_TYPE = 1 walks the twisted (supercell) zone: a single layer has none, and
    the helper refuses it with the reference's message (locality.cpp:1661-1663),
    as the driver does; the other k lists still run."""
    g = oracle.geom_prepare(L.make_geom(num_sheets=1, boundary_condition=1, supercell_mn=(4, 5), size=16,
                                        energy_rescale=13.0))
    with pytest.raises(ValueError, match="single layer"):
        L.k_path(g, 4, k_type=1)
    assert L.k_path(g, 4, k_type=2).shape == (4, 2)


def test_gkm_path_needs_a_bilayer_mn_cell():
    """K_TYPE = 4 takes the (M, N) cell of a bilayer, K_TYPE = 5 a trilayer; other
    cells are refused by the helper as by the driver. On the trilayer's cell the
    reference's K_TYPE = 4 list ends in NaN points (its M -> Gamma leg divides by
    zero: M lies on the y axis), which the helper refuses by name."""
    g = oracle.geom_prepare(L.make_geom(num_sheets=1, boundary_condition=1, supercell_mn=(4, 5), size=16,
                                        energy_rescale=13.0))
    with pytest.raises(ValueError, match="bilayer SUPERCELL_M_N"):
        L.k_path(g, 4, k_type=4)
    with pytest.raises(ValueError, match="trilayer supercell"):
        L.k_path(g, 4, k_type=5)
    g = oracle.geom_prepare(L.make_geom(num_sheets=3, boundary_condition=1, supercell_mn=(2, 1), size=20,
                                        heights=(0.0, 3.35, 6.7), angles_deg=(0, 0, 0), energy_rescale=13.0,
                                        trilayer_supercell=1))
    with pytest.raises(ValueError, match="divides by zero"):
        L.k_path(g, 2, k_type=4)
    assert L.k_path(g, 2, k_type=5).shape == (5, 2)
    g = oracle.geom_prepare(L.make_geom(boundary_condition=1, supercell_mn=(4, 5), size=16, energy_rescale=13.0))
    ks = L.k_path(g, 4, k_type=4)
    assert ks.shape == (12, 2)
    np.testing.assert_array_equal(ks[0], [0.0, 0.0])
