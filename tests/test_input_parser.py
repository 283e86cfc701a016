"""The C++ .in reader (leo2d_parse_input, host only) against the golden inputs.

The geometry it produces must be identical to the one the golden fixtures
were generated from, so the GPU job sees the reference's sheets, bounds,
angles and energy scale bit for bit.
"""
import ctypes
import os

import numpy as np
import pytest

from leo2d_gb300 import _abi
from tests._golden import BFIELD_CASES, CASES, GOLDEN, parse_in


def _parse(path):
    L = _abi.load()
    g = _abi.Geom()
    ints = np.zeros(10, np.int32)
    msg = ctypes.create_string_buffer(512)
    st = L.leo2d_parse_input(str(path).encode(), ctypes.byref(g), ints.ctypes.data_as(ctypes.c_void_p),
                             msg, len(msg))
    return st, g, ints, msg.value.decode()


@pytest.mark.parametrize("name", CASES)
def test_geometry_matches_fixture_spec(name):
    st, g, ints, msg = _parse(os.path.join(GOLDEN, "inputs", name + ".in"))
    assert st == 0 and ints[7] == 0, msg
    ref, kv = parse_in(name)
    # (REF_DUMP_SHIFT is the fixture generator's job shift, not an input key)
    for s in range(len(ref.shifts)):
        ref.shifts[s][0] = ref.shifts[s][1] = 0.0
    assert bytes(g) == bytes(ref)
    assert ints[2] == kv["P"] and ints[0] == {"LC": 2, "FIXED_SHIFT": 6}.get(kv.get("solver"), 1)
    assert ints[8] == kv["target_sheets"][0]


def test_unsupported_options_are_reported(tmp_path):
    p = tmp_path / "x.in"
    p.write_text("NUM_SHEETS = 1\nSTART_SHEET 1\nMATERIAL = MoS2\nEND_SHEET 1\nDIAGONALIZE = 1\n"
                 "STRAIN_TYPE = 2\nPOLY_ORDER = 30\nSOLVER_TYPE = STRAIN\n")
    st, g, ints, msg = _parse(p)
    assert st == 0
    assert ints[7] == 4 and "MoS2" in msg and "DIAGONALIZE" in msg and "STRAIN_TYPE" in msg


def test_vacancy_solver_keys():
    """SOLVER_TYPE = MLMC_VAC (3) and VD_FILE (4) with the MLMC keys parse as the
    reference reads them (main.cpp:410-430, 730-775)."""
    from tests._golden import GOLDEN as G
    st, g, ints, msg = _parse(os.path.join(G, "mlmc", "mlmc_L1.in"))
    assert st == 0 and ints[7] == 0, msg
    assert ints[0] == 3 and ints[3] == 1 and ints[2] == 64


@pytest.mark.parametrize("name", BFIELD_CASES)
def test_magnetic_field_inputs(name):
    """USE_B_FIELD = 1 with B_FIELD: the complex Hamiltonian's field reaches the geometry."""
    st, g, ints, msg = _parse(os.path.join(GOLDEN, "inputs", name + ".in"))
    assert st == 0 and ints[7] == 0, msg
    ref, kv = parse_in(name)
    assert g.b_field == kv["b_field"] == 1500.0
    assert bytes(g) == bytes(ref)


def test_magnetic_field_limits(tmp_path):
    # a field on a periodic supercell runs (generateCpxH's Peierls phase on every image)
    p = tmp_path / "x.in"
    p.write_text("NUM_SHEETS = 1\nSTART_SHEET 1\nMATERIAL = Graphene\nEND_SHEET 1\nBOUNDARY_CONDITION = 1\n"
                 "SUPERCELL_M_N = 2 3\nUSE_B_FIELD = 1\nB_FIELD = 10\nPOLY_ORDER = 32\n")
    st, g, ints, msg = _parse(p)
    assert st == 0 and ints[7] == 0 and g.b_field == 10.0
    # the Kubo observable in a field is refused by name
    p.write_text("NUM_SHEETS = 1\nSTART_SHEET 1\nMATERIAL = Graphene\nEND_SHEET 1\n"
                 "OBSERVABLE_TYPE = COND\nUSE_B_FIELD = 1\nB_FIELD = 10\nPOLY_ORDER = 32\n")
    st, g, ints, msg = _parse(p)
    assert st == 0 and ints[7] == 1 and "COND" in msg


def test_missing_file():
    st, g, ints, msg = _parse("/nonexistent/file.in")
    assert st == _abi.ERR_IO and "not found" in msg


def test_model_and_kpm_keys(tmp_path):
    p = tmp_path / "y.in"
    p.write_text("MAXSIZE = 30\nMINSIZE = -30\nMAX_R = 25.5\nNUM_SHEETS = 2\nMODEL = SIMPLE\n"
                 "START_SHEET 1\nMATERIAL = Graphene\nEND_SHEET 1\n"
                 "START_SHEET 2\nMATERIAL = Graphene\nHEIGHT = 3.35\nANGLE = 1.05\nEND_SHEET 2\n"
                 "KPM_VECTORS = PHASE\nKPM_SEED = 99\nKPM_BOUNDS = GERSHGORIN\nPOLY_ORDER = 64\n")
    st, g, ints, msg = _parse(p)
    assert st == 0 and ints[7] == 0
    assert g.model == _abi.MODEL_SIMPLE and g.max_R[0] == 25.5 and g.max_R[1] == 25.5
    assert g.angles[1] == (2 * np.pi * 1.05) / 360.0 and g.heights[1] == 3.35


def test_k_lists_outside_the_build_are_refused_on_the_host(tmp_path):
    """K_TYPE = 5 (the trilayer's Dirac points) is refused by name, and K_TYPE = 4
    away from a bilayer (M, N) cell too; both before any device is touched."""
    import leo2d_gb300 as L
    src = open(os.path.join(GOLDEN, "inputs", "sc32_ksamp_gkm_ldos.in")).read()
    p = tmp_path / "k5.in"
    p.write_text(src.replace("K_TYPE = 4", "K_TYPE = 5"))
    with pytest.raises(L.Leo2dError, match="K_TYPE = 5"):
        L.run_input(p, tmp_path)
    p.write_text(src.replace("SUPERCELL_M_N = 3 2", "SUPERCELL_M_N = 0 0"))
    with pytest.raises(L.Leo2dError, match="K_TYPE = 4"):
        L.run_input(p, tmp_path)


@pytest.mark.parametrize("name", CASES + BFIELD_CASES)
def test_prepared_geometry_matches_the_oracle(name):
    """leo2d_geom_prepare (the library's host code: lattices, supercell strides and
    angles, the helical trilayer's cell included) gives the oracle's prepared
    geometry byte for byte on every golden input."""
    import copy
    from oracle import oracle
    g, _ = parse_in(name)
    ours = copy.copy(g)
    assert _abi.load().leo2d_geom_prepare(ctypes.byref(ours)) == 0
    assert bytes(ours) == bytes(oracle.geom_prepare(g))


def test_trilayer_cell_and_supercell_groups(tmp_path):
    """TRILAYER_SUPERCELL = 1 selects the helical trilayer cell on three sheets (a
    later SUPERCELL_M_N selects the bilayer rule again, as main.cpp's order of
    keys does); elsewhere it is refused by name. SUPERCELL_GROUPS that put sheet
    1 alone against the rest are the cell built here; other groupings are
    refused by name."""
    sheets = "".join(f"START_SHEET {s}\nMATERIAL = Graphene\nHEIGHT = {3.35 * (s - 1)}\nEND_SHEET {s}\n"
                     for s in (1, 2, 3))
    head = "MAXSIZE = 20\nMINSIZE = -20\nBOUNDARY_CONDITION = 1\nNUM_SHEETS = 3\n"
    p = tmp_path / "t.in"
    p.write_text(head + "SUPERCELL_M_N = 2 1\nTRILAYER_SUPERCELL = 1\n" + sheets + "POLY_ORDER = 32\n")
    st, g, ints, msg = _parse(p)
    assert st == 0 and ints[7] == 0 and g.trilayer_supercell == 1, msg
    p.write_text(head + "TRILAYER_SUPERCELL = 1\nSUPERCELL_M_N = 2 1\n" + sheets + "POLY_ORDER = 32\n")
    st, g, ints, msg = _parse(p)
    assert st == 0 and g.trilayer_supercell == 0
    p.write_text(head.replace("NUM_SHEETS = 3", "NUM_SHEETS = 2") + "SUPERCELL_M_N = 2 1\nTRILAYER_SUPERCELL = 1\n"
                 + sheets.split("START_SHEET 3")[0] + "POLY_ORDER = 32\n")
    st, g, ints, msg = _parse(p)
    assert ints[7] == 1 and "TRILAYER_SUPERCELL" in msg
    for groups, ok in (("1 / 2 3 /", True), ("1 2 / 3 /", False), ("2 / 1 3 /", False)):
        p.write_text(head + "SUPERCELL_M_N = 2 1\n" + f"SUPERCELL_GROUPS = {groups}\n" + sheets + "POLY_ORDER = 32\n")
        st, g, ints, msg = _parse(p)
        assert st == 0 and (ints[7] == 0) == ok and (ok or "SUPERCELL_GROUPS" in msg), (groups, msg)
