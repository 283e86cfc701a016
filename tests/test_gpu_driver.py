"""`leo2d file.in` (leo2d_run_input) against the reference's own output files.

The reference binary's .cheb and _matrix.dat for each golden input (generated
by tests/golden/make_golden.py) must be reproduced: same layout, same numbers
at the printed precision (6 decimals, or 6 significant digits in
_matrix.dat), allowing one unit in the last printed digit where the FP64
results straddle a rounding boundary.
"""
import gzip
import os
import shutil
import subprocess

import numpy as np
import pytest

import leo2d_gb300 as L
from tests._golden import E2E_CASES, GOLDEN, e2e_text

pytestmark = pytest.mark.gpu


def _numbers(text):
    out = []
    for tok in text.replace(",", " ").split():
        try:
            out.append(float(tok))
        except ValueError:
            out.append(tok)
    return out


def _same(a, b, tol):
    na, nb = _numbers(a), _numbers(b)
    assert len(na) == len(nb)
    for x, y in zip(na, nb):
        if isinstance(x, float) and isinstance(y, float):
            assert abs(x - y) <= tol * max(1.0, abs(y)), (x, y)
        else:
            assert x == y


def _cond_rows(text, P):
    lines = text.split("\n")
    rows = [np.array([float(x) for x in ln.split()]) for ln in lines[2:] if ln.strip()]
    return np.array(lines[0].split(), dtype=float), np.stack(rows).reshape(-1, P, P)


@pytest.mark.parametrize("name", E2E_CASES)
def test_cheb_and_matrix_files(tmp_path, name):
    L.run_input(os.path.join(GOLDEN, "inputs", name + ".in"), tmp_path)
    ours = (tmp_path / (name + ".cheb")).read_text()
    ref = e2e_text(name, ".cheb")
    assert ours.count("\n") == ref.count("\n")
    if "_ksamp_" in name:
        # k-sampled jobs run the complex FP32 recursion: 1e-4 of the largest value;
        # the k points themselves are written as the reference writes them
        fo = np.array([x for x in _numbers(ours) if isinstance(x, float)])
        fr = np.array([x for x in _numbers(ref) if isinstance(x, float)])
        assert [x for x in _numbers(ours) if not isinstance(x, float)] == \
            [x for x in _numbers(ref) if not isinstance(x, float)]
        assert len(fo) == len(fr) and np.abs(fo - fr).max() <= 1e-4 * np.abs(fr).max() + 2e-6
        assert (tmp_path / (name + ".kpts")).read_text() == e2e_text(name, ".kpts")
    elif name == "flake_cond":
        # Kubo moments: the recursion is FP32, so compare at 1e-4 of the largest
        # moment. The reference defines the first target's columns 0..P-2 only
        # (the second target's block is NaN and column P-1 is never written).
        P = 32
        e, mu = _cond_rows(ours, P)
        er, mur = _cond_rows(ref, P)
        np.testing.assert_allclose(e, er, atol=1.01e-6)
        d = np.abs(mu[0, :, :P - 1] - mur[0, :, :P - 1]).max()
        assert d < 1e-4 * np.abs(mur[0, :, :P - 1]).max() + 2e-6
        assert np.all(np.isfinite(mu))
    else:
        _same(ours, ref, 1.01e-6)
    m = tmp_path / (name + "_matrix.dat")
    mref = e2e_text(name, "_matrix.dat")
    _same(m.read_text(), mref, 1e-5)


def test_driver_executable(tmp_path):
    exe = os.path.join(os.path.dirname(L._abi.LIB_PATH), "..", "bin", "leo2d")
    inp = os.path.join(GOLDEN, "inputs", "flake_trace.in")
    r = subprocess.run([exe, inp, str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _same((tmp_path / "flake_trace.cheb").read_text(), e2e_text("flake_trace", ".cheb"), 1.01e-6)


def test_unsupported_input_is_refused(tmp_path):
    p = tmp_path / "bad.in"
    p.write_text(open(os.path.join(GOLDEN, "inputs", "flake_trace.in")).read() + "DIAGONALIZE = 1\n")
    with pytest.raises(L.Leo2dError, match="DIAGONALIZE"):
        L.run_input(p, tmp_path)
    p.write_text(open(os.path.join(GOLDEN, "inputs", "flake_trace.in")).read().replace(
        "POLY_ORDER = 64", "POLY_ORDER = 62"))
    with pytest.raises(L.Leo2dError, match="divisible 4"):
        L.run_input(p, tmp_path)
    # the k list of K_TYPE 5 (the trilayer's Dirac points) is not built
    p.write_text(open(os.path.join(GOLDEN, "inputs", "sc32_ksamp_path_ldos.in")).read().replace(
        "K_TYPE = 1", "K_TYPE = 5"))
    with pytest.raises(L.Leo2dError, match="K_TYPE = 5"):
        L.run_input(p, tmp_path)
    # K_TYPE 4 samples a bilayer (M, N) cell's zone
    p.write_text(open(os.path.join(GOLDEN, "inputs", "sc32_ksamp_path_ldos.in")).read().replace(
        "K_TYPE = 1", "K_TYPE = 4").replace("SUPERCELL_M_N = 3 2", "SUPERCELL_M_N = 0 0"))
    with pytest.raises(L.Leo2dError, match="K_TYPE = 4"):
        L.run_input(p, tmp_path)
