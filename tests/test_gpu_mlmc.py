"""The MLMC vacancy run of `leo2d file.in` (leo2d_run_input) against the files
the reference's own main() wrote for the same two-level run
(tests/golden/mlmc, made by make_mlmc_golden.py).

Level 2 runs three MLMC_VAC jobs (vacancies removed from a 5 deg flake, trace
DOS of the reference's Gaussian vectors with the vacancy jobs' num_dofs) into
its mean (E) and second moment (V), and saves each job's DOS under temp/ as a
cluster original of the next level down. Level 1 runs two plain jobs and three
cluster members whose differences from those originals go to DE and DV. Every
binary file (raw FP64) must match: the FP64 recursion reproduces the
reference's DOS to 1e-9 of its largest value.
"""
import os
import shutil

import numpy as np
import pytest

import leo2d_gb300 as L
from tests._golden import GOLDEN

pytestmark = pytest.mark.gpu
HERE = os.path.join(GOLDEN, "mlmc")


def test_two_level_mlmc_files(tmp_path):
    for f in ("mlmc_L2.in", "mlmc_L1.in", "vac_L2.dat", "vac_L1.dat"):
        shutil.copy(os.path.join(HERE, f), tmp_path)
    (tmp_path / "out").mkdir()
    (tmp_path / "temp").mkdir()
    for f in ("mlmc_L2.in", "mlmc_L1.in"):
        L.run_input(tmp_path / f, tmp_path)
    assert not (tmp_path / "mlmc_flake.cheb").exists()  # an MLMC run writes statistics only
    with np.load(os.path.join(HERE, "mlmc.npz")) as z:
        gold = {k: z[k] for k in z.files}
    written = sorted(f"{d}/{f}" for d in ("out", "temp") for f in os.listdir(tmp_path / d))
    assert written == sorted(gold)
    for k, ref in gold.items():
        ours = np.fromfile(tmp_path / k, dtype=np.float64)
        assert ours.shape == ref.shape, k
        assert np.max(np.abs(ours - ref)) <= 1e-9 * max(np.max(np.abs(ref)), 1e-30), k


def test_mlmc_refuses_bad_cluster_ids(tmp_path):
    """A job of a cluster the run does not hold (CLUSTERID past MLMC_NUM_CLUSTERS)."""
    shutil.copy(os.path.join(HERE, "mlmc_L1.in"), tmp_path)
    (tmp_path / "vac_L1.dat").write_text("JOBID = 1\nCLUSTERID = 3\nVAC = 5\n")
    (tmp_path / "out").mkdir()
    (tmp_path / "temp").mkdir()
    with pytest.raises(L.Leo2dError) as e:
        L.run_input(tmp_path / "mlmc_L1.in", tmp_path)
    assert "CLUSTERID" in str(e.value)
