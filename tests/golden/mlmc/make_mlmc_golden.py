"""Golden files of a two-level MLMC vacancy run, written by the reference's own
main() (oracle/_ref/leo2d_ref, two in-process MPI ranks).

Run in the build container (it needs the reference built by
`make -f oracle/Makefile.ref`):

    python tests/golden/mlmc/make_mlmc_golden.py

In one working directory (with out/ and temp/ made first, as the reference
expects them) it runs mlmc_L2.in (MLMC_LEVEL 2 of 2: three vacancy jobs whose
trace DOS go to the level's mean and second moment, and to temp/ as the next
level's cluster originals) and then mlmc_L1.in (level 1: two plain jobs and
three jobs of clusters 1 and 2, whose differences from the originals go to DE
and DV). The binary files under out/ (raw FP64) are stored in mlmc.npz.
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
REF = os.path.join(REPO, "oracle", "_ref", "leo2d_ref")


def main():
    if not os.path.exists(REF):
        sys.exit("build the reference first: make -f oracle/Makefile.ref -j8")
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for f in ("mlmc_L2.in", "mlmc_L1.in", "vac_L2.dat", "vac_L1.dat"):
            shutil.copy(os.path.join(HERE, f), d)
        os.mkdir(os.path.join(d, "out"))
        os.mkdir(os.path.join(d, "temp"))
        env = dict(os.environ, LEO2D_REF_RANKS="2")
        for f in ("mlmc_L2.in", "mlmc_L1.in"):
            subprocess.run([REF, f], cwd=d, check=True, stdout=subprocess.DEVNULL, env=env)
        for sub in ("out", "temp"):
            for f in sorted(os.listdir(os.path.join(d, sub))):
                out[sub + "/" + f] = np.fromfile(os.path.join(d, sub, f), dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "mlmc.npz"), **out)
    for k, v in out.items():
        print(k, v.shape)


if __name__ == "__main__":
    main()
