"""Generates the golden fixtures in tests/golden/ from the reference's own code.

Run in the build container (it needs the reference sources, compiled by
`make -f oracle/Makefile.ref`):

    python tests/golden/make_golden.py [name ...]   # default: every input

For every LEO2D input in tests/golden/inputs/ it runs
  * oracle/_ref/ref_dump  - the reference's geometry, generateRealH and KPM
    functions on job 1 (with REF_DUMP_VACANCIES, on the vacancy solvers' path
    with that list) - and stores their arrays in <name>.npz;
  * oracle/_ref/leo2d_ref - the reference's unmodified main() on two
    in-process MPI ranks - and stores the .cheb and _matrix.dat it writes in
    e2e/<name>.cheb.gz and e2e/<name>_matrix.dat.gz.
The fixtures are committed; the tests read them without the reference.
"""
import gzip
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_DIR = os.path.join(REPO, "oracle", "_ref")

INT32 = {"meta", "index_to_grid", "intra_pairs", "intra_sc", "inter_pairs", "inter_sc",
         "rowptr", "col", "targets", "vacancies", "n_kept"}
# arrays that are large and fully determined by others are left out of the fixture
SKIP = {"index_to_pos", "trace_vectors"}


def run_dump(inp, name):
    out = {}
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([os.path.join(REF_DIR, "ref_dump"), inp, d], check=True,
                       stdout=subprocess.DEVNULL)
        for f in sorted(os.listdir(d)):
            key = f[:-4]
            if key in SKIP:
                continue
            dt = np.int32 if key in INT32 else np.float64
            out[key] = np.fromfile(os.path.join(d, f), dtype=dt)
    meta = out["meta"]
    is_cond = meta[7] == 1
    if not is_cond:
        # dxH / dyH only matter for the conductivity fixtures
        out.pop("val_dx", None)
        out.pop("val_dy", None)
        out.pop("alpha0_x", None)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return out


def run_e2e(inp, name):
    os.makedirs(os.path.join(HERE, "e2e"), exist_ok=True)
    with tempfile.TemporaryDirectory() as d:
        shutil.copy(inp, d)
        env = dict(os.environ, LEO2D_REF_RANKS="2")
        subprocess.run([os.path.join(REF_DIR, "leo2d_ref"), os.path.basename(inp)], cwd=d,
                       check=True, stdout=subprocess.DEVNULL, env=env)
        for suffix in (".cheb", "_matrix.dat", ".kpts"):
            src = os.path.join(d, name + suffix)
            if os.path.exists(src):
                dst = os.path.join(HERE, "e2e", name + suffix + ".gz")
                with open(src, "rb") as fi, open(dst, "wb") as raw, gzip.GzipFile(
                        fileobj=raw, mode="wb", mtime=0) as fo:
                    fo.write(fi.read())


def main():
    if not os.path.exists(os.path.join(REF_DIR, "ref_dump")):
        sys.exit("build the reference first: make -f oracle/Makefile.ref -j8")
    inputs = sorted(f for f in os.listdir(os.path.join(HERE, "inputs")) if f.endswith(".in"))
    if len(sys.argv) > 1:
        inputs = [f for f in inputs if f[:-3] in sys.argv[1:]]
    for f in inputs:
        name = f[:-3]
        inp = os.path.join(HERE, "inputs", f)
        arrs = run_dump(inp, name)
        # vacancy lists and k vectors are ref_dump keys (the reference's own
        # main() takes them from its solver files and k grids): no end-to-end
        # files for those
        if "REF_DUMP_" not in open(inp).read():
            run_e2e(inp, name)
        m = arrs["meta"]
        print(f"{name}: N={m[0]} nnz={m[1]} intra={m[2]} inter={m[3]} targets={m[4]} P={m[5]}")


if __name__ == "__main__":
    main()
