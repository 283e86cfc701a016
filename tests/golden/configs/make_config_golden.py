"""Golden digests of the two smallest workloads at their full sizes, from the
reference's own code.

Run in the build container (it needs the reference sources, compiled by
`make -f oracle/Makefile.ref`):

    python tests/golden/configs/make_config_golden.py [name ...]

For cfg0_flake.in (the 5.09 deg twisted-bilayer flake of radius 147.6 A, 51,560
orbitals, reference hoppings, P = 1000, two of the reference's Gaussian trace
vectors) and cfg1_sc3132.in (the commensurate (31,32) supercell at 1.05 deg,
11,908 orbitals, periodic, P = 4096, two vectors) it runs oracle/_ref/ref_dump
- the reference's Sheet/Hstruct geometry, generateRealH and computeDosTraceKPM
on job 1 - and stores what the GPU tests compare against, small enough to
commit: SHA-256 digests of the CSR arrays (row pointers and columns as int32,
values as FP64 bytes), every 997th entry's column and value, the row pointers
themselves, each row's sum of values and of their magnitudes, the moments of
both vectors, the DOS at the Chebyshev nodes and a digest of the trace vectors
(which oracle.reference_gaussian reproduces).
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
REF_DUMP = os.path.join(REPO, "oracle", "_ref", "ref_dump")
STRIDE = 997


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make(name):
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([REF_DUMP, os.path.join(HERE, name + ".in"), d], check=True, stdout=subprocess.DEVNULL)
        rd = lambda k, dt: np.fromfile(os.path.join(d, k + ".bin"), dtype=dt)
        meta = rd("meta", np.int32)
        rowptr, col, val = rd("rowptr", np.int32), rd("col", np.int32), rd("val", np.float64)
        moments, dos = rd("moments", np.float64), rd("dos", np.float64)
        tv = rd("trace_vectors", np.float64)
        targets = rd("targets", np.int32)
    n, nnz, P = int(meta[0]), int(meta[1]), int(meta[5])
    idx = np.arange(0, nnz, STRIDE, dtype=np.int64)
    out = {"meta": meta, "rowptr": rowptr, "sample_idx": idx, "sample_col": col[idx], "sample_val": val[idx],
           "moments": moments.reshape(-1, P), "dos": dos, "targets": targets,
           "val_sum": np.array([val.sum(), np.abs(val).sum(), (val * val).sum()]),
           "row_sum": np.add.reduceat(val, rowptr[:-1].astype(np.int64)),
           "row_abs": np.add.reduceat(np.abs(val), rowptr[:-1].astype(np.int64)),
           "digests": np.array([sha(rowptr), sha(col), sha(val), sha(tv)])}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(f"{name}: N={n} nnz={nnz} P={P} samples={len(idx)} vectors={out['moments'].shape[0]}")


def main():
    if not os.path.exists(REF_DUMP):
        sys.exit("build the reference first: make -f oracle/Makefile.ref -j8")
    names = sys.argv[1:] or sorted(f[:-3] for f in os.listdir(HERE) if f.endswith(".in"))
    for name in names:
        make(name)


if __name__ == "__main__":
    main()
