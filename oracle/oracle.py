"""Python binding of the CPU oracle (oracle/leo2d_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the tests, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use it as the checker. The GPU library never imports it.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
if REPO not in sys.path:
    sys.path.insert(0, REPO)
from leo2d_gb300._abi import Geom, make_geom  # noqa: E402  (struct layout only)

LIB = os.path.join(HERE, "liboracle.so")
SRC = [os.path.join(HERE, "leo2d_oracle.cpp"), os.path.join(HERE, "cpu_baseline.cpp")]


def build(force=False):
    """Compiles liboracle.so with -ffp-contract=off (no fused multiply-add)."""
    newest = max(os.path.getmtime(p) for p in SRC + [os.path.join(HERE, "leo2d_oracle.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
           "-o", LIB] + SRC
    subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Built:
    """Geometry + pairs + CSR of one job (stored zeros kept), host arrays."""

    def __init__(self, geom):
        L = lib()
        g = Geom()
        ctypes.memmove(ctypes.byref(g), ctypes.byref(geom), ctypes.sizeof(Geom))
        if not g.prepared:
            if L.oracle_geom_prepare(ctypes.byref(g)) != 0:
                raise ValueError("oracle_geom_prepare failed")
        self.geom = g
        h = ctypes.c_void_p()
        if L.oracle_build(ctypes.byref(g), ctypes.byref(h)) != 0:
            raise ValueError("oracle_build failed")
        n, nnz, ni, ne = (ctypes.c_int64() for _ in range(4))
        L.oracle_info(h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(ni), ctypes.byref(ne))
        self.n, self.nnz, self.n_intra, self.n_inter = n.value, nnz.value, ni.value, ne.value
        N, NNZ = self.n, self.nnz
        self.rowptr = np.zeros(N + 1, np.int64)
        self.col = np.zeros(NNZ, np.int32)
        self.val = np.zeros(NNZ)
        self.val_dx = np.zeros(NNZ)
        self.val_dy = np.zeros(NNZ)
        self.index_to_grid = np.zeros(4 * N, np.int32)
        self.pos = np.zeros(3 * N)
        L.oracle_get(h, _p(self.rowptr), _p(self.col), _p(self.val), _p(self.val_dx),
                     _p(self.val_dy), _p(self.index_to_grid), _p(self.pos))
        self.intra_pairs = np.zeros(2 * self.n_intra, np.int32)
        self.intra_t = np.zeros(self.n_intra)
        self.intra_sc = np.zeros(2 * self.n_intra, np.int32)
        self.inter_pairs = np.zeros(2 * self.n_inter, np.int32)
        self.inter_sc = np.zeros(2 * self.n_inter, np.int32)
        L.oracle_get_pairs(h, _p(self.intra_pairs), _p(self.intra_t), _p(self.intra_sc),
                           _p(self.inter_pairs), _p(self.inter_sc))
        self._h = h

    def shift_configs(self):
        """Per-orbital disregistry [n][2] (Hstruct::getShiftConfigs); bilayers only."""
        out = np.zeros(2 * self.n)
        if lib().oracle_shift_configs(self._h, _p(out)) != 0:
            raise ValueError("shift configurations need exactly two sheets")
        return out.reshape(self.n, 2)

    def targets(self, target_sheets):
        ts = np.asarray(target_sheets, np.int32)
        out = np.zeros(16 * len(ts), np.int64)
        c = lib().oracle_targets(self._h, _p(ts), ctypes.c_int32(len(ts)), _p(out),
                                 ctypes.c_int64(len(out)))
        return out[:c]

    def bloch(self, kx, ky):
        """(re, im) of the k-sampled job's complex H~ (generateCpxH with k_vec), CSR order."""
        re, im = np.zeros(self.nnz), np.zeros(self.nnz)
        lib().oracle_bloch(self._h, ctypes.c_double(kx), ctypes.c_double(ky), _p(re), _p(im))
        return re, im

    def compact(self):
        """(rowptr, col, val) without the entries whose value is exactly zero."""
        keep = self.val != 0.0
        counts = np.add.reduceat(keep.astype(np.int64), self.rowptr[:-1]) if self.nnz else None
        rp = np.zeros(self.n + 1, np.int64)
        if self.nnz:
            empty = self.rowptr[:-1] == self.rowptr[1:]
            counts[empty] = 0
            rp[1:] = np.cumsum(counts)
        return rp, self.col[keep], self.val[keep]

    def __del__(self):
        try:
            lib().oracle_free(self._h)
        except Exception:
            pass


def geom_prepare(geom):
    g = Geom()
    ctypes.memmove(ctypes.byref(g), ctypes.byref(geom), ctypes.sizeof(Geom))
    if lib().oracle_geom_prepare(ctypes.byref(g)) != 0:
        raise ValueError("oracle_geom_prepare failed")
    return g


def _csr_args(rowptr, col, val):
    return (ctypes.c_int64(len(rowptr) - 1), _p(np.ascontiguousarray(rowptr, np.int64)),
            _p(np.ascontiguousarray(col, np.int32)), _p(np.ascontiguousarray(val, np.float64)))


def kpm_trace(rowptr, col, val, vectors, P, literal=True):
    rowptr = np.ascontiguousarray(rowptr, np.int64)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    vectors = np.ascontiguousarray(vectors, np.float64)
    R = vectors.shape[0]
    mu = np.zeros((R, P))
    f = lib().oracle_kpm_trace if literal else lib().oracle_kpm_trace_doubling
    f(ctypes.c_int64(len(rowptr) - 1), _p(rowptr), _p(col), _p(val), ctypes.c_int32(R),
      _p(vectors), ctypes.c_int32(P), _p(mu))
    return mu


def peierls(rowptr, col, val, pos, B):
    """Complex H~ of a flake in the field B (tesla): (re, im) per entry."""
    rowptr = np.ascontiguousarray(rowptr, np.int64)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    pos = np.ascontiguousarray(pos, np.float64).reshape(-1)
    re, im = np.zeros(len(val)), np.zeros(len(val))
    lib().oracle_peierls(ctypes.c_int64(len(rowptr) - 1), _p(rowptr), _p(col), _p(val), _p(pos),
                         ctypes.c_double(B), _p(re), _p(im))
    return re, im


def kpm_trace_cpx(rowptr, col, re, im, vectors, P):
    """computeDosTraceKPM's complex branch with real start vectors [R][n]."""
    args = [np.ascontiguousarray(x, t) for x, t in ((rowptr, np.int64), (col, np.int32), (re, np.float64),
                                                    (im, np.float64), (vectors, np.float64))]
    R = args[4].shape[0]
    mu = np.zeros((R, P))
    lib().oracle_kpm_trace_cpx(ctypes.c_int64(len(rowptr) - 1), *(_p(a) for a in args[:4]), ctypes.c_int32(R),
                               _p(args[4]), ctypes.c_int32(P), _p(mu))
    return mu


def kpm_ldos_cpx(rowptr, col, re, im, targets, P):
    args = [np.ascontiguousarray(x, t) for x, t in ((rowptr, np.int64), (col, np.int32), (re, np.float64),
                                                    (im, np.float64), (targets, np.int64))]
    mu = np.zeros((len(targets), P))
    lib().oracle_kpm_ldos_cpx(ctypes.c_int64(len(rowptr) - 1), *(_p(a) for a in args[:5]),
                              ctypes.c_int64(len(targets)), ctypes.c_int32(P), _p(mu))
    return mu


def kpm_trace_cpx_doubling(rowptr, col, re, im, vre, vim, P):
    """Complex recursion from complex start vectors, every moment by doubling."""
    args = [np.ascontiguousarray(x, t) for x, t in ((rowptr, np.int64), (col, np.int32), (re, np.float64),
                                                    (im, np.float64), (vre, np.float64), (vim, np.float64))]
    R = args[4].shape[0]
    mu = np.zeros((R, P))
    lib().oracle_kpm_trace_cpx_doubling(ctypes.c_int64(len(rowptr) - 1), *(_p(a) for a in args[:4]),
                                        ctypes.c_int32(R), _p(args[4]), _p(args[5]), ctypes.c_int32(P), _p(mu))
    return mu


def kpm_ldos(rowptr, col, val, targets, P):
    rowptr = np.ascontiguousarray(rowptr, np.int64)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    targets = np.ascontiguousarray(targets, np.int64)
    mu = np.zeros((len(targets), P))
    lib().oracle_kpm_ldos(ctypes.c_int64(len(rowptr) - 1), _p(rowptr), _p(col), _p(val),
                          _p(targets), ctypes.c_int64(len(targets)), ctypes.c_int32(P), _p(mu))
    return mu


def kpm_cond(rowptr, col, val, val_dx, targets, P):
    rowptr = np.ascontiguousarray(rowptr, np.int64)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    val_dx = np.ascontiguousarray(val_dx, np.float64)
    targets = np.ascontiguousarray(targets, np.int64)
    out = np.zeros((len(targets), P, P))
    lib().oracle_kpm_cond(ctypes.c_int64(len(rowptr) - 1), _p(rowptr), _p(col), _p(val),
                          _p(val_dx), _p(targets), ctypes.c_int64(len(targets)),
                          ctypes.c_int32(P), _p(out))
    return out


def kpm_cond_trace(rowptr, col, val, val_dx, vectors, M):
    rowptr = np.ascontiguousarray(rowptr, np.int64)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    val_dx = np.ascontiguousarray(val_dx, np.float64)
    vectors = np.ascontiguousarray(vectors, np.float64)
    out = np.zeros((M, M))
    lib().oracle_kpm_cond_trace(ctypes.c_int64(len(rowptr) - 1), _p(rowptr), _p(col), _p(val),
                                _p(val_dx), ctypes.c_int32(vectors.shape[0]), _p(vectors),
                                ctypes.c_int32(M), _p(out))
    return out


def dos_transform(mu, P, rescale, shift, scale=1.0):
    mu = np.ascontiguousarray(mu, np.float64).reshape(-1, P)
    dos = np.zeros(P)
    E = np.zeros(P)
    lib().oracle_dos_transform(_p(mu), ctypes.c_int32(P), ctypes.c_int32(mu.shape[0]),
                               ctypes.c_double(rescale), ctypes.c_double(shift),
                               ctypes.c_double(scale), _p(dos), _p(E))
    return dos, E


def dos_reconstruct(mu, energies, rescale, center, scale=1.0):
    mu = np.ascontiguousarray(mu, np.float64)
    E = np.ascontiguousarray(energies, np.float64)
    out = np.zeros(len(E))
    lib().oracle_dos_reconstruct(_p(mu), ctypes.c_int32(len(mu)), _p(E), ctypes.c_int64(len(E)),
                                 ctypes.c_double(rescale), ctypes.c_double(center),
                                 ctypes.c_double(scale), _p(out))
    return out


def cond_transform(M):
    M = np.ascontiguousarray(M, np.float64)
    P = M.shape[0]
    out = np.zeros((P, P))
    lib().oracle_cond_transform(_p(M), ctypes.c_int32(P), _p(out))
    return out


def cond_sigma(mu, energies, rescale, center, scale=1.0):
    mu = np.ascontiguousarray(mu, np.float64)
    E = np.ascontiguousarray(energies, np.float64)
    out = np.zeros(len(E))
    lib().oracle_cond_sigma(_p(mu), ctypes.c_int32(mu.shape[0]), _p(E), ctypes.c_int64(len(E)),
                            ctypes.c_double(rescale), ctypes.c_double(center),
                            ctypes.c_double(scale), _p(out))
    return out


def vacancy_reduction(n, orbitals):
    """reduction[i] = removed orbitals below i (workerChebSolve's relabelling); kept count."""
    orb = np.ascontiguousarray(orbitals, np.int64)
    red = np.zeros(n + 1, np.int64)
    lib().oracle_vacancy_reduction.restype = ctypes.c_int64
    kept = lib().oracle_vacancy_reduction(ctypes.c_int64(n), _p(orb), ctypes.c_int64(len(orb)), _p(red))
    return red, int(kept)


def remove_orbitals(rowptr, col, values, orbitals):
    """generateRealH's vacancy skips on a full CSR: (rowptr, col, [values...]) of the
    kept orbitals, renumbered in order; `values` is a list of up to three arrays."""
    lib().oracle_remove_orbitals.restype = ctypes.c_int64
    rowptr = np.ascontiguousarray(rowptr, np.int64)
    col = np.ascontiguousarray(col, np.int32)
    n = len(rowptr) - 1
    red, kept = vacancy_reduction(n, orbitals)
    vals = [np.ascontiguousarray(v, np.float64) for v in values] + [None] * (3 - len(values))
    outs = [np.zeros(len(col)) if v is not None else None for v in vals]
    rp = np.zeros(kept + 1, np.int64)
    c = np.zeros(len(col), np.int32)
    nnz = lib().oracle_remove_orbitals(ctypes.c_int64(n), _p(rowptr), _p(col), *[_p(v) for v in vals],
                                       _p(red), _p(rp), _p(c), *[_p(o) for o in outs])
    return rp, c[:nnz], [o[:nnz] for o in outs if o is not None]


def gershgorin(rowptr, col, val):
    lo, hi = ctypes.c_double(), ctypes.c_double()
    n, a, b, c = _csr_args(rowptr, col, val)
    lib().oracle_gershgorin(n, a, b, c, ctypes.byref(lo), ctypes.byref(hi))
    return lo.value, hi.value


def phase_vectors(seed, first_vector, R, n):
    re = np.zeros((R, n))
    im = np.zeros((R, n))
    lib().oracle_phase_vectors(ctypes.c_uint64(seed), ctypes.c_uint64(first_vector),
                               ctypes.c_int32(R), ctypes.c_int64(n), _p(re), _p(im))
    return re, im


def reference_gaussian(R, n):
    out = np.zeros((R, n))
    lib().oracle_reference_gaussian(ctypes.c_int32(R), ctypes.c_int64(n), _p(out))
    return out
