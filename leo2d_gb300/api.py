"""Python view of the C ABI (include/leo2d_gpu.h) used by the tests and bench.

Every call goes straight to libleo2d_gb300.so; failures raise Leo2dError with
the library's status and message. There is no computation in Python and no
fallback: without the library or a CUDA device the calls raise.
"""
import ctypes

import numpy as np

from . import _abi
from ._abi import Geom, KpmCfg


class Leo2dError(RuntimeError):
    def __init__(self, status, msg):
        name = _abi.STATUS_NAMES[status] if 0 <= status < len(_abi.STATUS_NAMES) else str(status)
        super().__init__(f"LEO2D_ERR_{name}: {msg}")
        self.status = status


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Context:
    def __init__(self, device=0):
        self.lib = _abi.load()
        h = ctypes.c_void_p()
        st = self.lib.leo2d_ctx_create(ctypes.byref(h), device)
        if st != _abi.OK:
            raise Leo2dError(st, "leo2d_ctx_create failed (see stderr)")
        self.h = h

    def check(self, st):
        if st != _abi.OK:
            msg = self.lib.leo2d_last_error(self.h)
            raise Leo2dError(st, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.lib.leo2d_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- profiling -------------------------------------------------------
    def set_profiling(self, on):
        self.check(self.lib.leo2d_ctx_set_profiling(self.h, 1 if on else 0))

    def kernel_stats(self, name):
        n = ctypes.c_int64()
        ms = ctypes.c_double()
        self.check(self.lib.leo2d_ctx_kernel_stats(self.h, name.encode(), ctypes.byref(n),
                                                   ctypes.byref(ms)))
        return n.value, ms.value

    def reset_stats(self):
        self.check(self.lib.leo2d_ctx_reset_stats(self.h))

    def launch_count(self):
        return self.lib.leo2d_ctx_launch_count(self.h)

    def set_option(self, key, value):
        self.check(self.lib.leo2d_ctx_set_option(self.h, key.encode(), int(value)))

    def set_spin_limit(self, n):
        self.check(self.lib.leo2d_ctx_set_spin_limit(self.h, n))

    # -- assembly --------------------------------------------------------
    def prepare(self, geom):
        g = Geom()
        ctypes.memmove(ctypes.byref(g), ctypes.byref(geom), ctypes.sizeof(Geom))
        self.check(self.lib.leo2d_geom_prepare(ctypes.byref(g)))
        return g

    def build_csr(self, geom, keep_zeros=False, with_dx=False):
        g = geom if geom.prepared else self.prepare(geom)
        flags = (_abi.CSR_KEEP_ZEROS if keep_zeros else 0) | (_abi.CSR_WITH_DX if with_dx else 0)
        h = ctypes.c_void_p()
        self.check(self.lib.leo2d_build_csr(self.h, ctypes.byref(g), flags, ctypes.byref(h)))
        return Csr(self, h)

    def upload_csr(self, rowptr, col, val, val_dx=None, pos=None):
        rowptr = np.ascontiguousarray(rowptr, np.int64)
        col = np.ascontiguousarray(col, np.int32)
        val = np.ascontiguousarray(val, np.float64)
        if val_dx is not None:
            val_dx = np.ascontiguousarray(val_dx, np.float64)
        if pos is not None:
            pos = np.ascontiguousarray(pos, np.float64)
        h = ctypes.c_void_p()
        self.check(self.lib.leo2d_csr_upload(self.h, len(rowptr) - 1, len(col), _p(rowptr), _p(col),
                                             _p(val), _p(val_dx), _p(pos), ctypes.byref(h)))
        return Csr(self, h)

    # -- transforms ------------------------------------------------------
    def dos_transform(self, mu, P, rescale, shift, scale=1.0):
        mu = np.ascontiguousarray(mu, np.float64).reshape(-1, P)
        dos = np.zeros(P)
        E = np.zeros(P)
        self.check(self.lib.leo2d_dos_transform(self.h, _p(mu), P, mu.shape[0], rescale, shift,
                                                scale, _p(dos), _p(E)))
        return dos, E

    def cond_transform(self, M):
        M = np.ascontiguousarray(M, np.float64)
        out = np.zeros_like(M)
        self.check(self.lib.leo2d_cond_transform(self.h, _p(M), M.shape[0], _p(out)))
        return out

    def cond_sigma(self, mu, energies, rescale, center, scale=1.0):
        mu = np.ascontiguousarray(mu, np.float64)
        E = np.ascontiguousarray(energies, np.float64)
        out = np.zeros(len(E))
        self.check(self.lib.leo2d_cond_sigma(self.h, _p(mu), mu.shape[0], _p(E), len(E), rescale,
                                             center, scale, _p(out)))
        return out

    def tc_gemm(self, a_bf16, b_bf16):
        """D = A B^T on the tensor cores; a [M][K], b [N][K] as uint16 BF16 bits."""
        a = np.ascontiguousarray(a_bf16, np.uint16)
        b = np.ascontiguousarray(b_bf16, np.uint16)
        M, K = a.shape
        N, K2 = b.shape
        if K != K2:
            raise ValueError("inner dimensions differ")
        d = np.zeros((M, N), np.float32)
        self.check(self.lib.leo2d_tc_gemm(self.h, _p(a), _p(b), M, N, K, _p(d)))
        return d

    def tc_gemm_tf32x3(self, a, b):
        """D [128][N] = A [128][K] B [N][K]^T from three TF32 tensor-core products per K step."""
        a = np.ascontiguousarray(a, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        if a.shape[0] != 128 or a.shape[1] != b.shape[1]:
            raise ValueError("a must be [128][K] and b [N][K]")
        d = np.zeros((128, b.shape[0]), np.float32)
        self.check(self.lib.leo2d_tc_gemm_tf32x3(self.h, _p(a), _p(b), b.shape[0], b.shape[1], _p(d)))
        return d

    def dos_reconstruct(self, mu, energies, rescale, center, scale=1.0):
        mu = np.ascontiguousarray(mu, np.float64)
        E = np.ascontiguousarray(energies, np.float64)
        out = np.zeros(len(E))
        self.check(self.lib.leo2d_dos_reconstruct(self.h, _p(mu), len(mu), _p(E), len(E), rescale,
                                                  center, scale, _p(out)))
        return out


def vacancy_rows(n, vacancies, orbitals):
    """Rows of `orbitals` (reference numbering) in the matrix with `vacancies`
    removed: i - (removed orbitals below i), as computeDosKPM maps its targets
    (locality.cpp:5963). Duplicates and out-of-range vacancies count nothing."""
    gone = np.zeros(n, bool)
    v = np.asarray(vacancies, np.int64)
    gone[v[(v >= 0) & (v < n)]] = True
    below = np.concatenate([[0], np.cumsum(gone)])
    o = np.asarray(orbitals, np.int64)
    return o - below[o]


def _reciprocal(a2):
    """b1, b2 of the lattice a1, a2 (Locality::getReciprocal, locality.cpp:7215-7262)."""
    a = np.array([[a2[0][0], a2[0][1], 0.0], [a2[1][0], a2[1][1], 0.0], [0.0, 0.0, 1.0]])

    def cross(x, y, d):
        return (x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0])[d]

    den1 = den2 = 0.0
    for j in range(3):
        den1 += a[0][j] * cross(a[1], a[2], j)
        den2 += a[1][j] * cross(a[2], a[0], j)
    return [[2 * np.pi * cross(a[1], a[2], k) / den1 for k in range(2)],
            [2 * np.pi * cross(a[2], a[0], k) / den2 for k in range(2)]]


def k_grid(geom, n1, n2):
    """Bloch vectors of grid k-sampling (K_TYPE = 0, locality.cpp:1617-1650), in job
    order (k1 outer, k2 inner): k = (k1/n1) b1 + (k2/n2) b2, with b1, b2 the
    reciprocal vectors of the prepared supercell (Locality::getReciprocal,
    locality.cpp:7215-7262). Returns [n1 * n2][2]."""
    b = _reciprocal(geom.supercell)
    out = []
    for k1 in range(n1):
        for k2 in range(n2):
            out.append([(k1 / n1) * b[0][0] + (k2 / n2) * b[1][0], (k1 / n1) * b[0][1] + (k2 / n2) * b[1][1]])
    return np.array(out)


def k_path(geom, n, k_type=1):
    """Bloch vectors of a k path (locality.cpp:1655-1990), n points in job order.

    The path runs through corners P_0 .. P_L; point i sits at c = L i / n, on leg j
    = the first with c <= j + 1 (the last leg takes the rest), at
    (j+1-c) P_j + (c-j) P_j+1.
      k_type 1: supercell zone, K -> Gamma -> M -> K
      k_type 2: sheet 0's own zone, Gamma -> M -> K -> Gamma
      k_type 3: supercell zone, Gamma -> M -> K -> K' -> Gamma
    Supercell zone: K = b2 turned by -30 degrees over 2 cos 30, K' = K turned by
    -60 degrees, M = b2 / 2. Sheet 0's zone: b from its lattice turned by its angle
    (Locality::getReciprocal(int), locality.cpp:7168-7213), M = b1 / 2, K = M
    turned by 30 degrees over cos 30. Returns [n][2].

    k_type 4 (locality.cpp:1990-2159): n points on each leg of Gamma -> K -> M ->
    Gamma in the zone of a bilayer (M, N) cell, walked as the driver walks it
    (k_path_gkm). Returns [3 n][2].
    k_type 5 (locality.cpp:2161-2250): the trilayer's K points joined
    (k_path_dirac). Returns [2 n + 1][2]."""
    if k_type == 4:
        return k_path_gkm(geom, n)
    if k_type == 5:
        return k_path_dirac(geom, n)
    gm = [0.0, 0.0]
    if k_type == 1 and geom.num_sheets < 2:  # locality.cpp:1661-1663, as the driver
        raise ValueError("cannot use K_TYPE == 1 (twisted BZ) for a single layer")
    if k_type == 2:
        th = geom.angles[0]
        lat = geom.lattice[0]
        a0 = [[lat[i][0] * np.cos(th) - lat[i][1] * np.sin(th), lat[i][0] * np.sin(th) + lat[i][1] * np.cos(th)]
              for i in range(2)]
        b = _reciprocal(a0)
        h = (np.pi / 3.0) / 2.0
        mm = [b[0][0] / 2.0, b[0][1] / 2.0]
        kk = [(mm[0] * np.cos(h) - mm[1] * np.sin(h)) / np.cos(h), (mm[0] * np.sin(h) + mm[1] * np.cos(h)) / np.cos(h)]
        pts = [gm, mm, kk, gm]
    elif k_type in (1, 3):
        b = _reciprocal(geom.supercell)
        r = 1.0 / (2.0 * np.cos(np.pi / 6))
        kk = [r * (np.cos(-np.pi / 6) * b[1][0] - np.sin(-np.pi / 6) * b[1][1]),
              r * (np.sin(-np.pi / 6) * b[1][0] + np.cos(-np.pi / 6) * b[1][1])]
        mm = [b[1][0] / 2.0, b[1][1] / 2.0]
        if k_type == 1:
            pts = [kk, gm, mm, kk]
        else:
            k2 = [np.cos(-np.pi / 3) * kk[0] - np.sin(-np.pi / 3) * kk[1],
                  np.sin(-np.pi / 3) * kk[0] + np.cos(-np.pi / 3) * kk[1]]
            pts = [gm, mm, kk, k2, gm]
    else:
        raise ValueError("k_type must be 1 to 5")
    legs = len(pts) - 1
    out = []
    for i in range(n):
        c = (float(legs) / n) * i
        j = 0
        while j < legs - 1 and c > j + 1:
            j += 1
        out.append([((j + 1.0) - c) * pts[j][d] + (c - j) * pts[j + 1][d] for d in range(2)])
    return np.array(out)


def _sheet_reciprocal(geom, s):
    """b1, b2 of sheet s's lattice turned by its angle (Locality::getReciprocal(int),
    locality.cpp:7168-7213)."""
    import math
    th = geom.angles[s]
    lat = geom.lattice[s]
    return _reciprocal([[lat[i][0] * math.cos(th) - lat[i][1] * math.sin(th),
                         lat[i][0] * math.sin(th) + lat[i][1] * math.cos(th)] for i in range(2)])


def k_path_gkm(geom, nk):
    """K_TYPE 4's Bloch vectors (locality.cpp:1990-2159): nk points on each leg of
    Gamma -> K -> M -> Gamma of the zone of the (M, N) supercell of a bilayer,
    A = [N M; -M M+N] (M > N) or [M N; -N M+N] in sheet 0's unrotated lattice
    vectors; M = (b1 + b2) / 2 and K = b2 turned by +30 degrees over sqrt 3. Each
    leg runs by the reference's slope and intercept, in its order of operations
    (the second leg adds no intercept; the third runs along y from M when M's
    coordinates are equal). The trilayer's cell [0 q; -q q] puts M on the y axis,
    where the reference's third leg divides by zero (NaN k points): refused.
    Returns [3 nk][2]."""
    import math
    if geom.num_sheets == 3:
        raise ValueError("K_TYPE = 4 on a trilayer: the reference's M -> Gamma leg divides by zero there")
    if geom.num_sheets != 2 or geom.boundary_condition != 1 or (geom.supercell_m == 0 and geom.supercell_n == 0):
        raise ValueError("K_TYPE = 4 samples the zone of a bilayer SUPERCELL_M_N supercell")
    M, N = geom.supercell_m, geom.supercell_n
    A11, A12, A21, A22 = (N, M, -M, M + N) if M > N else (M, N, -N, M + N)
    a = geom.lattice[0]
    sc = [[A11 * a[0][0] + A12 * a[1][0], A11 * a[0][1] + A12 * a[1][1]],
          [A21 * a[0][0] + A22 * a[1][0], A21 * a[0][1] + A22 * a[1][1]]]
    b = _reciprocal(sc)
    r3, al = math.sqrt(3.0), math.pi / 6
    rot = [[math.cos(al), math.sin(al)], [-math.sin(al), math.cos(al)]]
    gm = [0.0, 0.0]
    m = [0.5 * (b[0][i] + b[1][i]) for i in range(2)]
    k = [0.0, 0.0]
    for i in range(2):
        for j in range(2):
            k[i] = k[i] + rot[i][j] * b[1][j] / r3
    s1 = (k[1] - gm[1]) / (k[0] - gm[0])
    s2 = (m[1] - k[1]) / (m[0] - k[0])
    s3 = (gm[1] - m[1]) / (gm[0] - m[0])
    c1 = (k[0] * gm[1] - gm[0] * k[1]) / (k[0] - gm[0])
    c3 = (gm[0] * m[1] - m[0] * gm[1]) / (gm[0] - m[0])
    l1, l2, l3 = k[0] - gm[0], m[0] - k[0], gm[0] - m[0]
    out = []
    for i in range(3 * nk):
        if i < nk:
            out.append([gm[0] + i * l1 / nk, gm[1] + s1 * i * l1 / nk + c1])
        elif i < 2 * nk:
            n2 = i - nk
            out.append([k[0] + n2 * l2 / nk, k[1] + s2 * n2 * l2 / nk])
        else:
            n3 = i - 2 * nk
            if m[0] == m[1]:
                out.append([m[0], m[1] + n3 * (gm[1] - m[1]) / nk])
            else:
                out.append([m[0] + n3 * l3 / nk, m[1] + s3 * n3 * l3 / nk + c3])
    return np.array(out)


def k_path_dirac(geom, nk):
    """K_TYPE 5's Bloch vectors (locality.cpp:2161-2250): the K points of the three
    sheets of a trilayer supercell, K_s = (2 b_s1 + b_s2) / 3 of sheet s's turned
    lattice, joined: nk points from K_0 towards K_1, nk from K_1 towards K_2, each
    on its line's slope and intercept, then K_2. Returns [2 nk + 1][2]."""
    if geom.num_sheets != 3 or geom.boundary_condition != 1:
        raise ValueError("K_TYPE = 5 joins the K points of a trilayer supercell's three sheets")
    kl = []
    for s in range(3):
        b = _sheet_reciprocal(geom, s)
        kl.append([1.0 / 3.0 * (2.0 * b[0][i] + b[1][i]) for i in range(2)])
    s1 = (kl[1][1] - kl[0][1]) / (kl[1][0] - kl[0][0])
    s2 = (kl[2][1] - kl[1][1]) / (kl[2][0] - kl[1][0])
    m1 = kl[1][1] - s1 * kl[1][0]
    m2 = kl[2][1] - s2 * kl[2][0]
    l1, l2 = kl[1][0] - kl[0][0], kl[2][0] - kl[1][0]
    out = []
    for i in range(2 * nk + 1):
        if i < nk:
            kx = kl[0][0] + i * l1 / nk
            out.append([kx, s1 * kx + m1])
        elif i < 2 * nk:
            kx = kl[1][0] + (i - nk) * l2 / nk
            out.append([kx, s2 * kx + m2])
        else:
            out.append([kl[2][0], kl[2][1]])
    return np.array(out)


def run_input(path, out_dir=".", device=0):
    """The `leo2d` driver through the C ABI; raises Leo2dError with the reason."""
    lib = _abi.load()
    buf = ctypes.create_string_buffer(2048)
    st = lib.leo2d_run_input(str(path).encode(), str(out_dir).encode(), device, buf, len(buf))
    if st != _abi.OK:
        raise Leo2dError(st, buf.value.decode())


def kpm_cfg(P, R=1, kind=_abi.VEC_PHASE, precision=_abi.FP32, block=0, rows_per_warp=0, seed=0,
            first_vector=0):
    c = KpmCfg()
    c.poly_order, c.num_vectors, c.vector_kind, c.precision = P, R, kind, precision
    c.block, c.rows_per_warp, c.seed, c.first_vector = block, rows_per_warp, seed, first_vector
    return c


class Csr:
    def __init__(self, ctx, h):
        self.ctx = ctx
        self.h = h
        n, nnz, ni, ne = (ctypes.c_int64() for _ in range(4))
        ctx.check(ctx.lib.leo2d_csr_info(h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(ni),
                                         ctypes.byref(ne)))
        self.n, self.nnz, self.n_intra, self.n_inter = n.value, nnz.value, ni.value, ne.value

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.leo2d_csr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def download(self, dx=False):
        rp = np.zeros(self.n + 1, np.int64)
        col = np.zeros(self.nnz, np.int32)
        val = np.zeros(self.nnz)
        vdx = np.zeros(self.nnz) if dx else None
        vdy = np.zeros(self.nnz) if dx else None
        self.ctx.check(self.ctx.lib.leo2d_csr_download(self.ctx.h, self.h, _p(rp), _p(col), _p(val),
                                                       _p(vdx), _p(vdy)))
        return (rp, col, val, vdx, vdy) if dx else (rp, col, val)

    def remove_orbitals(self, orbitals):
        """The matrix with these orbitals (vacancies, 0-based) removed, the rest
        renumbered in order (the reference's vacancy solvers); a new Csr."""
        orb = np.ascontiguousarray(orbitals, np.int64)
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.leo2d_csr_remove_orbitals(self.ctx.h, self.h, _p(orb) if len(orb) else None,
                                                              len(orb), ctypes.byref(h)))
        return Csr(self.ctx, h)

    def download_imag(self):
        """Imaginary parts of the stored entries (a complex Hamiltonian: b_field != 0)."""
        im = np.zeros(self.nnz)
        self.ctx.check(self.ctx.lib.leo2d_csr_download_imag(self.ctx.h, self.h, _p(im)))
        return im

    def geometry(self):
        grid = np.zeros(4 * self.n, np.int32)
        pos = np.zeros(3 * self.n)
        self.ctx.check(self.ctx.lib.leo2d_csr_geometry(self.ctx.h, self.h, _p(grid), _p(pos)))
        return grid, pos

    def shift_configs(self):
        """Per-orbital disregistry [n][2] (Hstruct::getShiftConfigs); bilayers."""
        out = np.zeros((self.n, 2))
        self.ctx.check(self.ctx.lib.leo2d_csr_shift_configs(self.ctx.h, self.h, _p(out)))
        return out

    def site_features(self, twist_deg):
        """The learned control variate's 16 feature columns of every orbital [n][16]."""
        x = np.zeros((self.n, 16), np.float32)
        self.ctx.check(self.ctx.lib.leo2d_mlp_site_features(self.ctx.h, self.h, twist_deg, _p(x)))
        return x

    def tc_info(self):
        """Tensor-core tiles: (tiles, mean window, largest window, most entries per tile)."""
        t, w, mw, me = ctypes.c_int64(), ctypes.c_double(), ctypes.c_int32(), ctypes.c_int32()
        self.ctx.check(self.ctx.lib.leo2d_csr_tc_info(self.h, ctypes.byref(t), ctypes.byref(w), ctypes.byref(mw),
                                                      ctypes.byref(me)))
        return t.value, w.value, mw.value, me.value

    def rb_info(self):
        """Row blocks: (blocks, slots stored, distinct slots, most slots of a block, largest tile bytes)."""
        b, s, u, ms, mt = (ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32(),
                           ctypes.c_int64())
        self.ctx.check(self.ctx.lib.leo2d_csr_rb_info(self.h, ctypes.byref(b), ctypes.byref(s), ctypes.byref(u),
                                                      ctypes.byref(ms), ctypes.byref(mt)))
        return b.value, s.value, u.value, ms.value, mt.value

    def rt_info(self):
        """8-row blocks of the tensor-core step: (blocks, k-steps stored, distinct slots, most slots of a block)."""
        b, k, u, ms = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int32()
        self.ctx.check(self.ctx.lib.leo2d_csr_rt_info(self.h, ctypes.byref(b), ctypes.byref(k), ctypes.byref(u),
                                                      ctypes.byref(ms)))
        return b.value, k.value, u.value, ms.value

    def bounds(self):
        lo, hi = ctypes.c_double(), ctypes.c_double()
        self.ctx.check(self.ctx.lib.leo2d_csr_bounds(self.ctx.h, self.h, ctypes.byref(lo),
                                                     ctypes.byref(hi)))
        return lo.value, hi.value

    def rescale(self, rescale, shift):
        self.ctx.check(self.ctx.lib.leo2d_csr_rescale(self.ctx.h, self.h, rescale, shift))

    def kpm_dos(self, cfg, host_vectors=None):
        mu = np.zeros((cfg.num_vectors, cfg.poly_order))
        hv = None if host_vectors is None else np.ascontiguousarray(host_vectors, np.float64)
        self.ctx.check(self.ctx.lib.leo2d_kpm_dos(self.ctx.h, self.h, ctypes.byref(cfg), _p(hv),
                                                  _p(mu)))
        return mu

    def kpm_dos_cv(self, mlp, cfg, twist_deg, num_sites, site_seed=0, weights=None, parts=False):
        """Trace moments [P] with the network as control variate (leo2d_kpm_dos_cv)."""
        P = cfg.poly_order
        mu = np.zeros(P)
        w = None if weights is None else np.ascontiguousarray(weights, np.float64)
        pt = np.zeros((3, 256)) if parts else None
        self.ctx.check(self.ctx.lib.leo2d_kpm_dos_cv(self.ctx.h, self.h, mlp.h, ctypes.byref(cfg), twist_deg,
                                                     num_sites, site_seed, _p(w), _p(mu), _p(pt)))
        return (mu, pt) if parts else mu

    def step_kernel(self, cfg):
        """(kernel, block): the step kernel a kpm_dos call with cfg runs (0 tiled, 1 register,
        2 tensor cores, 3 row blocks) and its vector-block width."""
        k, b = ctypes.c_int32(), ctypes.c_int32()
        self.ctx.check(self.ctx.lib.leo2d_kpm_step_kernel(self.ctx.h, self.h, ctypes.byref(cfg),
                                                          ctypes.byref(k), ctypes.byref(b)))
        return k.value, b.value

    def autotune(self, cfg):
        b, r = ctypes.c_int32(), ctypes.c_int32()
        self.ctx.check(self.ctx.lib.leo2d_kpm_autotune(self.ctx.h, self.h, ctypes.byref(cfg),
                                                       ctypes.byref(b), ctypes.byref(r)))
        return b.value, r.value

    def kpm_cond(self, cfg, targets=None):
        P = cfg.poly_order
        if targets is None:
            out = np.zeros((P, P))
            self.ctx.check(self.ctx.lib.leo2d_kpm_cond(self.ctx.h, self.h, ctypes.byref(cfg), None, 0,
                                                       _p(out)))
            return out
        t = np.ascontiguousarray(targets, np.int64)
        out = np.zeros((len(t), P, P))
        self.ctx.check(self.ctx.lib.leo2d_kpm_cond(self.ctx.h, self.h, ctypes.byref(cfg), _p(t), len(t),
                                                   _p(out)))
        return out

    def kpm_ldos(self, cfg, targets):
        t = np.ascontiguousarray(targets, np.int64)
        mu = np.zeros((len(t), cfg.poly_order))
        self.ctx.check(self.ctx.lib.leo2d_kpm_ldos(self.ctx.h, self.h, ctypes.byref(cfg), _p(t), len(t),
                                                   _p(mu)))
        return mu


class Batch:
    """Several rescaled matrices run together: one launch per Chebyshev step, one
    CUDA graph per run (leo2d_batch_*). The matrices must outlive the batch."""

    def __init__(self, ctx, csrs, cfg):
        self.ctx = ctx
        self.csrs = list(csrs)  # keeps the matrices alive
        self.cfg = cfg
        arr = (ctypes.c_void_p * len(self.csrs))(*[c.h for c in self.csrs])
        h = ctypes.c_void_p()
        ctx.check(ctx.lib.leo2d_batch_create(ctx.h, arr, len(self.csrs), ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        cols, warps, rows, grid = (ctypes.c_int32() for _ in range(4))
        lpr = ctypes.c_int64()
        ctx.check(ctx.lib.leo2d_batch_info(h, ctypes.byref(cols), ctypes.byref(warps), ctypes.byref(rows),
                                           ctypes.byref(grid), ctypes.byref(lpr)))
        self.block_cols, self.warps, self.rows_per_item = cols.value, warps.value, rows.value
        self.grid, self.launches_per_run = grid.value, lpr.value

    def run(self, seed=None, first_vector=None):
        """Moments [num matrices][R][P] of one replay."""
        seed = self.cfg.seed if seed is None else seed
        first = self.cfg.first_vector if first_vector is None else first_vector
        mu = np.zeros((len(self.csrs), self.cfg.num_vectors, self.cfg.poly_order))
        self.ctx.check(self.ctx.lib.leo2d_batch_run(self.h, seed, first, _p(mu)))
        return mu

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.leo2d_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mlp:
    """The learned control variate's network (leo2d_mlp_*): 16 site features ->
    3 x 256 GELU -> the first 256 site-resolved Chebyshev moments, on the
    tensor cores."""

    N_OUT = 256

    def __init__(self, ctx, seed=0):
        self.ctx = ctx
        h = ctypes.c_void_p()
        ctx.check(ctx.lib.leo2d_mlp_create(ctx.h, seed, ctypes.byref(h)))
        self.h = h
        self.n_params = ctx.lib.leo2d_mlp_param_count()

    def params(self):
        p = np.zeros(self.n_params, np.float32)
        self.ctx.check(self.ctx.lib.leo2d_mlp_get_params(self.h, _p(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.n_params:
            raise ValueError("wrong parameter count")
        self.ctx.check(self.ctx.lib.leo2d_mlp_set_params(self.h, _p(p)))

    def set_loss_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        self.ctx.check(self.ctx.lib.leo2d_mlp_set_loss_weights(self.h, _p(w)))

    def grad(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        loss = ctypes.c_double()
        g = np.zeros(self.n_params, np.float32)
        self.ctx.check(self.ctx.lib.leo2d_mlp_grad(self.h, _p(x), x.shape[1], _p(t), x.shape[0],
                                                   ctypes.byref(loss), _p(g)))
        return loss.value, g

    def train(self, x, t, steps, batch=4096, lr=1e-3, seed=0):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        hist = np.zeros(max(steps, 1))
        self.ctx.check(self.ctx.lib.leo2d_mlp_train(self.h, _p(x), x.shape[1], _p(t), x.shape[0], steps, batch,
                                                    lr, seed, _p(hist)))
        return hist[:steps]

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((x.shape[0], self.N_OUT), np.float32)
        self.ctx.check(self.ctx.lib.leo2d_mlp_predict(self.h, _p(x), x.shape[1], x.shape[0], _p(y)))
        return y

    def site_sum(self, csr, twist_deg):
        out = np.zeros(self.N_OUT)
        self.ctx.check(self.ctx.lib.leo2d_mlp_site_sum(self.h, csr.h, twist_deg, _p(out)))
        return out

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.leo2d_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
