"""ctypes mirror of include/leo2d_gpu.h (the C ABI of libleo2d_gb300.so).

This module only declares types and prototypes and loads the in-tree shared
library. It never computes anything itself: when the library is missing the
load fails with an error that says how to build it.
"""
import ctypes
import os

MAX_SHEETS = 8
HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libleo2d_gb300.so")

c_i32, c_i64, c_u32, c_u64, c_dbl = (ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32,
                                     ctypes.c_uint64, ctypes.c_double)
c_void_p = ctypes.c_void_p

# leo2d_status
OK, ERR_BAD_ARG, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_NONFINITE, ERR_UNSUPPORTED, ERR_IO = range(8)
STATUS_NAMES = ["OK", "BAD_ARG", "OOM", "CUDA", "TIMEOUT", "NONFINITE", "UNSUPPORTED", "IO"]

MODEL_REF, MODEL_SIMPLE = 0, 1
CSR_KEEP_ZEROS, CSR_WITH_DX = 0x1, 0x2
VEC_PHASE, VEC_HOST, VEC_GAUSSIAN = 0, 1, 2
FP32, FP64 = 0, 1


class Geom(ctypes.Structure):
    """leo2d_geom (include/leo2d_gpu.h)."""
    _fields_ = [
        ("num_sheets", c_i32), ("model", c_i32), ("boundary_condition", c_i32),
        ("sc_search_size", c_i32), ("supercell_m", c_i32), ("supercell_n", c_i32),
        ("min_shape", c_i32 * 2 * MAX_SHEETS), ("max_shape", c_i32 * 2 * MAX_SHEETS),
        ("max_R", c_dbl * MAX_SHEETS), ("heights", c_dbl * MAX_SHEETS),
        ("angles", c_dbl * MAX_SHEETS), ("energy_rescale", c_dbl), ("energy_shift", c_dbl),
        ("lattice", c_dbl * 2 * 2 * MAX_SHEETS), ("sheet_supercell", c_dbl * 2 * 2 * MAX_SHEETS),
        ("sheet_sc_stride", c_i32 * 2 * 2 * MAX_SHEETS), ("supercell", c_dbl * 2 * 2),
        ("prepared", c_i32), ("b_field", c_dbl), ("k_vec", c_dbl * 2),
        ("shifts", c_dbl * 2 * MAX_SHEETS), ("e_field", c_dbl), ("trilayer_supercell", c_i32),
    ]


class KpmCfg(ctypes.Structure):
    """leo2d_kpm_cfg (include/leo2d_gpu.h)."""
    _fields_ = [
        ("poly_order", c_i32), ("num_vectors", c_i32), ("vector_kind", c_i32),
        ("precision", c_i32), ("block", c_i32), ("rows_per_warp", c_i32),
        ("seed", c_u64), ("first_vector", c_u64),
    ]


def make_geom(num_sheets=2, model=MODEL_REF, boundary_condition=0, size=50, max_R=None,
              heights=(0.0, 3.35), angles_deg=(0.0, 0.0), energy_rescale=20.0,
              energy_shift=0.0, supercell_mn=None, sc_search_size=1, b_field=0.0, k_vec=None,
              shifts=None, e_field=0.0, trilayer_supercell=0):
    """A Geom filled the way main.cpp fills Sdata for MAXSIZE=size, MINSIZE=-size.

    Angles are given in degrees and converted as main.cpp:345-351 does.
    """
    import math
    g = Geom()
    g.num_sheets = num_sheets
    g.model = model
    g.boundary_condition = boundary_condition
    g.sc_search_size = sc_search_size
    for s in range(num_sheets):
        g.min_shape[s][0] = -size
        g.min_shape[s][1] = -size
        g.max_shape[s][0] = size
        g.max_shape[s][1] = size
        g.max_R[s] = float(size) if max_R is None else float(max_R)
        g.heights[s] = float(heights[s])
        g.angles[s] = (2 * math.pi * float(angles_deg[s])) / (360.0)
    g.energy_rescale = energy_rescale
    g.energy_shift = energy_shift
    if supercell_mn is not None:
        g.supercell_m, g.supercell_n = supercell_mn
    g.b_field = float(b_field)
    if k_vec is not None:
        g.k_vec[0], g.k_vec[1] = float(k_vec[0]), float(k_vec[1])
    g.e_field = float(e_field)
    g.trilayer_supercell = int(trilayer_supercell)
    if shifts is not None:  # {sheet: (s1, s2)}: fractions of the sheet's lattice vectors
        for s, (a, b) in dict(shifts).items():
            g.shifts[s][0], g.shifts[s][1] = float(a), float(b)
    return g


_lib = None


def load():
    """Loads libleo2d_gb300.so from the package tree (built by __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_GLOBAL)
    _declare(lib)
    _lib = lib
    return lib


P = c_void_p  # any pointer argument (numpy arrays passed via .ctypes.data)


def _declare(lib):
    def fn(name, res, *args):
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = list(args)

    gp = ctypes.POINTER(Geom)
    cp = ctypes.POINTER(KpmCfg)
    pp = ctypes.POINTER(c_void_p)
    fn("leo2d_ctx_create", c_i32, pp, ctypes.c_int)
    fn("leo2d_ctx_destroy", c_i32, c_void_p)
    fn("leo2d_last_error", ctypes.c_char_p, c_void_p)
    fn("leo2d_status_string", ctypes.c_char_p, c_i32)
    fn("leo2d_abi_version", ctypes.c_int)
    fn("leo2d_ctx_stream", c_void_p, c_void_p)
    fn("leo2d_ctx_set_spin_limit", c_i32, c_void_p, c_u64)
    fn("leo2d_ctx_set_profiling", c_i32, c_void_p, ctypes.c_int)
    fn("leo2d_ctx_kernel_stats", c_i32, c_void_p, ctypes.c_char_p, P, P)
    fn("leo2d_ctx_reset_stats", c_i32, c_void_p)
    fn("leo2d_ctx_launch_count", c_i64, c_void_p)
    fn("leo2d_ctx_set_option", c_i32, c_void_p, ctypes.c_char_p, c_i64)
    fn("leo2d_geom_prepare", c_i32, gp)
    fn("leo2d_build_csr", c_i32, c_void_p, gp, c_u32, pp)
    fn("leo2d_csr_destroy", c_i32, c_void_p)
    fn("leo2d_csr_info", c_i32, c_void_p, P, P, P, P)
    fn("leo2d_csr_download", c_i32, c_void_p, c_void_p, P, P, P, P, P)
    fn("leo2d_csr_geometry", c_i32, c_void_p, c_void_p, P, P)
    fn("leo2d_csr_upload", c_i32, c_void_p, c_i64, c_i64, P, P, P, P, P, pp)
    fn("leo2d_csr_bounds", c_i32, c_void_p, c_void_p, P, P)
    fn("leo2d_csr_rescale", c_i32, c_void_p, c_void_p, c_dbl, c_dbl)
    fn("leo2d_csr_shift_configs", c_i32, c_void_p, c_void_p, P)
    fn("leo2d_kpm_dos", c_i32, c_void_p, c_void_p, cp, P, P)
    fn("leo2d_kpm_ldos", c_i32, c_void_p, c_void_p, cp, P, c_i64, P)
    fn("leo2d_kpm_autotune", c_i32, c_void_p, c_void_p, cp, P, P)
    fn("leo2d_kpm_step_kernel", c_i32, c_void_p, c_void_p, cp, P, P)
    fn("leo2d_dos_transform", c_i32, c_void_p, P, c_i32, c_i32, c_dbl, c_dbl, c_dbl, P, P)
    fn("leo2d_dos_reconstruct", c_i32, c_void_p, P, c_i32, P, c_i64, c_dbl, c_dbl, c_dbl, P)
    fn("leo2d_batch_create", c_i32, c_void_p, P, c_i32, cp, pp)
    fn("leo2d_batch_run", c_i32, c_void_p, c_u64, c_u64, P)
    fn("leo2d_batch_info", c_i32, c_void_p, P, P, P, P, P)
    fn("leo2d_batch_destroy", c_i32, c_void_p)
    fn("leo2d_tc_gemm", c_i32, c_void_p, P, P, c_i64, c_i64, c_i64, P)
    fn("leo2d_tc_gemm_tf32x3", c_i32, c_void_p, P, P, c_i64, c_i64, P)
    fn("leo2d_csr_tc_info", c_i32, c_void_p, P, P, P, P)
    fn("leo2d_csr_rb_info", c_i32, c_void_p, P, P, P, P, P)
    fn("leo2d_csr_rt_info", c_i32, c_void_p, P, P, P, P)
    fn("leo2d_csr_download_imag", c_i32, c_void_p, c_void_p, P)
    fn("leo2d_csr_remove_orbitals", c_i32, c_void_p, c_void_p, P, c_i64, pp)
    fn("leo2d_mlp_param_count", c_i64)
    fn("leo2d_mlp_create", c_i32, c_void_p, c_u64, pp)
    fn("leo2d_mlp_destroy", c_i32, c_void_p)
    fn("leo2d_mlp_get_params", c_i32, c_void_p, P)
    fn("leo2d_mlp_set_params", c_i32, c_void_p, P)
    fn("leo2d_mlp_set_loss_weights", c_i32, c_void_p, P)
    fn("leo2d_mlp_grad", c_i32, c_void_p, P, c_i32, P, c_i64, P, P)
    fn("leo2d_mlp_train", c_i32, c_void_p, P, c_i32, P, c_i64, c_i32, c_i32, ctypes.c_float, c_u64, P)
    fn("leo2d_mlp_predict", c_i32, c_void_p, P, c_i32, c_i64, P)
    fn("leo2d_mlp_site_features", c_i32, c_void_p, c_void_p, c_dbl, P)
    fn("leo2d_mlp_site_sum", c_i32, c_void_p, c_void_p, c_dbl, P)
    fn("leo2d_kpm_dos_cv", c_i32, c_void_p, c_void_p, c_void_p, cp, c_dbl, c_i64, c_u64, P, P, P)
    fn("leo2d_kpm_cond", c_i32, c_void_p, c_void_p, cp, P, c_i64, P)
    fn("leo2d_cond_transform", c_i32, c_void_p, P, c_i32, P)
    fn("leo2d_cond_sigma", c_i32, c_void_p, P, c_i32, P, c_i64, c_dbl, c_dbl, c_dbl, P)
    fn("leo2d_run_input", c_i32, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p,
       ctypes.c_size_t)
    fn("leo2d_parse_input", c_i32, ctypes.c_char_p, gp, P, ctypes.c_char_p, ctypes.c_size_t)
    for name, res, args in _EXTRA:
        if hasattr(lib, name):
            fn(name, res, *args)


# entry points declared when present (added alongside their kernels)
_EXTRA = [
    ("leo2d_kpm_dos_noalloc", c_i32, (P, P, P, c_i64, c_i32, c_i32, c_u64, c_u64, P, c_void_p)),
]


def exported_symbols_from_header(header_path=None):
    """Names of every function declared in include/*.h (for the ABI test)."""
    import re
    import glob
    if header_path is None:
        inc = os.path.join(os.path.dirname(HERE), "include")
        paths = sorted(glob.glob(os.path.join(inc, "*.h")))
    else:
        paths = [header_path]
    names = []
    for p in paths:
        txt = open(p).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(leo2d_[a-z0-9_]+)\s*\(", txt):
            if m.group(1) not in names:
                names.append(m.group(1))
    return names
