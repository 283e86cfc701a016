"""Shared helpers: load golden fixtures and rebuild their geometry specs."""
import gzip
import math
import os

import numpy as np

from leo2d_gb300._abi import Geom, MODEL_REF

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def e2e_text(name, suffix):
    with gzip.open(os.path.join(GOLDEN, "e2e", name + suffix + ".gz"), "rt") as f:
        return f.read()


def load_config(name):
    """Digests of a full-size workload (tests/golden/configs)."""
    with np.load(os.path.join(GOLDEN, "configs", name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def parse_in(name, folder="inputs"):
    """Reads a fixture's .in with the token rules of main.cpp:75-911 (subset).

    Test helper only: the product parser is C++ (leo2d_gb300/host/input.cpp)
    and is checked against the same files.
    """
    path = os.path.join(GOLDEN, folder, name + ".in")
    g = Geom()
    g.sc_search_size = 1
    g.model = MODEL_REF
    mn = mx = None
    max_R = 0.0
    height = angle = 0.0
    cur = -1
    kv = {"target_sheets": []}
    for line in open(path):
        tk = line.rstrip("\n").split(" ")
        for p, key in enumerate(tk):
            v = lambda k: tk[p + k] if p + k < len(tk) else ""
            if key == "MAXSIZE":
                mx = int(v(2)); max_R = float(mx)
            elif key == "MINSIZE":
                mn = int(v(2))
            elif key == "MAX_R":
                max_R = float(v(2))
            elif key == "BOUNDARY_CONDITION":
                g.boundary_condition = int(v(2))
                kv["periodic"] = g.boundary_condition == 1
            elif key == "NUM_SHEETS":
                g.num_sheets = int(v(2))
            elif key == "SUPERCELL_M_N":
                g.supercell_m, g.supercell_n = int(v(2)), int(v(3))
                g.trilayer_supercell = 0
            elif key == "TRILAYER_SUPERCELL":
                if int(v(2)) == 1:
                    g.trilayer_supercell = 1
            elif key == "START_SHEET":
                cur = int(v(1)) - 1
            elif key == "END_SHEET":
                if cur == int(v(1)) - 1:
                    g.heights[cur] = height
                    g.angles[cur] = angle
                    cur = -1
            elif key == "MATERIAL":
                g.min_shape[cur][0] = g.min_shape[cur][1] = mn
                g.max_shape[cur][0] = g.max_shape[cur][1] = mx
                g.max_R[cur] = max_R
            elif key == "HEIGHT":
                height = float(v(2))
            elif key == "ANGLE":
                angle = (2 * math.pi * float(v(2))) / (360.0)
            elif key == "ENERGY_RESCALE":
                g.energy_rescale = float(v(2))
            elif key == "ENERGY_SHIFT":
                g.energy_shift = float(v(2))
            elif key == "POLY_ORDER":
                kv["P"] = int(v(2))
            elif key == "TARGET_SHEETS":
                kv["target_sheets"] = [int(v(2)) - 1]
            elif key == "USE_B_FIELD":
                kv["use_b"] = int(v(2))
            elif key == "B_FIELD":
                kv["b_field"] = float(v(2))
            elif key == "SOLVER_TYPE":
                kv["solver"] = v(2)
            elif key == "USE_E_FIELD":
                kv["use_e"] = int(v(2))
            elif key == "E_FIELD":
                kv["e_field"] = float(v(2))
            elif key == "REF_DUMP_KVEC":  # a fixture-generator key: the job's Bloch vector
                kv["k_vec"] = [float(x) for x in v(2).split(",")]
            elif key == "REF_DUMP_SHIFT":  # a fixture-generator key: "sheet,s1,s2" of the job
                sh = v(2).split(",")
                kv["shift"] = (int(sh[0]) - 1, float(sh[1]), float(sh[2]))
    if kv.get("use_b"):
        g.b_field = kv.get("b_field", 0.0)
    if kv.get("use_e"):
        g.e_field = kv.get("e_field", 0.0)
    if "k_vec" in kv:
        g.k_vec[0], g.k_vec[1] = kv["k_vec"]
    if kv.get("solver") == "FIXED_SHIFT":  # its one job shifts every sheet but the first
        for s in range(1, g.num_sheets):
            g.shifts[s][0] = g.shifts[s][1] = 1.0 / 3.0
    if "shift" in kv:
        s, a, b = kv["shift"]
        g.shifts[s][0], g.shifts[s][1] = a, b
    return g, kv


ALL = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))
# real Hamiltonians (generateRealH) and complex ones in a magnetic field (generateCpxH)
CASES = [c for c in ALL if "bfield" not in c and "_vac_" not in c and "_kvec_" not in c]
BFIELD_CASES = [c for c in ALL if "bfield" in c]
# complex Hamiltonians: a magnetic field, or a Bloch vector of a k-sampled periodic job
KVEC_CASES = [c for c in ALL if "_kvec_" in c]
# the cases whose .cheb and _matrix.dat the reference's own main() wrote
E2E_CASES = [c for c in CASES if os.path.exists(os.path.join(GOLDEN, "e2e", c + ".cheb.gz"))]
COMPLEX_CASES = BFIELD_CASES + KVEC_CASES
# vacancies (the vacancy solvers' matrix): <base>_vac_<kind> pairs with <base>_<kind>
VAC_CASES = [c for c in ALL if "_vac_" in c]


def vac_base(name):
    """The fixture of the same job without vacancies."""
    return name.replace("_vac_", "_")
