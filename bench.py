"""Benchmark: time-to-DOS of the KPM path on a 10M-orbital twisted-bilayer flake.

Workload (one GB300): twisted bilayer graphene disk, twist 0.5 deg, radius
2042 A (~1.0e7 pz orbitals), simple model (a = 2.46 A, t = -2.7 eV,
t_perp(r) = 0.33 exp(-(r-3.35)/0.45) eV, r < 8 A), Gershgorin bounds x 1.01,
P = 1024 Chebyshev moments, Jackson kernel, DOS on 4001 energies spanning the
rescaled band. Inputs are synthetic: the geometry is generated by the
library's own GPU assembly.

A step = one DOS estimate from the Hamiltonian resident in HBM: R random-phase
vectors through the fused FP32 Chebyshev recursion (FP64 moment sums), then
the FP64 Jackson/Chebyshev reconstruction. R is the smallest number of
vectors whose DOS is within 1e-3 relative L1 error of a stochastic reference
(R_ref vectors, independent seed), found once before timing; so
value = time-to-DOS at 1e-3 L1 error (seconds, lower is better).
e2e = the same DOS through the C ABI from the host geometry description,
including GPU assembly, with moments and DOS copied back to host memory.
Vector blocks (>= 80 MB per block at this size) exceed the 126 MB L2 together
with the 8 GB matrix, so every step streams from HBM; no L2 flush is needed.

--impl reference times the reference's CPU recursion (the oracle port of
Locality::computeDosTraceKPM + SpMatrix::vectorMultiply, FP64) on the host
cores on a bounded sample of the same workload and extrapolates to it.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "time-to-DOS at 1e-3 L1 err (plain GPU KPM; CV-surrogate reported beside it)"
UNIT = "s"
TWIST_DEG = 0.5
RADIUS = 2042.0
P = 1024
N_E = 4001
TARGET_L1 = 1e-3
CPU_STEPS = 4       # Chebyshev steps the CPU baseline times on the full flake
REF_VECTORS = 13    # vectors the device arm needs for 1e-3 L1 on this flake (its calibration, seeds fixed)


def geom(L, radius=RADIUS, twist=TWIST_DEG):
    # |i| <= R/a + |j|/2 with |j| <= R/(a sqrt(3)/2) for sites of the disk
    size = int(math.ceil(radius / 2.46 * (1.0 + 1.0 / math.sqrt(3.0)))) + 4
    return L.make_geom(model=L.MODEL_SIMPLE, size=size, max_R=radius, heights=(0.0, 3.35),
                       angles_deg=(0.0, twist), energy_rescale=1.0)


def energies(a, b):
    x = -1.0 + 2.0 * (np.arange(N_E) + 0.5) / N_E
    return b + a * x


def l1(d, ref):
    return float(np.abs(d - ref).sum() / np.abs(ref).sum())


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "samples": len(sm), "reasons": sorted(reasons)}


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def step_bytes(n, nnz_true, cols):
    """Algorithmic bytes of one Chebyshev step over a block of `cols` FP32 columns."""
    return nnz_true * (4 + 4) + (n + 1) * 8 + 3 * n * cols * 4


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- CPU baseline

class CpuFlake:
    """The workload's flake built on the host cores (oracle_simple_flake_csr: the
    simple model's compact Hamiltonian in the reference row order, rescaled by
    (a, b) as H~ = (H - b) / a), for the CPU baseline at full size."""

    def __init__(self, L, threads, radius=RADIUS, twist=TWIST_DEG, a=None, b=0.0):
        import ctypes
        from oracle import oracle
        self.oracle = oracle
        lib = oracle.lib()
        lib.oracle_flake_sites.restype = ctypes.c_int64
        lib.oracle_simple_flake_csr.restype = ctypes.c_int64
        g = oracle.geom_prepare(geom(L, radius=radius, twist=twist))
        t0 = time.perf_counter()
        n = lib.oracle_flake_sites(ctypes.byref(g))
        rp = np.zeros(n + 1, np.int64)
        args = (ctypes.byref(g), ctypes.c_double(1.0 if a is None else a), ctypes.c_double(-b), ctypes.c_int(threads))
        nnz = lib.oracle_simple_flake_csr(*args, oracle._p(rp), None, None, ctypes.c_int64(0))
        col = np.empty(nnz, np.int32)
        val = np.empty(nnz, np.float64)
        lib.oracle_simple_flake_csr(*args, oracle._p(rp), oracle._p(col), oracle._p(val), ctypes.c_int64(nnz))
        if a is None:  # Gershgorin bounds x 1.01 of the host-built matrix, then rescale in place
            lo, hi = oracle.gershgorin(rp, col, val)
            a, b = 1.01 * (hi - lo) / 2, (hi + lo) / 2
            lib.oracle_rescale_csr(ctypes.c_int64(n), oracle._p(rp), oracle._p(col), oracle._p(val),
                                   ctypes.c_double(a), ctypes.c_double(-b))
        self.build_s = time.perf_counter() - t0
        self.n, self.nnz, self.rp, self.col, self.val, self.a, self.b = n, nnz, rp, col, val, a, b

    def time_steps(self, threads, steps):
        """Seconds per Chebyshev step of `threads` vectors on `threads` host threads."""
        import ctypes
        lib = self.oracle.lib()
        lib.oracle_cpu_kpm_steps.restype = ctypes.c_double
        chk = ctypes.c_double()
        t = lib.oracle_cpu_kpm_steps(ctypes.c_int64(self.n), self.oracle._p(self.rp), self.oracle._p(self.col),
                                     self.oracle._p(self.val), ctypes.c_int32(threads), ctypes.c_int32(steps),
                                     ctypes.c_int32(threads), ctypes.byref(chk))
        return t / steps

    def moments(self, seed, first, R, P, threads):
        """FP64 doubling moments of R Philox random-phase vectors (real and imaginary
        parts summed), the same recursion and vectors as the device's trace."""
        import ctypes
        o = self.oracle
        re, im = o.phase_vectors(seed, first, R, self.n)
        vec = np.ascontiguousarray(np.concatenate([re, im]))
        mu = np.zeros((2 * R, P))
        o.lib().oracle_kpm_trace_doubling_threads(
            ctypes.c_int64(self.n), o._p(self.rp), o._p(self.col), o._p(self.val), ctypes.c_int32(2 * R),
            o._p(vec), ctypes.c_int32(P), ctypes.c_int32(threads), o._p(mu))
        return mu[:R] + mu[R:]


# ---------------------------------------------------------------- profiling case

def kernel_case(args):
    """A few Chebyshev-step launches on a mid-size flake, for ncu captures."""
    import leo2d_gb300 as L
    radius = args.radius if args.radius != RADIUS else 1000.0
    with L.Context(0) as ctx:
        if args.step_kernel >= 0:
            ctx.set_option("step_kernel", args.step_kernel)
        for key in ("rt_stage", "rt_warps", "rt_depth", "rt_group", "rt_chunk", "rt_rows"):
            if getattr(args, key) is not None:
                ctx.set_option(key, getattr(args, key))
        csr = ctx.build_csr(ctx.prepare(geom(L, radius=radius)))
        lo, hi = csr.bounds()
        csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
        cfg = L.kpm_cfg(16, R=max(1, args.kernel_case // 2), block=args.kernel_case, seed=1)
        for _ in range(2):
            csr.kpm_dos(cfg)
        ctx.reset_stats()
        ctx.set_profiling(True)
        csr.kpm_dos(cfg)
        ctx.set_profiling(False)
        k, ms = ctx.kernel_stats("cheb_step")
        nnz_true = csr.nnz
        gbs = step_bytes(csr.n, nnz_true, args.kernel_case) / (ms / k * 1e-3) / 1e9
        # a second build of the same flake: the assembly kernel's CUDA-event time
        # and the whole build's wall time
        ctx.reset_stats()
        ctx.set_profiling(True)
        gp = ctx.prepare(geom(L, radius=radius))
        t0 = time.perf_counter()
        c2 = ctx.build_csr(gp)
        build_ms = (time.perf_counter() - t0) * 1e3
        ctx.set_profiling(False)
        ka, asm_ms = ctx.kernel_stats("flake_rows_fill")
        c2.close()
        print(json.dumps({"kernel_case": {"n": csr.n, "nnz": csr.nnz, "cols": args.kernel_case,
                                          "step_kernel": args.step_kernel, "radius_A": radius,
                                          "step_kernel_run": csr.step_kernel(cfg)[0],
                                          "rb_info": list(csr.rb_info()), "rt_info": list(csr.rt_info()),
                                          "step_ms": round(ms / k, 4), "step_gbs": round(gbs, 1),
                                          "assembly_kernel_ms": round(asm_ms / max(ka, 1), 3),
                                          "build_ms": round(build_ms, 2)}}))


# ---------------------------------------------------------------- learned control variate

CV_EDGE = 40.0      # A: orbitals nearer the edge are not a function of the stacking features
CV_SITES_PER_FLAKE = 4096


def cv_training_set(L, ctx, a, b):
    """Site-resolved moments (first 256) from the commensurate 1.05 deg supercell
    (31,32) with periodic boundaries (every orbital), four flakes of the batched
    family (twist 0.8-3.0 deg) and two flakes at 0.5 and 0.65 deg so that the
    twist input covers the target's (bulk orbitals, 4096 per flake), at spectral
    scale (a, b)."""
    cfg = L.kpm_cfg(256, R=1)
    xs, ts = [], []
    g = L.make_geom(model=L.MODEL_SIMPLE, boundary_condition=1, size=100, supercell_mn=(31, 32),
                    energy_rescale=1.0)
    gp = ctx.prepare(g)
    csr = ctx.build_csr(gp)
    twist = math.degrees(abs(gp.angles[1] - gp.angles[0]))
    lo, hi = csr.bounds()
    systems = [(csr, twist, None, max(abs(lo - b), abs(hi - b)))]
    rng = np.random.default_rng(11)
    twists, radii = batch_flakes()
    for th, rad in list(zip(twists, radii))[:4] + [(0.5, 260.0), (0.65, 260.0)]:
        rad = float(min(max(rad, 150.0), 260.0))
        c = ctx.build_csr(ctx.prepare(geom(L, radius=rad, twist=float(th))))
        lo, hi = c.bounds()
        systems.append((c, float(th), rad, max(abs(lo - b), abs(hi - b))))
    a_needed = max(x[3] for x in systems)  # Gershgorin bounds the spectrum: a must cover it
    for c, th, rad, _ in systems:
        c.rescale(a, -b)
        if rad is None:
            sel = np.arange(c.n)
        else:
            _, pos = c.geometry()
            p = pos.reshape(-1, 3)
            bulk = np.nonzero(np.hypot(p[:, 0], p[:, 1]) < rad - CV_EDGE)[0]
            sel = np.sort(rng.choice(bulk, size=min(CV_SITES_PER_FLAKE, len(bulk)), replace=False))
        xs.append(c.site_features(th)[sel])
        ts.append(c.kpm_ldos(cfg, sel))
        c.close()
    return np.concatenate(xs), np.concatenate(ts).astype(np.float32), a_needed


def run_cv(L, ctx, csr, a, b, n, dos_of, d_ref, mu_cal, R_plain, t_plain, stream):
    """Time-to-DOS at the same 1e-3 L1 target with the learned control variate.

    Estimator (leo2d_kpm_dos_cv): moments n < 256 = w_n [sum_i f_n(i) + N mean over
    S uniform orbitals of (mu_n(s) - f_n(s))] + (1 - w_n) [random-phase mean], the
    rest from the random-phase vectors; w_n fixed from pilot variances (phase: the
    spread of the calibration vectors; sites: an independent pilot draw), so the
    estimate is unbiased. The cheapest (vectors, sites) pair that reaches 1e-3 is
    found on one realisation, as for the plain count, then timed end to end."""
    import torch
    t0 = time.perf_counter()
    x, t, a_needed = cv_training_set(L, ctx, a, b)
    if a_needed > a * 1.0000001:
        return {"skipped": f"training systems need spectral scale {a_needed:.4f} > {a:.4f}"}
    mlp = L.Mlp(ctx, seed=0)
    hist = mlp.train(x, t, steps=3000, batch=4096, lr=2e-3, seed=1)
    t_train = time.perf_counter() - t0
    twist = TWIST_DEG
    # pilot: residual variance of the network on the target (independent sites)
    pilot_sites = 128
    rng = np.random.default_rng(999)
    ps = rng.integers(0, n, pilot_sites)
    mu_p = csr.kpm_ldos(L.kpm_cfg(256, R=1), ps)
    f_p = mlp.predict(csr.site_features(twist)[ps]).astype(np.float64)
    var_res = (mu_p - f_p).var(axis=0, ddof=1)
    var_site = mu_p.var(axis=0, ddof=1)
    var_phase = mu_cal[:, :256].var(axis=0, ddof=1)  # per vector, trace units
    # one realisation: per-vector phase moments and the control-variate parts per
    # site count, combined exactly as leo2d_kpm_dos_cv combines them
    R_max = 2 * R_plain
    ph_all = csr.kpm_dos(L.kpm_cfg(P, R=R_max, seed=4242))
    R_same = None  # plain vector count on this realisation
    for R in range(1, R_max + 1):
        if l1(dos_of(ph_all[:R].mean(axis=0)), d_ref) <= TARGET_L1:
            R_same = R
            break
    best = None
    for S in (64, 128):
        _, parts = csr.kpm_dos_cv(mlp, L.kpm_cfg(P, R=0), twist, S, site_seed=17 + S, parts=True)
        cvp = parts[0] + parts[1]
        v_cv = n * n * var_res / S
        for R in range(1, R_max + 1):
            w = (var_phase / R) / (var_phase / R + v_cv)
            mu = ph_all[:R].mean(axis=0)
            mu[:256] = w * cvp + (1 - w) * mu[:256]
            e = l1(dos_of(mu), d_ref)
            if e <= TARGET_L1:
                if best is None or R < best[0]:
                    best = (R, S, e, w)
                break
    out = {"train_rows": int(x.shape[0]), "train_steps": 3000, "train_s": round(t_train, 2),
           "train_loss_first_last": [float(hist[0]), float(hist[-1])],
           "site_var_over_residual_var": {f"{lo}-{hi}": float(var_site[lo:hi].mean() / var_res[lo:hi].mean())
                                          for lo, hi in ((1, 16), (16, 128), (128, 256))},
           "phase_var_over_site_var_per_unit": float(np.mean(var_phase[16:128]) / (n * n * var_site[16:128].mean())),
           "pilot_sites": pilot_sites, "plain_vectors_same_realisation": R_same}
    if best is None:
        out["time_to_dos_s"] = None
        out["note"] = "no (vectors <= 2 x plain count, sites <= 128) pair reached 1e-3"
        mlp.close()
        return out
    R, S, e, w = best
    cfg = L.kpm_cfg(P, R=R, seed=4242)
    csr.kpm_dos_cv(mlp, cfg, twist, S, site_seed=17 + S, weights=w)  # warm
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    mu = csr.kpm_dos_cv(mlp, cfg, twist, S, site_seed=17 + S, weights=w)
    d = dos_of(mu)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_cv = ev0.elapsed_time(ev1) / 1000.0
    out.update({"time_to_dos_s": round(t_cv, 6), "vectors": R, "sites": S, "l1": e,
                "speedup_vs_plain": round(t_plain / t_cv, 4), "plain_vectors": R_plain})
    if R_same is not None:
        cfg_p = L.kpm_cfg(P, R=R_same, seed=4242)
        ev0.record(stream)
        dos_of(csr.kpm_dos(cfg_p).mean(axis=0))
        ev1.record(stream)
        torch.cuda.synchronize()
        t_same = ev0.elapsed_time(ev1) / 1000.0
        out.update({"plain_time_same_realisation_s": round(t_same, 6),
                    "speedup_vs_plain_same_realisation": round(t_same / t_cv, 4)})
    mlp.close()
    return out


# ---------------------------------------------------------------- periodic supercell and Kubo

def _timed(stream, fn, steps, warmup):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        out = fn()
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1) / 1000.0 / steps, out


def run_periodic(args):
    """Commensurate TBLG (31,32), 1.05 deg, periodic: 11,908 orbitals, P = 4096, one block
    of 64 random-phase vectors, FP32 recursion; per-energy error against the FP64
    recursion on the same vectors (itself checked against the CPU oracle on one vector)."""
    import torch
    import leo2d_gb300 as L
    from oracle import oracle
    ctx = L.Context(0)
    g = L.make_geom(model=L.MODEL_SIMPLE, boundary_condition=1, size=100, supercell_mn=(31, 32),
                    energy_rescale=1.0)
    gp = ctx.prepare(g)
    csr = ctx.build_csr(gp)
    lo, hi = csr.bounds()
    a, b = 1.01 * (hi - lo) / 2, (hi + lo) / 2
    csr.rescale(a, -b)
    Pp, R = 4096, 64
    cfg32 = L.kpm_cfg(Pp, R=R, seed=3)
    cfg64 = L.kpm_cfg(Pp, R=R, seed=3, precision=L.FP64)
    cols, rows = csr.autotune(cfg32)  # untimed
    stream = torch.cuda.ExternalStream(ctx.lib.leo2d_ctx_stream(ctx.h))
    E = energies(a, b)
    dos = lambda mu: ctx.dos_reconstruct(mu.mean(axis=0), E, a, b, 1.0 / csr.n)
    l0 = ctx.launch_count()
    t32, d32 = _timed(stream, lambda: dos(csr.kpm_dos(cfg32)), args.steps, args.warmup)
    launches = (ctx.launch_count() - l0) // (args.steps + args.warmup)
    t64, d64 = _timed(stream, lambda: dos(csr.kpm_dos(cfg64)), 1, 1)
    err = np.abs(d32 - d64) / np.abs(d64).max()
    # the FP64 recursion against the CPU oracle, one vector
    rp, col, val = csr.download()
    re_, im_ = oracle.phase_vectors(3, 0, 1, csr.n)
    mo = (oracle.kpm_trace(rp, col, val, re_, Pp, literal=False) +
          oracle.kpm_trace(rp, col, val, im_, Pp, literal=False))[0]
    m64 = csr.kpm_dos(L.kpm_cfg(Pp, R=1, seed=3, precision=L.FP64))[0]
    out = {"metric": "periodic-supercell DOS (P=4096, 64 vectors, FP32 recursion)", "value": round(t32, 6),
           "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(t32 * 1000, 3), "higher_is_better": False, "dtype": "fp32",
           "data": "synthetic (commensurate supercell, Philox vectors)",
           "config": {"workload": "TBLG (31,32) 1.05 deg periodic, simple model, P=4096, 64 random-phase vectors, "
                                  "4001 energies", "orbitals": csr.n, "nnz": csr.nnz,
                      "twist_deg": math.degrees(abs(gp.angles[1] - gp.angles[0])), "block_cols": cols},
           "fp64_time_s": round(t64, 6),
           "error_vs_fp64_per_energy": {"max": float(err.max()), "mean": float(err.mean()),
                                        "p99": float(np.quantile(err, 0.99))},
           "l1_vs_fp64": l1(d32, d64),
           "fp64_gpu_vs_cpu_oracle_moments": float(np.abs(m64 - mo).max() / np.abs(mo).max()),
           "gpu_launches": int(launches)}
    print(json.dumps(out))
    ctx.close()


def run_cfg0(args):
    """Plain KPM DOS in FP64 on the 5.09 deg flake of radius 60 a = 147.6 A (simple
    model, ~52k orbitals): Gershgorin bounds x 1.01, P = 1000 (Jackson), 16 random-
    phase vectors, DOS on 4001 energies. value: one DOS from the resident matrix;
    e2e: from the host geometry through the C ABI; the CPU baseline runs the
    reference's recursion on the same flake built on the host, in full (no
    extrapolation), and checks the device's FP64 moments against it."""
    import torch
    import leo2d_gb300 as L
    radius, twist, Pc, R = 60 * 2.46, 5.09, 1000, 16
    ctx = L.Context(0)
    g = ctx.prepare(geom(L, radius=radius, twist=twist))
    csr = ctx.build_csr(g)
    lo, hi = csr.bounds()
    a, b = 1.01 * (hi - lo) / 2, (hi + lo) / 2
    csr.rescale(a, -b)
    n, nnz = csr.n, csr.nnz
    x = -1.0 + 2.0 * (np.arange(N_E) + 0.5) / N_E
    cfg = L.kpm_cfg(Pc, R=R, seed=5, precision=L.FP64)
    cols, _ = csr.autotune(cfg)
    kernel_id, _ = csr.step_kernel(cfg)
    stream = torch.cuda.ExternalStream(ctx.lib.leo2d_ctx_stream(ctx.h))
    dos = lambda mu, c=csr, aa=a, bb=b: ctx.dos_reconstruct(mu.mean(axis=0), bb + aa * x, aa, bb, 1.0 / c.n)
    for _ in range(max(args.warmup, 1)):
        dos(csr.kpm_dos(cfg))
    ctx.reset_stats()
    ctx.set_profiling(True)
    l0 = ctx.launch_count()
    with Clocks(0) as clk:
        t, d = _timed(stream, lambda: dos(csr.kpm_dos(cfg)), args.steps, 0)
    launches = (ctx.launch_count() - l0) // args.steps
    k_n, k_ms = ctx.kernel_stats("cheb_step")
    ctx.set_profiling(False)

    def e2e_once():
        c2 = ctx.build_csr(g)
        lo2, hi2 = c2.bounds()
        a2, b2 = 1.01 * (hi2 - lo2) / 2, (hi2 + lo2) / 2
        c2.rescale(a2, -b2)
        mu = c2.kpm_dos(cfg)
        out = dos(mu, c2, a2, b2)
        c2.close()
        return mu, out

    e2e_once()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        mu_e, _ = e2e_once()
    t_e2e = (time.perf_counter() - t0) / args.steps
    import ctypes
    peak, peak_kind = peaks()
    bytes_step = nnz * (4 + 8) + (n + 1) * 8 + 3 * n * cols * 8  # FP64 values and vectors
    launch_ms = k_ms / k_n
    achieved = bytes_step / (launch_ms / 1000.0) / 1e9
    threads = os.cpu_count() or 1
    cf = CpuFlake(L, threads, radius=radius, twist=twist, a=a, b=b)
    t_cpu = cf.time_steps(min(threads, R), Pc // 2) * (Pc // 2) * math.ceil(R / min(threads, R))
    mu_cpu = cf.moments(5, 0, 2, Pc, threads)
    mu_gpu = csr.kpm_dos(L.kpm_cfg(Pc, R=2, seed=5, precision=L.FP64))
    out = {"metric": "plain KPM DOS, FP64 (P=1000, 16 random-phase vectors, 4001 energies)",
           "value": round(t, 6), "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 1),
           "ms_per_step": round(t * 1000, 3), "higher_is_better": False, "scaling": "strong", "vs_baseline": None,
           "dtype": "fp64", "data": "synthetic (geometry generated on the GPU; random-phase vectors, Philox)",
           "config": {"workload": f"TBLG flake {twist} deg, R={radius:.1f} A, {n} orbitals, simple model, "
                                  f"P={Pc}, {R} random-phase vectors, {N_E} energies",
                      "orbitals": n, "nnz": nnz, "block_cols": cols,
                      "l2": "matrix and vector blocks fit the L2 (tens of MB): the steps run from L2"},
           "e2e": {"value": round(t_e2e, 6), "unit": "s", "h2d_bytes_per_step": ctypes.sizeof(L.Geom),
                   "d2h_bytes_per_step": int(mu_e.nbytes + N_E * 8)},
           "gpu_launches": int(launches),
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(achieved / peak, 4), "traffic": None,
                        "kernel": {0: "k_cheb_tile<double>", 1: "k_cheb_step<double>"}.get(kernel_id, str(kernel_id)),
                        "bytes_per_launch": bytes_step, "launch_ms": round(launch_ms, 4), "peak_kind": peak_kind,
                        "note": "working set in L2: the fraction of HBM is a bandwidth figure, not an HBM bound"},
           # what bounds this workload: the FP64 FMAs (2 flops per entry and column)
           # on GB300's small FP64 unit
           "compute": {"bound": "fp64", "achieved_gflops": round(2.0 * nnz * cols / (launch_ms / 1000.0) / 1e9, 1),
                       "peak_gflops": 1250.0, "peak_kind": "nominal GB300 FP64 (no measured figure)",
                       "frac": round(2.0 * nnz * cols / (launch_ms / 1000.0) / 1e9 / 1250.0, 4)},
           "clocks": clk.summary(),
           "cpu_baseline": {"value": round(t_cpu, 3), "unit": "s", "cores": min(threads, R), "kind": "port",
                            "sample": f"the whole workload: oracle FP64 recursion, {R} vectors x {Pc // 2} steps on "
                                      f"{min(threads, R)} threads over the same flake built on the host "
                                      f"({cf.nnz} entries)"},
           "parity": {"fp64_gpu_vs_fp64_host_moments_max_rel": float(np.max(np.abs(mu_gpu - mu_cpu)) /
                                                                     np.max(np.abs(mu_cpu))),
                      "vectors": 2, "moments": Pc}}
    print(json.dumps(out))
    ctx.close()


def run_cv_bound(args):
    """What a perfect control variate could buy: on a 0.5 deg flake of ~1e5 orbitals,
    the exact moments of every orbital (unit start vectors, FP64-summed FP32
    recursion, leo2d_kpm_ldos) give the exact trace moments. The plain estimate
    takes R random-phase vectors; the ideal control variate knows moments 0..255
    exactly (a surrogate with zero residual) and takes R' phase vectors for the
    rest. Both are run to 1e-3 L1 of the exact DOS on several independent
    realisations; time-to-DOS is proportional to the vector count, so R / R' is
    the largest speed-up any surrogate of the first 256 moments can give."""
    import leo2d_gb300 as L
    radius = args.cv_radius
    P_cv, P_s, seeds = P, 256, (101, 202, 303, 404)
    ctx = L.Context(0)
    csr = ctx.build_csr(ctx.prepare(geom(L, radius=radius)))
    lo, hi = csr.bounds()
    a, b = 1.01 * (hi - lo) / 2, (hi + lo) / 2
    csr.rescale(a, -b)
    n = csr.n
    E = energies(a, b)
    dos_of = lambda mu: ctx.dos_reconstruct(mu, E, a, b, 1.0 / n)
    t0 = time.perf_counter()
    exact = np.zeros(P_cv)
    blk = 4096
    for s0 in range(0, n, blk):
        tg = np.arange(s0, min(n, s0 + blk), dtype=np.int64)
        exact += csr.kpm_ldos(L.kpm_cfg(P_cv, R=1), tg).sum(axis=0)
    t_exact = time.perf_counter() - t0
    # the site moments sum to Tr T_n, what one random-phase vector estimates
    d_exact = dos_of(exact)
    R_max = args.cv_max_vectors
    res = []
    for sd in seeds:
        ph = csr.kpm_dos(L.kpm_cfg(P_cv, R=R_max, seed=sd))
        cs = np.cumsum(ph, axis=0)
        r_plain = r_cv = None
        for R in range(1, R_max + 1):
            mu = cs[R - 1] / R
            if r_plain is None and l1(dos_of(mu), d_exact) <= TARGET_L1:
                r_plain = R
            if r_cv is None:
                mc = mu.copy()
                mc[:P_s] = exact[:P_s]
                if l1(dos_of(mc), d_exact) <= TARGET_L1:
                    r_cv = R
            if r_plain is not None and r_cv is not None:
                break
        res.append((r_plain, r_cv))
    rp = [x[0] for x in res]
    rc = [x[1] for x in res]
    ok = all(x is not None for x in rp + rc)
    out = {"metric": "time-to-DOS speed-up bound of a perfect control variate of the first 256 moments",
           "value": round(float(np.mean(rp)) / float(np.mean(rc)), 3) if ok else None, "unit": "x",
           "higher_is_better": True, "n_gpus": 1, "dtype": "fp32 recursion, fp64 moments", "data": "synthetic",
           "config": {"workload": f"TBLG flake {TWIST_DEG} deg, R={radius:.0f} A, {n} orbitals, simple model, "
                                  f"P={P_cv}, {N_E} energies, 1e-3 L1 against the exact DOS",
                      "orbitals": n, "surrogate_moments": P_s, "realisations": len(seeds)},
           "plain_vectors": rp, "ideal_cv_vectors": rc, "exact_moments_s": round(t_exact, 1),
           "note": "time-to-DOS is proportional to the vector count; the ideal surrogate costs nothing here"}
    print(json.dumps(out))
    ctx.close()


def run_bfield(args):
    """The headline flake in a perpendicular field (complex Hamiltonian, Peierls phases):
    one DOS of 16 random-phase vectors (32 columns), P = 1024, FP32 complex row-block step;
    against the same recursion in FP64 on the CPU oracle for a 162k-orbital flake."""
    import torch
    import leo2d_gb300 as L
    from oracle import oracle
    B = 20.0
    ctx = L.Context(0)
    if args.step_kernel >= 0:  # 3: the 4-row complex step, 5: the 8-row one
        ctx.set_option("step_kernel", args.step_kernel)
    g = geom(L, radius=args.radius)
    g.b_field = B
    t0 = time.perf_counter()
    csr = ctx.build_csr(ctx.prepare(g))
    lo, hi = csr.bounds()
    a, b = 1.01 * (hi - lo) / 2, (hi + lo) / 2
    csr.rescale(a, -b)
    t_build = time.perf_counter() - t0
    n, nnz = csr.n, csr.nnz
    cfg = L.kpm_cfg(P, R=16, seed=7)
    stream = torch.cuda.ExternalStream(ctx.lib.leo2d_ctx_stream(ctx.h))
    E = energies(a, b)
    dos = lambda mu: ctx.dos_reconstruct(mu.mean(axis=0), E, a, b, 1.0 / n)
    csr.kpm_dos(cfg)  # builds the ordered copy and the row blocks (untimed)
    ctx.reset_stats()
    ctx.set_profiling(True)
    l0 = ctx.launch_count()
    t, d = _timed(stream, lambda: dos(csr.kpm_dos(cfg)), args.steps, args.warmup)
    launches = (ctx.launch_count() - l0) // (args.steps + args.warmup)
    k_n, k_ms = ctx.kernel_stats("cheb_step")
    ctx.set_profiling(False)
    step_ms = k_ms / k_n
    # complex H: (col, re, im) per entry, 32 FP32 columns (16 complex vectors)
    bytes_step = nnz * 12 + (n + 1) * 8 + 3 * n * 32 * 4
    peak, peak_kind = peaks()
    # parity on a 162k-orbital flake of the same model and field: FP32 GPU vs FP64 CPU oracle
    gs = geom(L, radius=260.0)
    gs.b_field = B
    cs = ctx.build_csr(ctx.prepare(gs))
    los, his = cs.bounds()
    cs.rescale(1.01 * (his - los) / 2, -(his + los) / 2)
    Ps, Rs = 256, 2
    ms = cs.kpm_dos(L.kpm_cfg(Ps, R=Rs, seed=5))
    rp, col, val = cs.download()
    im = cs.download_imag()
    vr, vi = oracle.phase_vectors(5, 0, Rs, cs.n)
    mo = oracle.kpm_trace_cpx_doubling(rp, col, val, im, vr, vi, Ps)
    out = {"metric": "DOS in a magnetic field (complex H, P=1024, 16 vectors, FP32 recursion)",
           "value": round(t, 6), "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(t * 1000, 3), "higher_is_better": False, "dtype": "fp32",
           "data": "synthetic (geometry generated on the GPU; random-phase vectors, Philox)",
           "config": {"workload": f"TBLG flake {TWIST_DEG} deg, R={args.radius:.0f} A, B={B} T, simple model, "
                                  f"P={P}, 16 complex vectors, {N_E} energies",
                      "orbitals": n, "nnz": nnz, "b_field_T": B},
           "build_s": round(t_build, 3),
           "roofline": {"bound": "hbm", "achieved": round(bytes_step / (step_ms / 1000) / 1e9, 1), "peak": peak,
                        "unit": "GB/s", "frac": round(bytes_step / (step_ms / 1000) / 1e9 / peak, 4),
                        "kernel": {3: "k_cheb_rb complex", 5: "k_cheb_rt complex"}.get(
                            csr.step_kernel(cfg)[0], str(csr.step_kernel(cfg)[0])), "bytes_per_launch": bytes_step,
                        "launch_ms": round(step_ms, 4), "peak_kind": peak_kind},
           "fp32_gpu_vs_fp64_oracle_moments_162k": float(np.abs(ms - mo).max() / np.abs(mo).max()),
           "gpu_launches": int(launches)}
    print(json.dumps(out))
    ctx.close()


def run_kubo(args):
    """Kubo sigma_xx(E): 1.5 deg flake of ~2M orbitals, 512 x 512 moments, 32 random-phase
    vectors (trace), FP32 recursion with FP64 moment products, 2001 energies. FP32 against
    the FP64 CPU oracle on a 20k-orbital flake of the same model and twist (one vector)."""
    import torch
    import leo2d_gb300 as L
    from oracle import oracle
    ctx = L.Context(0)
    M, R, twist = args.kubo_moments, args.kubo_vectors, 1.5
    radius = math.sqrt(args.kubo_orbitals / 2.398)
    # no stored dxH: the trace moments build it inside the row-block step
    csr = ctx.build_csr(ctx.prepare(geom(L, radius=radius, twist=twist)))
    lo, hi = csr.bounds()
    a, b = 1.01 * (hi - lo) / 2, (hi + lo) / 2
    csr.rescale(a, -b)
    cfg = L.kpm_cfg(M, R=R, seed=21)
    stream = torch.cuda.ExternalStream(ctx.lib.leo2d_ctx_stream(ctx.h))
    Ek = b + a * np.linspace(-0.99, 0.99, 2001)
    sig = lambda mu: ctx.cond_sigma(mu, Ek, a, b, 1.0 / csr.n)
    l0 = ctx.launch_count()
    t, s = _timed(stream, lambda: sig(csr.kpm_cond(cfg)), args.steps, min(args.warmup, 1))
    launches = (ctx.launch_count() - l0) // (args.steps + min(args.warmup, 1))
    # where the time goes (one more run with per-launch events)
    ctx.reset_stats()
    ctx.set_profiling(True)
    csr.kpm_cond(cfg)
    ctx.set_profiling(False)
    split = {k: round(ctx.kernel_stats(k)[1] / 1000.0, 4)
             for k in ("cheb_step", "cheb_step_vel", "cond_gemm", "cond_gemm_sum", "rb_xrel")}
    steps_run = ctx.kernel_stats("cheb_step")[0] + ctx.kernel_stats("cheb_step_vel")[0]
    # FP32 vs FP64 oracle on a small flake
    small = ctx.build_csr(ctx.prepare(geom(L, radius=math.sqrt(2.0e4 / 2.398), twist=twist)), with_dx=True)
    slo, shi = small.bounds()
    sa, sb = 1.01 * (shi - slo) / 2, (shi + slo) / 2
    small.rescale(sa, -sb)
    Ms = 128
    mu32 = small.kpm_cond(L.kpm_cfg(Ms, R=1, seed=5))
    rp, col, val, dx, dy = small.download(dx=True)
    re_, im_ = oracle.phase_vectors(5, 0, 1, small.n)
    mu64 = oracle.kpm_cond_trace(rp, col, val, dx, re_, Ms) + oracle.kpm_cond_trace(rp, col, val, dx, im_, Ms)
    Es = sb + sa * np.linspace(-0.99, 0.99, 2001)
    s32 = ctx.cond_sigma(mu32, Es, sa, sb, 1.0 / small.n)
    s64 = ctx.cond_sigma(mu64, Es, sa, sb, 1.0 / small.n)
    out = {"metric": f"Kubo sigma_xx(E) ({M}x{M} moments, {R} random-phase vectors, 2001 energies)",
           "value": round(t, 6), "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": min(args.warmup, 1),
           "ms_per_step": round(t * 1000, 3), "higher_is_better": False, "dtype": "fp32",
           "data": "synthetic (geometry generated on the GPU, Philox vectors)",
           "config": {"workload": f"TBLG flake {twist} deg, ~{args.kubo_orbitals:.3g} orbitals, simple model, "
                                  f"J=i[H,x] built in the step, M={M}, {R} vectors, 2001 energies",
                      "orbitals": csr.n, "nnz": csr.nnz},
           "fp32_vs_fp64_oracle": {"orbitals": small.n, "moments": Ms,
                                   "mu_max_rel": float(np.abs(mu32 - mu64).max() / np.abs(mu64).max()),
                                   "sigma_max_rel": float(np.abs(s32 - s64).max() / np.abs(s64).max())},
           "sigma_range": [float(s.min()), float(s.max())], "kernel_seconds": split, "step_launches": int(steps_run),
           "gpu_launches": int(launches)}
    print(json.dumps(out))
    ctx.close()


def run_mlp(args):
    """The learned control variate's network on the tensor cores: Adam training steps
    (batch 8192, graph-replayed) and inference of the moment sum over every orbital of
    the flake of --radius (default: the 10M-orbital 0.5 deg flake)."""
    import torch
    import leo2d_gb300 as L
    ctx = L.Context(0)
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, (65536, 16)).astype(np.float32)
    t = rng.normal(0, 0.3, (65536, 256)).astype(np.float32)
    mlp = L.Mlp(ctx, seed=0)
    B = 8192
    stream = torch.cuda.ExternalStream(ctx.lib.leo2d_ctx_stream(ctx.h))
    t_step = float("nan")
    if not args.mlp_infer_only:
        mlp.train(x, t, steps=5, batch=B)
        t_short, _ = _timed(stream, lambda: mlp.train(x, t, steps=20, batch=B, seed=2), 1, 0)
        t_long, _ = _timed(stream, lambda: mlp.train(x, t, steps=220, batch=B, seed=3), 1, 0)
        t_step = (t_long - t_short) / 200.0
    layer_macs = 64 * 256 + 3 * 256 * 256
    flops_step = 2 * B * layer_macs * 2 + 2 * B * 3 * 256 * 256  # forward, weight gradients, input gradients
    csr = ctx.build_csr(ctx.prepare(geom(L, radius=args.radius)))
    # the forward alone: the fused launch (default) and one GEMM per layer
    # (mlp_fused = 0), each timed per launch on the library's stream; the
    # whole call also computes the disregistry features of every orbital
    fwd = {}
    for fused in (0, 1):
        ctx.set_option("mlp_fused", fused)
        mlp.site_sum(csr, TWIST_DEG)
        ctx.reset_stats()
        ctx.set_profiling(True)
        t_call, _ = _timed(stream, lambda: mlp.site_sum(csr, TWIST_DEG), args.steps, 1)
        names = ("mlp_fused", "mlp_fused_sums") if fused else ("tc_gemm", "mlp_sum")
        ms = 0.0
        for nm in names:
            k_n, k_ms = ctx.kernel_stats(nm)
            ms += k_ms / max(args.steps, 1)
        ctx.set_profiling(False)
        fwd[fused] = (t_call, ms / 1000.0)
    t_inf, t_fwd = fwd[1]
    flops_inf = 2 * csr.n * layer_macs
    peak = 1900.0
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["bf16_tflops"])
    except (OSError, ValueError, KeyError):
        pass
    out = {"metric": "control-variate network: inference over every orbital (16 -> 3x256 GELU -> 256, BF16)",
           "value": round(t_inf, 6), "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": 1,
           "higher_is_better": False, "dtype": "bf16 (fp32 accumulation)", "data": "synthetic",
           "config": {"workload": f"site sums over {csr.n} orbitals; training batch {B}", "orbitals": csr.n},
           "forward_s": round(t_fwd, 6), "forward_tflops": round(flops_inf / t_fwd / 1e12, 1),
           "layered_call_s": round(fwd[0][0], 6), "layered_forward_s": round(fwd[0][1], 6),
           "layered_forward_tflops": round(flops_inf / fwd[0][1] / 1e12, 1),
           "inference_tflops": round(flops_inf / t_inf / 1e12, 1),
           "train_step_ms": round(t_step * 1000, 4), "train_tflops": round(flops_step / t_step / 1e12, 1),
           "roofline": {"bound": "tensor", "achieved": round(flops_inf / t_fwd / 1e12, 1), "peak": peak,
                        "unit": "TFLOP/s", "frac": round(flops_inf / t_fwd / 1e12 / peak, 4),
                        "kernel": "k_mlp_fused (+ k_mlp_fused_sums)", "launch_ms": round(t_fwd * 1000, 4),
                        "peak_kind": "measured (cuBLAS bf16 burst)"}}
    print(json.dumps(out))
    mlp.close()
    ctx.close()


# ---------------------------------------------------------------- batched flakes

BATCH_F, BATCH_P, BATCH_R = 32, 2048, 32


def batch_flakes(seed=2024):
    """Twist U[0.8, 3.0] deg and sizes log-uniform in [2e4, 5e5] orbitals (seeded);
    radius from the simple model's 2.398 orbitals per A^2 of disk (two layers)."""
    rng = np.random.default_rng(seed)
    twists = rng.uniform(0.8, 3.0, BATCH_F)
    sizes = np.exp(rng.uniform(math.log(2e4), math.log(5e5), BATCH_F))
    return twists, np.sqrt(sizes / 2.398)


def run_batch(args):
    import torch
    import leo2d_gb300 as L
    ctx = L.Context(0)
    twists, radii = batch_flakes()
    t0 = time.perf_counter()
    csrs = []
    for th, rad in zip(twists, radii):
        csr = ctx.build_csr(ctx.prepare(geom(L, radius=float(rad), twist=float(th))))
        lo, hi = csr.bounds()
        csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
        csrs.append(csr)
    t_build = time.perf_counter() - t0
    ns = [c.n for c in csrs]
    nnzs = [c.nnz for c in csrs]
    cfg = L.kpm_cfg(BATCH_P, R=BATCH_R, seed=5)
    t0 = time.perf_counter()
    b = L.Batch(ctx, csrs, cfg)  # untimed: autotune + graph capture
    t_create = time.perf_counter() - t0
    torch.cuda.set_device(0)
    stream = torch.cuda.ExternalStream(ctx.lib.leo2d_ctx_stream(ctx.h))
    for _ in range(args.warmup):
        b.run()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = ctx.launch_count()
    with Clocks(0) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            mu = b.run()
        ev1.record(stream)
        torch.cuda.synchronize()
    t_batch = ev0.elapsed_time(ev1) / 1000.0 / args.steps
    launches = ctx.launch_count() - l0
    # the same work one flake at a time through the single-matrix path
    ev2, ev3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for c in csrs[:2]:
        c.kpm_dos(cfg)
    ev2.record(stream)
    singles = [c.kpm_dos(cfg) for c in csrs]
    ev3.record(stream)
    torch.cuda.synchronize()
    t_seq = ev2.elapsed_time(ev3) / 1000.0
    dev = max(float(np.max(np.abs(mu[f] - singles[f])) / np.max(np.abs(singles[f]))) for f in range(BATCH_F))
    C = b.block_cols
    passes = -(-2 * BATCH_R // C)
    bytes_run = sum(step_bytes(n, z, C) for n, z in zip(ns, nnzs)) * (BATCH_P // 2) * passes
    peak, peak_kind = peaks()
    achieved = bytes_run / t_batch / 1e9
    out = {"metric": "batched KPM moments (32 flakes, P=2048, 32 random-phase vectors each)",
           "value": round(t_batch, 6), "unit": "s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(t_batch * 1000, 3), "higher_is_better": False, "scaling": "strong",
           "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded flakes, Philox vectors)",
           "config": {"workload": "32 TBLG flakes, twist U[0.8,3.0] deg, 20k-500k orbitals (log-uniform), "
                                  "simple model, P=2048, 32 random-phase vectors each",
                      "orbitals_total": int(sum(ns)), "orbitals_min": int(min(ns)), "orbitals_max": int(max(ns)),
                      "nnz_total": int(sum(nnzs)), "block_cols": C, "warps": b.warps,
                      "rows_per_slot": b.rows_per_item, "grid": b.grid, "passes": passes,
                      "graph_launches_per_run": b.launches_per_run, "batch_create_s": round(t_create, 2),
                      "build_s": round(t_build, 2),
                      "l2": "vector blocks of all flakes (>= 1.6 GB) exceed L2"},
           "sequential_s": round(t_seq, 6), "speedup_vs_sequential": round(t_seq / t_batch, 3),
           "max_rel_dev_vs_single": dev,
           "gpu_launches": int(launches),
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                        "kernel": "cheb_batch_step (whole replay: fills, steps, reductions)"},
           "clocks": clk.summary()}
    print(json.dumps(out))
    b.close()
    ctx.close()


# ---------------------------------------------------------------- main

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--radius", type=float, default=RADIUS)
    ap.add_argument("--ref-vectors", type=int, default=256)
    ap.add_argument("--no-cv", action="store_true", help="skip the learned control-variate comparison")
    ap.add_argument("--mlp-infer-only", action="store_true",
                    help="mlp workload: skip the training measurement (profiling the inference products)")
    ap.add_argument("--max-vectors", type=int, default=128)
    ap.add_argument("--kubo-orbitals", type=float, default=2.0e6,
                    help="kubo2m: flake size in orbitals (smaller cases for profiling)")
    ap.add_argument("--kubo-moments", type=int, default=512, help="kubo2m: M of the M x M moments")
    ap.add_argument("--kubo-vectors", type=int, default=32, help="kubo2m: random-phase vectors")
    ap.add_argument("--cv-radius", type=float, default=205.0,
                    help="cvbound: flake radius (A); 205 A is about 1e5 orbitals")
    ap.add_argument("--cv-max-vectors", type=int, default=4096, help="cvbound: most phase vectors tried")
    ap.add_argument("--workload", default="flake10m",
                    choices=["flake10m", "cfg0", "cvbound", "batch32", "periodic", "kubo2m", "mlp", "bfield"],
                    help="flake10m: time-to-DOS on the 10M-orbital flake (the headline); cfg0: FP64 DOS of the "
                         "5.09 deg flake of ~52k orbitals, P=1000, 16 vectors; cvbound: the speed-up a perfect "
                         "control variate of the first 256 moments could give (exact site moments of a ~1e5-orbital "
                         "flake); batch32: 32 "
                         "flakes of 20k-500k orbitals in one batched, graph-replayed run; periodic: the "
                         "1.05 deg (31,32) supercell, P=4096, 64 vectors, FP32 vs FP64 per energy; kubo2m: "
                         "sigma_xx(E) of a 2M-orbital 1.5 deg flake, 512x512 moments, 32 vectors; mlp: the "
                         "control variate's network (training steps, inference over the flake of --radius); "
                         "bfield: the flake of --radius in a 20 T field (complex Hamiltonian)")
    ap.add_argument("--step-kernel", type=int, default=-1, choices=[-1, 0, 1, 2, 3, 5],
                    help="force the Chebyshev step kernel: 0 tiled gathers, 1 register gathers, 2 tensor cores, "
                         "3 row blocks, 5 row blocks of 8 on the tensor cores (default: the autotuner's choice)")
    ap.add_argument("--rt-stage", type=int, default=None, choices=[0, 1, 2],
                    help="8-row tensor-core step: T_n rows staged in registers (0), shared memory by cp.async (1) "
                         "or shared memory by TMA row gathers (2)")
    ap.add_argument("--rt-warps", type=int, default=None, help="8-row tensor-core step: warps per CTA")
    ap.add_argument("--rt-depth", type=int, default=None, help="8-row tensor-core step: k-steps in flight")
    ap.add_argument("--rt-group", type=int, default=None, help="tensor-core row-block step: blocks per warp run")
    ap.add_argument("--rt-chunk", type=int, default=None,
                    help="tensor-core row-block step: tiles per CTA between grid-wide jumps")
    ap.add_argument("--rt-rows", type=int, default=None, choices=[8, 16],
                    help="tensor-core row-block step: rows per block")
    ap.add_argument("--kernel-case", type=int, default=0, metavar="COLS",
                    help="profiling case: two short DOS runs (P=16) of COLS-wide vector blocks on the flake "
                         "of --radius (1000 A: 2.4M orbitals), then exit; prints no bench line")
    args = ap.parse_args()
    if args.kernel_case:
        return kernel_case(args)
    if args.workload == "cvbound" and args.impl == "ours":
        return run_cv_bound(args)
    if args.workload == "cfg0" and args.impl == "ours":
        return run_cfg0(args)
    if args.workload == "batch32" and args.impl == "ours":
        return run_batch(args)
    if args.workload == "periodic" and args.impl == "ours":
        return run_periodic(args)
    if args.workload == "kubo2m" and args.impl == "ours":
        return run_kubo(args)
    if args.workload == "mlp" and args.impl == "ours":
        return run_mlp(args)
    if args.workload == "bfield" and args.impl == "ours":
        return run_bfield(args)
    ws, rank, local, pg = dist_setup()
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return
        run_reference(args, threads)
        return

    import leo2d_gb300 as L
    ctx = L.Context(local)
    if args.step_kernel >= 0:
        ctx.set_option("step_kernel", args.step_kernel)
    for key in ("rt_stage", "rt_warps", "rt_depth", "rt_group", "rt_chunk", "rt_rows"):
        if getattr(args, key) is not None:
            ctx.set_option(key, getattr(args, key))
    g = ctx.prepare(geom(L, radius=args.radius))
    t0 = time.perf_counter()
    csr = ctx.build_csr(g)
    lo, hi = csr.bounds()
    a, b = 1.01 * (hi - lo) / 2, (hi + lo) / 2
    csr.rescale(a, -b)
    t_build = time.perf_counter() - t0
    n, nnz = csr.n, csr.nnz
    E = energies(a, b)

    def dos_of(mu_mean):
        return ctx.dos_reconstruct(mu_mean, E, a, b, 1.0 / n)

    # stochastic reference (independent seed) and calibration of R
    mu_ref = csr.kpm_dos(L.kpm_cfg(P, R=args.ref_vectors, seed=1_000_003))
    d_ref = dos_of(mu_ref.mean(axis=0))
    mu_cal = csr.kpm_dos(L.kpm_cfg(P, R=args.max_vectors, seed=7))
    errs = []
    R_needed = None
    csum = np.cumsum(mu_cal, axis=0)
    for R in range(1, args.max_vectors + 1):
        e = l1(dos_of(csum[R - 1] / R), d_ref)
        errs.append(e)
        if R_needed is None and e <= TARGET_L1:
            R_needed = R
    if R_needed is None:
        R_needed = args.max_vectors
    # FP32 recursion against FP64 on the same vectors (2 vectors)
    mu64 = csr.kpm_dos(L.kpm_cfg(P, R=2, seed=11, precision=L.FP64))
    mu32 = csr.kpm_dos(L.kpm_cfg(P, R=2, seed=11, precision=L.FP32))
    fp32_l1 = l1(dos_of(mu32.mean(axis=0)), dos_of(mu64.mean(axis=0)))

    # replicas: each rank runs a contiguous share of the R vectors (global
    # Philox indices), then one FP64 all-reduce of the moment sums
    from leo2d_gb300.replicas import reduce_moments, vector_share
    first, count = vector_share(R_needed, rank, ws)
    cfg = L.kpm_cfg(P, R=max(count, 1), seed=7, first_vector=first)
    t_tune = time.perf_counter()
    cols, rows = csr.autotune(cfg)  # untimed: picks the step kernel, block width and its shape
    t_tune = time.perf_counter() - t_tune
    kernel_id, _ = csr.step_kernel(cfg)
    kernel_name = {0: "k_cheb_tile (tiled CSR gathers)", 1: "k_cheb_step (register gathers)",
                   2: "k_cheb_tc (tensor cores)", 3: "k_cheb_rb (row blocks)",
                   4: "k_cheb_rbw (row blocks, shared-memory windows)",
                   5: "k_cheb_rt (8-row blocks, tensor cores)"}[kernel_id]

    import torch
    torch.cuda.set_device(local)
    stream = torch.cuda.ExternalStream(ctx.lib.leo2d_ctx_stream(ctx.h))

    def one_dos():
        mu = csr.kpm_dos(cfg)[:count]
        return dos_of(reduce_moments(mu.sum(axis=0), count, pg))

    for _ in range(args.warmup):
        one_dos()
    ctx.reset_stats()
    ctx.set_profiling(True)
    launches0 = ctx.launch_count()
    barrier(pg)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            d = one_dos()
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier(pg)
    t_dev = ev0.elapsed_time(ev1) / 1000.0 / args.steps
    launches = ctx.launch_count() - launches0
    k_n, k_ms = ctx.kernel_stats("cheb_step")
    ctx.set_profiling(False)
    t_dev_max = max_over_ranks(pg, t_dev)
    final_err = l1(d, d_ref)

    # the learned control variate (same target, same reference DOS)
    cv = None
    if not args.no_cv and ws == 1:
        cv = run_cv(L, ctx, csr, a, b, n, dos_of, d_ref, mu_cal, R_needed, t_dev, stream)

    # e2e: geometry description on the host -> DOS in host memory, through the C ABI
    def e2e_once():
        c2 = ctx.build_csr(g)
        lo2, hi2 = c2.bounds()
        a2, b2 = 1.01 * (hi2 - lo2) / 2, (hi2 + lo2) / 2
        c2.rescale(a2, -b2)
        mu = c2.kpm_dos(cfg)[:count]
        out = ctx.dos_reconstruct(reduce_moments(mu.sum(axis=0), count, pg), energies(a2, b2), a2, b2, 1.0 / n)
        c2.close()
        return mu, out

    e2e_once()
    barrier(pg)
    t1 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        mu_e, _ = e2e_once()
    t_e2e = max_over_ranks(pg, (time.perf_counter() - t1) / e2e_steps)
    import ctypes
    h2d = ctypes.sizeof(L.Geom) + P * 8 + N_E * 8
    d2h = mu_e.nbytes + N_E * 8 + 2 * 8

    peak, peak_kind = peaks()
    bytes_step = step_bytes(n, nnz, cols)  # per launch: one pass over one vector block
    achieved = bytes_step / (k_ms / k_n / 1000.0) / 1e9 if k_n else None
    # DRAM bytes per launch from the committed ncu capture of the same kernel on
    # a 2.4M-orbital flake, scaled to this launch by the algorithmic bytes
    # (traffic grows with rows and entries)
    traffic = None
    tp = os.path.join(REPO, "profiles", "cheb_step_traffic.json")
    if os.path.exists(tp):
        try:
            t = json.load(open(tp))[{0: "tiled", 3: "row_blocks", 4: "row_blocks_windows",
                                     5: "row_blocks_8_tensor_cores"}[kernel_id]]
            traffic = int(bytes_step * t["dram_bytes_per_launch"] / t["algorithmic_bytes_per_launch"])
        except (OSError, ValueError, KeyError, ZeroDivisionError):
            traffic = None

    out = {
        "metric": METRIC, "value": round(t_dev_max, 6), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_dev_max * 1000, 3),
        "higher_is_better": False, "scaling": "strong", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (geometry generated on the GPU; random-phase vectors, Philox)",
        "config": {"workload": f"TBLG flake {TWIST_DEG} deg, R={args.radius:.0f} A, {n} orbitals, "
                               f"simple model, P={P}, {N_E} energies",
                   "orbitals": n, "nnz": nnz, "poly_order": P, "vectors_to_1e-3": R_needed,
                   "ref_vectors": args.ref_vectors, "final_l1": final_err,
                   "fp32_vs_fp64_l1": fp32_l1, "block_cols": cols, "rows_per_slot": rows,
                   "passes_per_step": -(-2 * R_needed // cols), "autotune_s": round(t_tune, 2),
                   "l2": "inputs larger than L2 (8 GB matrix streamed every step)",
                   "parallelism": f"replicas x{ws}"},
        "e2e": {"value": round(t_e2e, 6), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1) if achieved else None,
                     "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4) if achieved else None, "traffic": traffic,
                     "kernel": kernel_name, "bytes_per_launch": bytes_step,
                     "launch_ms": round(k_ms / k_n, 4) if k_n else None,
                     "peak_kind": peak_kind},
        "clocks": clk.summary(),
        "build_s": round(t_build, 3),
        "l1_curve": [round(x, 6) for x in errs[:16]],
        "cv": cv,
    }
    if rank == 0 and ws == 1:
        # the reference's CPU recursion on the same full-size flake, built on the
        # host cores with the same rescale; and its FP64 moments of one of the
        # timed phase vectors against the device's FP32 ones
        cf = CpuFlake(L, threads, a=a, b=b)
        cf.time_steps(threads, 1)  # warm
        t_step = cf.time_steps(threads, CPU_STEPS)
        cpu_t = math.ceil(R_needed / threads) * (P // 2) * t_step
        out["cpu_baseline"] = {"value": round(cpu_t, 3), "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"oracle FP64 recursion (the reference's in-tree SpMV loop per vector) on "
                                         f"the full {cf.n}-orbital flake built on the host ({cf.nnz} entries), "
                                         f"{threads} vectors on {threads} threads, {CPU_STEPS} timed steps of "
                                         f"{t_step:.3f} s; x {P // 2} steps x {math.ceil(R_needed / threads)} "
                                         f"batch(es) for {R_needed} vectors",
                               "host_build_s": round(cf.build_s, 2)}
        Pc = 16
        mu_cpu = cf.moments(7, 0, 1, Pc, threads)
        mu_gpu = csr.kpm_dos(L.kpm_cfg(Pc, R=1, seed=7))
        out["parity_full_size"] = {
            "orbitals": n, "gpu_entries": nnz, "host_entries": cf.nnz, "moments": Pc, "vectors": 1,
            "fp32_gpu_vs_fp64_host_max_rel": float(np.max(np.abs(mu_gpu - mu_cpu)) / np.max(np.abs(mu_cpu)))}
        del cf
    if rank == 0:
        print(json.dumps(out))
    ctx.close()


def run_reference(args, threads):
    """CPU reference arm: the oracle port of the reference recursion (Locality::
    computeDosTraceKPM with SpMatrix::vectorMultiply's in-tree loop, one vector per
    worker) on the host cores, on the full 10M-orbital flake built on the host.
    A step is one Chebyshev step of `threads` vectors on `threads` threads;
    value = the mean timed step x P/2 steps x the vector batches R needs."""
    import leo2d_gb300 as L
    cf = CpuFlake(L, threads)
    cf.time_steps(threads, max(1, args.warmup))
    t_step = cf.time_steps(threads, max(1, args.steps))
    R = int(os.environ.get("LEO2D_BENCH_VECTORS", str(REF_VECTORS)))
    v = math.ceil(R / threads) * (P // 2) * t_step
    out = {"impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": UNIT,
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(t_step * 1000, 1), "higher_is_better": False,
           "scaling": "strong", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
           "config": {"workload": f"TBLG flake {TWIST_DEG} deg, R={RADIUS:.0f} A, {cf.n} orbitals, "
                                  f"simple model, P={P}, {N_E} energies", "orbitals": cf.n, "nnz": cf.nnz,
                      "vectors": R},
           "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"oracle FP64 recursion on the full {cf.n}-orbital flake built on the host "
                                      f"({cf.nnz} entries, {cf.build_s:.1f} s), {threads} vectors on {threads} "
                                      f"threads, {max(1, args.steps)} timed steps of {t_step:.3f} s; "
                                      f"x {P // 2} steps x {math.ceil(R / threads)} batch(es) for {R} vectors"},
           "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
