"""The 8-row tensor-core Chebyshev step (step_kernel = 5) against the gather
kernel and the FP64 oracle.

The step sums each row over its block's k-steps of 8 slots with TF32 products
split three ways (lo*hi + hi*lo + hi*hi, about 21 significant bits), so FP32
moments agree with the gather kernel's to rounding (2e-5 of the largest) and
with the FP64 oracle to 1e-4 (the FP32 bar). Repeated runs are bit-identical;
launch shapes (T_n rows staged in registers, in shared memory by cp.async or
by TMA row gathers; warps, rows in flight, blocks per run, tiles per CTA)
change the order in which the dots are summed and nothing else.
"""
import numpy as np
import pytest

import leo2d_gb300 as L
from oracle import oracle

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.fixture(scope="module")
def ctx():
    with L.Context(0) as c:
        yield c


def _flake(ctx, size, twist, model=L.MODEL_SIMPLE, keep_zeros=False):
    g = L.make_geom(model=model, size=size, angles_deg=(0.0, twist), energy_rescale=1.0)
    csr = ctx.build_csr(ctx.prepare(g), keep_zeros=keep_zeros)
    lo, hi = csr.bounds()
    csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
    return csr


def _run(ctx, variant, fn, **opts):
    ctx.set_option("step_kernel", variant)
    ctx.set_option("reorder", 1)
    for k, v in opts.items():
        ctx.set_option(k, v)
    try:
        return fn()
    finally:
        ctx.set_option("step_kernel", -1)
        ctx.set_option("reorder", -1)
        for k in ("rt_warps", "rt_depth", "rt_group", "rt_chunk", "rt_rows"):
            ctx.set_option(k, 0)
        ctx.set_option("rt_stage", -1)
        ctx.set_option("reorder_curve", 1)
        ctx.set_option("reorder_patch_dA", 0)


def _oracle_trace(csr, seed, R, P):
    rp, col, val = csr.download()
    re, im = oracle.phase_vectors(seed, 0, R, csr.n)
    return (oracle.kpm_trace(rp, col, val, re, P, literal=False) +
            oracle.kpm_trace(rp, col, val, im, P, literal=False))


@pytest.mark.parametrize("size,twist,model", [(22, 3.0, L.MODEL_SIMPLE), (37, 1.2, L.MODEL_SIMPLE),
                                             (25, 5.09, L.MODEL_REF)])
def test_rt_dos_matches(ctx, size, twist, model):
    csr = _flake(ctx, size, twist, model)
    P, R = 96, 16
    cfg = L.kpm_cfg(P, R=R, seed=3, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_dos(cfg))
    got = _run(ctx, 5, lambda: csr.kpm_dos(cfg))
    blocks, ksteps, union, max_slots = csr.rt_info()
    assert blocks == (csr.n + 7) // 8
    assert union <= 8 * ksteps < union + 8 * blocks
    assert union < csr.nnz and max_slots > 0
    assert _rel(got, ref) < 2e-5
    again = _run(ctx, 5, lambda: csr.kpm_dos(cfg))
    np.testing.assert_array_equal(got, again)
    assert _rel(got, _oracle_trace(csr, 3, R, P)) < 1e-4


@pytest.mark.parametrize("opts", [{"rt_stage": 1, "rt_warps": 8, "rt_depth": 3},
                                  {"rt_stage": 1, "rt_warps": 12, "rt_depth": 7},
                                  {"rt_stage": 1, "rt_warps": 24, "rt_depth": 3},
                                  {"rt_stage": 0, "rt_warps": 16, "rt_depth": 2},
                                  {"rt_stage": 0, "rt_warps": 12, "rt_depth": 6},
                                  {"rt_stage": 0, "rt_warps": 8, "rt_depth": 6},
                                  {"rt_stage": 2, "rt_warps": 16, "rt_depth": 3},
                                  {"rt_stage": 2, "rt_warps": 12, "rt_depth": 7},
                                  {"rt_stage": 2, "rt_warps": 8, "rt_depth": 7},
                                  {"rt_stage": 2, "rt_group": 3, "rt_chunk": 5},
                                  {"rt_rows": 16}, {"rt_rows": 16, "rt_warps": 12},
                                  {"rt_rows": 16, "rt_group": 3, "rt_chunk": 5},
                                  {"rt_group": 1}, {"rt_group": 7},
                                  {"rt_chunk": 1}, {"rt_chunk": 5, "rt_group": 3}])
def test_rt_launch_shapes(ctx, opts):
    """Warps, depth, blocks per run and tiles per CTA change the schedule (and the
    order of the dot sums), not the vectors."""
    csr = _flake(ctx, 30, 2.0)
    cfg = L.kpm_cfg(64, R=16, seed=5, block=32)
    base = _run(ctx, 5, lambda: csr.kpm_dos(cfg))
    got = _run(ctx, 5, lambda: csr.kpm_dos(cfg), **opts)
    rows = opts.get("rt_rows", 8)
    assert csr.rt_info()[0] == (csr.n + rows - 1) // rows
    assert _rel(got, base) < 1e-6


def test_rt_orderings(ctx):
    """The curve ordering and the reference-index ordering inside a patch, and
    other patch edges: different blocks, the same moments to rounding."""
    csr = _flake(ctx, 34, 1.5)
    cfg = L.kpm_cfg(64, R=16, seed=6, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_dos(cfg))
    curve = _run(ctx, 5, lambda: csr.kpm_dos(cfg))
    k_curve = csr.rt_info()[1]
    plain = _run(ctx, 5, lambda: csr.kpm_dos(cfg), reorder_curve=0)
    k_plain = csr.rt_info()[1]
    small = _run(ctx, 5, lambda: csr.kpm_dos(cfg), reorder_patch_dA=160)
    for got in (curve, plain, small):
        assert _rel(got, ref) < 2e-5
    assert k_curve < k_plain  # compact clusters of 8 rows share more columns


def test_rt_ldos_and_host_vectors(ctx):
    """Unit start vectors and host (Gaussian) vectors; after a second rescale the
    blocks are rebuilt."""
    csr = _flake(ctx, 26, 1.6)
    P = 64
    targets = np.arange(0, csr.n, max(1, csr.n // 40))[:32]
    cfg = L.kpm_cfg(P, R=1, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_ldos(cfg, targets))
    got = _run(ctx, 5, lambda: csr.kpm_ldos(cfg, targets))
    assert _rel(got, ref) < 2e-5
    rp, col, val = csr.download()
    assert _rel(got, oracle.kpm_ldos(rp, col, val, targets, P)) < 1e-4
    R = 20
    vec = np.random.default_rng(4).normal(size=(R, csr.n))
    cfgh = L.kpm_cfg(48, R=R, kind=L.VEC_HOST, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_dos(cfgh, vec))
    got = _run(ctx, 5, lambda: csr.kpm_dos(cfgh, vec))
    assert _rel(got, ref) < 2e-5
    csr.rescale(1.5, 0.0)
    assert csr.rt_info()[0] == 0  # dropped with the ordered copy
    ref2 = _run(ctx, 0, lambda: csr.kpm_dos(cfgh, vec))
    got2 = _run(ctx, 5, lambda: csr.kpm_dos(cfgh, vec))
    assert _rel(got2, ref2) < 2e-5
    assert _rel(got2, got) > 1e-3  # the values really changed


@pytest.mark.parametrize("rows", [8, 16])
def test_rt_ragged_last_block(ctx, rows):
    """Row counts that leave a partial last block (n not a multiple of the rows
    per block)."""
    seen = set()
    for size in (9, 10, 11, 13):
        csr = _flake(ctx, size, 4.0)
        seen.add(csr.n % rows)
        cfg = L.kpm_cfg(32, R=16, seed=9, block=32)
        ref = _run(ctx, 0, lambda: csr.kpm_dos(cfg))
        got = _run(ctx, 5, lambda: csr.kpm_dos(cfg), rt_rows=rows)
        assert csr.rt_info()[0] == (csr.n + rows - 1) // rows
        assert _rel(got, ref) < 2e-5, (size, csr.n)
    assert seen - {0}


def test_rt_stored_zeros(ctx):
    """A matrix that keeps every in-window pair (stored zeros): the 8-row blocks
    hold the zeros, or, for blocks past the build limit of 2048 entries, the
    recursion runs the gather kernels instead; the moments agree either way."""
    csr = _flake(ctx, 24, 2.5, keep_zeros=True)
    cfg = L.kpm_cfg(32, R=16, seed=2, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_dos(cfg))
    got = _run(ctx, 5, lambda: csr.kpm_dos(cfg))
    assert _rel(got, ref) < 2e-5
    assert _rel(got, _oracle_trace(csr, 2, 16, 32)) < 1e-4


@pytest.mark.parametrize("size,twist,model", [(23, 2.6, L.MODEL_SIMPLE), (25, 5.09, L.MODEL_REF)])
def test_rt_tma_gathers(ctx, size, twist, model):
    """T_n rows fetched by TMA row gathers (four 128-byte rows per copy, the
    128-byte swizzle) give the moments of the cp.async form to rounding and of
    the FP64 oracle to the FP32 bar; ragged last blocks included."""
    csr = _flake(ctx, size, twist, model)
    P, R = 80, 16
    cfg = L.kpm_cfg(P, R=R, seed=11, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_dos(cfg))
    cp = _run(ctx, 5, lambda: csr.kpm_dos(cfg), rt_stage=1, rt_warps=16, rt_depth=3)
    got = _run(ctx, 5, lambda: csr.kpm_dos(cfg), rt_stage=2, rt_warps=16, rt_depth=3)
    assert csr.rt_info()[0] == (csr.n + 7) // 8
    assert _rel(got, cp) < 1e-6
    assert _rel(got, ref) < 2e-5
    again = _run(ctx, 5, lambda: csr.kpm_dos(cfg), rt_stage=2, rt_warps=16, rt_depth=3)
    np.testing.assert_array_equal(got, again)
    assert _rel(got, _oracle_trace(csr, 11, R, P)) < 1e-4


def test_rt_tma_timeout_reports(ctx):
    """The bounded wait of the TMA form: a barrier nobody completes gives
    LEO2D_ERR_TIMEOUT, and the context keeps working afterwards."""
    csr = _flake(ctx, 20, 3.0)
    cfg = L.kpm_cfg(16, R=16, seed=1, block=32)
    ok = _run(ctx, 5, lambda: csr.kpm_dos(cfg), rt_stage=2, rt_warps=16, rt_depth=3)
    ctx.set_spin_limit(2000)
    ctx.set_option("test_unsatisfied_wait", 1)
    try:
        with pytest.raises(L.Leo2dError) as e:
            _run(ctx, 5, lambda: csr.kpm_dos(cfg), rt_stage=2, rt_warps=16, rt_depth=3)
        assert e.value.status == L._abi.ERR_TIMEOUT
        assert "wait ran out" in str(e.value)
    finally:
        ctx.set_option("test_unsatisfied_wait", 0)
        ctx.set_spin_limit(0)
    again = _run(ctx, 5, lambda: csr.kpm_dos(cfg), rt_stage=2, rt_warps=16, rt_depth=3)
    np.testing.assert_array_equal(ok, again)


@pytest.mark.parametrize("size,twist,model", [(22, 3.0, L.MODEL_SIMPLE), (37, 1.2, L.MODEL_SIMPLE),
                                             (25, 5.09, L.MODEL_REF)])
def test_rt16_dos_matches(ctx, size, twist, model):
    """Blocks of 16 rows (two n-tiles sharing each k-step's gathered rows): the
    moments of the gather kernel to rounding, of the FP64 oracle to the FP32
    bar, bit-identical on repeat; fewer union slots per row than 8-row blocks."""
    csr = _flake(ctx, size, twist, model)
    P, R = 96, 16
    cfg = L.kpm_cfg(P, R=R, seed=3, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_dos(cfg))
    _run(ctx, 5, lambda: csr.kpm_dos(cfg), rt_rows=8)
    union8 = csr.rt_info()[2]
    got = _run(ctx, 5, lambda: csr.kpm_dos(cfg), rt_rows=16)
    blocks, ksteps, union, max_slots = csr.rt_info()
    assert blocks == (csr.n + 15) // 16
    assert union <= 8 * ksteps < union + 8 * blocks
    assert union < union8 and max_slots > 0
    assert _rel(got, ref) < 2e-5
    again = _run(ctx, 5, lambda: csr.kpm_dos(cfg), rt_rows=16)
    np.testing.assert_array_equal(got, again)
    assert _rel(got, _oracle_trace(csr, 3, R, P)) < 1e-4


def test_rt16_stored_zeros_and_host_vectors(ctx):
    """16-row blocks over a matrix with stored zeros, and host (Gaussian) start
    vectors."""
    csr = _flake(ctx, 24, 2.5, keep_zeros=True)
    cfg = L.kpm_cfg(32, R=16, seed=2, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_dos(cfg))
    got = _run(ctx, 5, lambda: csr.kpm_dos(cfg), rt_rows=16)
    assert _rel(got, ref) < 2e-5
    vec = np.random.default_rng(8).normal(size=(20, csr.n))
    cfgh = L.kpm_cfg(48, R=20, kind=L.VEC_HOST, block=32)
    ref = _run(ctx, 0, lambda: csr.kpm_dos(cfgh, vec))
    got = _run(ctx, 5, lambda: csr.kpm_dos(cfgh, vec), rt_rows=16)
    assert _rel(got, ref) < 2e-5
