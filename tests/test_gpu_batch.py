"""Batched flakes (leo2d_batch_*) replayed from a CUDA graph: every step of a
32-column pass over ordered flakes in one cooperative launch (the 8-row
tensor-core step, CTA groups meeting at per-flake barriers), otherwise one
launch per Chebyshev step over all the matrices.

Each flake's moments must equal those of the single-matrix recursion on the
same Philox vectors. Both are FP32 recursions with FP64 moment sums, but the
batched grid splits rows into different tiles, so FP32 partial sums round
differently: tolerance 1e-5 of the largest moment. One flake is also checked
against the FP64 oracle (1e-4, the FP32 bar). Replays are bit-identical.
"""
import numpy as np
import pytest

import leo2d_gb300 as L
from oracle import oracle

pytestmark = pytest.mark.gpu
FP32_RTOL = 1e-4


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.fixture(scope="module")
def ctx():
    with L.Context(0) as c:
        yield c


@pytest.fixture(scope="module")
def flakes(ctx):
    out = []
    for size, twist in ((9, 1.2), (14, 2.5), (6, 0.9), (20, 3.0)):
        g = L.make_geom(model=L.MODEL_SIMPLE, size=size, angles_deg=(0.0, twist), energy_rescale=1.0)
        csr = ctx.build_csr(ctx.prepare(g))
        lo, hi = csr.bounds()
        csr.rescale(1.01 * (hi - lo) / 2, -(hi + lo) / 2)
        out.append(csr)
    return out


@pytest.mark.parametrize("block", [0, 8, 16, 32, 64])
def test_batch_matches_single(ctx, flakes, block):
    P, R, seed = 64, 5, 17
    cfg = L.kpm_cfg(P, R=R, seed=seed, block=block)
    b = L.Batch(ctx, flakes, cfg)
    mu = b.run()
    assert mu.shape == (len(flakes), R, P)
    for f, csr in enumerate(flakes):
        single = csr.kpm_dos(L.kpm_cfg(P, R=R, seed=seed))
        assert _rel(mu[f], single) < 1e-5, (f, block)
    again = b.run()
    np.testing.assert_array_equal(mu, again)
    if block:
        assert b.block_cols == block
    if b.warps == 16:  # the one-launch form (32-column passes over ordered flakes)
        passes = -(-2 * R // b.block_cols)
        assert b.launches_per_run == passes * (2 * len(flakes) + 1)
    else:
        assert b.launches_per_run >= P // 2
    b.close()


def test_batch_seed_and_first_vector(ctx, flakes):
    P, R = 32, 3
    b = L.Batch(ctx, flakes[:2], L.kpm_cfg(P, R=R, seed=1, block=16))
    mu = b.run(seed=99, first_vector=7)
    for f in range(2):
        single = flakes[f].kpm_dos(L.kpm_cfg(P, R=R, seed=99, first_vector=7))
        assert _rel(mu[f], single) < 1e-5
    b.close()


def test_batch_vs_oracle(ctx, flakes):
    P, R, seed = 48, 4, 3
    b = L.Batch(ctx, flakes, L.kpm_cfg(P, R=R, seed=seed, block=16))
    mu = b.run()
    csr = flakes[1]
    rp, col, val = csr.download()
    re, im = oracle.phase_vectors(seed, 0, R, csr.n)
    ref = oracle.kpm_trace(rp, col, val, re, P, literal=False) + oracle.kpm_trace(rp, col, val, im, P, literal=False)
    assert _rel(mu[1], ref) < FP32_RTOL
    b.close()


def test_batch_rejects(ctx, flakes):
    with pytest.raises(L.Leo2dError, match="twice"):
        L.Batch(ctx, [flakes[0], flakes[0]], L.kpm_cfg(16, R=1))
    with pytest.raises(L.Leo2dError, match="FP32"):
        L.Batch(ctx, flakes[:1], L.kpm_cfg(16, R=1, precision=L.FP64))
    with pytest.raises(L.Leo2dError, match="random-phase"):
        L.Batch(ctx, flakes[:1], L.kpm_cfg(16, R=1, kind=L.VEC_GAUSSIAN))


def test_batch_row_blocks(ctx, flakes):
    """With step_kernel 3, flakes with positions at 32 columns run the 4-row step in
    one launch per step (24 warps per CTA, a block group per flake): each flake's
    vectors are those of the single-matrix 4-row step, so the moments agree with it
    to the order of the FP64 dot sums, and with the FP64 oracle to 1e-4."""
    P, R, seed = 64, 16, 8
    ctx.set_option("step_kernel", 3)
    ctx.set_option("reorder", 1)
    try:
        b = L.Batch(ctx, flakes, L.kpm_cfg(P, R=R, seed=seed, block=32))
        assert b.warps == 24 and b.block_cols == 32
        mu = b.run()
        np.testing.assert_array_equal(mu, b.run())
        singles = [c.kpm_dos(L.kpm_cfg(P, R=R, seed=seed, block=32)) for c in flakes]
    finally:
        ctx.set_option("step_kernel", -1)
        ctx.set_option("reorder", -1)
    for f in range(len(flakes)):
        assert _rel(mu[f], singles[f]) < 1e-9, f
    csr = flakes[3]
    rp, col, val = csr.download()
    re, im = oracle.phase_vectors(seed, 0, R, csr.n)
    ref = oracle.kpm_trace(rp, col, val, re, P, literal=False) + oracle.kpm_trace(rp, col, val, im, P, literal=False)
    assert _rel(mu[3], ref) < FP32_RTOL
    b.close()


def test_batch_one_launch_per_pass(ctx, flakes):
    """By default, ordered flakes at 32 columns run every step of a pass in ONE
    cooperative launch of the 8-row tensor-core step (16 warps per CTA, the CTAs of
    each flake meeting at a barrier between steps): per pass the graph holds the
    fills, that launch and the final reductions. The rows are those of the
    single-matrix 8-row step; the moment sums group blocks differently (1e-5), and
    the FP64 oracle holds at the FP32 bar. Replays are bit-identical."""
    P, R, seed = 64, 20, 8  # 40 columns: two passes, the second partly empty
    b = L.Batch(ctx, flakes, L.kpm_cfg(P, R=R, seed=seed))
    assert b.warps == 16 and b.block_cols == 32
    F, passes = len(flakes), 2
    assert b.launches_per_run == passes * (2 * F + 1)
    mu = b.run()
    np.testing.assert_array_equal(mu, b.run())
    ctx.set_option("step_kernel", 5)
    ctx.set_option("reorder", 1)
    try:
        singles = [c.kpm_dos(L.kpm_cfg(P, R=R, seed=seed, block=32)) for c in flakes]
    finally:
        ctx.set_option("step_kernel", -1)
        ctx.set_option("reorder", -1)
    for f in range(F):
        assert _rel(mu[f], singles[f]) < 1e-5, f
    # the single runs rebuilt each flake's 8-row blocks for one CTA per SM: the
    # next run rebuilds them for the batch's CTA groups and gives the same moments
    np.testing.assert_array_equal(mu, b.run())
    csr = flakes[2]
    rp, col, val = csr.download()
    re, im = oracle.phase_vectors(seed, 0, R, csr.n)
    ref = oracle.kpm_trace(rp, col, val, re, P, literal=False) + oracle.kpm_trace(rp, col, val, im, P, literal=False)
    assert _rel(mu[2], ref) < FP32_RTOL
    b.close()


def test_batch_one_launch_barrier_gives_up(ctx, flakes):
    """The step barriers of the one-launch form are bounded: with a test hook that
    makes each barrier wait for one arrival more than its flake's CTAs make, every
    CTA gives up after the spin limit, the run reports LEO2D_ERR_TIMEOUT, and the
    context runs the next batch normally."""
    P, R, seed = 16, 4, 3
    ctx.set_spin_limit(2000)
    ctx.set_option("test_unsatisfied_wait", 1)
    try:
        b = L.Batch(ctx, flakes, L.kpm_cfg(P, R=R, seed=seed))
        with pytest.raises(L.Leo2dError) as e:
            b.run()
        assert e.value.status == L._abi.ERR_TIMEOUT
        b.close()
    finally:
        ctx.set_option("test_unsatisfied_wait", 0)
        ctx.set_spin_limit(0)
    b = L.Batch(ctx, flakes, L.kpm_cfg(P, R=R, seed=seed))
    mu = b.run()
    for f, csr in enumerate(flakes):
        assert _rel(mu[f], csr.kpm_dos(L.kpm_cfg(P, R=R, seed=seed))) < 1e-5
    b.close()
