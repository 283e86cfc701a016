"""Replicas on several GPUs: vector shares and the one moment reduction.

The stochastic trace is a sum over independent vectors, so N GPUs each hold
the whole Hamiltonian and run a contiguous share of the vectors. The only
exchange is an FP64 sum of the per-rank moment sums (the reference's MPI farm
hands out whole jobs instead, locality.cpp:2295-2309, and its root sums the
returned cheb_coeffs). Vector indices are global, so the union of the shares
is the same set of Philox vectors that one GPU would draw.
"""


def vector_share(total, rank, world):
    """(first, count) of the contiguous share of `total` vectors for `rank`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(int(total), int(world))
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def reduce_moments(mu_sum, count, group=None):
    """All-reduces per-rank moment sums (FP64) and vector counts; returns the mean.

    `mu_sum` is a NumPy array (any shape) holding the sum over this rank's
    vectors; `group` is the torch.distributed module (or None for one rank).
    Works on gloo (CPU tensors) and NCCL (CUDA tensors).
    """
    import numpy as np
    mu_sum = np.asarray(mu_sum, dtype=np.float64)
    if group is None:
        return mu_sum / count
    import torch
    dev = "cuda" if group.get_backend() == "nccl" else "cpu"
    t = torch.from_numpy(np.append(mu_sum.ravel(), float(count))).to(dev)
    group.all_reduce(t, op=group.ReduceOp.SUM)
    t = t.cpu().numpy()
    return (t[:-1] / t[-1]).reshape(mu_sum.shape)
