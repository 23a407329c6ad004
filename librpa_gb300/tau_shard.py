"""Tau sharding of the RPA correlation energy across ranks (one process, one GPU per rank).

chi0(q, omega) = sum_tau gamma(omega, tau) FT[chi0(R, tau)] (LibRPA chi0.cpp:507-596) is a sum
over the minimax tau points, and each term needs only that tau's G(R, +-tau).  Rank r
therefore builds the partial sum over a contiguous slice of tau points
(LibrpaGB300Options.tau_begin / tau_end, stage CHI0), one all-reduce over the process group
adds the partials, and every rank then evaluates E_c from the full chi0(q, omega) (stage EC).
The all-reduce is the path's only exchange step; its size is n_omega * n_q * sum_pairs
n_mu n_nu complex numbers.
"""
from __future__ import annotations

import numpy as np

from . import STAGE_CHI0, STAGE_EC, gb300_options


def tau_slices(n_tau: int, world: int) -> list[tuple[int, int]]:
    """Contiguous, balanced [begin, end) slices of n_tau points over `world` ranks (the first
    n_tau % world ranks take one point more); every point in exactly one slice."""
    if n_tau < 0 or world < 1:
        raise ValueError("n_tau >= 0 and world >= 1 required")
    base, extra = divmod(n_tau, world)
    out, b = [], 0
    for r in range(world):
        e = b + base + (1 if r < extra else 0)
        out.append((b, e))
        b = e
    return out


def allreduce_sum(a: np.ndarray, group=None) -> np.ndarray:
    """Sum a complex128 array over the ranks of the default (or given) process group.  NCCL
    groups reduce a CUDA copy, gloo groups the host array."""
    import torch
    import torch.distributed as dist

    flat = np.ascontiguousarray(a, np.complex128).view(np.float64)
    t = torch.from_numpy(flat.copy())
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy().view(np.complex128).reshape(np.shape(a))


def sharded_correlation_energy(h, opts, n_ibz: int, group=None, reduce=allreduce_sum, **gb_options):
    """E_c with this rank's tau slice; `h` is a Handler with the system loaded, `opts` the
    LibrpaOptions of the call, gb_options further LibrpaGB300Options fields.  Returns what
    Handler.get_rpa_correlation_energy returns, identical on every rank."""
    import torch.distributed as dist

    rank = dist.get_rank(group) if dist.is_initialized() else 0
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    b, e = tau_slices(int(opts.nfreq), world)[rank]
    h.set_gb300_options(gb300_options(**gb_options, tau_begin=b, tau_end=e, stage=STAGE_CHI0))
    h.get_rpa_correlation_energy(opts, n_ibz)
    part = h.chi0_qw()
    total = reduce(part, group) if world > 1 else part
    h.load_chi0_qw(total)
    h.set_gb300_options(gb300_options(**gb_options, stage=STAGE_EC))
    return h.get_rpa_correlation_energy(opts, n_ibz)
