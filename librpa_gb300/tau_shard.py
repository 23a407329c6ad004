"""Tau and q sharding of the RPA correlation energy across ranks (one process, one GPU per rank).

chi0(q, omega) = sum_tau gamma(omega, tau) FT[chi0(R, tau)] (LibRPA chi0.cpp:507-596) is a sum
over the minimax tau points, and each term needs only that tau's G(R, +-tau).  Rank r
therefore builds the partial sum over a contiguous slice of tau points
(LibrpaGB300Options.tau_begin / tau_end, stage CHI0).  One reduce-scatter over the process
group, keyed by q, hands each rank the summed chi0(q, omega) of its own slice of IBZ q points.
The rank then evaluates the E_c terms of those q (stage EC with q_begin / q_end), and an
all-reduce of the n_q per-q sums gives every rank the same E_c.  The reduce-scatter is the
path's one bulk exchange: n_omega * n_q * sum_pairs n_mu n_nu complex numbers in total.
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


def q_slices(n_q: int, world: int) -> list[tuple[int, int]]:
    """Contiguous, balanced [begin, end) slices of the IBZ q points over `world` ranks."""
    return tau_slices(n_q, world)


def reduce_scatter_q(part: np.ndarray, n_w: int, n_q: int, group=None) -> tuple[np.ndarray, tuple[int, int]]:
    """Sum the [omega][q][pair blocks] partials over the ranks; this rank receives the sum for
    its own q slice (returned in the full layout, other q zero) and the slice.  NCCL groups use
    one reduce-scatter of q-major, equally padded rank blocks; gloo, which has no
    reduce-scatter, all-reduces the same buffer and keeps this rank's block."""
    import torch
    import torch.distributed as dist

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    a = np.ascontiguousarray(part, np.complex128).reshape(n_w, n_q, -1)
    sl = q_slices(n_q, world)
    width = max(1, max(e - b for b, e in sl))
    buf = np.zeros((world, width, n_w, a.shape[2]), np.complex128)
    for r, (b, e) in enumerate(sl):
        buf[r, :e - b] = a[:, b:e, :].transpose(1, 0, 2)
    t = torch.from_numpy(buf.view(np.float64).reshape(-1).copy())
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
        out = torch.empty(t.numel() // world, dtype=t.dtype, device=t.device)
        dist.reduce_scatter_tensor(out, t, op=dist.ReduceOp.SUM, group=group)
    else:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        out = t.view(world, -1)[rank]
    mine = out.cpu().numpy().view(np.complex128).reshape(width, n_w, a.shape[2])
    b, e = sl[rank]
    full = np.zeros_like(a)
    full[:, b:e, :] = mine[:e - b].transpose(1, 0, 2)
    return full.reshape(-1), (b, e)


def reduce_scatter_q_tensor(part, n_w: int, n_q: int, group=None):
    """reduce_scatter_q on a torch tensor: `part` holds the complex [omega][q][pair blocks]
    partial as float64 pairs (re, im), on this rank's GPU for NCCL groups or on the host for
    gloo.  The rank-blocked packing, the collective and the unpacking into the full layout (other
    q zero) all run where the tensor lives, so an NCCL group never copies chi0 to the host."""
    import torch
    import torch.distributed as dist

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    a = part.reshape(n_w, n_q, -1)
    sl = q_slices(n_q, world)
    width = max(1, max(e - b for b, e in sl))
    buf = torch.zeros((world, width, n_w, a.shape[2]), dtype=a.dtype, device=a.device)
    for r, (b, e) in enumerate(sl):
        buf[r, :e - b] = a[:, b:e, :].transpose(0, 1)
    if dist.get_backend(group) == "nccl":
        out = torch.empty(width * n_w * a.shape[2], dtype=a.dtype, device=a.device)
        dist.reduce_scatter_tensor(out, buf.reshape(-1), op=dist.ReduceOp.SUM, group=group)
    else:
        dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
        out = buf[rank]
    mine = out.reshape(width, n_w, a.shape[2])
    b, e = sl[rank]
    full = torch.zeros_like(a)
    full[:, b:e, :] = mine[:e - b].transpose(0, 1)
    return full.reshape(-1), (b, e)


def sharded_correlation_energy(h, opts, n_ibz: int, group=None, resident=None, stats=None, **gb_options):
    """E_c with this rank's tau slice and q slice; `h` is a Handler with the system loaded,
    `opts` the LibrpaOptions of the call, gb_options further LibrpaGB300Options fields.
    resident (default: on for NCCL groups) exchanges chi0(q, omega) as a torch tensor copied
    device to device out of and back into the library (librpa_gb300_copy_chi0_qw /
    librpa_gb300_load_chi0_qw with on_device = 1); otherwise through host numpy arrays.
    stats, a list, receives the handler's counters after each of the two stages.
    Returns (E_c, per-q contributions), identical on every rank."""
    import torch.distributed as dist

    rank = dist.get_rank(group) if dist.is_initialized() else 0
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    n_w = int(opts.nfreq)
    b, e = tau_slices(n_w, world)[rank]
    h.set_gb300_options(gb300_options(**gb_options, tau_begin=b, tau_end=e, stage=STAGE_CHI0))
    h.get_rpa_correlation_energy(opts, n_ibz)
    if stats is not None:
        stats.append(h.stats())
    qa, qe = 0, n_ibz
    if world > 1:
        nccl = dist.get_backend(group) == "nccl"
        if resident is None:
            resident = nccl
        if resident:
            import torch
            dev = torch.device("cuda", torch.cuda.current_device()) if nccl else torch.device("cpu")
            mine, (qa, qe) = reduce_scatter_q_tensor(h.chi0_qw_tensor(dev), n_w, n_ibz, group)
            h.load_chi0_qw_tensor(mine)
        else:
            mine, (qa, qe) = reduce_scatter_q(h.chi0_qw(), n_w, n_ibz, group)
            h.load_chi0_qw(mine)
    # world 1: the kept chi0(q, omega) is already the full sum
    h.set_gb300_options(gb300_options(**gb_options, stage=STAGE_EC, q_begin=qa, q_end=qe))
    _, per_q = h.get_rpa_correlation_energy(opts, n_ibz)
    if stats is not None:
        stats.append(h.stats())
    per_q = np.asarray(per_q, np.complex128)
    if world > 1:
        per_q = allreduce_sum(per_q, group)
    return float(per_q.sum().real), per_q
