"""Tau and q sharding across ranks on CPU: the slice partitions, and the sharded E_c with two
and three gloo ranks.  The per-rank compute is the oracle standing in for a GPU; what is tested
is the partition, the stage sequence, the reduce-scatter by q and the all-reduce of the per-q
sums in tau_shard.sharded_correlation_energy."""
import os
import socket

import numpy as np
import pytest

import librpa_gb300 as L
from librpa_gb300 import synthetic as sy
from librpa_gb300.tau_shard import sharded_correlation_energy, tau_slices


@pytest.mark.parametrize("n_tau,world", [(16, 1), (16, 2), (16, 3), (24, 5), (3, 4), (0, 2), (32, 8)])
def test_tau_slices_partition(n_tau, world):
    sl = tau_slices(n_tau, world)
    assert len(sl) == world
    covered = [t for b, e in sl for t in range(b, e)]
    assert covered == list(range(n_tau))
    sizes = [e - b for b, e in sl]
    assert max(sizes) - min(sizes) <= 1


def _system():
    return sy.small_periodic(n_atoms=2, nao=[3, 4], nabf=[6, 8], period=(2, 1, 1), nocc=2, seed=9)


class OracleHandler:
    """The Handler calls the sharding uses, computed by the oracle (tests only)."""

    def __init__(self, s):
        from conftest import oracle_input
        from oracle.rpa_oracle import Options
        self.inp = oracle_input(s)
        self.oopts = Options(nfreq=s.nfreq, minimax_emin=s.minimax_emin, minimax_emax=s.minimax_emax)
        self.go = None
        self.kept = None
        self.shape = None

    def set_gb300_options(self, go):
        self.go = go

    def get_rpa_correlation_energy(self, opts, n_ibz):
        from oracle.rpa_oracle import chi0q_partial, ec_from_chi0q
        if self.go.stage == L.STAGE_CHI0:
            chi0q = chi0q_partial(self.inp, self.oopts, self.go.tau_begin, self.go.tau_end)
            self.shape = [[{k: v.shape for k, v in d.items()} for d in row] for row in chi0q]
            self.kept = np.concatenate([v.ravel() for row in chi0q for d in row for v in d.values()])
            return 0.0, np.zeros(n_ibz, complex)
        assert self.go.stage == L.STAGE_EC
        chi0q, off = [], 0
        for row in self.shape:
            out_row = []
            for d in row:
                blk = {}
                for k, shp in d.items():
                    n = shp[0] * shp[1]
                    blk[k] = self.kept[off:off + n].reshape(shp)
                    off += n
                out_row.append(blk)
            chi0q.append(out_row)
        ec, per_q, _ = ec_from_chi0q(self.inp, self.oopts, chi0q)
        per_q = np.asarray(per_q, complex)
        qa, qe = self.go.q_begin, (len(per_q) if self.go.q_end < 0 else self.go.q_end)
        keep = np.zeros(len(per_q), bool)
        keep[qa:qe] = True
        per_q = np.where(keep, per_q, 0)  # the E_c terms of this call's q slice only
        return per_q.sum().real, per_q

    def chi0_qw(self):
        return self.kept.copy()

    def load_chi0_qw(self, a):
        self.kept = np.array(a, np.complex128)

    def chi0_qw_tensor(self, device):
        import torch
        return torch.from_numpy(self.kept.view(np.float64).copy()).to(device)

    def load_chi0_qw_tensor(self, t):
        self.kept = t.cpu().numpy().view(np.complex128).copy()


def _rank_main(rank, world, port, out_dir, resident=False):
    import sys
    sys.path.insert(0, os.path.dirname(__file__))
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        s = _system()
        h = OracleHandler(s)
        opts = L.Options(nfreq=s.nfreq, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI)
        ec, per_q = sharded_correlation_energy(h, opts, L.n_ibz(s), resident=resident)
        np.save(os.path.join(out_dir, f"ec{rank}.npy"), np.array([ec]))
        np.save(os.path.join(out_dir, f"perq{rank}.npy"), per_q)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world,resident", [(2, False), (3, False), (2, True), (3, True)])
def test_gloo_ranks_sharded_ec_matches_unsharded(tmp_path, lib, world, resident):
    """resident: the exchange runs on torch tensors (the NCCL path's packing and unpacking, here
    on host tensors over gloo) instead of numpy arrays."""
    import torch.multiprocessing as mp
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path), resident), nprocs=world,
                       start_method="spawn")
    from conftest import oracle_input
    from oracle.rpa_oracle import Options, rpa_correlation_energy
    s = _system()
    r = rpa_correlation_energy(oracle_input(s), Options(nfreq=s.nfreq, minimax_emin=s.minimax_emin,
                                                        minimax_emax=s.minimax_emax))
    ref = r["ec"].real
    ecs = [float(np.load(tmp_path / f"ec{k}.npy")[0]) for k in range(world)]
    perqs = [np.load(tmp_path / f"perq{k}.npy") for k in range(world)]
    # every rank ends with the same per-q sums and E_c; each q was evaluated by one rank only
    assert all(e == ecs[0] for e in ecs)
    assert all(np.array_equal(p, perqs[0]) for p in perqs)
    assert abs(ecs[0] - ref) <= 1e-12 * abs(ref)
    np.testing.assert_allclose(perqs[0], np.asarray(r["per_q"]), rtol=1e-11, atol=1e-15)


def _rs_main(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist
    from librpa_gb300.tau_shard import reduce_scatter_q, reduce_scatter_q_tensor
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(rank)
        part = rng.standard_normal(5 * 7 * 6) + 1j * rng.standard_normal(5 * 7 * 6)
        a, sa = reduce_scatter_q(part, 5, 7)
        t, st = reduce_scatter_q_tensor(torch.from_numpy(part.view(np.float64).copy()), 5, 7)
        assert sa == st
        np.save(os.path.join(out_dir, f"rs{rank}.npy"), np.stack([a, t.numpy().view(np.complex128)]))
    finally:
        dist.destroy_process_group()


def test_tensor_reduce_scatter_equals_numpy_form(tmp_path):
    """The tensor form of the q-keyed reduce-scatter gives each rank the numpy form's result, and
    that result is the sum over ranks on the rank's own q slice, zero elsewhere."""
    import torch.multiprocessing as mp
    from librpa_gb300.tau_shard import q_slices
    world = 3
    mp.start_processes(_rs_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    total = np.zeros(210, complex)
    for r in range(world):
        rng = np.random.default_rng(r)
        total += rng.standard_normal(210) + 1j * rng.standard_normal(210)
    total = total.reshape(5, 7, 6)
    for r, (b, e) in enumerate(q_slices(7, world)):
        got = np.load(tmp_path / f"rs{r}.npy")
        assert np.array_equal(got[0], got[1])
        want = np.zeros_like(total)
        want[:, b:e] = total[:, b:e]
        np.testing.assert_allclose(got[1].reshape(5, 7, 6), want, rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("n_q,world", [(2, 2), (2, 3), (27, 4), (1, 2)])
def test_q_slices_partition(n_q, world):
    from librpa_gb300.tau_shard import q_slices
    sl = q_slices(n_q, world)
    assert [q for b, e in sl for q in range(b, e)] == list(range(n_q))
