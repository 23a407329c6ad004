"""Seeded synthetic RPA inputs with the shapes of the benchmark configurations.

The generated arrays are in the form the librpa_set_* entry points take them
(occupations as raw band occupations, eigenvectors band-major, RI coefficients
as (n_i*n_j) x n_mu row-major blocks, Coulomb blocks for upper atom pairs).

Workloads (sizes as named in the benchmark table):
  fcc2_k222   : 2-atom fcc cell (a = 3.57 A), 2x2x2 k, 13 NAO / 40 ABF per atom,
                26 bands with 4 occupied, 16 minimax points.
  fcc16_k333  : 2x2x2 supercell of that cell (16 atoms), 3x3x3 k, 104 bands with
                16 occupied, 13 NAO / 40 ABF per atom.
  mixed64_g   : 64 atoms of random species (NAO/ABF 5/20, 13/60, 26/110), Gamma only.
  sc256_g     : 256 atoms, 13 NAO / 40 ABF, C decay length 1.5 A, Gamma only.
  batch32_small (BATCHES): 32 independent Gamma cells of 2-8 atoms of random species
                (NAO/ABF 5/20, 13/60, 26/110), 24 minimax points (the small-cell batch
                of the mixed-species configuration).

Distributions: KS energies uniform in [-0.8,-0.2] Ha (occupied) and
[0.1,2.0] Ha (virtual); eigenvectors from the QR factor of a complex
Gaussian with psi(-k) = conj(psi(k)); C = sigma_C * N(0,1) * exp(-d / decay);
V(q) = A A^H + 0.1 I with A complex Gaussian / sqrt(N) and V(-q) = conj(V(q)).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

ANGSTROM = 1.8897259886  # Bohr per Angstrom
MINIMAX_EMIN = 0.25
MINIMAX_RANGE = {16: 100.0, 24: 3000.0, 32: 10000.0}


def _window(nfreq):
    return MINIMAX_EMIN, MINIMAX_EMIN * MINIMAX_RANGE.get(nfreq, 100.0)


@dataclass
class SynthSystem:
    name: str
    n_spins: int
    n_kpts: int
    n_bands: int
    n_ao: int
    period: tuple
    latvec: np.ndarray      # rows a1..a3, Bohr
    kvecs: np.ndarray       # (nk, 3) Cartesian Bohr^-1 (incl. 2 pi)
    ibz_map: np.ndarray     # (nk,)
    positions: np.ndarray   # (nat, 3) Bohr
    types: np.ndarray       # (nat,)
    nao: list
    nabf: list
    wg: np.ndarray          # (ns, nk, nb) raw occupations (2 for occupied, spin-unpolarised)
    ekb: np.ndarray
    efermi: float
    wfc: np.ndarray         # (ns, nk, nb, nao) complex128
    Cs: dict                # (I, J, R) -> (n_i*n_j, n_mu)
    Vq: dict                # (ik, I, J) I<=J -> complex (n_mu, n_nu)
    nfreq: int = 16
    # Minimax energy window passed as LibrpaOptions.minimax_emin/emax.  The
    # synthetic band structures are narrow (e_max/e_min ~ 9), where GreenX's
    # tabulated grids make the cosine-weight fit singular; a window of
    # e_max/e_min = MINIMAX_RANGE[nfreq] keeps the fit well conditioned.
    minimax_emin: float = 0.25
    minimax_emax: float = 25.0

    @property
    def n_atoms(self):
        return len(self.nao)


def _r_grid(period):
    return [(x, y, z)
            for x in range(-(period[0] // 2), (period[0] - 1) // 2 + 1)
            for y in range(-(period[1] // 2), (period[1] - 1) // 2 + 1)
            for z in range(-(period[2] // 2), (period[2] - 1) // 2 + 1)]


def _kmesh(period, latvec):
    """Gamma-centred mesh; returns Cartesian k (with 2 pi) and fractional coords."""
    recip = 2.0 * math.pi * np.linalg.inv(latvec).T  # rows b_i, a_i.b_j = 2pi d_ij
    fr = []
    for i in range(period[0]):
        for j in range(period[1]):
            for k in range(period[2]):
                fr.append((i / period[0], j / period[1], k / period[2]))
    fr = np.array(fr)
    return fr @ recip, fr


def _partner(fr, period):
    """Index of -k for each k on the mesh."""
    key = {}
    for i, f in enumerate(fr):
        key[tuple(int(round(x * p)) % p for x, p in zip(f, period))] = i
    out = []
    for f in fr:
        out.append(key[tuple((-int(round(x * p))) % p for x, p in zip(f, period))])
    return np.array(out)


def _mean_field(rng, nk, nb, nao, nocc, partner):
    ekb = np.zeros((1, nk, nb))
    wfc = np.zeros((1, nk, nb, nao), complex)
    done = set()
    for k in range(nk):
        if k in done:
            continue
        p = partner[k]
        e = np.concatenate([np.sort(rng.uniform(-0.8, -0.2, nocc)),
                            np.sort(rng.uniform(0.1, 2.0, nb - nocc))])
        z = rng.standard_normal((nao, nb)) + 1j * rng.standard_normal((nao, nb))
        if p == k:
            z = z.real + 0j  # self-partner k: real orthogonal vectors keep G(R) real
        q, r = np.linalg.qr(z)
        q = q * np.sign(np.diag(r).real)[None, :]
        ekb[0, k] = e
        wfc[0, k] = q.T
        if p != k:
            ekb[0, p] = e
            wfc[0, p] = q.T.conj()
            done.add(p)
        done.add(k)
    wg = np.zeros((1, nk, nb))
    wg[:, :, :nocc] = 2.0
    homo = ekb[0, :, nocc - 1].max()
    lumo = ekb[0, :, nocc].min()
    return wg, ekb, wfc, 0.5 * (homo + lumo)


def _cs(rng, positions, latvec, cells, nao, nabf, decay_bohr, sigma):
    Cs = {}
    nat = len(nao)
    for I in range(nat):
        for J in range(nat):
            for R in cells:
                d = np.linalg.norm(positions[J] + np.asarray(R, float) @ latvec - positions[I])
                amp = sigma * math.exp(-d / decay_bohr)
                Cs[(I, J, R)] = amp * rng.standard_normal((nao[I] * nao[J], nabf[I]))
    return Cs


def _vq(rng, nabf, nk, partner):
    n = int(sum(nabf))
    off = np.concatenate([[0], np.cumsum(nabf)]).astype(int)
    Vq = {}
    full = {}
    for k in range(nk):
        p = partner[k]
        if p in full:
            full[k] = full[p].conj()
            continue
        a = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / math.sqrt(n)
        v = a @ a.conj().T + 0.1 * np.eye(n)
        if p == k:
            v = v.real + 0j
        full[k] = v
    for k, v in full.items():
        for I in range(len(nabf)):
            for J in range(I, len(nabf)):
                Vq[(k, I, J)] = v[off[I]:off[I + 1], off[J]:off[J + 1]].copy()
    return Vq


def fcc_cell(a_ang=3.57):
    a = a_ang * ANGSTROM
    lat = 0.5 * a * np.array([[0.0, 1.0, 1.0], [1.0, 0.0, 1.0], [1.0, 1.0, 0.0]])
    pos = np.array([[0.0, 0.0, 0.0], [0.25 * a, 0.25 * a, 0.25 * a]])
    return lat, pos


def make_periodic(name, lat, pos, period, nao_at, nabf_at, nb, nocc, seed,
                  decay_ang=2.0, sigma_c=0.02, nfreq=16):
    rng = np.random.default_rng(seed)
    nat = len(pos)
    nao_t = int(sum(nao_at))
    kv, fr = _kmesh(period, lat)
    nk = len(kv)
    partner = _partner(fr, period)
    wg, ekb, wfc, ef = _mean_field(rng, nk, nb, nao_t, nocc, partner)
    cells = _r_grid(period)
    Cs = _cs(rng, pos, lat, cells, nao_at, nabf_at, decay_ang * ANGSTROM, sigma_c)
    Vq = _vq(rng, nabf_at, nk, partner)
    return SynthSystem(name=name, n_spins=1, n_kpts=nk, n_bands=nb, n_ao=nao_t, period=tuple(period),
                       latvec=lat, kvecs=kv, ibz_map=np.arange(nk), positions=pos,
                       types=np.zeros(nat, int), nao=list(nao_at), nabf=list(nabf_at),
                       wg=wg, ekb=ekb, efermi=ef, wfc=wfc, Cs=Cs, Vq=Vq, nfreq=nfreq,
                       minimax_emin=_window(nfreq)[0], minimax_emax=_window(nfreq)[1])


def fcc2_k222(seed=1234, **kw):
    lat, pos = fcc_cell()
    return make_periodic("fcc2_k222", lat, pos, (2, 2, 2), [13] * 2, [40] * 2, 26, 4, seed, **kw)


def fcc16_k333(seed=4321, **kw):
    lat, pos = fcc_cell()
    sup = 2.0 * lat
    ps = []
    for n1 in range(2):
        for n2 in range(2):
            for n3 in range(2):
                shift = n1 * lat[0] + n2 * lat[1] + n3 * lat[2]
                ps.extend(pos + shift)
    ps = np.array(ps)
    return make_periodic("fcc16_k333", sup, ps, (3, 3, 3), [13] * 16, [40] * 16, 104, 16, seed, **kw)


def small_periodic(n_atoms=2, nao=5, nabf=12, period=(2, 1, 1), nb=None, nocc=2, seed=7, **kw):
    """Tiny cell for fast parity tests (any period, uneven blocks allowed via lists)."""
    lat, pos0 = fcc_cell()
    rng = np.random.default_rng(seed + 99)
    pos = pos0[:1] + rng.uniform(0, 3.0, (n_atoms, 3))
    nao_at = nao if isinstance(nao, (list, tuple)) else [nao] * n_atoms
    nabf_at = nabf if isinstance(nabf, (list, tuple)) else [nabf] * n_atoms
    nb = nb or int(sum(nao_at))
    return make_periodic("small", lat, pos, period, nao_at, nabf_at, nb, nocc, seed, **kw)


def cluster_gamma(name, n_atoms, species, seed, spacing_ang=2.5, decay_ang=2.0, sigma_c=0.02, nfreq=16):
    """Gamma-only cell: atoms on a simple-cubic packing, random species (nao, nabf) choices."""
    rng = np.random.default_rng(seed)
    side = int(math.ceil(n_atoms ** (1.0 / 3.0)))
    pos = []
    for i in range(side):
        for j in range(side):
            for k in range(side):
                if len(pos) < n_atoms:
                    pos.append([i, j, k])
    pos = np.array(pos, float) * spacing_ang * ANGSTROM
    box = (side * spacing_ang + 20.0) * ANGSTROM
    lat = np.eye(3) * box
    types = rng.integers(0, len(species), n_atoms)
    nao_at = [species[t][0] for t in types]
    nabf_at = [species[t][1] for t in types]
    nao_t = int(sum(nao_at))
    nb = nao_t
    nocc = max(1, nao_t // 4)
    kv = np.zeros((1, 3))
    wg, ekb, wfc, ef = _mean_field(rng, 1, nb, nao_t, nocc, np.array([0]))
    Cs = _cs(rng, pos, lat, [(0, 0, 0)], nao_at, nabf_at, decay_ang * ANGSTROM, sigma_c)
    Vq = _vq(rng, nabf_at, 1, np.array([0]))
    return SynthSystem(name=name, n_spins=1, n_kpts=1, n_bands=nb, n_ao=nao_t, period=(1, 1, 1),
                       latvec=lat, kvecs=kv, ibz_map=np.zeros(1, int), positions=pos, types=types,
                       nao=nao_at, nabf=nabf_at, wg=wg, ekb=ekb, efermi=ef, wfc=wfc, Cs=Cs, Vq=Vq,
                       nfreq=nfreq, minimax_emin=_window(nfreq)[0], minimax_emax=_window(nfreq)[1])


def mixed64_g(seed=64):
    return cluster_gamma("mixed64_g", 64, [(5, 20), (13, 60), (26, 110)], seed, nfreq=24)


def batch32_small(seed=32):
    """32 independent Gamma-only cells of 2-8 atoms of random species, each its own system."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(2, 9, 32)
    return [cluster_gamma(f"batch32_small_{i}", int(n), [(5, 20), (13, 60), (26, 110)], seed * 1000 + i, nfreq=24)
            for i, n in enumerate(sizes)]


def sc256_g(seed=256):
    return cluster_gamma("sc256_g", 256, [(13, 40)], seed, decay_ang=1.5, nfreq=16)


# workloads that are a list of independent systems, each evaluated by its own call
BATCHES = {
    "batch32_small": batch32_small,
}

WORKLOADS = {
    "fcc2_k222": fcc2_k222,
    "fcc16_k333": fcc16_k333,
    "mixed64_g": mixed64_g,
    "sc256_g": sc256_g,
}


def to_oracle_input(s: SynthSystem):
    """Convert to the oracle's input record (test-side helper)."""
    from oracle.rpa_oracle import RPAInput  # noqa: local import, tests only
    return RPAInput(n_spins=s.n_spins, n_kpts=s.n_kpts, n_bands=s.n_bands, n_ao=s.n_ao, wg=s.wg,
                    ekb=s.ekb, efermi=s.efermi, wfc=s.wfc, latvec=s.latvec, period=s.period,
                    kvecs=s.kvecs, ibz_map=s.ibz_map, nao=s.nao, nabf=s.nabf, Cs=s.Cs, Vq=s.Vq,
                    positions=s.positions)


def with_cells_relabelled(s, split: bool = False):
    """The same system with every C block's cell vector given in [0, n) (the Born-von Karman
    range FHI-aims writes) instead of the centred range; split=True also spreads each block over
    two images one period apart (halves that LibRI's folding sums back)."""
    import copy

    t = copy.copy(s)
    per = tuple(s.period)
    cs = {}
    for (I, J, R), m in s.Cs.items():
        r0 = tuple(int(R[d]) % per[d] for d in range(3))
        if not split:
            cs[(I, J, r0)] = m
            continue
        r1 = (r0[0] + per[0], r0[1], r0[2])
        cs[(I, J, r0)] = m * 0.5
        cs[(I, J, r1)] = m - m * 0.5
    t.Cs = cs
    return t
