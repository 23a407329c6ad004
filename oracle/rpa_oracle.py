"""Oracle (test infrastructure only): space-time RPA correlation energy in numpy FP64.

This is a CPU restatement of LibRPA's ``task=rpa`` hot path with the LibRI
routing.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline
leg may import it, and only as the checker; the product never calls it.

Reference functions followed (paths inside the LibRPA project):

* occupations scaled by 1/n_k ............ src/api/input.cpp:62-99 (line 82)
* E_min / E_max (gap, band width) ........ src/core/meanfield.cpp:151-197
* grid options (minimax_emin/emax) ....... src/api/dataset_helper.cpp:11-30
* BvK cell list, centred ................. src/core/pbc.cpp:178-190
* k fractional coordinates, -0 clean ..... src/core/pbc.cpp:79-108
* IBZ list and weights ................... src/core/pbc.cpp:110-153
* G(R, +-tau) builder (LibRI serial) ..... src/core/chi0.cpp:303-426
    weights w+ = max(0, 1/nk - f*ns/2), w- = f*ns/2, exp(min(0,-tau(e-ef))),
    kphase exp(-i 2pi kfrac.R), sign -1 for tau<0, Re() per atom block
* chi0s = two cal_loop3 passes ........... thirdparty/LibRI/include/RI/physics/RPA.hpp:104-137
    labels a1b1_a2b2 / a1b2_a2b1 ......... thirdparty/LibRI/include/RI/ri/LRI-cal_loop3.hpp:902-1032
    periodic keys (Rb-Ra) % period ....... thirdparty/LibRI/include/RI/ri/LRI_Cal_Tools.h:44-60
    centred modulo [-n/2, (n-1)/2] ....... thirdparty/LibRI/include/RI/global/Array_Operator.hpp:15-24
* FT + CT into chi0(q, omega) ............ src/core/chi0.cpp:507-596 (prefactor 2/n_s at :592)
* E_c, k-points (complex, BLACS form) .... src/core/epsilon.cpp:270-558, log(+-u_ii) at :600-693
* E_c, Gamma only (real parts) .......... src/core/epsilon.cpp:43-268, :560-598
* upper atom blocks -> full Hermitian .... src/math/utils_matrix_m_mpi.h:393-455
* ABF shrink U chi0 U^H (use_shrink_abfs)  src/core/chi0.cpp:711-898, applied at :1110-1137
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass, field, replace

import numpy as np
import scipy.linalg

from .minimax import minimax_grid

TWO_PI = 2.0 * math.pi


@dataclass
class RPAInput:
    """Mean-field + RI input exactly as the librpa_set_* calls receive it."""

    n_spins: int
    n_kpts: int
    n_bands: int
    n_ao: int
    wg: np.ndarray            # (n_spins, n_kpts, n_bands) raw occupations (NOT divided by n_k)
    ekb: np.ndarray           # (n_spins, n_kpts, n_bands) Hartree
    efermi: float
    wfc: np.ndarray           # (n_spins, n_kpts, n_bands, n_ao) complex, band-major
    latvec: np.ndarray        # (3,3), rows a1, a2, a3 in Bohr (librpa_set_latvec_and_G order)
    period: tuple             # (nk1, nk2, nk3)
    kvecs: np.ndarray         # (n_kpts, 3) Cartesian, Bohr^-1 (with 2 pi)
    ibz_map: np.ndarray       # (n_kpts,) int, full k -> ibz representative (full index)
    nao: list                 # NAOs per atom
    nabf: list                # ABFs per atom
    Cs: dict                  # (I, J, (R1,R2,R3)) -> (n_i*n_j, n_mu) row-major
    Vq: dict                  # (ik_full, I, J) with I <= J -> complex (n_mu, n_nu)
    positions: np.ndarray | None = None  # (n_atoms, 3) Cartesian Bohr (screening features only)
    # ABF shrink (use_shrink_abfs): small ABFs per atom (the basis of Vq then) and U(q) per IBZ q
    nabf_small: list | None = None
    sinvS: dict | None = None             # iq_ibz -> (sum nabf_small, sum nabf) complex
    Cs_small: dict | None = None          # RI blocks of the small basis (exchange of a shrunk input)

    @property
    def n_atoms(self):
        return len(self.nao)


@dataclass
class Options:
    nfreq: int = 16
    minimax_emin: float = -1.0
    minimax_emax: float = -1.0
    minimax_regulation: float = 0.0
    n_bands_chi0: int = -1
    vq_threshold: float = 0.0
    libri_chi0_threshold_C: float = 0.0
    libri_chi0_threshold_G: float = 0.0
    use_shrink_abfs: bool = False


# ----------------------------------------------------------------------------- helpers

def centred_mod(v, n):
    """LibRI Array_Operator operator% : (i % n + 3n/2) % n - n/2 with C integer semantics."""
    out = []
    for i, p in zip(v, n):
        r = int(math.fmod(i, p))           # C '%' truncates toward zero
        r = (r + (3 * p) // 2) % p          # operand is non-negative here
        out.append(r - p // 2)
    return tuple(out)


def r_grid(period):
    """construct_R_grid (pbc.cpp:178-190): x outer, z inner."""
    return [(x, y, z)
            for x in range(-(period[0] // 2), (period[0] - 1) // 2 + 1)
            for y in range(-(period[1] // 2), (period[1] - 1) // 2 + 1)
            for z in range(-(period[2] // 2), (period[2] - 1) // 2 + 1)]


def k_lists(inp: RPAInput):
    klist = inp.kvecs / TWO_PI                              # Cartesian / 2pi
    kfrac = klist @ inp.latvec.T                            # latvec * kvec
    kfrac = np.where(np.abs(kfrac) < 1e-8, 0.0, kfrac)
    ibz_order, weight = [], {}
    for ik in range(inp.n_kpts):
        r = int(inp.ibz_map[ik])
        if r not in weight:
            ibz_order.append(r)
            weight[r] = 0.0
        weight[r] += 1.0 / inp.n_kpts
    return klist, kfrac, ibz_order, [weight[r] for r in ibz_order]


def e_min_max(inp: RPAInput):
    """MeanField::get_E_min_max + get_band_gap, fed with wg/nk as the setter stores it."""
    wg = inp.wg / inp.n_kpts
    lb, ub = np.inf, np.finfo(float).tiny
    homo, lumo = -1e6, 1e6
    for s in range(inp.n_spins):
        for k in range(inp.n_kpts):
            lb = min(lb, inp.ekb[s, k, 0])
            ub = max(ub, inp.ekb[s, k, -1])
        midpoint = 1.0 / (inp.n_spins * inp.n_kpts * 1)
        for k in range(inp.n_kpts):
            hl = -1
            for n in range(inp.n_bands):
                if wg[s, k, n] >= midpoint:
                    hl = n
            lumo = min(lumo, inp.ekb[s, k, hl + 1])
            if hl != -1:
                homo = max(homo, inp.ekb[s, k, hl])
    return lumo - homo, ub - lb


def grids_for(inp: RPAInput, opts: Options):
    emin_mf, emax_mf = e_min_max(inp)
    emax = opts.minimax_emax if opts.minimax_emax > 0 else emax_mf
    emin = opts.minimax_emin if opts.minimax_emin > 0 else emin_mf
    return minimax_grid(opts.nfreq, emin, emax, opts.minimax_regulation)


# ----------------------------------------------------------------------------- G(R, tau)

def tau_scale(inp: RPAInput, ispin: int, tau: float, nbands_g: int = -1):
    """Per (k, band) factor exp(min(0, -tau (e - ef))) * w(+-) (chi0.cpp:348-365)."""
    wg = inp.wg[ispin] / inp.n_kpts
    if tau > 0:
        w = 1.0 / inp.n_kpts - wg / 2.0 * inp.n_spins
        w = np.where(w < 0, 0.0, w)
    else:
        w = wg * (0.5 * inp.n_spins)
    sc = -tau * (inp.ekb[ispin] - inp.efermi)
    sc = np.where(sc > 0, 0.0, sc)
    s = np.exp(sc) * w
    if nbands_g >= 0:
        s = s.copy()
        s[:, nbands_g:] = 0.0
    return s


def build_gf(inp: RPAInput, ispin: int, tau: float, kfrac, rlist, nbands_g: int = -1):
    """G(R, tau) full n_ao x n_ao real matrices per R (chi0.cpp:303-426)."""
    s = tau_scale(inp, ispin, tau, nbands_g)
    out = {}
    mats = []
    for ik in range(inp.n_kpts):
        ev = inp.wfc[ispin, ik]                  # (nb, nao)
        mats.append(ev.T @ (s[ik][:, None] * ev.conj()))
    for R in rlist:
        acc = np.zeros((inp.n_ao, inp.n_ao), complex)
        for ik in range(inp.n_kpts):
            ang = -float(np.dot(kfrac[ik], R)) * TWO_PI
            acc += complex(math.cos(ang), math.sin(ang)) * mats[ik]
        if tau < 0:
            acc = -acc
        out[R] = acc.real.copy()
    return out


def blocks_of(full: dict, nao):
    """Cut full G(R) into atom blocks G[(I, J, R)] (n_I x n_J row-major)."""
    off = np.concatenate([[0], np.cumsum(nao)])
    res = {}
    for R, m in full.items():
        for I in range(len(nao)):
            for J in range(len(nao)):
                res[(I, J, R)] = m[off[I]:off[I + 1], off[J]:off[J + 1]]
    return res


# ----------------------------------------------------------------------------- chi0 (LibRI algebra)

def cs_tensors(inp: RPAInput, threshold: float = 0.0):
    """LibRI form C[I][(J,R)] with shape (n_mu, n_i, n_j) (input.cpp:525-541).

    As LibRI's set_tensors does (RI_Tools::cal_period, LRI-set.hpp:47-52 and RI_Tools.hpp:49-67),
    the cell vector is first taken modulo the BvK period into the centred range, blocks that land
    on the same key are summed, and only then the threshold filter applies."""
    summed = {}
    for (I, J, R), m in inp.Cs.items():
        ni, nj = inp.nao[I], inp.nao[J]
        t = m.T.reshape(m.shape[1], ni, nj)
        key = (I, J, centred_mod(tuple(R), inp.period))
        summed[key] = summed[key] + t if key in summed else t
    out = {}
    for key, t in summed.items():
        if threshold > 0 and np.abs(t).max() <= threshold:  # kept when max-norm > threshold (LRI.hpp:20-25)
            continue
        out[key] = t
    return out


def _filter_g(G: dict, threshold: float):
    """LibRI's set_Gs_pos / set_Gs_neg filter (LRI-set.hpp:56-61): keep blocks with max |G| > threshold."""
    if threshold <= 0:
        return G
    return {k: v for k, v in G.items() if np.abs(v).max() > threshold}


def screen_blocks(chi0s: dict, threshold: float):
    """The same max-norm rule applied to chi0(I, J, R, tau) blocks: keep max |chi0| > threshold.

    Plain block screening of the GPU library (LibrpaGB300Options.screen_threshold); the
    reference applies this rule to its input tensors only."""
    return {k: v for k, v in chi0s.items() if np.abs(v).max() > threshold}


def cal_chi0s_loops(C: dict, Gpos: dict, Gneg: dict, n_atoms: int, period, acc: dict | None = None):
    """Literal restatement of RPA::cal_chi0s = two LRI::cal_loop3 passes.

    Loop nest and contraction order follow LRI-cal_loop3.hpp:902-1032.  Keys are
    (atom, cell) with cells in the centred BvK range; tensors missing from a map
    are skipped exactly like ``if (D.empty()) continue``.
    """
    cells = r_grid(period)
    sites = [(A, c) for A in range(n_atoms) for c in cells]
    acc = {} if acc is None else acc

    def sub(b, a):
        return centred_mod((b[0] - a[0], b[1] - a[1], b[2] - a[2]), period)

    def add(key, val):
        if key in acc:
            acc[key] = acc[key] + val
        else:
            acc[key] = val.copy()

    for Ga, Gb in ((Gpos, Gneg), (Gneg, Gpos)):
        # label a1b1_a2b2 : D_mul = sum_Aa2 a2b2 * a0a1a2 ; D_result = D_mul * a1b1 * b
        for I in range(n_atoms):
            for (L, RL) in sites:
                D_mul = None
                for (K, RK) in sites:
                    Da = C.get((I, K, RK))
                    if Da is None:
                        continue
                    Da2b2 = Gb.get((K, L, sub(RL, RK)))
                    if Da2b2 is None:
                        continue
                    # b2a0a1[l, mu, i] = sum_k a2b2[k, l] * a0a1a2[mu, i, k]
                    t = np.einsum("kl,mik->lmi", Da2b2, Da)
                    D_mul = t if D_mul is None else D_mul + t
                if D_mul is None:
                    continue
                for (J, RJ) in sites:
                    Db = C.get((J, L, sub(RL, RJ)))
                    if Db is None:
                        continue
                    Da1b1 = Ga.get((I, J, RJ))
                    if Da1b1 is None:
                        continue
                    # b1b2a0[j, l, mu] = sum_i a1b1[i, j] * D_mul[l, mu, i]
                    t2 = np.einsum("ij,lmi->jlm", Da1b1, D_mul)
                    # a0b0[mu, nu] = sum_{j,l} t2[j, l, mu] * b0b1b2[nu, j, l]
                    add((I, J, RJ), np.einsum("jlm,njl->mn", t2, Db))
        # label a1b2_a2b1 : D_mul1 = b * a1b2 ; D_mul2 = a2b1 * a ; D_result = D_mul2 * D_mul1
        for I in range(n_atoms):
            for (J, RJ) in sites:
                D_mul1 = None
                for (L, RL) in sites:
                    Db = C.get((J, L, sub(RL, RJ)))
                    if Db is None:
                        continue
                    Da1b2 = Ga.get((I, L, RL))
                    if Da1b2 is None:
                        continue
                    # b0b1a1[nu, j, i] = sum_l b0b1b2[nu, j, l] * a1b2[i, l]
                    t = np.einsum("njl,il->nji", Db, Da1b2)
                    D_mul1 = t if D_mul1 is None else D_mul1 + t
                if D_mul1 is None:
                    continue
                D_mul2 = None
                for (K, RK) in sites:
                    Da = C.get((I, K, RK))
                    if Da is None:
                        continue
                    Da2b1 = Gb.get((K, J, sub(RJ, RK)))
                    if Da2b1 is None:
                        continue
                    # b1a1a0[j, i, mu] = sum_k a2b1[k, j] * a1a0a2[i, mu, k]
                    t = np.einsum("kj,mik->jim", Da2b1, Da)
                    D_mul2 = t if D_mul2 is None else D_mul2 + t
                if D_mul2 is None:
                    continue
                # a0b0[mu, nu] = sum_{j,i} D_mul2[j, i, mu] * D_mul1[nu, j, i]
                add((I, J, RJ), np.einsum("jim,nji->mn", D_mul2, D_mul1))
    return acc


def cal_chi0s_dense(C: dict, Gpos: dict, Gneg: dict, nao, nabf, period, rows=None, cols=None, timings=None):
    """The same chi0s as cal_chi0s_loops, evaluated with supercell matrices.

    Faster reformulation used at sizes where the literal loops are too slow; it
    is checked against ``cal_chi0s_loops`` in the tests.  With
    X_b^I[mu i; (L,RL) l] = sum_{(K,RK),k} C^I[mu,i,(K,RK) k] Gb[K;L,RL-RK]_{kl}:
      T1 = sum Ga[I;J,RJ]_{ij} X_b^I[mu i;(L,RL) l] C^J[nu,j,(L,RL-RJ) l]
      T2 = sum X_b^I[mu i;(J,RJ) j] X_a^J[nu j;(I,-RJ) i]
    which uses the symmetry Re G[I;L,R]_{il} = Re G[L;I,-R]_{li} of the G builder.
    """
    n_at = len(nao)
    cells = r_grid(period)
    nc = len(cells)
    cidx = {c: i for i, c in enumerate(cells)}
    aoff = np.concatenate([[0], np.cumsum(nao)]).astype(int)
    nao_t = int(aoff[-1])
    nsup = nc * nao_t

    def sub(b, a):
        return centred_mod((b[0] - a[0], b[1] - a[1], b[2] - a[2]), period)

    def gsuper(G):
        S = np.zeros((nsup, nsup))
        for ck, RK in enumerate(cells):
            for cl, RL in enumerate(cells):
                d = sub(RL, RK)
                for K in range(n_at):
                    for L in range(n_at):
                        g = G.get((K, L, d))
                        if g is None:
                            continue
                        S[ck * nao_t + aoff[K]: ck * nao_t + aoff[K + 1],
                          cl * nao_t + aoff[L]: cl * nao_t + aoff[L + 1]] = g
        return S

    def crow(I):
        """C^I as matrix [(mu,i), (cell,K,k)]."""
        M = np.zeros((nabf[I] * nao[I], nsup))
        for c, R in enumerate(cells):
            for K in range(n_at):
                t = C.get((I, K, R))
                if t is None:
                    continue
                M[:, c * nao_t + aoff[K]: c * nao_t + aoff[K + 1]] = t.reshape(nabf[I] * nao[I], nao[K])
        return M

    Gsp, Gsn = gsuper(Gpos), gsuper(Gneg)
    rows = list(range(n_at)) if rows is None else list(rows)
    cols = list(range(n_at)) if cols is None else list(cols)
    need = set(rows) | set(cols)  # X^J of every output column atom enters T2
    import time as _time
    _t0 = _time.perf_counter()
    Cm = {I: crow(I) for I in need}
    X = {"+": {I: Cm[I] @ Gsp for I in need}, "-": {I: Cm[I] @ Gsn for I in need}}
    if timings is not None:
        timings["x_per_atom"] = (_time.perf_counter() - _t0) / len(need)
        _t0 = _time.perf_counter()
    # column permutation taking (cL, L, l) -> (cell(RL - RJ), L, l) for each RJ
    perm = {}
    colcell = np.repeat(np.arange(nc), nao_t)
    colao = np.tile(np.arange(nao_t), nc)
    for RJ in cells:
        cj = cidx[RJ]
        dc = np.array([cidx[sub(cells[c], RJ)] for c in range(nc)])
        perm[RJ] = dc[colcell] * nao_t + colao
    out = {}
    for I in rows:
        for J in cols:
            CmJ = Cm[J]
            for RJ in cells:
                acc = np.zeros((nabf[I], nabf[J]))
                CJs = CmJ[:, perm[RJ]].reshape(nabf[J], nao[J] * nsup)  # [nu, (j, K)]
                cj = cidx[RJ]
                cmi = cidx[centred_mod((-RJ[0], -RJ[1], -RJ[2]), period)]
                for a, b in (("+", "-"), ("-", "+")):
                    Ga = Gpos if a == "+" else Gneg
                    g = Ga.get((I, J, RJ))
                    XbI = X[b][I].reshape(nabf[I], nao[I], nsup)
                    if g is not None:
                        # E[mu, j, K] = sum_i g[i,j] XbI[mu,i,K];  T1 = E[mu,(j,K)] CJs[nu,(j,K)]^T
                        E = np.einsum("ij,miK->mjK", g, XbI, optimize=True).reshape(nabf[I], nao[J] * nsup)
                        acc += E @ CJs.T
                    XaJ = X[a][J].reshape(nabf[J], nao[J], nsup)
                    x1 = XbI[:, :, cj * nao_t + aoff[J]: cj * nao_t + aoff[J + 1]]     # [mu,i,j]
                    x2 = XaJ[:, :, cmi * nao_t + aoff[I]: cmi * nao_t + aoff[I + 1]]   # [nu,j,i]
                    acc += x1.reshape(nabf[I], -1) @ x2.transpose(0, 2, 1).reshape(nabf[J], -1).T
                out[(I, J, RJ)] = acc
    if timings is not None:
        timings["blocks_per_pair"] = (_time.perf_counter() - _t0) / (len(rows) * len(cols))
    return out


# ----------------------------------------------------------------------------- FT + CT

def upper_pairs(n_atoms):
    return [(I, J) for I in range(n_atoms) for J in range(I, n_atoms)]


def ft_ct_accumulate(chi0q, chi0s: dict, it: int, grid, klist_ibz, latvec, n_spins, pairs):
    """chi_libri_ft_ct (chi0.cpp:507-596): chi0q[iw][iq][(I,J)] += 2/ns * gamma * e^{i2pi q.R} chi0(R)."""
    nfreq = len(grid["omega"])
    for iw in range(nfreq):
        trans = grid["cos_t2f"][iw, it]
        for iq, q in enumerate(klist_ibz):
            for (Mu, Nu) in pairs:
                tgt = chi0q[iw][iq][(Mu, Nu)]
                for (I, J, R), chi in chi0s.items():
                    if I != Mu or J != Nu:
                        continue
                    arg = float(np.dot(q, np.asarray(R, float) @ latvec)) * TWO_PI
                    tgt += (2.0 / n_spins) * (trans * complex(math.cos(arg), math.sin(arg))) * chi


# ----------------------------------------------------------------------------- E_c

def assemble_full(blocks: dict, nb, conj=True, dtype=complex):
    off = np.concatenate([[0], np.cumsum(nb)]).astype(int)
    n = int(off[-1])
    M = np.zeros((n, n), dtype)
    na = len(nb)
    for I in range(na):
        for J in range(I, na):
            b = blocks.get((I, J))
            if b is None:
                continue
            M[off[I]:off[I + 1], off[J]:off[J + 1]] = b
            if J > I:
                M[off[J]:off[J + 1], off[I]:off[I + 1]] = (b.conj().T if conj else b.T)
    return M


def shrink_chi0q(chi0q, sinvS: dict, nabf_large, nabf_small):
    """shrink_abfs_chi0 (chi0.cpp:711-898) for every (omega, IBZ q): the full chi0(q) of the large
    ABF basis from its upper atom-pair blocks (Hermitian fill, collect_block_from_ALL_IJ_Tensor),
    chi0_s = U(q) chi0 U(q)^H (the two pgemm calls, :829-836), and chi0_s's upper atom-pair blocks
    in the small basis (map_block_to_IJ_storage_new).  The reference applies it to chi0(q, tau)
    ahead of the cosine transform (:1110-1137); both steps are linear, so applying it to
    chi0(q, omega) gives the same chi0_s(q, omega)."""
    offs = np.concatenate([[0], np.cumsum(nabf_small)]).astype(int)
    na = len(nabf_small)
    out = []
    for row in chi0q:
        orow = []
        for iq, blocks in enumerate(row):
            U = sinvS[iq]
            X = U @ assemble_full(blocks, nabf_large) @ U.conj().T
            orow.append({(I, J): X[offs[I]:offs[I + 1], offs[J]:offs[J + 1]].copy()
                         for I in range(na) for J in range(I, na)})
        out.append(orow)
    return out


def ln_det_pm(M):
    """LU (partial pivot) then sum log(+-u_ii), sign by Re(u_ii) > 0 (epsilon.cpp:578-592, :640-671)."""
    lu, _piv = scipy.linalg.lu_factor(M, check_finite=False)
    d = np.diag(lu)
    if np.iscomplexobj(d):
        return complex(np.sum(np.log(np.where(d.real > 0, d, -d))))
    return float(np.sum(np.log(np.where(d > 0, d, -d))))


def correlation_energy(chi0q, inp: RPAInput, grid, ibz_order, ibz_weight, opts: Options):
    """Returns (E_c complex, per-IBZ-q complex contributions, per (w,q) terms)."""
    nb = inp.nabf
    tot = 0.0 + 0.0j
    per_q = []
    terms = {}
    gamma_only = inp.n_kpts == 1
    for iq, ikf in enumerate(ibz_order):
        vblocks = {}
        for (I, J) in upper_pairs(inp.n_atoms):
            v = inp.Vq.get((ikf, I, J))
            if v is None:
                continue
            if np.abs(v.real).max() < opts.vq_threshold:
                continue
            vblocks[(I, J)] = v
        cq = 0.0 + 0.0j
        for iw in range(len(grid["omega"])):
            if gamma_only:
                V = assemble_full({k: v.real for k, v in vblocks.items()}, nb, dtype=float)
                X = assemble_full({k: v.real for k, v in chi0q[iw][iq].items()}, nb, dtype=float)
            else:
                V = assemble_full(vblocks, nb)
                X = assemble_full(chi0q[iw][iq], nb)
            P = V @ X
            tr = np.trace(P)
            ld = ln_det_pm(np.eye(P.shape[0]) - P)
            val = complex(tr + ld) * grid["omega_w"][iw] * ibz_weight[iq] / TWO_PI
            terms[(iw, iq)] = (complex(tr), complex(ld))
            cq += val
        per_q.append(cq)
        tot += cq
    return tot, per_q, terms


# ----------------------------------------------------------------------------- driver

def chi0q_partial(inp: RPAInput, opts: Options, tau_begin: int, tau_end: int):
    """chi0(q, omega) summed over the minimax tau points [tau_begin, tau_end) only (a tau shard)."""
    grid = grids_for(inp, opts)
    klist, kfrac, ibz_order, ibz_weight = k_lists(inp)
    rlist = r_grid(inp.period)
    klist_ibz = [klist[i] for i in ibz_order]
    pairs = upper_pairs(inp.n_atoms)
    C = cs_tensors(inp, opts.libri_chi0_threshold_C)
    chi0q = [[{p: np.zeros((inp.nabf[p[0]], inp.nabf[p[1]]), complex) for p in pairs}
              for _ in ibz_order] for _ in range(opts.nfreq)]
    for it in range(tau_begin, tau_end):
        tau = grid["tau"][it]
        for s in range(inp.n_spins):
            Gp = blocks_of(build_gf(inp, s, tau, kfrac, rlist, opts.n_bands_chi0), inp.nao)
            Gn = blocks_of(build_gf(inp, s, -tau, kfrac, rlist, opts.n_bands_chi0), inp.nao)
            chi0s = cal_chi0s_dense(C, Gp, Gn, inp.nao, inp.nabf, inp.period)
            ft_ct_accumulate(chi0q, chi0s, it, grid, klist_ibz, inp.latvec, inp.n_spins, pairs)
    return chi0q


def ec_from_chi0q(inp: RPAInput, opts: Options, chi0q):
    """E_c (correlation_energy) from a given chi0(q, omega)."""
    grid = grids_for(inp, opts)
    _, _, ibz_order, ibz_weight = k_lists(inp)
    return correlation_energy(chi0q, inp, grid, ibz_order, ibz_weight, opts)


def rpa_correlation_energy(inp: RPAInput, opts: Options | None = None, chi0_impl: str = "dense",
                           keep_chi0s: bool = False, block_threshold: float | None = None):
    """Full oracle pipeline; returns a dict with E_c and intermediates."""
    opts = opts or Options()
    grid = grids_for(inp, opts)
    klist, kfrac, ibz_order, ibz_weight = k_lists(inp)
    rlist = r_grid(inp.period)
    klist_ibz = [klist[i] for i in ibz_order]
    pairs = upper_pairs(inp.n_atoms)
    C = cs_tensors(inp, opts.libri_chi0_threshold_C)
    chi0q = [[{p: np.zeros((inp.nabf[p[0]], inp.nabf[p[1]]), complex) for p in pairs}
              for _ in ibz_order] for _ in range(opts.nfreq)]
    chi0s_all = []
    for it, tau in enumerate(grid["tau"]):
        for s in range(inp.n_spins):
            Gp = _filter_g(blocks_of(build_gf(inp, s, tau, kfrac, rlist, opts.n_bands_chi0), inp.nao),
                           opts.libri_chi0_threshold_G)
            Gn = _filter_g(blocks_of(build_gf(inp, s, -tau, kfrac, rlist, opts.n_bands_chi0), inp.nao),
                           opts.libri_chi0_threshold_G)
            if chi0_impl == "loops":
                chi0s = cal_chi0s_loops(C, Gp, Gn, inp.n_atoms, inp.period)
            else:
                chi0s = cal_chi0s_dense(C, Gp, Gn, inp.nao, inp.nabf, inp.period)
            if block_threshold is not None:
                chi0s = screen_blocks(chi0s, block_threshold)
            if keep_chi0s:
                chi0s_all.append(chi0s)
            ft_ct_accumulate(chi0q, chi0s, it, grid, klist_ibz, inp.latvec, inp.n_spins, pairs)
    ec_inp, ec_chi0q = inp, chi0q
    if opts.use_shrink_abfs:
        # chi0 of the Cs basis -> the small basis of the Coulomb matrix (chi0.cpp:1110-1137)
        ec_chi0q = shrink_chi0q(chi0q, inp.sinvS, inp.nabf, inp.nabf_small)
        ec_inp = replace(inp, nabf=list(inp.nabf_small))
    ec, per_q, terms = correlation_energy(ec_chi0q, ec_inp, grid, ibz_order, ibz_weight, opts)
    return {"ec": ec, "per_q": per_q, "grid": grid, "chi0q": chi0q, "terms": terms,
            "chi0s": chi0s_all, "ibz_order": ibz_order, "ibz_weight": ibz_weight}
