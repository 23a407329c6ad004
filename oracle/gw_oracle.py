"""Oracle (test infrastructure only): exact exchange on k-grids and G0W0 quasi-particle
energies at the Gamma point.

CPU FP64 restatement of LibRPA's EXX (task = exx, any k-grid: exx_kgrid) and G0W0 chain
(task = g0w0, Gamma-only inputs: molecules and Gamma-point cells; g0w0_gamma), built on the RPA
oracle's chi0(q, omega):

  exchange  H(R) = LibRI Exx::cal_Hs, labels a0b0_{a1b1,a1b2,a2b1,a2b2}
                   (thirdparty/LibRI/include/RI/physics/Exx.hpp:242-283) with
                   D(R) = MeanField::get_dmat_cplx_R (src/core/meanfield.cpp:201-244) and
                   V(R) = FT_Vq of the truncated Coulomb (src/core/coulmat.cpp:7-90);
                   v_exx_n = -<psi_n|H(k)|psi_n> (src/core/exx.cpp:820-860)
  W_c       Wc(omega) = Vcut^1/2 [(1 - V^1/2 chi0 V^1/2)^-1 - 1] Vcut^1/2, square roots by
                   eigen-decomposition with eigenvalues below the threshold dropped
                   (src/core/epsilon.cpp:1763-2322, default branch without head correction;
                   power_hemat_blacs src/math/utils_matrix_m_mpi.h:597-720)
            Wc(tau) = sum_omega costrans_f2t(tau, omega) Wc(omega)
                   (CT_FT_Wc_freq_q, src/core/epsilon.cpp:2490-2660; one k-point: no q sum)
  Sigma_c   Sigma(+-tau) = LibRI GW::cal_Sigmas with the same four labels
                   (thirdparty/LibRI/include/RI/physics/GW.hpp:102-125), G(+-tau) of
                   src/core/meanfield.cpp:270-307;
            Sigma(i omega) = sum_tau [cos_t2f 1/2 (S+ + S-) + i sin_t2f 1/2 (S+ - S-)]
                   (src/core/gw.cpp:627-700); KS diagonal <psi_n|Sigma|psi_n> (gw.cpp:1100-1140)
  continuation  Thiele reciprocal differences (AnalyContPade, src/core/analycont.cpp:12-70)
  QP equation   damped fixed point (qpe_solver_pade_self_consistent, src/core/qpe_solver.cpp)

g0w0_kgrid extends the chain to k-grids: W_c at the IBZ q-points (with the head of the
dielectric matrix replaced by eps_mac at Gamma when asked), the q -> R transform with the
time-reversed partners (FT_Wc_freq_q, epsilon.cpp:2323-2488), Sigma_c(R) shifted to the nearest
BvK image and summed into Sigma_c(k) (gw.cpp:1010-1140).  A shrunk input (inp.sinvS) forms chi0
and W_c in the small ABF basis and unfolds W_c as U^H W_c U for the self-energy
(src/gw_old.cpp:55-280), its exchange on the small basis's RI coefficients; LibRI's block
filters (thr_v / thr_d, thr_w / thr_g) drop the blocks set_Vs / set_Ds / set_Ws / set_Gs drop.

Pinned by the reference's own regression outputs: the H2O molecule (24 states, 16 minimax
points, 16 Pade parameters; tests/golden/h2o_g0w0.npz), the spin-polarised Li atom
(li_g0w0.npz), the periodic BCC He exchange on a 2x2x2 k-grid (he_exx.npz) and the MgO G0W0
run on a 3x3x3 k-grid with 14 IBZ points and the head correction (mgo_g0w0.npz).
"""
from __future__ import annotations

import math
import dataclasses
from dataclasses import dataclass

import numpy as np

from .rpa_oracle import (TWO_PI, Options, RPAInput, assemble_full, blocks_of, build_gf, centred_mod,
                         chi0q_partial, cs_tensors, grids_for, k_lists, r_grid, shrink_chi0q, upper_pairs)

HA2EV = 27.211386245988  # src/utils/constants.cpp:13 (the driver's default "internal" choice)


# ----------------------------------------------------------------------------- LibRI loop3, 4 labels

def cal_hs_loops(C: dict, W: dict, D: dict, n_atoms: int, period):
    """H = LRI::cal_loop3 over labels a0b0_a1b1, a0b0_a1b2, a0b0_a2b1, a0b0_a2b2.

    a = C[(I, K, RK)] (mu on I, i on I, k on K@RK), b = C[(J, L, RL - RJ)] (nu on J@RJ, j, l on
    L@RL), a0b0 = W[(I, J, RJ)].  The label names the two orbital indices that D contracts; the
    other two index the result:
      a2b2: D[k, l] -> H[(I, J)]_{ij}      a1b1: D[i, j] -> H[(K, L)]_{kl}
      a1b2: D[i, l] -> H[(K, J)]_{kj}      a2b1: D[k, j] -> H[(I, L)]_{il}
    Blocks missing from a map are skipped (an empty tensor contributes nothing).
    """
    cells = r_grid(period)
    sites = [(A, c) for A in range(n_atoms) for c in cells]
    H = {}

    def sub(b, a):
        return centred_mod((b[0] - a[0], b[1] - a[1], b[2] - a[2]), period)

    def add(key, val):
        if key in H:
            H[key] = H[key] + val
        else:
            H[key] = val.copy()

    for I in range(n_atoms):
        for (K, RK) in sites:
            Ca = C.get((I, K, RK))
            if Ca is None:
                continue
            for (J, RJ) in sites:
                Wab = W.get((I, J, RJ))
                if Wab is None:
                    continue
                # a W: (nu, i, k) = sum_mu W[mu, nu] Ca[mu, i, k]
                CW = np.einsum("mn,mik->nik", Wab, Ca)
                for (L, RL) in sites:
                    Cb = C.get((J, L, sub(RL, RJ)))
                    if Cb is None:
                        continue
                    # T[i, k, j, l] = sum_nu CW[nu, i, k] Cb[nu, j, l]
                    T = np.einsum("nik,njl->ikjl", CW, Cb)
                    d = D.get((K, L, sub(RL, RK)))
                    if d is not None:
                        add((I, J, RJ), np.einsum("ikjl,kl->ij", T, d))
                    d = D.get((I, J, RJ))
                    if d is not None:
                        add((K, L, sub(RL, RK)), np.einsum("ikjl,ij->kl", T, d))
                    d = D.get((I, L, RL))
                    if d is not None:
                        add((K, J, sub(RJ, RK)), np.einsum("ikjl,il->kj", T, d))
                    d = D.get((K, J, sub(RJ, RK)))
                    if d is not None:
                        add((I, L, RL), np.einsum("ikjl,kj->il", T, d))
    return H


def cal_hs_batched(C: dict, W: dict, D: dict, n_atoms: int, period):
    """cal_hs_loops with the innermost site loop (L, R_L) batched over the cells of each L atom:
    the same sums, in a different order.  For k-grids, where the literal loops are slow."""
    cells = r_grid(period)
    sites = [(A, c) for A in range(n_atoms) for c in cells]
    H = {}

    def sub(b, a):
        return centred_mod((b[0] - a[0], b[1] - a[1], b[2] - a[2]), period)

    def add(key, val):
        if key in H:
            H[key] = H[key] + val
        else:
            H[key] = val.copy()

    for I in range(n_atoms):
        for (K, RK) in sites:
            Ca = C.get((I, K, RK))
            if Ca is None:
                continue
            for (J, RJ) in sites:
                Wab = W.get((I, J, RJ))
                if Wab is None:
                    continue
                CW = np.einsum("mn,mik->nik", Wab, Ca)
                d_ij = D.get((I, J, RJ))
                d_kj = D.get((K, J, sub(RJ, RK)))
                for L in range(n_atoms):
                    RLs = [RL for RL in cells if (J, L, sub(RL, RJ)) in C]
                    if not RLs:
                        continue
                    Cb = np.stack([C[(J, L, sub(RL, RJ))] for RL in RLs])  # (c, nu, j, l)
                    # a2b2: D[k, l] with (K, L@RL); result (I, J@RJ)
                    sel = [c for c, RL in enumerate(RLs) if (K, L, sub(RL, RK)) in D]
                    if sel:
                        Ds = np.stack([D[(K, L, sub(RLs[c], RK))] for c in sel])
                        Y = np.einsum("cnjl,ckl->cnjk", Cb[sel], Ds, optimize=True)
                        add((I, J, RJ), np.einsum("nik,cnjk->ij", CW, Y, optimize=True))
                    # a1b1: D[i, j]; result (K@RK, L@RL)
                    if d_ij is not None:
                        Z = np.einsum("nik,ij->nkj", CW, d_ij, optimize=True)
                        R = np.einsum("nkj,cnjl->ckl", Z, Cb, optimize=True)
                        for c, RL in enumerate(RLs):
                            add((K, L, sub(RL, RK)), R[c])
                    # a1b2: D[i, l] with (I, L@RL); result (K@RK, J@RJ)
                    sel = [c for c, RL in enumerate(RLs) if (I, L, RL) in D]
                    if sel:
                        Ds = np.stack([D[(I, L, RLs[c])] for c in sel])
                        P = np.einsum("nik,cil->cnkl", CW, Ds, optimize=True)
                        add((K, J, sub(RJ, RK)), np.einsum("cnkl,cnjl->kj", P, Cb[sel], optimize=True))
                    # a2b1: D[k, j]; result (I, L@RL)
                    if d_kj is not None:
                        Q = np.einsum("nik,kj->nij", CW, d_kj, optimize=True)
                        R = np.einsum("nij,cnjl->cil", Q, Cb, optimize=True)
                        for c, RL in enumerate(RLs):
                            add((I, L, RL), R[c])
    return H


def cal_hs_cells(C: dict, W: dict, D: dict, nao, nabf, period):
    """The four-label sum of cal_hs_loops vectorised over the BvK cells: for each quadruple of
    atoms (I, J, K, L) the cell sums become batched contractions over cell-indexed arrays
    (absent blocks are zeros, which add nothing).  With u = R_L - R_J (the cell of C^J's second
    atom) and v = R_J - R_K:
      a2b2: H[I,J,R_J]   = sum C[I,K,R_K] W[I,J,R_J] E1[v],  E1[v] = sum_u C[J,L,u] D[K,L,v+u]
      a1b1: H[K,L,v+u]  += sum C[I,K,R_K] W[I,J,R_J] D[I,J,R_J] C[J,L,u]
      a1b2: H[K,J,v]    += sum C[I,K,R_K] W[I,J,R_J] P[R_J],  P[R_J] = sum_u C[J,L,u] D[I,L,R_J+u]
      a2b1: H[I,L,R_J+u] += sum S[R_J] C[J,L,u],  S[R_J] = W[I,J,R_J]^T sum_K C[I,K,R_K] D[K,J,v]
    Returns every (X, Y, R) block, zero blocks included."""
    cells = r_grid(period)
    nc = len(cells)
    cidx = {c: i for i, c in enumerate(cells)}
    add = np.array([[cidx[centred_mod(tuple(a[d] + b[d] for d in range(3)), period)] for b in cells] for a in cells])
    sub = np.array([[cidx[centred_mod(tuple(a[d] - b[d] for d in range(3)), period)] for b in cells] for a in cells])
    na = len(nao)

    def arr(T, A, B, shape):
        out = np.zeros((nc,) + shape)
        for c, R in enumerate(cells):
            t = T.get((A, B, R))
            if t is not None:
                out[c] = t
        return out

    Ca = {(A, B): arr(C, A, B, (nabf[A], nao[A], nao[B])) for A in range(na) for B in range(na)}
    Wa = {(A, B): arr(W, A, B, (nabf[A], nabf[B])) for A in range(na) for B in range(na)}
    Da = {(A, B): arr(D, A, B, (nao[A], nao[B])) for A in range(na) for B in range(na)}
    H = {(A, B): np.zeros((nc, nao[A], nao[B])) for A in range(na) for B in range(na)}
    RJ, RK = np.meshgrid(np.arange(nc), np.arange(nc), indexing="ij")  # [R_J, R_K]
    V = sub[RJ, RK]                                                   # v = R_J - R_K
    for I in range(na):
        for J in range(na):
            Wij = Wa[(I, J)]                       # [R_J] mu nu
            Dij = Da[(I, J)]                       # [R_J] i j
            for K in range(na):
                Cik = Ca[(I, K)]                   # [R_K] mu i k
                # a2b1 intermediate: T[R_J] = sum_{R_K} C[I,K,R_K] D[K,J,R_J - R_K]
                Dkj = Da[(K, J)][V]                # [R_J, R_K] k j
                Tsum = np.einsum("bmik,abkj->amij", Cik, Dkj, optimize=True)
                S4 = np.einsum("amn,amij->anij", Wij, Tsum, optimize=True)  # [R_J] nu i j
                for L in range(na):
                    Cjl = Ca[(J, L)]               # [u] nu j l
                    # a2b2
                    Dkl = Da[(K, L)]               # [w] k l
                    E1 = np.einsum("unjl,vukl->vnjk", Cjl, Dkl[add], optimize=True)  # [v] nu j k
                    CW = np.einsum("amn,bmik->abnik", Wij, Cik, optimize=True)         # [R_J, R_K]
                    H[(I, J)] += np.einsum("abnik,abnjk->aij", CW, E1[V], optimize=True)
                    # a1b1: result cell v + u
                    F = np.einsum("abnik,aij->abnkj", CW, Dij, optimize=True)
                    G = np.einsum("abnkj,unjl->abukl", F, Cjl, optimize=True)
                    tgt = add[V.reshape(-1)].reshape(nc, nc, nc)  # cell v + u for [R_J, R_K, u]
                    np.add.at(H[(K, L)], tgt.reshape(-1), G.reshape((-1,) + G.shape[3:]))
                    # a1b2: result cell v
                    Dil = Da[(I, L)]               # [R_L] i l
                    P = np.einsum("unjl,auil->anji", Cjl, Dil[add], optimize=True)  # [R_J] nu j i
                    Qm = np.einsum("amn,anji->amji", Wij, P, optimize=True)
                    R3 = np.einsum("bmik,amji->abkj", Cik, Qm, optimize=True)
                    np.add.at(H[(K, J)], V.reshape(-1), R3.reshape((-1,) + R3.shape[2:]))
                    # a2b1: result cell R_J + u
                    R4 = np.einsum("anij,unjl->auil", S4, Cjl, optimize=True)
                    np.add.at(H[(I, L)], add.reshape(-1), R4.reshape((-1,) + R4.shape[2:]))
    return {(A, B, cells[c]): H[(A, B)][c] for (A, B) in H for c in range(nc)}


def ordered_blocks(full: np.ndarray, nb) -> dict:
    """Atom blocks (I, J, (0,0,0)) of a full Gamma-point matrix, all ordered pairs."""
    off = np.concatenate([[0], np.cumsum(nb)]).astype(int)
    return {(I, J, (0, 0, 0)): full[off[I]:off[I + 1], off[J]:off[J + 1]].copy()
            for I in range(len(nb)) for J in range(len(nb))}


def full_from_blocks(blocks: dict, nb) -> np.ndarray:
    off = np.concatenate([[0], np.cumsum(nb)]).astype(int)
    dtype = next(iter(blocks.values())).dtype if blocks else float  # no blocks: every one filtered out
    M = np.zeros((off[-1], off[-1]), dtype)
    for (I, J, _R), b in blocks.items():
        M[off[I]:off[I + 1], off[J]:off[J + 1]] += b
    return M


# ----------------------------------------------------------------------------- W_c

def power_hemat(A: np.ndarray, power: float, threshold: float):
    """Z diag(w^p) Z^H over ascending eigenvalues, those below the threshold set to zero
    (utils_matrix_m_mpi.h:677-720: n_filtered = first index with w >= threshold)."""
    w, Z = np.linalg.eigh(A)
    nf = len(w)
    for i in range(len(w)):
        if w[i] >= threshold:
            nf = i
            break
    wp = np.zeros_like(w)
    wp[nf:] = np.power(w[nf:], power)
    return (Z * wp) @ Z.conj().T


def wc_freq(chi0: np.ndarray, v_eps: np.ndarray, v_cut: np.ndarray, sqrt_threshold: float = 0.0):
    """Wc = Vcut^1/2 [eps^-1 - 1] Vcut^1/2, eps = 1 - V^1/2 chi0 V^1/2 (epsilon.cpp:2140-2300)."""
    s = power_hemat(v_eps, 0.5, sqrt_threshold)
    sc = power_hemat(v_cut, 0.5, sqrt_threshold)
    eps = np.eye(len(s)) - s @ chi0 @ s
    x = np.linalg.solve(eps, sc) - sc
    return sc @ x


# ----------------------------------------------------------------------------- continuation + QPE

class Pade:
    """AnalyContPade (analycont.cpp:12-70): Thiele's reciprocal differences on n_pars points."""

    def __init__(self, n_pars: int, xs, data):
        xs = list(xs)
        data = list(data)
        n_data = len(data)
        if n_pars < 0:
            n_pars = n_data
        if n_data <= n_pars:
            n_pars = n_data
            px, dn = xs, data
        else:
            step = n_data // (n_pars - 1)
            px = [xs[i * step] for i in range(n_pars - 1)] + [None]
            dn = [data[i * step] for i in range(n_pars - 1)] + [data[n_data - 1]]
            px[n_pars - 1] = 0j  # par_x of the last point is left value-initialised (analycont.cpp:35-41)
        g = np.zeros((n_pars, n_pars), complex)
        g[:, 0] = dn
        for p in range(1, n_pars):
            for i in range(p, n_pars):
                g[i, p] = (g[p - 1, p - 1] - g[i, p - 1]) / ((px[i] - px[p - 1]) * g[i, p - 1])
        self.n = n_pars
        self.x = np.array(px, complex)
        self.y = np.array([g[i, i] for i in range(n_pars)])

    def __call__(self, x: complex) -> complex:
        t = 1.0 + 0j
        for p in range(self.n - 1, 0, -1):
            t = 1.0 + self.y[p] * (x - self.x[p - 1]) / t
        return self.y[0] / t


def qpe_solve(pade: Pade, e_mf, e_fermi, vxc, sigma_x, diff_init=1.0e-3, thres=1.0e-5, n_iter_max=200):
    """qpe_solver_pade_self_consistent (qpe_solver.cpp): returns (info, e_qp, sigc)."""
    escale = 0.1
    n_iter = 0
    e_last = e_mf
    diff = diff_init
    sig_last = 0j
    while True:
        n_iter += 1
        if not n_iter <= n_iter_max:
            break
        e_this = e_last + escale * diff
        sig = pade(complex(e_this - e_fermi))
        diff = e_mf - vxc + sigma_x + sig.real - e_this
        e_last = e_mf - vxc + sigma_x + sig.real
        sig_last = sig
        if abs(diff) < thres or n_iter == n_iter_max - 1:
            break
    info = 1 if n_iter > n_iter_max - 1 else 0
    return info, e_last, sig_last


# ----------------------------------------------------------------------------- periodic exchange

def coulomb_r(inp: RPAInput, vq: dict, rlist):
    """FT_Vq (coulmat.cpp:7-90) with ordered atom pairs: V(R) = Re sum_q sum_{q' in star(q)}
    e^{-i 2 pi q'.R} / n_k V(q) (conjugated for q' != q, the time-reversed partner)."""
    klist, _, ibz_order, _ = k_lists(inp)
    star = {r: [k for k in range(inp.n_kpts) if int(inp.ibz_map[k]) == r] for r in ibz_order}
    out = {}
    for R in rlist:
        Rc = np.asarray(R, float) @ inp.latvec
        for (iq, I, J), v in vq.items():
            acc = np.zeros_like(v, dtype=complex)
            acc_t = np.zeros((v.shape[1], v.shape[0]), complex)
            for kb in star[iq]:
                ph = np.exp(-1j * TWO_PI * float(np.dot(klist[kb], Rc))) / inp.n_kpts
                if kb == iq:
                    acc += v * ph
                    acc_t += v.conj().T * ph
                else:
                    acc += v.conj() * ph
                    acc_t += v.T * ph
            key = (I, J, tuple(R))
            out[key] = out.get(key, 0) + acc.real
            if I != J and (iq, J, I) not in vq:
                key = (J, I, tuple(R))
                out[key] = out.get(key, 0) + acc_t.real
    return out


def dmat_r(inp: RPAInput, ispin: int, rlist):
    """get_dmat_cplx_R (meanfield.cpp:201-244): D(R) = sum_k e^{-i 2 pi k.R} D(k),
    D(k)_ij = sum_n w_n psi_ni psi_nj^*, real part; atom blocks of every ordered pair."""
    _, kfrac, _, _ = k_lists(inp)
    wg = inp.wg[ispin] / inp.n_kpts
    dk = []
    for k in range(inp.n_kpts):
        ev = inp.wfc[ispin, k]
        w = np.zeros(inp.n_bands)
        for n in range(inp.n_bands):
            w[n] = wg[k, n] * 0.5 * inp.n_spins
            if w[n] < 1e-4 / inp.n_kpts:
                w[n] = 0.0
                break
        dk.append(ev.T @ (w[:, None] * ev.conj()))
    full = {}
    for R in rlist:
        acc = np.zeros((inp.n_ao, inp.n_ao), complex)
        for k in range(inp.n_kpts):
            acc += np.exp(-1j * TWO_PI * float(np.dot(kfrac[k], R))) * dk[k]
        full[tuple(R)] = acc.real
    return blocks_of(full, inp.nao)


def shift_bvk(H: dict, inp: RPAInput):
    """Each (I, J, R) block moved to the image R + n period (n in {-1, 0, 1}^3) nearest to
    x_I - x_J - R (exx.cpp:683-725; applied when fractional coordinates are set)."""
    frac = inp.positions @ np.linalg.inv(inp.latvec)
    per = np.asarray(inp.period)
    out = {}
    for (I, J, R), m in H.items():
        best, Rb = math.inf, None
        for i in (-1, 0, 1):
            for j in (-1, 0, 1):
                for k in (-1, 0, 1):
                    Rij = np.asarray(R) + per * np.array([i, j, k])
                    d = (frac[I] - frac[J] - Rij) @ inp.latvec
                    n2 = float(d @ d)
                    if n2 < best:
                        best, Rb = n2, tuple(int(x) for x in Rij)
        out[(I, J, Rb)] = m
    return out


@dataclass
class BandPoints:
    """k-points off the SCF grid (task = exx_band / g0w0_band): fractional coordinates, their
    mean-field eigenpairs and v_xc (librpa_set_band_kvec, set_band_occ_eigval, set_wfc_band)."""
    kfrac: np.ndarray   # (n, 3)
    wfc: np.ndarray     # (n_spins, n, n_bands, n_ao)
    ekb: np.ndarray     # (n_spins, n, n_bands) Hartree
    efermi: float
    vxc: np.ndarray | None = None  # (n_spins, n, n_bands) Hartree


def drop_small(blocks: dict, threshold: float) -> dict:
    """LibRI's set_tensors filter (threshold_filter, RI_Tools.hpp:16-27): an atom-pair block is kept
    only if its largest |x| exceeds the threshold (0: every block)."""
    if threshold <= 0:
        return blocks
    return {k: v for k, v in blocks.items() if np.abs(v).max() > threshold}


def small_basis_view(inp: RPAInput) -> RPAInput:
    """A shrunk input as its exchange sees it: the RI coefficients and ABF counts of the small
    basis (Exx::build on Cs_shrinked_data, driver/task_gw_band.cpp:92-99)."""
    if inp.Cs_small is None:
        raise ValueError("use_shrink_abfs: the exchange needs the RI coefficients of the small basis")
    return dataclasses.replace(inp, Cs=inp.Cs_small, nabf=list(inp.nabf_small))


def exx_kgrid(inp: RPAInput, v_cut: dict, band: BandPoints | None = None, thr_v: float = 0.0, thr_d: float = 0.0):
    """v_exx[s, k, n] (Hartree) on the SCF k-grid (task = exx; exx.cpp:213-500, :720-860), or at
    the band points: H(R) summed with e^{i 2 pi k.R} at any k (Exx::build_KS_band).  A shrunk
    input (inp.sinvS set) takes the small basis, where v_cut is then given.  thr_v / thr_d: LibRI's
    block filters of V(R) and D(R)."""
    if inp.sinvS is not None:
        inp = small_basis_view(inp)
    _, kfrac, _, _ = k_lists(inp)
    kpts, wfc = (kfrac, inp.wfc) if band is None else (band.kfrac, band.wfc)
    rlist = r_grid(inp.period)
    C = cs_tensors(inp, 0.0)
    VR = drop_small(coulomb_r(inp, v_cut, rlist), thr_v)   # libri_exx_threshold_V / _D (exx.cpp:365-418)
    out = np.zeros((inp.n_spins, len(kpts), inp.n_bands))
    off = np.concatenate([[0], np.cumsum(inp.nao)]).astype(int)
    for s in range(inp.n_spins):
        H = cal_hs_cells(C, VR, drop_small(dmat_r(inp, s, rlist), thr_d), inp.nao, inp.nabf, inp.period)
        H = shift_bvk(H, inp)
        for k in range(len(kpts)):
            Hk = np.zeros((inp.n_ao, inp.n_ao), complex)
            for (I, J, R), m in H.items():
                ph = np.exp(1j * TWO_PI * float(np.dot(kpts[k], R)))
                Hk[off[I]:off[I + 1], off[J]:off[J + 1]] += ph * m
            ev = wfc[s, k]
            out[s, k] = -np.einsum("ni,ij,nj->n", ev.conj(), Hk, ev).real
    return out


# ----------------------------------------------------------------------------- pipeline

def dmat(inp: RPAInput, ispin: int) -> np.ndarray:
    """D = sum_n w_n psi_n psi_n^*, w = wg/n_k * n_s/2, states taken up to the first below
    1e-4/n_k (meanfield.cpp:201-228); Gamma point, real part."""
    wg = inp.wg[ispin, 0] / inp.n_kpts
    ev = inp.wfc[ispin, 0]
    D = np.zeros((inp.n_ao, inp.n_ao), complex)
    for n in range(inp.n_bands):
        w = wg[n] * 0.5 * inp.n_spins
        if w < 1e-4 / inp.n_kpts:
            break
        D += w * np.outer(ev[n], ev[n].conj())
    return D.real


def g0w0_gamma(inp: RPAInput, v_cut: dict, vxc: np.ndarray, opts: Options | None = None,
               n_params: int = -1, sqrt_threshold: float = 0.0, thr_w: float = 0.0, thr_g: float = 0.0):
    """G0W0 at the Gamma point.  inp.Vq holds the Coulomb matrix of the dielectric function,
    v_cut the truncated Coulomb (W and exchange); vxc (n_spins, 1, n_states) in Hartree.
    Returns per spin arrays (Hartree): vexx, sigc (complex, at e_qp), e_qp, sigc_iw (KS
    diagonal on the imaginary axis) and the grids."""
    if inp.n_kpts != 1 or tuple(inp.period) != (1, 1, 1):
        raise ValueError("the G0W0 oracle covers Gamma-only inputs")
    opts = opts or Options()
    grid = grids_for(inp, opts)
    nb, nao = inp.nabf, inp.nao
    nf = opts.nfreq
    C = cs_tensors(inp, 0.0)
    z = (0, 0, 0)

    # chi0(omega) at q = 0 and the two Coulomb matrices (real at Gamma)
    chi0q = chi0q_partial(inp, opts, 0, nf)
    pairs = upper_pairs(inp.n_atoms)
    v_eps = assemble_full({p: inp.Vq[(0, *p)].real for p in pairs if (0, *p) in inp.Vq}, nb, dtype=float)
    v_c = assemble_full({p: v_cut[(0, *p)].real for p in pairs if (0, *p) in v_cut}, nb, dtype=float)

    # exchange: V(R = 0) of the truncated Coulomb, all ordered pairs
    VR = ordered_blocks(v_c, nb)
    out = {"grid": grid, "vexx": [], "sigc": [], "e_qp": [], "sigc_iw": [], "info": []}
    for s in range(inp.n_spins):
        D = ordered_blocks(dmat(inp, s), nao)
        H = full_from_blocks(cal_hs_loops(C, VR, D, inp.n_atoms, (1, 1, 1)), nao)
        ev = inp.wfc[s, 0]
        out["vexx"].append(-np.einsum("ni,ij,nj->n", ev.conj(), H, ev).real)

    # Wc(omega) -> Wc(tau)
    Wf = []
    for iw in range(nf):
        X = assemble_full({k: v.real for k, v in chi0q[iw][0].items()}, nb, dtype=float)
        Wf.append(wc_freq(X, v_eps, v_c, sqrt_threshold))
    Wt = [sum(grid["cos_f2t"][it, iw] * Wf[iw] for iw in range(nf)) for it in range(nf)]

    kfrac = np.zeros((1, 3))
    for s in range(inp.n_spins):
        sig_w = np.zeros((nf, inp.n_ao, inp.n_ao), complex)
        for it, tau in enumerate(grid["tau"]):
            # libri_g0w0_threshold_Wc / _G (gw.cpp:459-616)
            Wb = drop_small(ordered_blocks(Wt[it], nb), thr_w)
            Gp = drop_small(blocks_of(build_gf(inp, s, tau, kfrac, [z]), nao), thr_g)
            Gn = drop_small(blocks_of(build_gf(inp, s, -tau, kfrac, [z]), nao), thr_g)
            Sp = full_from_blocks(cal_hs_loops(C, Wb, Gp, inp.n_atoms, (1, 1, 1)), nao)
            Sn = full_from_blocks(cal_hs_loops(C, Wb, Gn, inp.n_atoms, (1, 1, 1)), nao)
            cos_part, sin_part = 0.5 * (Sp + Sn), 0.5 * (Sp - Sn)
            for iw in range(nf):
                sig_w[iw] += grid["cos_t2f"][iw, it] * cos_part + 1j * grid["sin_t2f"][iw, it] * sin_part
        ev = inp.wfc[s, 0]
        sig_ks = np.einsum("ni,wij,nj->nw", ev.conj(), sig_w, ev)
        xs = [1j * w for w in grid["omega"]]
        e_qp, sigc, info = [], [], []
        for n in range(inp.n_bands):
            pade = Pade(n_params, xs, sig_ks[n])
            f, e, sg = qpe_solve(pade, inp.ekb[s, 0, n], inp.efermi, vxc[s, 0, n], out["vexx"][s][n])
            info.append(f)
            e_qp.append(e)
            sigc.append(sg)
        out["sigc_iw"].append(sig_ks)
        out["e_qp"].append(np.array(e_qp))
        out["sigc"].append(np.array(sigc))
        out["info"].append(info)
    return out


# ----------------------------------------------------------------------------- G0W0 on k-grids

def power_hemat_real(A: np.ndarray, power: float, threshold: float):
    """power_hemat_blacs_real (utils_matrix_m_mpi.h:886-1010), used at the Gamma point: the
    eigenpairs of Re A with eigenvalues in descending order, those below the threshold (counted
    from the smallest) set to zero.  Returns (A^p, Z, Z w^p (column scaled), n_nonsingular)."""
    w, Z = np.linalg.eigh(-A.real)
    w = -w
    n = len(w)
    n_filtered = n
    for i in range(n):
        if w[n - 1 - i] >= threshold:
            n_filtered = i
            break
    nn = n - n_filtered
    wp = np.zeros(n)
    wp[:nn] = np.power(w[:nn], power)
    scaled = Z * wp
    return scaled @ Z.T, Z, scaled, nn


def wc_freq_head(chi0, v_eps, v_cut, epsmac, sqrt_threshold=0.0):
    """The Gamma-point branch with the head of the dielectric matrix replaced (replace_w_head,
    option_dielect_func != 3; epsilon.cpp:2030-2120): in the basis of V's eigenvectors (descending
    eigenvalues), eps = 1 - Z (L^1/2 Z^T chi0 Z L^1/2)' Z^T where ' sets the (0, 0) element (the
    largest Coulomb eigenvalue) to 1 - eps_mac."""
    _, Z, sq, nn = power_hemat_real(v_eps, 0.5, sqrt_threshold)
    X = sq[:, :nn].conj().T @ chi0 @ sq[:, :nn]
    X[0, 0] = 1.0 - epsmac
    eps = np.eye(len(Z)) - Z[:, :nn] @ X @ Z[:, :nn].conj().T
    sc = power_hemat(v_cut, 0.5, sqrt_threshold)
    return sc @ (np.linalg.solve(eps, sc) - sc)


def g0w0_kgrid(inp: RPAInput, v_cut: dict, vxc: np.ndarray, opts: Options | None = None, n_params: int = -1,
               epsmac=None, sqrt_threshold: float = 0.0, band: BandPoints | None = None, thr_w: float = 0.0,
               thr_g: float = 0.0):
    """G0W0 on the SCF k-grid (task = g0w0 with k-points; epsilon.cpp:1763-2322, :2323-2660,
    gw.cpp:217-876, :884-1240).  inp.Vq: Coulomb matrix of the dielectric function at the IBZ
    q-points, v_cut: truncated Coulomb there; epsmac: the macroscopic dielectric function at the
    minimax frequencies (replace_w_head with option 0 copies dielecfunc_out), or None.
    Returns per spin (n_k, n_states) arrays in Hartree: vexx, sigc at e_qp, e_qp.  With band,
    Sigma_c(R) and H_x(R) are summed at the band points instead and the QP equation takes their
    eigenvalues, Fermi level and v_xc (librpa_get_g0w0_sigc_band_k, compute_g0w0.cpp:300-366)."""
    opts = opts or Options()
    grid = grids_for(inp, opts)
    nb, nao = inp.nabf, inp.nao
    nf = opts.nfreq
    klist, kfrac, ibz_order, _ = k_lists(inp)
    rl = r_grid(inp.period)
    C = cs_tensors(inp, 0.0)
    pairs = upper_pairs(inp.n_atoms)
    nbt = int(sum(nb))
    chi0q = chi0q_partial(inp, opts, 0, nf)
    # ABF shrink: chi0 and W_c in the small basis of the Coulomb matrices (shrink_abfs_chi0,
    # chi0.cpp:711-898), W_c taken back to the RI basis as U^H W_c U (unfold_abfs_Wc,
    # src/gw_old.cpp:208-225) for the self-energy
    shrink = inp.sinvS is not None
    nbw = list(inp.nabf_small) if shrink else nb
    if shrink:
        chi0q = shrink_chi0q(chi0q, inp.sinvS, nb, nbw)
    nbwt = int(sum(nbw))

    # Wc(q, omega) at the IBZ points
    Wq = {}
    for iq, kq in enumerate(ibz_order):
        v_e = assemble_full({p: inp.Vq[(kq, *p)] for p in pairs if (kq, *p) in inp.Vq}, nbw)
        v_c = assemble_full({p: v_cut[(kq, *p)] for p in pairs if (kq, *p) in v_cut}, nbw)
        gamma = bool(np.all(np.abs(klist[kq]) < 1e-10))
        for iw in range(nf):
            X = assemble_full(chi0q[iw][iq], nbw)
            if gamma and epsmac is not None:
                W = wc_freq_head(X, v_e, v_c, epsmac[iw], sqrt_threshold)
            else:
                s_e = power_hemat(v_e, 0.5, sqrt_threshold)
                s_c = power_hemat(v_c, 0.5, sqrt_threshold)
                eps = np.eye(nbwt) - s_e @ X @ s_e
                W = s_c @ (np.linalg.solve(eps, s_c) - s_c)
            if shrink:
                U = inp.sinvS[iq]
                W = U.conj().T @ W @ U
            Wq[(iq, iw)] = W

    # Wc(R, omega) (FT_Wc_freq_q: the BZ from the IBZ with W(-q) = W(q)^*, 1/n_k), real part,
    # then Wc(R, tau) = sum_omega f2t(tau, omega) Wc(R, omega)
    ibz_of = {kq: iq for iq, kq in enumerate(ibz_order)}
    WR = {}
    for c, R in enumerate(rl):
        Rc = np.asarray(R, float) @ inp.latvec
        for iw in range(nf):
            acc = np.zeros((nbt, nbt), complex)
            for k in range(inp.n_kpts):
                rep = int(inp.ibz_map[k])
                m = Wq[(ibz_of[rep], iw)]
                if k != rep:
                    m = m.conj()
                acc += np.exp(-1j * TWO_PI * float(np.dot(klist[k], Rc))) / inp.n_kpts * m
            WR[(c, iw)] = acc.real
    Wt = []
    for it in range(nf):
        blocks = {}
        off = np.concatenate([[0], np.cumsum(nb)]).astype(int)
        for c, R in enumerate(rl):
            full = sum(grid["cos_f2t"][it, iw] * WR[(c, iw)] for iw in range(nf))
            for I in range(inp.n_atoms):
                for J in range(inp.n_atoms):
                    blocks[(I, J, tuple(R))] = full[off[I]:off[I + 1], off[J]:off[J + 1]].copy()
        Wt.append(drop_small(blocks, thr_w))   # libri_g0w0_threshold_Wc (gw.cpp:459-470)

    out = {"grid": grid, "vexx": exx_kgrid(inp, v_cut, band), "sigc": [], "e_qp": [], "sigc_iw": []}
    if band is None:
        kpts, wfc, ekb, ef, vx = kfrac, inp.wfc, inp.ekb, inp.efermi, vxc
    else:
        kpts, wfc, ekb, ef, vx = band.kfrac, band.wfc, band.ekb, band.efermi, band.vxc
    offa = np.concatenate([[0], np.cumsum(nao)]).astype(int)
    for s in range(inp.n_spins):
        sig_R = {}  # (I, J, R) -> (nf, n_I, n_J) complex
        for it, tau in enumerate(grid["tau"]):
            Gp = drop_small(blocks_of(build_gf(inp, s, tau, kfrac, rl), nao), thr_g)
            Gn = drop_small(blocks_of(build_gf(inp, s, -tau, kfrac, rl), nao), thr_g)
            Sp = cal_hs_cells(C, Wt[it], Gp, nao, nb, inp.period)
            Sn = cal_hs_cells(C, Wt[it], Gn, nao, nb, inp.period)
            for key in Sp:
                if key not in Sn:
                    continue
                cp, sn = 0.5 * (Sp[key] + Sn[key]), 0.5 * (Sp[key] - Sn[key])
                acc = sig_R.setdefault(key, np.zeros((nf,) + cp.shape, complex))
                for iw in range(nf):
                    acc[iw] += grid["cos_t2f"][iw, it] * cp + 1j * grid["sin_t2f"][iw, it] * sn
        sig_R = shift_bvk(sig_R, inp)
        nkp = len(kpts)
        sig_ks = np.zeros((nkp, inp.n_bands, nf), complex)
        for k in range(nkp):
            Sk = np.zeros((nf, inp.n_ao, inp.n_ao), complex)
            for (I, J, R), m in sig_R.items():
                ph = np.exp(1j * TWO_PI * float(np.dot(kpts[k], R)))
                Sk[:, offa[I]:offa[I + 1], offa[J]:offa[J + 1]] += ph * m
            ev = wfc[s, k]
            sig_ks[k] = np.einsum("ni,wij,nj->nw", ev.conj(), Sk, ev)
        xs = [1j * w for w in grid["omega"]]
        e_qp = np.zeros((nkp, inp.n_bands))
        sigc = np.zeros((nkp, inp.n_bands), complex)
        for k in range(nkp):
            for n in range(inp.n_bands):
                pade = Pade(n_params, xs, sig_ks[k, n])
                _f, e, sg = qpe_solve(pade, ekb[s, k, n], ef, vx[s, k, n], out["vexx"][s, k, n])
                e_qp[k, n], sigc[k, n] = e, sg
        out["sigc_iw"].append(sig_ks)
        out["e_qp"].append(e_qp)
        out["sigc"].append(sigc)
    return out
