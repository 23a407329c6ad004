"""The RPA correlation-energy path on the host cores, FP64, in large BLAS calls.

Test and measurement infrastructure only: the reference CPU arm and the CPU baseline of
bench.py time this, and the tests check it against the literal restatement in rpa_oracle.py.
It computes what LibRPA's task = rpa computes with the LibRI routing, in the same algebra as
``rpa_oracle.cal_chi0s_dense`` (itself checked against the literal LibRI loops of
``cal_chi0s_loops``), organised so that the work lands in a few multithreaded GEMMs per
(tau, spin) instead of per-block numpy calls:

  G(R, +-tau)   build_gf_Rt_libri_serial, src/core/chi0.cpp:303-426 (one GEMM per k, one
                phase GEMM over k)
  X(+-) = C G_super(+-)              first contraction of LRI::cal_loop3 (LRI-cal_loop3.hpp:902-965)
  T1 = sum_pass sum_{i,j,K} Ga_ij X_b^I[mu i; K] C^J[nu j; K - R]  (both passes share C^J, so the
                two passes' E = G^T X terms are summed before the contraction with C^J)
  T2 = sum_pass X_b^I[mu i; (R, J) j] X_a^J[nu j; (-R, I) i]       (labels a1b2_a2b1, :969-1032)
  FT + CT       chi_libri_ft_ct, src/core/chi0.cpp:507-596, with the tau -> omega cosine
                transform deferred to one GEMM over tau at the end
  E_c           compute_RPA_correlation_blacs_2d, src/core/epsilon.cpp:414-536: Pi = V chi0,
                LU, sum log(+-u_ii) + tr Pi per (q, omega)

The work is split into stages so that a caller can time them one at a time: ``tau_slice(it)``
for each minimax tau point, then ``correlation_energy()``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.linalg

from .rpa_oracle import (TWO_PI, Options, RPAInput, centred_mod, cs_tensors, grids_for, k_lists, r_grid,
                         tau_scale, upper_pairs)


_KERNEL = None


def _kernel():
    """The OpenMP chi0 kernel (cpu_chi0.cpp), built on first use."""
    global _KERNEL
    if _KERNEL is None:
        from .build_cpu import build
        lib = C.CDLL(str(build()))
        f = lib.cpu_chi0_tau
        f.restype = C.c_int
        f.argtypes = [C.c_int] + [C.c_void_p] * 4 + [C.c_int, C.c_int] + [C.c_void_p] * 8 + [C.c_longlong, C.c_void_p]
        lu = lib.cpu_lu_logdet
        lu.restype = C.c_int
        lu.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        _KERNEL = (f, lu)
    return _KERNEL


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class CpuPath:
    def __init__(self, inp: RPAInput, opts: Options | None = None, kernel: str = "openmp"):
        """kernel: "openmp" (cpu_chi0.cpp, the timed path) or "numpy" (the same algebra in
        per-block numpy calls; the check of the OpenMP kernel)."""
        opts = opts or Options()
        self.kernel = kernel
        self.inp, self.opts = inp, opts
        self.grid = grids_for(inp, opts)
        klist, kfrac, ibz_order, ibz_weight = k_lists(inp)
        self.kfrac, self.ibz_order, self.ibz_weight = kfrac, ibz_order, ibz_weight
        self.cells = r_grid(inp.period)
        nc = self.nc = len(self.cells)
        cidx = {c: i for i, c in enumerate(self.cells)}
        nao, nabf = list(inp.nao), list(inp.nabf)
        self.nao, self.nabf = nao, nabf
        n_at = self.n_at = len(nao)
        self.aoff = np.concatenate([[0], np.cumsum(nao)]).astype(int)
        self.boff = np.concatenate([[0], np.cumsum(nabf)]).astype(int)
        nt_ao = self.n_ao = int(self.aoff[-1])
        self.nsup = nc * nt_ao
        self.N = int(self.boff[-1])

        def sub(b, a):
            return centred_mod((b[0] - a[0], b[1] - a[1], b[2] - a[2]), inp.period)

        # cell of R_L - R_K for (K, L): the G_super block index
        self.dmat = np.array([[cidx[sub(RL, RK)] for RL in self.cells] for RK in self.cells])
        # for each R_J: cell of R_L - R_J for every column cell R_L (the C^J frame shift)
        self.dshift = np.array([[cidx[sub(RL, RJ)] for RL in self.cells] for RJ in self.cells])
        self.cneg = np.array([cidx[centred_mod((-R[0], -R[1], -R[2]), inp.period)] for R in self.cells])
        # G(R) phases e^{-i 2 pi k.R} (chi0.cpp:379-380) and FT phases e^{+i 2 pi q.(R latvec)} (:582)
        R = np.array(self.cells, float)
        self.gphase = np.exp(-1j * TWO_PI * (R @ kfrac.T))                       # [cell][k]
        qv = np.array([klist[i] for i in ibz_order])
        self.qphase = np.exp(1j * TWO_PI * (qv @ (R @ inp.latvec).T))             # [q][cell]
        # C^I as [(mu, i), (cell, K, k)] (LibRI cell folding and threshold: cs_tensors)
        cst = cs_tensors(inp, opts.libri_chi0_threshold_C)
        self.crow = []
        for I in range(n_at):
            M = np.zeros((nabf[I] * nao[I], self.nsup))
            for c, Rc in enumerate(self.cells):
                for K in range(n_at):
                    t = cst.get((I, K, Rc))
                    if t is not None:
                        M[:, c * nt_ao + self.aoff[K]: c * nt_ao + self.aoff[K + 1]] = t.reshape(nabf[I] * nao[I], nao[K])
            self.crow.append(M)
        self.call = np.vstack(self.crow)
        self.rowoff = np.concatenate([[0], np.cumsum([nabf[I] * nao[I] for I in range(n_at)])]).astype(int)
        # C^J as [nu][cell][ao][j] (the contraction's B operand, j innermost)
        self.ct = [self.crow[J].reshape(nabf[J], nao[J], nc, nt_ao).transpose(0, 2, 3, 1).copy() for J in range(n_at)]
        # upper atom pairs and the element offsets of their b_I x b_J blocks
        self.pairs = upper_pairs(n_at)
        self.eoff = np.concatenate([[0], np.cumsum([nabf[I] * nabf[J] for I, J in self.pairs])]).astype(int)
        self.e_tot = int(self.eoff[-1])
        nt = len(self.grid["tau"])
        self.nq = len(ibz_order)
        self.chi0q_tau = np.zeros((nt, self.nq, self.e_tot), complex)
        self.gamma_only = inp.n_kpts == 1
        # V(q): full matrices of the IBZ q points, blocks below vq_threshold dropped (input.cpp:577)
        self.V = []
        for ikf in ibz_order:
            M = np.zeros((self.N, self.N), complex)
            for (I, J) in self.pairs:
                v = inp.Vq.get((ikf, I, J))
                if v is None or np.abs(v.real).max() < opts.vq_threshold:
                    continue
                M[self.boff[I]:self.boff[I + 1], self.boff[J]:self.boff[J + 1]] = v
                if J > I:
                    M[self.boff[J]:self.boff[J + 1], self.boff[I]:self.boff[I + 1]] = v.conj().T
            self.V.append(M.real.copy() if self.gamma_only else M)
        # scatter indices of the upper pair blocks into an N x N matrix; diagonal-block mask
        idx, diag = [], []
        for (I, J) in self.pairs:
            r = np.arange(self.boff[I], self.boff[I + 1])[:, None]
            c = np.arange(self.boff[J], self.boff[J + 1])[None, :]
            idx.append((r * self.N + c).ravel())
            diag.append(np.full(nabf[I] * nabf[J], I == J))
        self.scatter = np.concatenate(idx)
        self.offdiag = ~np.concatenate(diag)
        if kernel == "openmp":
            # the OpenMP kernel's C^J operands: [nu][cell][ao][j], j padded to an even count
            self.ct_pad = []
            for J in range(n_at):
                ajp = (nao[J] + 1) // 2 * 2
                t = np.zeros((nabf[J], nc, nt_ao, ajp))
                t[..., :nao[J]] = self.ct[J]
                self.ct_pad.append(t)
            self.ct_ptrs = (C.c_void_p * n_at)(*[t.ctypes.data for t in self.ct_pad])
            self.k_args = dict(
                nao=np.asarray(nao, np.int32), nabf=np.asarray(nabf, np.int32), aoff=self.aoff.astype(np.int32),
                rowoff=self.rowoff.astype(np.int64), dshift=np.ascontiguousarray(self.dshift, np.int32),
                cneg=self.cneg.astype(np.int32), eoff=self.eoff.astype(np.int64))

    # ------------------------------------------------------------------ stages
    def _gf(self, ispin, tau):
        """G(R, tau) for every cell, [cell][ao][ao] (chi0.cpp:303-426)."""
        s = tau_scale(self.inp, ispin, tau, self.opts.n_bands_chi0)
        A = np.stack([ev.T @ (s[ik][:, None] * ev.conj()) for ik, ev in enumerate(self.inp.wfc[ispin])])
        G = (self.gphase @ A.reshape(len(A), -1)).real.reshape(self.nc, self.n_ao, self.n_ao)
        return -G if tau < 0 else G

    def _gsuper(self, G):
        S = G[self.dmat]                                      # [cK][cL][k][l]
        return S.transpose(0, 2, 1, 3).reshape(self.nsup, self.nsup)

    def tau_slice(self, it: int):
        """chi0(R, tau_it) of every upper atom pair and cell, Fourier-transformed to the IBZ q
        points and stored for the cosine transform of correlation_energy()."""
        tau = self.grid["tau"][it]
        nc, n_ao, nsup = self.nc, self.n_ao, self.nsup
        nao, nabf, aoff = self.nao, self.nabf, self.aoff
        chi0R = np.zeros((nc, self.e_tot))
        for s in range(self.inp.n_spins):
            G = {+1: self._gf(s, tau), -1: self._gf(s, -tau)}
            X = {sg: self.call @ self._gsuper(G[sg]) for sg in (+1, -1)}
            if self.kernel == "openmp":
                a = self.k_args
                Gp, Gm = np.ascontiguousarray(G[+1]), np.ascontiguousarray(G[-1])
                _kernel()[0](self.n_at, _p(a["nao"]), _p(a["nabf"]), _p(a["aoff"]), _p(a["rowoff"]), nc, n_ao,
                          _p(X[+1]), _p(X[-1]), _p(Gp), _p(Gm), C.cast(self.ct_ptrs, C.c_void_p), _p(a["dshift"]),
                          _p(a["cneg"]), _p(a["eoff"]), self.e_tot, _p(chi0R))
                continue
            # both passes of X_b^I in one operand [(mu, K), (pass, i)]: pass 0 = X(-) with G(+),
            # pass 1 = X(+) with G(-)
            XX = []
            for I in range(self.n_at):
                r0, r1 = self.rowoff[I], self.rowoff[I + 1]
                xm = X[-1][r0:r1].reshape(nabf[I], nao[I], nsup)
                xp = X[+1][r0:r1].reshape(nabf[I], nao[I], nsup)
                XX.append(np.concatenate([xm, xp], axis=1).transpose(0, 2, 1).reshape(nabf[I] * nsup, 2 * nao[I]))
            for J in range(self.n_at):
                for c in range(nc):
                    CJs = self.ct[J][:, self.dshift[c]].reshape(nabf[J], nsup * nao[J])   # [nu, (K, j)]
                    cm = self.cneg[c]
                    for I in range(J + 1):
                        p = self.pairs.index((I, J))
                        gI = slice(aoff[I], aoff[I + 1])
                        gJ = slice(aoff[J], aoff[J + 1])
                        GG = np.concatenate([G[+1][c][gI, gJ], G[-1][c][gI, gJ]], axis=0)   # [(pass, i), j]
                        E = XX[I] @ GG                                                      # [(mu, K), j]
                        acc = E.reshape(nabf[I], nsup * nao[J]) @ CJs.T
                        r0 = self.rowoff[I]
                        q0 = self.rowoff[J]
                        for b, a in ((-1, +1), (+1, -1)):
                            x1 = X[b][r0:r0 + nabf[I] * nao[I], c * n_ao + aoff[J]: c * n_ao + aoff[J + 1]]
                            x2 = X[a][q0:q0 + nabf[J] * nao[J], cm * n_ao + aoff[I]: cm * n_ao + aoff[I + 1]]
                            acc += x1.reshape(nabf[I], -1) @ x2.reshape(nabf[J], nao[J], nao[I]).transpose(0, 2, 1).reshape(nabf[J], -1).T
                        chi0R[c, self.eoff[p]:self.eoff[p + 1]] += acc.ravel()
        self.chi0q_tau[it] += (2.0 / self.inp.n_spins) * (self.qphase @ chi0R)

    def correlation_energy(self):
        """E_c and the per-IBZ-q contributions from the tau slices computed so far."""
        g = self.grid
        nw = len(g["omega"])
        nt = len(g["tau"])
        chi0q = (np.asarray(g["cos_t2f"], float)[:, :nt] @ self.chi0q_tau.reshape(nt, -1)).reshape(nw, self.nq, self.e_tot)
        N = self.N
        dt = float if self.gamma_only else complex
        per_q = []
        for iq in range(self.nq):
            # chi0(q, omega) of every omega as full matrices [omega][N][N] (lower blocks = adjoints)
            X = np.zeros((nw, N * N), dt)
            Xs = np.zeros((nw, N * N), dt)
            v = chi0q[:, iq].real if self.gamma_only else chi0q[:, iq]
            X[:, self.scatter] = v
            Xs[:, self.scatter[self.offdiag]] = v[:, self.offdiag]
            X = X.reshape(nw, N, N) + Xs.reshape(nw, N, N).conj().transpose(0, 2, 1)
            # Pi = V chi0 for all omega in one GEMM
            P = (self.V[iq] @ X.transpose(1, 0, 2).reshape(N, nw * N)).reshape(N, nw, N).transpose(1, 0, 2)
            tr = np.einsum("wii->w", P)
            M = np.ascontiguousarray(np.eye(N, dtype=dt)[None] - P)
            ld = self._logdet(M)
            cq = np.sum((tr + ld) * np.asarray(g["omega_w"])) * self.ibz_weight[iq] / TWO_PI
            per_q.append(complex(cq))
        return complex(sum(per_q)), per_q

    def _logdet(self, M):
        """sum_i log(+-u_ii) of the LU of each M[w] (epsilon.cpp:489-536)."""
        nw, N = M.shape[0], M.shape[1]
        if self.kernel == "openmp":
            out = np.zeros(2 * nw)
            _kernel()[1](N, nw, 0 if self.gamma_only else 1, _p(M), _p(out))
            return out[0::2] + 1j * out[1::2] if not self.gamma_only else out[0::2]
        res = []
        for w in range(nw):
            lu, _ = scipy.linalg.lu_factor(M[w], check_finite=False)
            d = np.diag(lu)
            if np.iscomplexobj(d):
                res.append(complex(np.sum(np.log(np.where(d.real > 0, d, -d)))))
            else:
                res.append(float(np.sum(np.log(np.where(d > 0, d, -d)))))
        return np.array(res)

    def run(self):
        for it in range(len(self.grid["tau"])):
            self.tau_slice(it)
        return self.correlation_energy()

    def flops_per_tau(self):
        """FLOPs of one tau slice (per spin): X GEMMs, E = G^T X, T1 and T2 over the upper pairs."""
        nsup, nc = self.nsup, self.nc
        rows_c = int(self.rowoff[-1])
        f = 2.0 * 2.0 * rows_c * nsup * nsup
        for (I, J) in self.pairs:
            aI, aJ, bI, bJ = self.nao[I], self.nao[J], self.nabf[I], self.nabf[J]
            f += nc * (2.0 * bI * nsup * 2 * aI * aJ + 2.0 * bI * bJ * aJ * nsup + 2 * 2.0 * bI * bJ * aI * aJ)
        return f * self.inp.n_spins
