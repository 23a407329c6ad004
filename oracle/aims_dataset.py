"""Oracle (test infrastructure only): reader for LibRPA's FHI-aims dataset export.

Follows the driver readers of the reference (driver/read_data.cpp):
  band_out          read_scf_occ_eigenvalues   :32-140
  stru_out          read_stru                  :1814-1867
  bz_sampling_out   read_bz_sampling           :1869-1916
  basis_out         read_basis                 :1976-2011
  KS_eigenvector_*  handle_KS_file             :184-284  (order: ao, spinor, band, spin)
  Cs_data_*         handle_Cs_file_binary      :690-747  (keep if max|C| >= cs_threshold, default 1e-6)
                    handle_Cs_file (text)      :618-688
  coulomb_mat_*     handle_Vq_row_file         :1472-1650 (binary and text; upper atom blocks)
  coulomb_cut_*     the same format (truncated Coulomb of G0W0, driver/task/g0w0.cpp:33-45)
  vxc_out           read_vxc                   :142-182
  shrink_sinvS_*    handle_sinvS_file          :2455-2568 (ABF shrink transform U(q), text and binary)
  Cs_shrinked_data_* read_ri_shrink            :2570-2622 (only its per-atom n_mu: the small ABF basis)
Binary (FHI-aims) or text (ABACUS) is told apart as the reference does (check_Cs_file_binary,
check_coulomb_file_binary, :414-453): a file whose first token parses as an integer is text.
"""
from __future__ import annotations

import glob
import os
import struct

import numpy as np

from .rpa_oracle import RPAInput


def _tokens(path):
    with open(path) as f:
        return f.read().split()


def is_text_file(path) -> bool:
    """The first whitespace-separated token parses as an integer (read_data.cpp:414-453)."""
    with open(path, "rb") as f:
        head = f.read(64)
    try:
        tok = head.split()[0].decode("ascii")
        int(tok)
        return True
    except (IndexError, UnicodeDecodeError, ValueError):
        return False


def _cs_headers(fn):
    """(I, J, R1, R2, R3, n_i, n_j, n_mu) of every block of one Cs_data file, 1-based atoms."""
    out = []
    if is_text_file(fn):
        t = _tokens(fn)
        p = 2
        while p + 8 <= len(t):
            v = [int(x) for x in t[p:p + 8]]
            out.append(v)
            p += 8 + v[5] * v[6] * v[7]
        return out
    raw = open(fn, "rb").read()
    _natom, _ncell, nblk = struct.unpack_from("<3i", raw, 0)
    off = 12
    for _ in range(nblk):
        v = list(struct.unpack_from("<8i", raw, off))
        out.append(v)
        off += 32 + 8 * v[5] * v[6] * v[7]
    return out


def _basis_from_cs(d: str, nat: int, prefix: str = "Cs_data"):
    """read_basis_from_Cs (read_data.cpp:2083-2152): per atom, n_i and n_mu of blocks where it is
    the first atom and n_j where it is the second."""
    aw, aa = {}, {}
    for fn in sorted(glob.glob(d + prefix + "*")):
        for I, J, _r1, _r2, _r3, ni, nj, nmu in _cs_headers(fn):
            aw[I - 1] = ni
            aw[J - 1] = nj
            aa[I - 1] = nmu
    return [aw[a] for a in range(nat)], [aa[a] for a in range(nat)]


def read_dataset(d: str, cs_threshold: float = 1e-6) -> RPAInput:
    d = d.rstrip("/") + "/"
    t = _tokens(d + "band_out")
    nk, ns, nb, nao = int(t[0]), int(t[1]), int(t[2]), int(t[3])
    efermi = float(t[4])
    p = 5
    wg = np.zeros((ns, nk, nb))
    ekb = np.zeros((ns, nk, nb))
    for _ in range(nk):
        for _s in range(ns):
            k = int(t[p]) - 1
            s = int(t[p + 1]) - 1
            p += 2
            for n in range(nb):
                wg[s, k, n] = float(t[p + 1])
                ekb[s, k, n] = float(t[p + 2])
                p += 4

    t = _tokens(d + "stru_out")
    lat = np.array([float(x) for x in t[0:9]]).reshape(3, 3)
    nat = int(t[18])
    pos = np.zeros((nat, 3))
    types = []
    p = 19
    for a in range(nat):
        pos[a] = [float(x) for x in t[p:p + 3]]
        types.append(int(t[p + 3]) - 1)
        p += 4

    if os.path.exists(d + "bz_sampling_out"):
        t = _tokens(d + "bz_sampling_out")
        period = (int(t[0]), int(t[1]), int(t[2]))
        nkf = int(t[3])
        p = 5
        kv = np.zeros((nkf, 3))
        ibz = np.zeros(nkf, int)
        for i in range(nkf):
            kv[i] = [float(x) for x in t[p + 5:p + 8]]
            ibz[i] = int(t[p + 9]) - 1
            p += 10
    else:
        t = _tokens(d + "stru_out")
        p = 19 + 4 * nat
        period = (int(t[p]), int(t[p + 1]), int(t[p + 2]))
        p += 3
        nkf = period[0] * period[1] * period[2]
        kv = np.array([float(x) for x in t[p:p + 3 * nkf]]).reshape(nkf, 3)
        p += 3 * nkf
        ibz = np.array([int(x) - 1 for x in t[p:p + nkf]])

    if os.path.exists(d + "basis_out"):
        t = _tokens(d + "basis_out")
        ntypes = int(t[0])
        p = 4
        mw, ma = {}, {}
        for _ in range(ntypes):
            ty = int(t[p]) - 1
            mw[ty] = int(t[p + 1])
            ma[ty] = int(t[p + 2])
            p += 3
        nao_at = [mw[types[a]] for a in range(nat)]
        nabf_at = [ma[types[a]] for a in range(nat)]
    else:
        nao_at, nabf_at = _basis_from_cs(d, nat)

    wfc = np.zeros((ns, nk, nb, nao), complex)
    for fn in sorted(glob.glob(d + "KS_eigenvector*")):
        t = _tokens(fn)
        p = 0
        while p < len(t):
            ik = int(t[p]) - 1
            p += 1
            if p >= len(t):
                break
            for iw in range(nao):
                for ib in range(nb):
                    for s in range(ns):
                        wfc[s, ik, ib, iw] = complex(float(t[p]), float(t[p + 1]))
                        p += 2

    Cs = read_cs(d, "Cs_data", cs_threshold)

    nabf_small = sinvS = Cs_small = None
    if glob.glob(d + "shrink_sinvS*"):
        # ABF shrink (use_shrink_abfs): the Coulomb matrices are given in the small basis, the
        # exchange takes the RI coefficients of that basis (Cs_shrinked_data)
        nabf_small = _basis_from_cs(d, nat, "Cs_shrinked_data")[1]
        sinvS = read_sinvS(d, "shrink_sinvS")
        Cs_small = read_cs(d, "Cs_shrinked_data", cs_threshold)
    Vq = read_coulomb(d, "coulomb_mat", nabf_small if nabf_small is not None else nabf_at)

    return RPAInput(n_spins=ns, n_kpts=nk, n_bands=nb, n_ao=nao, wg=wg, ekb=ekb, efermi=efermi,
                    wfc=wfc, latvec=lat, period=period, kvecs=kv, ibz_map=ibz,
                    nao=nao_at, nabf=nabf_at, Cs=Cs, Vq=Vq, positions=pos, nabf_small=nabf_small,
                    sinvS=sinvS, Cs_small=Cs_small)


def read_cs(d: str, prefix: str, cs_threshold: float) -> dict:
    """RI blocks {(I, J, R): (n_i n_j, n_mu)} of the Cs files with the given prefix, text or binary
    (handle_Cs_file, read_data.cpp:690-747), blocks whose max |C| is below cs_threshold dropped."""
    Cs = {}
    for fn in sorted(glob.glob(d + prefix + "*")):
        if is_text_file(fn):
            t = _tokens(fn)
            p = 2  # natom, ncell
            while p + 8 <= len(t):
                I, J, r1, r2, r3, ni, nj, nmu = (int(x) for x in t[p:p + 8])
                p += 8
                cnt = ni * nj * nmu
                m = np.array([float(x) for x in t[p:p + cnt]]).reshape(ni * nj, nmu)
                p += cnt
                if np.abs(m).max() >= cs_threshold:
                    Cs[(I - 1, J - 1, (r1, r2, r3))] = m
            continue
        raw = open(fn, "rb").read()
        natom, ncell, nblk = struct.unpack_from("<3i", raw, 0)
        off = 12
        for _ in range(nblk):
            I, J, r1, r2, r3, ni, nj, nmu = struct.unpack_from("<8i", raw, off)
            off += 32
            cnt = ni * nj * nmu
            m = np.frombuffer(raw, "<f8", cnt, off).reshape(ni * nj, nmu).copy()
            off += 8 * cnt
            if np.abs(m).max() >= cs_threshold:
                Cs[(I - 1, J - 1, (r1, r2, r3))] = m
    return Cs


def read_coulomb(d: str, prefix: str, nabf_at) -> dict:
    """V(q) upper atom blocks {(iq, I, J): (n_mu, n_nu) complex} from the binary row files."""
    d = d.rstrip("/") + "/"
    nat = len(nabf_at)
    aoff = np.concatenate([[0], np.cumsum(nabf_at)]).astype(int)
    Vq = {}

    def check(nbb):
        if nbb != aoff[-1]:
            raise ValueError(f"Coulomb matrices are {nbb} x {nbb} but the bases give {aoff[-1]} auxiliary "
                             "functions (shrunk ABF sets are not supported)")
    for fn in sorted(glob.glob(d + prefix + "*")):
        if is_text_file(fn):
            t = _tokens(fn)
            p = 1  # n_irk
            full = {}
            while p + 7 <= len(t):
                nbb, br, er, bc, ec, iq = (int(x) for x in t[p:p + 6])
                check(nbb)
                p += 7  # the q weight follows iq
                br, er, bc, ec, iq = br - 1, er - 1, bc - 1, ec - 1, iq - 1
                nr, nc = er - br + 1, ec - bc + 1
                v = np.array([float(x) for x in t[p:p + 2 * nr * nc]]).reshape(nr, nc, 2)
                p += 2 * nr * nc
                M = full.setdefault(iq, np.zeros((nbb, nbb), complex))
                M[br:er + 1, bc:ec + 1] = v[..., 0] + 1j * v[..., 1]
            for iq, M in full.items():
                for I in range(nat):
                    for J in range(I, nat):
                        Vq[(iq, I, J)] = M[aoff[I]:aoff[I + 1], aoff[J]:aoff[J + 1]].copy()
            continue
        raw = open(fn, "rb").read()
        _nirk, nloc = struct.unpack_from("<2i", raw, 0)
        off = 8
        full = {}
        for _ in range(nloc):
            nbb, br, er, bc, ec, iq = struct.unpack_from("<6i", raw, off)
            check(nbb)
            off += 24
            off += 8  # q weight
            br, er, bc, ec, iq = br - 1, er - 1, bc - 1, ec - 1, iq - 1
            nr, nc = er - br + 1, ec - bc + 1
            blk = np.frombuffer(raw, "<c16", nr * nc, off).reshape(nr, nc)
            off += 16 * nr * nc
            M = full.setdefault(iq, np.zeros((nbb, nbb), complex))
            M[br:er + 1, bc:ec + 1] = blk
        for iq, M in full.items():
            for I in range(nat):
                for J in range(I, nat):
                    Vq[(iq, I, J)] = M[aoff[I]:aoff[I + 1], aoff[J]:aoff[J + 1]].copy()
    return Vq


def read_sinvS(d: str, prefix: str) -> dict:
    """U(q) = sinvS(q) of the ABF shrink, {iq_ibz: (n_small, n_large) complex}: per IBZ q, row
    blocks [brow, erow] x [bcol, ecol] (1-based) filled row-major (handle_sinvS_file,
    read_data.cpp:2455-2568, the "for abacus" orientation: rows are the small ABFs)."""
    d = d.rstrip("/") + "/"
    U = {}
    for fn in sorted(glob.glob(d + prefix + "*")):
        if is_text_file(fn):
            t = _tokens(fn)
            p = 1  # n_irk
            while p + 8 <= len(t):
                ns_, nl, br, er, bc, ec, iq = (int(x) for x in t[p:p + 7])
                p += 8  # the q weight follows iq
                nr, nc = er - br + 1, ec - bc + 1
                v = np.array([float(x) for x in t[p:p + 2 * nr * nc]]).reshape(nr, nc, 2)
                p += 2 * nr * nc
                M = U.setdefault(iq - 1, np.zeros((ns_, nl), complex))
                M[br - 1:er, bc - 1:ec] = v[..., 0] + 1j * v[..., 1]
            continue
        raw = open(fn, "rb").read()
        _nirk, nloc = struct.unpack_from("<2i", raw, 0)
        off = 8
        for _ in range(nloc):
            ns_, nl, br, er, bc, ec, iq = struct.unpack_from("<7i", raw, off)
            off += 28 + 8  # q weight
            nr, nc = er - br + 1, ec - bc + 1
            blk = np.frombuffer(raw, "<c16", nr * nc, off).reshape(nr, nc)
            off += 16 * nr * nc
            M = U.setdefault(iq - 1, np.zeros((ns_, nl), complex))
            M[br - 1:er, bc - 1:ec] = blk
    return U


def read_vxc(path: str) -> np.ndarray:
    """<psi_n|v_xc|psi_n> in Hartree, shape (n_spins, n_kpts, n_states) (read_data.cpp:142-182:
    header n_kpts n_spins n_states, then per k and spin one "Ha eV" pair per state)."""
    t = _tokens(path)
    nk, ns, nst = int(t[0]), int(t[1]), int(t[2])
    out = np.zeros((ns, nk, nst))
    p = 3
    for k in range(nk):
        for s in range(ns):
            for i in range(nst):
                out[s, k, i] = float(t[p])
                p += 2
    return out
