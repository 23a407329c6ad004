"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import json
import sys
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def lib():
    """The in-tree C-ABI library, built on demand."""
    from librpa_gb300.build import build
    import librpa_gb300 as L
    build()
    return L.load_library()


def _blocks(meta, data, nabf):
    out, off = {}, 0
    for ik, I, J in meta:
        n = nabf[I] * nabf[J]
        out[(int(ik), int(I), int(J))] = data[off:off + n].reshape(nabf[I], nabf[J])
        off += n
    return out


def load_h2o(fixture="h2o_libri.npz"):
    """Regression dataset inputs (golden fixture made by tests/golden/make_fixtures.py)."""
    z = np.load(GOLDEN / fixture)
    Cs = {}
    off = 0
    nao = [int(x) for x in z["nao"]]
    nabf = [int(x) for x in z["nabf"]]
    for I, J, r1, r2, r3 in z["cs_meta"]:
        n = nao[I] * nao[J] * nabf[I]
        Cs[(int(I), int(J), (int(r1), int(r2), int(r3)))] = z["cs_data"][off:off + n].reshape(nao[I] * nao[J], nabf[I])
        off += n
    Vq = {}
    off = 0
    for ik, I, J in z["vq_meta"]:
        n = nabf[I] * nabf[J]
        Vq[(int(ik), int(I), int(J))] = z["vq_data"][off:off + n].reshape(nabf[I], nabf[J])
        off += n
    return SimpleNamespace(
        name="h2o", n_spins=int(z["n_spins"]), n_kpts=int(z["n_kpts"]), n_bands=int(z["n_bands"]),
        n_ao=int(z["n_ao"]), wg=z["wg"], ekb=z["ekb"], efermi=float(z["efermi"]), wfc=z["wfc"],
        latvec=z["latvec"], period=tuple(int(x) for x in z["period"]), kvecs=z["kvecs"],
        ibz_map=z["ibz_map"], nao=nao, nabf=nabf, positions=z["positions"], types=np.zeros(len(nao), int),
        Cs=Cs, Vq=Vq, nfreq=int(z["nfreq"]),
        ec_reference=float(z["ec_reference"]) if "ec_reference" in z else None,
        minimax_emin=-1.0, minimax_emax=-1.0)


def load_li_g0w0():
    """The spin-polarised Li atom G0W0 regression case: inputs, truncated Coulomb, v_xc and the
    reference quasi-particle tables (one per spin)."""
    s = load_h2o("li_g0w0.npz")
    z = np.load(GOLDEN / "li_g0w0.npz")
    s.name = "li"
    s.v_cut = _blocks(z["vcut_meta"], z["vcut_data"], s.nabf)
    s.vxc = z["vxc"]
    s.qp_tables = z["tables"]
    s.n_params_anacon = int(z["n_params_anacon"])
    return s


def load_h2o_g0w0():
    """H2O G0W0 regression inputs: the RPA fixture (its Coulomb matrix is the run's truncated
    Coulomb) plus the dielectric Coulomb matrix, v_xc and the reference quasi-particle table."""
    s = load_h2o()
    z = np.load(GOLDEN / "h2o_g0w0.npz")
    s.v_cut = s.Vq
    s.Vq = _blocks(z["veps_meta"], z["veps_data"], s.nabf)
    s.vxc = z["vxc"]
    s.qp_table = z["table"]
    s.nfreq = int(z["nfreq"])
    s.n_params_anacon = int(z["n_params_anacon"])
    return s


def load_he_exx():
    """The periodic BCC He exchange case: inputs, truncated Coulomb V(q) and the reference
    v_exx tables (per k-point: band, Hartree, eV)."""
    s = load_h2o("he_exx.npz")
    z = np.load(GOLDEN / "he_exx.npz")
    s.name = "he_exx"
    s.v_cut = _blocks(z["vcut_meta"], z["vcut_data"], s.nabf)
    s.exx_tables = z["tables"]
    return s


def load_mgo():
    """MgO G0W0 case (3x3x3 k-points, 14 IBZ points): inputs, truncated Coulomb, v_xc, eps_mac
    at the minimax frequencies and the reference quasi-particle tables ([k][state][column], eV)."""
    s = load_h2o("mgo_g0w0.npz")
    z = np.load(GOLDEN / "mgo_g0w0.npz")
    s.name = "mgo"
    s.v_cut = _blocks(z["vcut_meta"], z["vcut_data"], s.nabf)
    s.vxc = z["vxc"]
    s.epsmac = z["epsmac"]
    s.qp_tables = z["tables"]
    s.n_params_anacon = int(z["n_params_anacon"])
    return s


_BN_DIR = None


def bn_shrink_dir():
    """The BN shrink dataset (tests/golden/bn_shrink_dataset.tar.gz) extracted once per session."""
    global _BN_DIR
    if _BN_DIR is None:
        import atexit
        import shutil
        import tarfile
        import tempfile
        td = tempfile.mkdtemp(prefix="bn_shrink_")
        atexit.register(shutil.rmtree, td, True)
        with tarfile.open(GOLDEN / "bn_shrink_dataset.tar.gz") as tf:
            tf.extractall(td, filter="data")
        _BN_DIR = next(Path(td).rglob("band_out")).parent
    return _BN_DIR


_BN_INPUT = None


def load_bn_shrink():
    """The ABACUS BN case with an ABF shrink, read as the reference's driver reads it: Cs in the
    large ABF basis (60 + 59), the Coulomb matrix in the small basis (17 + 17) and U(q) = sinvS(q)
    per IBZ point.  The text files are parsed once per session; each call returns a fresh record
    (the arrays are shared: tests must not change them in place)."""
    global _BN_INPUT
    from oracle.aims_dataset import read_dataset
    if _BN_INPUT is None:
        _BN_INPUT = read_dataset(str(bn_shrink_dir()))
    inp = _BN_INPUT
    return SimpleNamespace(**{k: getattr(inp, k) for k in inp.__dataclass_fields__}, name="bn_shrink",
                           types=np.zeros(len(inp.nao), int), nfreq=16, minimax_emin=-1.0, minimax_emax=-1.0)


def load_bn_shrink_g0w0():
    """The BN shrink case as its G0W0 run reads it: load_bn_shrink plus the truncated Coulomb
    matrix and v_xc (small basis / Hartree) and the reference's quasi-particle tables
    ([k][state][column], eV)."""
    from oracle.aims_dataset import read_coulomb, read_vxc
    s = load_bn_shrink()
    d = str(bn_shrink_dir()).rstrip("/") + "/"
    z = np.load(GOLDEN / "bn_shrink_g0w0.npz")
    s.name = "bn_shrink_g0w0"
    s.v_cut = read_coulomb(d, "coulomb_cut", s.nabf_small)
    s.vxc = read_vxc(d + "vxc_out")
    s.qp_tables = z["tables"]
    s.nfreq = int(z["nfreq"])
    s.n_params_anacon = int(z["n_params_anacon"])
    s.sqrt_coulomb_threshold = float(z["sqrt_coulomb_threshold"])
    return s


def shrunk_copy(s, nabf_small, seed=5, unitary=False):
    """s with an ABF shrink added: per IBZ point a U(q) of orthonormal rows (a complex unitary
    when unitary=True and the sizes agree; real at the Gamma point) and the Coulomb matrix taken to
    the small basis as U V U^H.  With a unitary U, E_c is that of s itself."""
    import copy
    from oracle.rpa_oracle import assemble_full
    rng = np.random.default_rng(seed)
    t = copy.copy(s)
    nl, ns_ = int(sum(s.nabf)), int(sum(nabf_small))
    assert ns_ <= nl and (not unitary or ns_ == nl)
    gamma = s.n_kpts == 1
    reps = list(dict.fromkeys(int(x) for x in s.ibz_map))
    offs = np.concatenate([[0], np.cumsum(nabf_small)]).astype(int)
    na = len(s.nabf)
    t.nabf_small, t.sinvS, t.Vq = list(nabf_small), {}, {}
    for iq, ik in enumerate(reps):
        A = rng.standard_normal((nl, nl)) + (0 if gamma else 1j * rng.standard_normal((nl, nl)))
        Q, _ = np.linalg.qr(A)
        U = Q[:ns_].conj() if not gamma else Q[:ns_].real.copy()
        t.sinvS[iq] = U
        V = U @ assemble_full({(I, J): v for (k, I, J), v in s.Vq.items() if k == ik}, s.nabf) @ U.conj().T
        for I in range(na):
            for J in range(I, na):
                t.Vq[(ik, I, J)] = V[offs[I]:offs[I + 1], offs[J]:offs[J + 1]].copy()
    return t


def minimax_ref():
    return json.loads((GOLDEN / "minimax_ref.json").read_text())


def he_ref():
    return json.loads((GOLDEN / "he_bcc_gamma.json").read_text())


def oracle_input(s):
    from oracle.rpa_oracle import RPAInput
    return RPAInput(n_spins=s.n_spins, n_kpts=s.n_kpts, n_bands=s.n_bands, n_ao=s.n_ao, wg=s.wg, ekb=s.ekb,
                    efermi=s.efermi, wfc=s.wfc, latvec=s.latvec, period=s.period, kvecs=s.kvecs,
                    ibz_map=s.ibz_map, nao=s.nao, nabf=s.nabf, Cs=s.Cs, Vq=s.Vq, positions=s.positions,
                    nabf_small=getattr(s, "nabf_small", None), sinvS=getattr(s, "sinvS", None),
                    Cs_small=getattr(s, "Cs_small", None))
