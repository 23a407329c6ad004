"""Generate the golden fixtures of tests/golden/ from the LibRPA reference tree.

Run where a LibRPA source tree is available, naming it by argument or by the environment
variable LIBRPA_REFERENCE:
    python tests/golden/make_fixtures.py /path/to/reference [fixture ...]

Produces (all committed, so the tests need no reference tree at run time):
  h2o_libri.npz      inputs of the H2O regression dataset
                     (regression_tests/testcases/rpa_aims_mole_H2O_libri/dataset.tar.gz),
                     read with the driver's formats and cs_threshold 1e-6, plus the
                     reference E_c printed in refs/rpa_aims_mole_H2O_libri/librpa/librpa_omp1_np4.out
  minimax_ref.json   grids printed by the reference run (16 points, H2O window):
                     omega/tau nodes and weights (16 digits), cosine/sine t->f and cosine
                     f->t matrices (6 significant digits); the 6-point omega nodes/weights
                     asserted in src/test/test_timefreq.cpp (check_minimax_ng6_HF_123); the
                     32-point grids of the H2 G0W0 run (nodes, weights, t->f matrices)
  he_bcc_gamma.json  the BCC He known-answer test of src/test/test_meanfield.cpp
                     (eigenpairs, Fermi level, expected density matrix and G(tau -> 0-))
  h2o_dataset.tar.gz the H2O regression dataset itself (the reference's FHI-aims export, copied
                     unchanged), for the task = rpa driver test
  h2o_g0w0.npz       inputs of the H2O G0W0 regression dataset
                     (regression_tests/testcases/g0w0_aims_mole_H2O_libri/dataset.tar.gz) that
                     h2o_libri.npz lacks: the Coulomb matrix of the dielectric function
                     (coulomb_mat, upper atom blocks) and <psi_n|v_xc|psi_n> (vxc_out); its
                     Cs, eigenpairs and truncated Coulomb (coulomb_cut) are checked to equal
                     h2o_libri.npz's.  Plus the quasi-particle table printed by the reference run
                     (refs/g0w0_aims_mole_H2O_libri/librpa/librpa.out: state, occ, e_mf, v_xc,
                     v_exx, ReSigc, ImSigc, e_qp in eV) and its librpa.in settings.

  li_g0w0.npz        the spin-polarised Li atom G0W0 regression case
                     (regression_tests/testcases/g0w0_aims_Li_atom_libri/dataset.tar.gz):
                     all of its inputs in the h2o_libri.npz layout, its truncated Coulomb and
                     v_xc, and both spin channels' quasi-particle tables
                     (refs/g0w0_aims_Li_atom_libri/librpa/librpa.out)

  he_bcc_dataset.tar.gz  the BCC He dataset itself (copied unchanged), for the driver's periodic test
  li_dataset.tar.gz  the spin-polarised Li atom dataset itself (copied unchanged), for the driver
  mgo_g0w0.npz       the MgO G0W0 case (3x3x3 k-points, 14 IBZ points; bare and truncated Coulomb,
                     v_xc, eps_mac of dielecfunc_out) and its 27 quasi-particle tables
                     (refs/g0w0_aims_MgO_libri/librpa/librpa.out)
  he_exx.npz         the periodic BCC He exchange case (2-atom cubic cell, 2x2x2 k-points;
                     regression_tests/testcases/exx_aims_bccHe_k_parallel_libri/dataset.tar.gz):
                     its inputs (bare Coulomb V(q) included, for RPA runs on real periodic
                     FHI-aims data), truncated Coulomb V(q) and the v_exx tables of every k-point
                     printed by the reference run (refs/exx_aims_bccHe_k_parallel_libri/librpa/
                     librpa.out, Hartree and eV; the suite checks the first to 1e-4)

  h2o_g0w0_dataset.tar.gz  the H2O G0W0 regression dataset itself (copied unchanged), for the
                     driver's task = g0w0 test
  bn_shrink_dataset.tar.gz  the ABACUS BN case with an ABF shrink (2 atoms, 2x2x2 k; 60 + 59
                     ABFs, shrunk to 17 + 17) copied unchanged
                     (regression_tests/testcases/g0w0_band_abacus_BN_shrink_libri/input_librpa.tar.gz):
                     Cs of the large basis, Coulomb matrix of the small one, shrink_sinvS, and the
                     Cs_shrinked_data (the RI coefficients of the small basis); the reference prints
                     no E_c for it
  bn_shrink_g0w0.npz the quasi-particle tables of the same case's G0W0 run on its 2x2x2 k-grid
                     (refs/g0w0_band_abacus_BN_shrink_libri/librpa.out: 8 k-points x 26 states, eV;
                     16 minimax points, 16 Pade parameters, sqrt_coulomb_threshold 1e-8 from its
                     librpa.in; the suite checks the first table to 1e-4 eV)

Fixtures can be regenerated one at a time: make_fixtures.py <reference> [h2o|minimax|he_bcc|
h2o_dataset|he_dataset|li_dataset|g0w0|li_g0w0|he_exx|mgo_g0w0|bn_shrink|h2o_g0w0_dataset ...].
"""
from __future__ import annotations

import json
import re
import os
import sys
import tarfile
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle.aims_dataset import read_coulomb, read_dataset, read_vxc  # noqa: E402


def _floats(s):
    return [float(x) for x in re.findall(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?", s)]


def h2o(ref: Path):
    tgz = ref / "regression_tests/testcases/rpa_aims_mole_H2O_libri/dataset.tar.gz"
    log = (ref / "regression_tests/refs/rpa_aims_mole_H2O_libri/librpa/librpa_omp1_np4.out").read_text()
    ec = float(re.search(r"Total EcRPA:\s*([-0-9.Ee+]+)", log).group(1))
    with tempfile.TemporaryDirectory() as td:
        with tarfile.open(tgz) as tf:
            tf.extractall(td, filter="data")
        d = next(Path(td).rglob("band_out")).parent
        inp = read_dataset(str(d))
    keys = sorted(inp.Cs)
    cs_meta = np.array([[I, J, *R] for (I, J, R) in keys], np.int32)
    cs_data = np.concatenate([inp.Cs[k].ravel() for k in keys])
    vkeys = sorted(inp.Vq)
    vq_meta = np.array(vkeys, np.int32)
    vq_data = np.concatenate([inp.Vq[k].ravel() for k in vkeys])
    np.savez_compressed(
        HERE / "h2o_libri.npz",
        n_spins=inp.n_spins, n_kpts=inp.n_kpts, n_bands=inp.n_bands, n_ao=inp.n_ao,
        wg=inp.wg, ekb=inp.ekb, efermi=inp.efermi, wfc=inp.wfc, latvec=inp.latvec,
        period=np.array(inp.period), kvecs=inp.kvecs, ibz_map=inp.ibz_map,
        nao=np.array(inp.nao), nabf=np.array(inp.nabf), positions=inp.positions,
        cs_meta=cs_meta, cs_data=cs_data, vq_meta=vq_meta, vq_data=vq_data,
        ec_reference=ec, nfreq=16)
    print("h2o_libri.npz: E_c reference", ec)


def minimax(ref: Path):
    log = (ref / "regression_tests/refs/rpa_aims_mole_H2O/librpa/librpa_omp1_np4.out").read_text().splitlines()

    def table(start_pat, n=16):
        i = next(k for k, l in enumerate(log) if start_pat in l)
        rows = [_floats(log[i + 1 + r]) for r in range(n)]
        return [r[1] for r in rows], [r[2] for r in rows], i + 1 + n

    om, omw, end = table("Frequency node & weight")
    tau, tauw, end = table("Time node & weight")

    def matrix(after, title, n=16):
        i = next(k for k in range(after, len(log)) if title in log[k])
        i += 2  # skip "nr = 16, nc = 16"
        return [_floats(log[i + r]) for r in range(n)], i + n

    cos_t2f, e1 = matrix(end, "Cosine transform matrix")
    sin_t2f, e2 = matrix(e1, "Sine transform matrix")
    cos_f2t, _ = matrix(e2, "Cosine transform matrix")
    band = {}
    # The H2O window comes from the dataset (gap, band width); record it from the same band_out.
    tf = (ref / "src/test/test_timefreq.cpp").read_text()
    body = tf[tf.index("void check_minimax_ng6_HF_123"):]
    emin = float(re.search(r"emin\s*=\s*([0-9.eE+-]+)", body).group(1))
    emax = float(re.search(r"emax\s*=\s*([0-9.eE+-]+)", body).group(1))
    fn = _floats(re.search(r"freq_node\s*=\s*\{([^}]*)\}", body).group(1))
    fw = _floats(re.search(r"freq_weight\s*=\s*\{([^}]*)\}", body).group(1))
    out = {
        "h2o16": {"omega": om, "omega_w": omw, "tau": tau, "tau_w": tauw,
                  "cos_t2f": cos_t2f, "sin_t2f": sin_t2f, "cos_f2t": cos_f2t},
        "ng6_HF_123": {"emin": emin, "emax": emax, "omega": fn, "omega_w": fw, "tol": 1e-5},
        "h2_32": _minimax_h2_32(ref),
    }
    (HERE / "minimax_ref.json").write_text(json.dumps(out, indent=1))
    print("minimax_ref.json written")


def _minimax_h2_32(ref: Path):
    """32-point grids printed by the H2 G0W0 run (refs/g0w0_aims_mole_H2_libri/librpa/librpa.out)
    with the window its band_out gives (gap, band width).  The cosine f->t matrix is left out: at
    32 points its least-squares fit is singular to double precision (condition number ~7e16), so
    the printed weights are not reproducible across LAPACK builds."""
    from oracle.rpa_oracle import e_min_max
    log = (ref / "regression_tests/refs/g0w0_aims_mole_H2_libri/librpa/librpa.out").read_text().splitlines()
    n = 32

    def table(start_pat):
        i = next(k for k, l in enumerate(log) if start_pat in l)
        rows = [_floats(log[i + 1 + r]) for r in range(n)]
        return [r[1] for r in rows], [r[2] for r in rows], i + 1 + n

    om, omw, end = table("Frequency node & weight")
    tau, tauw, end = table("Time node & weight")

    def matrix(after, title):
        i = next(k for k in range(after, len(log)) if title in log[k])
        i += 2
        return [_floats(log[i + r]) for r in range(n)], i + n

    cos_t2f, e1 = matrix(end, "Cosine transform matrix")
    sin_t2f, _ = matrix(e1, "Sine transform matrix")
    tgz = ref / "regression_tests/testcases/g0w0_aims_mole_H2_libri/dataset.tar.gz"
    with tempfile.TemporaryDirectory() as td:
        with tarfile.open(tgz) as tf:
            tf.extractall(td, filter="data")
        d = next(Path(td).rglob("band_out")).parent
        gap, width = e_min_max(read_dataset(str(d)))
    return {"emin": float(gap), "emax": float(width), "omega": om, "omega_w": omw, "tau": tau, "tau_w": tauw,
            "cos_t2f": cos_t2f, "sin_t2f": sin_t2f}


def he_bcc(ref: Path):
    src = (ref / "src/test/test_meanfield.cpp").read_text()
    body = src[src.index("test_BCC_He_gamma_minimal_basis_aims"):]
    ef = float(re.search(r"get_efermi\(\)\s*=\s*([0-9.eE+-]+)", body).group(1))
    eig = _floats(re.search(r"std::vector<double> eig\s*\{([^}]*)\}", body).group(1))
    wk = _floats(re.search(r"wkc_gamma_T\s*\{([^}]*)\}", body).group(1))
    checks = []
    for m in re.finditer(r"fequal\((dmat_gamma|gf_gamma)\((\d+),\s*(\d+)\),\s*\{\s*([-0-9.eE+]+)\s*,", body):
        checks.append({"what": m.group(1), "i": int(m.group(2)), "j": int(m.group(3)), "value": float(m.group(4))})
    out = {"efermi": ef, "eig": eig, "wkc_gamma_T": wk, "n_occ_bands": 2, "occupation": 2.0,
           "tau": -1e-12, "thres": 1e-10, "checks": checks}
    (HERE / "he_bcc_gamma.json").write_text(json.dumps(out, indent=1))
    print("he_bcc_gamma.json written:", len(checks), "checks")


def h2o_dataset(ref: Path):
    import shutil
    src = ref / "regression_tests/testcases/rpa_aims_mole_H2O_libri/dataset.tar.gz"
    shutil.copyfile(src, HERE / "h2o_dataset.tar.gz")
    print("h2o_dataset.tar.gz written")


def mgo_g0w0(ref: Path):
    """The MgO G0W0 case (2 atoms, 3x3x3 k-points reduced to 14 IBZ points by time reversal; bare and
    truncated Coulomb at the IBZ points, v_xc, the macroscopic dielectric function of its head
    correction) and its 27 quasi-particle tables.  Also the only real input with an IBZ reduction,
    for RPA runs."""
    case = "g0w0_aims_MgO_libri"
    tgz = ref / f"regression_tests/testcases/{case}/dataset.tar.gz"
    log = (ref / f"regression_tests/refs/{case}/librpa/librpa.out").read_text().splitlines()
    tables = np.array(_qp_tables(log))
    with tempfile.TemporaryDirectory() as td:
        with tarfile.open(tgz) as tf:
            tf.extractall(td, filter="data")
        d = next(Path(td).rglob("band_out")).parent
        inp = read_dataset(str(d))
        cut = read_coulomb(str(d), "coulomb_cut", inp.nabf)
        vxc = read_vxc(str(d / "vxc_out"))
        # dielecfunc_out: omega, Re eps_mac, Im eps_mac; replace_w_head with option 0 copies the
        # real parts onto the minimax frequencies (read_dielec_func, interpolate_dielec_func)
        epsmac = np.array([_floats(l)[1] for l in (d / "dielecfunc_out").read_text().splitlines() if l.strip()])
    keys = sorted(inp.Cs)
    ckeys = sorted(cut)
    np.savez_compressed(
        HERE / "mgo_g0w0.npz",
        n_spins=inp.n_spins, n_kpts=inp.n_kpts, n_bands=inp.n_bands, n_ao=inp.n_ao,
        wg=inp.wg, ekb=inp.ekb, efermi=inp.efermi, wfc=inp.wfc, latvec=inp.latvec,
        period=np.array(inp.period), kvecs=inp.kvecs, ibz_map=inp.ibz_map,
        nao=np.array(inp.nao), nabf=np.array(inp.nabf), positions=inp.positions,
        cs_meta=np.array([[I, J, *R] for (I, J, R) in keys], np.int32),
        cs_data=np.concatenate([inp.Cs[k].ravel() for k in keys]),
        vq_meta=np.array(sorted(inp.Vq), np.int32),
        vq_data=np.concatenate([inp.Vq[k].ravel() for k in sorted(inp.Vq)]),
        vcut_meta=np.array(ckeys, np.int32), vcut_data=np.concatenate([cut[k].ravel() for k in ckeys]),
        vxc=vxc, epsmac=epsmac, tables=tables, nfreq=6, n_params_anacon=-1)
    print("mgo_g0w0.npz written:", tables.shape)


def li_dataset(ref: Path):
    import shutil
    src = ref / "regression_tests/testcases/g0w0_aims_Li_atom_libri/dataset.tar.gz"
    shutil.copyfile(src, HERE / "li_dataset.tar.gz")
    print("li_dataset.tar.gz written")


def he_dataset(ref: Path):
    import shutil
    src = ref / "regression_tests/testcases/exx_aims_bccHe_k_parallel_libri/dataset.tar.gz"
    shutil.copyfile(src, HERE / "he_bcc_dataset.tar.gz")
    print("he_bcc_dataset.tar.gz written")


def g0w0(ref: Path):
    tgz = ref / "regression_tests/testcases/g0w0_aims_mole_H2O_libri/dataset.tar.gz"
    rpa_tgz = ref / "regression_tests/testcases/rpa_aims_mole_H2O_libri/dataset.tar.gz"
    log = (ref / "regression_tests/refs/g0w0_aims_mole_H2O_libri/librpa/librpa.out").read_text().splitlines()
    i0 = next(k for k, l in enumerate(log) if re.match(r"State\s+occ\s+e_mf", l)) + 2
    table = []
    while i0 < len(log) and log[i0].strip():
        table.append(_floats(log[i0]))
        i0 += 1
    params = (ref / "regression_tests/testcases/g0w0_aims_mole_H2O_libri/librpa/librpa.in").read_text()
    nfreq = int(re.search(r"nfreq\s*=\s*(\d+)", params).group(1))
    n_params = int(re.search(r"n_params_anacon\s*=\s*(\d+)", params).group(1))
    with tempfile.TemporaryDirectory() as td, tempfile.TemporaryDirectory() as td2:
        with tarfile.open(tgz) as tf:
            tf.extractall(td, filter="data")
        with tarfile.open(rpa_tgz) as tf:
            tf.extractall(td2, filter="data")
        d = next(Path(td).rglob("band_out")).parent
        d2 = next(Path(td2).rglob("band_out")).parent
        inp = read_dataset(str(d))
        rpa = read_dataset(str(d2))
        cut = read_coulomb(str(d), "coulomb_cut", inp.nabf)
        vxc = read_vxc(str(d / "vxc_out"))
    # what the G0W0 run shares with the RPA fixture
    assert sorted(inp.Cs) == sorted(rpa.Cs) and all(np.array_equal(inp.Cs[k], rpa.Cs[k]) for k in inp.Cs)
    assert np.array_equal(inp.wfc, rpa.wfc) and np.array_equal(inp.ekb, rpa.ekb) and np.array_equal(inp.wg, rpa.wg)
    assert sorted(cut) == sorted(rpa.Vq) and all(np.array_equal(cut[k], rpa.Vq[k]) for k in cut)
    vkeys = sorted(inp.Vq)
    np.savez_compressed(
        HERE / "h2o_g0w0.npz",
        veps_meta=np.array(vkeys, np.int32),
        veps_data=np.concatenate([inp.Vq[k].ravel() for k in vkeys]),
        vxc=vxc, table=np.array(table), nfreq=nfreq, n_params_anacon=n_params)
    print("h2o_g0w0.npz written:", len(table), "states")


def _qp_tables(log_lines):
    """Every "State occ e_mf ..." table of a G0W0 log (one per spin channel and k-point)."""
    tables = []
    for k, l in enumerate(log_lines):
        if re.match(r"State\s+occ\s+e_mf", l):
            i, rows = k + 2, []
            while i < len(log_lines) and log_lines[i].strip():
                rows.append(_floats(log_lines[i]))
                i += 1
            tables.append(rows)
    return tables


def li_g0w0(ref: Path):
    case = "g0w0_aims_Li_atom_libri"
    tgz = ref / f"regression_tests/testcases/{case}/dataset.tar.gz"
    log = (ref / f"regression_tests/refs/{case}/librpa/librpa.out").read_text().splitlines()
    params = (ref / f"regression_tests/testcases/{case}/librpa/librpa.in").read_text()
    nfreq = int(re.search(r"nfreq\s*=\s*(\d+)", params).group(1))
    m = re.search(r"n_params_anacon\s*=\s*(-?\d+)", params)
    n_params = int(m.group(1)) if m else -1  # the option's default (src/api/options.cpp:45)
    with tempfile.TemporaryDirectory() as td:
        with tarfile.open(tgz) as tf:
            tf.extractall(td, filter="data")
        d = next(Path(td).rglob("band_out")).parent
        inp = read_dataset(str(d))
        cut = read_coulomb(str(d), "coulomb_cut", inp.nabf)
        vxc = read_vxc(str(d / "vxc_out"))
    keys = sorted(inp.Cs)
    vkeys = sorted(inp.Vq)
    ckeys = sorted(cut)
    np.savez_compressed(
        HERE / "li_g0w0.npz",
        n_spins=inp.n_spins, n_kpts=inp.n_kpts, n_bands=inp.n_bands, n_ao=inp.n_ao,
        wg=inp.wg, ekb=inp.ekb, efermi=inp.efermi, wfc=inp.wfc, latvec=inp.latvec,
        period=np.array(inp.period), kvecs=inp.kvecs, ibz_map=inp.ibz_map,
        nao=np.array(inp.nao), nabf=np.array(inp.nabf), positions=inp.positions,
        cs_meta=np.array([[I, J, *R] for (I, J, R) in keys], np.int32),
        cs_data=np.concatenate([inp.Cs[k].ravel() for k in keys]),
        vq_meta=np.array(vkeys, np.int32), vq_data=np.concatenate([inp.Vq[k].ravel() for k in vkeys]),
        vcut_meta=np.array(ckeys, np.int32), vcut_data=np.concatenate([cut[k].ravel() for k in ckeys]),
        vxc=vxc, tables=np.array(_qp_tables(log)), nfreq=nfreq, n_params_anacon=n_params)
    print("li_g0w0.npz written")


def he_exx(ref: Path):
    case = "exx_aims_bccHe_k_parallel_libri"
    tgz = ref / f"regression_tests/testcases/{case}/dataset.tar.gz"
    log = (ref / f"regression_tests/refs/{case}/librpa/librpa.out").read_text().splitlines()
    tables = []
    for k, l in enumerate(log):
        if re.match(r"Band\s+e_exx", l):
            i, rows = k + 1, []
            while i < len(log) and log[i].strip():
                rows.append(_floats(log[i]))
                i += 1
            tables.append(rows)
    with tempfile.TemporaryDirectory() as td:
        with tarfile.open(tgz) as tf:
            tf.extractall(td, filter="data")
        d = next(Path(td).rglob("band_out")).parent
        inp = read_dataset(str(d))
        cut = read_coulomb(str(d), "coulomb_cut", inp.nabf)
    keys = sorted(inp.Cs)
    ckeys = sorted(cut)
    np.savez_compressed(
        HERE / "he_exx.npz",
        n_spins=inp.n_spins, n_kpts=inp.n_kpts, n_bands=inp.n_bands, n_ao=inp.n_ao,
        wg=inp.wg, ekb=inp.ekb, efermi=inp.efermi, wfc=inp.wfc, latvec=inp.latvec,
        period=np.array(inp.period), kvecs=inp.kvecs, ibz_map=inp.ibz_map,
        nao=np.array(inp.nao), nabf=np.array(inp.nabf), positions=inp.positions,
        cs_meta=np.array([[I, J, *R] for (I, J, R) in keys], np.int32),
        cs_data=np.concatenate([inp.Cs[k].ravel() for k in keys]),
        vq_meta=np.array(sorted(inp.Vq), np.int32),
        vq_data=np.concatenate([inp.Vq[k].ravel() for k in sorted(inp.Vq)]),
        vcut_meta=np.array(ckeys, np.int32), vcut_data=np.concatenate([cut[k].ravel() for k in ckeys]),
        tables=np.array(tables), nfreq=16)
    print("he_exx.npz written:", len(tables), "k-points")


def h2o_g0w0_dataset(ref: Path):
    import shutil
    src = ref / "regression_tests/testcases/g0w0_aims_mole_H2O_libri/dataset.tar.gz"
    shutil.copyfile(src, HERE / "h2o_g0w0_dataset.tar.gz")
    print("h2o_g0w0_dataset.tar.gz written")


def bn_shrink(ref: Path):
    import shutil
    src = ref / "regression_tests/testcases/g0w0_band_abacus_BN_shrink_libri/input_librpa.tar.gz"
    shutil.copyfile(src, HERE / "bn_shrink_dataset.tar.gz")
    print("bn_shrink_dataset.tar.gz written")
    # the quasi-particle tables its G0W0 run printed on the 2x2x2 k-grid (the band path was skipped)
    log = (ref / "regression_tests/refs/g0w0_band_abacus_BN_shrink_libri/librpa.out").read_text().splitlines()
    tables = np.array(_qp_tables(log))
    assert tables.shape == (8, 26, 8), tables.shape
    np.savez_compressed(HERE / "bn_shrink_g0w0.npz", tables=tables, nfreq=16, n_params_anacon=16,
                        sqrt_coulomb_threshold=1e-8)
    print("bn_shrink_g0w0.npz written")


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LIBRPA_REFERENCE")
    if not src:
        sys.exit("usage: make_fixtures.py /path/to/reference [fixture ...] (or set LIBRPA_REFERENCE)")
    ref = Path(src)
    which = sys.argv[2:] or ["h2o", "h2o_dataset", "he_dataset", "li_dataset", "minimax", "he_bcc", "g0w0",
                             "li_g0w0", "he_exx", "mgo_g0w0", "bn_shrink", "h2o_g0w0_dataset"]
    for name in which:
        {"h2o": h2o, "h2o_dataset": h2o_dataset, "minimax": minimax, "he_bcc": he_bcc, "g0w0": g0w0,
         "li_g0w0": li_g0w0, "he_exx": he_exx, "he_dataset": he_dataset, "li_dataset": li_dataset,
         "mgo_g0w0": mgo_g0w0, "bn_shrink": bn_shrink,
         "h2o_g0w0_dataset": h2o_g0w0_dataset}[name](ref)
