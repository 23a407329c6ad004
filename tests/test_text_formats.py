"""Text (ABACUS-style) RI coefficient and Coulomb files, in the reference's text layouts
(driver/read_data.cpp:618-688 and :1580-1650), read by the oracle's reader and the task = rpa
driver: a text copy of the periodic BCC He dataset, without basis_out (the sizes then come from
the RI blocks, as read_basis_from_Cs does), gives the binary original's inputs (no GPU) and its
E_c (GPU).  A Coulomb matrix whose size differs from the auxiliary basis is refused."""
import re
import struct
import subprocess
import tarfile
from pathlib import Path

import numpy as np
import pytest

from oracle.aims_dataset import read_coulomb, read_dataset

ROOT = Path(__file__).resolve().parent.parent
HE = ROOT / "tests" / "golden" / "he_bcc_dataset.tar.gz"


def _to_text(d: Path):
    """Rewrite Cs_data_* and coulomb_*_* of dataset directory d from binary to text, in place."""
    for fn in sorted(d.glob("Cs_data*")):
        raw = fn.read_bytes()
        natom, ncell, nblk = struct.unpack_from("<3i", raw, 0)
        off, lines = 12, [f"{natom}   {ncell}"]
        for _ in range(nblk):
            v = struct.unpack_from("<8i", raw, off)
            off += 32
            cnt = v[5] * v[6] * v[7]
            vals = np.frombuffer(raw, "<f8", cnt, off)
            off += 8 * cnt
            lines.append(" ".join(str(x) for x in v[:6]))
            lines.append(f"{v[6]}   {v[7]}")
            lines += [f"{x:.17e}" for x in vals]
        fn.write_text("\n".join(lines) + "\n")
    for fn in sorted(list(d.glob("coulomb_mat*")) + list(d.glob("coulomb_cut*"))):
        raw = fn.read_bytes()
        nirk, nloc = struct.unpack_from("<2i", raw, 0)
        off, lines = 8, [str(nirk)]
        for _ in range(nloc):
            nbb, br, er, bc, ec, iq = struct.unpack_from("<6i", raw, off)
            (w,) = struct.unpack_from("<d", raw, off + 24)
            off += 32
            n = (er - br + 1) * (ec - bc + 1)
            vals = np.frombuffer(raw, "<c16", n, off)
            off += 16 * n
            lines.append(f"{nbb} {br} {er} {bc} {ec}")
            lines.append(f"{iq} {w!r}")
            lines += [f"{z.real:.17e} {z.imag:.17e}" for z in vals]
        fn.write_text("\n".join(lines) + "\n")


@pytest.fixture()
def he_dirs(tmp_path):
    out = []
    for name in ("bin", "txt"):
        with tarfile.open(HE) as tf:
            tf.extractall(tmp_path / name, filter="data")
        out.append(next((tmp_path / name).rglob("band_out")).parent)
    _to_text(out[1])
    (out[1] / "basis_out").unlink()  # as in ABACUS exports: sizes come from the RI blocks
    return out


def test_oracle_reads_text_like_binary(he_dirs):
    b, t = he_dirs
    ib, it = read_dataset(str(b)), read_dataset(str(t))
    assert sorted(ib.Cs) == sorted(it.Cs) and len(ib.Cs) > 0
    for k in ib.Cs:
        np.testing.assert_array_equal(ib.Cs[k], it.Cs[k])
    assert sorted(ib.Vq) == sorted(it.Vq)
    for k in ib.Vq:
        np.testing.assert_array_equal(ib.Vq[k], it.Vq[k])
    cb, ct = read_coulomb(str(b), "coulomb_cut", ib.nabf), read_coulomb(str(t), "coulomb_cut", ib.nabf)
    for k in cb:
        np.testing.assert_array_equal(cb[k], ct[k])


def _driver(lib):
    from librpa_gb300.build import DRIVER
    assert DRIVER.exists(), "driver not built"
    return str(DRIVER)


def _run(lib, d: Path, extra=""):
    (d.parent / "librpa.in").write_text(f"task = rpa\ninput_dir = {d}\nnfreq = 16\nparallel_routing = libri\n{extra}")
    return subprocess.run([_driver(lib)], cwd=d.parent, capture_output=True, text=True, timeout=600)


def test_driver_parses_text_files_without_gpu(he_dirs, lib):
    if lib.librpa_gb300_device_count() > 0:
        pytest.skip("a GPU is visible: the GPU test covers the full run")
    r = _run(lib, he_dirs[1])
    assert r.returncode == 1
    assert "CUDA" in r.stderr or "device" in r.stderr, r.stderr


@pytest.mark.gpu
def test_driver_text_and_binary_give_one_ec(he_dirs, lib):
    extra = "gb300_chi0_precision = fp64\ngb300_ec_path = lu\n"
    ec = []
    for d in he_dirs:
        r = _run(lib, d, extra)
        assert r.returncode == 0, r.stderr
        ec.append(float(re.search(r"\| Total EcRPA:\s*([-0-9.eE+]+)", r.stdout).group(1)))
    assert abs(ec[0] - ec[1]) <= 1e-12, ec


def test_coulomb_size_mismatch_is_refused(he_dirs):
    b, _t = he_dirs
    with pytest.raises(ValueError, match="auxiliary"):
        read_coulomb(str(b), "coulomb_mat", [13, 12])


def test_driver_reads_the_abf_shrink_without_gpu(lib, tmp_path):
    """use_shrink_abfs = t on the ABACUS BN shrink dataset: the driver reads the small basis from
    Cs_shrinked_data, U(q) from shrink_sinvS and the 34 x 34 Coulomb matrix, then stops at the
    missing GPU (without use_shrink_abfs the Coulomb size is refused with a hint)."""
    if lib.librpa_gb300_device_count() > 0:
        pytest.skip("a GPU is visible: the GPU test covers the full run")
    from conftest import bn_shrink_dir
    d = bn_shrink_dir()
    r = _run(lib, d, "use_shrink_abfs = t\n")
    assert r.returncode == 1 and ("CUDA" in r.stderr or "device" in r.stderr), r.stderr
    r = _run(lib, d)
    assert r.returncode == 1 and "use_shrink_abfs = t" in r.stderr, r.stderr


@pytest.mark.gpu
def test_driver_abf_shrink_gives_the_library_ec(lib):
    """The driver on the BN shrink dataset prints the E_c the library gives through its C API
    for the same inputs (FP64 chi0, LU form)."""
    import librpa_gb300 as L
    from conftest import bn_shrink_dir, load_bn_shrink
    d = bn_shrink_dir()
    r = _run(lib, d, "use_shrink_abfs = t\ngb300_chi0_precision = fp64\ngb300_ec_path = lu\n")
    assert r.returncode == 0, r.stderr
    ec = float(re.search(r"\| Total EcRPA:\s*([-0-9.eE+]+)", r.stdout).group(1))
    s = load_bn_shrink()
    h = L.Handler()
    L.load_system(h, s)
    h.set_gb300_options(L.gb300_options(chi0_precision=L.CHI0_FP64, ec_path=L.EC_LU_FP64))
    ref, _ = h.get_rpa_correlation_energy(L.Options(nfreq=16, tfgrids_type=L.Minimax, parallel_routing=L.LIBRI,
                                                    use_shrink_abfs=1), L.n_ibz(s))
    assert abs(ec - ref) <= 1e-8, (ec, ref)
