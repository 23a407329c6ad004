"""The task = rpa driver (librpa_gb300/chi0_main, the counterpart of the reference's
chi0_main task=rpa) on the H2O regression dataset of the reference (tests/golden)."""
import re
import subprocess
import tarfile
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
DATASET = ROOT / "tests" / "golden" / "h2o_dataset.tar.gz"
EC_REF = -0.306258510  # refs/rpa_aims_mole_H2O_libri/librpa/librpa_omp1_np4.out:273


HE_DATASET = ROOT / "tests" / "golden" / "he_bcc_dataset.tar.gz"
LI_DATASET = ROOT / "tests" / "golden" / "li_dataset.tar.gz"


def _prepare(tmp_path, extra="", dataset=DATASET):
    with tarfile.open(dataset) as tf:
        tf.extractall(tmp_path, filter="data")
    data = next(tmp_path.rglob("band_out")).parent
    (tmp_path / "librpa.in").write_text(f"# driver parameters\ntask = rpa\ninput_dir = {data}\nnfreq = 16\n"
                                        f"parallel_routing = libri\n{extra}")
    return tmp_path


def _driver(lib):
    from librpa_gb300.build import DRIVER
    assert DRIVER.exists(), "driver not built"
    return str(DRIVER)


def test_driver_reads_dataset_without_gpu(tmp_path, lib):
    """Everything up to the GPU call: on a machine without a GPU the driver reads all files and
    then reports the missing device (not a parse error)."""
    if lib.librpa_gb300_device_count() > 0:
        pytest.skip("a GPU is visible: the GPU test covers the full run")
    d = _prepare(tmp_path)
    r = subprocess.run([_driver(lib)], cwd=d, capture_output=True, text=True, timeout=120)
    assert r.returncode == 1
    assert "CUDA" in r.stderr or "device" in r.stderr, r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("extra,tol", [("gb300_chi0_precision = fp64\ngb300_ec_path = lu\n", 2e-9),
                                       ("", 3 * 3.674932e-6)])
def test_driver_h2o_regression(tmp_path, lib, extra, tol):
    d = _prepare(tmp_path, extra)
    r = subprocess.run([_driver(lib)], cwd=d, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "RPA correlation energy (Hartree)" in r.stdout
    ec = float(re.search(r"\| Total EcRPA:\s*([-0-9.eE+]+)", r.stdout).group(1))
    assert abs(ec - EC_REF) <= max(tol, 1e-9), (ec, EC_REF)


def test_driver_reads_periodic_dataset_without_gpu(tmp_path, lib):
    """The periodic BCC He dataset (8 k-points, cells in [0, 2)) parses up to the GPU call."""
    if lib.librpa_gb300_device_count() > 0:
        pytest.skip("a GPU is visible: the GPU test covers the full run")
    d = _prepare(tmp_path, dataset=HE_DATASET)
    r = subprocess.run([_driver(lib)], cwd=d, capture_output=True, text=True, timeout=120)
    assert r.returncode == 1
    assert "CUDA" in r.stderr or "device" in r.stderr, r.stderr


@pytest.mark.gpu
def test_driver_he_bcc_periodic(tmp_path, lib):
    """task = rpa on real periodic FHI-aims files (BCC He, 2x2x2 k-points) against the oracle."""
    from conftest import load_he_exx, oracle_input
    from oracle.rpa_oracle import Options, rpa_correlation_energy
    ref = rpa_correlation_energy(oracle_input(load_he_exx()), Options(nfreq=16))["ec"].real
    d = _prepare(tmp_path, "gb300_chi0_precision = fp64\ngb300_ec_path = lu\n", dataset=HE_DATASET)
    r = subprocess.run([_driver(lib)], cwd=d, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    ec = float(re.search(r"\| Total EcRPA:\s*([-0-9.eE+]+)", r.stdout).group(1))
    assert abs(ec - ref) <= 1e-9, (ec, ref)


def test_driver_reads_spin_polarised_dataset_without_gpu(tmp_path, lib):
    """The spin-polarised Li atom dataset (two spin channels) parses up to the GPU call."""
    if lib.librpa_gb300_device_count() > 0:
        pytest.skip("a GPU is visible: the GPU test covers the full run")
    d = _prepare(tmp_path, dataset=LI_DATASET)
    r = subprocess.run([_driver(lib)], cwd=d, capture_output=True, text=True, timeout=120)
    assert r.returncode == 1
    assert "CUDA" in r.stderr or "device" in r.stderr, r.stderr


@pytest.mark.gpu
def test_driver_li_spin_polarised(tmp_path, lib):
    """task = rpa on the spin-polarised Li atom files against the oracle."""
    from conftest import load_li_g0w0, oracle_input
    from oracle.rpa_oracle import Options, rpa_correlation_energy
    ref = rpa_correlation_energy(oracle_input(load_li_g0w0()), Options(nfreq=16))["ec"].real
    d = _prepare(tmp_path, "gb300_chi0_precision = fp64\ngb300_ec_path = lu\n", dataset=LI_DATASET)
    r = subprocess.run([_driver(lib)], cwd=d, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    ec = float(re.search(r"\| Total EcRPA:\s*([-0-9.eE+]+)", r.stdout).group(1))
    assert abs(ec - ref) <= 1e-9, (ec, ref)


H2O_G0W0_DATASET = ROOT / "tests" / "golden" / "h2o_g0w0_dataset.tar.gz"


def _run_task(tmp_path, lib, task, dataset, extra=""):
    with tarfile.open(dataset) as tf:
        tf.extractall(tmp_path, filter="data")
    data = next(tmp_path.rglob("band_out")).parent
    (tmp_path / "librpa.in").write_text(f"task = {task}\ninput_dir = {data}\nparallel_routing = libri\n{extra}")
    return subprocess.run([_driver(lib)], cwd=tmp_path, capture_output=True, text=True, timeout=900)


def test_driver_exx_and_g0w0_tasks_read_without_gpu(tmp_path, lib):
    """task = exx (BCC He) and task = g0w0 (H2O) parse their extra files up to the GPU call."""
    if lib.librpa_gb300_device_count() > 0:
        pytest.skip("a GPU is visible: the GPU tests cover the full runs")
    r = _run_task(tmp_path / "exx", lib, "exx", HE_DATASET)
    assert r.returncode == 1 and ("CUDA" in r.stderr or "device" in r.stderr), r.stderr
    r = _run_task(tmp_path / "g0w0", lib, "g0w0", H2O_G0W0_DATASET, "nfreq = 16\nn_params_anacon = 16\n")
    assert r.returncode == 1 and ("CUDA" in r.stderr or "device" in r.stderr), r.stderr


@pytest.mark.gpu
def test_driver_exx_task_bcc_he(tmp_path, lib):
    """task = exx on the reference's BCC He exchange dataset: the printed v_exx tables (Band,
    e_exx in Hartree and eV, every k-point) match the reference's printed tables."""
    import numpy as np
    from conftest import load_he_exx
    r = _run_task(tmp_path, lib, "exx", HE_DATASET)
    assert r.returncode == 0, r.stderr
    rows = [[float(x) for x in l.split()] for l in r.stdout.splitlines() if re.match(r"^\s*\d+\s+-?\d+\.\d{5}\s+-?\d+\.\d{5}\s*$", l)]
    got = np.array(rows).reshape(8, 8, 3)
    np.testing.assert_allclose(got, load_he_exx().exx_tables, rtol=0, atol=1.1e-5)


@pytest.mark.gpu
def test_driver_g0w0_task_h2o(tmp_path, lib):
    """task = g0w0 on the reference's H2O G0W0 dataset with its own settings (16 minimax points,
    16 Pade parameters), FP64 chi0: the printed quasi-particle table matches the reference's."""
    import numpy as np
    from conftest import load_h2o_g0w0
    r = _run_task(tmp_path, lib, "g0w0", H2O_G0W0_DATASET,
                  "nfreq = 16\nn_params_anacon = 16\ngb300_chi0_precision = fp64\n")
    assert r.returncode == 0, r.stderr
    rows = [[float(x) for x in l.split()] for l in r.stdout.splitlines()
            if re.match(r"^\s*\d+(\s+-?\d+\.\d{5}){7}\s*$", l)]
    got = np.array(rows)
    t = load_h2o_g0w0().qp_table
    assert got.shape == t.shape, (got.shape, t.shape)
    np.testing.assert_allclose(got[:, 2:], t[:, 2:], rtol=0, atol=1.1e-5)


BN_SHRINK_DATASET = ROOT / "tests" / "golden" / "bn_shrink_dataset.tar.gz"


@pytest.mark.gpu
def test_driver_g0w0_band_task_bn_shrink(tmp_path, lib):
    """task = g0w0_band on the reference's ABACUS BN shrink dataset with its own librpa.in settings
    (16 points, use_shrink_abfs, sqrt_coulomb_threshold 1e-8; no band path file, so the k-grid
    tables only, as the reference printed them), FP64 chi0: v_xc and v_exx at print precision,
    Sigma_c within 2e-4 eV and e_qp within 4e-4 eV of the reference's tables (the bounds the oracle
    itself meets on this case)."""
    import numpy as np
    from conftest import load_bn_shrink_g0w0
    r = _run_task(tmp_path, lib, "g0w0_band", BN_SHRINK_DATASET,
                  "nfreq = 16\nn_params_anacon = 16\nuse_shrink_abfs = t\nsqrt_coulomb_threshold = 1e-8\n"
                  "gb300_chi0_precision = fp64\n")
    assert r.returncode == 0, r.stderr
    rows = [[float(x) for x in l.split()] for l in r.stdout.splitlines()
            if re.match(r"^\s*\d+(\s+-?\d+\.\d{5}){7}\s*$", l)]
    got = np.array(rows).reshape(8, 26, 8)
    t = load_bn_shrink_g0w0().qp_tables
    np.testing.assert_allclose(got[:, :, :5], t[:, :, :5], rtol=0, atol=1.1e-5)
    np.testing.assert_allclose(got[:, :, 5:7], t[:, :, 5:7], rtol=0, atol=2e-4)
    np.testing.assert_allclose(got[:, :, 7], t[:, :, 7], rtol=0, atol=4e-4)
