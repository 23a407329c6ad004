"""GB300-native space-time RPA correlation energy (LibRPA task=rpa hot path).

The product is the C-ABI shared library ``liblibrpa_gb300.so`` built in-tree
from ``csrc/`` (C++ host + hand-written sm_103a CUDA).  This module is a thin
ctypes mirror of LibRPA's C++ wrapper (include/librpa.hpp: ``librpa::Options``
and ``librpa::Handler``) so Python callers and the tests use the same names,
argument meaning and error behaviour as C/C++/Fortran callers of librpa.h.

There is no CPU fallback: if the library is missing, ``load_library`` raises,
and the compute calls report "no CUDA device visible" on a machine without a GPU.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "liblibrpa_gb300.so"

LIBRPA_MAX_STRLEN = 200
# enums (librpa_enums.h)
ROUTING_UNSET, AUTO, RTAU, ATOMPAIR, LIBRI = -101, -51, 0, 1, 2
TFGRID_UNSET, GaussLegendre, GaussChebyshevI, GaussChebyshevII, Minimax, EvenSpaced, EvenSpaced_TF = (
    -101, 0, 1, 2, 3, 4, 5)
CHI0_FP64, CHI0_BF16X3, CHI0_FP32 = 0, 1, 2
EC_LU_FP64, EC_CHOL, EC_CHOL_FP64 = 0, 1, 2
SIGMA_FP64, SIGMA_BF16X3 = 0, 1
SCREEN_OFF, SCREEN_THRESHOLD, SCREEN_MLP = 0, 1, 2
MLP_IN = 9
MLP_NPARAM, MLP_NNORM = 64 * MLP_IN + 64 + 64 * 64 + 64 + 64 + 1, 2 * MLP_IN + 3
STAGE_FULL, STAGE_CHI0, STAGE_EC = 0, 1, 2


class LibrpaOptions(C.Structure):
    """Byte-identical mirror of LibrpaOptions (librpa_options.h)."""

    _fields_ = [
        ("output_dir", C.c_char * LIBRPA_MAX_STRLEN),
        ("parallel_routing", C.c_int),
        ("output_level", C.c_int),
        ("vq_threshold", C.c_double),
        ("use_kpara_scf_eigvec", C.c_int),
        ("tfgrids_type", C.c_int),
        ("nfreq", C.c_int),
        ("tfgrids_freq_min", C.c_double),
        ("tfgrids_freq_interval", C.c_double),
        ("tfgrids_freq_max", C.c_double),
        ("tfgrids_time_min", C.c_double),
        ("tfgrids_time_interval", C.c_double),
        ("minimax_emin", C.c_double),
        ("minimax_emax", C.c_double),
        ("minimax_regulation", C.c_double),
        ("use_fullcoul_exx", C.c_int),
        ("use_fullcoul_eps", C.c_int),
        ("use_fullcoul_wc", C.c_int),
        ("n_bands_chi0", C.c_int),
        ("n_bands_sigc", C.c_int),
        ("gf_threshold", C.c_double),
        ("use_scalapack_ecrpa", C.c_int),
        ("use_shrink_abfs", C.c_int),
        ("use_shrink_chi", C.c_int),
        ("n_params_anacon", C.c_int),
        ("use_scalapack_gw_wc", C.c_int),
        ("use_cholesky_gw_wc", C.c_int),
        ("replace_w_head", C.c_int),
        ("option_dielect_func", C.c_int),
        ("use_2d_dielectric", C.c_int),
        ("load_sigc_from_file", C.c_int),
        ("sqrt_coulomb_threshold", C.c_double),
        ("libri_chi0_threshold_C", C.c_double),
        ("libri_chi0_threshold_G", C.c_double),
        ("libri_exx_threshold_C", C.c_double),
        ("libri_exx_threshold_D", C.c_double),
        ("libri_exx_threshold_V", C.c_double),
        ("libri_g0w0_threshold_C", C.c_double),
        ("libri_g0w0_threshold_G", C.c_double),
        ("libri_g0w0_threshold_Wc", C.c_double),
        ("output_gw_sigc_mat", C.c_int),
        ("output_gw_sigc_mat_rt", C.c_int),
        ("output_gw_sigc_mat_rf", C.c_int),
        ("option_output_Wc_Rf_mat", C.c_int),
    ]


class GB300Options(C.Structure):
    _fields_ = [
        ("chi0_precision", C.c_int),
        ("ec_path", C.c_int),
        ("screen_mode", C.c_int),
        ("screen_threshold", C.c_double),
        ("audit_fraction", C.c_double),
        ("seed", C.c_ulonglong),
        ("use_cuda_graph", C.c_int),
        ("keep_chi0", C.c_int),
        ("device", C.c_int),
        ("reuse_device_inputs", C.c_int), ("tau_begin", C.c_int), ("tau_end", C.c_int), ("stage", C.c_int),
        ("q_begin", C.c_int), ("q_end", C.c_int), ("sigma_precision", C.c_int),
    ]


class GB300Stats(C.Structure):
    _fields_ = [
        ("t_total", C.c_double), ("t_grids", C.c_double), ("t_upload", C.c_double), ("t_gf", C.c_double),
        ("t_chi0", C.c_double), ("t_ftct", C.c_double), ("t_ec", C.c_double),
        ("chi0_flops", C.c_double), ("chi0_flops_libri", C.c_double), ("ec_flops", C.c_double),
        ("gf_flops", C.c_double), ("ftct_bytes", C.c_double), ("n_launches", C.c_longlong),
        ("blocks_total", C.c_longlong), ("blocks_computed", C.c_longlong), ("blocks_audited", C.c_longlong),
        ("audit_max_dropped", C.c_double), ("dt_chi0_kernel_ms", C.c_double), ("n_chi0_kernel", C.c_longlong),
        ("h2d_bytes", C.c_double), ("d2h_bytes", C.c_double), ("screen_fallbacks", C.c_longlong),
        ("ec_lu_fallback_q", C.c_longlong), ("t1_narrow", C.c_int), ("t1_kparts", C.c_int),
        ("chi0_precision_used", C.c_int),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


# Every symbol the public headers declare (include/*.h); the load test checks all of them.
EXPORTS = [
    "librpa_get_build_info", "librpa_get_major_version", "librpa_get_minor_version", "librpa_get_patch_version",
    "librpa_init_global", "librpa_finalize_global", "librpa_test", "librpa_print_profile",
    "librpa_init_options", "librpa_set_output_dir", "librpa_create_handler", "librpa_destroy_handler",
    "librpa_set_scf_dimension", "librpa_set_wg_ekb_efermi", "librpa_set_wfc", "librpa_set_wfc_spinor",
    "librpa_set_wfc_packed", "librpa_set_wfc_spinor_packed", "librpa_set_ao_basis_wfc", "librpa_set_ao_basis_aux",
    "librpa_set_latvec_and_G", "librpa_set_atoms", "librpa_set_kgrids_kvec", "librpa_set_ibz_mapping",
    "librpa_set_lri_coeff", "librpa_set_aux_bare_coulomb_k_atom_pair", "librpa_set_aux_cut_coulomb_k_atom_pair",
    "librpa_set_aux_bare_coulomb_k_2d_block", "librpa_set_aux_cut_coulomb_k_2d_block",
    "librpa_set_dielect_func_imagfreq", "librpa_set_band_kvec", "librpa_set_band_occ_eigval",
    "librpa_set_wfc_band", "librpa_set_wfc_band_spinor", "librpa_set_wfc_band_packed",
    "librpa_set_wfc_band_spinor_packed", "librpa_reset_band_data",
    "librpa_get_imaginary_frequency_grids", "librpa_get_rpa_correlation_energy",
    "librpa_build_exx", "librpa_get_exx_pot_kgrid", "librpa_get_exx_pot_band_k", "librpa_build_g0w0_sigma",
    "librpa_get_g0w0_sigc_kgrid", "librpa_get_g0w0_sigc_band_k",
    "librpa_gb300_init_options", "librpa_gb300_set_options", "librpa_gb300_get_stats",
    "librpa_get_last_error", "librpa_get_last_error_code", "librpa_gb300_minimax_grid",
    "librpa_gb300_get_chi0_block", "librpa_gb300_device_count", "librpa_gb300_selftest_tc_gemm",
    "librpa_gb300_tc_gemm_noalloc", "librpa_gb300_train_screening", "librpa_gb300_screening_samples",
    "librpa_gb300_get_screening_samples", "librpa_gb300_add_screening_samples", "librpa_gb300_get_screening_model",
    "librpa_gb300_clear_grid_cache", "librpa_gb300_get_g0w0_sigc_iw", "librpa_gb300_get_g0w0_sigc_iw_k", "librpa_gb300_get_rpa_correlation_energy_batch",
    "librpa_gb300_set_shrink_basis", "librpa_gb300_set_shrink_sinvS", "librpa_gb300_set_shrink_lri_coeff",
    "librpa_gb300_set_screening_model",
    "librpa_gb300_clear_screening", "librpa_gb300_mlp_loss_grad", "librpa_gb300_chi0_qw_elems",
    "librpa_gb300_copy_chi0_qw", "librpa_gb300_load_chi0_qw", "librpa_gb300_selftest_chol_ozaki",
    "librpa_gb300_solve_qpe", "librpa_gb300_phase_tables", "librpa_gb300_interpolate_dielec_func",
]

_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def load_library(path: str | Path | None = None):
    """Load the in-tree shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    vp = C.c_void_p
    d, i = C.c_double, C.c_int
    sig = {
        "librpa_get_build_info": (C.c_char_p, []),
        "librpa_get_major_version": (i, []),
        "librpa_init_options": (None, [C.POINTER(LibrpaOptions)]),
        "librpa_set_output_dir": (None, [C.POINTER(LibrpaOptions), C.c_char_p]),
        "librpa_create_handler": (vp, [i]),
        "librpa_destroy_handler": (None, [vp]),
        "librpa_set_scf_dimension": (None, [vp, i, i, i, i, i]),
        "librpa_set_wg_ekb_efermi": (None, [vp, i, i, i, _dp, _dp, d]),
        "librpa_set_wfc": (None, [vp, i, i, i, i, _dp, _dp]),
        "librpa_set_wfc_packed": (None, [vp, i, i, i, i, _dp]),
        "librpa_set_ao_basis_wfc": (None, [vp, i, np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")]),
        "librpa_set_ao_basis_aux": (None, [vp, i, np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")]),
        "librpa_set_latvec_and_G": (None, [vp, _dp, _dp]),
        "librpa_set_atoms": (None, [vp, i, _ip, _dp]),
        "librpa_set_kgrids_kvec": (None, [vp, i, i, i, _dp]),
        "librpa_set_ibz_mapping": (None, [vp, i, _ip]),
        "librpa_set_lri_coeff": (None, [vp, i, i, i, i, i, i, _ip, _dp]),
        "librpa_set_aux_bare_coulomb_k_atom_pair": (None, [vp, i, i, i, i, i, _dp, _dp, d]),
        "librpa_set_aux_bare_coulomb_k_2d_block": (None, [vp, i, i, i, i, i, _dp, _dp]),
        "librpa_set_dielect_func_imagfreq": (None, [vp, i, _dp, _dp]),
        "librpa_set_band_kvec": (None, [vp, i, _dp]),
        "librpa_set_band_occ_eigval": (None, [vp, i, i, i, _dp, _dp]),
        "librpa_set_wfc_band": (None, [vp, i, i, i, i, _dp, _dp]),
        "librpa_reset_band_data": (None, [vp]),
        "librpa_get_exx_pot_band_k": (None, [vp, C.POINTER(LibrpaOptions), i, i, _ip, i, i, _dp]),
        "librpa_get_g0w0_sigc_band_k": (None, [vp, C.POINTER(LibrpaOptions), i, i, _ip, i, i, _dp, _dp, _dp, _dp]),
        "librpa_get_imaginary_frequency_grids": (None, [vp, C.POINTER(LibrpaOptions), _dp, _dp]),
        "librpa_get_rpa_correlation_energy": (d, [vp, C.POINTER(LibrpaOptions), i, _dp, _dp]),
        "librpa_build_exx": (None, [vp, C.POINTER(LibrpaOptions)]),
        "librpa_set_aux_cut_coulomb_k_atom_pair": (None, [vp, i, i, i, i, i, _dp, _dp, d]),
        "librpa_set_aux_cut_coulomb_k_2d_block": (None, [vp, i, i, i, i, i, _dp, _dp]),
        "librpa_get_exx_pot_kgrid": (None, [vp, C.POINTER(LibrpaOptions), i, i, _ip, i, i, _dp]),
        "librpa_build_g0w0_sigma": (None, [vp, C.POINTER(LibrpaOptions)]),
        "librpa_get_g0w0_sigc_kgrid": (None, [vp, C.POINTER(LibrpaOptions), i, i, _ip, i, i, _dp, _dp, _dp, _dp]),
        "librpa_gb300_get_g0w0_sigc_iw": (i, [vp, i, i, i, _dp, _dp]),
        "librpa_gb300_get_g0w0_sigc_iw_k": (i, [vp, i, i, i, i, _dp, _dp]),
        "librpa_gb300_get_rpa_correlation_energy_batch": (i, [vp, i, vp, i, _dp]),
        "librpa_gb300_set_shrink_basis": (None, [vp, i, np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")]),
        "librpa_gb300_set_shrink_sinvS": (None, [vp, i, i, i, _dp, _dp]),
        "librpa_gb300_set_shrink_lri_coeff": (None, [vp, i, i, i, i, i, _ip, _dp]),
        "librpa_gb300_init_options": (None, [C.POINTER(GB300Options)]),
        "librpa_gb300_set_options": (None, [vp, C.POINTER(GB300Options)]),
        "librpa_gb300_get_stats": (None, [vp, C.POINTER(GB300Stats)]),
        "librpa_get_last_error": (C.c_char_p, [vp]),
        "librpa_get_last_error_code": (i, [vp]),
        "librpa_gb300_minimax_grid": (i, [i, d, d, d, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.POINTER(d)]),
        "librpa_gb300_get_chi0_block": (i, [vp, i, i, i, i, _dp, _dp]),
        "librpa_gb300_device_count": (i, []),
        "librpa_gb300_selftest_tc_gemm": (d, [i, i, i, i, i]),
        "librpa_gb300_selftest_chol_ozaki": (d, [i, i, i, i, d, C.POINTER(C.c_double)]),
        "librpa_gb300_tc_gemm_noalloc": (i, [i, i, i, C.c_void_p, C.c_void_p, C.c_void_p, i,
                                             C.c_void_p]),
        "librpa_gb300_train_screening": (i, [vp, i, d, C.POINTER(C.c_double)]),
        "librpa_gb300_screening_samples": (C.c_longlong, [vp]),
        "librpa_gb300_get_screening_samples": (i, [vp, vp, vp, C.c_longlong]),
        "librpa_gb300_add_screening_samples": (i, [vp, vp, vp, C.c_longlong]),
        "librpa_gb300_clear_grid_cache": (None, []),
        "librpa_gb300_get_screening_model": (i, [vp, vp, vp]),
        "librpa_gb300_set_screening_model": (i, [vp, vp, vp]),
        "librpa_gb300_clear_screening": (None, [vp]),
        "librpa_gb300_chi0_qw_elems": (C.c_longlong, [vp]),
        "librpa_gb300_copy_chi0_qw": (i, [vp, vp, i]),
        "librpa_gb300_load_chi0_qw": (i, [vp, vp, C.c_longlong, i]),
        "librpa_gb300_mlp_loss_grad": (i, [vp, vp, vp, vp, i, vp, C.POINTER(C.c_double)]),
        "librpa_gb300_solve_qpe": (i, [i, i, _dp, _dp, _dp, i, _dp, d, _dp, _dp, _dp, _dp, _dp]),
        "librpa_gb300_phase_tables": (i, [vp, vp, vp, vp, vp, vp, vp, vp]),
        "librpa_gb300_interpolate_dielec_func": (i, [i, i, _dp, _dp, i, _dp, _dp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class LibrpaError(RuntimeError):
    pass


class Options(LibrpaOptions):
    """librpa::Options: LibrpaOptions initialised with LibRPA's defaults."""

    def __init__(self, **kw):
        super().__init__()
        load_library().librpa_init_options(C.byref(self))
        for k, v in kw.items():
            setattr(self, k, v)

    def set_output_dir(self, d: str):
        load_library().librpa_set_output_dir(C.byref(self), d.encode())


def gb300_options(**kw) -> GB300Options:
    o = GB300Options()
    load_library().librpa_gb300_init_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Handler:
    """librpa::Handler mirror (RAII over librpa_create_handler / librpa_destroy_handler)."""

    def __init__(self, comm: int = 0):
        self.lib = load_library()
        self.h = self.lib.librpa_create_handler(comm)
        if not self.h:
            raise LibrpaError(self.lib.librpa_get_last_error(None).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.librpa_destroy_handler(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -------------------------------------------------- errors
    def last_error(self) -> str:
        return self.lib.librpa_get_last_error(self.h).decode()

    def _check(self):
        if self.lib.librpa_get_last_error_code(self.h):
            raise LibrpaError(self.last_error())

    # -------------------------------------------------- input (librpa.hpp:196-291)
    def set_scf_dimension(self, nspins, nkpts, nstates, nbasis, nspinor=1):
        self.lib.librpa_set_scf_dimension(self.h, nspins, nkpts, nstates, nbasis, nspinor)
        self._check()

    def set_wg_ekb_efermi(self, nspins, nkpts, nstates, wg, ekb, efermi):
        self.lib.librpa_set_wg_ekb_efermi(self.h, nspins, nkpts, nstates, _f64(wg).ravel(), _f64(ekb).ravel(),
                                          float(efermi))
        self._check()

    def set_wfc(self, ispin, ik, nstates_local, nbasis_local, wfc_real, wfc_imag):
        self.lib.librpa_set_wfc(self.h, ispin, ik, nstates_local, nbasis_local, _f64(wfc_real).ravel(),
                                _f64(wfc_imag).ravel())
        self._check()

    def set_wfc_packed(self, ispin, ik, nstates_local, nbasis_local, wfc_ri):
        self.lib.librpa_set_wfc_packed(self.h, ispin, ik, nstates_local, nbasis_local, _f64(wfc_ri).ravel())
        self._check()

    def set_ao_basis_wfc(self, nbs):
        a = np.ascontiguousarray(nbs, dtype=np.uint64)
        self.lib.librpa_set_ao_basis_wfc(self.h, len(a), a)
        self._check()

    def set_ao_basis_aux(self, nbs):
        a = np.ascontiguousarray(nbs, dtype=np.uint64)
        self.lib.librpa_set_ao_basis_aux(self.h, len(a), a)
        self._check()

    def set_shrink_basis(self, nbs_small):
        """Small ABF count per atom of the ABF shrink (use_shrink_abfs)."""
        a = np.ascontiguousarray(nbs_small, dtype=np.uint64)
        self.lib.librpa_gb300_set_shrink_basis(self.h, len(a), a)
        self._check()

    def set_shrink_sinvS(self, ik, U):
        """U(q) (n_small x n_large) of the IBZ point whose representative is k index ik."""
        U = np.asarray(U)
        self.lib.librpa_gb300_set_shrink_sinvS(self.h, ik, U.shape[0], U.shape[1], _f64(U.real).ravel(),
                                               _f64(U.imag).ravel())
        self._check()

    def set_shrink_lri_coeff(self, I, J, nbasis_i, nbasis_j, naux_mu_small, R, Cs):
        """An RI block in the small ABF basis (the exchange of a shrunk input)."""
        r = np.ascontiguousarray(R, dtype=np.int32)
        self.lib.librpa_gb300_set_shrink_lri_coeff(self.h, I, J, nbasis_i, nbasis_j, naux_mu_small, r, _f64(Cs).ravel())
        self._check()

    def set_latvec_and_G(self, lat_mat, G_mat):
        self.lib.librpa_set_latvec_and_G(self.h, _f64(lat_mat).ravel(), _f64(G_mat).ravel())
        self._check()

    def set_atoms(self, types, pos_cart):
        t = np.ascontiguousarray(types, dtype=np.int32)
        self.lib.librpa_set_atoms(self.h, len(t), t, _f64(pos_cart).ravel())
        self._check()

    def set_kgrids_kvec(self, nk1, nk2, nk3, kvecs):
        self.lib.librpa_set_kgrids_kvec(self.h, nk1, nk2, nk3, _f64(kvecs).ravel())
        self._check()

    def set_ibz_mapping(self, map_ibzk):
        m = np.ascontiguousarray(map_ibzk, dtype=np.int32)
        self.lib.librpa_set_ibz_mapping(self.h, len(m), m)
        self._check()

    def set_lri_coeff(self, routing, I, J, nbasis_i, nbasis_j, naux_mu, R, Cs):
        r = np.ascontiguousarray(R, dtype=np.int32)
        self.lib.librpa_set_lri_coeff(self.h, routing, I, J, nbasis_i, nbasis_j, naux_mu, r, _f64(Cs).ravel())
        self._check()

    def set_aux_bare_coulomb_k_atom_pair(self, ik, I, J, naux_mu, naux_nu, Vq_real, Vq_imag, vq_threshold=0.0):
        self.lib.librpa_set_aux_bare_coulomb_k_atom_pair(self.h, ik, I, J, naux_mu, naux_nu, _f64(Vq_real).ravel(),
                                                          _f64(Vq_imag).ravel(), float(vq_threshold))
        self._check()

    def set_aux_cut_coulomb_k_atom_pair(self, ik, I, J, naux_mu, naux_nu, Vq_real, Vq_imag, vq_threshold=0.0):
        self.lib.librpa_set_aux_cut_coulomb_k_atom_pair(self.h, ik, I, J, naux_mu, naux_nu, _f64(Vq_real).ravel(),
                                                         _f64(Vq_imag).ravel(), float(vq_threshold))
        self._check()

    def get_exx_pot_kgrid(self, opts, n_spins, iks, i_state_low, i_state_high):
        """v_exx [n_spins][len(iks)][states] (compute_exx.cpp layout); raises LibrpaError on failure."""
        iks = np.ascontiguousarray(iks, np.int32)
        nc = i_state_high - i_state_low
        out = np.zeros(n_spins * len(iks) * max(nc, 0))
        self.lib.librpa_get_exx_pot_kgrid(self.h, C.byref(opts), n_spins, len(iks), iks, i_state_low, i_state_high,
                                          out)
        self._check()
        return out.reshape(n_spins, len(iks), nc)

    def get_g0w0_sigc_kgrid(self, opts, n_spins, iks, i_state_low, i_state_high, vxc, vexx):
        """Sigma_c at the quasi-particle energy, complex [n_spins][len(iks)][states]; NaN where the
        quasi-particle solver failed.  vxc, vexx in the same layout (Hartree)."""
        iks = np.ascontiguousarray(iks, np.int32)
        nc = i_state_high - i_state_low
        re = np.zeros(n_spins * len(iks) * max(nc, 0))
        im = np.zeros_like(re)
        self.lib.librpa_get_g0w0_sigc_kgrid(self.h, C.byref(opts), n_spins, len(iks), iks, i_state_low,
                                            i_state_high, _f64(vxc).ravel(), _f64(vexx).ravel(), re, im)
        self._check()
        return (re + 1j * im).reshape(n_spins, len(iks), nc)

    def set_dielect_func_imagfreq(self, omegas, dielect_func):
        """The macroscopic dielectric function on the imaginary axis (replace_w_head)."""
        om = _f64(omegas).ravel()
        self.lib.librpa_set_dielect_func_imagfreq(self.h, len(om), om, _f64(dielect_func).ravel())
        self._check()

    def set_band_points(self, kfrac, occ, eig, wfc):
        """Band k-points off the SCF grid: fractional coordinates (n, 3), occupations and
        eigenvalues (n_spins, n, n_states) and eigenvectors (n_spins, n, n_states, n_ao)."""
        kf = _f64(kfrac).reshape(-1, 3)
        occ, eig = _f64(occ), _f64(eig)
        ns, nk, nst = eig.shape
        self.lib.librpa_set_band_kvec(self.h, nk, kf.ravel())
        self._check()
        self.lib.librpa_set_band_occ_eigval(self.h, ns, nk, nst, occ.ravel(), eig.ravel())
        self._check()
        for sp in range(ns):
            for k in range(nk):
                w = np.asarray(wfc[sp, k])
                self.lib.librpa_set_wfc_band(self.h, sp, k, w.shape[0], w.shape[1], _f64(w.real).ravel(),
                                             _f64(w.imag).ravel())
                self._check()

    def get_exx_pot_band_k(self, opts, n_spins, iks_band, i_state_low, i_state_high):
        """v_exx at band k-points [n_spins][len(iks_band)][states] (Hartree)."""
        iks = np.ascontiguousarray(iks_band, np.int32)
        nc = i_state_high - i_state_low
        out = np.zeros(n_spins * len(iks) * max(nc, 0))
        self.lib.librpa_get_exx_pot_band_k(self.h, C.byref(opts), n_spins, len(iks), iks, i_state_low, i_state_high,
                                           out)
        self._check()
        return out.reshape(n_spins, len(iks), nc)

    def get_g0w0_sigc_band_k(self, opts, n_spins, iks_band, i_state_low, i_state_high, vxc, vexx):
        """Sigma_c at the quasi-particle energy at band k-points, complex [n_spins][len(iks_band)][states]."""
        iks = np.ascontiguousarray(iks_band, np.int32)
        nc = i_state_high - i_state_low
        re = np.zeros(n_spins * len(iks) * max(nc, 0))
        im = np.zeros_like(re)
        self.lib.librpa_get_g0w0_sigc_band_k(self.h, C.byref(opts), n_spins, len(iks), iks, i_state_low,
                                             i_state_high, _f64(vxc).ravel(), _f64(vexx).ravel(), re, im)
        self._check()
        return (re + 1j * im).reshape(n_spins, len(iks), nc)

    def g0w0_sigc_iw(self, ispin, lo, hi, nfreq, ik=0):
        """KS-diagonal Sigma_c(i omega) [state][omega] of the last G0W0 build at SCF k-point ik."""
        re = np.zeros((hi - lo) * nfreq)
        im = np.zeros_like(re)
        if self.lib.librpa_gb300_get_g0w0_sigc_iw_k(self.h, ispin, ik, lo, hi, re, im) != 0:
            raise LibrpaError(self.last_error())
        return (re + 1j * im).reshape(hi - lo, nfreq)

    def set_aux_bare_coulomb_k_2d_block(self, ik, mu_begin, mu_end, nu_begin, nu_end, Vq_real, Vq_imag):
        self.lib.librpa_set_aux_bare_coulomb_k_2d_block(self.h, ik, mu_begin, mu_end, nu_begin, nu_end,
                                                         _f64(Vq_real).ravel(), _f64(Vq_imag).ravel())
        self._check()

    # -------------------------------------------------- extensions
    def set_gb300_options(self, o: GB300Options):
        self.lib.librpa_gb300_set_options(self.h, C.byref(o))
        self._check()

    def chi0_qw(self) -> np.ndarray:
        """Copy of the kept chi0(q, omega) (complex128, [omega][q][pair blocks], flattened)."""
        n = self.lib.librpa_gb300_chi0_qw_elems(self.h)
        if n <= 0:
            raise LibrpaError(self.last_error() or "no chi0(q, omega) kept")
        out = np.zeros(n, np.complex128)
        if self.lib.librpa_gb300_copy_chi0_qw(self.h, out.ctypes.data_as(C.c_void_p), 0) != 0:
            raise LibrpaError(self.last_error())
        return out

    def load_chi0_qw(self, a: np.ndarray):
        """Replace the kept chi0(q, omega) (e.g. with a sum of tau-shard partials)."""
        a = np.ascontiguousarray(a, np.complex128)
        if self.lib.librpa_gb300_load_chi0_qw(self.h, a.ctypes.data_as(C.c_void_p), a.size, 0) != 0:
            raise LibrpaError(self.last_error())

    def chi0_qw_tensor(self, device):
        """The kept chi0(q, omega) as a float64 torch tensor of (re, im) pairs on `device`; a CUDA
        device gets a device-to-device copy (it must be the handler's GPU)."""
        import torch
        n = self.lib.librpa_gb300_chi0_qw_elems(self.h)
        if n <= 0:
            raise LibrpaError(self.last_error() or "no chi0(q, omega) kept")
        t = torch.empty(2 * n, dtype=torch.float64, device=device)
        if t.is_cuda:
            torch.cuda.current_stream(t.device).synchronize()
        if self.lib.librpa_gb300_copy_chi0_qw(self.h, C.c_void_p(t.data_ptr()), int(t.is_cuda)) != 0:
            raise LibrpaError(self.last_error())
        return t

    def load_chi0_qw_tensor(self, t):
        """Replace the kept chi0(q, omega) from a float64 (re, im) torch tensor (host or GPU)."""
        import torch
        t = t.contiguous()
        if t.dtype != torch.float64 or t.numel() % 2:
            raise LibrpaError("chi0(q, omega) tensor must be float64 (re, im) pairs")
        if t.is_cuda:
            torch.cuda.current_stream(t.device).synchronize()
        if self.lib.librpa_gb300_load_chi0_qw(self.h, C.c_void_p(t.data_ptr()), t.numel() // 2, int(t.is_cuda)) != 0:
            raise LibrpaError(self.last_error())

    def stats(self) -> dict:
        s = GB300Stats()
        self.lib.librpa_gb300_get_stats(self.h, C.byref(s))
        return s.as_dict()

    def get_chi0_block(self, ifreq, iq, I, J, n_mu, n_nu):
        re = np.zeros(n_mu * n_nu)
        im = np.zeros(n_mu * n_nu)
        if self.lib.librpa_gb300_get_chi0_block(self.h, ifreq, iq, I, J, re, im) != 0:
            raise LibrpaError(self.last_error())
        return (re + 1j * im).reshape(n_mu, n_nu)

    # -------------------------------------------------- compute (librpa.hpp:294-305)
    def get_imaginary_frequency_grids(self, opts: Options):
        om = np.zeros(opts.nfreq)
        w = np.zeros(opts.nfreq)
        self.lib.librpa_get_imaginary_frequency_grids(self.h, C.byref(opts), om, w)
        self._check()
        return om, w

    def get_rpa_correlation_energy(self, opts: Options, n_ibz_kpoints: int):
        """Returns (E_c, per-IBZ-k complex contributions); raises LibrpaError on failure."""
        re = np.zeros(max(n_ibz_kpoints, 1))
        im = np.zeros(max(n_ibz_kpoints, 1))
        ec = self.lib.librpa_get_rpa_correlation_energy(self.h, C.byref(opts), n_ibz_kpoints, re, im)
        if math.isnan(ec):
            raise LibrpaError(self.last_error())
        return ec, re[:n_ibz_kpoints] + 1j * im[:n_ibz_kpoints]


def phase_tables(h, n_kpts):
    """The host index/phase tables of the GPU path for handler h (librpa_gb300_phase_tables)."""
    lib = load_library()
    nc, nq = C.c_int(0), C.c_int(0)
    null = None
    if lib.librpa_gb300_phase_tables(h.h, C.byref(nc), C.byref(nq), null, null, null, null, null) != 0:
        raise LibrpaError(h.last_error())
    nk = n_kpts
    cells = np.zeros(3 * nc.value, np.int32)
    rep = np.zeros(nq.value, np.int32)
    w = np.zeros(nq.value)
    gp = np.zeros(2 * nk * nc.value)
    qp = np.zeros(2 * nq.value * nc.value)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)
    if lib.librpa_gb300_phase_tables(h.h, None, None, ptr(cells), ptr(rep), ptr(w), ptr(gp), ptr(qp)) != 0:
        raise LibrpaError(h.last_error())
    return {"cells": cells.reshape(-1, 3), "ibz_rep": rep, "ibz_w": w,
            "g_phase": gp.reshape(nk, nc.value, 2), "q_phase": qp.reshape(nq.value, nc.value, 2)}


def solve_qpe(omegas, sigc_iw, e_mf, e_fermi, vxc, vexx, n_params=-1):
    """Pade continuation + quasi-particle equation per state (librpa_gb300_solve_qpe, host only).
    sigc_iw: (n_states, n_freq) complex.  Returns (e_qp, sigc_qp complex, n_unconverged)."""
    lib = load_library()
    sig = np.ascontiguousarray(sigc_iw, complex)
    ns, nf = sig.shape
    e_qp, sr, si = np.zeros(ns), np.zeros(ns), np.zeros(ns)
    f64 = lambda a: np.ascontiguousarray(a, np.float64)
    rc = lib.librpa_gb300_solve_qpe(ns, nf, f64(omegas), f64(sig.real), f64(sig.imag), n_params, f64(e_mf),
                                    float(e_fermi), f64(vxc), f64(vexx), e_qp, sr, si)
    if rc < 0:
        raise LibrpaError(lib.librpa_get_last_error(None).decode())
    return e_qp, sr + 1j * si, rc


def interpolate_dielec_func(option, omega_in, eps_in, omega_target):
    """eps(i omega) mapped onto target frequencies as the G0W0 head correction maps it onto the
    minimax ones (librpa_gb300_interpolate_dielec_func, host only): option 0 the given values,
    1 cubic spline, 2 Havriliak-Negami fit."""
    lib = load_library()
    f64 = lambda a: np.ascontiguousarray(a, np.float64)
    om, eps, tg = f64(omega_in), f64(eps_in), f64(omega_target)
    out = np.zeros(len(tg))
    if lib.librpa_gb300_interpolate_dielec_func(int(option), len(om), om, eps, len(tg), tg, out) != 0:
        raise LibrpaError(lib.librpa_get_last_error(None).decode())
    return out


def minimax_grid(n, emin, emax, regularization=0.0):
    """Host-only minimax grid (librpa_gb300_minimax_grid)."""
    lib = load_library()
    a = [np.zeros(n) for _ in range(4)] + [np.zeros(n * n) for _ in range(3)]
    dual = C.c_double(0)
    rc = lib.librpa_gb300_minimax_grid(n, emin, emax, regularization, *a, C.byref(dual))
    if rc != 0:
        raise LibrpaError(lib.librpa_get_last_error(None).decode())
    return {"tau": a[0], "tau_w": a[1], "omega": a[2], "omega_w": a[3],
            "cos_t2f": a[4].reshape(n, n), "cos_f2t": a[5].reshape(n, n), "sin_t2f": a[6].reshape(n, n),
            "cosft_duality_error": dual.value}


def load_system(h: Handler, s, routing=LIBRI):
    """Feed a SynthSystem-like record through the librpa_set_* calls (as a DFT code would)."""
    h.set_scf_dimension(s.n_spins, s.n_kpts, s.n_bands, s.n_ao)
    h.set_wg_ekb_efermi(s.n_spins, s.n_kpts, s.n_bands, s.wg, s.ekb, s.efermi)
    for isp in range(s.n_spins):
        for ik in range(s.n_kpts):
            w = s.wfc[isp, ik]
            h.set_wfc(isp, ik, s.n_bands, s.n_ao, w.real, w.imag)
    h.set_ao_basis_wfc(s.nao)
    h.set_ao_basis_aux(s.nabf)
    recip = 2.0 * math.pi * np.linalg.inv(s.latvec).T
    h.set_latvec_and_G(s.latvec, recip)
    types = getattr(s, "types", np.zeros(len(s.nao), int))
    if s.positions is not None:
        h.set_atoms(types, s.positions)
    h.set_kgrids_kvec(*s.period, s.kvecs)
    h.set_ibz_mapping(s.ibz_map)
    for (I, J, R), m in s.Cs.items():
        h.set_lri_coeff(routing, I, J, s.nao[I], s.nao[J], s.nabf[I], R, m)
    # with an ABF shrink the Coulomb matrix is in the small basis, U(q) keyed by IBZ order
    nbv = getattr(s, "nabf_small", None) or s.nabf
    for (ik, I, J), v in s.Vq.items():
        h.set_aux_bare_coulomb_k_atom_pair(ik, I, J, nbv[I], nbv[J], v.real, v.imag, 0.0)
    if getattr(s, "sinvS", None):
        h.set_shrink_basis(s.nabf_small)
        reps = list(dict.fromkeys(int(x) for x in s.ibz_map))
        for iq, U in s.sinvS.items():
            h.set_shrink_sinvS(reps[iq], U)
        for (I, J, R), m in (getattr(s, "Cs_small", None) or {}).items():
            h.set_shrink_lri_coeff(I, J, s.nao[I], s.nao[J], s.nabf_small[I], R, m)
    for (ik, I, J), v in getattr(s, "v_cut", {}).items():
        h.set_aux_cut_coulomb_k_atom_pair(ik, I, J, nbv[I], nbv[J], v.real, v.imag, 0.0)


def rpa_correlation_energy_batch(handlers, opts, n_threads=0):
    """E_c of several independent handlers in one concurrent call; opts: one Options or a list."""
    lib = load_library()
    n = len(handlers)
    hs = (C.c_void_p * n)(*[h.h for h in handlers])
    ol = opts if isinstance(opts, (list, tuple)) else [opts] * n
    oa = (LibrpaOptions * n)()
    for i, o in enumerate(ol):
        oa[i] = LibrpaOptions.from_buffer_copy(o)
    ec = np.zeros(n)
    failed = lib.librpa_gb300_get_rpa_correlation_energy_batch(hs, n, oa, n_threads, ec)
    if failed < 0:
        raise LibrpaError(lib.librpa_get_last_error(None).decode())
    if failed > 0:
        msgs = [h.last_error() for h, e in zip(handlers, ec) if math.isnan(e)]
        raise LibrpaError(f"{failed} of {n} calls failed: " + "; ".join(msgs[:3]))
    return ec


def n_ibz(s) -> int:
    return len(set(int(x) for x in s.ibz_map))
