#pragma once
/*
 * GB300 extensions to the LibRPA C API.
 *
 * Everything here is additive: none of it exists in LibRPA, and a caller that
 * uses only librpa.h keeps the reference's behaviour.  Knobs that LibRPA does
 * not have (precision mode, block screening, learned screening) live in
 * LibrpaGB300Options instead of LibrpaOptions, whose layout is frozen by the
 * Fortran binding.
 */
#include "librpa_handler.h"
#include "librpa_options.h"

#ifdef __cplusplus
extern "C" {
#endif

/* chi0 contraction precision */
#define LIBRPA_GB300_CHI0_FP64 0      /* plain FP64 SIMT kernels (reference-precision GPU path) */
#define LIBRPA_GB300_CHI0_BF16X3 1    /* 3-term BF16 split products on tcgen05, FP32 accumulate in TMEM */
#define LIBRPA_GB300_CHI0_FP32 2      /* FP32 SIMT kernels (diagnostic middle ground) */

/* E_c kernel path */
#define LIBRPA_GB300_EC_LU_FP64 0     /* Pi = V chi0 in FP64, FP64 LU, sum log(+-u_ii) (LibRPA form) */
#define LIBRPA_GB300_EC_CHOL 1        /* L^H chi0 L split-precision GEMMs, FP64 Cholesky */
#define LIBRPA_GB300_EC_CHOL_FP64 2   /* the same Cholesky form with FP64 GEMMs: an all-FP64 E_c */

/* block screening of chi0 contributions */
#define LIBRPA_GB300_SCREEN_OFF 0
#define LIBRPA_GB300_SCREEN_THRESHOLD 1   /* contract every chi0(I,J,R,tau) block, drop those with
                                             max |chi0| <= screen_threshold (LibRI's max-norm filter
                                             rule); log block features and norms for training */
#define LIBRPA_GB300_SCREEN_MLP 2         /* contract only blocks a trained MLP predicts above the
                                             threshold, plus a random audit share of the others;
                                             the threshold rule still decides and is the fallback */

typedef struct
{
    int chi0_precision;      /* LIBRPA_GB300_CHI0_*   (default BF16X3) */
    int ec_path;             /* LIBRPA_GB300_EC_*     (default CHOL)   */
    int screen_mode;         /* LIBRPA_GB300_SCREEN_* (default OFF)    */
    double screen_threshold; /* block-norm threshold for screening (default 1e-6) */
    double audit_fraction;   /* share of skipped blocks computed exactly (default 0.02) */
    unsigned long long seed; /* audit sampling seed */
    int use_cuda_graph;      /* reserved: this build launches the per-tau sequence directly */
    int keep_chi0;           /* keep chi0(q, omega) on the device for librpa_gb300_get_chi0_block */
    int device;              /* CUDA device ordinal (default 0) */
    int reuse_device_inputs; /* keep the staged inputs on the device between calls while no
                                librpa_set_* call changed them (default 1); 0 re-uploads every call
                                (into the device buffers the handler keeps while sizes agree) */
    /* tau sharding (one slice of the minimax tau points per rank; the chi0(q, omega) partial
     * sums are reduced over ranks before E_c): */
    int tau_begin;           /* first tau point of this call (default 0) */
    int tau_end;             /* one past the last; -1 = all (default -1) */
    int stage;               /* LIBRPA_GB300_STAGE_* (default FULL) */
    /* q sharding of E_c: the E_c of a FULL or EC call covers the IBZ q points [q_begin, q_end)
     * only; the per-q outputs of the others are 0 (a rank then owns those q of the reduce-
     * scattered chi0(q, omega) and the per-q sums are all-reduced) */
    int q_begin;             /* first IBZ q point (default 0) */
    int q_end;               /* one past the last; -1 = all (default -1) */
    int sigma_precision;     /* LIBRPA_GB300_SIGMA_*: the contraction of the G0W0 correlation
                                self-energy (default FP64; the exchange is always FP64) */
} LibrpaGB300Options;

/* G0W0 correlation self-energy contraction precision */
#define LIBRPA_GB300_SIGMA_FP64 0     /* FP64 GEMMs */
#define LIBRPA_GB300_SIGMA_BF16X3 1   /* 3-term BF16 split GEMMs on tcgen05, FP32 accumulate, the
                                         long contraction cut into chunks summed in FP64 */

#define LIBRPA_GB300_STAGE_FULL 0   /* chi0 over [tau_begin, tau_end) and E_c */
#define LIBRPA_GB300_STAGE_CHI0 1   /* chi0(q, omega) over [tau_begin, tau_end), kept on the device;
                                       the call returns 0 (no E_c) */
#define LIBRPA_GB300_STAGE_EC 2     /* E_c from the kept chi0(q, omega) (after
                                       librpa_gb300_load_chi0_qw); no chi0 work */

/* Timing and work counters of the last librpa_get_rpa_correlation_energy call. */
typedef struct
{
    double t_total;        /* wall seconds of the whole call */
    double t_grids;        /* minimax grid set-up (host) */
    double t_upload;       /* host -> device staging of the dataset */
    double t_gf;           /* G(R, +-tau) build (device) */
    double t_chi0;         /* chi0(R, tau) contraction (device) */
    double t_ftct;         /* R->q Fourier and tau->omega cosine transform (device) */
    double t_ec;           /* Pi / log-det / trace (device) */
    double chi0_flops;     /* FLOPs executed by the chi0 contraction kernels (useful work, split terms not counted) */
    double chi0_flops_libri; /* FLOPs the LibRI loop order would spend on the same blocks */
    double ec_flops;       /* FLOPs of the E_c stage */
    double gf_flops;       /* FLOPs of the G build */
    double ftct_bytes;     /* algorithmic bytes of the FT/CT kernels */
    long long n_launches;  /* kernels launched by this library during the call */
    long long blocks_total;     /* (I<=J, R) chi0 blocks in the problem */
    long long blocks_computed;  /* blocks actually contracted */
    long long blocks_audited;   /* skipped-by-predictor blocks computed for the audit */
    double audit_max_dropped;   /* largest block norm among audited skipped blocks */
    double dt_chi0_kernel_ms;   /* CUDA-event time of the dominant chi0 kernel, summed over launches */
    long long n_chi0_kernel;    /* launches of the dominant chi0 kernel */
    double h2d_bytes;           /* host -> device bytes staged by this call (0 when the cache was reused) */
    double d2h_bytes;           /* device -> host bytes of results */
    long long screen_fallbacks; /* (tau, spin) steps where an audited skipped block exceeded the
                                   threshold and every block was contracted */
    long long ec_lu_fallback_q; /* IBZ q points whose V(q) had no Cholesky factor (indefinite, as
                                   the Gamma-point bare Coulomb matrix of a crystal can be) and
                                   whose E_c term the Cholesky path took by the LU form instead */
    int t1_narrow;              /* tensor-core chi0 contraction: 1 = 16 producer warps of 2 columns,
                                   0 = 8 of 4 columns (the tuner's choice for this shape) */
    int t1_kparts;              /* K parts per 128-row tile of that contraction (tuner's choice) */
    int chi0_precision_used;    /* the chi0 path that ran (LIBRPA_GB300_CHI0_*): BF16X3 requested
                                   on atoms beyond the tensor-core tiles (more than 32 NAOs or
                                   128 ABFs) runs the FP32 path */
} LibrpaGB300Stats;

/* Set defaults. */
void librpa_gb300_init_options(LibrpaGB300Options *o);
/* Attach options to a handler (copied). */
void librpa_gb300_set_options(LibrpaHandler *h, const LibrpaGB300Options *o);
/* Counters of the last RPA call on this handler. */
void librpa_gb300_get_stats(LibrpaHandler *h, LibrpaGB300Stats *s);

/* Last error recorded on this handler (h may be NULL for the process-wide
 * last error); empty string when none.  Errors never escape as C++ exceptions. */
const char *librpa_get_last_error(LibrpaHandler *h);
/* 0 when the last call on h succeeded. */
int librpa_get_last_error_code(LibrpaHandler *h);

/* Minimax grids without a handler (host only, no GPU needed).  Arrays of
 * length n (tau, tau_w, omega, omega_w) and n*n (row-major cos_t2f[w][t],
 * cos_f2t[t][w], sin_t2f[w][t]).  Returns 0 on success. */
int librpa_gb300_minimax_grid(int n, double emin, double emax, double regularization,
                              double *tau, double *tau_w, double *omega, double *omega_w,
                              double *cos_t2f, double *cos_f2t, double *sin_t2f,
                              double *duality_error);

/* No counterpart in the reference: forget the minimax grids this process has fitted.  E_c calls
 * keep the grids of the last few (n, e_min, e_max, regularization) windows and reuse them;
 * after this call the next E_c call fits its grids again, as every call of the reference does
 * (TFGrids::generate_minimax, src/core/timefreq.cpp:193-236).  Host only. */
void librpa_gb300_clear_grid_cache(void);

/* G0W0 quasi-particle equation for n_states states (host only, no GPU needed): the Thiele-Pade
 * continuation of each state's Sigma_c(i omega_k), k < n_freq (sigc_re/im[state * n_freq + k],
 * omega_k > 0 the imaginary frequencies), with n_params parameters (< 0: all points), then the
 * damped fixed point e = e_mf - vxc + vexx + Re Sigma_c(e - e_fermi).  Replaces the per-state
 * loop of librpa_get_g0w0_sigc_kgrid (src/api/compute_g0w0.cpp:270-300; AnalyContPade,
 * src/core/analycont.cpp:12-70; qpe_solver_pade_self_consistent, src/core/qpe_solver.cpp).
 * Outputs per state: e_qp and Sigma_c(e_qp); NaN where the iteration hit its limit (counted in
 * the return value) or the continued fraction broke down (0/0), as the reference reports them.
 * Returns the number of states that hit the iteration limit, or -1 on error. */
int librpa_gb300_solve_qpe(int n_states, int n_freq, const double *omegas, const double *sigc_re,
                           const double *sigc_im, int n_params, const double *e_mf, double e_fermi,
                           const double *vxc, const double *vexx, double *e_qp, double *sigc_qp_re,
                           double *sigc_qp_im);

/* Diagnostic (no counterpart in the reference; host only, no GPU needed): the index and phase
 * tables the GPU path builds from the handler's data.  With all arrays NULL it only writes
 * *n_cells and *n_q.  Then: cells[3 n_cells] (the BvK cell vectors, centred range, x outer,
 * z inner: construct_R_grid, src/core/pbc.cpp:178-190), ibz_rep[n_q] (full k index of each IBZ
 * point, first-seen order) and ibz_w[n_q] (count / n_k) (pbc.cpp:110-153), g_phase[n_k][n_cells][2]
 * = (cos, sin) of 2 pi kfrac_k . R (G(R) = sum_k e^{-i...} G(k), src/core/chi0.cpp:379-380) and
 * q_phase[n_q][n_cells][2] = (cos, sin) of 2 pi q . (R latvec) (FT of chi0, chi0.cpp:582).
 * Returns 0 on success. */
int librpa_gb300_phase_tables(LibrpaHandler *h, int *n_cells, int *n_q, int *cells, int *ibz_rep, double *ibz_w,
                              double *g_phase, double *q_phase);

/* After a call with keep_chi0 = 1: copy chi0(q_ibz, omega) block (I<=J) to the
 * caller as two row-major n_mu x n_nu arrays.  Returns 0 on success. */
int librpa_gb300_get_chi0_block(LibrpaHandler *h, int ifreq, int iq_ibz, int I, int J,
                                double *re, double *im);

/* Kept chi0(q, omega) (keep_chi0 or STAGE_CHI0; no counterpart in the reference): number of
 * complex elements, [omega][q_ibz][upper-pair blocks] in the order of librpa_gb300_get_chi0_block;
 * copy out to, or replace from, interleaved (re, im) doubles on the host (on_device = 0) or
 * the current device (on_device = 1).  Used to all-reduce tau-shard partial sums. */
long long librpa_gb300_chi0_qw_elems(LibrpaHandler *h);
int librpa_gb300_copy_chi0_qw(LibrpaHandler *h, double *dst, int on_device);
int librpa_gb300_load_chi0_qw(LibrpaHandler *h, const double *src, long long n_elems, int on_device);

/* Learned screening (no counterpart in the reference).  The model is a 9-64-64-1 GELU MLP
 * (FP16 weights, FP32 accumulation) predicting log10 max |chi0(I,J,R,tau)| from nine features
 * of the block: distance (Bohr), log10 tau, log10(max|C_I| max|C_J|), log10 max |G(+tau)_IJ(R)|,
 * log10 max |G(-tau)_IJ(R)|, log10(n_abf(I) n_abf(J)), log10(n_ao(I) n_ao(J)) and the species
 * of I and of J (the types given to librpa_set_atoms).  Its training data are the blocks logged
 * by calls with screen_mode = LIBRPA_GB300_SCREEN_THRESHOLD, on this handler or added from
 * others with librpa_gb300_add_screening_samples.
 * librpa_gb300_train_screening trains it on the GPU (Adam, `iterations` steps of up to 16384
 * samples); a screen_mode = MLP call trains it itself when needed.  Returns 0 on success and
 * writes the training RMSE (log10 units) to *rmse. */
int librpa_gb300_train_screening(LibrpaHandler *h, int iterations, double learning_rate, double *rmse);
/* Logged samples: count, and a copy (x: n x 9 features, y: n targets). */
long long librpa_gb300_screening_samples(LibrpaHandler *h);
int librpa_gb300_get_screening_samples(LibrpaHandler *h, float *x, float *y, long long n);
/* Append n samples (x: n x 9 features, y: n targets) logged elsewhere, e.g. by the plain runs
 * of other systems, to this handler's training set.  Returns 0 on success. */
int librpa_gb300_add_screening_samples(LibrpaHandler *h, const float *x, const float *y, long long n);
/* The trained model: 4865 parameters (W1[64][9], b1[64], W2[64][64], b2[64], W3[64], b3) and
 * 21 normalisation values (feature means[9], scales[9], target mean, target scale, decision
 * margin).  get returns 0 when a model exists; set installs one. */
int librpa_gb300_get_screening_model(LibrpaHandler *h, float *params, float *norm);
int librpa_gb300_set_screening_model(LibrpaHandler *h, const float *params, const float *norm);
/* Drop the logged samples and the model. */
void librpa_gb300_clear_screening(LibrpaHandler *h);
/* The MLP's training kernels on one batch: mean squared error on normalised targets and its
 * gradient for the given FP32 parameters (rounded to FP16 as the forward pass uses them).
 * For checking the GPU gradients against a CPU restatement.  Returns 0 on success. */
int librpa_gb300_mlp_loss_grad(const float *params, const float *norm, const float *x, const float *y, int n,
                               float *grad, double *loss);

/* No counterpart in the reference: after librpa_build_g0w0_sigma, the KS-diagonal correlation
 * self-energy on the imaginary axis that the quasi-particle step continues, at k-point 0 (the
 * Gamma point, or the first point of a k-grid), re/im[(state - i_state_low) * nfreq + ifreq] for
 * states [i_state_low, i_state_high) of spin ispin.  Returns 0 on success. */
int librpa_gb300_get_g0w0_sigc_iw(LibrpaHandler *h, int ispin, int i_state_low, int i_state_high, double *re,
                                  double *im);
/* The same at k-point ik of the SCF grid. */
int librpa_gb300_get_g0w0_sigc_iw_k(LibrpaHandler *h, int ispin, int ik, int i_state_low, int i_state_high, double *re,
                                    double *im);

/* No counterpart in the reference (the internal interpolate_dielec_func,
 * src/core/dielecmodel.cpp:65-104, exposed for checking): the macroscopic dielectric function
 * eps(i omega) given at n_in frequencies, mapped onto n_out target frequencies as the G0W0 head
 * correction maps it onto the minimax frequencies.  option 0: the values unchanged (n_in must
 * equal n_out); 1: cubic spline (src/math/interpolate.cpp); 2: least-squares fit of the two-term
 * Havriliak-Negami model (src/math/fitting.cpp).  Host work; needs no GPU.  Returns 0 on success,
 * 1 on error (message: librpa_get_last_error(NULL)). */
int librpa_gb300_interpolate_dielec_func(int option, int n_in, const double *omega_in, const double *eps_in,
                                         int n_out, const double *omega_out, double *eps_out);

/* No counterpart in the reference: librpa_get_rpa_correlation_energy for n independent handlers
 * (separate systems, such as a batch of small cells), opts[i] for handler i, run concurrently on
 * up to n_threads host threads (0: up to 4), each call on its own CUDA stream so that their GPU
 * work overlaps.  ec[i] receives handler i's E_c, NaN on error with the message on that handler.
 * The handlers must be distinct.  Returns the number of failed calls, or -1 on a bad argument
 * (null pointers, a handler listed twice) with the message in librpa_get_last_error(NULL). */
int librpa_gb300_get_rpa_correlation_energy_batch(LibrpaHandler **hs, int n, const LibrpaOptions *opts, int n_threads,
                                                  double *ec);

/* ABF shrink (LibrpaOptions.use_shrink_abfs): chi0 is built in the ABF basis of the RI
 * coefficients (librpa_set_ao_basis_aux), then taken to a smaller ABF basis by
 * chi0_s(q) = U(q) chi0(q) U(q)^H (shrink_abfs_chi0, src/core/chi0.cpp:711-898), and E_c is
 * evaluated there, with the Coulomb matrix given in the small basis.  The reference holds these
 * inputs in Dataset::basis_aux_shrink and Dataset::sinvS (src/api/dataset.h:67-88) and its driver
 * reads them from Cs_shrinked_data_* and shrink_sinvS_* (driver/read_data.cpp:2455-2622); its C
 * API has no setter for them.
 * set_shrink_basis: small ABF count per atom.
 * set_shrink_sinvS: U(q) for the IBZ point whose representative is k index ik (the index the
 * Coulomb setters use), n_small x n_large row-major (rows: small ABFs); im may be NULL (real U).
 * At the Gamma point U must be real. */
void librpa_gb300_set_shrink_basis(LibrpaHandler *h, int natoms, const size_t *nbs_aux_small);
void librpa_gb300_set_shrink_sinvS(LibrpaHandler *h, int ik, int n_small, int n_large, const double *re,
                                   const double *im);
/* The RI coefficients in the small basis (the reference driver's Cs_shrinked_data), for the
 * exchange and G0W0 of a shrunk input: the exchange contracts them with the truncated Coulomb
 * matrix of the small basis, while chi0 and the correlation self-energy use those of
 * librpa_set_lri_coeff, W_c being taken back to that basis as U^H W_c U (unfold_abfs_Wc).
 * Arguments as librpa_set_lri_coeff, with naux_mu the small ABF count of atom I. */
void librpa_gb300_set_shrink_lri_coeff(LibrpaHandler *h, int I, int J, int nbasis_i, int nbasis_j, int naux_mu,
                                       const int R[3], const double *Cs_in);

/* Number of CUDA devices visible (0 when there is no GPU). */
int librpa_gb300_device_count(void);

/* Diagnostic: a random M x N x K product through the tcgen05 split-precision GEMM
 * (pieces = 2: 3 BF16 products; 3: 6 BF16 products) compared on the device with the FP64
 * CUDA-core GEMM.  Returns max|diff| / max|ref| (NaN on error). */
double librpa_gb300_selftest_tc_gemm(int M, int N, int K, int seed, int pieces);

/* Diagnostic: `batch` random N x N SPD matrices D (X X^T / N + shift I) D (X uniform, D a
 * diagonal scaling spread over spread_decades decades; a small shift makes them ill-conditioned)
 * factored by the FP64 CUDA-core Cholesky and by the variant whose panel solves and trailing
 * updates run on the tensor cores as exact 7-bit integer slice products.  Returns the largest
 * |ln det difference| (NaN on error); *max_rel_l (may be NULL) receives
 * max |L difference| / max |L|. */
double librpa_gb300_selftest_chol_ozaki(int N, int batch, int seed, int spread_decades, double shift,
                                        double *max_rel_l);

/* No counterpart in the reference.  D = A * B through the tcgen05 split-precision GEMM
 * (pieces = 2 or 3, as above) without allocating device memory, for callers that cannot
 * let a library allocate (a host code that has already sized its own pool to the whole
 * GPU).  A (M x K), B (K x N): FP64 row-major, D (M x N): FP32 row-major, all device
 * pointers on the current device; stream is a cudaStream_t (NULL: the legacy stream).
 * Scratch is a fixed 32 MiB device array inside the library: sizes needing more than
 * pieces * (M + N) * ceil(K / 64) * 64 * 2 bytes (+ alignment) <= 32 MiB are rejected.
 * The first call on a device does set-up (scratch address lookup, kernel attributes):
 * make it before any stream capture.  Calls whose GPU work overlaps race on the one
 * scratch array.  Synchronises the stream before returning.  Returns 0 on success,
 * nonzero on error (message in librpa_get_last_error(NULL)). */
int librpa_gb300_tc_gemm_noalloc(int M, int N, int K, const double *A, const double *B, float *D,
                                 int pieces, void *stream);

#ifdef __cplusplus
}
#endif
