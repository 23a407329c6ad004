// GPU pipeline of librpa_get_rpa_correlation_energy.
//
// Per imaginary time tau (and spin):
//   1. s(+-tau) weights, A_k = Psi^T diag(s) conj(Psi), G(R,+-tau) = sgn Re sum_k e^{-i2pi k.R} A_k
//      (chi0.cpp:303-426)
//   2. supercell G and X(+-) = C * G_super(+-)      (first contraction of LRI::cal_loop3)
//   3. chi0(R,tau) upper atom-pair blocks = two G+/G- passes of the a1b1_a2b2 and
//      a1b2_a2b1 contractions (RPA.hpp:104-137, LRI-cal_loop3.hpp:902-1032)
//   4. chi0(q,w) += 2/n_s gamma(w,tau) e^{i2pi q.R} chi0(R,tau)   (chi0.cpp:507-596)
// then per IBZ q: Pi = V chi0(q,w), tr Pi, ln det(I - Pi) and
//   E_c = sum_{q,w} w_w w_q / 2pi [ln det(I - Pi) + tr Pi]   (epsilon.cpp:270-558, :43-268)
//
// HBM layout (row-major everywhere):
//   C      [(I, mu, i)][(cell, K, k)]          rows_c x n_sup
//   G(+-)  [sign][cell][i][j]                  2 x n_c x n_ao x n_ao
//   Gs     [sign][(cK,k)][(cL,l)]              2 x n_sup x n_sup
//   X(+-)  [sign][(I, mu, i)][(cL, L, l)]      2 x rows_c x n_sup
//   chi0R  [pair I<=J][cell][mu][nu]           one tau at a time
//   chi0q  [w][q_ibz][pair][mu][nu] complex    accumulated over tau
#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <numeric>
#include <random>

#include "chi0_fast.h"
#include "common.h"
#include "cs_fold.h"
#include "host_tables.h"
#include "dataset.h"
#include "ec_tc.h"
#include "gk_tc.h"
#include "screen.h"
#include "tc_gemm.h"
#include "kernels.h"
#include "minimax.h"

namespace gb {

namespace {

struct EventTimer
{
    cudaEvent_t a = nullptr, b = nullptr;
    EventTimer()
    {
        GB_CUDA(cudaEventCreate(&a));
        GB_CUDA(cudaEventCreate(&b));
    }
    ~EventTimer()
    {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
    void start(cudaStream_t s) { GB_CUDA(cudaEventRecord(a, s)); }
    void stop(cudaStream_t s) { GB_CUDA(cudaEventRecord(b, s)); }
    double ms()
    {
        GB_CUDA(cudaEventSynchronize(b));
        float t = 0;
        GB_CUDA(cudaEventElapsedTime(&t, a, b));
        return t;
    }
};

} // namespace

int device_count()
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess)
    {
        cudaGetLastError();
        return 0;
    }
    return n;
}

void release_kept(Dataset &ds)
{
    if (ds.kept_chi0) cudaFree(ds.kept_chi0);
    ds.kept_chi0 = nullptr;
    ds.kept_chi0_bytes = 0;
}

RpaResult run_rpa_gpu(Dataset &ds, const LibrpaOptions &opts, const TimeFreqGrids &tf, int nbands_g)
{
    const double t_begin = wall_seconds();
    LibrpaGB300Stats &S = ds.stats;
    const LibrpaGB300Options &go = ds.gbopt;
    const int ndev = device_count();
    GB_REQUIRE(ndev > 0, "no CUDA device visible: the GB300 RPA path has no CPU fallback");
    GB_CUDA(cudaSetDevice(go.device));

    // ------------------------------------------------------------ host-side tables
    const int n_at = ds.n_atoms();
    GB_REQUIRE(n_at > 0, "number of atoms unknown: set atoms or bases first");
    GB_REQUIRE(static_cast<int>(ds.nao_at.size()) == n_at && static_cast<int>(ds.nabf_at.size()) == n_at,
               "wave-function and auxiliary bases must be set for every atom");
    GB_REQUIRE(ds.n_spinor == 1, "spinor (SOC) wave functions are not supported by the GPU RPA path");
    const int nk = ds.n_kpts, nb = ds.n_states, nao = ds.n_ao, ns = ds.n_spins;
    GB_REQUIRE(nk > 0 && nb > 0 && nao > 0 && ns > 0, "mean-field dimensions not set");
    GB_REQUIRE(ds.occ_set, "occupations/eigenvalues not set");
    for (size_t i = 0; i < ds.wfc_set.size(); ++i) GB_REQUIRE(ds.wfc_set[i], "wave function missing for some (spin, k)");
    std::vector<int> ao_off(n_at), abf_off(n_at + 1, 0);
    std::vector<long long> rowc_off(n_at);
    int tot_ao = 0, max_nao = 0, max_nabf = 0;
    long long rows_c = 0;
    for (int I = 0; I < n_at; ++I)
    {
        ao_off[I] = tot_ao;
        tot_ao += ds.nao_at[I];
        abf_off[I + 1] = abf_off[I] + ds.nabf_at[I];
        rowc_off[I] = rows_c;
        rows_c += static_cast<long long>(ds.nabf_at[I]) * ds.nao_at[I];
        max_nao = std::max(max_nao, ds.nao_at[I]);
        max_nabf = std::max(max_nabf, ds.nabf_at[I]);
    }
    GB_REQUIRE(tot_ao == nao, "sum of per-atom NAOs differs from the mean-field basis size");
    const int N = abf_off[n_at];
    const PhaseTables pt = build_phase_tables(ds);
    const Cells &cells = pt.cells;
    const int nc = pt.nc;
    GB_REQUIRE(nc == nk, "number of BvK cells must equal the number of k points");
    const std::vector<int> &cdiff = pt.cdiff, &cneg = pt.cneg;
    const long long n_sup = static_cast<long long>(nc) * nao;
    const std::vector<double> &gcos = pt.gcos, &gsin = pt.gsin;   // G phases (chi0.cpp:379-380)
    const std::vector<int> &ibz_rep = pt.ibz_rep;                 // IBZ list (pbc.cpp:110-153)
    const std::vector<double> &ibz_w = pt.ibz_w;
    const int nq = pt.nq;
    const std::vector<double> &qcos = pt.qcos, &qsin = pt.qsin;   // FT phases (chi0.cpp:582)

    // upper atom pairs
    std::vector<int> pI, pJ, pair_of(static_cast<size_t>(n_at) * n_at, -1);
    std::vector<long long> r_off, e_off;
    long long r_tot = 0, e_tot = 0;
    for (int I = 0; I < n_at; ++I)
        for (int J = I; J < n_at; ++J)
        {
            pair_of[I * n_at + J] = static_cast<int>(pI.size());
            pI.push_back(I);
            pJ.push_back(J);
            r_off.push_back(r_tot);
            e_off.push_back(e_tot);
            const long long el = static_cast<long long>(ds.nabf_at[I]) * ds.nabf_at[J];
            r_tot += el * nc;
            e_tot += el;
        }
    const int n_pairs = static_cast<int>(pI.size());
    std::vector<int> atom_of(N);
    for (int I = 0; I < n_at; ++I)
        for (int a = abf_off[I]; a < abf_off[I + 1]; ++a) atom_of[a] = I;

    // RI blocks -> (I, J, cell) table: cell vectors folded into the BvK cell list, blocks that
    // fold onto one key summed, then LibRI's threshold filter (cs_fold.h)
    for (const CsBlock &b : ds.cs_blocks)
    {
        GB_REQUIRE(b.I >= 0 && b.I < n_at && b.J >= 0 && b.J < n_at, "RI block atom index out of range");
        GB_REQUIRE(b.ni == ds.nao_at[b.I] && b.nj == ds.nao_at[b.J] && b.nmu == ds.nabf_at[b.I],
                   "RI block dimensions inconsistent with the bases");
    }
    CsFold csf = fold_cs_blocks(
        ds.cs_blocks, ds.cs_blob.data(), ds.cs_blob.size(), ds.period,
        [&](const std::array<int, 3> &R) { return cells.find(R[0], R[1], R[2]); }, opts.libri_chi0_threshold_C);
    const std::vector<long long> &cs_off = csf.off;
    const std::vector<int> &cs_meta = csf.meta;

    // Coulomb blocks per IBZ q (upper pairs)
    std::vector<std::vector<int>> vq_of_q(nq);
    for (size_t bi = 0; bi < ds.vq_blocks.size(); ++bi)
    {
        const VqBlock &b = ds.vq_blocks[bi];
        for (int q = 0; q < nq; ++q)
            if (ibz_rep[q] == b.ik && b.I <= b.J) vq_of_q[q].push_back(static_cast<int>(bi));
    }

    // ------------------------------------------------------------ device staging
    cudaStream_t st;
    GB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard
    {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{st};
    long long launches = 0;
    const double t_up0 = wall_seconds();
    auto d_ao_off = to_dev(ao_off, st);
    auto d_nao = to_dev(ds.nao_at, st);
    auto d_nabf = to_dev(ds.nabf_at, st);
    auto d_rowc = to_dev(rowc_off, st);
    auto d_cdiff = to_dev(cdiff, st);
    auto d_cneg = to_dev(cneg, st);
    auto d_gcos = to_dev(gcos, st);
    auto d_gsin = to_dev(gsin, st);
    auto d_qcos = to_dev(qcos, st);
    auto d_qsin = to_dev(qsin, st);
    auto d_pI = to_dev(pI, st);
    auto d_pJ = to_dev(pJ, st);
    auto d_roff = to_dev(r_off, st);
    auto d_eoff = to_dev(e_off, st);
    auto d_pair_of = to_dev(pair_of, st);
    auto d_atom_of = to_dev(atom_of, st);
    std::vector<int> abf_off_n(abf_off.begin(), abf_off.end() - 1);
    auto d_abf_off = to_dev(abf_off_n, st);
    // Inputs staged once per input generation (reused while no setter ran).  Their device buffers
    // are kept with the handler: a call that re-stages (a setter ran, or reuse_device_inputs = 0)
    // copies into them again when the sizes still fit, instead of freeing and allocating ~1 GB.
    struct DeviceInputs
    {
        unsigned long long generation = 0;
        int device = -1;
        DevBuf<double> ekb, wg, C, csblob;
        DevBuf<cuDoubleComplex> psi, vblob;
        long long rows_c = 0, n_sup = 0;
    };
    std::shared_ptr<DeviceInputs> din = std::static_pointer_cast<DeviceInputs>(ds.dev_cache);
    const bool reuse = go.reuse_device_inputs && din && din->generation == ds.generation &&
                       din->device == go.device && din->rows_c == rows_c && din->n_sup == n_sup;
    double h2d = 0.0;
    if (!reuse)
    {
        const size_t n_cs = ds.cs_blob.size() + csf.extra.size();
        const bool fits = din && din->device == go.device && din->rows_c == rows_c && din->n_sup == n_sup &&
                          din->ekb.size() == ds.ekb.size() &&
                          din->wg.size() == ds.wg.size() && din->psi.size() == ds.wfc.size() &&
                          din->vblob.size() == ds.vq_blob.size() && din->csblob.size() == n_cs;
        if (!fits)
        {
            ds.dev_cache.reset();
            din.reset();
            din = std::make_shared<DeviceInputs>();
            din->device = go.device;
            din->rows_c = rows_c;
            din->n_sup = n_sup;
            din->ekb.alloc(ds.ekb.size());
            din->wg.alloc(ds.wg.size());
            din->psi.alloc(ds.wfc.size());
            din->vblob.alloc(ds.vq_blob.size());
            din->csblob.alloc(n_cs);
            din->C.alloc(static_cast<size_t>(rows_c) * n_sup);
        }
        din->generation = ds.generation;
        din->ekb.upload(ds.ekb.data(), ds.ekb.size(), st);
        din->wg.upload(ds.wg.data(), ds.wg.size(), st);
        din->psi.upload(reinterpret_cast<const cuDoubleComplex *>(ds.wfc.data()), ds.wfc.size(), st);
        din->vblob.upload(reinterpret_cast<const cuDoubleComplex *>(ds.vq_blob.data()), ds.vq_blob.size(), st);
        DevBuf<double> &d_csblob = din->csblob;
        d_csblob.upload(ds.cs_blob.data(), ds.cs_blob.size(), st);
        if (!csf.extra.empty())
            GB_CUDA(cudaMemcpyAsync(d_csblob.get() + ds.cs_blob.size(), csf.extra.data(),
                                    csf.extra.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        auto d_csoff = to_dev(cs_off, st);
        auto d_csmeta = to_dev(cs_meta, st);
        h2d = 8.0 * (ds.ekb.size() + ds.wg.size() + ds.cs_blob.size()) + 16.0 * (ds.wfc.size() + ds.vq_blob.size());
        din->C.zero(st);
        Geom gs;
        gs.n_at = n_at;
        gs.n_c = nc;
        gs.n_ao = nao;
        gs.n_sup = static_cast<int>(n_sup);
        gs.ao_off = d_ao_off.get();
        gs.nao = d_nao.get();
        gs.nabf = d_nabf.get();
        gs.rowc_off = d_rowc.get();
        launch_cs_scatter(d_csblob.get(), d_csoff.get(), d_csmeta.get(), static_cast<int>(cs_off.size()), gs,
                          din->C.get(), st);
        ++launches;
        GB_CUDA(cudaStreamSynchronize(st));
        ds.dev_cache = din;
    }
    S.h2d_bytes = h2d;
    DevBuf<double> &d_ekb = din->ekb, &d_wg = din->wg;
    DevBuf<cuDoubleComplex> &d_psi = din->psi;

    Geom g;
    g.n_at = n_at;
    g.n_c = nc;
    g.n_ao = nao;
    g.n_sup = static_cast<int>(n_sup);
    g.max_nao = max_nao;
    g.max_nabf = max_nabf;
    g.rows_c = rows_c;
    g.ao_off = d_ao_off.get();
    g.nao = d_nao.get();
    g.nabf = d_nabf.get();
    g.rowc_off = d_rowc.get();
    g.cdiff = d_cdiff.get();
    g.cneg = d_cneg.get();
    Pairs pr;
    pr.n_pairs = n_pairs;
    pr.I = d_pI.get();
    pr.J = d_pJ.get();
    pr.r_off = d_roff.get();
    pr.e_off = d_eoff.get();
    pr.e_total = e_tot;

    DevBuf<double> &d_C = din->C;
    GB_CUDA(cudaStreamSynchronize(st));
    S.t_upload = wall_seconds() - t_up0;

    // ------------------------------------------------------------ tau loop
    const int nw = tf.n;
    DevBuf<double> d_s(2ull * nk * nb);
    // Atoms beyond the tensor-core contraction's tiles (32 NAOs and 128 ABFs per atom) run the
    // FP32 path (SIMT contraction, no limit on the ABF count; NAOs up to its shared-memory tile)
    const int prec = go.chi0_precision == LIBRPA_GB300_CHI0_BF16X3 && (max_nao > 32 || max_nabf > 128)
                         ? LIBRPA_GB300_CHI0_FP32
                         : go.chi0_precision;
    S.chi0_precision_used = prec;
    const bool tc_path = prec == LIBRPA_GB300_CHI0_BF16X3;
    DevBuf<cuDoubleComplex> d_A(tc_path ? 0 : 2ull * nk * nao * nao);
    DevBuf<double> d_G(2ull * nc * nao * nao);
    // the supercell G and FP64 X serve the FP64 and FP32 paths; the tensor-core path builds its
    // split operands from G directly
    DevBuf<double> d_Gs(tc_path ? 0 : 2ull * n_sup * n_sup);
    DevBuf<double> d_X(prec == LIBRPA_GB300_CHI0_FP64 ? 2ull * rows_c * n_sup : 0);
    DevBuf<int> d_err(1);
    d_err.zero(st);
    std::unique_ptr<GkTc> gk;
    if (tc_path)
    {
        bool psi_real = true;
        for (const auto &z : ds.wfc)
            if (z.imag() != 0.0)
            {
                psi_real = false;
                break;
            }
        gk = std::make_unique<GkTc>(nk, nb, nao, psi_real);
    }
    // Reduced-precision paths keep the chi0(R) of a batch of (tau, spin) slots and transform the
    // batch in one pass (launch_ftct_slots: chi0(q, w) read and written once per batch, not once
    // per slot); the FP64 path transforms each slot in FP64 (launch_ftct).  Batches are sized to
    // keep the slots within about 16 GB.
    const bool batch_ft = prec != LIBRPA_GB300_CHI0_FP64 && ftct_slots_smem(nc, nq, tf.n) <= 227 * 1024;
    const int n_slots_all =
        go.stage != LIBRPA_GB300_STAGE_EC
            ? (std::min(go.tau_end < 0 ? tf.n : go.tau_end, tf.n) - std::max(0, go.tau_begin)) * ns
            : 0;
    const int slot_batch =
        batch_ft ? std::max(1, std::min(n_slots_all, static_cast<int>(16.0e9 / (8.0 * std::max<long long>(r_tot, 1)))))
                 : 0;
    DevBuf<double> d_chi0R(batch_ft ? 0 : static_cast<size_t>(r_tot));
    DevBuf<double> d_slots(batch_ft ? static_cast<size_t>(slot_batch) * r_tot : 0);
    DevBuf<float2> d_qph;
    if (batch_ft)
    {
        std::vector<float2> qph(static_cast<size_t>(nq) * nc);
        for (size_t t = 0; t < qph.size(); ++t)
            qph[t] = make_float2(static_cast<float>(qcos[t]), static_cast<float>(qsin[t]));
        d_qph = to_dev(qph, st);
    }
    DevBuf<double> d_gslot(batch_ft ? static_cast<size_t>(tf.n) * slot_batch : 0);
    std::vector<double> h_gslot;
    int slots_filled = 0;
    double ftct_bytes = 0.0;
    DevBuf<cuDoubleComplex> d_chi0q(static_cast<size_t>(nw) * nq * e_tot);
    d_chi0q.zero(st);
    DevBuf<double> d_gamma(static_cast<size_t>(nw));

    std::unique_ptr<Chi0Fast> fast;
    if (prec != LIBRPA_GB300_CHI0_FP64) fast = std::make_unique<Chi0Fast>(prec, g, pr, d_C.get(), st);

    // ---- block screening set-up
    const int smode = go.screen_mode;
    GB_REQUIRE(smode == LIBRPA_GB300_SCREEN_OFF || smode == LIBRPA_GB300_SCREEN_THRESHOLD ||
                   smode == LIBRPA_GB300_SCREEN_MLP,
               "unknown screen_mode " + std::to_string(smode));
    const double sthr = go.screen_threshold;
    const double thr_g = opts.libri_chi0_threshold_G;
    const int n_blk = n_pairs * nc;
    DevBuf<double> d_bnorm;
    DevBuf<float> d_feat, d_pred, d_dist, d_cmax, d_kind;
    std::vector<double> h_norm;
    std::vector<float> h_feat, h_pred;
    std::vector<unsigned char> active, audited;
    long long blk_computed = 0, blk_audited = 0, fallbacks = 0;
    double audit_max = 0.0;
    std::mt19937_64 audit_rng(go.seed);
    if (smode != LIBRPA_GB300_SCREEN_OFF)
    {
        GB_REQUIRE(sthr >= 0.0, "screen_threshold must be >= 0");
        // block distance |tau_J + R - tau_I| (Bohr) and the largest |C| of each atom's RI blocks
        std::vector<float> dist(n_blk), cmax(n_at, 0.0f);
        for (int p = 0; p < n_pairs; ++p)
            for (int c = 0; c < nc; ++c)
            {
                double d2 = 0.0;
                for (int d = 0; d < 3; ++d)
                {
                    double Rc = 0.0;
                    for (int a = 0; a < 3; ++a) Rc += cells.R[c][a] * ds.latvec[a * 3 + d];
                    const double pi = ds.positions.size() >= 3ull * n_at ? ds.positions[3 * pI[p] + d] : 0.0;
                    const double pj = ds.positions.size() >= 3ull * n_at ? ds.positions[3 * pJ[p] + d] : 0.0;
                    d2 += (pj + Rc - pi) * (pj + Rc - pi);
                }
                dist[static_cast<size_t>(p) * nc + c] = static_cast<float>(std::sqrt(d2));
            }
        for (const CsBlock &b : ds.cs_blocks)
        {
            const size_t n = static_cast<size_t>(b.ni) * b.nj * b.nmu;
            double mx = 0.0;
            for (size_t t = 0; t < n; ++t) mx = std::max(mx, std::fabs(ds.cs_blob[b.offset + t]));
            cmax[b.I] = std::max(cmax[b.I], static_cast<float>(mx));
        }
        d_dist.alloc(n_blk);
        d_dist.upload(dist.data(), n_blk, st);
        d_cmax.alloc(n_at);
        d_cmax.upload(cmax.data(), n_at, st);
        // species of each atom: the type given to librpa_set_atoms (0 when none was given)
        std::vector<float> kind(n_at, 0.0f);
        if (static_cast<int>(ds.types.size()) >= n_at)
            for (int I = 0; I < n_at; ++I) kind[I] = static_cast<float>(ds.types[I]);
        d_kind.alloc(n_at);
        d_kind.upload(kind.data(), n_at, st);
        d_bnorm.alloc(n_blk);
        d_feat.alloc(static_cast<size_t>(n_blk) * MLP_IN);
        h_norm.resize(n_blk);
        h_feat.resize(static_cast<size_t>(n_blk) * MLP_IN);
    }
    TcChi0 *tcp = nullptr;
    if (smode == LIBRPA_GB300_SCREEN_MLP)
    {
        tcp = fast ? fast->tensor_path() : nullptr;
        GB_REQUIRE(tcp, "learned screening needs the tensor-core chi0 path (chi0_precision = BF16X3)");
        if (!ds.screen_model.trained)
        {
            GB_REQUIRE(ds.screen_log.size() >= 16,
                       "learned screening needs a trained model: run with plain threshold screening first "
                       "(its block norms are the training data) or call librpa_gb300_train_screening");
            mlp_train(ds.screen_model, ds.screen_log.x, ds.screen_log.y, 600, 3e-3, go.seed, st);
        }
        d_pred.alloc(n_blk);
        h_pred.resize(n_blk);
        active.resize(n_blk);
        audited.resize(n_blk);
    }

    EventTimer ev_gf, ev_x, ev_chi, ev_ft;
    double t_gf = 0, t_chi = 0, t_ft = 0;
    double flops_chi = 0.0, flops_libri = 0.0;
    S.dt_chi0_kernel_ms = 0.0;
    S.n_chi0_kernel = 0;
    const double fac = 2.0 / ns;
    // tau slice and stage (tau sharding: partial chi0(q, omega) sums are reduced across ranks)
    const int tb = std::max(0, go.tau_begin), te = go.tau_end < 0 ? nw : std::min(go.tau_end, nw);
    GB_REQUIRE(go.stage >= LIBRPA_GB300_STAGE_FULL && go.stage <= LIBRPA_GB300_STAGE_EC, "unknown stage");
    GB_REQUIRE(tb <= te, "tau_begin > tau_end");
    const bool do_chi0 = go.stage != LIBRPA_GB300_STAGE_EC;
    if (!do_chi0)
    {
        GB_REQUIRE(ds.kept_chi0 && ds.kept_chi0_bytes == d_chi0q.bytes(),
                   "STAGE_EC needs the chi0(q, omega) of a STAGE_CHI0 call on the same data (librpa_gb300_load_chi0_qw)");
        GB_CUDA(cudaMemcpyAsync(d_chi0q.get(), ds.kept_chi0, ds.kept_chi0_bytes, cudaMemcpyDeviceToDevice, st));
    }
    for (int it = do_chi0 ? tb : te; it < te; ++it)
    {
        const double tau = tf.tau[it];
        std::vector<double> gam(nw);
        for (int w = 0; w < nw; ++w) gam[w] = tf.cos_t2f[static_cast<size_t>(w) * nw + it];
        d_gamma.upload(gam.data(), nw, st);
        for (int is = 0; is < ns; ++is)
        {
            double *chi0R_cur = batch_ft ? d_slots.get() + static_cast<size_t>(slots_filled) * r_tot : d_chi0R.get();
            ev_gf.start(st);
            launch_tau_scale(d_ekb.get() + static_cast<size_t>(is) * nk * nb, d_wg.get() + static_cast<size_t>(is) * nk * nb,
                             nk, nb, ds.efermi, tau, ns, nbands_g, d_s.get(), st);
            if (gk)
                launches += 1 + gk->run(d_psi.get() + static_cast<size_t>(is) * nk * nb * nao, d_s.get(), d_gcos.get(),
                                        d_gsin.get(), nc, d_G.get(), d_err.get(), st);
            else
            {
                launch_gk_build(d_psi.get() + static_cast<size_t>(is) * nk * nb * nao, d_s.get(), nk, nb, nao, d_A.get(), st);
                launch_phase_sum(d_A.get(), d_gcos.get(), d_gsin.get(), nk, nc, nao, d_G.get(), st);
                launches += 3;
            }
            if (thr_g > 0.0)
            {
                launch_g_block_filter(d_G.get(), g, thr_g, st);  // LibRI set_Gs_pos / set_Gs_neg filter
                ++launches;
            }
            if (!gk)
            {
                launch_gsuper(d_G.get(), g, d_Gs.get(), st);  // from the filtered blocks
                ++launches;
            }
            ev_gf.stop(st);
            t_gf += ev_gf.ms();
            ev_chi.start(st);
            const double *Gp = d_G.get(), *Gm = d_G.get() + static_cast<size_t>(nc) * nao * nao;
            if (prec == LIBRPA_GB300_CHI0_FP64)
            {
                launch_dgemm(static_cast<int>(rows_c), static_cast<int>(n_sup), static_cast<int>(n_sup), d_C.get(), n_sup, 0,
                             d_Gs.get(), n_sup, n_sup * n_sup, d_X.get(), n_sup, rows_c * n_sup, 2, 1.0, 0.0, st);
                ev_x.start(st);
                launch_chi0_fp64(d_X.get(), d_X.get() + rows_c * n_sup, d_C.get(), Gp, Gm, g, pr, chi0R_cur, st);
                ev_x.stop(st);
                launches += 2;
            }
            else if (smode == LIBRPA_GB300_SCREEN_MLP)
            {
                // predicted block norms -> contract the blocks above the threshold and an audit
                // share of the rest; an audited block above the threshold means fall back
                ev_x.start(st);
                launches += tcp->prepare(d_G.get(), st);
                launch_block_features(d_G.get(), g, pr, d_dist.get(), d_cmax.get(), d_kind.get(), tau, d_feat.get(), st);
                mlp_predict(ds.screen_model, d_feat.get(), n_blk, d_pred.get(), st);
                launches += 3;
                d_pred.download(h_pred.data(), n_blk, st);
                GB_CUDA(cudaStreamSynchronize(st));
                const double cut = std::log10(std::max(sthr, 1e-300)) - ds.screen_model.norm[MLP_NNORM - 1];
                std::uniform_real_distribution<double> u01(0.0, 1.0);
                long long n_act = 0;
                for (int b = 0; b < n_blk; ++b)
                {
                    const bool keep = h_pred[b] > cut;
                    audited[b] = !keep && u01(audit_rng) < go.audit_fraction;
                    active[b] = keep || audited[b];
                    n_act += active[b];
                    blk_audited += audited[b];
                }
                launches += tcp->contract(d_G.get(), chi0R_cur, active.data(), true, st);
                launch_block_maxnorm(chi0R_cur, g, pr, d_bnorm.get(), st);
                ++launches;
                d_bnorm.download(h_norm.data(), n_blk, st);
                GB_CUDA(cudaStreamSynchronize(st));
                bool violated = false;
                for (int b = 0; b < n_blk; ++b)
                    if (audited[b])
                    {
                        audit_max = std::max(audit_max, h_norm[b]);
                        violated = violated || h_norm[b] > sthr;
                    }
                if (violated)
                {
                    for (int b = 0; b < n_blk; ++b) active[b] = !active[b];
                    launches += tcp->contract(d_G.get(), chi0R_cur, active.data(), false, st);
                    launch_block_maxnorm(chi0R_cur, g, pr, d_bnorm.get(), st);
                    ++launches;
                    n_act = n_blk;
                    ++fallbacks;
                }
                blk_computed += n_act;
                ev_x.stop(st);
            }
            else
            {
                ev_x.start(st);
                launches += fast->run(d_Gs.get(), Gp, Gm, chi0R_cur, st);
                ev_x.stop(st);
            }
            if (smode == LIBRPA_GB300_SCREEN_THRESHOLD)
            {
                // plain screening: every block computed; its features and norm are logged
                launch_block_maxnorm(chi0R_cur, g, pr, d_bnorm.get(), st);
                launch_block_features(d_G.get(), g, pr, d_dist.get(), d_cmax.get(), d_kind.get(), tau, d_feat.get(), st);
                launches += 2;
                d_bnorm.download(h_norm.data(), n_blk, st);
                d_feat.download(h_feat.data(), h_feat.size(), st);
                GB_CUDA(cudaStreamSynchronize(st));
                ds.screen_log.x.insert(ds.screen_log.x.end(), h_feat.begin(), h_feat.end());
                for (int b = 0; b < n_blk; ++b)
                    ds.screen_log.y.push_back(h_norm[b] > 0.0 ? static_cast<float>(std::log10(h_norm[b])) : -40.0f);
                blk_computed += n_blk;
            }
            if (smode != LIBRPA_GB300_SCREEN_OFF)
            {
                launch_block_drop(chi0R_cur, g, pr, d_bnorm.get(), sthr, st);  // keep max-norm > threshold
                ++launches;
            }
            ev_chi.stop(st);
            t_chi += ev_chi.ms();
            S.dt_chi0_kernel_ms += ev_x.ms();
            S.n_chi0_kernel += 1;
            ev_ft.start(st);
            if (batch_ft)
            {
                // this slot's column of the transform; the batch runs once full or at the last slot
                for (int w = 0; w < nw; ++w) h_gslot.push_back(fac * gam[w]);
                ++slots_filled;
                if (slots_filled == slot_batch || (it == te - 1 && is == ns - 1))
                {
                    std::vector<double> gt(static_cast<size_t>(nw) * slots_filled);  // [w][slot]
                    for (int sl = 0; sl < slots_filled; ++sl)
                        for (int w = 0; w < nw; ++w)
                            gt[static_cast<size_t>(w) * slots_filled + sl] = h_gslot[static_cast<size_t>(sl) * nw + w];
                    d_gslot.upload(gt.data(), gt.size(), st);
                    launch_ftct_slots(d_slots.get(), r_tot, slots_filled, g, pr, d_qph.get(), nq, d_gslot.get(), nw,
                                      d_chi0q.get(), st);
                    ++launches;
                    ftct_bytes += 8.0 * r_tot * slots_filled + 2.0 * 16.0 * nw * nq * e_tot;
                    GB_CUDA(cudaStreamSynchronize(st));  // the slots and gt are reused after this
                    h_gslot.clear();
                    slots_filled = 0;
                }
            }
            else
            {
                launch_ftct(chi0R_cur, g, pr, d_qcos.get(), d_qsin.get(), nq, d_gamma.get(), nw, fac, d_chi0q.get(), st);
                ++launches;
                ftct_bytes += 8.0 * r_tot + 2.0 * 16.0 * nw * nq * e_tot;
            }
            ev_ft.stop(st);
            t_ft += ev_ft.ms();
        }
    }
    // FLOP counts per tau and spin.
    //  ours: X GEMMs 2 * 2 rows_c n_sup^2; per upper (pair, cell) and pass:
    //        E = g^T X (2 bI aI aJ n_sup), T1 (2 bI bJ aJ n_sup), T2 (2 bI bJ aI aJ)
    //  LibRI (all ordered pairs, both passes), LRI-cal_loop3.hpp:902-1032:
    //   a1b1_a2b2: sum_I 2 bI aI n_sup^2 + sum_{I,J} nc (2 aJ bI aI + 2 bI bJ aJ) n_sup
    //   a1b2_a2b1: sum_{I,J} nc (2 bJ aJ aI n_sup + 2 aJ aI bI n_sup + 2 bI bJ aJ aI)
    {
        double per = 2.0 * 2.0 * static_cast<double>(rows_c) * n_sup * n_sup;
        for (int p = 0; p < n_pairs; ++p)
        {
            const double aI = ds.nao_at[pI[p]], aJ = ds.nao_at[pJ[p]], bI = ds.nabf_at[pI[p]], bJ = ds.nabf_at[pJ[p]];
            per += nc * 2.0 * (2.0 * bI * aI * aJ * n_sup + 2.0 * bI * bJ * aJ * n_sup + 2.0 * bI * bJ * aI * aJ);
        }
        double lib = 0.0;
        for (int I = 0; I < n_at; ++I)
        {
            const double aI = ds.nao_at[I], bI = ds.nabf_at[I];
            lib += 2.0 * bI * aI * static_cast<double>(n_sup) * n_sup;
            for (int J = 0; J < n_at; ++J)
            {
                const double aJ = ds.nao_at[J], bJ = ds.nabf_at[J];
                lib += nc * (2.0 * aJ * bI * aI + 2.0 * bI * bJ * aJ) * n_sup;
                lib += nc * (2.0 * bJ * aJ * aI * n_sup + 2.0 * aJ * aI * bI * n_sup + 2.0 * bI * bJ * aJ * aI);
            }
        }
        flops_chi = per * (do_chi0 ? te - tb : 0) * ns;
        flops_libri = 2.0 * lib * (do_chi0 ? te - tb : 0) * ns;
    }
    {
        int herr = 0;
        d_err.download(&herr, 1, st);
        GB_CUDA(cudaStreamSynchronize(st));
        GB_REQUIRE(herr == 0, "tensor-core G build reported wait timeout code " + std::to_string(herr));
    }
    if (TcChi0 *tp = fast ? fast->tensor_path() : nullptr)
    {
        int nar = 0, kp = 0;
        tp->launch_choice(nar, kp);
        S.t1_narrow = nar;
        S.t1_kparts = kp;
    }
    S.t_gf = t_gf * 1e-3;
    S.t_chi0 = t_chi * 1e-3;
    S.t_ftct = t_ft * 1e-3;
    S.chi0_flops = flops_chi;
    S.chi0_flops_libri = flops_libri;
    S.gf_flops = static_cast<double>(do_chi0 ? te - tb : 0) * ns * 2.0 * (8.0 * nk * nao * nao * nb + 4.0 * nc * nk * nao * nao);
    S.ftct_bytes = ftct_bytes;
    d_X.release();
    d_Gs.release();
    fast.reset();

    if (go.stage == LIBRPA_GB300_STAGE_CHI0)
    {
        // keep the partial chi0(q, w) and stop before E_c
        release_kept(ds);
        ds.kept_chi0_bytes = d_chi0q.bytes();
        GB_CUDA(cudaMalloc(&ds.kept_chi0, ds.kept_chi0_bytes));
        GB_CUDA(cudaMemcpyAsync(ds.kept_chi0, d_chi0q.get(), ds.kept_chi0_bytes, cudaMemcpyDeviceToDevice, st));
        ds.kept_pair_offset.assign(e_off.begin(), e_off.end());
        ds.kept_pair_elems = static_cast<size_t>(e_tot);
        ds.kept_nfreq = nw;
        ds.kept_nq = nq;
        GB_CUDA(cudaStreamSynchronize(st));
        S.n_launches = launches;
        S.blocks_total = static_cast<long long>(n_blk) * (te - tb) * ns;
        S.blocks_computed = smode == LIBRPA_GB300_SCREEN_OFF ? S.blocks_total : blk_computed;
        S.t_total = wall_seconds() - t_begin;
        RpaResult part;
        part.per_q.assign(nq, cplx(0, 0));
        return part;
    }

    // ------------------------------------------------------------ E_c
    EventTimer ev_ec;
    ev_ec.start(st);
    const bool gamma_only = (nk == 1);
    RpaResult res;
    res.per_q.assign(nq, cplx(0, 0));
    // q sharding: this call's E_c covers the IBZ q points [qa, qe)
    const int qa = std::max(0, go.q_begin), qe = go.q_end < 0 ? nq : std::min(go.q_end, nq);
    GB_REQUIRE(qa <= qe, "q_begin > q_end");
    // The basis E_c runs in: the ABFs of chi0, or with use_shrink_abfs the small ABFs of the
    // Coulomb matrix, chi0(q, w) taken there by U(q) chi0 U(q)^H (shrink_abfs_chi0,
    // chi0.cpp:711-898).  The reference transforms chi0(q, tau) ahead of the cosine transform
    // (chi0.cpp:1110-1137); both steps are linear, so transforming chi0(q, w) is the same.
    const bool shrink = opts.use_shrink_abfs == LIBRPA_SWITCH_ON;
    const std::vector<int> &nabf_e = shrink ? ds.shrink_nabf : ds.nabf_at;
    int Ne = N;
    long long e_tot_e = e_tot;
    const cuDoubleComplex *chi0_e = d_chi0q.get();
    const int *atom_of_e = d_atom_of.get(), *abf_off_e = d_abf_off.get(), *nabf_dev_e = d_nabf.get();
    const long long *eoff_e = d_eoff.get();
    DevBuf<int> d_atom_of_s, d_abf_off_s, d_nabf_s;
    DevBuf<long long> d_eoff_s;
    DevBuf<cuDoubleComplex> d_chi0q_s;
    if (shrink)
    {
        GB_REQUIRE(static_cast<int>(ds.shrink_nabf.size()) == n_at,
                   "use_shrink_abfs: the small ABF basis must be set for every atom (librpa_gb300_set_shrink_basis)");
        std::vector<int> abf_off_s(n_at + 1, 0);
        for (int I = 0; I < n_at; ++I)
        {
            GB_REQUIRE(ds.shrink_nabf[I] > 0, "use_shrink_abfs: small ABF counts must be positive");
            abf_off_s[I + 1] = abf_off_s[I] + ds.shrink_nabf[I];
        }
        Ne = abf_off_s[n_at];
        std::vector<int> atom_of_s(Ne);
        for (int I = 0; I < n_at; ++I)
            for (int a = abf_off_s[I]; a < abf_off_s[I + 1]; ++a) atom_of_s[a] = I;
        std::vector<long long> e_off_s;
        e_tot_e = 0;
        for (int p = 0; p < n_pairs; ++p)
        {
            e_off_s.push_back(e_tot_e);
            e_tot_e += static_cast<long long>(ds.shrink_nabf[pI[p]]) * ds.shrink_nabf[pJ[p]];
        }
        abf_off_s.pop_back();
        d_atom_of_s = to_dev(atom_of_s, st);
        d_abf_off_s = to_dev(abf_off_s, st);
        d_nabf_s = to_dev(ds.shrink_nabf, st);
        d_eoff_s = to_dev(e_off_s, st);
        d_chi0q_s.alloc(static_cast<size_t>(nw) * nq * e_tot_e);
        d_chi0q_s.zero(st);
        const long long NL2 = static_cast<long long>(N) * N, NSL = static_cast<long long>(Ne) * N,
                        NS2 = static_cast<long long>(Ne) * Ne;
        DevBuf<cuDoubleComplex> XL(static_cast<size_t>(nw) * NL2), T(static_cast<size_t>(nw) * NSL),
            XS(static_cast<size_t>(nw) * NS2), U(NSL), UH(NSL);
        std::vector<cuDoubleComplex> hu(NSL), huh(NSL);
        for (int q = qa; q < qe; ++q)
        {
            auto it = ds.shrink_u.find(ibz_rep[q]);
            GB_REQUIRE(it != ds.shrink_u.end(), "use_shrink_abfs: no shrink transform U(q) for IBZ k index " +
                                                    std::to_string(ibz_rep[q]) + " (librpa_gb300_set_shrink_sinvS)");
            const Dataset::ShrinkU &su = it->second;
            GB_REQUIRE(su.n_small == Ne && su.n_large == N,
                       "use_shrink_abfs: U(q) must be (sum of small ABFs) x (sum of ABFs) = " + std::to_string(Ne) +
                           " x " + std::to_string(N));
            for (int r = 0; r < Ne; ++r)
                for (int c = 0; c < N; ++c)
                {
                    const cplx v = su.u[static_cast<size_t>(r) * N + c];
                    // the Gamma-point E_c is real (epsilon.cpp:43-268): a complex U(Gamma) would
                    // leave an imaginary part that path drops
                    GB_REQUIRE(!gamma_only || v.imag() == 0.0, "use_shrink_abfs: U(q) must be real at the Gamma point");
                    hu[static_cast<size_t>(r) * N + c] = make_cuDoubleComplex(v.real(), v.imag());
                    huh[static_cast<size_t>(c) * Ne + r] = make_cuDoubleComplex(v.real(), -v.imag());
                }
            U.upload(hu.data(), NSL, st);
            UH.upload(huh.data(), NSL, st);
            // chi0(q, w) of the large basis in full (Hermitian fill), then U chi0 U^H per w
            launch_assemble_chi0(d_chi0q.get() + static_cast<long long>(q) * e_tot, static_cast<long long>(nq) * e_tot, nw,
                                 N, d_atom_of.get(), d_abf_off.get(), d_nabf.get(), d_pair_of.get(), n_at, d_eoff.get(),
                                 false, XL.get(), nullptr, NL2, st);
            launch_zgemm(Ne, N, N, U.get(), N, 0, XL.get(), N, NL2, T.get(), N, NSL, nw, st);
            launch_zgemm(Ne, Ne, N, T.get(), N, NSL, UH.get(), Ne, 0, XS.get(), Ne, NS2, nw, st);
            launch_scatter_pairs(XS.get(), NS2, nw, Ne, d_pI.get(), d_pJ.get(), n_pairs, d_abf_off_s.get(),
                                 d_nabf_s.get(), d_eoff_s.get(), d_chi0q_s.get() + static_cast<long long>(q) * e_tot_e,
                                 static_cast<long long>(nq) * e_tot_e, st);
            launches += 4;
            GB_CUDA(cudaStreamSynchronize(st));  // hu / huh are refilled for the next q
        }
        chi0_e = d_chi0q_s.get();
        atom_of_e = d_atom_of_s.get();
        abf_off_e = d_abf_off_s.get();
        nabf_dev_e = d_nabf_s.get();
        eoff_e = d_eoff_s.get();
    }
    const long long NN = static_cast<long long>(Ne) * Ne;
    double ec_flops = 0.0;
    GB_REQUIRE(go.ec_path == LIBRPA_GB300_EC_LU_FP64 || go.ec_path == LIBRPA_GB300_EC_CHOL ||
                   go.ec_path == LIBRPA_GB300_EC_CHOL_FP64,
               "unknown ec_path " + std::to_string(go.ec_path));
    const bool use_chol = go.ec_path != LIBRPA_GB300_EC_LU_FP64;
    // V(q) from the blocks of this q inside the staged Coulomb blob
    auto assemble_v = [&](int q, void *V) {
        std::vector<long long> voff;
        std::vector<int> vIJ;
        for (int bi : vq_of_q[q])
        {
            const VqBlock &b = ds.vq_blocks[bi];
            GB_REQUIRE(b.nmu == nabf_e[b.I] && b.nnu == nabf_e[b.J], "Coulomb block dimensions inconsistent");
            voff.push_back(static_cast<long long>(b.offset));
            vIJ.push_back(b.I);
            vIJ.push_back(b.J);
        }
        auto d_voff = to_dev(voff, st);
        auto d_vIJ = to_dev(vIJ, st);
        if (gamma_only)
        {
            GB_CUDA(cudaMemsetAsync(V, 0, sizeof(double) * NN, st));
            launch_assemble_v(din->vblob.get(), d_voff.get(), d_vIJ.get(), static_cast<int>(voff.size()), abf_off_e,
                              nabf_dev_e, Ne, true, nullptr, static_cast<double *>(V), st);
        }
        else
        {
            GB_CUDA(cudaMemsetAsync(V, 0, sizeof(cuDoubleComplex) * NN, st));
            launch_assemble_v(din->vblob.get(), d_voff.get(), d_vIJ.get(), static_cast<int>(voff.size()), abf_off_e,
                              nabf_dev_e, Ne, false, static_cast<cuDoubleComplex *>(V), nullptr, st);
        }
        GB_CUDA(cudaStreamSynchronize(st));  // the block tables go out of scope
        ++launches;
    };
    // Reference form for one q: Pi = V chi0 in FP64, LU with partial pivoting, sum log(+-u_ii)
    // + tr Pi (epsilon.cpp:414-536).  It needs no definiteness of V(q).
    auto ec_lu_q = [&](int q)
    {
        // V(q) full: blocks of this q inside the staged Coulomb blob
        std::vector<long long> voff;
        std::vector<int> vIJ;
        for (int bi : vq_of_q[q])
        {
            const VqBlock &b = ds.vq_blocks[bi];
            GB_REQUIRE(b.nmu == nabf_e[b.I] && b.nnu == nabf_e[b.J], "Coulomb block dimensions inconsistent");
            voff.push_back(static_cast<long long>(b.offset));
            vIJ.push_back(b.I);
            vIJ.push_back(b.J);
        }
        auto d_voff = to_dev(voff, st);
        auto d_vIJ = to_dev(vIJ, st);
        const cuDoubleComplex *vbase = din->vblob.get();
        std::vector<double> tr_h(gamma_only ? nw : 2 * nw), ld_h(gamma_only ? nw : 2 * nw);
        if (gamma_only)
        {
            DevBuf<double> V(NN), X(NN * nw), P(NN * nw), tr(nw), ld(nw);
            V.zero(st);
            launch_assemble_v(vbase, d_voff.get(), d_vIJ.get(), static_cast<int>(voff.size()), abf_off_e,
                              nabf_dev_e, Ne, true, nullptr, V.get(), st);
            launch_assemble_chi0(chi0_e + static_cast<long long>(q) * e_tot_e, static_cast<long long>(nq) * e_tot_e, nw, Ne,
                                 atom_of_e, abf_off_e, nabf_dev_e, d_pair_of.get(), n_at, eoff_e, true,
                                 nullptr, X.get(), NN, st);
            launch_dgemm(Ne, Ne, Ne, V.get(), Ne, 0, X.get(), Ne, NN, P.get(), Ne, NN, nw, 1.0, 0.0, st);
            launch_trace_and_negate_r(P.get(), Ne, nw, tr.get(), st);
            launch_lu_logdet_r(P.get(), Ne, nw, ld.get(), st);
            launches += 5;
            tr.download(tr_h.data(), nw, st);
            ld.download(ld_h.data(), nw, st);
            GB_CUDA(cudaStreamSynchronize(st));
            for (int w = 0; w < nw; ++w)
            {
                const cplx v = cplx(tr_h[w] + ld_h[w], 0.0) * tf.omega_w[w] * ibz_w[q] / (2.0 * M_PI);
                res.per_q[q] += v;
            }
            ec_flops += nw * (2.0 * Ne * Ne * Ne + 2.0 * Ne * Ne * Ne / 3.0);
        }
        else
        {
            DevBuf<cuDoubleComplex> V(NN), X(NN * nw), P(NN * nw), tr(nw), ld(nw);
            V.zero(st);
            launch_assemble_v(vbase, d_voff.get(), d_vIJ.get(), static_cast<int>(voff.size()), abf_off_e,
                              nabf_dev_e, Ne, false, V.get(), nullptr, st);
            launch_assemble_chi0(chi0_e + static_cast<long long>(q) * e_tot_e, static_cast<long long>(nq) * e_tot_e, nw, Ne,
                                 atom_of_e, abf_off_e, nabf_dev_e, d_pair_of.get(), n_at, eoff_e, false,
                                 X.get(), nullptr, NN, st);
            launch_zgemm(Ne, Ne, Ne, V.get(), Ne, 0, X.get(), Ne, NN, P.get(), Ne, NN, nw, st);
            launch_trace_and_negate_c(P.get(), Ne, nw, tr.get(), st);
            launch_lu_logdet_c(P.get(), Ne, nw, ld.get(), st);
            launches += 5;
            tr.download(reinterpret_cast<cuDoubleComplex *>(tr_h.data()), nw, st);
            ld.download(reinterpret_cast<cuDoubleComplex *>(ld_h.data()), nw, st);
            GB_CUDA(cudaStreamSynchronize(st));
            for (int w = 0; w < nw; ++w)
            {
                const cplx v = (cplx(tr_h[2 * w], tr_h[2 * w + 1]) + cplx(ld_h[2 * w], ld_h[2 * w + 1])) *
                               tf.omega_w[w] * ibz_w[q] / (2.0 * M_PI);
                res.per_q[q] += v;
            }
            ec_flops += nw * (8.0 * Ne * Ne * Ne + 8.0 * Ne * Ne * Ne / 3.0);
        }
    };
    int lu_fallback_q = 0;
    if (use_chol)
    {
        // every q's V = L L^H in one batched factorisation, M' = I - L^H chi0 L per q on the tensor
        // cores, then one batched FP64 Cholesky of all the M'; q points go in batches that keep
        // the M' store within about 24 GB
        const size_t esz = gamma_only ? sizeof(double) : sizeof(cuDoubleComplex);
        // complex M' is factored as its real 2N x 2N embedding: 32 bytes per element of M'
        const double per_q = static_cast<double>(nw) * NN * (gamma_only ? esz : 2 * esz) + NN * esz;
        const int qb = std::max(1, std::min(std::max(qe - qa, 1), static_cast<int>(24.0e9 / per_q)));
        EcChol ecc(Ne, nw, !gamma_only, qb, go.ec_path == LIBRPA_GB300_EC_CHOL_FP64);
        DevBuf<unsigned char> Vall(static_cast<size_t>(qb) * NN * esz), X(static_cast<size_t>(nw) * NN * esz);
        for (int q0 = qa; q0 < qe; q0 += qb)
        {
            const int nb = std::min(qb, qe - q0);
            for (int s = 0; s < nb; ++s) assemble_v(q0 + s, Vall.get() + static_cast<size_t>(s) * NN * esz);
            std::vector<int> badv;
            launches += ecc.factor_v(Vall.get(), nb, badv, st);
            // q whose V(q) has no Cholesky factor (an indefinite Gamma-point Coulomb matrix)
            // take the LU form; the others fill the batch slots in order
            std::vector<int> slot_q;
            for (int s = 0; s < nb; ++s)
            {
                const int q = q0 + s;
                if (badv[s])
                {
                    ec_lu_q(q);
                    ++lu_fallback_q;
                    continue;
                }
                launch_assemble_chi0(chi0_e + static_cast<long long>(q) * e_tot_e, static_cast<long long>(nq) * e_tot_e,
                                     nw, Ne, atom_of_e, abf_off_e, nabf_dev_e, d_pair_of.get(), n_at,
                                     eoff_e, gamma_only,
                                     gamma_only ? nullptr : reinterpret_cast<cuDoubleComplex *>(X.get()),
                                     gamma_only ? reinterpret_cast<double *>(X.get()) : nullptr, NN, st);
                launches += 1 + ecc.stage_q(Vall.get() + static_cast<size_t>(s) * NN * esz, X.get(),
                                            static_cast<int>(slot_q.size()), st);
                slot_q.push_back(q);
            }
            const int ns_ok = static_cast<int>(slot_q.size());
            if (ns_ok == 0) continue;
            std::vector<cplx> tr, ld;
            launches += ecc.finish(ns_ok, tr, ld, st);
            for (int s = 0; s < ns_ok; ++s)
                for (int w = 0; w < nw; ++w)
                    res.per_q[slot_q[s]] += (tr[s * nw + w] + ld[s * nw + w]) * tf.omega_w[w] * ibz_w[slot_q[s]] / (2.0 * M_PI);
            ec_flops += ns_ok * nw * (gamma_only ? (2.0 * 2.0 * Ne * Ne * Ne + Ne * static_cast<double>(Ne) * Ne / 3.0)
                                                 : (2.0 * 8.0 * Ne * Ne * Ne + 4.0 * Ne * static_cast<double>(Ne) * Ne / 3.0));
        }
    }
    for (int q = qa; q < qe && !use_chol; ++q) ec_lu_q(q);
    ev_ec.stop(st);
    S.t_ec = ev_ec.ms() * 1e-3;
    S.ec_flops = ec_flops;
    S.ec_lu_fallback_q = lu_fallback_q;
    for (const cplx &v : res.per_q) res.ec += v;

    // keep chi0(q, w) for inspection (a STAGE_EC call keeps the loaded one)
    if (go.stage == LIBRPA_GB300_STAGE_FULL) release_kept(ds);
    if (go.keep_chi0 && go.stage == LIBRPA_GB300_STAGE_FULL)
    {
        ds.kept_chi0_bytes = d_chi0q.bytes();
        GB_CUDA(cudaMalloc(&ds.kept_chi0, ds.kept_chi0_bytes));
        GB_CUDA(cudaMemcpyAsync(ds.kept_chi0, d_chi0q.get(), ds.kept_chi0_bytes, cudaMemcpyDeviceToDevice, st));
        ds.kept_pair_offset.assign(e_off.begin(), e_off.end());
        ds.kept_pair_elems = static_cast<size_t>(e_tot);
        ds.kept_nfreq = nw;
        ds.kept_nq = nq;
    }
    GB_CUDA(cudaStreamSynchronize(st));
    S.n_launches = launches;
    S.d2h_bytes = 16.0 * 2 * nw * nq;
    S.blocks_total = static_cast<long long>(n_blk) * (do_chi0 ? te - tb : 0) * ns;
    S.blocks_computed = smode == LIBRPA_GB300_SCREEN_OFF ? S.blocks_total : blk_computed;
    S.blocks_audited = blk_audited;
    S.audit_max_dropped = audit_max;
    S.screen_fallbacks = fallbacks;
    S.t_total = wall_seconds() - t_begin;
    return res;
}

} // namespace gb
