// chi0_main: the task = rpa / exx / g0w0 driver of LibRPA (driver/main.cpp, driver/task/rpa.cpp,
// exx.cpp, g0w0.cpp) on top of this library's C API.
//
// Reads `librpa.in` (key = value lines, '#' comments, the last occurrence of a key wins, as in
// driver/inputfile.cpp) from the working directory, reads the FHI-aims export named by
// input_dir (formats of driver/read_data.cpp), passes it through the librpa_set_* calls and
// prints the RPA correlation energy in the layout of driver/task/rpa.cpp (task = exx: the v_exx
// tables of task/exx.cpp; task = g0w0: the quasi-particle tables of task/g0w0.cpp, with the
// keys n_params_anacon, replace_w_head, option_dielect_func, sqrt_coulomb_threshold).
//
// Keys: task (rpa, exx, g0w0), input_dir, nfreq, tfgrids_type, parallel_routing, cs_threshold,
// vq_threshold, libri_chi0_threshold_C, libri_chi0_threshold_G, minimax_emin/emax, and the
// GPU controls gb300_chi0_precision (fp64 | bf16x3 | fp32), gb300_ec_path (lu | chol |
// chol_fp64), gb300_screen_mode (off | threshold | mlp), gb300_screen_threshold,
// gb300_sigma_precision (fp64 | bf16x3: the G0W0 self-energy's contraction).
// use_shrink_abfs = t reads the ABF shrink as driver/read_data.cpp:2455-2622 does: the small ABF
// count per atom from the Cs_shrinked_data headers, U(q) from shrink_sinvS_*, and the Coulomb
// matrix in the small basis.
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <dirent.h>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "librpa.h"

namespace {

using cplx = std::complex<double>;

[[noreturn]] void die(const std::string &msg)
{
    throw std::runtime_error(msg);
}

std::string trim(const std::string &s)
{
    size_t b = s.find_first_not_of(" \t\r\n"), e = s.find_last_not_of(" \t\r\n");
    return b == std::string::npos ? "" : s.substr(b, e - b + 1);
}

std::string lower(std::string s)
{
    for (auto &c : s) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    return s;
}

std::map<std::string, std::string> read_params(const std::string &fn)
{
    std::map<std::string, std::string> p;
    std::ifstream f(fn);
    if (!f) return p;
    std::string line;
    while (std::getline(f, line))
    {
        const auto h = line.find('#');
        if (h != std::string::npos) line = line.substr(0, h);
        const auto eq = line.find('=');
        if (eq == std::string::npos) continue;
        p[trim(line.substr(0, eq))] = trim(line.substr(eq + 1));  // later lines win
    }
    return p;
}

std::vector<std::string> tokens(const std::string &fn)
{
    std::ifstream f(fn);
    if (!f) die("cannot open " + fn);
    std::vector<std::string> t;
    std::string w;
    while (f >> w) t.push_back(w);
    return t;
}

std::vector<char> slurp(const std::string &fn)
{
    std::ifstream f(fn, std::ios::binary);
    if (!f) die("cannot open " + fn);
    return std::vector<char>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

std::vector<std::string> files_with_prefix(const std::string &dir, const std::string &prefix)
{
    std::vector<std::string> out;
    if (DIR *d = opendir(dir.c_str()))
    {
        while (dirent *e = readdir(d))
        {
            const std::string n = e->d_name;
            if (n.compare(0, prefix.size(), prefix) == 0) out.push_back(dir + n);
        }
        closedir(d);
    }
    std::sort(out.begin(), out.end());
    return out;
}

bool exists(const std::string &fn)
{
    std::ifstream f(fn);
    return static_cast<bool>(f);
}

// The reference's format check (check_Cs_file_binary / check_coulomb_file_binary,
// driver/read_data.cpp:414-453): a file whose first token parses as an integer is text (the
// ASCII files ABACUS writes), otherwise unformatted binary (FHI-aims).
bool is_text_file(const std::string &fn)
{
    std::ifstream f(fn);
    int v = 0;
    f >> v;
    return static_cast<bool>(f);
}

template <typename T>
T get(const std::vector<char> &raw, size_t &off)
{
    if (off + sizeof(T) > raw.size()) die("binary file ended early");
    T v;
    std::memcpy(&v, raw.data() + off, sizeof(T));
    off += sizeof(T);
    return v;
}

struct Mesh
{
    int nk = 0, ns = 0, nb = 0, nao = 0, nat = 0;
    std::vector<int> types, nao_at, nabf_at, ibz;
    int period[3] = {1, 1, 1};
    std::vector<double> kvecs;
};

} // namespace

int main()
{
    try
    {
        const auto p = read_params("librpa.in");
        auto par = [&](const std::string &k, const std::string &d) { return p.count(k) ? p.at(k) : d; };
        // task = g0w0_band runs the k-grid part of driver/task/g0w0_band.cpp; the band path along
        // band_kpath_info is skipped, as the reference skips it when that file is absent
        const std::string task_in = lower(par("task", "rpa"));
        const bool band_task = task_in == "g0w0_band";
        const std::string task = band_task ? "g0w0" : task_in;
        if (task != "rpa" && task != "exx" && task != "g0w0")
            die("this driver runs task = rpa, exx, g0w0 or g0w0_band (got " + task_in + ")");
        std::string dir = par("input_dir", "./");
        if (dir.back() != '/') dir += '/';
        const double cs_threshold = std::stod(par("cs_threshold", "1e-6"));

        LibrpaOptions opts;
        librpa_init_options(&opts);
        opts.nfreq = std::stoi(par("nfreq", "16"));
        const std::string tf = lower(par("tfgrids_type", "minimax"));
        opts.tfgrids_type = tf == "minimax" ? Minimax : tf == "evenspaced_tf" ? EvenSpaced_TF
                          : tf == "evenspaced" ? EvenSpaced : tf == "gl" ? GaussLegendre : Minimax;
        const std::string rt = lower(par("parallel_routing", "libri"));
        opts.parallel_routing = rt == "rtau" ? RTAU : rt == "atompair" ? ATOMPAIR : rt == "auto" ? AUTO : LIBRI;
        opts.vq_threshold = std::stod(par("vq_threshold", "0"));
        opts.libri_chi0_threshold_C = std::stod(par("libri_chi0_threshold_C", "0"));
        opts.libri_chi0_threshold_G = std::stod(par("libri_chi0_threshold_G", "0"));
        opts.minimax_emin = std::stod(par("minimax_emin", "-1"));
        opts.minimax_emax = std::stod(par("minimax_emax", "-1"));
        opts.n_params_anacon = std::stoi(par("n_params_anacon", std::to_string(opts.n_params_anacon)));
        opts.option_dielect_func = std::stoi(par("option_dielect_func", std::to_string(opts.option_dielect_func)));
        opts.sqrt_coulomb_threshold = std::stod(par("sqrt_coulomb_threshold", std::to_string(opts.sqrt_coulomb_threshold)));
        const std::string rwh = lower(par("replace_w_head", "f"));
        opts.replace_w_head = (rwh == "t" || rwh == "true" || rwh == ".true." || rwh == "1") ? LIBRPA_SWITCH_ON
                                                                                             : LIBRPA_SWITCH_OFF;
        const std::string shr = lower(par("use_shrink_abfs", "f"));
        const bool shrink = shr == "t" || shr == "true" || shr == ".true." || shr == "1";
        opts.use_shrink_abfs = shrink ? LIBRPA_SWITCH_ON : LIBRPA_SWITCH_OFF;

        LibrpaHandler *h = librpa_create_handler(0);
        if (!h) die(librpa_get_last_error(nullptr));
        LibrpaGB300Options go;
        librpa_gb300_init_options(&go);
        const std::string prec = lower(par("gb300_chi0_precision", "bf16x3"));
        go.chi0_precision = prec == "fp64" ? LIBRPA_GB300_CHI0_FP64 : prec == "fp32" ? LIBRPA_GB300_CHI0_FP32
                                                                                    : LIBRPA_GB300_CHI0_BF16X3;
        const std::string ecp = lower(par("gb300_ec_path", "chol"));
        go.ec_path = ecp == "lu" ? LIBRPA_GB300_EC_LU_FP64 : ecp == "chol_fp64" ? LIBRPA_GB300_EC_CHOL_FP64
                                                                                 : LIBRPA_GB300_EC_CHOL;
        const std::string sm = lower(par("gb300_screen_mode", "off"));
        go.screen_mode = sm == "threshold" ? LIBRPA_GB300_SCREEN_THRESHOLD : sm == "mlp" ? LIBRPA_GB300_SCREEN_MLP
                                                                                         : LIBRPA_GB300_SCREEN_OFF;
        go.screen_threshold = std::stod(par("gb300_screen_threshold", "1e-6"));
        go.sigma_precision = lower(par("gb300_sigma_precision", "fp64")) == "bf16x3" ? LIBRPA_GB300_SIGMA_BF16X3
                                                                                    : LIBRPA_GB300_SIGMA_FP64;
        librpa_gb300_set_options(h, &go);

        Mesh m;
        std::vector<double> wg_h, ekb_h;  // occupations (as read) and eigenvalues [s][k][n]
        double latv[9] = {0};            // lattice vectors, rows a1, a2, a3 (Bohr)
        // band_out (read_data.cpp:32-140): nk ns nb nao efermi, then per (k, s) block n f e e_eV
        {
            const auto t = tokens(dir + "band_out");
            size_t q = 0;
            m.nk = std::stoi(t.at(q++));
            m.ns = std::stoi(t.at(q++));
            m.nb = std::stoi(t.at(q++));
            m.nao = std::stoi(t.at(q++));
            const double ef = std::stod(t.at(q++));
            std::vector<double> &wg = wg_h, &ekb = ekb_h;
            wg.assign(static_cast<size_t>(m.ns) * m.nk * m.nb, 0.0);
            ekb.assign(wg.size(), 0.0);
            for (int kk = 0; kk < m.nk; ++kk)
                for (int ss = 0; ss < m.ns; ++ss)
                {
                    const int k = std::stoi(t.at(q)) - 1, s = std::stoi(t.at(q + 1)) - 1;
                    q += 2;
                    for (int n = 0; n < m.nb; ++n, q += 4)
                    {
                        const size_t i = (static_cast<size_t>(s) * m.nk + k) * m.nb + n;
                        wg[i] = std::stod(t.at(q + 1));
                        ekb[i] = std::stod(t.at(q + 2));
                    }
                }
            librpa_set_scf_dimension(h, m.ns, m.nk, m.nb, m.nao, 1);
            librpa_set_wg_ekb_efermi(h, m.ns, m.nk, m.nb, wg.data(), ekb.data(), ef);
        }
        // stru_out (read_data.cpp:1814-1867): lattice, reciprocal lattice, natoms, positions + types
        std::vector<std::string> stru = tokens(dir + "stru_out");
        {
            double lat[9], G[9];
            for (int i = 0; i < 9; ++i) lat[i] = std::stod(stru.at(i));
            std::copy(lat, lat + 9, latv);
            for (int i = 0; i < 9; ++i) G[i] = std::stod(stru.at(9 + i));
            librpa_set_latvec_and_G(h, lat, G);
            m.nat = std::stoi(stru.at(18));
            std::vector<double> pos(3 * m.nat);
            m.types.resize(m.nat);
            size_t q = 19;
            for (int a = 0; a < m.nat; ++a, q += 4)
            {
                for (int d = 0; d < 3; ++d) pos[3 * a + d] = std::stod(stru.at(q + d));
                m.types[a] = std::stoi(stru.at(q + 3)) - 1;
            }
            librpa_set_atoms(h, m.nat, m.types.data(), pos.data());
        }
        // k mesh: bz_sampling_out (read_data.cpp:1869-1916) or the tail of stru_out
        if (exists(dir + "bz_sampling_out"))
        {
            const auto t = tokens(dir + "bz_sampling_out");
            for (int d = 0; d < 3; ++d) m.period[d] = std::stoi(t.at(d));
            const int nkf = std::stoi(t.at(3));
            m.kvecs.resize(3 * nkf);
            m.ibz.resize(nkf);
            size_t q = 5;
            for (int i = 0; i < nkf; ++i, q += 10)
            {
                for (int d = 0; d < 3; ++d) m.kvecs[3 * i + d] = std::stod(t.at(q + 5 + d));
                m.ibz[i] = std::stoi(t.at(q + 9)) - 1;
            }
        }
        else
        {
            size_t q = 19 + 4 * static_cast<size_t>(m.nat);
            for (int d = 0; d < 3; ++d) m.period[d] = std::stoi(stru.at(q++));
            const int nkf = m.period[0] * m.period[1] * m.period[2];
            m.kvecs.resize(3 * nkf);
            for (int i = 0; i < 3 * nkf; ++i) m.kvecs[i] = std::stod(stru.at(q++));
            m.ibz.resize(nkf);
            for (int i = 0; i < nkf; ++i) m.ibz[i] = std::stoi(stru.at(q++)) - 1;
        }
        librpa_set_kgrids_kvec(h, m.period[0], m.period[1], m.period[2], m.kvecs.data());
        librpa_set_ibz_mapping(h, static_cast<int>(m.ibz.size()), m.ibz.data());
        // basis_out (read_data.cpp:1976-2011): ntypes, 3 header numbers, then (type, n_wfc, n_aux);
        // without it (ABACUS exports) the sizes come from the RI blocks, as read_basis_from_Cs
        // does (read_data.cpp:2083-2152): n_i and n_mu of the first atom, n_j of the second
        if (!exists(dir + "basis_out"))
        {
            std::map<int, int> aw, aa;
            for (const auto &fn : files_with_prefix(dir, "Cs_data"))
            {
                auto note = [&](const int *v) {
                    aw[v[0] - 1] = v[5];
                    aw[v[1] - 1] = v[6];
                    aa[v[0] - 1] = v[7];
                };
                if (is_text_file(fn))
                {
                    const auto t = tokens(fn);
                    size_t q = 2;
                    while (q + 8 <= t.size())
                    {
                        int v[8];
                        for (int i = 0; i < 8; ++i) v[i] = std::stoi(t[q + i]);
                        note(v);
                        q += 8 + static_cast<size_t>(v[5]) * v[6] * v[7];
                    }
                    continue;
                }
                const auto raw = slurp(fn);
                size_t off = 8;
                const int nblk = get<int>(raw, off);
                for (int b = 0; b < nblk; ++b)
                {
                    int v[8];
                    for (auto &x : v) x = get<int>(raw, off);
                    note(v);
                    off += 8 * static_cast<size_t>(v[5]) * v[6] * v[7];
                }
            }
            std::vector<size_t> nw(m.nat), na(m.nat);
            for (int a = 0; a < m.nat; ++a)
            {
                if (!aw.count(a) || !aa.count(a)) die("no RI block gives the basis sizes of atom " + std::to_string(a + 1));
                nw[a] = static_cast<size_t>(aw[a]);
                na[a] = static_cast<size_t>(aa[a]);
                m.nao_at.push_back(aw[a]);
                m.nabf_at.push_back(aa[a]);
            }
            librpa_set_ao_basis_wfc(h, m.nat, nw.data());
            librpa_set_ao_basis_aux(h, m.nat, na.data());
        }
        else
        {
            const auto t = tokens(dir + "basis_out");
            const int ntypes = std::stoi(t.at(0));
            std::map<int, std::pair<int, int>> per_type;
            size_t q = 4;
            for (int i = 0; i < ntypes; ++i, q += 3)
                per_type[std::stoi(t.at(q)) - 1] = {std::stoi(t.at(q + 1)), std::stoi(t.at(q + 2))};
            std::vector<size_t> nw(m.nat), na(m.nat);
            for (int a = 0; a < m.nat; ++a)
            {
                if (!per_type.count(m.types[a])) die("basis_out lacks atom type " + std::to_string(m.types[a] + 1));
                nw[a] = per_type[m.types[a]].first;
                na[a] = per_type[m.types[a]].second;
                m.nao_at.push_back(static_cast<int>(nw[a]));
                m.nabf_at.push_back(static_cast<int>(na[a]));
            }
            librpa_set_ao_basis_wfc(h, m.nat, nw.data());
            librpa_set_ao_basis_aux(h, m.nat, na.data());
        }
        // KS_eigenvector* (read_data.cpp:184-284): per k: index, then (re, im) in the order
        // ao, band, spin (slowest to fastest: ao outermost)
        {
            const size_t per_k = static_cast<size_t>(m.nao) * m.nb * m.ns;
            std::vector<std::vector<double>> re(static_cast<size_t>(m.ns) * m.nk), im(re.size());
            for (const auto &fn : files_with_prefix(dir, "KS_eigenvector"))
            {
                const auto t = tokens(fn);
                size_t q = 0;
                while (q < t.size())
                {
                    const int ik = std::stoi(t[q++]) - 1;
                    if (q + 2 * per_k > t.size()) die("truncated eigenvector file " + fn);
                    for (int s = 0; s < m.ns; ++s)
                    {
                        re[static_cast<size_t>(s) * m.nk + ik].assign(static_cast<size_t>(m.nb) * m.nao, 0.0);
                        im[static_cast<size_t>(s) * m.nk + ik].assign(static_cast<size_t>(m.nb) * m.nao, 0.0);
                    }
                    for (int iw = 0; iw < m.nao; ++iw)
                        for (int ib = 0; ib < m.nb; ++ib)
                            for (int s = 0; s < m.ns; ++s, q += 2)
                            {
                                auto &R = re[static_cast<size_t>(s) * m.nk + ik];
                                auto &I = im[static_cast<size_t>(s) * m.nk + ik];
                                R[static_cast<size_t>(ib) * m.nao + iw] = std::stod(t[q]);
                                I[static_cast<size_t>(ib) * m.nao + iw] = std::stod(t[q + 1]);
                            }
                }
            }
            for (int s = 0; s < m.ns; ++s)
                for (int k = 0; k < m.nk; ++k)
                {
                    const auto &R = re[static_cast<size_t>(s) * m.nk + k];
                    if (R.empty()) die("no eigenvectors for k point " + std::to_string(k + 1));
                    librpa_set_wfc(h, s, k, m.nb, m.nao, R.data(), im[static_cast<size_t>(s) * m.nk + k].data());
                }
        }
        // Cs_data*: binary (read_data.cpp:690-747): natom ncell nblocks, then per block
        // I J R1 R2 R3 n_i n_j n_mu and n_i*n_j*n_mu doubles; text (read_data.cpp:618-688):
        // natom ncell, then blocks of the same 8 integers and values to the end of the file.
        // A block is kept if max |C| >= cs_threshold.
        auto set_cs = [&](const int *v, std::vector<double> &c) {
            double mx = 0.0;
            for (double x : c) mx = std::max(mx, std::fabs(x));
            if (mx < cs_threshold) return;
            const int R[3] = {v[2], v[3], v[4]};
            librpa_set_lri_coeff(h, static_cast<LibrpaParallelRouting>(opts.parallel_routing), v[0] - 1, v[1] - 1,
                                 v[5], v[6], v[7], R, c.data());
        };
        auto for_each_cs_block = [&](const std::string &prefix, const auto &fn_block) {
            for (const auto &fn : files_with_prefix(dir, prefix))
            {
                if (is_text_file(fn))
                {
                    const auto t = tokens(fn);
                    size_t q = 2;  // natom, ncell
                    while (q + 8 <= t.size())
                    {
                        int v[8];
                        for (int i = 0; i < 8; ++i) v[i] = std::stoi(t[q + i]);
                        q += 8;
                        const size_t cnt = static_cast<size_t>(v[5]) * v[6] * v[7];
                        if (q + cnt > t.size()) die("truncated RI file " + fn);
                        std::vector<double> c(cnt);
                        for (size_t i = 0; i < cnt; ++i) c[i] = std::stod(t[q + i]);
                        q += cnt;
                        fn_block(v, c);
                    }
                    continue;
                }
                const auto raw = slurp(fn);
                size_t off = 0;
                get<int>(raw, off);
                get<int>(raw, off);
                const int nblk = get<int>(raw, off);
                for (int b = 0; b < nblk; ++b)
                {
                    int v[8];
                    for (auto &x : v) x = get<int>(raw, off);
                    const size_t cnt = static_cast<size_t>(v[5]) * v[6] * v[7];
                    if (off + 8 * cnt > raw.size()) die("truncated RI file " + fn);
                    std::vector<double> c(cnt);
                    std::memcpy(c.data(), raw.data() + off, 8 * cnt);
                    off += 8 * cnt;
                    fn_block(v, c);
                }
            }
        };
        for_each_cs_block("Cs_data", set_cs);
        // ABF shrink: small basis from the n_mu of the Cs_shrinked_data blocks (first atom of a
        // block), U(q) from shrink_sinvS_* (handle_sinvS_file, read_data.cpp:2455-2568: n_irk, then
        // blocks n_small n_large brow erow bcol ecol iq q_weight and the (re, im) of the rows; iq
        // counts the IBZ points in order)
        std::vector<int> nabf_v = m.nabf_at;  // the basis of the Coulomb matrix
        if (shrink)
        {
            // the blocks also carry the RI coefficients of the small basis (the exchange of a
            // shrunk input, driver/task_gw_band.cpp:92-99), read with the same threshold
            std::map<int, int> aa;
            std::vector<std::pair<std::array<int, 8>, std::vector<double>>> small_cs;
            for_each_cs_block("Cs_shrinked_data", [&](const int *v, std::vector<double> &c) {
                aa[v[0] - 1] = v[7];
                double mx = 0.0;
                for (double x : c) mx = std::max(mx, std::fabs(x));
                if (mx < cs_threshold) return;
                std::array<int, 8> key;
                std::copy(v, v + 8, key.begin());
                small_cs.emplace_back(key, std::move(c));
            });
            std::vector<size_t> ns(m.nat);
            for (int a = 0; a < m.nat; ++a)
            {
                if (!aa.count(a)) die("use_shrink_abfs: no Cs_shrinked_data block gives the small basis of atom " +
                                      std::to_string(a + 1));
                ns[a] = static_cast<size_t>(aa[a]);
                nabf_v[a] = aa[a];
            }
            librpa_gb300_set_shrink_basis(h, m.nat, ns.data());
            for (const auto &kb : small_cs)
            {
                const int *v = kb.first.data();
                const int R[3] = {v[2], v[3], v[4]};
                librpa_gb300_set_shrink_lri_coeff(h, v[0] - 1, v[1] - 1, v[5], v[6], v[7], R, kb.second.data());
            }
            std::vector<int> reps;  // IBZ representatives in order of appearance
            for (int k : m.ibz)
                if (std::find(reps.begin(), reps.end(), k) == reps.end()) reps.push_back(k);
            std::map<int, std::vector<cplx>> U;
            int n_s = 0, n_l = 0;
            auto block = [&](int nsm, int nlg, int br, int er, int bc, int ec, int iq, const std::string &fn) {
                if (er < br || ec < bc || br < 0 || bc < 0 || er >= nsm || ec >= nlg || iq < 0 ||
                    iq >= static_cast<int>(reps.size()))
                    die("bad shrink transform block header in " + fn);
                n_s = nsm;
                n_l = nlg;
                auto &M = U[iq];
                M.resize(static_cast<size_t>(nsm) * nlg);
                return &M;
            };
            for (const auto &fn : files_with_prefix(dir, "shrink_sinvS"))
            {
                if (is_text_file(fn))
                {
                    const auto t = tokens(fn);
                    size_t q = 1;
                    while (q + 8 <= t.size())
                    {
                        int v[7];
                        for (int i = 0; i < 7; ++i) v[i] = std::stoi(t[q + i]);
                        q += 8;
                        auto *M = block(v[0], v[1], v[2] - 1, v[3] - 1, v[4] - 1, v[5] - 1, v[6] - 1, fn);
                        const size_t cnt = static_cast<size_t>(v[3] - v[2] + 1) * (v[5] - v[4] + 1);
                        if (q + 2 * cnt > t.size()) die("truncated shrink transform file " + fn);
                        for (int r = v[2] - 1; r < v[3]; ++r)
                            for (int c = v[4] - 1; c < v[5]; ++c, q += 2)
                                (*M)[static_cast<size_t>(r) * v[1] + c] = cplx(std::stod(t[q]), std::stod(t[q + 1]));
                    }
                    continue;
                }
                const auto raw = slurp(fn);
                size_t off = 0;
                get<int>(raw, off);
                const int nloc = get<int>(raw, off);
                for (int b = 0; b < nloc; ++b)
                {
                    int v[7];
                    for (auto &x : v) x = get<int>(raw, off);
                    get<double>(raw, off);
                    auto *M = block(v[0], v[1], v[2] - 1, v[3] - 1, v[4] - 1, v[5] - 1, v[6] - 1, fn);
                    for (int r = v[2] - 1; r < v[3]; ++r)
                        for (int c = v[4] - 1; c < v[5]; ++c)
                        {
                            const double x = get<double>(raw, off), y = get<double>(raw, off);
                            (*M)[static_cast<size_t>(r) * v[1] + c] = cplx(x, y);
                        }
                }
            }
            if (U.empty()) die("use_shrink_abfs: no shrink_sinvS file in " + dir);
            for (const auto &[iq, M] : U)
            {
                std::vector<double> ur(M.size()), ui(M.size());
                for (size_t i = 0; i < M.size(); ++i)
                {
                    ur[i] = M[i].real();
                    ui[i] = M[i].imag();
                }
                librpa_gb300_set_shrink_sinvS(h, reps[iq], n_s, n_l, ur.data(), ui.data());
            }
        }
        // coulomb_mat* / coulomb_cut* binary (read_data.cpp:1472-1577): n_irk n_local, then per
        // block nbasbas brow erow bcol ecol iq q_weight and the rows (complex); atom-pair blocks I <= J
        auto read_coulomb = [&](const std::string &prefix, const std::vector<int> &nabf_v, bool cut) {
            std::vector<int> off_at(m.nat + 1, 0);
            for (int a = 0; a < m.nat; ++a) off_at[a + 1] = off_at[a] + nabf_v[a];
            std::map<int, std::vector<cplx>> full;
            int nbb = 0;
            for (const auto &fn : files_with_prefix(dir, prefix))
            {
                if (is_text_file(fn))
                {
                    // text (read_data.cpp:1580-1650): n_irk, then blocks of nbasbas brow erow bcol
                    // ecol, iq q_weight and the (re, im) pairs of the rows
                    const auto t = tokens(fn);
                    size_t q = 1;
                    while (q + 7 <= t.size())
                    {
                        nbb = std::stoi(t[q]);
                        const int br = std::stoi(t[q + 1]) - 1, er = std::stoi(t[q + 2]) - 1;
                        const int bc = std::stoi(t[q + 3]) - 1, ec = std::stoi(t[q + 4]) - 1;
                        const int iq = std::stoi(t[q + 5]) - 1;
                        q += 7;
                        if (er < br || ec < bc || iq < 0 || br < 0 || bc < 0 || er >= nbb || ec >= nbb)
                            die("bad Coulomb block header in " + fn);
                        const size_t cnt = static_cast<size_t>(er - br + 1) * (ec - bc + 1);
                        if (q + 2 * cnt > t.size()) die("truncated Coulomb file " + fn);
                        auto &M = full[iq];
                        M.resize(static_cast<size_t>(nbb) * nbb);
                        for (int r = br; r <= er; ++r)
                            for (int c = bc; c <= ec; ++c, q += 2)
                                M[static_cast<size_t>(r) * nbb + c] = cplx(std::stod(t[q]), std::stod(t[q + 1]));
                    }
                    continue;
                }
                const auto raw = slurp(fn);
                size_t off = 0;
                get<int>(raw, off);
                const int nloc = get<int>(raw, off);
                for (int b = 0; b < nloc; ++b)
                {
                    nbb = get<int>(raw, off);
                    const int br = get<int>(raw, off) - 1, er = get<int>(raw, off) - 1;
                    const int bc = get<int>(raw, off) - 1, ec = get<int>(raw, off) - 1;
                    const int iq = get<int>(raw, off) - 1;
                    get<double>(raw, off);
                    auto &M = full[iq];
                    M.resize(static_cast<size_t>(nbb) * nbb);
                    const int nc = ec - bc + 1;
                    for (int r = br; r <= er; ++r)
                        for (int c = 0; c < nc; ++c)
                        {
                            const double x = get<double>(raw, off), y = get<double>(raw, off);
                            M[static_cast<size_t>(r) * nbb + bc + c] = cplx(x, y);
                        }
                }
            }
            if (!full.empty() && nbb != off_at[m.nat])
                die("Coulomb matrices are " + std::to_string(nbb) + " x " + std::to_string(nbb) + " but the bases give " +
                    std::to_string(off_at[m.nat]) + " auxiliary functions" +
                    (shrink ? "" : " (a shrunk ABF set needs use_shrink_abfs = t)"));
            for (const auto &[iq, M] : full)
                for (int I = 0; I < m.nat; ++I)
                    for (int J = I; J < m.nat; ++J)
                    {
                        const int nm = nabf_v[I], nn = nabf_v[J];
                        std::vector<double> vr(static_cast<size_t>(nm) * nn), vi(vr.size());
                        for (int a = 0; a < nm; ++a)
                            for (int c = 0; c < nn; ++c)
                            {
                                const cplx z = M[static_cast<size_t>(off_at[I] + a) * nbb + off_at[J] + c];
                                vr[static_cast<size_t>(a) * nn + c] = z.real();
                                vi[static_cast<size_t>(a) * nn + c] = z.imag();
                            }
                        if (cut)
                            librpa_set_aux_cut_coulomb_k_atom_pair(h, iq, I, J, nm, nn, vr.data(), vi.data(),
                                                                   opts.vq_threshold);
                        else
                            librpa_set_aux_bare_coulomb_k_atom_pair(h, iq, I, J, nm, nn, vr.data(), vi.data(),
                                                                    opts.vq_threshold);
                    }
        };
        read_coulomb("coulomb_mat", nabf_v, false);

        if (task == "exx" || task == "g0w0")
        {
            // k fractions: k_cart / 2 pi times the lattice vectors
            std::vector<double> kfrac(3 * static_cast<size_t>(m.nk));
            for (int k = 0; k < m.nk; ++k)
                for (int d = 0; d < 3; ++d)
                {
                    double v = 0.0;
                    for (int e = 0; e < 3; ++e) v += m.kvecs[3 * k + e] / (2.0 * M_PI) * latv[3 * d + e];
                    kfrac[3 * k + d] = std::fabs(v) < 1e-12 ? 0.0 : v;
                }
            // driver/task/exx.cpp, driver/task/g0w0.cpp: the truncated Coulomb matrix, for G0W0 the
            // dielectric function of the head correction (dielecfunc_out: omega, Re, Im per line;
            // read_data.cpp:1211-1229) and v_xc (vxc_out: n_k n_s n_states, then per k and spin an
            // "Ha eV" pair per state; read_data.cpp:142-182)
            read_coulomb("coulomb_cut", nabf_v, true);
            std::vector<int> iks(m.nk);
            for (int k = 0; k < m.nk; ++k) iks[k] = k;
            const int nst = m.nb;
            std::vector<double> vexx(static_cast<size_t>(m.ns) * m.nk * nst);
            librpa_get_exx_pot_kgrid(h, &opts, m.ns, m.nk, iks.data(), 0, nst, vexx.data());
            if (librpa_get_last_error_code(h)) die(librpa_get_last_error(h));
            const double ha2ev = 27.211386245988;
            if (task == "exx")
            {
                for (int sp = 0; sp < m.ns; ++sp)
                {
                    std::printf("Spin channel %d\n", sp + 1);
                    for (int k = 0; k < m.nk; ++k)
                    {
                        std::printf("k-point %d: (%.5f, %.5f, %.5f)\n", k + 1, kfrac[3 * k], kfrac[3 * k + 1],
                                    kfrac[3 * k + 2]);
                        std::printf("%-4s  %-10s  %-10s\n", "Band", "e_exx (Ha)", "e_exx (eV)");
                        for (int n = 0; n < nst; ++n)
                        {
                            const double e = vexx[(static_cast<size_t>(sp) * m.nk + k) * nst + n];
                            std::printf("%4d  %10.5f  %10.5f\n", n + 1, e, ha2ev * e);
                        }
                        std::printf("\n");
                    }
                }
                librpa_destroy_handler(h);
                return 0;
            }
            if (opts.replace_w_head == LIBRPA_SWITCH_ON && exists(dir + "dielecfunc_out"))
            {
                std::vector<double> om, df;
                std::ifstream f(dir + "dielecfunc_out");
                double w, re, im;
                while (f >> w >> re >> im)
                {
                    om.push_back(w);
                    df.push_back(re);
                }
                librpa_set_dielect_func_imagfreq(h, static_cast<int>(om.size()), om.data(), df.data());
            }
            const auto tv = tokens(dir + "vxc_out");
            if (tv.size() < 3) die("cannot read vxc_out");
            const int vk = std::stoi(tv[0]), vs = std::stoi(tv[1]), vn = std::stoi(tv[2]);
            if (vk != m.nk || vs != m.ns || vn < nst) die("vxc_out dimensions differ from the mean field");
            std::vector<double> vxc(static_cast<size_t>(m.ns) * m.nk * nst);
            {
                size_t q = 3;
                for (int k = 0; k < vk; ++k)
                    for (int sp = 0; sp < vs; ++sp)
                        for (int n = 0; n < vn; ++n, q += 2)
                            if (n < nst) vxc[(static_cast<size_t>(sp) * m.nk + k) * nst + n] = std::stod(tv.at(q));
            }
            std::vector<double> sre(vxc.size()), sim(vxc.size());
            librpa_get_g0w0_sigc_kgrid(h, &opts, m.ns, m.nk, iks.data(), 0, nst, vxc.data(), vexx.data(), sre.data(),
                                       sim.data());
            if (librpa_get_last_error_code(h)) die(librpa_get_last_error(h));
            for (int sp = 0; sp < m.ns; ++sp)
                for (int k = 0; k < m.nk; ++k)
                    for (int n = 0; n < nst; ++n)
                        if (std::isnan(sre[(static_cast<size_t>(sp) * m.nk + k) * nst + n]))
                            std::printf("Warning! QPE solver failed for spin %d, kpoint %d, state %d\n", sp + 1, k + 1,
                                        n + 1);
            const std::string banner(124, '-');
            std::printf("Printing quasi-particle energy [unit: eV]\n\n");
            for (int sp = 0; sp < m.ns; ++sp)
                for (int k = 0; k < m.nk; ++k)
                {
                    std::printf("spin %2d, k-point %4d: (%.5f, %.5f, %.5f) \n", sp + 1, k + 1, kfrac[3 * k],
                                kfrac[3 * k + 1], kfrac[3 * k + 2]);
                    std::printf("%124s\n", banner.c_str());
                    std::printf("%5s %16s %16s %16s %16s %16s %16s %16s\n", "State", "occ", "e_mf", "v_xc", "v_exx",
                                "ReSigc", "ImSigc", "e_qp");
                    std::printf("%124s\n", banner.c_str());
                    for (int n = 0; n < nst; ++n)
                    {
                        const size_t o = (static_cast<size_t>(sp) * m.nk + k) * nst + n;
                        const double emf = ekb_h[o], e_qp = emf - vxc[o] + vexx[o] + sre[o];
                        std::printf("%5d %16.5f %16.5f %16.5f %16.5f %16.5f %16.5f %16.5f\n", n + 1, wg_h[o],
                                    emf * ha2ev, vxc[o] * ha2ev, vexx[o] * ha2ev, sre[o] * ha2ev, sim[o] * ha2ev,
                                    e_qp * ha2ev);
                    }
                    std::printf("\n");
                }
            librpa_destroy_handler(h);
            return 0;
        }

        int n_ibz = 0;
        {
            std::vector<int> seen;
            for (int k : m.ibz)
                if (std::find(seen.begin(), seen.end(), k) == seen.end()) seen.push_back(k);
            n_ibz = static_cast<int>(seen.size());
        }
        std::vector<double> re(n_ibz), im(n_ibz);
        const double ec = librpa_get_rpa_correlation_energy(h, &opts, n_ibz, re.data(), im.data());
        if (std::isnan(ec)) die(librpa_get_last_error(h));
        std::printf("RPA correlation energy (Hartree)\n");
        std::printf("| Weighted contribution from each k:\n");
        for (int i = 0; i < n_ibz; ++i) std::printf("| %d: (%.12g,%.12g)\n", i + 1, re[i], im[i]);
        std::printf("| Total EcRPA: %18.9f\n", ec);
        for (int i = 0; i < n_ibz; ++i)
            if (std::fabs(im[i]) > 1e-3)
                std::printf("Warning: considerable imaginary part of EcRPA = %f\n at IBZ k-point %d\n", im[i], i + 1);
        librpa_destroy_handler(h);
        return 0;
    }
    catch (const std::exception &e)
    {
        std::fprintf(stderr, "chi0_main: %s\n", e.what());
        return 1;
    }
}
