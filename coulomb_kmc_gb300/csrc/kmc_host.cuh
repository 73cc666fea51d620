// Part of the kmc_gb300.cu translation unit (included there, in order, after the kernels; it opens and closes
// its own anonymous namespace): host side: the system handle (kmc_system), launch bookkeeping and profiling, tables, operator set-up, store management and the launch sequences of propose and accept.
#pragma once
// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct kmc_system {
    kmc_params prm{};
    int tune[KMC_NTUNE] = {};
    int smem_sm = 0;  // shared memory per SM of the device (bytes)
    int prio_hi = 0;  // the device's highest stream / launch priority (numerically least)
    cudaStream_t stream = nullptr;
    // side stream of the accept: the move's energy and the multipole / lattice vector
    // updates run there beside the particle-to-local kernel (fork / join events)
    cudaStream_t side = nullptr, side2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join2 = nullptr;
    cudaEvent_t ev_lfork = nullptr, ev_ljoin = nullptr;  // lattice branch of propose
    cudaStream_t side3 = nullptr;                        // caller's branch beside an accept
    cudaEvent_t ev_join3 = nullptr, ev_fork3 = nullptr;
    double2 *d_snap = nullptr;  // [3][NH] old and new cells' expansions and g, before the accept
    // mixed pbc: per-charge far-lattice cache, h = A b in box units ([NH][hc_stride],
    // FP32 pairs) and b.h / 2 ([hc_stride]); valid while hc_valid
    float2 *d_hc = nullptr;
    double *d_hself = nullptr;
    int hc_stride = 0;
    bool hc_valid = false;
    Sys S{};
    bool initialised = false;
    // device buffers
    double *d_pos = nullptr, *d_q = nullptr;
    int *d_pcell = nullptr, *d_pslot = nullptr, *d_cnt = nullptr, *d_store_pid = nullptr;
    double *d_phin = nullptr;  // Sys::phin
    // device copies of the host arrays of kmc_propose_with_dats_host, grown as needed
    int64_t *hp_smc = nullptr, *hp_sites = nullptr, *hp_mask = nullptr;
    double *hp_ppos = nullptr, *hp_pq = nullptr, *hp_pde = nullptr;
    int64_t hp_nsite = 0, hp_n = 0, hp_nm = 0, hp_nq = 0;
    double4_32a *d_store = nullptr;
    double2 *d_lexp = nullptr, *d_mpole = nullptr;
    int *d_ar_ptr = nullptr, *d_ar_col = nullptr, *d_ai_ptr = nullptr, *d_ai_col = nullptr;
    double *d_ar_val = nullptr, *d_ai_val = nullptr;
    int *d_aru_ptr = nullptr, *d_aru_col = nullptr, *d_aiu_ptr = nullptr, *d_aiu_col = nullptr;
    double *d_aru_val = nullptr, *d_aiu_val = nullptr;
    float *d_ar32 = nullptr, *d_ai32 = nullptr;
    float2 *d_a2 = nullptr, *d_ai2 = nullptr;  // FP32 pairs of ar_val / ai_val
    float4 *d_st_hi = nullptr, *d_st_lo = nullptr, *d_lexp32 = nullptr;
    double *d_energy = nullptr;     // [0] energy, [1] single-move dE
    double *d_sp_part = nullptr;    // [kSpBlocks] single-move partials
    unsigned *d_sp_ticket = nullptr;  // single-move blocks finished (reset by the last)
    unsigned *d_mg_ticket = nullptr;  // multipole / lattice-vector blocks finished
    double *d_phin_part = nullptr;    // [kPhinBlocks] partial sums of the moved charge's near-field potential
    unsigned *d_phin_ticket = nullptr;  // near-potential update blocks finished (reset by the last)
    unsigned long long *d_err = nullptr; // [0] bad moves, [1] overflows, [2..5] refused move (pid + 1, position bits)
    int64_t layout_gen = 0;  // advances whenever device buffers a captured step reads are reallocated
    bool props_ready = false;  // a proposal set-up has run: the compacted proposals are valid
    AcceptRec *d_rec = nullptr;
    // proposal scratch
    Props P{};
    int64_t prop_n = 0, prop_nm = 0;
    // host staging for the moves path
    std::vector<int> h_cnt;         // host mirror of occupancy
    std::vector<int> h_pcell;       // host mirror of particle cells
    bool mirror_valid = false;
    // per-kernel CUDA-event timing (kmc_profile) and launch counter
    bool prof_on = false;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
    double prof_ms[32] = {0};
    int64_t prof_n[32] = {0};
    int64_t launches = 0;
    int64_t epoch = 0;  // launches ever made on the system (never reset; the driver's staleness check)
    // far-field host operator (folded)
    std::vector<int> ar_ptr, ar_col, ai_ptr, ai_col;
    std::vector<double> ar_val, ai_val;
    std::vector<int> fprog_i;     // far-lattice self term program (lattice_self_program)
    std::vector<double> fprog_d;
    int *d_fprog_i = nullptr;
    double *d_fprog_d = nullptr;
    float *d_fprog_f = nullptr;
    FSelf12 fs12{};               // the float program's reals when it has the L = 12 cubic shape
    int fs12_ok = 0;
    double *d_escale = nullptr;
    double *d_p2lsc = nullptr;
    std::vector<int> aru_ptr, aru_col, aiu_ptr, aiu_col;
    std::vector<double> aru_val, aiu_val;
};

namespace {

// kernel ids for kmc_profile_read (order = names in kmc_kernel_name)
enum KId { K_COUNT_SCAN = 0, K_SCAN_PART, K_SCATTER, K_OLD, K_NEW, K_LR, K_ACCEPT_PREP, K_ACCEPT_MPOLE, K_P2L,
           K_FILL, K_INIT, K_CELL_SORT, K_NEAR_CELL, K_LR_OLD, K_DIFF, K_REFRESH, K_SINGLE, K_LR_G,
           K_PHIN, K_NKERNELS };
const char *const g_kernel_names[K_NKERNELS] = {"count_scan", "scan_part", "scatter", "old_side", "new_side",
                                                "far_lattice", "accept_prep", "accept_multipole",
                                                "accept_p2l", "fill_moves", "initial_solve", "cell_sort",
                                                "near_far_cell", "far_lattice_old", "diff", "mixed_refresh",
                                                "single_move_fp64", "lattice_g_update",
                                                "near_potential_update"};

cudaEvent_t pool_event(kmc_system *s)
{
    if (!s->ev_pool.empty()) {
        cudaEvent_t e = s->ev_pool.back();
        s->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

// bracket one launch: call before (returns start event or null) and after
struct LaunchScope {
    kmc_system *s;
    int id;
    cudaStream_t st;
    cudaEvent_t a = nullptr;
    LaunchScope(kmc_system *s_, int id_, cudaStream_t st_ = nullptr) : s(s_), id(id_), st(st_ ? st_ : s_->stream)
    {
        s->launches++;
        s->epoch++;
        if (s->prof_on) {
            a = pool_event(s);
            cudaEventRecord(a, st);
        }
    }
    ~LaunchScope()
    {
        if (a) {
            cudaEvent_t b = pool_event(s);
            cudaEventRecord(b, st);
            s->ev_pending.push_back({id, {a, b}});
        }
    }
};

bool g_tables_ready = false;
std::vector<double> g_p2l_scale_host;  // host copy of c_p2l_scale

// Fork / join events of the accept path are recorded during stream captures.  They
// are kept in a process-wide pool instead of being destroyed with their system, so
// that the runtime never hands their handles out again to other code while it may
// still count them as recorded in a capture.
std::mutex g_ev_mutex;
std::vector<cudaEvent_t> g_ev_pool;

cudaError_t event_take(cudaEvent_t *e)
{
    {
        std::lock_guard<std::mutex> lk(g_ev_mutex);
        if (!g_ev_pool.empty()) {
            *e = g_ev_pool.back();
            g_ev_pool.pop_back();
            return cudaSuccess;
        }
    }
    return cudaEventCreateWithFlags(e, cudaEventDisableTiming);
}

void event_give(cudaEvent_t e)
{
    std::lock_guard<std::mutex> lk(g_ev_mutex);
    g_ev_pool.push_back(e);
}

int upload_tables()
{
    if (g_tables_ready) return KMC_OK;
    std::vector<double> a(KMC_LMAX * KMC_LMAX, 0.0), b(KMC_LMAX * KMC_LMAX, 0.0), d(KMC_LMAX, 0.0);
    for (int l = 0; l < KMC_LMAX; ++l)
        for (int m = 0; m < l; ++m) {
            const double s = std::sqrt((double)(l * l - m * m));
            a[l * KMC_LMAX + m] = (2.0 * l - 1.0) / s;
            b[l * KMC_LMAX + m] = std::sqrt((double)((l - 1) * (l - 1) - m * m)) / s;
        }
    for (int m = 1; m < KMC_LMAX; ++m) d[m] = -std::sqrt((2.0 * m - 1.0) / (2.0 * m));
    KMC_CUDA(cudaMemcpyToSymbol(c_rec_a, a.data(), sizeof(double) * a.size()));
    KMC_CUDA(cudaMemcpyToSymbol(c_rec_b, b.data(), sizeof(double) * b.size()));
    KMC_CUDA(cudaMemcpyToSymbol(c_rec_d, d.data(), sizeof(double) * d.size()));
    KMC_CUDA(cudaMemcpyToSymbol(g_rec_a, a.data(), sizeof(double) * a.size()));
    KMC_CUDA(cudaMemcpyToSymbol(g_rec_b, b.data(), sizeof(double) * b.size()));
    KMC_CUDA(cudaMemcpyToSymbol(g_rec_d, d.data(), sizeof(double) * d.size()));
    auto split = [](const std::vector<double> &v) {
        std::vector<float2> o(v.size());
        for (size_t i = 0; i < v.size(); ++i) {
            const float h = (float)v[i];
            o[i] = make_float2(h, (float)(v[i] - (double)h));
        }
        return o;
    };
    const std::vector<float2> a2 = split(a), b2 = split(b), d2 = split(d);
    KMC_CUDA(cudaMemcpyToSymbol(c_rec_a2, a2.data(), sizeof(float2) * a2.size()));
    KMC_CUDA(cudaMemcpyToSymbol(c_rec_b2, b2.data(), sizeof(float2) * b2.size()));
    KMC_CUDA(cudaMemcpyToSymbol(c_rec_d2, d2.data(), sizeof(float2) * d2.size()));
    KMC_CUDA(cudaMemcpyToSymbol(g_rec_a2, a2.data(), sizeof(float2) * a2.size()));
    KMC_CUDA(cudaMemcpyToSymbol(g_rec_b2, b2.data(), sizeof(float2) * b2.size()));
    KMC_CUDA(cudaMemcpyToSymbol(g_rec_d2, d2.data(), sizeof(float2) * d2.size()));
    {
        std::vector<double> beta(KMC_LMAX * KMC_LMAX, 0.0), scale(KMC_LMAX * KMC_LMAX, 0.0);
        double dm = 1.0;
        for (int m = 0; m < KMC_LMAX; ++m) {
            if (m > 0) dm *= d[m];
            double c = dm;
            scale[m * KMC_LMAX + m] = c;
            for (int l = m + 1; l < KMC_LMAX; ++l) {
                c *= a[l * KMC_LMAX + m];
                scale[l * KMC_LMAX + m] = c;
                if (l - 1 > m) beta[l * KMC_LMAX + m] = b[l * KMC_LMAX + m] / (a[l * KMC_LMAX + m] * a[(l - 1) * KMC_LMAX + m]);
            }
        }
        const std::vector<float2> beta2 = split(beta);
        KMC_CUDA(cudaMemcpyToSymbol(c_p2l_beta, beta2.data(), sizeof(float2) * beta2.size()));
        KMC_CUDA(cudaMemcpyToSymbol(c_p2l_beta64, beta.data(), sizeof(double) * beta.size()));
        KMC_CUDA(cudaMemcpyToSymbol(c_p2l_scale, scale.data(), sizeof(double) * scale.size()));
        g_p2l_scale_host = scale;
    }
    g_tables_ready = true;
    return KMC_OK;
}

template <typename T>
int dalloc(T **p, size_t n)
{
    if (*p) {
        cudaFree(*p);
        *p = nullptr;
    }
    if (n == 0) n = 1;
    KMC_CUDA(cudaMalloc((void **)p, n * sizeof(T)));
    return KMC_OK;
}

// Fold the reference-layout operator R (l^2 x l^2, rows/cols l(l+1)+m) and the
// dipole correction into two symmetric NH x NH quadratic forms over m >= 0:
//   E_LR(M) = 1/2 (ReM^T A_re ReM + ImM^T A_im ImM)
// using ReM_{l,-m} = ReM_{l,m}, ImM_{l,-m} = -ImM_{l,m}.
// regular solid harmonics Rg_l^m(x), 0 <= m <= l < LL, folded index (host, FP64)
void rg_host(const double x, const double y, const double z, const int LL, double *re, double *im)
{
    const double r2 = x * x + y * y + z * z;
    double dre = 1.0, dim = 0.0;
    for (int m = 0; m < LL; ++m) {
        if (m > 0) {
            const double t = -std::sqrt((2.0 * m - 1.0) / (2.0 * m));
            const double nre = t * (dre * x - dim * y), nim = t * (dre * y + dim * x);
            dre = nre;
            dim = nim;
        }
        double pre = 0.0, pim = 0.0, cre = dre, cim = dim;
        re[hidx(m, m)] = cre;
        im[hidx(m, m)] = cim;
        for (int l = m + 1; l < LL; ++l) {
            const double sq = std::sqrt((double)(l * l - m * m));
            const double a = (2.0 * l - 1.0) / sq, b = std::sqrt((double)((l - 1) * (l - 1) - m * m)) / sq;
            const double nre = a * z * cre - b * r2 * pre, nim = a * z * cim - b * r2 * pim;
            pre = cre;
            pim = cim;
            cre = nre;
            cim = nim;
            re[hidx(l, m)] = cre;
            im[hidx(l, m)] = cim;
        }
    }
}

// Gauss-Legendre nodes and weights on [-1, 1] (Newton iteration on P_n)
void gauss_legendre(const int n, std::vector<double> &x, std::vector<double> &w)
{
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < n; ++i) {
        double t = std::cos(pi * (i + 0.75) / (n + 0.5));
        double dp = 1.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = t;
            for (int k = 2; k <= n; ++k) {
                const double p2 = ((2.0 * k - 1.0) * t * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (t * p1 - p0) / (t * t - 1.0);
            const double dt = p1 / dp;
            t -= dt;
            if (std::fabs(dt) < 1e-16) break;
        }
        x[i] = t;
        w[i] = 2.0 / ((1.0 - t * t) * dp * dp);
    }
}

// The far-lattice self term of one unit charge, F(x) = 1/2 a(x)^T A a(x) with a(x)
// its folded multipole (re, im blocks), is a polynomial of degree <= 2L-2; its
// degree-d part is homogeneous, so
//   F(x) = sum_d sum_{lambda = d mod 2} r^(d - lambda) sum_mu [c Re Rg_lambda^mu(x) + c' Im Rg_lambda^mu(x)].
// The coefficients are projections on the unit sphere with a quadrature exact to
// degree 4L-4 (Gauss-Legendre in cos(theta) x uniform phi).  For the cubic lattice
// only mu = 0 mod 4 and real parts survive (31 terms at L = 12 instead of the
// 2,000-entry quadratic form).  The evaluation program (ints / reals) lists per
// column mu: mu, lambda_max, entries; reals: D_mu = prod d_k, the recurrence
// coefficients (a, b) for lambda = mu+1..lambda_max, then per entry its polynomial
// in r^2 (ascending powers).
void lattice_self_program(const int L, const std::vector<double> &Ar, const std::vector<double> &Ai, const double E,
                          std::vector<int> &pi, std::vector<double> &pd)
{
    const int NH = L * (L + 1) / 2, LL = 2 * L - 1, NHL = LL * (LL + 1) / 2;
    const int nt = 2 * L + 1, nph = 4 * L + 2;
    std::vector<double> gx, gw;
    gauss_legendre(nt, gx, gw);
    std::vector<int> lof(NH);
    for (int l = 0; l < L; ++l)
        for (int m = 0; m <= l; ++m) lof[hidx(l, m)] = l;
    const int nd = 2 * L - 1;
    const int nn = nt * nph;
    std::vector<double> Fd((size_t)nd * nn, 0.0), wn(nn), Bre((size_t)nn * NHL), Bim((size_t)nn * NHL);
    std::vector<double> are(NH), aim(NH), bre(NHL), bim(NHL);
    const double pi2 = 6.283185307179586477;
    for (int i = 0; i < nt; ++i)
        for (int j = 0; j < nph; ++j) {
            const int k = i * nph + j;
            const double ct = gx[i], st = std::sqrt(std::max(0.0, 1.0 - ct * ct)), ph = pi2 * j / nph;
            const double x = st * std::cos(ph), y = st * std::sin(ph), z = ct;
            wn[k] = gw[i] * pi2 / nph;
            rg_host(x, y, z, L, are.data(), aim.data());
            for (int h = 0; h < NH; ++h) aim[h] = -aim[h];  // multipole = conj(Rg)
            for (int r = 0; r < NH; ++r)
                for (int c = 0; c < NH; ++c) {
                    const double ar = Ar[(size_t)r * NH + c], ai = Ai[(size_t)r * NH + c];
                    if (ar == 0.0 && ai == 0.0) continue;
                    Fd[(size_t)(lof[r] + lof[c]) * nn + k] += 0.5 * (ar * are[r] * are[c] + ai * aim[r] * aim[c]);
                }
            rg_host(x, y, z, LL, bre.data(), bim.data());
            for (int h = 0; h < NHL; ++h) {
                Bre[(size_t)k * NHL + h] = bre[h];
                Bim[(size_t)k * NHL + h] = bim[h];
            }
        }
    struct Term {
        int mu, lam, kind, j;
        double c;
    };
    std::vector<Term> terms;
    const double rmax = 0.5 * std::sqrt(3.0) * E;
    double cmax = 0.0;
    for (int d = 0; d < nd; ++d)
        for (int lam = d % 2; lam <= d; lam += 2)
            for (int mu = 0; mu <= lam; ++mu)
                for (int kind = 0; kind < 2; ++kind) {
                    if (kind == 1 && mu == 0) continue;
                    const std::vector<double> &B = kind ? Bim : Bre;
                    double num = 0.0, den = 0.0;
                    for (int k = 0; k < nn; ++k) {
                        const double b = B[(size_t)k * NHL + hidx(lam, mu)];
                        num += wn[k] * Fd[(size_t)d * nn + k] * b;
                        den += wn[k] * b * b;
                    }
                    const double c = num / den;
                    const double contrib = std::fabs(c) * std::pow(rmax, d);
                    cmax = std::max(cmax, contrib);
                    terms.push_back({mu, lam, kind, (d - lam) / 2, c});
                }
    std::vector<Term> keep;
    for (const Term &t : terms)
        if (std::fabs(t.c) * std::pow(rmax, 2 * t.j + t.lam) > 1e-15 * cmax) keep.push_back(t);
    pi.clear();
    pd.clear();
    std::vector<int> mus;
    for (const Term &t : keep)
        if (std::find(mus.begin(), mus.end(), t.mu) == mus.end()) mus.push_back(t.mu);
    std::sort(mus.begin(), mus.end());
    pi.push_back((int)mus.size());
    double Dm = 1.0;
    int mprev = 0;
    for (int mu : mus) {
        for (int k = mprev + 1; k <= mu; ++k) Dm *= -std::sqrt((2.0 * k - 1.0) / (2.0 * k));
        mprev = mu;
        int lmax = mu;
        for (const Term &t : keep)
            if (t.mu == mu) lmax = std::max(lmax, t.lam);
        // entries of this column: distinct (lam, kind), sorted by lam
        std::vector<std::pair<int, int>> ents;
        for (const Term &t : keep)
            if (t.mu == mu && std::find(ents.begin(), ents.end(), std::make_pair(t.lam, t.kind)) == ents.end())
                ents.push_back({t.lam, t.kind});
        std::sort(ents.begin(), ents.end());
        pi.push_back(mu);
        pi.push_back(lmax);
        pi.push_back((int)ents.size());
        pd.push_back(Dm);
        for (int l = mu + 1; l <= lmax; ++l) {
            const double sq = std::sqrt((double)(l * l - mu * mu));
            pd.push_back((2.0 * l - 1.0) / sq);
            pd.push_back(std::sqrt((double)((l - 1) * (l - 1) - mu * mu)) / sq);
        }
        for (const auto &e : ents) {
            int jmax = 0;
            for (const Term &t : keep)
                if (t.mu == mu && t.lam == e.first && t.kind == e.second) jmax = std::max(jmax, t.j);
            pi.push_back(e.first);
            pi.push_back(e.second);
            pi.push_back(jmax + 1);
            std::vector<double> poly(jmax + 1, 0.0);
            for (const Term &t : keep)
                if (t.mu == mu && t.lam == e.first && t.kind == e.second) poly[t.j] += t.c;
            for (double v : poly) pd.push_back(v);
        }
    }
}

// true when lattice_self_program's integer program has the shape lattice_self_c12 unrolls
bool fself12_shape(const std::vector<int> &pi)
{
    std::vector<int> want{6};
    for (int mu = 0; mu <= 20; mu += 4) {
        const int first = fs12_first(mu);
        want.insert(want.end(), {mu, 22, (22 - first) / 2 + 1 + (mu == 0 ? 2 : 0)});
        if (mu == 0) want.insert(want.end(), {0, 0, 2, 2, 0, 1});
        for (int lam = first; lam <= 22; lam += 2) want.insert(want.end(), {lam, 0, 1});
    }
    return pi == want;
}

void fold_operator(kmc_system *s)
{
    const int L = s->prm.l, H = L * L;
    const int NH = L * (L + 1) / 2;
    std::vector<double> Ar((size_t)NH * NH, 0.0), Ai((size_t)NH * NH, 0.0);
    auto fold = [&](int full, int &h, double &sg) {
        int l = (int)std::floor(std::sqrt((double)full) + 1e-9);
        while (l * l > full) --l;
        while ((l + 1) * (l + 1) <= full) ++l;
        const int m = full - l * l - l;
        h = l * (l + 1) / 2 + std::abs(m);
        sg = m > 0 ? 1.0 : (m < 0 ? -1.0 : 0.0);
    };
    for (int row = 0; row < H; ++row)
        for (int64_t k = s->prm.lr_indptr[row]; k < s->prm.lr_indptr[row + 1]; ++k) {
            const int col = (int)s->prm.lr_indices[k];
            const double v = s->prm.lr_data[k];
            int hr, hc;
            double sr, sc;
            fold(row, hr, sr);
            fold(col, hc, sc);
            Ar[(size_t)hr * NH + hc] += v;
            Ai[(size_t)hr * NH + hc] += sr * sc * v;
        }
    // dipole correction (kmc_full_long_range.py:521-540) with M = E folded
    const int h11 = 1 * 2 / 2 + 1, h10 = 1 * 2 / 2 + 0;
    Ar[(size_t)h11 * NH + h11] += 2.0 * s->prm.lr_dipole[0];
    Ai[(size_t)h11 * NH + h11] += -2.0 * s->prm.lr_dipole[1];
    Ar[(size_t)h10 * NH + h10] += s->prm.lr_dipole[2];
    auto to_csr = [&](const std::vector<double> &A, std::vector<int> &ptr, std::vector<int> &col,
                      std::vector<double> &val) {
        ptr.assign(NH + 1, 0);
        col.clear();
        val.clear();
        for (int r = 0; r < NH; ++r) {
            for (int c = 0; c < NH; ++c) {
                const double v = A[(size_t)r * NH + c];
                if (v != 0.0) {
                    col.push_back(c);
                    val.push_back(v);
                }
            }
            ptr[r + 1] = (int)col.size();
        }
    };
    to_csr(Ar, s->ar_ptr, s->ar_col, s->ar_val);
    to_csr(Ai, s->ai_ptr, s->ai_col, s->ai_val);
    // upper triangles, off-diagonal doubled (A is symmetric)
    std::vector<double> Ur((size_t)NH * NH, 0.0), Ui((size_t)NH * NH, 0.0);
    for (int r = 0; r < NH; ++r)
        for (int c = r; c < NH; ++c) {
            const double f = c == r ? 1.0 : 2.0;
            Ur[(size_t)r * NH + c] = f * 0.5 * (Ar[(size_t)r * NH + c] + Ar[(size_t)c * NH + r]);
            Ui[(size_t)r * NH + c] = f * 0.5 * (Ai[(size_t)r * NH + c] + Ai[(size_t)c * NH + r]);
        }
    to_csr(Ur, s->aru_ptr, s->aru_col, s->aru_val);
    to_csr(Ui, s->aiu_ptr, s->aiu_col, s->aiu_val);
    std::vector<double> As((size_t)NH * NH), Bs((size_t)NH * NH);
    for (int r = 0; r < NH; ++r)
        for (int c = 0; c < NH; ++c) {
            As[(size_t)r * NH + c] = 0.5 * (Ar[(size_t)r * NH + c] + Ar[(size_t)c * NH + r]);
            Bs[(size_t)r * NH + c] = 0.5 * (Ai[(size_t)r * NH + c] + Ai[(size_t)c * NH + r]);
        }
    lattice_self_program(L, As, Bs, s->prm.extent, s->fprog_i, s->fprog_d);
}

int ensure_props(kmc_system *s, int64_t n, int64_t nm)
{
    if (n <= s->prop_n && nm <= s->prop_nm) return KMC_OK;
    n = std::max<int64_t>(n, s->prop_n);
    nm = std::max<int64_t>(nm, s->prop_nm);
    Props &P = s->P;
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    int rc;
    if ((rc = dalloc(&P.cnt, n))) return rc;
    if ((rc = dalloc(&P.scan, n))) return rc;
    if ((rc = dalloc(&P.part, nb))) return rc;
    if ((rc = dalloc(&P.old_pid, n))) return rc;
    if ((rc = dalloc(&P.es, n + 1))) return rc;
    if ((rc = dalloc(&P.u0p, n))) return rc;
    if ((rc = dalloc(&P.co, n))) return rc;
    if ((rc = dalloc(&P.coq, n))) return rc;
    if ((rc = dalloc(&P.h, s->S.pbc ? (size_t)n * s->S.NH : 1))) return rc;
    if ((rc = dalloc(&P.owner, nm))) return rc;
    if ((rc = dalloc(&P.ppos, 3 * nm))) return rc;
    if ((rc = dalloc(&P.pq, nm))) return rc;
    if ((rc = dalloc(&P.pc, nm))) return rc;
    if ((rc = dalloc(&P.rloc, nm))) return rc;
    if ((rc = dalloc(&P.pnew, nm))) return rc;
    if ((rc = dalloc(&P.dout, nm))) return rc;
    if ((rc = dalloc(&P.elr, s->S.pbc ? nm : 1))) return rc;
    if ((rc = dalloc(&P.upot, s->S.mixed ? nm : 1))) return rc;
    if ((rc = dalloc(&P.ugrid, s->S.mixed ? 2 * nm : 1))) return rc;
    if ((rc = dalloc(&P.obox, s->S.mixed && s->S.pbc ? 2 * n : 1))) return rc;
    if ((rc = dalloc(&P.cprops, nm))) return rc;
    if ((rc = dalloc(&P.totals, 2))) return rc;
    s->prop_n = n;
    s->prop_nm = nm;
    return KMC_OK;
}

void sync_sys_ptrs(kmc_system *s)
{
    Sys &S = s->S;
    S.store = s->d_store;
    S.store_pid = s->d_store_pid;
    S.cnt = s->d_cnt;
    S.pos = s->d_pos;
    S.q = s->d_q;
    S.pcell = s->d_pcell;
    S.pslot = s->d_pslot;
    S.phin = s->d_phin;
    S.lexp = s->d_lexp;
    S.mpole = s->d_mpole;
    S.ar_ptr = s->d_ar_ptr;
    S.ar_col = s->d_ar_col;
    S.ar_val = s->d_ar_val;
    S.ai_ptr = s->d_ai_ptr;
    S.ai_col = s->d_ai_col;
    S.ai_val = s->d_ai_val;
    S.aru_ptr = s->d_aru_ptr;
    S.aru_col = s->d_aru_col;
    S.aru_val = s->d_aru_val;
    S.aiu_ptr = s->d_aiu_ptr;
    S.aiu_col = s->d_aiu_col;
    S.aiu_val = s->d_aiu_val;
    S.a2_val = s->d_a2;
    S.ai2_val = s->d_ai2;
    S.ar32_val = s->d_ar32;
    S.ai32_val = s->d_ai32;
    S.fprog_i = s->d_fprog_i;
    S.fprog_d = s->d_fprog_d;
    S.fprog_f = s->d_fprog_f;
    S.escale = s->d_escale;
    S.p2lsc = s->d_p2lsc;
    S.st_hi = s->d_st_hi;
    S.st_lo = s->d_st_lo;
    S.lexp32 = s->d_lexp32;
}

// mode 0: the accepted move; mode 1: charges S.pos / S.q / S.pcell of `src` (default the
// system's own) times their images
int launch_p2l(kmc_system *s, int mode, int nsrc, const Sys *src = nullptr)
{
    const Sys &S = src ? *src : s->S;
    // acc [NH][cpb] + diagonal [L][cpb][L] + z/r^2, 1/r^2 [L][cpb]  (same sizes for the df32 variant)
    auto need = [&](int cpb) {
        return (size_t)S.NH * cpb * sizeof(double2) + (size_t)S.L * cpb * S.L * sizeof(double2) +
               2 * (size_t)S.L * cpb * sizeof(double);
    };
    // enough blocks to cover every SM at least twice, within the shared-memory budget
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int cpb = 32;
    while (cpb > 4 && (need(cpb) > 200 * 1024 || cpb * S.L > 1024 || (S.ncell + cpb - 1) / cpb < 2 * sms)) cpb /= 2;
    const size_t smem = need(cpb);
    dim3 block(cpb, S.L);
    dim3 grid((S.ncell + cpb - 1) / cpb);
    if (mode == 0 && S.accept_df32 && S.L <= 20) {
        // register form: 16 cells x L columns x G source groups per block
        int G = s->tune[KMC_TUNE_P2L_GROUPS];
        if (G <= 0) G = 2;
        while (G > 1 && kP2lCells * S.L * G > (S.L <= 12 ? 384 : 512)) --G;
        const size_t sm = p2l_df2_smem(S.L, S.NH, G);
        // Orders l >= ld accumulate in FP32.  Their increments reach a proposal's energy
        // scaled by (r/d)^l (r <= 0.87 cell widths, d >= 2); over 30,000 accepts of the
        // 48^3 lattice the expansions moved 1.6e-11 from the FP64 path and no proposal
        // difference changed by more than 1e-10.
        const int ld = s->tune[KMC_TUNE_P2L_FP32_FROM] > 0 ? s->tune[KMC_TUNE_P2L_FP32_FROM] : kP2lFp32From;
        dim3 blk(kP2lCells, S.L, G);
        dim3 grd((S.ncell + kP2lCells - 1) / kP2lCells);
        LaunchScope ls(s, K_P2L);
        if (S.L == kP2pL && ld == kP2pLd && s->tune[KMC_TUNE_P2L_PAIR] == 0) {
            // column pairs: 2 or 4 source groups (4 unless the groups setting asks for 2)
            const int gp = s->tune[KMC_TUNE_P2L_GROUPS] == 2 ? 2 : 4;
            const size_t smp = std::max(p2l_df2_smem(S.L, S.NH, 1), (size_t)gp * kP2lCells * S.NH * sizeof(float4));
            if (gp == 2)
                k_p2l_pair<2><<<grd, dim3(kP2lCells, 2, kP2pPairs), smp, s->stream>>>(S, s->d_rec, nsrc);
            else
                k_p2l_pair<4><<<grd, dim3(kP2lCells, 4, kP2pPairs), smp, s->stream>>>(S, s->d_rec, nsrc);
        } else if (S.L <= 8)
            k_p2l_df2<8><<<grd, blk, sm, s->stream>>>(S, s->d_rec, nsrc, ld);
        else if (S.L <= 12)
            k_p2l_df2<12><<<grd, blk, sm, s->stream>>>(S, s->d_rec, nsrc, ld);
        else if (S.L <= 16)
            k_p2l_df2<16><<<grd, blk, sm, s->stream>>>(S, s->d_rec, nsrc, ld);
        else
            k_p2l_df2<20><<<grd, blk, sm, s->stream>>>(S, s->d_rec, nsrc, ld);
    } else if (mode == 0 && S.accept_df32) {
        // source groups: as many as the sources need, within shared memory and 1024 threads
        auto need_df = [&](int cp, int G) {
            return (size_t)G * S.NH * cp * sizeof(float4) + (size_t)G * S.L * cp * S.L * sizeof(float4) +
                   2 * (size_t)G * S.L * cp * sizeof(float2);
        };
        int G = (nsrc + S.L - 1) / S.L;
        int cp = 8;
        while (G > 1 && (need_df(cp, G) > 110 * 1024 || cp * S.L * G > 1024)) --G;
        while (cp > 2 && (need_df(cp, G) > 110 * 1024 || cp * S.L * G > 1024)) cp /= 2;
        dim3 blk(cp, S.L, G);
        dim3 grd((S.ncell + cp - 1) / cp);
        LaunchScope ls(s, K_P2L);
        k_p2l_df<<<grd, blk, need_df(cp, G), s->stream>>>(S, s->d_rec, nsrc);
    } else if (mode == 0 && (S.L == 8 || S.L == 12 || S.L == 16) && s->tune[KMC_TUNE_P2L64] != 1 &&
               p2l64_smem(S.L, S.NH, 1, nsrc, kP64Groups) <= 200 * 1024) {
        // FP64 column pairs: cells x source groups x pairs, a warp per pair; the groups (and
        // so every rounding) depend only on the number of sources: 16, or as many as the
        // sources rounded up to a power of two when fewer (free space: the old and new
        // position, 2 groups); the cells per block (tuning: 2, 4, 8 at 16 groups, scaled up
        // with fewer groups to the same threads per block) change nothing in the results
        int G = kP64Groups;
        while (G > 1 && G / 2 >= nsrc) G /= 2;
        int cpb = s->tune[KMC_TUNE_P2L64_CELLS] > 0 ? s->tune[KMC_TUNE_P2L64_CELLS] : 2;
        cpb *= kP64Groups / G;
        const int cmin = 2 * kP64Groups / G;
        while (cpb > cmin && (p2l64_smem(S.L, S.NH, cpb, nsrc, G) > 200 * 1024 || (S.L > 12 && cpb * G > 4 * kP64Groups)))
            cpb /= 2;
        dim3 blk(cpb, G, S.L / 2);
        dim3 grd((S.ncell + cpb - 1) / cpb);
        size_t sm = p2l64_smem(S.L, S.NH, cpb, nsrc, G);
        // at most `per_sm` blocks resident per SM (tuning): the block's shared memory padded so
        // that one more does not fit, which leaves the rest of each SM to the other systems'
        // kernels (the near field) in a batch
        const int per_sm = s->tune[KMC_TUNE_P2L64_PER_SM];
        if (per_sm > 0 && s->smem_sm > 0) {
            const size_t pad = (size_t)s->smem_sm / (per_sm + 1) - 1024 + 256;
            if (pad > sm && pad <= 200 * 1024) sm = pad;
        }
        LaunchScope ls(s, K_P2L);
        if (S.L == 8)
            k_p2l64<8><<<grd, blk, sm, s->stream>>>(S, s->d_rec, nsrc);
        else if (S.L == 12)
            k_p2l64<12><<<grd, blk, sm, s->stream>>>(S, s->d_rec, nsrc);
        else
            k_p2l64<16><<<grd, blk, sm, s->stream>>>(S, s->d_rec, nsrc);
    } else if (mode == 0) {
        LaunchScope ls(s, K_P2L);
        k_p2l<0><<<grid, block, smem, s->stream>>>(S, s->d_rec, nsrc);
    } else {
        LaunchScope ls(s, K_INIT);
        k_p2l<1><<<grid, block, smem, s->stream>>>(S, s->d_rec, nsrc);
    }
    KMC_LAUNCH_CHECK();
    return KMC_OK;
}

int refresh_mixed(kmc_system *s, bool store, bool lexp);

int bin_host(const kmc_system *s, double x)
{
    long long c = (long long)((x + 0.5 * s->S.E) * s->S.inv_w);
    if (c >= s->S.n) c = s->S.n - 1;
    return (int)c;
}

// store (re)build from host positions/cells: slots in particle-index order
// (kmc_local.py:582-825 appends particles to each cell in index order)
int build_store(kmc_system *s, const std::vector<int> &pcell, int cap)
{
    Sys &S = s->S;
    const int N = S.N;
    std::vector<int> cnt(S.ncell, 0), slot(N);
    for (int i = 0; i < N; ++i) slot[i] = cnt[pcell[i]]++;
    int maxocc = 1;
    for (int c = 0; c < S.ncell; ++c) maxocc = std::max(maxocc, cnt[c]);
    if (cap < maxocc) cap = std::max(maxocc + 16, 2 * maxocc);
    cap = (cap + 3) & ~3;
    S.cap = cap;
    std::vector<double> hpos(3 * (size_t)N), hq(N);
    KMC_CUDA(cudaMemcpy(hpos.data(), s->d_pos, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost));
    KMC_CUDA(cudaMemcpy(hq.data(), s->d_q, sizeof(double) * N, cudaMemcpyDeviceToHost));
    std::vector<double4_32a> st((size_t)S.ncell * cap, make_double4_32a(0, 0, 0, 0));
    std::vector<int> sp((size_t)S.ncell * cap, -1);
    for (int i = 0; i < N; ++i) {
        const size_t a = (size_t)pcell[i] * cap + slot[i];
        st[a] = make_double4_32a(hpos[3 * i], hpos[3 * i + 1], hpos[3 * i + 2], hq[i]);
        sp[a] = i;
    }
    int rc;
    if ((rc = dalloc(&s->d_store, st.size()))) return rc;
    if ((rc = dalloc(&s->d_store_pid, sp.size()))) return rc;
    KMC_CUDA(cudaMemcpy(s->d_store, st.data(), sizeof(double4_32a) * st.size(), cudaMemcpyHostToDevice));
    KMC_CUDA(cudaMemcpy(s->d_store_pid, sp.data(), sizeof(int) * sp.size(), cudaMemcpyHostToDevice));
    KMC_CUDA(cudaMemcpy(s->d_cnt, cnt.data(), sizeof(int) * S.ncell, cudaMemcpyHostToDevice));
    KMC_CUDA(cudaMemcpy(s->d_pslot, slot.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    KMC_CUDA(cudaMemcpy(s->d_pcell, pcell.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    if (S.mixed) {
        if ((rc = dalloc(&s->d_st_hi, (size_t)S.ncell * cap))) return rc;
        if ((rc = dalloc(&s->d_st_lo, (size_t)S.ncell * cap))) return rc;
    }
    s->h_cnt = cnt;
    s->h_pcell = pcell;
    s->mirror_valid = true;
    sync_sys_ptrs(s);
    return refresh_mixed(s, true, false);
}

// grow the per-cell store capacity, keeping slot order
// Reallocate the cell store with `want` slots per cell (default: twice the
// current capacity), keeping every cell's slot order (the reference's
// _resize_particle_store, kmc_local.py:558-580).
int grow_store(kmc_system *s, int want = 0)
{
    Sys &S = s->S;
    std::vector<int> pcell(S.N);
    KMC_CUDA(cudaStreamSynchronize(s->stream));
    KMC_CUDA(cudaMemcpy(pcell.data(), s->d_pcell, sizeof(int) * S.N, cudaMemcpyDeviceToHost));
    std::vector<int> cnt(S.ncell), slot(S.N), spid((size_t)S.ncell * S.cap);
    KMC_CUDA(cudaMemcpy(cnt.data(), s->d_cnt, sizeof(int) * S.ncell, cudaMemcpyDeviceToHost));
    KMC_CUDA(cudaMemcpy(spid.data(), s->d_store_pid, sizeof(int) * spid.size(), cudaMemcpyDeviceToHost));
    std::vector<double4_32a> st((size_t)S.ncell * S.cap);
    KMC_CUDA(cudaMemcpy(st.data(), s->d_store, sizeof(double4_32a) * st.size(), cudaMemcpyDeviceToHost));
    int maxcnt = 1;
    for (int c = 0; c < S.ncell; ++c) maxcnt = std::max(maxcnt, cnt[c]);
    const int ncap = ((std::max(want > 0 ? want : 2 * S.cap, maxcnt) + 3) & ~3);
    std::vector<double4_32a> nst((size_t)S.ncell * ncap, make_double4_32a(0, 0, 0, 0));
    std::vector<int> nsp((size_t)S.ncell * ncap, -1);
    for (int c = 0; c < S.ncell; ++c)
        for (int k = 0; k < cnt[c]; ++k) {
            nst[(size_t)c * ncap + k] = st[(size_t)c * S.cap + k];
            nsp[(size_t)c * ncap + k] = spid[(size_t)c * S.cap + k];
        }
    int rc;
    if ((rc = dalloc(&s->d_store, nst.size()))) return rc;
    if ((rc = dalloc(&s->d_store_pid, nsp.size()))) return rc;
    KMC_CUDA(cudaMemcpy(s->d_store, nst.data(), sizeof(double4_32a) * nst.size(), cudaMemcpyHostToDevice));
    KMC_CUDA(cudaMemcpy(s->d_store_pid, nsp.data(), sizeof(int) * nsp.size(), cudaMemcpyHostToDevice));
    S.cap = ncap;
    s->layout_gen++;
    if (S.mixed) {
        if ((rc = dalloc(&s->d_st_hi, (size_t)S.ncell * ncap))) return rc;
        if ((rc = dalloc(&s->d_st_lo, (size_t)S.ncell * ncap))) return rc;
    }
    s->h_cnt = cnt;
    s->h_pcell = pcell;
    s->mirror_valid = true;
    sync_sys_ptrs(s);
    return refresh_mixed(s, true, false);
}


// g = A M (state), after every change of M
int update_g(kmc_system *s, cudaStream_t st = nullptr)
{
    if (!s->S.pbc) return KMC_OK;
    if (!st) st = s->stream;
    LaunchScope ls(s, K_LR_G, st);
    k_lr_g<<<1, 256, (size_t)s->S.NH * sizeof(double2), st>>>(s->S, s->P);
    KMC_LAUNCH_CHECK();
    return KMC_OK;
}

// Per-charge far-lattice cache (mixed pbc): all charges (rec == nullptr, after a
// change of the charge set) or the accepted one (rec on the device, on stream st).
int lr_cache_fill(kmc_system *s, const AcceptRec *rec = nullptr, cudaStream_t st = nullptr)
{
    const Sys &S = s->S;
    if (!S.mixed || !S.pbc) return KMC_OK;
    if (!st) st = s->stream;
    int rc;
    if (!rec && S.N > s->hc_stride) {
        s->hc_valid = false;
        if ((rc = dalloc(&s->d_hc, (size_t)S.NH * S.N)) || (rc = dalloc(&s->d_hself, (size_t)S.N))) return rc;
        s->hc_stride = S.N;
    }
    if (rec && !s->hc_valid) return KMC_OK;
    if (!S.accept_df32) {
        // FP64 accept contributions: the operator applied in FP64 as well
        const unsigned gb = rec ? 1u : (unsigned)((S.N + kLf64Warps - 1) / kLf64Warps);
        if (gb == 0) {
            s->hc_valid = true;
            return KMC_OK;
        }
        LaunchScope ls(s, rec ? K_ACCEPT_MPOLE : K_LR_OLD, st);
        if (rec)
            k_lr_refresh64<<<1, kLr1Threads, S.NH * sizeof(double2) + kLr1Threads * sizeof(double), st>>>(
                S, s->d_hc, s->hc_stride, s->d_hself, rec);
        else
            k_lr_fill64<<<gb, kLf64Warps * 32, (size_t)kLf64Warps * S.NH * sizeof(double2), st>>>(
                S, s->d_hc, s->hc_stride, s->d_hself, rec);
        KMC_LAUNCH_CHECK();
        if (!rec) s->hc_valid = true;
        return KMC_OK;
    }
    const size_t nnz = s->ar_val.size() + s->ai_val.size();
    const bool staged = lr_old_mixed_smem(S.NH, nnz, true) <= 200 * 1024;
    if (rec) {
        LaunchScope ls(s, K_ACCEPT_MPOLE, st);
        const size_t sm = (((size_t)4 * S.NH + 2 * S.L * S.L + S.L + 1) & ~(size_t)1) * sizeof(float),
                     smf = sm + nnz * sizeof(float2);
        const bool fits = smf <= 48 * 1024;  // the folded form copied beside the planes
        if (staged && fits)
            k_lr_refresh_one<true, true><<<1, 256, smf, st>>>(S, s->d_hc, s->hc_stride, s->d_hself, rec);
        else if (staged)
            k_lr_refresh_one<true, false><<<1, 256, sm, st>>>(S, s->d_hc, s->hc_stride, s->d_hself, rec);
        else
            k_lr_refresh_one<false, false><<<1, 256, sm, st>>>(S, s->d_hc, s->hc_stride, s->d_hself, rec);
        KMC_LAUNCH_CHECK();
        return KMC_OK;
    }
    const unsigned gb = (unsigned)((S.N + kLrThreads - 1) / kLrThreads);
    if (gb == 0) {
        s->hc_valid = true;
        return KMC_OK;
    }
    LaunchScope ls(s, K_LR_OLD, st);
    if (staged)
        k_lr_old_mixed<true, true><<<gb, kLrThreads, lr_old_mixed_smem(S.NH, nnz, true), st>>>(
            S, s->P, s->d_hc, s->hc_stride, s->d_hself, rec);
    else
        k_lr_old_mixed<false, true><<<gb, kLrThreads, lr_old_mixed_smem(S.NH, nnz, false), st>>>(
            S, s->P, s->d_hc, s->hc_stride, s->d_hself, rec);
    KMC_LAUNCH_CHECK();
    if (!rec) s->hc_valid = true;
    return KMC_OK;
}

int refresh_mixed(kmc_system *s, bool store, bool lexp)
{
    const Sys &S = s->S;
    if (!S.mixed) return KMC_OK;
    LaunchScope ls(s, K_REFRESH);
    if (store) {
        const size_t n = (size_t)S.ncell * S.cap;
        k_refresh_store32<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(S);
        KMC_LAUNCH_CHECK();
    }
    if (lexp) {
        const size_t n = (size_t)S.ncell * S.NH;
        k_refresh_lexp32<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(S);
        KMC_LAUNCH_CHECK();
    }
    return KMC_OK;
}

// lattice term (pbc) or plain difference, after u0p / pnew are ready
// Far-lattice term (pbc) on stream st: the old-side constants co and h = A b per
// moving charge, then the new-side part of every proposal into P.elr.
int launch_lattice(kmc_system *s, cudaStream_t st, int64_t n_old_grid, int64_t n_new_grid, bool mixed)
{
    const Sys &S = s->S;
    const int tb = 128;
    const unsigned go = (unsigned)((n_old_grid + tb - 1) / tb), gn = (unsigned)((n_new_grid + tb - 1) / tb);
    // the mixed mode with FP64 accept contributions applies the lattice operator in FP64
    // (the per-charge cache of k_lr_fill64): the FP32 operator variants are not used
    const bool op64 = mixed && !S.accept_df32 && s->hc_valid;
    if (mixed && !op64 && s->tune[KMC_TUNE_LR_FUSED] == 1) {
        const size_t nnz = s->ar_val.size() + s->ai_val.size();
        const bool staged = lr_fused_smem(S.NH, nnz, true) <= 200 * 1024 && s->tune[KMC_TUNE_LR_STAGE] == 0;
        const unsigned gb = (unsigned)((n_old_grid + kLfMovers - 1) / kLfMovers);
        LaunchScope ls(s, K_LR, st);
        if (staged)
            k_lr_fused_mixed<true><<<gb, kLfMovers * kLfWarps, lr_fused_smem(S.NH, nnz, true), st>>>(S, s->P);
        else
            k_lr_fused_mixed<false><<<gb, kLfMovers * kLfWarps, lr_fused_smem(S.NH, nnz, false), st>>>(S, s->P);
        KMC_LAUNCH_CHECK();
        return KMC_OK;
    }
    // proposals per block of the per-proposal lattice kernels (tuning; the per-thread
    // arithmetic does not depend on it)
    const int lrt = s->tune[KMC_TUNE_LR_THREADS] > 0 ? s->tune[KMC_TUNE_LR_THREADS] : kLrNewThreads;
    if (op64 || (mixed && s->hc_valid && s->tune[KMC_TUNE_LR_NOCACHE] == 0)) {
        {
            LaunchScope ls(s, K_LR_OLD, st);
            const unsigned gco = (unsigned)((n_old_grid + lrt - 1) / lrt);
            if (S.L == 12)
                k_lr_co_mixed<12><<<gco, lrt, S.NH * sizeof(float4), st>>>(S, s->P, s->d_hself);
            else
                k_lr_co_mixed<<<gco, lrt, S.NH * sizeof(float4), st>>>(S, s->P, s->d_hself);
        }
        KMC_LAUNCH_CHECK();
        {
            LaunchScope ls(s, K_LR, st);
            const unsigned gnw = (unsigned)((n_new_grid + lrt - 1) / lrt);
            const size_t sm = S.NH * sizeof(float4);
            if (S.L == 12 && s->fs12_ok && s->tune[KMC_TUNE_FSELF_GENERIC] == 0)
                k_lr_new_mixed<true, 12, true><<<gnw, lrt, sm, st>>>(S, s->P, s->d_hc, s->hc_stride,
                                                                                 s->fs12);
            else if (S.L == 12)
                k_lr_new_mixed<true, 12><<<gnw, lrt, sm, st>>>(S, s->P, s->d_hc, s->hc_stride, s->fs12);
            else
                k_lr_new_mixed<true><<<gnw, lrt, sm, st>>>(S, s->P, s->d_hc, s->hc_stride, s->fs12);
        }
        KMC_LAUNCH_CHECK();
        return KMC_OK;
    }
    if (mixed) {
        float2 *h32 = reinterpret_cast<float2 *>(s->P.h);
        const int hstride = (int)s->prop_n;
        {
            LaunchScope ls(s, K_LR_OLD, st);
            const size_t nnz = s->ar_val.size() + s->ai_val.size();
            const unsigned gb = (unsigned)((n_old_grid + kLrThreads - 1) / kLrThreads);
            if (lr_old_mixed_smem(S.NH, nnz, true) <= 200 * 1024)
                k_lr_old_mixed<true><<<gb, kLrThreads, lr_old_mixed_smem(S.NH, nnz, true), st>>>(S, s->P, h32,
                                                                                                  hstride);
            else
                k_lr_old_mixed<false><<<gb, kLrThreads, lr_old_mixed_smem(S.NH, nnz, false), st>>>(S, s->P, h32,
                                                                                                    hstride);
        }
        KMC_LAUNCH_CHECK();
        {
            LaunchScope ls(s, K_LR, st);
            const unsigned gnw = (unsigned)((n_new_grid + kLrNewThreads - 1) / kLrNewThreads);
            if (S.L == 12 && s->fs12_ok && s->tune[KMC_TUNE_FSELF_GENERIC] == 0)
                k_lr_new_mixed<false, 12, true><<<gnw, kLrNewThreads, S.NH * sizeof(float4), st>>>(S, s->P, h32,
                                                                                                  hstride, s->fs12);
            else
                k_lr_new_mixed<false><<<gnw, kLrNewThreads, S.NH * sizeof(float4), st>>>(S, s->P, h32, hstride,
                                                                                       s->fs12);
        }
        KMC_LAUNCH_CHECK();
        return KMC_OK;
    }
    {
        LaunchScope ls(s, K_LR_OLD, st);
        if (S.NH <= 136)
            k_lr_old<136><<<go, tb, 0, st>>>(S, s->P);
        else
            k_lr_old<KMC_LMAX *(KMC_LMAX + 1) / 2><<<go, tb, 0, st>>>(S, s->P);
    }
    KMC_LAUNCH_CHECK();
    {
        LaunchScope ls(s, K_LR, st);
        if (S.NH <= 136)
            k_lr_new<136><<<gn, tb, 0, st>>>(S, s->P);
        else
            k_lr_new<KMC_LMAX *(KMC_LMAX + 1) / 2><<<gn, tb, 0, st>>>(S, s->P);
    }
    KMC_LAUNCH_CHECK();
    return KMC_OK;
}

// The lattice term depends only on the compacted proposals, not on the near field:
// it runs on the side stream while the main stream computes the near field.
int lattice_fork(kmc_system *s, int64_t n_old_grid, int64_t n_new_grid, bool mixed)
{
    if (!s->S.pbc) return KMC_OK;
    KMC_CUDA(cudaEventRecord(s->ev_lfork, s->stream));
    KMC_CUDA(cudaStreamWaitEvent(s->side, s->ev_lfork, 0));
    const int rc = launch_lattice(s, s->side, n_old_grid, n_new_grid, mixed);
    if (rc) return rc;
    KMC_CUDA(cudaEventRecord(s->ev_ljoin, s->side));
    return KMC_OK;
}

// join the lattice branch and write the differences in rate_location order
int run_finish(kmc_system *s, int64_t n_new_grid, double *out)
{
    const Sys &S = s->S;
    if (S.pbc) KMC_CUDA(cudaStreamWaitEvent(s->stream, s->ev_ljoin, 0));
    const int tb = 128;
    LaunchScope ls(s, K_DIFF);
    k_diff<<<(unsigned)((n_new_grid + tb - 1) / tb), tb, 0, s->stream>>>(S, s->P, out);
    KMC_LAUNCH_CHECK();
    return KMC_OK;
}

// thread-per-item near/far (small explicit-move batches)
int run_old_new(kmc_system *s, int64_t n_old_grid, int64_t n_new_grid, double *out)
{
    const Sys &S = s->S;
    const int tb = 128;
    int rc = lattice_fork(s, n_old_grid, n_new_grid, false);
    if (rc) return rc;
    {
        LaunchScope ls(s, K_OLD);
        k_old<<<(unsigned)((n_old_grid + tb - 1) / tb), tb, 0, s->stream>>>(S, s->P, 0);
    }
    KMC_LAUNCH_CHECK();
    {
        LaunchScope ls(s, K_NEW);
        k_new<<<(unsigned)((n_new_grid + tb - 1) / tb), tb, 0, s->stream>>>(S, s->P, out);
    }
    KMC_LAUNCH_CHECK();
    return run_finish(s, n_new_grid, out);
}

// cell-staged near/far (full proposal batches); proposals' cells already counted
// Proposal set-up of propose_with_dats on stream st (setup_propose_with_dats,
// kmc_mpi_decomp.py:489-736): active moves counted and compacted in
// exclusive_sum order, then grouped by target cell.  Writes only the proposal
// buffers (and the bad-move counter), so it may run beside an accept.
int propose_prepare(kmc_system *s, cudaStream_t st, int N, int M, const int64_t *site_max_counts,
                    const int64_t *current_sites, const double *prop_positions, const int64_t *prop_masks,
                    const double *prop_charges, const bool check = true, const int *prop_cells = nullptr)
{
    const Sys &S = s->S;
    const int nb = (N + kScanBlock - 1) / kScanBlock;
    s->props_ready = true;
    KMC_CUDA(cudaMemsetAsync(s->P.ccount, 0, sizeof(int) * S.ncell, st));
    {
        LaunchScope ls(s, K_COUNT_SCAN, st);
        k_count_scan<<<nb, kScanBlock, 0, st>>>(N, M, (const long long *)site_max_counts,
                                                (const long long *)current_sites, (const long long *)prop_masks,
                                                s->P);
    }
    KMC_LAUNCH_CHECK();
    {
        LaunchScope ls(s, K_SCAN_PART, st);
        k_scan_part<<<1, kScanBlock, 0, st>>>(nb, s->P);
    }
    KMC_LAUNCH_CHECK();
    {
        LaunchScope ls(s, K_SCATTER, st);
        const unsigned gs = (unsigned)(((long long)N * M + 127) / 128);
        if (check)
            k_scatter<true><<<gs, 128, 0, st>>>(S, N, M, prop_positions, (const long long *)prop_masks, prop_charges,
                                               prop_cells, s->P, s->d_err);
        else
            k_scatter<false><<<gs, 128, 0, st>>>(S, N, M, prop_positions, (const long long *)prop_masks,
                                                prop_charges, prop_cells, s->P, s->d_err);
    }
    KMC_LAUNCH_CHECK();
    {
        LaunchScope ls(s, K_CELL_SORT, st);
        k_cell_scan<<<1, 1024, 0, st>>>(S.ncell, s->P);
    }
    KMC_LAUNCH_CHECK();
    {
        LaunchScope ls(s, K_CELL_SORT, st);
        k_cell_place<<<(unsigned)(((long long)N * M + 127) / 128), 128, 0, st>>>(s->P);
    }
    KMC_LAUNCH_CHECK();
    return KMC_OK;
}

// The moved pair's self term stays in the mixed near field for every boundary
// condition: there it is formed from the same grid coordinates as the near-field pair
// of the proposal with the charge's old slot, whose rounding it cancels (a separate
// evaluation in box units left ~2.5e-8 of 1/|x_new - x_old| for short moves).
bool lattice_takes_self(const kmc_system *s)
{
    (void)s;
    return false;
}

// Evaluation of prepared proposals on the system's stream: the lattice term on
// the side stream beside the near field, then the differences.
int propose_evaluate(kmc_system *s, int64_t n_old_grid, int64_t n_new_grid, double *out)
{
    const Sys &S = s->S;
    int rc = lattice_fork(s, n_old_grid, n_new_grid, S.mixed != 0);
    if (rc) return rc;
    // the moving charges' near-field potentials from S.phin unless the tuning asks for
    // them summed afresh (the accepts keep S.phin current either way)
    const bool kept = s->tune[KMC_TUNE_NEAR_OLD] != 1;
    if (S.mixed) {
        // 128 staged neighbours per chunk keep a one-warp block near 7 KB of shared
        // memory, so about 28 blocks fit an SM and a 4,096-cell grid runs in one wave
        const int chunk = s->tune[KMC_TUNE_NEAR_CHUNK] == 1 ? 256 : (s->tune[KMC_TUNE_NEAR_CHUNK] == 2 ? 64 : 128);
        const size_t smem =
            chunk * (2 * sizeof(float4) + 2 * sizeof(int) + sizeof(unsigned long long)) + (size_t)S.NH * sizeof(float4);
        LaunchScope ls(s, K_NEAR_CELL);
        const bool scalar = s->tune[KMC_TUNE_NEAR_SCALAR] == 1;
        // blocks per cell (tuning): the item rounds of a cell spread over `split` blocks,
        // results unchanged
        const int split = s->tune[KMC_TUNE_NEAR_SPLIT] > 0 ? s->tune[KMC_TUNE_NEAR_SPLIT] : 1;
        const bool sil = lattice_takes_self(s);
        // the mixed near field at the device's highest scheduling priority (tuning): when
        // many systems' kernels wait for SM resources, its blocks go first and the FP64
        // accept kernels of other systems fill what is left; results unchanged
        const int prio = s->tune[KMC_TUNE_NEAR_PRIORITY] == 1 ? s->prio_hi : 0;
        void (*kern)(const Sys, Props, const bool, const int, const bool);
        if (scalar && chunk == 256)
            kern = k_near_cell_mixed<false, 256>;
        else if (scalar)
            kern = k_near_cell_mixed<false, 128>;
        else if (chunk == 256)
            kern = k_near_cell_mixed<true, 256>;
        else if (chunk == 64)
            kern = S.L == 12 ? k_near_cell_mixed<true, 64, 12> : k_near_cell_mixed<true, 64>;
        else
            kern = S.L == 12 ? k_near_cell_mixed<true, 128, 12> : k_near_cell_mixed<true, 128>;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)(S.ncell * split));
        cfg.blockDim = dim3(kNearMixedThreads);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = s->stream;
        cudaLaunchAttribute attr[1];
        if (prio != 0) {
            attr[0].id = cudaLaunchAttributePriority;
            attr[0].val.priority = prio;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
        }
        KMC_CUDA(cudaLaunchKernelEx(&cfg, kern, S, s->P, sil, split, kept));
    } else {
        const size_t smem = kNearChunk * (sizeof(double4_32a) + sizeof(int)) + (size_t)S.NH * sizeof(double2);
        LaunchScope ls(s, K_NEAR_CELL);
        k_near_cell<<<S.ncell, kNearThreads, smem, s->stream>>>(S, s->P, kept);
    }
    KMC_LAUNCH_CHECK();
    return run_finish(s, n_new_grid, out);
}

} // namespace
