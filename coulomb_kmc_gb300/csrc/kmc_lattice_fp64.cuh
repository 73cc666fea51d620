// Part of the kmc_gb300.cu translation unit (included there, in order, inside its
// anonymous namespace unless it says otherwise): the FP64 far-field lattice term: g = A M, the far-lattice self-term polynomial F and the per-charge / per-proposal kernels.
#pragma once
// ---------------------------------------------------------------------------
// far-field lattice term (pbc): dE_LR = d^T A (M + d/2), d = q' m(x_n) - q m(x_o)
// (long_range_energy, kmc_full_long_range.py:710-858, as a difference of the
//  quadratic form E_LR(M) = 1/2 M^T A M)
// ---------------------------------------------------------------------------
// g = A M, part of the state: recomputed whenever M changes (initialise, accept),
// so E_LR(M) = 1/2 M^T g and every proposal's lattice term reads g.
__global__ void k_lr_g(const Sys S, Props P)
{
    extern __shared__ double2 gsm[];  // M [NH]
    for (int r = threadIdx.x; r < S.NH; r += blockDim.x) gsm[r] = S.mpole[r];
    __syncthreads();
    for (int r = threadIdx.x; r < S.NH; r += blockDim.x) {
        double t = 0.0, u = 0.0;
        for (int k = S.ar_ptr[r]; k < S.ar_ptr[r + 1]; ++k) t += S.ar_val[k] * gsm[S.ar_col[k]].x;
        for (int k = S.ai_ptr[r]; k < S.ai_ptr[r + 1]; ++k) u += S.ai_val[k] * gsm[S.ai_col[k]].y;
        P.g[r] = make_double2(t, u);
    }
}

// per moving charge: b = q m(x_old), h = A b, co = b^T h / 2 - b^T g
// F(x) from the evaluation program of lattice_self_program: per column mu the
// diagonal D_mu (x + i y)^mu, the regular-harmonic recurrence up in lambda, and per
// listed (lambda, re/im) a polynomial in r^2.
template <typename T>
__device__ __forceinline__ T lattice_self(const int *__restrict__ pi, const T *__restrict__ pd, const T x, const T y,
                                          const T z)
{
    const T r2 = x * x + y * y + z * z;
    T acc = T(0), wre = T(1), wim = T(0);
    int mcur = 0, io = 1, dof = 0;
    const int ncol = __ldg(&pi[0]);
    for (int c = 0; c < ncol; ++c) {
        const int mu = __ldg(&pi[io]), lmax = __ldg(&pi[io + 1]), nent = __ldg(&pi[io + 2]);
        io += 3;
        for (; mcur < mu; ++mcur) {
            const T nr = wre * x - wim * y;
            wim = wre * y + wim * x;
            wre = nr;
        }
        const T D = __ldg(&pd[dof]);
        const int rec = dof + 1;
        dof = rec + 2 * (lmax - mu);
        T cre = D * wre, cim = D * wim, qre = T(0), qim = T(0);
        int lam = mu;
        for (int e = 0; e < nent; ++e) {
            const int el = __ldg(&pi[io]), kind = __ldg(&pi[io + 1]), np = __ldg(&pi[io + 2]);
            io += 3;
            for (; lam < el; ++lam) {
                const T a = __ldg(&pd[rec + 2 * (lam - mu)]), b = __ldg(&pd[rec + 2 * (lam - mu) + 1]);
                const T az = a * z, br = b * r2;
                const T nre = az * cre - br * qre, nim = az * cim - br * qim;
                qre = cre;
                qim = cim;
                cre = nre;
                cim = nim;
            }
            T poly = T(0);
            for (int k = np - 1; k >= 0; --k) poly = poly * r2 + __ldg(&pd[dof + k]);
            dof += np;
            acc += poly * (kind ? cim : cre);
        }
    }
    return acc;
}

// The program lattice_self_program writes for the cubic lattice at L = 12 has a fixed
// shape (fself12_shape checks it on the host): columns mu = 0, 4, ..., 20, each
// recurring to lambda = 22, real entries lambda = 12, 14, ..., 22 (from lambda = mu
// when mu > 12) with one coefficient each, and in column 0 also lambda = 0 (c0 + c1 r^2)
// and lambda = 2.  With that shape known at compile time the reals ride in the kernel's
// parameter bank and the loops unroll: about 350 FP32 operations per point instead of
// the interpreter's loads and loop control.
constexpr int kFs12Reals = 183;
struct FSelf12 {
    float v[kFs12Reals + 1];  // lattice_self_program's reals in program order, F32, box units
};
__host__ __device__ constexpr int fs12_first(int mu) { return mu > 12 ? mu : 12; }
__host__ __device__ constexpr int fs12_col_reals(int mu)
{
    return 1 + 2 * (22 - mu) + (22 - fs12_first(mu)) / 2 + 1 + (mu == 0 ? 3 : 0);
}
__host__ __device__ constexpr int fs12_off(int mu) { return mu == 0 ? 0 : fs12_off(mu - 4) + fs12_col_reals(mu - 4); }
static_assert(fs12_off(24) == kFs12Reals, "F program layout at L = 12");

// one column: c_lambda = Re(D_mu (x + i y)^mu) recurred in lambda, dotted with the entries
template <int MU>
__device__ __forceinline__ float fself12_column(const float *__restrict__ v, const float wre, const float z,
                                                const float r2)
{
    constexpr int OFF = fs12_off(MU), REC = OFF + 1, ENT = REC + 2 * (22 - MU), FIRST = fs12_first(MU);
    constexpr int E12 = ENT + (MU == 0 ? 3 : 0);  // entry of lambda = FIRST
    float c = v[OFF] * wre, q = 0.0f, acc = 0.0f;
    if (MU == 0) acc = fmaf(v[ENT + 1], r2, v[ENT]) * c;
    if (MU >= 12) acc = v[E12] * c;
#pragma unroll
    for (int lam = MU + 1; lam <= 22; ++lam) {
        const float az = v[REC + 2 * (lam - MU - 1)] * z, br = v[REC + 2 * (lam - MU - 1) + 1] * r2;
        const float nc = fmaf(az, c, -(br * q));
        q = c;
        c = nc;
        if (MU == 0 && lam == 2) acc = fmaf(v[ENT + 2], c, acc);
        if (lam >= FIRST && lam > MU && (lam & 1) == 0) acc = fmaf(v[E12 + (lam - FIRST) / 2], c, acc);
    }
    return acc;
}

__device__ __forceinline__ float lattice_self_c12(const float *__restrict__ v, const float x, const float y,
                                                  const float z)
{
    const float r2 = x * x + y * y + z * z;
    const float sr = x * x - y * y, si = 2.0f * x * y;      // (x + i y)^2
    const float w4r = sr * sr - si * si, w4i = 2.0f * sr * si;  // (x + i y)^4
    float wr = w4r, wi = w4i;
    const auto next = [&]() {  // (x + i y)^(mu + 4)
        const float t = wr * w4r - wi * w4i;
        wi = wr * w4i + wi * w4r;
        wr = t;
        return wr;
    };
    float acc = fself12_column<0>(v, 1.0f, z, r2) + fself12_column<4>(v, wr, z, r2);
    acc += fself12_column<8>(v, next(), z, r2);
    acc += fself12_column<12>(v, next(), z, r2);
    acc += fself12_column<16>(v, next(), z, r2);
    acc += fself12_column<20>(v, next(), z, r2);
    return acc;
}

template <int NHMAX>
__global__ void k_lr_old(const Sys S, Props P)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= P.totals[0]) return;
    const int px = P.old_pid[o];
    double2 b[NHMAX];
    const int NH = S.NH;
    multipole_fp64(b, S.L, S.q[px], S.pos[3 * (size_t)px], S.pos[3 * (size_t)px + 1], S.pos[3 * (size_t)px + 2]);
    double bh = 0.0, bg = 0.0;
    double2 *h = P.h + (size_t)o * NH;
    for (int r = 0; r < NH; ++r) {
        double t = 0.0, u = 0.0;
        for (int k = __ldg(&S.ar_ptr[r]); k < __ldg(&S.ar_ptr[r + 1]); ++k)
            t += __ldg(&S.ar_val[k]) * b[__ldg(&S.ar_col[k])].x;
        for (int k = __ldg(&S.ai_ptr[r]); k < __ldg(&S.ai_ptr[r + 1]); ++k)
            u += __ldg(&S.ai_val[k]) * b[__ldg(&S.ai_col[k])].y;
        h[r] = make_double2(t, u);
        bh += b[r].x * t + b[r].y * u;
        const double2 gg = P.g[r];
        bg += b[r].x * gg.x + b[r].y * gg.y;
    }
    P.co[o] = 0.5 * bh - bg;
}

// per proposal: dE_LR = a^T g - a^T h + a^T A a / 2 + co, a = q' m(x_new)
// (long_range_energy, kmc_full_long_range.py:710-858, as a difference of
//  E_LR(M) = 1/2 M^T A M), then the final difference (diff_lib)
template <int NHMAX>
__global__ void k_lr_new(const Sys S, Props P)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.totals[1]) return;
    const int o = P.owner[p];
    double2 a[NHMAX];
    const int NH = S.NH;
    multipole_fp64(a, S.L, P.pq[p], P.ppos[3 * (size_t)p], P.ppos[3 * (size_t)p + 1], P.ppos[3 * (size_t)p + 2]);
    const double2 *h = P.h + (size_t)o * NH;
    double lin = 0.0;
    for (int r = 0; r < NH; ++r) {
        const double2 gg = P.g[r];
        const double2 hh = h[r];
        lin += a[r].x * (gg.x - hh.x) + a[r].y * (gg.y - hh.y);
    }
    // a^T A a / 2 = q'^2 F(x_new)
    const double qn = P.pq[p];
    const double F = lattice_self<double>(S.fprog_i, S.fprog_d, P.ppos[3 * (size_t)p], P.ppos[3 * (size_t)p + 1],
                                          P.ppos[3 * (size_t)p + 2]);
    P.elr[p] = lin + qn * qn * F + P.co[o];
}
