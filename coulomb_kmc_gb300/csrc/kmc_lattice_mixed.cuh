// Part of the kmc_gb300.cu translation unit (included there, in order, inside its
// anonymous namespace unless it says otherwise): the mixed-precision lattice term: the per-charge cache h = A b (FP32 and FP64 fills), the fused and split per-proposal kernels.
#pragma once
constexpr int kLrThreads = 64;

// delta_lm = q' conj Rg(x_new) - q conj Rg(x_old), both chains in lockstep, FP32,
// written to shared memory transposed: d[h * kLrThreads + tid]
// Mixed lattice term, split as in the FP64 path (k_lr_old / k_lr_new):
//   per moving charge  b = q_o a(x_o),  h = A b,  co = b^T h / 2 - b.g
//   per proposal       a = q_n a(x_n),  dE_LR = a.(g - h) + q_n^2 F(x_n) + co
// with F the far-lattice self term polynomial.  h = A b runs in FP32 with b in
// shared memory (real and imaginary planes, one column per thread) and the
// folded form staged once per block; b.g and a.g take l <= 2 in double-FP32.
// h is stored transposed, h32[r][o] (float2), for coalesced access.
// l <= 2 part of a . g for a = q conj Rg(x) (box units), in double-FP32 from
// double-FP32 coordinates and charge: these orders meet the largest entries of g
// (the dipole correction among them), where FP32 coordinates alone (2^-25 box
// units) would cost ~1e-7 in an energy difference.  Same recurrences as the FP32
// column loops, with the constants' low words.
__device__ __forceinline__ df32 lattice_low_dot(const df32 q, const df32 x, const df32 y, const df32 z,
                                                const float4 *__restrict__ g)
{
    auto K = [](const float2 v) { return df_make(v.x, v.y); };
    auto G = [&](const int h, df32 &gr, df32 &gi) {
        const float4 v = g[h];
        gr = df_make(v.x, v.z);
        gi = df_make(v.y, v.w);
    };
    const df32 r2 = df_add(df_add(df_mul(x, x), df_mul(y, y)), df_mul(z, z));
    // column m = 0: Rg_00 = 1, c10 = a_10 z, c20 = a_20 z c10 - b_20 r^2
    const df32 c10 = df_mul(K(c_rec_a2[1 * KMC_LMAX + 0]), z);
    const df32 c20 = df_sub(df_mul(df_mul(K(c_rec_a2[2 * KMC_LMAX + 0]), z), c10),
                            df_mul(K(c_rec_b2[2 * KMC_LMAX + 0]), r2));
    // column m = 1: c11 = d_1 (x + i y), c21 = a_21 z c11
    const df32 t1 = K(c_rec_d2[1]);
    const df32 c11r = df_mul(t1, x), c11i = df_mul(t1, y);
    const df32 a21z = df_mul(K(c_rec_a2[2 * KMC_LMAX + 1]), z);
    const df32 c21r = df_mul(a21z, c11r), c21i = df_mul(a21z, c11i);
    // column m = 2: c22 = d_2 (c11 (x + i y))
    const df32 t2 = K(c_rec_d2[2]);
    const df32 c22r = df_mul(t2, df_fms(c11r, x, c11i, y));
    const df32 c22i = df_mul(t2, df_fma2(c11r, y, c11i, x));
    df32 gr, gi;
    G(0, gr, gi);
    df32 acc = gr;
    G(1, gr, gi);
    acc = df_add(acc, df_mul(c10, gr));
    G(2, gr, gi);
    acc = df_add(acc, df_fms(c11r, gr, c11i, gi));
    G(3, gr, gi);
    acc = df_add(acc, df_mul(c20, gr));
    G(4, gr, gi);
    acc = df_add(acc, df_fms(c21r, gr, c21i, gi));
    G(5, gr, gi);
    acc = df_add(acc, df_fms(c22r, gr, c22i, gi));
    return df_mul(q, acc);
}

// Global-memory copies of the recurrence constants for code whose threads index
// them by their own column m: constant-bank reads with different addresses across a
// warp are serialised, while these go through L1 like any other load.
__device__ double g_rec_a[KMC_LMAX * KMC_LMAX], g_rec_b[KMC_LMAX * KMC_LMAX], g_rec_d[KMC_LMAX];
__device__ float2 g_rec_a2[KMC_LMAX * KMC_LMAX], g_rec_b2[KMC_LMAX * KMC_LMAX], g_rec_d2[KMC_LMAX];

// The FP64 recurrence constants of orders below L staged in shared memory by the
// whole block in one parallel round of loads (the caller synchronises), so that
// the per-column chains read shared memory instead of waiting on a load at every
// step: a_lm and b_lm at l * L + m, d_m.
struct RecTab {
    const double *a, *b, *d;
    int L;
};
__host__ __device__ constexpr int rec_tab_size(const int L) { return 2 * L * L + L; }
__device__ __forceinline__ RecTab stage_rec(double *t, const int L)
{
    for (int k = threadIdx.x; k < L * L; k += blockDim.x) {
        const int l = k / L, m = k - l * L;
        t[k] = g_rec_a[l * KMC_LMAX + m];
        t[L * L + k] = g_rec_b[l * KMC_LMAX + m];
    }
    for (int k = threadIdx.x; k < L; k += blockDim.x) t[2 * L * L + k] = g_rec_d[k];
    return RecTab{t, t + L * L, t + 2 * L * L, L};
}

__device__ __forceinline__ void multipole_planes_f32(float *bre, float *bim, const int stride, const int L,
                                                     const float q, const float x, const float y, const float z)
{
    const float r2 = x * x + y * y + z * z;
    float dre = 1.0f, dim = 0.0f;
    for (int m = 0; m < L; ++m) {
        if (m > 0) {
            const float t = c_rec_d2[m].x;
            const float nr = t * (dre * x - dim * y), ni = t * (dre * y + dim * x);
            dre = nr;
            dim = ni;
        }
        float pre = 0.0f, pim = 0.0f, cre = dre, cim = dim;
        bre[hidx(m, m) * stride] = q * cre;
        bim[hidx(m, m) * stride] = -q * cim;
        for (int l = m + 1; l < L; ++l) {
            const float a = c_rec_a2[l * KMC_LMAX + m].x * z, b = c_rec_b2[l * KMC_LMAX + m].x * r2;
            const float nr = a * cre - b * pre, ni = a * cim - b * pim;
            pre = cre;
            pim = cim;
            cre = nr;
            cim = ni;
            bre[hidx(l, m) * stride] = q * cre;
            bim[hidx(l, m) * stride] = -q * cim;
        }
    }
}

size_t lr_old_mixed_smem(const int NH, const size_t nnz, const bool staged)
{
    return (size_t)NH * sizeof(float4) + 2 * (size_t)NH * kLrThreads * sizeof(float) +
           (staged ? nnz * sizeof(float2) : 0) + 2 * (size_t)(NH + 1) * sizeof(int);
}

// STAGED: the folded form in shared memory (fits up to l = 16); otherwise read through the read-only cache.
// FILL: h = A b depends on a charge's own position only, so it is kept per charge
// between moves: the block computes h and b.h / 2 for charges (all of them, or
// the accepted one when rec is given) into h32[r][pid] and hself[pid], and
// nothing that depends on g.
template <bool STAGED, bool FILL = false>
__global__ void __launch_bounds__(kLrThreads) k_lr_old_mixed(const Sys S, Props P, float2 *h32, const int hstride,
                                                            double *hself = nullptr, const AcceptRec *rec = nullptr)
{
    extern __shared__ float4 lsm4[];
    const int NH = S.NH;
    float4 *g = lsm4;                                                     // [NH] (re hi, im hi, re lo, im lo)
    float *bre = reinterpret_cast<float *>(g + NH);                       // [NH][kLrThreads]
    float *bim = bre + (size_t)NH * kLrThreads;
    const int nr_ = S.ar_ptr[NH], ni_ = S.ai_ptr[NH];
    float2 *ue = reinterpret_cast<float2 *>(bim + (size_t)NH * kLrThreads);  // [nr_ + ni_] (value, column offset)
    int *rp = reinterpret_cast<int *>(ue + (STAGED ? nr_ + ni_ : 0));    // [2][NH + 1]
    const int tid = threadIdx.x;
    for (int r = tid; r < NH; r += blockDim.x) {
        const df32 gr = df_from_double(P.g[r].x * S.escale[r]), gi = df_from_double(P.g[r].y * S.escale[r]);
        g[r] = make_float4(gr.hi, gi.hi, gr.lo, gi.lo);
    }
    if (STAGED) {
        for (int k = tid; k < nr_; k += blockDim.x)
            ue[k] = make_float2(S.ar32_val[k], __int_as_float(S.ar_col[k] * kLrThreads));
        for (int k = tid; k < ni_; k += blockDim.x)
            ue[nr_ + k] = make_float2(S.ai32_val[k], __int_as_float(S.ai_col[k] * kLrThreads));
    }
    for (int r = tid; r <= NH; r += blockDim.x) {
        rp[r] = S.ar_ptr[r];
        rp[NH + 1 + r] = nr_ + S.ai_ptr[r];
    }
    const int o = blockIdx.x * blockDim.x + tid;
    bool act;
    int px = 0;
    if (FILL) {
        act = rec ? (o == 0 && !rec->skip) : o < S.N;
        if (act) px = rec ? rec->pid : o;
    } else {
        act = o < P.totals[0];
        if (act) px = P.old_pid[o];
    }
    if (act) {
        multipole_planes_f32(bre + tid, bim + tid, kLrThreads, S.L, (float)S.q[px], (float)(S.pos[3 * (size_t)px] * S.inv_E),
                             (float)(S.pos[3 * (size_t)px + 1] * S.inv_E), (float)(S.pos[3 * (size_t)px + 2] * S.inv_E));
    }
    __syncthreads();
    if (!act) return;
    const float *myre = bre + tid, *myim = bim + tid;
    df32 bg = df_make(0.0f, 0.0f);
    if (!FILL) {
        const df32 xd = df_from_double(S.pos[3 * (size_t)px] * S.inv_E),
                   yd = df_from_double(S.pos[3 * (size_t)px + 1] * S.inv_E),
                   zd = df_from_double(S.pos[3 * (size_t)px + 2] * S.inv_E);
        bg = lattice_low_dot(df_from_double(S.q[px]), xd, yd, zd, g);
        P.obox[2 * (size_t)o] = make_float4(xd.hi, yd.hi, zd.hi, 0.0f);
        P.obox[2 * (size_t)o + 1] = make_float4(xd.lo, yd.lo, zd.lo, 0.0f);
    }
    float bg32 = 0.0f, bh = 0.0f;
    for (int r = 0; r < NH; ++r) {
        const float xr = myre[r * kLrThreads], xi = myim[r * kLrThreads];
        const float4 gg = g[r];
        if (r >= 6) bg32 = fmaf(xr, gg.x, fmaf(xi, gg.y, bg32));
        float t0 = 0.0f, t1 = 0.0f, u0 = 0.0f, u1 = 0.0f;
        int k = rp[r];
        const int kb = rp[r + 1];
        if (STAGED) {
            for (; k + 1 < kb; k += 2) {
                const float2 e0 = ue[k], e1 = ue[k + 1];
                t0 = fmaf(e0.x, myre[__float_as_int(e0.y)], t0);
                t1 = fmaf(e1.x, myre[__float_as_int(e1.y)], t1);
            }
            if (k < kb) t0 = fmaf(ue[k].x, myre[__float_as_int(ue[k].y)], t0);
        } else {
            for (; k < kb; ++k) t0 = fmaf(__ldg(&S.ar32_val[k]), myre[__ldg(&S.ar_col[k]) * kLrThreads], t0);
        }
        k = rp[NH + 1 + r];
        const int kd = rp[NH + 2 + r];
        if (STAGED) {
            for (; k + 1 < kd; k += 2) {
                const float2 e0 = ue[k], e1 = ue[k + 1];
                u0 = fmaf(e0.x, myim[__float_as_int(e0.y)], u0);
                u1 = fmaf(e1.x, myim[__float_as_int(e1.y)], u1);
            }
            if (k < kd) u0 = fmaf(ue[k].x, myim[__float_as_int(ue[k].y)], u0);
        } else {
            for (; k < kd; ++k)
                u0 = fmaf(__ldg(&S.ai32_val[k - nr_]), myim[__ldg(&S.ai_col[k - nr_]) * kLrThreads], u0);
        }
        const float t = t0 + t1, u = u0 + u1;
        h32[(size_t)r * hstride + (FILL ? px : o)] = make_float2(t, u);
        bh = fmaf(xr, t, fmaf(xi, u, bh));
    }
    if (FILL)
        hself[px] = 0.5 * (double)bh;
    else
        P.co[o] = S.inv_E * (0.5 * (double)bh - (df_to_double(bg) + (double)bg32));
        P.coq[o] = S.inv_E * (0.5 * (double)bh);
}

// The accepted charge's cache entry, with the block's threads over the rows of
// A: the same operations in the same order as k_lr_old_mixed<STAGED, true> does
// for one charge (b column by column, each row's products split over two
// accumulators when STAGED, b.h summed over rows in order).  SMEM: the folded form
// is first copied to shared memory by all threads (coalesced) so that the row sums
// do not wait on scattered global loads.
template <bool STAGED, bool SMEM>
__global__ void k_lr_refresh_one(const Sys S, float2 *h32, const int hstride, double *hself, const AcceptRec *rec)
{
    extern __shared__ float lro_sm[];
    const int NH = S.NH, L = S.L;
    float *bre = lro_sm, *bim = bre + NH, *tt = bim + NH, *uu = tt + NH;
    float *ta = uu + NH, *tb = ta + L * L, *td = tb + L * L;  // recurrence constants (high words)
    float2 *ue = reinterpret_cast<float2 *>(lro_sm + (((size_t)4 * NH + 2 * L * L + L + 1) & ~(size_t)1));  // SMEM
    if (rec->skip) return;
    const int px = rec->pid;
    const int nr_ = S.ar_ptr[NH], ni_ = S.ai_ptr[NH];
    for (int k = threadIdx.x; k < L * L; k += blockDim.x) {
        const int l = k / L, m = k - l * L;
        ta[k] = g_rec_a2[l * KMC_LMAX + m].x;
        tb[k] = g_rec_b2[l * KMC_LMAX + m].x;
    }
    for (int k = threadIdx.x; k < L; k += blockDim.x) td[k] = g_rec_d2[k].x;
    __syncthreads();
    if (threadIdx.x < L) {
        // column m of b = q a(x); the diagonal is carried up from m = 0 with the same
        // roundings as multipole_planes_f32
        const int m = threadIdx.x;
        const float q = (float)S.q[px], x = (float)(S.pos[3 * (size_t)px] * S.inv_E),
                    y = (float)(S.pos[3 * (size_t)px + 1] * S.inv_E), z = (float)(S.pos[3 * (size_t)px + 2] * S.inv_E);
        const float r2 = x * x + y * y + z * z;
        float dre = 1.0f, dim = 0.0f;
        for (int k = 1; k <= m; ++k) {
            const float t = td[k];
            const float nr = t * (dre * x - dim * y), ni = t * (dre * y + dim * x);
            dre = nr;
            dim = ni;
        }
        float pre = 0.0f, pim = 0.0f, cre = dre, cim = dim;
        bre[hidx(m, m)] = q * cre;
        bim[hidx(m, m)] = -q * cim;
        for (int l = m + 1; l < L; ++l) {
            const float a = ta[l * L + m] * z, b = tb[l * L + m] * r2;
            const float nr = a * cre - b * pre, ni = a * cim - b * pim;
            pre = cre;
            pim = cim;
            cre = nr;
            cim = ni;
            bre[hidx(l, m)] = q * cre;
            bim[hidx(l, m)] = -q * cim;
        }
    }
    if (SMEM) {
        for (int k = threadIdx.x; k < nr_; k += blockDim.x) ue[k] = make_float2(S.ar32_val[k], __int_as_float(S.ar_col[k]));
        for (int k = threadIdx.x; k < ni_; k += blockDim.x)
            ue[nr_ + k] = make_float2(S.ai32_val[k], __int_as_float(S.ai_col[k]));
    }
    __syncthreads();
    auto av = [&](const int k) { return SMEM ? ue[k].x : S.ar32_val[k]; };
    auto ac = [&](const int k) { return SMEM ? __float_as_int(ue[k].y) : S.ar_col[k]; };
    auto iv = [&](const int k) { return SMEM ? ue[nr_ + k].x : S.ai32_val[k]; };
    auto ic = [&](const int k) { return SMEM ? __float_as_int(ue[nr_ + k].y) : S.ai_col[k]; };
    for (int r = threadIdx.x; r < NH; r += blockDim.x) {
        float t0 = 0.0f, t1 = 0.0f, u0 = 0.0f, u1 = 0.0f;
        int k = S.ar_ptr[r];
        const int kb = S.ar_ptr[r + 1];
        if (STAGED) {
            for (; k + 1 < kb; k += 2) {
                t0 = fmaf(av(k), bre[ac(k)], t0);
                t1 = fmaf(av(k + 1), bre[ac(k + 1)], t1);
            }
        }
        for (; k < kb; ++k) t0 = fmaf(av(k), bre[ac(k)], t0);
        k = S.ai_ptr[r];
        const int kd = S.ai_ptr[r + 1];
        if (STAGED) {
            for (; k + 1 < kd; k += 2) {
                u0 = fmaf(iv(k), bim[ic(k)], u0);
                u1 = fmaf(iv(k + 1), bim[ic(k + 1)], u1);
            }
        }
        for (; k < kd; ++k) u0 = fmaf(iv(k), bim[ic(k)], u0);
        const float t = t0 + t1, u = u0 + u1;
        tt[r] = t;
        uu[r] = u;
        h32[(size_t)r * hstride + px] = make_float2(t, u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float bh = 0.0f;
        for (int r = 0; r < NH; ++r) bh = fmaf(bre[r], tt[r], fmaf(bim[r], uu[r], bh));
        hself[px] = 0.5 * (double)bh;
    }
}


// The per-charge lattice cache h = A b, b = q a(x), and b.h / 2 with the operator
// applied in FP64 (the mixed mode with FP64 accept contributions), stored in the box
// units the mixed lattice kernels read: h_box[r] = E^(l_r + 1) h[r] rounded to FP32
// pairs (re, im), hself = E b.h / 2.  One warp per charge: the multipole columns over
// the lanes into shared memory (multipole_warp_add), then the rows of A over the
// lanes.  rec: the accepted charge only (one warp); otherwise every charge.
constexpr int kLf64Warps = 4;
__global__ void __launch_bounds__(kLf64Warps * 32) k_lr_fill64(const Sys S, float2 *h32, const int hstride,
                                                               double *hself, const AcceptRec *rec)
{
    extern __shared__ double2 lf64[];  // [warps][NH]
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int o = blockIdx.x * kLf64Warps + wid;
    int px;
    if (rec) {
        if (o != 0 || rec->skip) return;
        px = rec->pid;
    } else {
        if (o >= S.N) return;
        px = o;
    }
    const int NH = S.NH;
    double2 *b = lf64 + (size_t)wid * NH;
    multipole_warp_add(b, S.L, S.q[px], S.pos[3 * (size_t)px], S.pos[3 * (size_t)px + 1],
                       S.pos[3 * (size_t)px + 2], true);
    double bh = 0.0;
    for (int r = lane; r < NH; r += 32) {
        double t0 = 0.0, t1 = 0.0, u0 = 0.0, u1 = 0.0;
        int k = S.ar_ptr[r];
        const int kb = S.ar_ptr[r + 1];
        for (; k + 1 < kb; k += 2) {
            t0 = fma(S.ar_val[k], b[S.ar_col[k]].x, t0);
            t1 = fma(S.ar_val[k + 1], b[S.ar_col[k + 1]].x, t1);
        }
        if (k < kb) t0 = fma(S.ar_val[k], b[S.ar_col[k]].x, t0);
        k = S.ai_ptr[r];
        const int kd = S.ai_ptr[r + 1];
        for (; k + 1 < kd; k += 2) {
            u0 = fma(S.ai_val[k], b[S.ai_col[k]].y, u0);
            u1 = fma(S.ai_val[k + 1], b[S.ai_col[k + 1]].y, u1);
        }
        if (k < kd) u0 = fma(S.ai_val[k], b[S.ai_col[k]].y, u0);
        const double t = t0 + t1, u = u0 + u1, e = S.escale[r];
        h32[(size_t)r * hstride + px] = make_float2((float)(t * e), (float)(u * e));
        bh = fma(b[r].x, t, fma(b[r].y, u, bh));
    }
    bh = warp_sum(bh);
    if (lane == 0) hself[px] = 0.5 * S.E * bh;
}

// The accepted charge's FP64 cache entry on one block: warp 0 forms b = q a(x) (lanes
// over the m columns) in shared memory, then every thread takes rows of A (one row per
// thread; a 78-row form fits one pass of kLr1Threads), and b.h is summed by the block
// in a fixed order.  The same operations per row as k_lr_fill64, whose single warp
// walked the rows in turn.
constexpr int kLr1Threads = 256;
__global__ void __launch_bounds__(kLr1Threads) k_lr_refresh64(const Sys S, float2 *h32, const int hstride,
                                                            double *hself, const AcceptRec *rec)
{
    extern __shared__ double2 lr1[];  // b [NH], then the rows' b.h terms [kLr1Threads]
    if (rec->skip) return;
    const int px = rec->pid, NH = S.NH;
    double2 *b = lr1;
    double *part = reinterpret_cast<double *>(b + NH);
    if (threadIdx.x < 32)
        multipole_warp_add(b, S.L, S.q[px], S.pos[3 * (size_t)px], S.pos[3 * (size_t)px + 1],
                           S.pos[3 * (size_t)px + 2], true);
    __syncthreads();
    double bh = 0.0;
    for (int r = threadIdx.x; r < NH; r += blockDim.x) {
        double t0 = 0.0, t1 = 0.0, u0 = 0.0, u1 = 0.0;
        int k = S.ar_ptr[r];
        const int kb = S.ar_ptr[r + 1];
        for (; k + 1 < kb; k += 2) {
            t0 = fma(S.ar_val[k], b[S.ar_col[k]].x, t0);
            t1 = fma(S.ar_val[k + 1], b[S.ar_col[k + 1]].x, t1);
        }
        if (k < kb) t0 = fma(S.ar_val[k], b[S.ar_col[k]].x, t0);
        k = S.ai_ptr[r];
        const int kd = S.ai_ptr[r + 1];
        for (; k + 1 < kd; k += 2) {
            u0 = fma(S.ai_val[k], b[S.ai_col[k]].y, u0);
            u1 = fma(S.ai_val[k + 1], b[S.ai_col[k + 1]].y, u1);
        }
        if (k < kd) u0 = fma(S.ai_val[k], b[S.ai_col[k]].y, u0);
        const double t = t0 + t1, u = u0 + u1, e = S.escale[r];
        h32[(size_t)r * hstride + px] = make_float2((float)(t * e), (float)(u * e));
        bh = fma(b[r].x, t, fma(b[r].y, u, bh));
    }
    part[threadIdx.x] = bh;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) part[threadIdx.x] += part[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) hself[px] = 0.5 * S.E * part[0];
}

// Fused mixed lattice term: a block takes kLfMovers moving charges (one per lane)
// and kLfWarps warps.  (1) b = q_o a(x_o) into shared planes, columns m split over
// the warps; (2) h = A b and the old-side constant co = b.h / 2 - b.g, rows split
// over the warps, with A staged in shared memory; (3) every proposal of these
// charges: a = q_n a(x_n), a.(g - h) + q_n^2 F(x_n) + co.  h never leaves shared memory.
constexpr int kLfMovers = 32;
constexpr int kLfWarps = 4;

size_t lr_fused_smem(const int NH, const size_t nnz, const bool staged)
{
    return (size_t)NH * sizeof(float4) + 4 * (size_t)NH * kLfMovers * sizeof(float) +
           (staged ? nnz * sizeof(float2) : 0) + 2 * (size_t)(NH + 1) * sizeof(int) +
           (size_t)kLfWarps * kLfMovers * 3 * sizeof(float) + kLfMovers * sizeof(double);
}

template <bool STAGED>
__global__ void __launch_bounds__(kLfMovers *kLfWarps) k_lr_fused_mixed(const Sys S, Props P)
{
    extern __shared__ float4 lfsm[];
    const int NH = S.NH, L = S.L;
    float4 *g = lfsm;                                          // [NH]
    float *bre = reinterpret_cast<float *>(g + NH);            // [NH][kLfMovers]
    float *bim = bre + (size_t)NH * kLfMovers;
    float *hre = bim + (size_t)NH * kLfMovers;
    float *him = hre + (size_t)NH * kLfMovers;
    const int nr_ = S.ar_ptr[NH], ni_ = S.ai_ptr[NH];
    float2 *ue = reinterpret_cast<float2 *>(him + (size_t)NH * kLfMovers);
    int *rp = reinterpret_cast<int *>(ue + (STAGED ? nr_ + ni_ : 0));   // [2][NH + 1]
    float *red = reinterpret_cast<float *>(rp + 2 * (NH + 1));          // [3][kLfWarps][kLfMovers]
    double *co_s = reinterpret_cast<double *>(red + 3 * kLfWarps * kLfMovers);  // [kLfMovers]
    const int tid = threadIdx.x, lane = tid % kLfMovers, w = tid / kLfMovers;
    const int nthr = kLfMovers * kLfWarps;
    for (int r = tid; r < NH; r += nthr) {
        const df32 gr = df_from_double(P.g[r].x * S.escale[r]), gi = df_from_double(P.g[r].y * S.escale[r]);
        g[r] = make_float4(gr.hi, gi.hi, gr.lo, gi.lo);
    }
    if (STAGED) {
        for (int k = tid; k < nr_; k += nthr)
            ue[k] = make_float2(S.ar32_val[k], __int_as_float(S.ar_col[k] * kLfMovers));
        for (int k = tid; k < ni_; k += nthr)
            ue[nr_ + k] = make_float2(S.ai32_val[k], __int_as_float(S.ai_col[k] * kLfMovers));
    }
    for (int r = tid; r <= NH; r += nthr) {
        rp[r] = S.ar_ptr[r];
        rp[NH + 1 + r] = nr_ + S.ai_ptr[r];
    }
    const int nmov = P.totals[0];
    const int o0 = blockIdx.x * kLfMovers;
    const int o = o0 + lane;
    const bool mv = o < nmov;
    // (1) multipole of the old positions, columns m = w, w + kLfWarps, ...
    if (mv) {
        const int px = P.old_pid[o];
        const float q = (float)S.q[px], x = (float)(S.pos[3 * (size_t)px] * S.inv_E),
                    y = (float)(S.pos[3 * (size_t)px + 1] * S.inv_E), z = (float)(S.pos[3 * (size_t)px + 2] * S.inv_E);
        const float r2 = x * x + y * y + z * z;
        float dre = 1.0f, dim = 0.0f;
        for (int m = 0; m < L; ++m) {
            if (m > 0) {
                const float t = c_rec_d2[m].x;
                const float nr = t * (dre * x - dim * y), ni = t * (dre * y + dim * x);
                dre = nr;
                dim = ni;
            }
            if (m % kLfWarps != w) continue;
            float pre = 0.0f, pim = 0.0f, cre = dre, cim = dim;
            bre[hidx(m, m) * kLfMovers + lane] = q * cre;
            bim[hidx(m, m) * kLfMovers + lane] = -q * cim;
            for (int l = m + 1; l < L; ++l) {
                const float a = c_rec_a2[l * KMC_LMAX + m].x * z, b = c_rec_b2[l * KMC_LMAX + m].x * r2;
                const float nr = a * cre - b * pre, ni = a * cim - b * pim;
                pre = cre;
                pim = cim;
                cre = nr;
                cim = ni;
                bre[hidx(l, m) * kLfMovers + lane] = q * cre;
                bim[hidx(l, m) * kLfMovers + lane] = -q * cim;
            }
        }
    }
    __syncthreads();
    // (2) h = A b, rows r = w, w + kLfWarps, ...
    {
        const float *myre = bre + lane, *myim = bim + lane;
        float bh = 0.0f, bg32 = 0.0f, bgl = 0.0f;
        df32 bg = df_make(0.0f, 0.0f);
        if (w == 0 && mv) {
            const int px = P.old_pid[o];
            bg = lattice_low_dot(df_from_double(S.q[px]), df_from_double(S.pos[3 * (size_t)px] * S.inv_E),
                                 df_from_double(S.pos[3 * (size_t)px + 1] * S.inv_E),
                                 df_from_double(S.pos[3 * (size_t)px + 2] * S.inv_E), g);
        }
        for (int r = w; r < NH; r += kLfWarps) {
            float t0 = 0.0f, t1 = 0.0f, u0 = 0.0f, u1 = 0.0f;
            int k = rp[r];
            const int kb = rp[r + 1];
            if (STAGED) {
                for (; k + 1 < kb; k += 2) {
                    const float2 e0 = ue[k], e1 = ue[k + 1];
                    t0 = fmaf(e0.x, myre[__float_as_int(e0.y)], t0);
                    t1 = fmaf(e1.x, myre[__float_as_int(e1.y)], t1);
                }
                if (k < kb) t0 = fmaf(ue[k].x, myre[__float_as_int(ue[k].y)], t0);
            } else {
                for (; k < kb; ++k) t0 = fmaf(__ldg(&S.ar32_val[k]), myre[__ldg(&S.ar_col[k]) * kLfMovers], t0);
            }
            k = rp[NH + 1 + r];
            const int kd = rp[NH + 2 + r];
            if (STAGED) {
                for (; k + 1 < kd; k += 2) {
                    const float2 e0 = ue[k], e1 = ue[k + 1];
                    u0 = fmaf(e0.x, myim[__float_as_int(e0.y)], u0);
                    u1 = fmaf(e1.x, myim[__float_as_int(e1.y)], u1);
                }
                if (k < kd) u0 = fmaf(ue[k].x, myim[__float_as_int(ue[k].y)], u0);
            } else {
                for (; k < kd; ++k)
                    u0 = fmaf(__ldg(&S.ai32_val[k - nr_]), myim[__ldg(&S.ai_col[k - nr_]) * kLfMovers], u0);
            }
            const float t = t0 + t1, u = u0 + u1;
            hre[r * kLfMovers + lane] = t;
            him[r * kLfMovers + lane] = u;
            const float xr = myre[r * kLfMovers], xi = myim[r * kLfMovers];
            bh = fmaf(xr, t, fmaf(xi, u, bh));
            const float4 gg = g[r];
            if (r >= 6) bg32 = fmaf(xr, gg.x, fmaf(xi, gg.y, bg32));
        }
        bgl = bg.lo + bg32;
        red[(0 * kLfWarps + w) * kLfMovers + lane] = bh;
        red[(1 * kLfWarps + w) * kLfMovers + lane] = bg.hi;
        red[(2 * kLfWarps + w) * kLfMovers + lane] = bgl;
    }
    __syncthreads();
    if (w == 0) {
        double bh = 0.0, bgd = 0.0;
        for (int v = 0; v < kLfWarps; ++v) {
            bh += (double)red[(0 * kLfWarps + v) * kLfMovers + lane];
            bgd += (double)red[(1 * kLfWarps + v) * kLfMovers + lane] + (double)red[(2 * kLfWarps + v) * kLfMovers + lane];
        }
        co_s[lane] = S.inv_E * (0.5 * bh - bgd);
    }
    __syncthreads();
    // (3) the proposals of these moving charges
    if (o0 >= nmov) return;
    const int olast = min(o0 + kLfMovers, nmov);
    const int p_begin = P.es[o0], p_end = P.es[olast];
    for (int p = p_begin + tid; p < p_end; p += nthr) {
        const int ow = P.owner[p];
        const int loc = ow - o0;
        const df32 qd = df_from_double(P.pq[p]), xd = df_from_double(P.ppos[3 * (size_t)p] * S.inv_E),
                   yd = df_from_double(P.ppos[3 * (size_t)p + 1] * S.inv_E),
                   zd = df_from_double(P.ppos[3 * (size_t)p + 2] * S.inv_E);
        const float q = qd.hi, x = xd.hi, y = yd.hi, z = zd.hi;
        const float r2 = x * x + y * y + z * z;
        const df32 lg = lattice_low_dot(qd, xd, yd, zd, g);
        float lg32 = 0.0f, lh = 0.0f;
        float dre = 1.0f, dim = 0.0f;
        for (int m = 0; m < L; ++m) {
            if (m > 0) {
                const float t = c_rec_d2[m].x;
                const float nr = t * (dre * x - dim * y), ni = t * (dre * y + dim * x);
                dre = nr;
                dim = ni;
            }
            float pre = 0.0f, pim = 0.0f, cre = dre, cim = dim;
            for (int l = m; l < L; ++l) {
                if (l > m) {
                    const float a = c_rec_a2[l * KMC_LMAX + m].x * z, b = c_rec_b2[l * KMC_LMAX + m].x * r2;
                    const float nr = a * cre - b * pre, ni = a * cim - b * pim;
                    pre = cre;
                    pim = cim;
                    cre = nr;
                    cim = ni;
                }
                const int hh = hidx(l, m);
                const float ar = q * cre, ai = -q * cim;
                const float4 gg = g[hh];
                if (l > 2) lg32 = fmaf(ar, gg.x, fmaf(ai, gg.y, lg32));
                lh = fmaf(ar, hre[hh * kLfMovers + loc], fmaf(ai, him[hh * kLfMovers + loc], lh));
            }
        }
        const float F = lattice_self<float>(S.fprog_i, S.fprog_f, x, y, z);
        P.elr[p] = S.inv_E * ((df_to_double(lg) + (double)lg32) - (double)lh + (double)(q * q * F)) + co_s[loc];
    }
}

// per proposal: a = q_n a(x_n) generated column by column, dotted with g (l <= 2 in
// double-FP32) and with the owner's h; plus q_n^2 F(x_n); plus the old-side constant
constexpr int kLrNewThreads = 128;  // default proposals (moving charges) per block
constexpr int kLrMaxThreads = 256;  // one compiled kernel for every block size the tuning offers

// CACHED: h is the per-charge cache h32[r][pid] instead of h32[r][owner].
// LT > 0: the order is the compile-time LT (column loops unrolled, table offsets constant)
// FS: F(x) from the L = 12 cubic-lattice evaluator with fs's reals (else the interpreter)
template <bool CACHED, int LT = 0, bool FS = false>
__global__ void __launch_bounds__(kLrMaxThreads) k_lr_new_mixed(const Sys S, Props P, const float2 *h32,
                                                                const int hstride, const __grid_constant__ FSelf12 fs)
{
    static_assert(!FS || LT == 12, "the specialised F evaluator is the L = 12 shape");
    extern __shared__ float4 lrg_sm[];
    const int NH = S.NH, L = LT > 0 ? LT : S.L;
    for (int r = threadIdx.x; r < NH; r += blockDim.x) {
        const df32 gr = df_from_double(P.g[r].x * S.escale[r]), gi = df_from_double(P.g[r].y * S.escale[r]);
        lrg_sm[r] = make_float4(gr.hi, gi.hi, gr.lo, gi.lo);
    }
    __syncthreads();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.totals[1]) return;
    const int o = P.owner[p];
    const df32 qd = df_from_double(P.pq[p]), xd = df_from_double(P.ppos[3 * (size_t)p] * S.inv_E),
               yd = df_from_double(P.ppos[3 * (size_t)p + 1] * S.inv_E),
               zd = df_from_double(P.ppos[3 * (size_t)p + 2] * S.inv_E);
    const float q = qd.hi, x = xd.hi, y = yd.hi, z = zd.hi;
    const float r2 = x * x + y * y + z * z;
    const int po = P.old_pid[o];
    const float2 *hp = h32 + (CACHED ? po : o);
    // The linear lattice term q' a(x_new).g - q a(x_old).g is two large values whose
    // difference is small; when the charge keeps its value (q' = q) it is formed as
    // q (a(x_new) - a(x_old)).g, with the difference D of the harmonics carried through
    // the recurrences from the exact coordinate differences (no cancellation): per step
    // D_l = a (dz P_{l-1} + z_o D_{l-1}) - b (dr2 P_{l-2} + r2_o D_{l-2}), P the new
    // point's harmonics, and on the diagonal D_m = d_m ((dx + i dy) P_{m-1} + (x_o + i y_o) D_{m-1}).
    const double qo = S.q[po];
    const bool same = P.pq[p] == qo;
    const float4 ohv = P.obox[2 * (size_t)o], olv = P.obox[2 * (size_t)o + 1];
    const df32 xo = df_make(ohv.x, olv.x), yo = df_make(ohv.y, olv.y), zo = df_make(ohv.z, olv.z);
    df32 lg = lattice_low_dot(qd, xd, yd, zd, lrg_sm);
    if (same) lg = df_sub(lg, lattice_low_dot(qd, xo, yo, zo, lrg_sm));
    const df32 ddx = df_sub(xd, xo), ddy = df_sub(yd, yo), ddz = df_sub(zd, zo);
    const float dx = ddx.hi + ddx.lo, dy = ddy.hi + ddy.lo, dz = ddz.hi + ddz.lo;
    const float xo1 = ohv.x + olv.x, yo1 = ohv.y + olv.y, zo1 = ohv.z + olv.z;
    const float r2o = xo1 * xo1 + yo1 * yo1 + zo1 * zo1;
    const float dr2 = dx * (x + xo1) + dy * (y + yo1) + dz * (z + zo1);
    float lg32 = 0.0f, lh = 0.0f;
    float dre = 1.0f, dim = 0.0f, ere = 0.0f, eim = 0.0f;  // diagonal P_m^m and D_m^m
#pragma unroll
    for (int m = 0; m < L; ++m) {
        if (m > 0) {
            const float t = c_rec_d2[m].x;
            const float ne = t * ((dx * dre - dy * dim) + (xo1 * ere - yo1 * eim));
            const float nf = t * ((dx * dim + dy * dre) + (xo1 * eim + yo1 * ere));
            const float nr = t * (dre * x - dim * y), ni = t * (dre * y + dim * x);
            dre = nr;
            dim = ni;
            ere = ne;
            eim = nf;
        }
        float pre = 0.0f, pim = 0.0f, cre = dre, cim = dim;
        float qre = 0.0f, qim = 0.0f, fre = ere, fim = eim;  // D_{l-2}, D_{l-1}
#pragma unroll
        for (int l = m; l < L; ++l) {
            if (l > m) {
                const float ca = c_rec_a2[l * KMC_LMAX + m].x, cb = c_rec_b2[l * KMC_LMAX + m].x;
                const float a = ca * z, b = cb * r2;
                const float ner = ca * (dz * cre + zo1 * fre) - cb * (dr2 * pre + r2o * qre);
                const float nei = ca * (dz * cim + zo1 * fim) - cb * (dr2 * pim + r2o * qim);
                const float nr = a * cre - b * pre, ni = a * cim - b * pim;
                qre = fre;
                qim = fim;
                fre = ner;
                fim = nei;
                pre = cre;
                pim = cim;
                cre = nr;
                cim = ni;
            }
            const int hh = hidx(l, m);
            const float ar = q * cre, ai = -q * cim;
            const float4 gg = lrg_sm[hh];
            if (l > 2) {
                if (same)
                    lg32 = fmaf(q * fre, gg.x, fmaf(-q * fim, gg.y, lg32));
                else
                    lg32 = fmaf(ar, gg.x, fmaf(ai, gg.y, lg32));
            }
            const float2 hv = hp[(size_t)hh * hstride];
            lh = fmaf(ar, hv.x, fmaf(ai, hv.y, lh));
        }
    }
    const float F = FS ? lattice_self_c12(fs.v, x, y, z) : lattice_self<float>(S.fprog_i, S.fprog_f, x, y, z);
    // the moved pair's self term is the near field's (self_term_grid): formed from the
    // same grid coordinates as the near-field pair of the new position with the charge's
    // old slot, their roundings cancel, which matters for short moves (1/r large)
    P.elr[p] = S.inv_E * ((df_to_double(lg) + (double)lg32) - (double)lh + (double)(q * q * F)) +
               (same ? P.coq[o] : P.co[o]);
}

// Old-side constant from the per-charge cache: co = (b.h / 2 - b.g) / E with
// b = q_o a(x_o) generated column by column and dotted with g (l <= 2 in
// double-FP32, as in k_lr_old_mixed).
template <int LT = 0>
__global__ void __launch_bounds__(kLrMaxThreads) k_lr_co_mixed(const Sys S, Props P, const double *hself)
{
    extern __shared__ float4 lcg_sm[];
    const int NH = S.NH, L = LT > 0 ? LT : S.L;
    for (int r = threadIdx.x; r < NH; r += blockDim.x) {
        const df32 gr = df_from_double(P.g[r].x * S.escale[r]), gi = df_from_double(P.g[r].y * S.escale[r]);
        lcg_sm[r] = make_float4(gr.hi, gi.hi, gr.lo, gi.lo);
    }
    __syncthreads();
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= P.totals[0]) return;
    const int px = P.old_pid[o];
    const df32 qd = df_from_double(S.q[px]), xd = df_from_double(S.pos[3 * (size_t)px] * S.inv_E),
               yd = df_from_double(S.pos[3 * (size_t)px + 1] * S.inv_E),
               zd = df_from_double(S.pos[3 * (size_t)px + 2] * S.inv_E);
    const float q = qd.hi, x = xd.hi, y = yd.hi, z = zd.hi;
    const float r2 = x * x + y * y + z * z;
    const df32 bg = lattice_low_dot(qd, xd, yd, zd, lcg_sm);
    P.obox[2 * (size_t)o] = make_float4(xd.hi, yd.hi, zd.hi, 0.0f);
    P.obox[2 * (size_t)o + 1] = make_float4(xd.lo, yd.lo, zd.lo, 0.0f);
    float bg32 = 0.0f;
    float dre = 1.0f, dim = 0.0f;
#pragma unroll
    for (int m = 0; m < L; ++m) {
        if (m > 0) {
            const float t = c_rec_d2[m].x;
            const float nr = t * (dre * x - dim * y), ni = t * (dre * y + dim * x);
            dre = nr;
            dim = ni;
        }
        float pre = 0.0f, pim = 0.0f, cre = dre, cim = dim;
#pragma unroll
        for (int l = m; l < L; ++l) {
            if (l > m) {
                const float a = c_rec_a2[l * KMC_LMAX + m].x * z, b = c_rec_b2[l * KMC_LMAX + m].x * r2;
                const float nr = a * cre - b * pre, ni = a * cim - b * pim;
                pre = cre;
                pim = cim;
                cre = nr;
                cim = ni;
            }
            const float br = q * cre, bi = -q * cim;
            const float4 gg = lcg_sm[hidx(l, m)];
            if (l > 2) bg32 = fmaf(br, gg.x, fmaf(bi, gg.y, bg32));
        }
    }
    P.co[o] = S.inv_E * (hself[px] - (df_to_double(bg) + (double)bg32));
    P.coq[o] = S.inv_E * hself[px];
}
