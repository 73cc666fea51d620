// Part of the kmc_gb300.cu translation unit (included there, in order, inside its
// anonymous namespace unless it says otherwise): the FMM initial solve (P2M, M2M, M2L, L2L), the initial multipole and energy, the FMA-rate diagnostic.
#pragma once
// ---------------------------------------------------------------------------
// FMM initial solve (replaces ppmd PyFMM, kmc_fmm.py:463-476, 956-959):
// P2M at the finest level, M2M up, M2L over the interaction lists (children of
// the parent's neighbours that are not neighbours, periodic images limited to
// the 3x3x3 block for '27' and pbc), L2L down.  Expansions are folded (m >= 0);
// the translations follow the regular addition theorem
//   Rg_l^m(a + b) = sum_{j,k} C(l,m,j,k) Rg_j^k(a) Rg_{l-j}^{m-k}(b)
//   M2M: M'_nm = sum_jk C(n,m,j,k) M_jk conj Rg_{n-j}^{m-k}(c_old - c_new)
//   L2L: L'_jk = sum_nm C(n,m,j,k) L_nm Rg_{n-j}^{m-k}(c_new - c_old)
//   M2L: L_jk  = sum_nm A(j,k,n,m) M_nm Ir_{j+n}^{k-m}(c_src - c_tgt)
// with Rg^{-m} = conj Rg^m and Ir^{-m} = conj Ir^m.
// ---------------------------------------------------------------------------
struct FmmLevel {
    int n;          // cells per side
    double w;       // cell width
    double2 *M;     // [n^3][NH]
    double2 *Lx;    // [n^3][NH]
};

__device__ __forceinline__ double2 fold_get(const double2 *X, const int l, const int m)
{
    const double2 v = X[hidx(l, m < 0 ? -m : m)];
    return m < 0 ? make_double2(v.x, -v.y) : v;
}

__device__ __forceinline__ double lvl_centre(const double E, const double w, const int c)
{
    return (-0.5 * E + 0.5 * w) + c * w;
}

// regular solid harmonics Rg_l^m(x), m >= 0, l < LL into out (folded), computed by thread 0..LL-1 (column m)
__device__ void rg_columns(double2 *out, const int LL, const double x, const double y, const double z)
{
    const int m = threadIdx.x;
    if (m >= LL) return;
    const double r2 = x * x + y * y + z * z;
    double dre = 1.0, dim = 0.0;
    for (int k = 1; k <= m; ++k) {
        const double t = c_rec_d[k];
        const double nre = t * (dre * x - dim * y);
        const double nim = t * (dre * y + dim * x);
        dre = nre;
        dim = nim;
    }
    double pre = 0.0, pim = 0.0, cre = dre, cim = dim;
    out[hidx(m, m)] = make_double2(cre, cim);
    for (int l = m + 1; l < LL; ++l) {
        const double az = c_rec_a[l * KMC_LMAX + m] * z;
        const double br = c_rec_b[l * KMC_LMAX + m] * r2;
        const double nre = az * cre - br * pre;
        const double nim = az * cim - br * pim;
        pre = cre;
        pim = cim;
        cre = nre;
        cim = nim;
        out[hidx(l, m)] = make_double2(cre, cim);
    }
}

// irregular solid harmonics Ir_l^m(x), m >= 0, l < LL (folded), thread m; needs
// recurrence tables up to LL <= 2*KMC_LMAX-1 via the analytic coefficients
__device__ void ir_columns(double2 *out, const int LL, const double x, const double y, const double z)
{
    for (int m = threadIdx.x; m < LL; m += blockDim.x) {
        const double r2 = x * x + y * y + z * z;
        const double ri2 = 1.0 / r2;
        const double ri = sqrt(ri2);
        const double wre = x * ri2, wim = -y * ri2, zr = z * ri2;
        double ire = ri, iim = 0.0;
        for (int k = 1; k <= m; ++k) {
            const double t = -sqrt((2.0 * k - 1.0) / (2.0 * k));
            const double nre = t * (ire * wre - iim * wim);
            const double nim = t * (ire * wim + iim * wre);
            ire = nre;
            iim = nim;
        }
        double pre = 0.0, pim = 0.0;
        out[hidx(m, m)] = make_double2(ire, iim);
        for (int l = m + 1; l < LL; ++l) {
            const double sq = sqrt((double)(l * l - m * m));
            const double az = (2.0 * l - 1.0) / sq * zr;
            const double br = sqrt((double)((l - 1) * (l - 1) - m * m)) / sq * ri2;
            const double nre = az * ire - br * pre;
            const double nim = az * iim - br * pim;
            pre = ire;
            pim = iim;
            ire = nre;
            iim = nim;
            out[hidx(l, m)] = make_double2(ire, iim);
        }
    }
}

// P2M at the finest level: block per cell, thread m accumulates column m
__global__ void k_fmm_p2m(const Sys S, double2 *M)
{
    const int c = blockIdx.x, m = threadIdx.x;
    if (m >= S.L) return;
    const int cx = c % S.n, cy = (c / S.n) % S.n, cz = c / (S.n * S.n);
    const double ccx = cell_centre(S, cx), ccy = cell_centre(S, cy), ccz = cell_centre(S, cz);
    double acc_re[KMC_LMAX], acc_im[KMC_LMAX];
    for (int l = 0; l < KMC_LMAX; ++l) acc_re[l] = acc_im[l] = 0.0;
    const int k = S.cnt[c];
    for (int i = 0; i < k; ++i) {
        const double4_32a v = S.store[(size_t)c * S.cap + i];
        const double x = v.x - ccx, y = v.y - ccy, z = v.z - ccz, q = v.w;
        const double r2 = x * x + y * y + z * z;
        double dre = 1.0, dim = 0.0;
        for (int kk = 1; kk <= m; ++kk) {
            const double t = c_rec_d[kk];
            const double nre = t * (dre * x - dim * y);
            const double nim = t * (dre * y + dim * x);
            dre = nre;
            dim = nim;
        }
        double pre = 0.0, pim = 0.0, cre = dre, cim = dim;
        acc_re[m] += q * cre;
        acc_im[m] -= q * cim;
        for (int l = m + 1; l < S.L; ++l) {
            const double az = c_rec_a[l * KMC_LMAX + m] * z;
            const double br = c_rec_b[l * KMC_LMAX + m] * r2;
            const double nre = az * cre - br * pre;
            const double nim = az * cim - br * pim;
            pre = cre;
            pim = cim;
            cre = nre;
            cim = nim;
            acc_re[l] += q * cre;
            acc_im[l] -= q * cim;
        }
    }
    for (int l = m; l < S.L; ++l) M[(size_t)c * S.NH + hidx(l, m)] = make_double2(acc_re[l], acc_im[l]);
}

// M2M: block per parent cell at level (child level n_c = 2 n_p); thread per output (n,m)
__global__ void k_fmm_m2m(const Sys S, const FmmLevel par, const FmmLevel chl, const double *Ctab)
{
    extern __shared__ double2 m2msm[];
    const int NH = S.NH, L = S.L, L2 = L * L;
    double2 *Mc = m2msm;           // [8][NH]
    double2 *Rt = m2msm + 8 * NH;    // [8][NH] conj-less Rg(c_child - c_parent) per child
    const int p = blockIdx.x, np = par.n, nc = chl.n;
    const int px = p % np, py = (p / np) % np, pz = p / (np * np);
    for (int k = threadIdx.x; k < 8 * NH; k += blockDim.x) {
        const int ch = k / NH, h = k % NH;
        const int cx = 2 * px + (ch & 1), cy = 2 * py + ((ch >> 1) & 1), cz = 2 * pz + (ch >> 2);
        Mc[k] = chl.M[(size_t)(cx + nc * (cy + nc * cz)) * NH + h];
    }
    for (int ch = 0; ch < 8; ++ch) {
        const int cx = 2 * px + (ch & 1), cy = 2 * py + ((ch >> 1) & 1), cz = 2 * pz + (ch >> 2);
        const double tx = lvl_centre(S.E, chl.w, cx) - lvl_centre(S.E, par.w, px);
        const double ty = lvl_centre(S.E, chl.w, cy) - lvl_centre(S.E, par.w, py);
        const double tz = lvl_centre(S.E, chl.w, cz) - lvl_centre(S.E, par.w, pz);
        rg_columns(Rt + ch * NH, L, tx, ty, tz);
    }
    __syncthreads();
    for (int o = threadIdx.x; o < NH; o += blockDim.x) {
        int n = 0;
        while (hidx(n + 1, 0) <= o) ++n;
        const int m = o - hidx(n, 0);
        double re = 0.0, im = 0.0;
        for (int j = 0; j <= n; ++j)
            for (int k = -j; k <= j; ++k) {
                const int mk = m - k;
                if (mk < -(n - j) || mk > (n - j)) continue;
                const double cf = Ctab[(size_t)(n * n + n + m) * L2 + (j * j + j + k)];
                for (int ch = 0; ch < 8; ++ch) {
                    const double2 mj = fold_get(Mc + ch * NH, j, k);
                    double2 rr = fold_get(Rt + ch * NH, n - j, mk);
                    rr.y = -rr.y;  // conj
                    re += cf * (mj.x * rr.x - mj.y * rr.y);
                    im += cf * (mj.x * rr.y + mj.y * rr.x);
                }
            }
        par.M[(size_t)p * NH + o] = make_double2(re, im);
    }
}

// M2L: block per target cell at a level; loop over the interaction list
__global__ void k_fmm_m2l(const Sys S, const FmmLevel lv, const double *Atab)
{
    extern __shared__ double2 lsm2[];
    const int NH = S.NH, L = S.L;
    const int LL = 2 * L - 1, NHI = LL * (LL + 1) / 2;
    double2 *Ir = lsm2;          // [NHI]
    double2 *Ms = lsm2 + NHI;    // [NH]
    const int c = blockIdx.x, n = lv.n;
    const int cx = c % n, cy = (c / n) % n, cz = c / (n * n);
    const int px = cx >> 1, py = cy >> 1, pz = cz >> 1;
    double acc_re = 0.0, acc_im = 0.0;
    const int o = threadIdx.x;
    int jo = 0, ko = 0;
    if (o < NH) {
        while (hidx(jo + 1, 0) <= o) ++jo;
        ko = o - hidx(jo, 0);
    }
    for (int it = 0; it < 216; ++it) {
        const int sx = 2 * px - 2 + it % 6, sy = 2 * py - 2 + (it / 6) % 6, sz = 2 * pz - 2 + it / 36;
        if (abs(sx - cx) <= 1 && abs(sy - cy) <= 1 && abs(sz - cz) <= 1) continue;
        int wx = sx, wy = sy, wz = sz;
        double shx = 0.0, shy = 0.0, shz = 0.0;
        bool ok = true;
        if (wx < 0) { wx += n; shx = -S.E; ok = ok && S.periodic; } else if (wx >= n) { wx -= n; shx = S.E; ok = ok && S.periodic; }
        if (wy < 0) { wy += n; shy = -S.E; ok = ok && S.periodic; } else if (wy >= n) { wy -= n; shy = S.E; ok = ok && S.periodic; }
        if (wz < 0) { wz += n; shz = -S.E; ok = ok && S.periodic; } else if (wz >= n) { wz -= n; shz = S.E; ok = ok && S.periodic; }
        if (!ok) continue;
        const int sc = wx + n * (wy + n * wz);
        const double dx = (lvl_centre(S.E, lv.w, wx) + shx) - lvl_centre(S.E, lv.w, cx);
        const double dy = (lvl_centre(S.E, lv.w, wy) + shy) - lvl_centre(S.E, lv.w, cy);
        const double dz = (lvl_centre(S.E, lv.w, wz) + shz) - lvl_centre(S.E, lv.w, cz);
        __syncthreads();
        ir_columns(Ir, LL, dx, dy, dz);
        for (int k = threadIdx.x; k < NH; k += blockDim.x) Ms[k] = lv.M[(size_t)sc * NH + k];
        __syncthreads();
        if (o < NH) {
            for (int nn = 0; nn < L; ++nn)
                for (int m = -nn; m <= nn; ++m) {
                    const double a = Atab[(size_t)(nn * nn + nn + m) * NH + o];
                    if (a == 0.0) continue;
                    const double2 mm = fold_get(Ms, nn, m);
                    const double2 ii = fold_get(Ir, jo + nn, ko - m);
                    acc_re += a * (mm.x * ii.x - mm.y * ii.y);
                    acc_im += a * (mm.x * ii.y + mm.y * ii.x);
                }
        }
    }
    if (o < NH) {
        double2 *dst = lv.Lx + (size_t)c * NH + o;
        dst->x += acc_re;
        dst->y += acc_im;
    }
}

// L2L: block per child cell; thread per output (j,k)
__global__ void k_fmm_l2l(const Sys S, const FmmLevel par, const FmmLevel chl, const double *Ctab)
{
    extern __shared__ double2 l2sm[];
    const int NH = S.NH, L = S.L, L2 = L * L;
    double2 *Lp = l2sm;        // [NH]
    double2 *Ru = l2sm + NH;   // [NH]
    const int c = blockIdx.x, nc = chl.n, np = par.n;
    const int cx = c % nc, cy = (c / nc) % nc, cz = c / (nc * nc);
    const int px = cx >> 1, py = cy >> 1, pz = cz >> 1;
    const int p = px + np * (py + np * pz);
    for (int k = threadIdx.x; k < NH; k += blockDim.x) Lp[k] = par.Lx[(size_t)p * NH + k];
    rg_columns(Ru, L, lvl_centre(S.E, chl.w, cx) - lvl_centre(S.E, par.w, px),
               lvl_centre(S.E, chl.w, cy) - lvl_centre(S.E, par.w, py),
               lvl_centre(S.E, chl.w, cz) - lvl_centre(S.E, par.w, pz));
    __syncthreads();
    for (int o = threadIdx.x; o < NH; o += blockDim.x) {
        int j = 0;
        while (hidx(j + 1, 0) <= o) ++j;
        const int k = o - hidx(j, 0);
        double re = 0.0, im = 0.0;
        for (int nn = j; nn < L; ++nn)
            for (int m = -nn; m <= nn; ++m) {
                const int mk = m - k;
                if (mk < -(nn - j) || mk > (nn - j)) continue;
                const double cf = Ctab[(size_t)(nn * nn + nn + m) * L2 + (j * j + j + k)];
                const double2 lv = fold_get(Lp, nn, m);
                const double2 rr = fold_get(Ru, nn - j, mk);
                re += cf * (lv.x * rr.x - lv.y * rr.y);
                im += cf * (lv.x * rr.y + lv.y * rr.x);
            }
        double2 *dst = chl.Lx + (size_t)c * NH + o;
        dst->x += re;
        dst->y += im;
    }
}

// level-0 multipole of all charges (initial solve, kmc_full_long_range.py:83-118)
__global__ void k_init_mpole(Sys S)
{
    const int m = blockIdx.x;
    __shared__ double red[2][256];
    double acc_re[KMC_LMAX], acc_im[KMC_LMAX];
    for (int l = 0; l < KMC_LMAX; ++l) acc_re[l] = acc_im[l] = 0.0;
    for (int j = threadIdx.x; j < S.N; j += blockDim.x) {
        const double x = S.pos[3 * (size_t)j], y = S.pos[3 * (size_t)j + 1], z = S.pos[3 * (size_t)j + 2];
        const double q = S.q[j];
        const double r2 = x * x + y * y + z * z;
        double dre = 1.0, dim = 0.0;
        for (int k = 1; k <= m; ++k) {
            const double t = c_rec_d[k];
            const double nre = t * (dre * x - dim * y);
            const double nim = t * (dre * y + dim * x);
            dre = nre;
            dim = nim;
        }
        double pre = 0.0, pim = 0.0, cre = dre, cim = dim;
        acc_re[m] += q * cre;
        acc_im[m] += -q * cim;
        for (int l = m + 1; l < S.L; ++l) {
            const double az = c_rec_a[l * KMC_LMAX + m] * z;
            const double br = c_rec_b[l * KMC_LMAX + m] * r2;
            const double nre = az * cre - br * pre;
            const double nim = az * cim - br * pim;
            pre = cre;
            pim = cim;
            cre = nre;
            cim = nim;
            acc_re[l] += q * cre;
            acc_im[l] += -q * cim;
        }
    }
    for (int l = m; l < S.L; ++l) {
        red[0][threadIdx.x] = acc_re[l];
        red[1][threadIdx.x] = acc_im[l];
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) {
                red[0][threadIdx.x] += red[0][threadIdx.x + s];
                red[1][threadIdx.x] += red[1][threadIdx.x + s];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) S.mpole[hidx(l, m)] = make_double2(red[0][0], red[1][0]);
        __syncthreads();
    }
}

// E_LR(M) = 1/2 (ReM^T A_re ReM + ImM^T A_im ImM)

// E0 = 1/2 sum_i U0_i (+ E_LR(M)), deterministic single-block reduction
__global__ void k_init_energy(Sys S, Props P, double *energy)
{
    __shared__ double red[1024];
    double e = 0.0;
    for (int i = threadIdx.x; i < S.N; i += blockDim.x) e += P.u0p[i];
    red[threadIdx.x] = e;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    double tot = 0.5 * red[0];
    __syncthreads();
    if (S.pbc) tot += lr_energy_block(S, red);
    if (threadIdx.x == 0) *energy = S.unit * tot;
}

// Diagnostic: sustained FMA issue rate of the FP64 (or FP32) pipe, 8
// independent chains per thread.  Used only to measure the roofline
// denominator on the running GPU.
template <typename T>
__global__ void k_fma_rate(T *out, const int iters, const T seed)
{
    T a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + (T)(threadIdx.x + k);
    const T b = (T)0.999999, c = (T)1e-7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = a[k] * b + c;
    }
    T t = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) t += a[k];
    if (t == (T)-1) out[0] = t;  // keeps the chains live; never true
}
