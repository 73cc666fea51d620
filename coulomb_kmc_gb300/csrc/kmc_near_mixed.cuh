// Part of the kmc_gb300.cu translation unit (included there, in order, inside its
// anonymous namespace unless it says otherwise): the FP32-pair copies of the state and the mixed-precision near field (grid-split pair terms, packed FP32, one warp per cell).
#pragma once
// ---------------------------------------------------------------------------
// mixed precision copies
// ---------------------------------------------------------------------------
__device__ __forceinline__ void store32_write(const Sys &S, const size_t slot, const int cell, const double x,
                                              const double y, const double z, const double q)
{
    const int cx = cell % S.n, cy = (cell / S.n) % S.n, cz = cell / (S.n * S.n);
    const float2 rx = grid_split((x - cell_centre(S, cx)) * S.inv_w);
    const float2 ry = grid_split((y - cell_centre(S, cy)) * S.inv_w);
    const float2 rz = grid_split((z - cell_centre(S, cz)) * S.inv_w);
    const df32 rq = df_from_double(q);
    S.st_hi[slot] = make_float4(rx.x, ry.x, rz.x, rq.hi);
    S.st_lo[slot] = make_float4(rx.y, ry.y, rz.y, rq.lo);
}

__global__ void k_refresh_store32(const Sys S)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (size_t)S.ncell * S.cap) return;
    const int cell = (int)(k / S.cap), slot = (int)(k % S.cap);
    if (slot >= S.cnt[cell]) return;
    const double4_32a v = S.store[k];
    store32_write(S, k, cell, v.x, v.y, v.z, v.w);
}

__global__ void k_refresh_lexp32(const Sys S)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (size_t)S.ncell * S.NH) return;
    const double2 v = S.lexp[k];
    const df32 re = df_from_double(v.x), im = df_from_double(v.y);
    S.lexp32[k] = make_float4(re.hi, im.hi, re.lo, im.lo);
}

// ---------------------------------------------------------------------------
// mixed-precision cell-staged near field + expansion evaluation + self term.
// Pair terms in df32 (exact coordinate differences, df32 r^2, corrected rsqrt,
// compensated accumulation); expansion terms l <= 2 in df32, l > 2 in FP32
// with compensated accumulation; self term: moved pair in df32, images in FP32.
// Results are written as FP64 (hi + lo).
// ---------------------------------------------------------------------------
// LT > 0: the order is the compile-time LT (loops unrolled, table offsets constant)
template <int LT = 0>
__device__ __forceinline__ df32 far_eval_mixed(const float4 *Lc, const int Lr, const df32 x, const df32 y,
                                               const df32 z)
{
    const int L = LT > 0 ? LT : Lr;
    // FP32 part, l >= 3
    const float xf = x.hi, yf = y.hi, zf = z.hi;
    const float r2 = xf * xf + yf * yf + zf * zf;
    float dre = 1.0f, dim = 0.0f;
    df32 acc = df_make(0.0f, 0.0f);
#pragma unroll
    for (int m = 0; m < L; ++m) {
        if (m > 0) {
            const float t = c_rec_d2[m].x;
            const float nre = t * (dre * xf - dim * yf);
            const float nim = t * (dre * yf + dim * xf);
            dre = nre;
            dim = nim;
        }
        float pre = 0.0f, pim = 0.0f, cre = dre, cim = dim;
        float part = 0.0f;
#pragma unroll
        for (int l = m; l < L; ++l) {
            if (l > m) {
                const float az = c_rec_a2[l * KMC_LMAX + m].x * zf;
                const float br = c_rec_b2[l * KMC_LMAX + m].x * r2;
                const float nre = az * cre - br * pre;
                const float nim = az * cim - br * pim;
                pre = cre;
                pim = cim;
                cre = nre;
                cim = nim;
            }
            if (l >= 3) {
                const float4 Lv = Lc[hidx(l, m)];
                part += Lv.x * cre - Lv.y * cim;
            }
        }
        df_acc_f(acc, (m == 0) ? part : 2.0f * part);
    }
    // df32 part, l <= 2 (only orders that exist)
    const float4 L00 = Lc[0];
    df_acc(acc, df_make(L00.x, L00.z));
    if (L > 1) {
        const df32 r2d = df_add(df_add(df_mul(x, x), df_mul(y, y)), df_mul(z, z));
        // Rg_1^0 = z, Rg_1^1 = d1 (x + i y)
        const float4 L10 = Lc[hidx(1, 0)], L11 = Lc[hidx(1, 1)];
        df_acc(acc, df_mul(df_make(L10.x, L10.z), z));
        const df32 d1 = df_make(c_rec_d2[1].x, c_rec_d2[1].y);
        const df32 r11 = df_mul(d1, x), i11 = df_mul(d1, y);
        df32 t = df_sub(df_mul(df_make(L11.x, L11.z), r11), df_mul(df_make(L11.y, L11.w), i11));
        df_acc(acc, df_mul_f(t, 2.0f));
        if (L > 2) {
            // Rg_2^0 = 3/2 z^2 - 1/2 r^2 ; Rg_2^1 = sqrt(3) z Rg_1^1 ; Rg_2^2 = d2 (x + i y) Rg_1^1
            const float4 L20 = Lc[hidx(2, 0)], L21 = Lc[hidx(2, 1)], L22 = Lc[hidx(2, 2)];
            const df32 r20 = df_sub(df_mul_f(df_mul(z, z), 1.5f), df_mul_f(r2d, 0.5f));
            df_acc(acc, df_mul(df_make(L20.x, L20.z), r20));
            constexpr double kS3 = 1.7320508075688772;  // sqrt(3), split at compile time
            constexpr float kS3h = (float)kS3, kS3l = (float)(kS3 - (double)kS3h);
            const df32 s3z = df_mul(df_make(kS3h, kS3l), z);
            const df32 r21 = df_mul(s3z, r11), i21 = df_mul(s3z, i11);
            t = df_sub(df_mul(df_make(L21.x, L21.z), r21), df_mul(df_make(L21.y, L21.w), i21));
            df_acc(acc, df_mul_f(t, 2.0f));
            const df32 d2 = df_make(c_rec_d2[2].x, c_rec_d2[2].y);
            const df32 ux = df_mul(d2, x), uy = df_mul(d2, y);
            const df32 r22 = df_sub(df_mul(ux, r11), df_mul(uy, i11));
            const df32 i22 = df_add(df_mul(ux, i11), df_mul(uy, r11));
            t = df_sub(df_mul(df_make(L22.x, L22.z), r22), df_mul(df_make(L22.y, L22.w), i22));
            df_acc(acc, df_mul_f(t, 2.0f));
        }
    }
    return acc;
}


// q_j / r for an item (grid coordinates ph + pl, cell widths) and a staged
// neighbour (h = grid high words and q_hi, l = low words and q_lo):
//   s = ph - h and S = |s|^2 exact (grid_split: 12-bit high words);
//   r2l = 2 s.l + |l|^2 = l.(2 s + l) in FP32 (relative error of r^2 about
//   2^-24 |r2l| / r^2, ~2^-30 at the nearest lattice distance, 2^-24 for charges
//   within 2^-10 cell widths of each other);
//   r^2 = r2h + r2e exactly (fast two-sum, S >= |r2l| unless the pair is that close);
//   1/r = y + y/2 (1 - r^2 y^2) with y = rsqrtf(r2h), the residual r^2 y^2 - 1
//   formed with FMA from the exact square y^2 = yy + e (Newton's step for the
//   inverse square root, its error ~3/8 (1 - r^2 y^2)^2 ~ 2^-44);
//   the charge product error-free, the Newton term as q_hi y ~ th (2^-24 relative
//   of a 2^-22 correction).
// Returns th and the low part pl (q_j / r = th + pl).  near_pair_g and its packed
// form near_pair_g2 perform the same roundings in the same order.
struct NearPoint {
    float xh, xl, yh, yl, zh, zl;
};

__device__ __forceinline__ void near_pair_g(const NearPoint &p, const float4 h, const float4 l, float &th, float &pl)
{
    const float sx = p.xh - h.x, sy = p.yh - h.y, sz = p.zh - h.z;
    const float lx = p.xl - l.x, ly = p.yl - l.y, lz = p.zl - l.z;
    const float S2 = fmaf(sx, sx, fmaf(sy, sy, sz * sz));
    const float ux = fmaf(2.0f, sx, lx), uy = fmaf(2.0f, sy, ly), uz = fmaf(2.0f, sz, lz);
    const float r2l = fmaf(lx, ux, fmaf(ly, uy, lz * uz));
    const float r2h = S2 + r2l;
    const float r2e = r2l - (r2h - S2);
    const float y = rsqrtf(r2h);
    const float yy = y * y;
    const float e = fmaf(y, y, -yy);
    const float a1 = fmaf(r2h, yy, -1.0f);
    const float nrho = fmaf(r2h, e, fmaf(r2e, yy, a1));  // r^2 y^2 - 1
    th = h.w * y;
    pl = fmaf(h.w, y, -th);
    pl = fmaf(l.w, y, pl);
    pl = fmaf(-0.5f * th, nrho, pl);
}

// Packed form for two neighbours at once, lane i of each f2x holding neighbour
// i; the staged pair is four quads a = (x_hi, y_hi), b = (z_hi, q_hi),
// c = (x_lo, y_lo), d = (z_lo, q_lo).  Negations are sign-bit flips (exact, on
// the integer pipe).
struct NearPoint2 {
    f2x xh, xl, yh, yl, zh, zl;
    f2x mone, two, mhalf;  // packed constants -1, 2, -1/2, kept in registers across the pair loop
};

__device__ __forceinline__ void near_pair_g2(const NearPoint2 &p, const ulonglong2 a, const ulonglong2 b,
                                             const ulonglong2 c, const ulonglong2 d, f2x &th, f2x &pl)
{
    const f2x sx = f2_sub(p.xh, a.x), sy = f2_sub(p.yh, a.y), sz = f2_sub(p.zh, b.x);
    const f2x lx = f2_sub(p.xl, c.x), ly = f2_sub(p.yl, c.y), lz = f2_sub(p.zl, d.x);
    const f2x S2 = f2_fma(sx, sx, f2_fma(sy, sy, f2_mul(sz, sz)));
    const f2x ux = f2_fma(p.two, sx, lx), uy = f2_fma(p.two, sy, ly), uz = f2_fma(p.two, sz, lz);
    const f2x r2l = f2_fma(lx, ux, f2_fma(ly, uy, f2_mul(lz, uz)));
    const f2x r2h = f2_add(S2, r2l);
    const f2x r2e = f2_sub(r2l, f2_sub(r2h, S2));
    const f2x y = f2_rsqrt(r2h);
    const f2x yy = f2_mul(y, y);
    const f2x e = f2_fma(y, y, f2_neg(yy));
    const f2x a1 = f2_fma(r2h, yy, p.mone);
    const f2x nrho = f2_fma(r2h, e, f2_fma(r2e, yy, a1));
    th = f2_mul(b.y, y);
    pl = f2_fma(b.y, y, f2_neg(th));
    pl = f2_fma(d.y, y, pl);
    pl = f2_fma(f2_mul(p.mhalf, th), nrho, pl);
}

// The 26 periodic images of the moved-pair self term other than the nearest (ks, in
// (kx+1) + 3 (ky+1) + 9 (kz+1) numbering), as sum_k 1/|d + kE| - 1/|kE| plus 1/|d| when
// the nearest image is not k = 0; d in units with E = fn.  Pairs k, -k (13
// representatives) share D = |d|^2 + |kE|^2: |d +- kE|^2 = D +- 2 k.d, and
// 1/|d + kE| - 1/|kE| = -(2 k.d + |d|^2) / (|kE| e (|kE| + e)).  Each term is small
// beside the nearest image, so rsqrt and a fast reciprocal suffice.
__device__ __forceinline__ float self_images(const float dx, const float dy, const float dz, const float fn,
                                             const int ks)
{
    const float dd = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float fdx = fn * dx, fdy = fn * dy, fdz = fn * dz, nn = fn * fn;
    float im = ks != 13 ? rsqrtf(dd) : 0.0f;
#pragma unroll
    for (int t = 14; t < 27; ++t) {
        const int ix = t % 3 - 1, iy = (t / 3) % 3 - 1, iz = t / 9 - 1, k2 = ix * ix + iy * iy + iz * iz;
        const float kn = fn * (k2 == 1 ? 1.0f : (k2 == 2 ? 1.41421356f : 1.73205081f));
        const float kd = (ix ? (float)ix * fdx : 0.0f) + (iy ? (float)iy * fdy : 0.0f) + (iz ? (float)iz * fdz : 0.0f);
        const float D = fmaf((float)k2, nn, dd);
        const float ep = fmaf(2.0f, kd, D), em = fmaf(-2.0f, kd, D);
        const float yp = rsqrtf(ep), ym = rsqrtf(em);
        const float tp = fmaf(2.0f, kd, dd) * yp * __fdividef(1.0f, kn * fmaf(ep, yp, kn));
        const float tm = fmaf(-2.0f, kd, dd) * ym * __fdividef(1.0f, kn * fmaf(em, ym, kn));
        if (t != ks) im -= tp;
        if (26 - t != ks) im -= tm;
    }
    return im;
}

// Moved-pair self term (kmc_fmm_self_interaction.py:163-242) of proposal item gp
// (cell cx, cy, cz) and its charge's old position po, from the grid copies, in
// 1 / cell-width units: the sum over the 27 images d + kE of d = x_old - x_new
// (k in {-1,0,1}^3 per axis, as the reference takes them) plus the domain term
// -sum_{k != 0} 1/|kE|.  The image nearest to zero is formed in double-FP32 like
// a near-field pair (exact high-word differences), the other 26 in FP32 as
// 1/|d + kE| - 1/|kE| = -(2 kE.d + |d|^2) / (|kE| |d + kE| (|kE| + |d + kE|)) (or
// 1/|d| for k = 0), all of them small beside the nearest term.
__device__ __forceinline__ df32 self_term_grid(const Sys &S, const int cx, const int cy, const int cz, const int po,
                                               const NearPoint &gp)
{
    const int n = S.n, oc = S.pcell[po];
    const size_t a = (size_t)oc * S.cap + S.pslot[po];
    const float4 oh = S.st_hi[a], ol = S.st_lo[a];
    const float sh[3] = {(oh.x + (float)(oc % n - cx)) - gp.xh, (oh.y + (float)((oc / n) % n - cy)) - gp.yh,
                         (oh.z + (float)(oc / (n * n) - cz)) - gp.zh};
    const float sl[3] = {ol.x - gp.xl, ol.y - gp.yl, ol.z - gp.zl};
    int k[3] = {0, 0, 0};
    if (S.periodic)
        for (int t = 0; t < 3; ++t) k[t] = max(-1, min(1, (int)(-rintf(sh[t] / (float)n))));
    const NearPoint dp{sh[0] + (float)(k[0] * n), sl[0], sh[1] + (float)(k[1] * n), sl[1],
                       sh[2] + (float)(k[2] * n), sl[2]};
    float th, pl;
    near_pair_g(dp, make_float4(0.f, 0.f, 0.f, 1.f), make_float4(0.f, 0.f, 0.f, 0.f), th, pl);
    df32 e = df_make(th, pl);
    if (!S.periodic) return e;
    const int m2 = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
    if (m2) e = df_sub(e, df_rsqrt(df_make((float)(m2 * n * n), 0.f)));
    const float dx = sh[0] + sl[0], dy = sh[1] + sl[1], dz = sh[2] + sl[2];
    df_acc_f(e, self_images(dx, dy, dz, (float)n, (k[0] + 1) + 3 * (k[1] + 1) + 9 * (k[2] + 1)));
    return e;
}

// One warp per cell.  Items (moving charges of the cell, proposals into it) go in
// rounds of 32; in the last round each item gets s = 2^k lanes (s * items <= 32)
// that split its neighbour list and combine their sums by shuffles, so a cell
// with 32 + 5 items costs 1.25 rounds of the pair loop instead of 2.
constexpr int kNearMixedThreads = 32;

// PACKED: neighbours staged in pairs and summed two at a time with the packed
// FP32 instructions (near_pair_g2); otherwise one at a time (near_pair_g).
// LT > 0: the expansion order is the compile-time LT (far-field loops unrolled)
// self_in_lr: the per-proposal lattice kernel adds the moved pair's self term (pbc)
// kept: the moving charges' near-field potentials are taken from S.phin (kept by every
// accept), so they only evaluate the cell expansion; otherwise they are items of the
// pair loop like the proposals
template <bool PACKED, int CHUNK, int LT = 0>
// Registers held to what the residency allows: CHUNK 64 (~4.3 KB of shared memory) at most
// 64 a thread, so 32 blocks (the SM's limit) fit an SM; 27 blocks otherwise (~7.4 KB)
__global__ void __launch_bounds__(kNearMixedThreads, CHUNK <= 64 ? 32 : 27) k_near_cell_mixed(const Sys S, Props P, const bool self_in_lr,
                                                                        const int split, const bool kept)
{
    extern __shared__ float4 msm[];
    float4 *shi = msm;                       // [CHUNK]   (PACKED: [CHUNK / 2][4] pair quads)
    float4 *slo = shi + CHUNK;          // [CHUNK]
    float4 *lc = slo + CHUNK;           // [NH]
    int *spid = reinterpret_cast<int *>(lc + S.NH); // [CHUNK]
    int *sprop = spid + CHUNK;                  // [CHUNK] the cell's proposals, sorted
    unsigned long long *skey = reinterpret_cast<unsigned long long *>(sprop + CHUNK);  // [CHUNK] position keys
    int *ulead = reinterpret_cast<int *>(skey), *uidx = ulead + CHUNK;  // after the sort: leaders, unique index
    __shared__ int nb_cell[27], nb_off[28], nb_d[27][3];
    // `split` blocks per cell: block `half` takes the item rounds r = half, half + split, ...
    // (every item is computed exactly as with one block per cell, so the results do not
    // depend on `split`; the cell's set-up is repeated by each of its blocks)
    const int c = blockIdx.x / split, half = blockIdx.x - c * split;
    const int tid = threadIdx.x;
    const int n_old = S.cnt[c];
    const int p0 = P.cstart[c];
    const int np = P.cstart[c + 1] - p0;
    if (n_old + np == 0) return;
    const int n = S.n;
    const int cx = c % n, cy = (c / n) % n, cz = c / (n * n);
    if (tid < 27) {
        // slot 0 is the cell itself, so its charges are staged first: only those can be
        // an item's own charge, and only their pairs need the exclusion check
        const int o = tid == 0 ? 13 : (tid <= 13 ? tid - 1 : tid);
        const int dx = o % 3 - 1, dy = (o / 3) % 3 - 1, dz = o / 9 - 1;
        int nx = cx + dx, ny = cy + dy, nz = cz + dz;
        bool ok = true;
        if (nx < 0) { nx += n; ok = ok && S.periodic; } else if (nx >= n) { nx -= n; ok = ok && S.periodic; }
        if (ny < 0) { ny += n; ok = ok && S.periodic; } else if (ny >= n) { ny -= n; ok = ok && S.periodic; }
        if (nz < 0) { nz += n; ok = ok && S.periodic; } else if (nz >= n) { nz -= n; ok = ok && S.periodic; }
        const int cc = nx + n * (ny + n * nz);
        nb_cell[tid] = cc;
        nb_off[tid + 1] = ok ? S.cnt[cc] : 0;
        nb_d[tid][0] = dx;
        nb_d[tid][1] = dy;
        nb_d[tid][2] = dz;
    }
    for (int k = tid; k < S.NH; k += blockDim.x) lc[k] = S.lexp32[(size_t)c * S.NH + k];
    __syncthreads();
    if (tid == 0) {
        nb_off[0] = 0;
        for (int j = 0; j < 27; ++j) nb_off[j + 1] += nb_off[j];
    }
    __syncthreads();
    const int total_nb = nb_off[27];
    // Proposals arrive in cprops in atomic order; sort them by (position key, id) so
    // that which items share lanes in the last round (and so every rounding) does
    // not depend on that order, and so that proposals to the same position (hops of
    // different charges into one vacancy) are adjacent: their near-field sum and
    // cell expansion value depend on the position alone and are computed once (the
    // self term, which depends on the moving charge, per proposal afterwards).  A
    // cell with more than CHUNK proposals is not sorted and its items use one lane
    // each, which is order-independent as well.
    const bool sorted = np <= CHUNK;
    int nu = np;  // unique positions among the proposals (sorted cells)
    if (sorted) {
        int n2 = 1;
        while (n2 < np) n2 <<= 1;
        for (int k = tid; k < n2; k += blockDim.x) {
            int id = 0x7fffffff;
            unsigned long long key = ~0ull;
            if (k < np) {
                id = P.cprops[p0 + k];
                // a mix of the position's bits: equal positions give equal keys
                const unsigned long long bx = __double_as_longlong(P.ppos[3 * (size_t)id]),
                                         by = __double_as_longlong(P.ppos[3 * (size_t)id + 1]),
                                         bz = __double_as_longlong(P.ppos[3 * (size_t)id + 2]);
                key = (bx ^ (by * 0x9E3779B97F4A7C15ull) ^ (bz * 0xC2B2AE3D27D4EB4Full)) >> 1;
            }
            sprop[k] = id;
            skey[k] = key;
        }
        __syncthreads();
        for (int size = 2; size <= n2; size <<= 1)
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int a = tid; a < n2; a += blockDim.x) {
                    const int b = a ^ stride;
                    if (b > a) {
                        const unsigned long long ka = skey[a], kb = skey[b];
                        const int va = sprop[a], vb = sprop[b];
                        if ((ka > kb || (ka == kb && va > vb)) == ((a & size) == 0)) {
                            sprop[a] = vb;
                            sprop[b] = va;
                            skey[a] = kb;
                            skey[b] = ka;
                        }
                    }
                }
                __syncthreads();
            }
        // leaders: the first of each run of equal positions (exact comparison)
        bool lead[CHUNK / 32];
#pragma unroll
        for (int r = 0; r < CHUNK / 32; ++r) {
            const int k = 32 * r + tid;
            bool ld = false;
            if (k < np) {
                ld = k == 0 || skey[k] != skey[k - 1];
                if (!ld) {
                    const size_t a = 3 * (size_t)sprop[k], b = 3 * (size_t)sprop[k - 1];
                    ld = P.ppos[a] != P.ppos[b] || P.ppos[a + 1] != P.ppos[b + 1] || P.ppos[a + 2] != P.ppos[b + 2];
                }
            }
            lead[r] = ld;
        }
        __syncthreads();  // keys no longer read: their space holds leaders and indices
        int before = 0;
#pragma unroll
        for (int r = 0; r < CHUNK / 32; ++r) {
            const int k = 32 * r + tid;
            const unsigned bal = __ballot_sync(0xffffffffu, lead[r]);
            const int u = before + __popc(bal & ((1u << tid) - 1u)) + (lead[r] ? 0 : -1);
            if (k < np) {
                uidx[k] = u;
                if (lead[r]) ulead[u] = sprop[k];
            }
            before += __popc(bal);
        }
        nu = before;
        __syncthreads();
    }
    const int n_po = kept ? 0 : n_old;  // moving charges among the pair loop's items
    if (kept) {
        const df32 wd = df_make(S.w_hi, S.w_lo);
        for (int o = half * kNearMixedThreads + tid; o < n_old; o += split * kNearMixedThreads) {
            const size_t a = (size_t)c * S.cap + o;
            const int pidx = S.store_pid[a];
            if (P.cnt[pidx] <= 0) continue;
            const float4 gh = S.st_hi[a], gl = S.st_lo[a];
            const df32 ff = far_eval_mixed<LT>(lc, S.L, df_mul(df_make(gh.x, gl.x), wd),
                                               df_mul(df_make(gh.y, gl.y), wd), df_mul(df_make(gh.z, gl.z), wd));
            P.u0p[pidx] = S.q[pidx] * (S.phin[pidx] + df_to_double(ff));
        }
    }
    const int nitems = n_po + nu;
    for (int base = half * kNearMixedThreads; base < nitems; base += split * kNearMixedThreads) {
        const int rem = min(kNearMixedThreads, nitems - base);
        int sl = 1;
        while (sorted && sl * 2 * rem <= kNearMixedThreads) sl *= 2;
        const int item = base + tid / sl, sub = tid % sl;
        bool act = (tid / sl) < rem;
        double q = 0.0;
        float4 gh = make_float4(0.f, 0.f, 0.f, 0.f), gl = gh;
        int self = -1, pidx = -1, p = -1;
        if (act) {
            // the item's grid copy relative to this cell: the store's for a moving
            // charge, split here for a proposal
            if (item < n_po) {
                const size_t a = (size_t)c * S.cap + item;
                pidx = S.store_pid[a];
                act = P.cnt[pidx] > 0;
                self = pidx;
                gh = S.st_hi[a];
                gl = S.st_lo[a];
                q = S.q[pidx];
            } else {
                p = sorted ? ulead[item - n_po] : P.cprops[p0 + item - n_po];
                const float2 ux = grid_split((P.ppos[3 * (size_t)p] - cell_centre(S, cx)) * S.inv_w);
                const float2 uy = grid_split((P.ppos[3 * (size_t)p + 1] - cell_centre(S, cy)) * S.inv_w);
                const float2 uz = grid_split((P.ppos[3 * (size_t)p + 2] - cell_centre(S, cz)) * S.inv_w);
                gh = make_float4(ux.x, uy.x, uz.x, 0.f);
                gl = make_float4(ux.y, uy.y, uz.y, 0.f);
                q = P.pq[p];
                if (sorted && sub == 0 && !self_in_lr) {
                    P.ugrid[2 * (size_t)p] = gh;  // for the self terms of the position's proposals
                    P.ugrid[2 * (size_t)p + 1] = gl;
                }
            }
        }
        const NearPoint gp{gh.x, gl.x, gh.y, gl.y, gh.z, gl.z};
        const float2 gx = make_float2(gh.x, gl.x), gy = make_float2(gh.y, gl.y), gz = make_float2(gh.z, gl.z);
        df32 acc = df_make(0.0f, 0.0f), acc1 = df_make(0.0f, 0.0f);
        NearPoint2 pp;
        f2x a0h = 0ull, a0l = 0ull, a1h = 0ull, a1l = 0ull;  // 0ull: both lanes +0.0f
        if constexpr (PACKED) {
            pp.xh = f2_splat(gx.x);
            pp.xl = f2_splat(gx.y);
            pp.yh = f2_splat(gy.x);
            pp.yl = f2_splat(gy.y);
            pp.zh = f2_splat(gz.x);
            pp.zl = f2_splat(gz.y);
            pp.mone = f2_splat(-1.0f);
            pp.two = f2_splat(2.0f);
            pp.mhalf = f2_splat(-0.5f);
        }
        for (int k0 = 0; k0 < total_nb; k0 += CHUNK) {
            const int kn = min(CHUNK, total_nb - k0);
            // a neighbourhood that fits one chunk is staged once for all item rounds
            if (base == half * kNearMixedThreads || total_nb > CHUNK) {
                __syncthreads();
                int j = 0;  // the neighbour cell of kk; kk only grows, so the search resumes
                for (int k = tid; k < kn; k += blockDim.x) {
                    const int kk = k0 + k;
                    while (nb_off[j + 1] <= kk) ++j;
                    const size_t a = (size_t)nb_cell[j] * S.cap + (kk - nb_off[j]);
                    float4 h = S.st_hi[a];
                    const float4 l = S.st_lo[a];
                    // into this cell's frame: + d cell widths (exact on the grid)
                    h.x += (float)nb_d[j][0];
                    h.y += (float)nb_d[j][1];
                    h.z += (float)nb_d[j][2];
                    if constexpr (PACKED) {
                        float *f = reinterpret_cast<float *>(shi) + 16 * (k >> 1) + (k & 1);
                        f[0] = h.x; f[2] = h.y; f[4] = h.z; f[6] = h.w;
                        f[8] = l.x; f[10] = l.y; f[12] = l.z; f[14] = l.w;
                    } else {
                        shi[k] = h;
                        slo[k] = l;
                    }
                    spid[k] = S.store_pid[a];
                }
                if (PACKED && (kn & 1) && tid == 0) {
                    // odd count: a chargeless partner far outside the neighbourhood
                    float *f = reinterpret_cast<float *>(shi) + 16 * (kn >> 1) + 1;
                    f[0] = f[2] = f[4] = 64.0f;
                    f[6] = f[8] = f[10] = f[12] = f[14] = 0.0f;
                    spid[kn] = -2;
                }
                __syncthreads();
            }
            if (PACKED && act) {
                const ulonglong2 *q4 = reinterpret_cast<const ulonglong2 *>(shi);
                const int2 *pid2 = reinterpret_cast<const int2 *>(spid);
                const int npair = (kn + 1) >> 1;
                // pairs holding charges of this cell (staged first): with the exclusion check
                const int jo = (max(0, min(kn, n_old - k0)) + 1) >> 1;
                for (int j = sub; j < jo; j += sl) {
                    f2x th0, pl0;
                    near_pair_g2(pp, q4[4 * j], q4[4 * j + 1], q4[4 * j + 2], q4[4 * j + 3], th0, pl0);
                    const int2 i0 = pid2[j];
                    th0 = f2_zero_lanes(th0, i0.x == self, i0.y == self);
                    pl0 = f2_zero_lanes(pl0, i0.x == self, i0.y == self);
                    f2_acc(a0h, a0l, th0, pl0);
                }
                // the other cells' pairs: two per iteration, independent accumulators
                int j = jo + (((sub - jo) % sl) + sl) % sl;
                for (; j + sl < npair; j += 2 * sl) {
                    f2x th0, pl0, th1, pl1;
                    near_pair_g2(pp, q4[4 * j], q4[4 * j + 1], q4[4 * j + 2], q4[4 * j + 3], th0, pl0);
                    near_pair_g2(pp, q4[4 * (j + sl)], q4[4 * (j + sl) + 1], q4[4 * (j + sl) + 2],
                                 q4[4 * (j + sl) + 3], th1, pl1);
                    f2_acc(a0h, a0l, th0, pl0);
                    f2_acc(a1h, a1l, th1, pl1);
                }
                if (j < npair) {
                    f2x th0, pl0;
                    near_pair_g2(pp, q4[4 * j], q4[4 * j + 1], q4[4 * j + 2], q4[4 * j + 3], th0, pl0);
                    f2_acc(a0h, a0l, th0, pl0);
                }
            } else if (act) {
                // two neighbours per iteration, independent accumulators (more ILP per warp)
                int k = sub;
                for (; k + sl < kn; k += 2 * sl) {
                    float h0, e0, h1, e1;
                    near_pair_g(gp, shi[k], slo[k], h0, e0);
                    near_pair_g(gp, shi[k + sl], slo[k + sl], h1, e1);
                    if (spid[k] != self) df_acc(acc, df_make(h0, e0));
                    if (spid[k + sl] != self) df_acc(acc1, df_make(h1, e1));
                }
                if (k < kn && spid[k] != self) {
                    float h0, e0;
                    near_pair_g(gp, shi[k], slo[k], h0, e0);
                    df_acc(acc, df_make(h0, e0));
                }
            }
        }
        if constexpr (PACKED) {
            // four lane sums (two accumulators x two lanes)
            float h0, h1, h2, h3, l0, l1, l2, l3;
            f2_unpack(a0h, h0, h1);
            f2_unpack(a1h, h2, h3);
            f2_unpack(a0l, l0, l1);
            f2_unpack(a1l, l2, l3);
            acc = df_add(df_add(df_make(h0, l0), df_make(h1, l1)), df_add(df_make(h2, l2), df_make(h3, l3)));
        } else {
            acc = df_add(acc, acc1);
        }
        for (int off = sl / 2; off > 0; off >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, acc.hi, off);
            const float ol = __shfl_xor_sync(0xffffffffu, acc.lo, off);
            acc = df_add(acc, df_make(oh, ol));
        }
        if (act && sub == 0) {
            // far field at the point in position units (df32 from the grid copy)
            const df32 wd = df_make(S.w_hi, S.w_lo), iwd = df_make(S.iw_hi, S.iw_lo);
            const df32 px = df_mul(df_make(gx.x, gx.y), wd), py = df_mul(df_make(gy.x, gy.y), wd),
                       pz = df_mul(df_make(gz.x, gz.y), wd);
            const df32 ff = far_eval_mixed<LT>(lc, S.L, px, py, pz);
            const double pot = df_to_double(df_add(df_mul(acc, iwd), ff));
            if (self >= 0) {
                P.u0p[pidx] = q * pot;
            } else if (sorted) {
                P.upot[p] = pot;  // per position; the proposals take it below
            } else if (self_in_lr) {
                P.pnew[p] = q * pot;
            } else {
                const int po = P.old_pid[P.owner[p]];
                const double qo = S.q[po];
                const double usi = qo * qo * df_to_double(df_mul(self_term_grid(S, cx, cy, cz, po, gp), iwd));
                P.pnew[p] = q * pot - usi;
            }
        }
    }
    if (sorted) {
        // every proposal: its position's potential, its charge and its own self term
        __syncwarp();
        const df32 iwd = df_make(S.iw_hi, S.iw_lo);
        for (int k = tid; k < np; k += blockDim.x) {
            if (((n_po + uidx[k]) / kNearMixedThreads) % split != half) continue;  // another block's leader
            const int p = sprop[k], lp = ulead[uidx[k]];
            const double pot = P.upot[lp];
            if (self_in_lr) {
                P.pnew[p] = P.pq[p] * pot;
                continue;
            }
            const float4 h = P.ugrid[2 * (size_t)lp], l = P.ugrid[2 * (size_t)lp + 1];
            const NearPoint gp{h.x, l.x, h.y, l.y, h.z, l.z};  // the leader's position is this one's
            const int po = P.old_pid[P.owner[p]];
            const double qo = S.q[po];
            const double usi = qo * qo * df_to_double(df_mul(self_term_grid(S, cx, cy, cz, po, gp), iwd));
            P.pnew[p] = P.pq[p] * pot - usi;
        }
    }
}
