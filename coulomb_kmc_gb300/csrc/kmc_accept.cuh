// Part of the kmc_gb300.cu translation unit (included there, in order, inside its
// anonymous namespace unless it says otherwise): the accept: store update and record, multipole and g update, the particle-to-local kernels (FP64 per column, double-FP32 forms, FP64 column pairs).
#pragma once
// ---------------------------------------------------------------------------
// accept (kmc_fmm.py:811-912): store swap-remove / append, position, energy
// ---------------------------------------------------------------------------
// The accepted move's store update (kmc_local.py:180-357) on one block: thread 32
// bins the new position and checks that the new cell has a free slot; thread 0
// then extracts the charge from its old cell (swap with the cell's last slot)
// while thread 32 forms the new position's grid copy (the FP64 part); thread 0
// appends the charge to its new cell and fills the record; the block copies the
// old and new cells' expansions (and g) to `snap`, read by the single-move energy
// kernel while the particle-to-local kernel rewrites the expansions.  add_de:
// advance the energy by *d_de here (no single-move kernel).
// A full new cell (device-selected accepts only: the host path grows the store
// first, as the reference does, kmc_local.py:318-326) leaves the state untouched:
// the record says skip, the overflow counter (pend[1]) advances and the move is
// kept in pend[2..5] (pid + 1, position bits) for kmc_resolve_overflow; while a
// move is kept, every later accept is refused the same way, so the state stays
// the one before the refused move.
__global__ void k_accept_prep(Sys S, const int mode, const int pid_h, const double xh, const double yh,
                              const double zh, const long long *d_pid, const double *d_pos, const double *d_de,
                              double *energy, AcceptRec *rec, unsigned long long *pend, const int add_de,
                              double2 *snap, const double2 *g)
{
    __shared__ int s_co, s_cn, s_refuse;
    __shared__ float4 s_hi, s_lo;
    const int pid = mode ? (int)d_pid[0] : pid_h;
    if (pid < 0) {  // device selection rejected every move: nothing changes
        if (threadIdx.x == 0) rec->skip = 1;
        return;
    }
    const double xn = mode ? d_pos[0] : xh, yn = mode ? d_pos[1] : yh, zn = mode ? d_pos[2] : zh;
    if (threadIdx.x == 32) {
        const int cn = bin_cell(xn, yn, zn, S);
        const int co = S.pcell[pid];
        const int refuse = pend[2] != 0ull || (cn != co && S.cnt[cn] >= S.cap);
        s_cn = cn;
        s_co = co;
        s_refuse = refuse;
        rec->skip = refuse;
        if (refuse) {
            atomicAdd(pend + 1, 1ull);
            if (pend[2] == 0ull) {
                pend[3] = (unsigned long long)__double_as_longlong(xn);
                pend[4] = (unsigned long long)__double_as_longlong(yn);
                pend[5] = (unsigned long long)__double_as_longlong(zn);
                pend[2] = (unsigned long long)pid + 1ull;
            }
        }
    }
    // warps 0 and 1 meet here (named barrier 1): thread 32's cell and decision are
    // visible to thread 0; warps 2 and 3 read them after the block barrier below
    if (threadIdx.x < 64) asm volatile("bar.sync 1, 64;" ::: "memory");
    if (threadIdx.x == 32 && !s_refuse && S.mixed) {
        const int cn = s_cn;
        const int cx = cn % S.n, cy = (cn / S.n) % S.n, cz = cn / (S.n * S.n);
        const float2 rx = grid_split((xn - cell_centre(S, cx)) * S.inv_w);
        const float2 ry = grid_split((yn - cell_centre(S, cy)) * S.inv_w);
        const float2 rz = grid_split((zn - cell_centre(S, cz)) * S.inv_w);
        const df32 rq = df_from_double(S.q[pid]);
        s_hi = make_float4(rx.x, ry.x, rz.x, rq.hi);
        s_lo = make_float4(rx.y, ry.y, rz.y, rq.lo);
    }
    double xo = 0.0, yo = 0.0, zo = 0.0;
    if (threadIdx.x == 0 && !s_refuse) {
        const int co = s_co;
        xo = S.pos[3 * (size_t)pid];
        yo = S.pos[3 * (size_t)pid + 1];
        zo = S.pos[3 * (size_t)pid + 2];
        // extract: swap with the last slot (kmc_local.py:180-265)
        const int sl = S.pslot[pid];
        const int last = S.cnt[co] - 1;
        if (sl != last) {
            const size_t a = (size_t)co * S.cap + sl, b = (size_t)co * S.cap + last;
            S.store[a] = S.store[b];
            const int moved = S.store_pid[b];
            S.store_pid[a] = moved;
            S.pslot[moved] = sl;
            if (S.mixed) {
                S.st_hi[a] = S.st_hi[b];
                S.st_lo[a] = S.st_lo[b];
            }
        }
        S.cnt[co] = last;
    }
    __syncthreads();
    const int co = s_co, cn = s_cn;
    if (s_refuse) return;
    if (threadIdx.x == 0) {
        const double q = S.q[pid];
        // the reference's accept recomputes the energy with propose(), which returns
        // the unchanged energy for a null move (kmc_fmm.py:1094-1095): |x_o - x_n| < 1e-14
        const double ddx = xo - xn, ddy = yo - yn, ddz = zo - zn;
        const bool null_move = ddx * ddx + ddy * ddy + ddz * ddz < 1e-28;
        if (!null_move && add_de) *energy += *d_de;
        // inject: append (kmc_local.py:268-357); the slot exists (checked above)
        const int k = S.cnt[cn];
        const size_t a = (size_t)cn * S.cap + k;
        S.store[a] = make_double4_32a(xn, yn, zn, q);
        S.store_pid[a] = pid;
        S.pslot[pid] = k;
        S.cnt[cn] = k + 1;
        if (S.mixed) {
            S.st_hi[a] = s_hi;
            S.st_lo[a] = s_lo;
        }
        S.pcell[pid] = cn;
        S.pos[3 * (size_t)pid] = xn;
        S.pos[3 * (size_t)pid + 1] = yn;
        S.pos[3 * (size_t)pid + 2] = zn;
        rec->null_move = null_move;
        rec->pid = pid;
        rec->co = co;
        rec->cn = cn;
        rec->q = q;
        rec->xo = xo;
        rec->yo = yo;
        rec->zo = zo;
        rec->xn = xn;
        rec->yn = yn;
        rec->zn = zn;
        rec->to[0] = co % S.n;
        rec->to[1] = (co / S.n) % S.n;
        rec->to[2] = co / (S.n * S.n);
        rec->tn[0] = cn % S.n;
        rec->tn[1] = (cn / S.n) % S.n;
        rec->tn[2] = cn / (S.n * S.n);
    }
    if (snap)
        for (int k = threadIdx.x; k < S.NH; k += blockDim.x) {
            snap[k] = S.lexp[(size_t)co * S.NH + k];
            snap[S.NH + k] = S.lexp[(size_t)cn * S.NH + k];
            if (S.pbc) snap[2 * S.NH + k] = g[k];
        }
}



// Level-0 multipole update of an accepted move in FP64 (FullLongRangeEnergy.accept,
// kmc_full_long_range.py:270-316): M += q (conj Rg(x_new) - conj Rg(x_old)) (the
// reference's two updates, -q at the old position then +q at the new), and the
// lattice vector g = A M, over kMgBlocks blocks.  Every block forms the new M from
// the stored one (thread h < NH owns M_{l,m}: column recurrence up to its l) into
// shared memory, then takes every kMgBlocks-th group of rows of g with one warp
// per row (lanes over the row's entries, a shuffle reduction): short FP64
// dependency chains on many SMs instead of one block's long ones.  The last block
// to finish (a ticket, no waiting) stores M, after every block has read the old.
constexpr int kMgBlocks = 8, kMgThreads = 128;

// DF (the mixed paths): the increments of M and the rows of g in double-FP32 on the
// FP32 pipe (FP64 dependency chains are slow on GB300; ~48-bit significands keep g and
// M within ~1e-14 of the FP64 forms), in box units (coordinates x / E, the operator
// A E^(l + l' + 1) split into FP32 pairs at set-up: a2_val, ai2_val), which keeps every
// value in the FP32 range for any box up to l = 20.
template <bool DF>
__global__ void __launch_bounds__(kMgThreads) k_accept_mpole_g(Sys S, Props P, const AcceptRec *rec,
                                                              unsigned *ticket)
{
    extern __shared__ double2 mgs[];  // M after the move [NH]; DF: its FP32 pairs [NH]; the recurrence table
    __shared__ bool last;
    if (rec->skip) return;
    const AcceptRec r = *rec;
    const int NH = S.NH, L = S.L;
    float4 *m2 = reinterpret_cast<float4 *>(mgs + NH);
    RecTab T;
    float2 *t2 = reinterpret_cast<float2 *>(m2 + (DF ? NH : 0));  // DF: a, b (l * L + m), d
    if (DF) {
        for (int k = threadIdx.x; k < L * L; k += blockDim.x) {
            const int l = k / L, m = k - l * L;
            t2[k] = g_rec_a2[l * KMC_LMAX + m];
            t2[L * L + k] = g_rec_b2[l * KMC_LMAX + m];
        }
        for (int k = threadIdx.x; k < L; k += blockDim.x) t2[2 * L * L + k] = g_rec_d2[k];
    } else {
        T = stage_rec(reinterpret_cast<double *>(m2), L);
    }
    __syncthreads();
    for (int h = threadIdx.x; h < NH; h += blockDim.x) {
        int l = 0;
        while (hidx(l + 1, 0) <= h) ++l;
        const int m = h - hidx(l, 0);
        double dv[2][2];
        for (int pass = 0; pass < 2; ++pass) {
            const double x = pass == 0 ? r.xo : r.xn, y = pass == 0 ? r.yo : r.yn, z = pass == 0 ? r.zo : r.zn;
            if (DF) {
                // at x / E (box units: the harmonics of position-unit coordinates leave the
                // FP32 range for large boxes at high orders), scaled back by E^l in FP64
                const df32 xd = df_from_double(x * S.inv_E), yd = df_from_double(y * S.inv_E),
                           zd = df_from_double(z * S.inv_E);
                const df32 r2 = df_add(df_add(df_mul(xd, xd), df_mul(yd, yd)), df_mul(zd, zd));
                df32 dre = df_make(1.0f, 0.0f), dim = df_make(0.0f, 0.0f);
                for (int k = 1; k <= m; ++k) {
                    const float2 tv = t2[2 * L * L + k];
                    const df32 t = df_make(tv.x, tv.y);
                    const df32 nre = df_mul(t, df_fms(dre, xd, dim, yd));
                    const df32 nim = df_mul(t, df_fma2(dre, yd, dim, xd));
                    dre = nre;
                    dim = nim;
                }
                df32 pre = df_make(0.0f, 0.0f), pim = pre, cre = dre, cim = dim;
                for (int k = m + 1; k <= l; ++k) {
                    const float2 av = t2[k * L + m], bv = t2[L * L + k * L + m];
                    const df32 az = df_mul(df_make(av.x, av.y), zd), br = df_mul(df_make(bv.x, bv.y), r2);
                    const df32 nre = df_fms(az, cre, br, pre), nim = df_fms(az, cim, br, pim);
                    pre = cre;
                    pim = cim;
                    cre = nre;
                    cim = nim;
                }
                const double sc = S.escale[h] * S.inv_E;
                dv[pass][0] = df_to_double(cre) * sc;
                dv[pass][1] = df_to_double(cim) * sc;
            } else {
                const double r2 = x * x + y * y + z * z;
                double dre = 1.0, dim = 0.0;
                for (int k = 1; k <= m; ++k) {
                    const double t = T.d[k];
                    const double nre = t * (dre * x - dim * y);
                    const double nim = t * (dre * y + dim * x);
                    dre = nre;
                    dim = nim;
                }
                double pre = 0.0, pim = 0.0, cre = dre, cim = dim;
                for (int k = m + 1; k <= l; ++k) {
                    const double az = T.a[k * T.L + m] * z;
                    const double br = T.b[k * T.L + m] * r2;
                    const double nre = az * cre - br * pre;
                    const double nim = az * cim - br * pim;
                    pre = cre;
                    pim = cim;
                    cre = nre;
                    cim = nim;
                }
                dv[pass][0] = cre;
                dv[pass][1] = cim;
            }
        }
        // the same two updates as the reference's accept: -q at the old position, then +q at the new
        double2 v = S.mpole[h];
        v.x += -r.q * dv[0][0];
        v.y += r.q * dv[0][1];
        v.x += r.q * dv[1][0];
        v.y += -r.q * dv[1][1];
        mgs[h] = v;
        if (DF) {
            // in box units, M E^-(l + 1), against the box-unit operator pairs
            const double ie = 1.0 / S.escale[h];
            const df32 vr = df_from_double(v.x * ie), vi = df_from_double(v.y * ie);
            m2[h] = make_float4(vr.hi, vi.hi, vr.lo, vi.lo);
        }
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int row = blockIdx.x * nw + warp; row < NH; row += gridDim.x * nw) {
        if (DF) {
            df32 t = df_make(0.0f, 0.0f), u = t;
            for (int k = S.ar_ptr[row] + lane; k < S.ar_ptr[row + 1]; k += 32) {
                const float2 av = S.a2_val[k];
                const float4 mv = m2[S.ar_col[k]];
                df_acc(t, df_mul(df_make(av.x, av.y), df_make(mv.x, mv.z)));
            }
            for (int k = S.ai_ptr[row] + lane; k < S.ai_ptr[row + 1]; k += 32) {
                const float2 av = S.ai2_val[k];
                const float4 mv = m2[S.ai_col[k]];
                df_acc(u, df_mul(df_make(av.x, av.y), df_make(mv.y, mv.w)));
            }
            for (int off = 16; off > 0; off >>= 1) {
                t = df_add(t, df_make(__shfl_xor_sync(0xffffffffu, t.hi, off), __shfl_xor_sync(0xffffffffu, t.lo, off)));
                u = df_add(u, df_make(__shfl_xor_sync(0xffffffffu, u.hi, off), __shfl_xor_sync(0xffffffffu, u.lo, off)));
            }
            // box units: sum A E^(l + l' + 1) M E^-(l' + 1) = E^l (A M)_row
            if (lane == 0) {
                const double sc = S.E / S.escale[row];
                P.g[row] = make_double2(df_to_double(t) * sc, df_to_double(u) * sc);
            }
        } else {
            double t = 0.0, u = 0.0;
            for (int k = S.ar_ptr[row] + lane; k < S.ar_ptr[row + 1]; k += 32) t += S.ar_val[k] * mgs[S.ar_col[k]].x;
            for (int k = S.ai_ptr[row] + lane; k < S.ai_ptr[row + 1]; k += 32) u += S.ai_val[k] * mgs[S.ai_col[k]].y;
            for (int off = 16; off > 0; off >>= 1) {
                t += __shfl_xor_sync(0xffffffffu, t, off);
                u += __shfl_xor_sync(0xffffffffu, u, off);
            }
            if (lane == 0) P.g[row] = make_double2(t, u);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last) {
        for (int h = threadIdx.x; h < NH; h += blockDim.x) S.mpole[h] = mgs[h];
        if (threadIdx.x == 0) *ticket = 0u;
    }
}

// ---------------------------------------------------------------------------
// particle-to-local into every cell for a list of source charges, applying
// the well-separated rule of accept_local_exp (kmc_octal.py:961-1089).
// MODE 0: the 2*nimg images of an accepted move (old with -q, new with +q)
// MODE 1: all N charges times nimg images (initial solve)
// block = (cpb cells) x (L values of m); thread (cell, m) owns L_{l,m}, l >= m
// ---------------------------------------------------------------------------
struct Src {
    double x, y, z, q;
    int tx, ty, tz, pad;
};

__device__ __forceinline__ Src make_src(const Sys &S, const AcceptRec *rec, const int mode, const int s)
{
    int img;
    double px, py, pz, qq;
    int t0, t1, t2;
    if (mode == 0) {
        const int pass = s / S.nimg;
        img = s % S.nimg;
        const AcceptRec &r = *rec;
        px = pass ? r.xn : r.xo;
        py = pass ? r.yn : r.yo;
        pz = pass ? r.zn : r.zo;
        qq = pass ? r.q : -r.q;
        t0 = pass ? r.tn[0] : r.to[0];
        t1 = pass ? r.tn[1] : r.to[1];
        t2 = pass ? r.tn[2] : r.to[2];
    } else {
        const int j = s / S.nimg;
        img = s % S.nimg;
        px = S.pos[3 * (size_t)j];
        py = S.pos[3 * (size_t)j + 1];
        pz = S.pos[3 * (size_t)j + 2];
        qq = S.q[j];
        const int c = S.pcell[j];
        t0 = c % S.n;
        t1 = (c / S.n) % S.n;
        t2 = c / (S.n * S.n);
    }
    int ox = 0, oy = 0, oz = 0;
    if (S.nimg == 27) {
        ox = img % 3 - 1;
        oy = (img / 3) % 3 - 1;
        oz = img / 9 - 1;
    }
    Src v;
    v.x = ox * S.E + px;
    v.y = oy * S.E + py;
    v.z = oz * S.E + pz;
    v.q = qq;
    v.tx = ox * S.n + t0;
    v.ty = oy * S.n + t1;
    v.tz = oz * S.n + t2;
    v.pad = 0;
    return v;
}

// Particle-to-local into every cell for a list of source charges, with the
// well-separated rule of accept_local_exp (kmc_octal.py:961-1089):
// MODE 0: the 2*nimg images of an accepted move (old with -q, new with +q)
// MODE 1: all N charges times nimg images (initial solve)
// Block = cpb cells x L threads; sources go in chunks of L:
//   phase A: one thread per (cell, source) computes the geometry and the
//            diagonal Ir_m^m for all m into shared memory,
//   phase B: thread (cell, m) runs the l-chain of its m for every source of
//            the chunk and accumulates L_{l,m} (exclusive owner, no atomics).
template <int MODE>
__global__ void k_p2l(Sys S, const AcceptRec *rec, const int nsrc)
{
    if (MODE == 0 && rec->skip) return;
    extern __shared__ double4_32a smem4[];
    const int cpb = blockDim.x;
    const int NH = S.NH, L = S.L;
    const int SC = L;  // sources per chunk
    double2 *acc = reinterpret_cast<double2 *>(smem4);          // [NH][cpb]
    double2 *gd = acc + (size_t)NH * cpb;                         // [SC][cpb][L] diagonal Ir_m^m (times q)
    double *gz = reinterpret_cast<double *>(gd + (size_t)SC * cpb * L); // [SC][cpb] z / r^2
    double *gr = gz + (size_t)SC * cpb;                            // [SC][cpb] 1 / r^2 (0: not separated)
    const int ci = threadIdx.x, m = threadIdx.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
    for (int k = tid; k < NH * cpb; k += nthr) acc[k] = make_double2(0.0, 0.0);
    for (int s0 = 0; s0 < nsrc; s0 += SC) {
        const int ns = min(SC, nsrc - s0);
        __syncthreads();
        // phase A: (cell, source) pairs; nthr = cpb * L = cpb * SC, so one pair per thread
        {
            const int sidx = tid / cpb, pc = tid % cpb;
            const int cell = blockIdx.x * cpb + pc;
            double *zr_out = gz + (size_t)sidx * cpb + pc;
            double *r2_out = gr + (size_t)sidx * cpb + pc;
            if (sidx < ns && cell < S.ncell) {
                const Src v = make_src(S, rec, MODE, s0 + sidx);
                const int fx = cell % S.n, fy = (cell / S.n) % S.n, fz = cell / (S.n * S.n);
                const bool near = abs(v.tx - fx) < 2 && abs(v.ty - fy) < 2 && abs(v.tz - fz) < 2;
                if (!near) {
                    const double dx = v.x - cell_centre(S, fx), dy = v.y - cell_centre(S, fy),
                                 dz = v.z - cell_centre(S, fz);
                    const double ri = rsqrt(dx * dx + dy * dy + dz * dz);
                    const double ri2 = ri * ri;
                    const double wre = dx * ri2, wim = -dy * ri2;
                    double ire = v.q * ri, iim = 0.0;
                    double2 *dg = gd + ((size_t)sidx * cpb + pc) * L;
                    dg[0] = make_double2(ire, iim);
                    for (int k2 = 1; k2 < L; ++k2) {
                        const double t = c_rec_d[k2];
                        const double nre = t * (ire * wre - iim * wim);
                        const double nim = t * (ire * wim + iim * wre);
                        ire = nre;
                        iim = nim;
                        dg[k2] = make_double2(ire, iim);
                    }
                    *zr_out = dz * ri2;
                    *r2_out = ri2;
                } else {
                    *r2_out = 0.0;
                }
            } else if (sidx < SC) {
                *r2_out = 0.0;
            }
        }
        __syncthreads();
        // phase B
        const int cell = blockIdx.x * cpb + ci;
        if (cell < S.ncell) {
            for (int k = 0; k < ns; ++k) {
                const double ri2 = gr[(size_t)k * cpb + ci];
                if (ri2 == 0.0) continue;
                const double zr = gz[(size_t)k * cpb + ci];
                const double2 d0 = gd[((size_t)k * cpb + ci) * L + m];
                double ire = d0.x, iim = d0.y, pre = 0.0, pim = 0.0;
                double2 *ac = acc + (size_t)hidx(m, m) * cpb + ci;
                ac->x += ire;
                ac->y += iim;
                for (int l = m + 1; l < L; ++l) {
                    const double az = c_rec_a[l * KMC_LMAX + m] * zr;
                    const double br = c_rec_b[l * KMC_LMAX + m] * ri2;
                    const double nre = az * ire - br * pre;
                    const double nim = az * iim - br * pim;
                    pre = ire;
                    pim = iim;
                    ire = nre;
                    iim = nim;
                    double2 *a2 = acc + (size_t)hidx(l, m) * cpb + ci;
                    a2->x += ire;
                    a2->y += iim;
                }
            }
        }
    }
    __syncthreads();
    for (int k = tid; k < NH * cpb; k += nthr) {
        const int h = k / cpb, c = blockIdx.x * cpb + (k % cpb);
        if (c < S.ncell) {
            double2 *dst = S.lexp + (size_t)c * NH + h;
            const double2 a = acc[k];
            dst->x += a.x;
            dst->y += a.y;
        }
    }
}

// Double-FP32 variant of the accept particle-to-local (KMC_PREC_MIXED): same
// per-(cell, m) chains as k_p2l<0>, every product and sum in df32 (~48-bit
// significand).  Sources are split into blockDim.z groups of L so that more
// warps run per SM; group partial sums are reduced in a fixed order and added
// to the FP64 master expansions in FP64.
__global__ void k_p2l_df(Sys S, const AcceptRec *rec, const int nsrc)
{
    if (rec->skip) return;
    extern __shared__ float4 dfsm[];
    const int cpb = blockDim.x, G = blockDim.z;
    const int NH = S.NH, L = S.L;
    const int SC = G * L;  // sources per chunk
    float4 *acc = dfsm;                                   // [G][NH][cpb] (re hi, im hi, re lo, im lo)
    float4 *gd = acc + (size_t)G * NH * cpb;              // [SC][cpb][L] diagonal
    float2 *gz = reinterpret_cast<float2 *>(gd + (size_t)SC * cpb * L);  // [SC][cpb] z / r^2
    float2 *gr = gz + (size_t)SC * cpb;                                  // [SC][cpb] 1 / r^2 (hi 0 = skip)
    const int ci = threadIdx.x, m = threadIdx.y, grp = threadIdx.z;
    const int tid = (threadIdx.z * blockDim.y + threadIdx.y) * blockDim.x + threadIdx.x;
    const int nthr = blockDim.x * blockDim.y * blockDim.z;
    for (int k = tid; k < G * NH * cpb; k += nthr) acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 *myacc = acc + (size_t)grp * NH * cpb;
    for (int s0 = 0; s0 < nsrc; s0 += SC) {
        const int ns = min(SC, nsrc - s0);
        __syncthreads();
        {
            // phase A: one (cell, source) pair per thread: source index grp*L + m of the chunk
            const int sidx = grp * L + m, pc = ci;
            const int cell = blockIdx.x * cpb + pc;
            float2 *zr_out = gz + (size_t)sidx * cpb + pc;
            float2 *r2_out = gr + (size_t)sidx * cpb + pc;
            *r2_out = make_float2(0.f, 0.f);
            if (sidx < ns && cell < S.ncell) {
                const Src v = make_src(S, rec, 0, s0 + sidx);
                const int fx = cell % S.n, fy = (cell / S.n) % S.n, fz = cell / (S.n * S.n);
                const bool near = abs(v.tx - fx) < 2 && abs(v.ty - fy) < 2 && abs(v.tz - fz) < 2;
                if (!near) {
                    const df32 dx = df_from_double(v.x - cell_centre(S, fx));
                    const df32 dy = df_from_double(v.y - cell_centre(S, fy));
                    const df32 dz = df_from_double(v.z - cell_centre(S, fz));
                    const df32 r2 = df_add(df_add(df_mul(dx, dx), df_mul(dy, dy)), df_mul(dz, dz));
                    const df32 ri = df_rsqrt(r2);
                    const df32 rin = df_add(df_make(ri.hi, 0.f), df_make(ri.lo, 0.f));
                    const df32 ri2 = df_mul(rin, rin);
                    const df32 wre = df_mul(dx, ri2), wim = df_mul(df_make(-dy.hi, -dy.lo), ri2);
                    df32 ire = df_mul(df_from_double(v.q), rin), iim = df_make(0.f, 0.f);
                    float4 *dg = gd + ((size_t)sidx * cpb + pc) * L;
                    dg[0] = make_float4(ire.hi, iim.hi, ire.lo, iim.lo);
                    for (int k2 = 1; k2 < L; ++k2) {
                        const float2 t2 = c_rec_d2[k2];
                        const df32 t = df_make(t2.x, t2.y);
                        const df32 nre = df_mul(t, df_sub(df_mul(ire, wre), df_mul(iim, wim)));
                        const df32 nim = df_mul(t, df_add(df_mul(ire, wim), df_mul(iim, wre)));
                        ire = nre;
                        iim = nim;
                        dg[k2] = make_float4(ire.hi, iim.hi, ire.lo, iim.lo);
                    }
                    const df32 zr = df_mul(dz, ri2);
                    *zr_out = make_float2(zr.hi, zr.lo);
                    *r2_out = make_float2(ri2.hi, ri2.lo);
                }
            }
        }
        __syncthreads();
        // phase B: thread (cell, m, group) runs its m-chain for the group's L sources
        const int cell = blockIdx.x * cpb + ci;
        if (cell < S.ncell) {
            for (int k = grp * L; k < min((grp + 1) * L, ns); ++k) {
                const float2 r2f = gr[(size_t)k * cpb + ci];
                if (r2f.x == 0.f) continue;
                const df32 ri2 = df_make(r2f.x, r2f.y);
                const float2 zf = gz[(size_t)k * cpb + ci];
                const df32 zr = df_make(zf.x, zf.y);
                const float4 d0 = gd[((size_t)k * cpb + ci) * L + m];
                df32 ire = df_make(d0.x, d0.z), iim = df_make(d0.y, d0.w);
                df32 pre = df_make(0.f, 0.f), pim = df_make(0.f, 0.f);
                {
                    float4 *ac = myacc + (size_t)hidx(m, m) * cpb + ci;
                    df32 ar = df_make(ac->x, ac->z), ai = df_make(ac->y, ac->w);
                    df_acc(ar, ire);
                    df_acc(ai, iim);
                    *ac = make_float4(ar.hi, ai.hi, ar.lo, ai.lo);
                }
                for (int l = m + 1; l < L; ++l) {
                    const float2 a2 = c_rec_a2[l * KMC_LMAX + m], b2 = c_rec_b2[l * KMC_LMAX + m];
                    const df32 az = df_mul(df_make(a2.x, a2.y), zr);
                    const df32 br = df_mul(df_make(b2.x, b2.y), ri2);
                    const df32 nre = df_sub(df_mul(az, ire), df_mul(br, pre));
                    const df32 nim = df_sub(df_mul(az, iim), df_mul(br, pim));
                    pre = ire;
                    pim = iim;
                    ire = nre;
                    iim = nim;
                    float4 *a4 = myacc + (size_t)hidx(l, m) * cpb + ci;
                    df32 ar = df_make(a4->x, a4->z), ai = df_make(a4->y, a4->w);
                    df_acc(ar, ire);
                    df_acc(ai, iim);
                    *a4 = make_float4(ar.hi, ai.hi, ar.lo, ai.lo);
                }
            }
        }
    }
    __syncthreads();
    for (int k = tid; k < NH * cpb; k += nthr) {
        const int h = k / cpb, c = blockIdx.x * cpb + (k % cpb);
        if (c < S.ncell) {
            double re = 0.0, im = 0.0;
            for (int g2 = 0; g2 < G; ++g2) {
                const float4 a = acc[(size_t)g2 * NH * cpb + k];
                re += (double)a.x + (double)a.z;
                im += (double)a.y + (double)a.w;
            }
            double2 *dst = S.lexp + (size_t)c * NH + h;
            dst->x += re;
            dst->y += im;
        }
    }
}

// Double-FP32 accept P2L, register form.  Block = 16 cells x L columns x G
// source groups; thread (cell, m, group) keeps the column's L - m accumulators
// in registers and runs the scaled recurrence (c_p2l_beta) for its group's
// sources in cell-width units; the groups are summed in FP64 in a fixed order,
// scaled by C_lm w^{-l-1} and added to the FP64 local expansions.  Per chunk of
// up to kP2lChunk sources, the (cell, source) geometry is formed once in
// shared memory: r^-2, z r^-2, (x - i y) r^-2 and q r^-1, all double-FP32.
constexpr int kP2lCells = 16;
constexpr int kP2lChunk = 64;

size_t p2l_df2_smem(const int L, const int NH, const int G)
{
    const size_t geo = 5 * (size_t)kP2lChunk * kP2lCells * sizeof(float2) + (size_t)kP2lChunk * 4 * sizeof(float2) +
                       (size_t)kP2lChunk * 3 * sizeof(int);
    const size_t red = (size_t)(G > 1 ? G - 1 : 0) * NH * kP2lCells * sizeof(float4);
    (void)L;
    return geo > red ? geo : red;
}

constexpr int kP2lFp32From = 6;  // default first FP32 order of the double-FP32 accept

// One chunk of sources into shared memory for the P2L kernels: the sources split
// once to double-FP32 cell-width coordinates (relative to the centre of cell 0) and
// charge, then per (source, cell of the block) r^-2, z r^-2, (x - i y) r^-2 and
// q r^-1 in double-FP32; r^-2 = 0 marks a pair inside the near field.  Every thread
// of the block calls it (it holds the block's barriers).
__device__ __forceinline__ void p2l_chunk_geometry(const Sys &S, const AcceptRec *rec, const int s0, const int ns,
                                                   const int tid, const int nthr, float2 *g_ri2, float2 *g_zr,
                                                   float2 *g_wre, float2 *g_wim, float2 *g_qri, float2 *s_pos,
                                                   int *s_cell)
{
    __syncthreads();
    for (int k = tid; k < ns; k += nthr) {
        const Src v = make_src(S, rec, 0, s0 + k);
        const df32 ux = df_from_double((v.x + 0.5 * S.E) * S.inv_w - 0.5);
        const df32 uy = df_from_double((v.y + 0.5 * S.E) * S.inv_w - 0.5);
        const df32 uz = df_from_double((v.z + 0.5 * S.E) * S.inv_w - 0.5);
        const df32 uq = df_from_double(v.q);
        s_pos[k] = make_float2(ux.hi, ux.lo);
        s_pos[kP2lChunk + k] = make_float2(uy.hi, uy.lo);
        s_pos[2 * kP2lChunk + k] = make_float2(uz.hi, uz.lo);
        s_pos[3 * kP2lChunk + k] = make_float2(uq.hi, uq.lo);
        s_cell[k] = v.tx;
        s_cell[kP2lChunk + k] = v.ty;
        s_cell[2 * kP2lChunk + k] = v.tz;
    }
    __syncthreads();
    for (int k = tid; k < ns * kP2lCells; k += nthr) {
        const int sidx = k / kP2lCells, pc = k % kP2lCells;
        const int c = blockIdx.x * kP2lCells + pc;
        float2 ri2o = make_float2(0.f, 0.f);
        if (c < S.ncell) {
            const int fx = c % S.n, fy = (c / S.n) % S.n, fz = c / (S.n * S.n);
            const bool near = abs(s_cell[sidx] - fx) < 2 && abs(s_cell[kP2lChunk + sidx] - fy) < 2 &&
                              abs(s_cell[2 * kP2lChunk + sidx] - fz) < 2;
            if (!near) {
                const float2 sx = s_pos[sidx], sy = s_pos[kP2lChunk + sidx], sz = s_pos[2 * kP2lChunk + sidx];
                const df32 dx = df_add(df_make(sx.x, sx.y), df_make(-(float)fx, 0.f));
                const df32 dy = df_add(df_make(sy.x, sy.y), df_make(-(float)fy, 0.f));
                const df32 dz = df_add(df_make(sz.x, sz.y), df_make(-(float)fz, 0.f));
                const df32 r2 = df_add(df_add(df_mul(dx, dx), df_mul(dy, dy)), df_mul(dz, dz));
                const df32 ri0 = df_rsqrt(r2);
                float rh, rl;
                two_sum(ri0.hi, ri0.lo, rh, rl);
                const df32 ri = df_make(rh, rl);
                const df32 ri2 = df_mul(ri, ri);
                const df32 zr = df_mul(dz, ri2), wre = df_mul(dx, ri2), wim = df_mul(df_make(-dy.hi, -dy.lo), ri2);
                const float2 sq = s_pos[3 * kP2lChunk + sidx];
                const df32 qri = df_mul(df_make(sq.x, sq.y), ri);
                ri2o = make_float2(ri2.hi, ri2.lo);
                g_zr[k] = make_float2(zr.hi, zr.lo);
                g_wre[k] = make_float2(wre.hi, wre.lo);
                g_wim[k] = make_float2(wim.hi, wim.lo);
                g_qri[k] = make_float2(qri.hi, qri.lo);
            }
        }
        g_ri2[k] = ri2o;
    }
    __syncthreads();
}


// group 0: the groups' sums added in double-FP32 in a fixed order (on the FP32
// pipe: GB300 issues FP64 at a small fraction of the FP32 rate), converted once,
// scaled by C_lm w^(-l-1) and added to the FP64 local expansions; the near field's
// FP32-pair copy written alongside
__device__ __forceinline__ void p2p_commit(const Sys &S, const float4 *red, const int G, const int cell,
                                           const int ci, const int l, const int m, float hr, float hi, float lr,
                                           float li, const double wp)
{
    const int h = hidx(l, m);
    for (int g2 = 0; g2 < G - 1; ++g2) {
        const float4 v = red[((size_t)g2 * S.NH + h) * kP2lCells + ci];
        float sr, er, si, ei;
        two_sum(hr, v.x, sr, er);
        two_sum(hi, v.y, si, ei);
        hr = sr;
        hi = si;
        lr += er + v.z;
        li += ei + v.w;
    }
    const double re = (double)hr + (double)lr, im = (double)hi + (double)li;
    const double sc = c_p2l_scale[l * KMC_LMAX + m] * wp;
    double2 *dst = S.lexp + (size_t)cell * S.NH + h;
    const double2 nv = make_double2(dst->x + re * sc, dst->y + im * sc);
    *dst = nv;
    const df32 cr = df_from_double(nv.x), cim = df_from_double(nv.y);
    S.lexp32[(size_t)cell * S.NH + h] = make_float4(cr.hi, cim.hi, cr.lo, cim.lo);
}

template <int LT>
__global__ void __launch_bounds__(LT <= 12 ? 384 : 512, LT <= 12 ? 2 : 1) k_p2l_df2(Sys S, const AcceptRec *rec, const int nsrc,
                                                                                    const int ld)
{
    if (rec->skip) return;
    extern __shared__ float4 p2sm[];
    const int L = S.L, NH = S.NH, G = blockDim.z;
    float2 *g_ri2 = reinterpret_cast<float2 *>(p2sm);            // [kP2lChunk][kP2lCells] each
    float2 *g_zr = g_ri2 + kP2lChunk * kP2lCells;
    float2 *g_wre = g_zr + kP2lChunk * kP2lCells;
    float2 *g_wim = g_wre + kP2lChunk * kP2lCells;
    float2 *g_qri = g_wim + kP2lChunk * kP2lCells;
    // sources in cell-width units relative to the centre of cell 0, and charge, as df32
    // (split once per source here, so the (cell, source) set-up runs on the FP32 pipe)
    float2 *s_pos = g_qri + kP2lChunk * kP2lCells;                              // [4][kP2lChunk]
    int *s_cell = reinterpret_cast<int *>(s_pos + 4 * kP2lChunk);               // [3][kP2lChunk]
    const int ci = threadIdx.x, m = threadIdx.y, grp = threadIdx.z;
    const int tid = threadIdx.x + kP2lCells * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthr = kP2lCells * blockDim.y * blockDim.z;
    const int cell = blockIdx.x * kP2lCells + ci;

    float ahr[LT], alr[LT], ahi[LT], ali[LT];
#pragma unroll
    for (int j = 0; j < LT; ++j) ahr[j] = alr[j] = ahi[j] = ali[j] = 0.0f;

    for (int s0 = 0; s0 < nsrc; s0 += kP2lChunk) {
        const int ns = min(kP2lChunk, nsrc - s0);
        p2l_chunk_geometry(S, rec, s0, ns, tid, nthr, g_ri2, g_zr, g_wre, g_wim, g_qri, s_pos, s_cell);
        if (cell < S.ncell) {
            for (int k = grp; k < ns; k += G) {
                const int b = k * kP2lCells + ci;
                const float2 r2f = g_ri2[b];
                if (r2f.x == 0.f) continue;
                const df32 ri2 = df_make(r2f.x, r2f.y);
                const float2 zf = g_zr[b];
                const df32 zr = df_make(zf.x, zf.y);
                df32 jre, jim;
                if (m >= ld) {
                    // the whole column in FP32
                    const float2 q2 = g_qri[b], wr2 = g_wre[b], wi2 = g_wim[b];
                    float fr = q2.x, fi = 0.0f, pr = 0.0f, pi = 0.0f;
                    for (int t = 0; t < m; ++t) {
                        const float nr = fmaf(fr, wr2.x, -fi * wi2.x), ni = fmaf(fr, wi2.x, fi * wr2.x);
                        fr = nr;
                        fi = ni;
                    }
                    ahr[0] += fr;
                    ahi[0] += fi;
#pragma unroll
                    for (int j = 1; j < LT; ++j) {
                        if (m + j < L) {
                            const float br = c_p2l_beta[(m + j) * KMC_LMAX + m].x * r2f.x;
                            const float nr = fmaf(zf.x, fr, -br * pr), ni = fmaf(zf.x, fi, -br * pi);
                            pr = fr;
                            pi = fi;
                            fr = nr;
                            fi = ni;
                            ahr[j] += fr;
                            ahi[j] += fi;
                        }
                    }
                    continue;
                }
                {
                    const float2 q2 = g_qri[b], wr2 = g_wre[b], wi2 = g_wim[b];
                    const df32 wre = df_make(wr2.x, wr2.y), wim = df_make(wi2.x, wi2.y);
                    jre = df_make(q2.x, q2.y);
                    jim = df_make(0.f, 0.f);
                    for (int t = 0; t < m; ++t) {
                        const df32 nre = df_fms(jre, wre, jim, wim);
                        const df32 nim = df_fma2(jre, wim, jim, wre);
                        jre = nre;
                        jim = nim;
                    }
                }
                {
                    float s, e;
                    two_sum(ahr[0], jre.hi, s, e);
                    ahr[0] = s;
                    alr[0] += e + jre.lo;
                    two_sum(ahi[0], jim.hi, s, e);
                    ahi[0] = s;
                    ali[0] += e + jim.lo;
                }
                df32 pre = df_make(0.f, 0.f), pim = df_make(0.f, 0.f);
#pragma unroll
                for (int j = 1; j < LT; ++j) {
                    if (m + j < L && m + j >= ld) {
                        // orders from ld on in FP32, continuing from the double-FP32 high words
                        const float br = c_p2l_beta[(m + j) * KMC_LMAX + m].x * r2f.x;
                        const float nr = fmaf(zf.x, jre.hi, -br * pre.hi), ni = fmaf(zf.x, jim.hi, -br * pim.hi);
                        pre = jre;
                        pim = jim;
                        jre = df_make(nr, 0.f);
                        jim = df_make(ni, 0.f);
                        ahr[j] += nr;
                        ahi[j] += ni;
                    } else if (m + j < L) {
                        const float2 bt = c_p2l_beta[(m + j) * KMC_LMAX + m];
                        const df32 br = df_mul(df_make(bt.x, bt.y), ri2);
                        const df32 nre = df_fms(zr, jre, br, pre);
                        const df32 nim = df_fms(zr, jim, br, pim);
                        pre = jre;
                        pim = jim;
                        jre = nre;
                        jim = nim;
                        float s, e;
                        two_sum(ahr[j], jre.hi, s, e);
                        ahr[j] = s;
                        alr[j] += e + jre.lo;
                        two_sum(ahi[j], jim.hi, s, e);
                        ahi[j] = s;
                        ali[j] += e + jim.lo;
                    }
                }
            }
        }
    }
    // groups 1..G-1 hand their sums to group 0 through shared memory
    __syncthreads();
    float4 *red = p2sm;  // [G-1][NH][kP2lCells]
    if (grp > 0) {
#pragma unroll
        for (int j = 0; j < LT; ++j)
            if (m + j < L)
                red[((size_t)(grp - 1) * NH + hidx(m + j, m)) * kP2lCells + ci] =
                    make_float4(ahr[j], ahi[j], alr[j], ali[j]);
    }
    __syncthreads();
    if (grp == 0 && cell < S.ncell) {
        double wp = S.inv_w;
        for (int t = 0; t < m; ++t) wp *= S.inv_w;
#pragma unroll
        for (int j = 0; j < LT; ++j) {
            if (m + j < L) {
                // the near field's FP32-pair copy is written here too (no separate refresh)
                p2p_commit(S, red, G, cell, ci, m + j, m, ahr[j], ahi[j], alr[j], ali[j], wp);
            }
            wp *= S.inv_w;
        }
    }
}

// Column-pair form of the double-FP32 accept P2L for L = 12 with orders from 6 in
// FP32 (the default split).  In k_p2l_df2 a thread runs one column m, so the
// threads of columns 0-5 carry all the double-FP32 work and those of 6-11 idle
// beside them, and m is a runtime index.  Here thread (cell, source group, pair P)
// runs column P (double-FP32 to order 5, FP32 above) and column 11 - P (FP32, its
// diagonal continued from column P's), so every thread carries five double-FP32
// steps and 13 coefficients; warps hold one P, and a switch on P runs code in which
// the column, the recurrence constants and the accumulator indices are compile-time.
constexpr int kP2pL = 12, kP2pLd = 6, kP2pPairs = kP2pL / 2;

struct P2pAcc {
    float ahr[kP2pL], ahi[kP2pL];          // column P by order, high words
    float alr[kP2pLd], ali[kP2pLd];        // column P, low words of the double-FP32 orders
    float bhr[kP2pL - kP2pLd], bhi[kP2pL - kP2pLd];  // column 11 - P by order - 6
};

__device__ __forceinline__ void p2p_acc_df(float &h, float &l, const df32 v)
{
    float s, e;
    two_sum(h, v.hi, s, e);
    h = s;
    l += e + v.lo;
}

template <int P>
__device__ __forceinline__ void p2p_chunk(P2pAcc &a, const float2 *g_ri2, const float2 *g_zr, const float2 *g_wre,
                                          const float2 *g_wim, const float2 *g_qri, const int ns, const int ci,
                                          const int grp, const int G)
{
    constexpr int B = kP2pL - 1 - P;
    static_assert(P < kP2pLd && B >= kP2pLd, "column pair split");
    for (int k = grp; k < ns; k += G) {
        const int b = k * kP2lCells + ci;
        const float2 r2f = g_ri2[b];
        if (r2f.x == 0.f) continue;
        const float2 zf = g_zr[b], wr2 = g_wre[b], wi2 = g_wim[b], q2 = g_qri[b];
        const df32 ri2 = df_make(r2f.x, r2f.y), zr = df_make(zf.x, zf.y);
        const df32 wre = df_make(wr2.x, wr2.y), wim = df_make(wi2.x, wi2.y);
        // column P: the diagonal q r^-1 w^P, w = (x - i y) r^-2, then up in order
        df32 jre = df_make(q2.x, q2.y), jim = df_make(0.f, 0.f);
#pragma unroll 1
        for (int t = 0; t < P; ++t) {  // kept rolled: the six columns' code shares the instruction cache
            const df32 nre = df_fms(jre, wre, jim, wim);
            const df32 nim = df_fma2(jre, wim, jim, wre);
            jre = nre;
            jim = nim;
        }
        float cr = jre.hi, cim = jim.hi;  // seeds column B's diagonal
        p2p_acc_df(a.ahr[P], a.alr[P], jre);
        p2p_acc_df(a.ahi[P], a.ali[P], jim);
        df32 pre = df_make(0.f, 0.f), pim = df_make(0.f, 0.f);
#pragma unroll
        for (int l = P + 1; l < kP2pLd; ++l) {
            const float2 bt = c_p2l_beta[l * KMC_LMAX + P];
            const df32 br = df_mul(df_make(bt.x, bt.y), ri2);
            const df32 nre = df_fms(zr, jre, br, pre), nim = df_fms(zr, jim, br, pim);
            pre = jre;
            pim = jim;
            jre = nre;
            jim = nim;
            p2p_acc_df(a.ahr[l], a.alr[l], jre);
            p2p_acc_df(a.ahi[l], a.ali[l], jim);
        }
        // orders from 6 in FP32, continuing from the double-FP32 high words
        float fr = jre.hi, fi = jim.hi, gr = pre.hi, gi = pim.hi;
#pragma unroll
        for (int l = kP2pLd; l < kP2pL; ++l) {
            const float br = c_p2l_beta[l * KMC_LMAX + P].x * r2f.x;
            const float nr = fmaf(zf.x, fr, -br * gr), ni = fmaf(zf.x, fi, -br * gi);
            gr = fr;
            gi = fi;
            fr = nr;
            fi = ni;
            a.ahr[l] += fr;
            a.ahi[l] += fi;
        }
        // column B in FP32: diagonal w^B from column P's, then up in order
#pragma unroll 1
        for (int t = P; t < B; ++t) {
            const float nr = fmaf(cr, wr2.x, -cim * wi2.x), ni = fmaf(cr, wi2.x, cim * wr2.x);
            cr = nr;
            cim = ni;
        }
        a.bhr[B - kP2pLd] += cr;
        a.bhi[B - kP2pLd] += cim;
        float hr = 0.f, hi = 0.f;
#pragma unroll
        for (int l = B + 1; l < kP2pL; ++l) {
            const float br = c_p2l_beta[l * KMC_LMAX + B].x * r2f.x;
            const float nr = fmaf(zf.x, cr, -br * hr), ni = fmaf(zf.x, cim, -br * hi);
            hr = cr;
            hi = cim;
            cr = nr;
            cim = ni;
            a.bhr[l - kP2pLd] += cr;
            a.bhi[l - kP2pLd] += cim;
        }
    }
}

// a thread's sums (both columns) to shared memory, [group][cell][NH] (low words 0
// for the FP32 orders)
template <int P>
__device__ __forceinline__ void p2p_stash(const P2pAcc &a, float4 *red, const int grp, const int NH, const int ci)
{
    constexpr int B = kP2pL - 1 - P;
    float4 *dst = red + ((size_t)grp * kP2lCells + ci) * NH;
#pragma unroll
    for (int l = P; l < kP2pL; ++l)
        dst[hidx(l, P)] = make_float4(a.ahr[l], a.ahi[l], l < kP2pLd ? a.alr[l] : 0.f, l < kP2pLd ? a.ali[l] : 0.f);
#pragma unroll
    for (int l = B; l < kP2pL; ++l) dst[hidx(l, B)] = make_float4(a.bhr[l - kP2pLd], a.bhi[l - kP2pLd], 0.f, 0.f);
}

#define P2P_SWITCH(CALL)       \
    switch (pp) {              \
    case 0: CALL(0); break;    \
    case 1: CALL(1); break;    \
    case 2: CALL(2); break;    \
    case 3: CALL(3); break;    \
    case 4: CALL(4); break;    \
    default: CALL(5); break;   \
    }

// block (kP2lCells cells, G source groups, 6 pairs); G even keeps one pair per warp
template <int G>
__global__ void __launch_bounds__(kP2lCells * G * kP2pPairs, 768 / (kP2lCells * G * kP2pPairs))
    k_p2l_pair(Sys S, const AcceptRec *rec, const int nsrc)
{
    static_assert(G % 2 == 0 && kP2lCells == 16, "one pair per warp");
    if (rec->skip) return;
    extern __shared__ float4 p2sm[];
    float2 *g_ri2 = reinterpret_cast<float2 *>(p2sm);
    float2 *g_zr = g_ri2 + kP2lChunk * kP2lCells;
    float2 *g_wre = g_zr + kP2lChunk * kP2lCells;
    float2 *g_wim = g_wre + kP2lChunk * kP2lCells;
    float2 *g_qri = g_wim + kP2lChunk * kP2lCells;
    float2 *s_pos = g_qri + kP2lChunk * kP2lCells;
    int *s_cell = reinterpret_cast<int *>(s_pos + 4 * kP2lChunk);
    const int ci = threadIdx.x, grp = threadIdx.y, pp = threadIdx.z;
    const int tid = threadIdx.x + kP2lCells * (threadIdx.y + G * threadIdx.z);
    const int nthr = kP2lCells * G * kP2pPairs;
    const int cell = blockIdx.x * kP2lCells + ci;
    P2pAcc a;
#pragma unroll
    for (int l = 0; l < kP2pL; ++l) a.ahr[l] = a.ahi[l] = 0.f;
#pragma unroll
    for (int l = 0; l < kP2pLd; ++l) a.alr[l] = a.ali[l] = 0.f;
#pragma unroll
    for (int l = 0; l < kP2pL - kP2pLd; ++l) a.bhr[l] = a.bhi[l] = 0.f;
    for (int s0 = 0; s0 < nsrc; s0 += kP2lChunk) {
        const int ns = min(kP2lChunk, nsrc - s0);
        p2l_chunk_geometry(S, rec, s0, ns, tid, nthr, g_ri2, g_zr, g_wre, g_wim, g_qri, s_pos, s_cell);
        if (cell < S.ncell) {
#define P2P_CHUNK(K) p2p_chunk<K>(a, g_ri2, g_zr, g_wre, g_wim, g_qri, ns, ci, grp, G)
            P2P_SWITCH(P2P_CHUNK)
#undef P2P_CHUNK
        }
    }
    __syncthreads();
    float4 *red = p2sm;  // [G][kP2lCells][NH]
    if (cell < S.ncell) {
#define P2P_STASH(K) p2p_stash<K>(a, red, grp, S.NH, ci)
        P2P_SWITCH(P2P_STASH)
#undef P2P_STASH
    }
    __syncthreads();
    // every thread commits (cell, coefficient) items, coefficients of a cell adjacent:
    // the groups' sums in double-FP32 in a fixed order (FP32 pipe), one conversion,
    // scaled and added to the FP64 expansion, the FP32-pair copy alongside
    const int NH = S.NH;
    for (int k = tid; k < kP2lCells * NH; k += nthr) {
        const int c = k / NH, h = k - c * NH, cl = blockIdx.x * kP2lCells + c;
        if (cl >= S.ncell) break;
        float hr = 0.f, hi = 0.f, lr = 0.f, li = 0.f;
        for (int g2 = 0; g2 < G; ++g2) {
            const float4 v = red[((size_t)g2 * kP2lCells + c) * NH + h];
            float sr, er, si, ei;
            two_sum(hr, v.x, sr, er);
            two_sum(hi, v.y, si, ei);
            hr = sr;
            hi = si;
            lr += er + v.z;
            li += ei + v.w;
        }
        const double sc = __ldg(&S.p2lsc[h]);
        const double re = (double)hr + (double)lr, im = (double)hi + (double)li;
        double2 *dst = S.lexp + (size_t)cl * NH + h;
        const double2 nv = make_double2(dst->x + re * sc, dst->y + im * sc);
        *dst = nv;
        const df32 cr = df_from_double(nv.x), cim = df_from_double(nv.y);
        S.lexp32[(size_t)cl * NH + h] = make_float4(cr.hi, cim.hi, cr.lo, cim.lo);
    }
}
#undef P2P_SWITCH

// ---------------------------------------------------------------------------
// FP64 accept particle-to-local in column pairs (precision fp64 and the mixed
// mode with FP64 accept contributions; accept_local_exp, kmc_octal.py:961-1089):
// every product and sum in FP64.  GB300 issues an FP64 warp instruction far less
// often than an FP32 one, so the kernel spends as few FP64 operations per
// (cell, source image) as the recurrence allows and keeps the FP64 pipe fed:
//  * scaled irregular recurrence J_l = (z/r^2) J_{l-1} - beta_lm r^-2 J_{l-2}
//    (one coefficient product per step; the scale C_lm w^-(l+1) is applied once
//    per output coefficient, not per source), coordinates in cell widths;
//  * the geometry of each (cell, source) -- z/r^2, 1/r^2 and the diagonal
//    J_m^m = (q/r) w^m, w = (x - i y)/r^2, for every m -- is formed once per
//    block in shared memory and shared by the column pairs;
//  * a thread owns the column pair (P, LT-1-P) of one cell for one group of
//    sources: LT+1 orders per source for every thread (balanced), accumulated in
//    registers (no shared-memory read-modify-write per step);
//  * a warp is one column pair over CPB cells x (32 / CPB) source groups, so the
//    compile-time pair index is warp-uniform; few cells per block give many
//    short blocks (several waves over the SMs, small tail);
//  * the groups' sums meet in shared memory and every thread commits (cell,
//    coefficient) items in a fixed group order.
// Block (CPB cells, 32 / CPB groups, LT/2 pairs).
// ---------------------------------------------------------------------------
__constant__ double c_p2l_beta64[KMC_LMAX * KMC_LMAX];
constexpr int kP64Groups = 16;  // source groups of k_p2l64 (sources g, g + 16, ... per group)

template <int LT, int P>
struct P64Acc {
    double ar[LT - P], ai[LT - P];  // column P, orders P .. LT-1
    double br[P + 1], bi[P + 1];    // column LT-1-P, orders LT-1-P .. LT-1
};

// one (cell, source) item's geometry: z / r^2, 1 / r^2 (0: not well separated) and
// the diagonal J_m^m for m < LT, padded to LT + 1 entries
template <int LT>
struct P64Geo {
    static constexpr int kStride = LT + 1;  // double2 per item (diagonal; [LT] holds (z/r^2, 1/r^2))
};

template <int LT, int P>
__device__ __forceinline__ void p64_pair(P64Acc<LT, P> &a, const double2 *__restrict__ geo, const int ns,
                                         const int ci, const int cpb, const int grp, const int G)
{
    constexpr int B = LT - 1 - P;
    constexpr int ST = P64Geo<LT>::kStride;
#pragma unroll
    for (int l = 0; l < LT - P; ++l) a.ar[l] = a.ai[l] = 0.0;
#pragma unroll
    for (int l = 0; l <= P; ++l) a.br[l] = a.bi[l] = 0.0;
    for (int k = grp; k < ns; k += G) {
        const double2 *it = geo + ((size_t)k * cpb + ci) * ST;
        const double2 zg = it[LT];
        const double zr = zg.x, ri2 = zg.y;
        if (ri2 == 0.0) continue;
        double2 d = it[P];
        double jre = d.x, jim = d.y, pre = 0.0, pim = 0.0;
        a.ar[0] += jre;
        a.ai[0] += jim;
#pragma unroll
        for (int l = P + 1; l < LT; ++l) {
            const double br = c_p2l_beta64[l * KMC_LMAX + P] * ri2;
            const double nre = fma(zr, jre, -br * pre), nim = fma(zr, jim, -br * pim);
            pre = jre;
            pim = jim;
            jre = nre;
            jim = nim;
            a.ar[l - P] += jre;
            a.ai[l - P] += jim;
        }
        d = it[B];
        jre = d.x;
        jim = d.y;
        pre = 0.0;
        pim = 0.0;
        a.br[0] += jre;
        a.bi[0] += jim;
#pragma unroll
        for (int l = B + 1; l < LT; ++l) {
            const double br = c_p2l_beta64[l * KMC_LMAX + B] * ri2;
            const double nre = fma(zr, jre, -br * pre), nim = fma(zr, jim, -br * pim);
            pre = jre;
            pim = jim;
            jre = nre;
            jim = nim;
            a.br[l - B] += jre;
            a.bi[l - B] += jim;
        }
    }
}

template <int LT, int P>
__device__ __forceinline__ void p64_stash(const P64Acc<LT, P> &a, double2 *red, const int NH)
{
    constexpr int B = LT - 1 - P;
#pragma unroll
    for (int l = P; l < LT; ++l) red[hidx(l, P)] = make_double2(a.ar[l - P], a.ai[l - P]);
#pragma unroll
    for (int l = B; l < LT; ++l) red[hidx(l, B)] = make_double2(a.br[l - B], a.bi[l - B]);
}

template <int LT, int P>
__device__ __forceinline__ void p64_run(const double2 *geo, const int ns, const int ci, const int cpb, const int grp,
                                        const int G, double2 *red, const int NH, const bool active)
{
    P64Acc<LT, P> a;
    if (active) p64_pair<LT, P>(a, geo, ns, ci, cpb, grp, G);
    __syncthreads();  // every thread has read the geometry: the reduction area may overwrite it
    if (active) p64_stash<LT, P>(a, red + ((size_t)grp * cpb + ci) * NH, NH);
}

template <int LT>
__global__ void __launch_bounds__(kP64Groups * (LT <= 12 ? 8 : 4) * (LT / 2)) k_p2l64(Sys S, const AcceptRec *rec, const int nsrc)
{
    static_assert(LT % 2 == 0 && LT >= 4 && LT <= 16, "column pairs of an even order");
    constexpr int ST = P64Geo<LT>::kStride;
    if (rec->skip) return;
    extern __shared__ double2 p64sm[];
    const int cpb = blockDim.x, G = blockDim.y;
    const int ci = threadIdx.x, grp = threadIdx.y, pp = threadIdx.z;
    const int tid = threadIdx.x + cpb * (threadIdx.y + G * threadIdx.z);
    const int nthr = cpb * G * (LT / 2);
    const int NH = S.NH;
    double2 *geo = p64sm;   // [nsrc][cpb][ST]
    double2 *red = p64sm;   // [G][cpb][NH], after the pairs are done with the geometry
    // geometry of every (source, cell) item: the sources' images in cell widths, the
    // well-separated rule (neighbour cells get nothing), the diagonal chain
    for (int k = tid; k < nsrc * cpb; k += nthr) {
        const int sidx = k / cpb, pc = k - sidx * cpb;
        const int c = blockIdx.x * cpb + pc;
        double2 *it = geo + (size_t)k * ST;
        double zr = 0.0, ri2 = 0.0;
        if (c < S.ncell) {
            const Src v = make_src(S, rec, 0, sidx);
            const int fx = c % S.n, fy = (c / S.n) % S.n, fz = c / (S.n * S.n);
            if (!(abs(v.tx - fx) < 2 && abs(v.ty - fy) < 2 && abs(v.tz - fz) < 2)) {
                const double dx = ((v.x + 0.5 * S.E) * S.inv_w - 0.5) - fx;
                const double dy = ((v.y + 0.5 * S.E) * S.inv_w - 0.5) - fy;
                const double dz = ((v.z + 0.5 * S.E) * S.inv_w - 0.5) - fz;
                const double ri = rsqrt(dx * dx + dy * dy + dz * dz);
                ri2 = ri * ri;
                zr = dz * ri2;
                const double wre = dx * ri2, wim = -dy * ri2;
                double jre = v.q * ri, jim = 0.0;
                it[0] = make_double2(jre, jim);
#pragma unroll
                for (int m = 1; m < LT; ++m) {
                    const double nre = fma(jre, wre, -jim * wim), nim = fma(jre, wim, jim * wre);
                    jre = nre;
                    jim = nim;
                    it[m] = make_double2(jre, jim);
                }
            }
        }
        it[LT] = make_double2(zr, ri2);
    }
    __syncthreads();
    const bool active = blockIdx.x * cpb + ci < S.ncell;
#define P64_CASE(K)                                                                                    \
    case K:                                                                                            \
        p64_run<LT, (K < LT / 2 ? K : 0)>(geo, nsrc, ci, cpb, grp, G, red, NH, active && K < LT / 2); \
        break;
    switch (pp) {
        P64_CASE(0)
        P64_CASE(1)
        P64_CASE(2)
        P64_CASE(3)
        P64_CASE(4)
        P64_CASE(5)
        P64_CASE(6)
        P64_CASE(7)
    default: break;
    }
#undef P64_CASE
    __syncthreads();
    for (int k = tid; k < cpb * NH; k += nthr) {
        const int c = k / NH, h = k - c * NH, cl = blockIdx.x * cpb + c;
        if (cl >= S.ncell) break;
        double re = 0.0, im = 0.0;
        for (int g2 = 0; g2 < G; ++g2) {
            const double2 v = red[((size_t)g2 * cpb + c) * NH + h];
            re += v.x;
            im += v.y;
        }
        const double sc = __ldg(&S.p2lsc[h]);
        double2 *dst = S.lexp + (size_t)cl * NH + h;
        const double2 nv = make_double2(fma(re, sc, dst->x), fma(im, sc, dst->y));
        *dst = nv;
        if (S.mixed) {
            const df32 cr = df_from_double(nv.x), cim = df_from_double(nv.y);
            S.lexp32[(size_t)cl * NH + h] = make_float4(cr.hi, cim.hi, cr.lo, cim.lo);
        }
    }
}

// shared memory of k_p2l64: the geometry of every (source, cell) item, then the
// groups' sums (the same area)
size_t p2l64_smem(const int L, const int NH, const int cpb, const int nsrc, const int G)
{
    const size_t geo = (size_t)nsrc * cpb * (L + 1) * sizeof(double2);
    const size_t red = (size_t)G * cpb * NH * sizeof(double2);
    return std::max(geo, red);
}

// ---------------------------------------------------------------------------
// The near-field potential of every charge (S.phin) across an accepted move of
// charge k from a (cell co) to b (cell cn).  The old side of a proposal is its
// charge times its potential, near field plus cell expansion (direct_old,
// kmc_local.py:956-1019, recomputed on every propose there); the near-field part
// changes only for the charges whose 27 cells hold co or cn, so it is kept per
// charge and updated here: every other charge j loses q_k / |x_j - a'| for each of
// its neighbour cells (with that cell's periodic shift) that is co, and gains
// q_k / |x_j - b'| for each that is cn; k's potential at b is the sum of q_j over
// those same distances to b (the neighbour relation is symmetric, images
// included).  Blocks 0..26 take the cells around co, 27..53 those around cn (a
// cell listed before is left to its first block), one thread per charge, the
// offsets in a fixed order: each charge is updated once, the same way on every
// run.  k's potential: a fixed-order tree per block, the blocks' partial sums
// added in block order by the last block to finish (a ticket, no waiting).  Runs
// after k_accept_prep (positions and the store final); nothing for a refused or
// skipped accept.
// ---------------------------------------------------------------------------
constexpr int kPhinThreads = 128, kPhinBlocks = 54;

// neighbour cell `o` (0..26, x fastest) of cell (cx, cy, cz) and its periodic shift;
// false where a free-space neighbour does not exist
__device__ __forceinline__ bool nb_cell_shift(const Sys &S, const int cx, const int cy, const int cz, const int o,
                                              int &cell, double &sx, double &sy, double &sz)
{
    int c3[3] = {cx + o % 3 - 1, cy + (o / 3) % 3 - 1, cz + o / 9 - 1};
    double sh[3] = {0.0, 0.0, 0.0};
    for (int t = 0; t < 3; ++t) {
        if (c3[t] < 0) {
            if (!S.periodic) return false;
            c3[t] += S.n;
            sh[t] = -S.E;
        } else if (c3[t] >= S.n) {
            if (!S.periodic) return false;
            c3[t] -= S.n;
            sh[t] = S.E;
        }
    }
    cell = c3[0] + S.n * (c3[1] + S.n * c3[2]);
    sx = sh[0];
    sy = sh[1];
    sz = sh[2];
    return true;
}

__global__ void __launch_bounds__(kPhinThreads) k_phin_move(const Sys S, const AcceptRec *rec, double *part,
                                                            unsigned *ticket)
{
    __shared__ int cand[kPhinBlocks], nbc[27];
    __shared__ double nbs[27][3], red[kPhinThreads];
    __shared__ bool last;
    if (rec->skip) return;
    const int k = rec->pid, co = rec->co, cn = rec->cn, n = S.n;
    const int b = blockIdx.x, t = threadIdx.x;
    const double q = rec->q;
    double sx, sy, sz;
    if (t < kPhinBlocks) {
        const int base = t < 27 ? co : cn;
        int c;
        cand[t] = nb_cell_shift(S, base % n, (base / n) % n, base / (n * n), t % 27, c, sx, sy, sz) ? c : -1;
    }
    __syncthreads();
    const int mine = cand[b];
    bool dup = true;
    if (mine >= 0) dup = __syncthreads_or(t < b && cand[t] == mine);
    double w = 0.0;  // this thread's part of k's potential at b
    if (!dup) {
        if (t < 27) {
            int c;
            nbc[t] = nb_cell_shift(S, mine % n, (mine / n) % n, mine / (n * n), t, c, sx, sy, sz) ? c : -1;
            nbs[t][0] = sx;
            nbs[t][1] = sy;
            nbs[t][2] = sz;
        }
        __syncthreads();
        const int cnt = S.cnt[mine];
        for (int i = t; i < cnt; i += blockDim.x) {
            const size_t a = (size_t)mine * S.cap + i;
            const int j = S.store_pid[a];
            if (j == k) continue;
            const double4_32a v = S.store[a];
            double d = 0.0, u = 0.0;
            for (int o = 0; o < 27; ++o) {
                const int nb = nbc[o];
                if (nb == co) {
                    const double dx = v.x - (rec->xo + nbs[o][0]), dy = v.y - (rec->yo + nbs[o][1]),
                                 dz = v.z - (rec->zo + nbs[o][2]);
                    d -= q * rsqrt(dx * dx + dy * dy + dz * dz);
                }
                if (nb == cn) {
                    const double dx = v.x - (rec->xn + nbs[o][0]), dy = v.y - (rec->yn + nbs[o][1]),
                                 dz = v.z - (rec->zn + nbs[o][2]);
                    const double inv = rsqrt(dx * dx + dy * dy + dz * dz);
                    d += q * inv;
                    u += inv;
                }
            }
            S.phin[j] += d;
            w += v.w * u;
        }
    }
    red[t] = w;
    __syncthreads();
    for (int h = kPhinThreads / 2; h > 0; h >>= 1) {
        if (t < h) red[t] += red[t + h];
        __syncthreads();
    }
    if (t == 0) {
        part[b] = red[0];
        __threadfence();
        last = atomicAdd(ticket, 1u) == (unsigned)gridDim.x - 1u;
    }
    __syncthreads();
    if (last && t == 0) {
        __threadfence();
        const volatile double *vp = part;
        double sum = 0.0;
        for (int e = 0; e < kPhinBlocks; ++e) sum += vp[e];
        S.phin[k] = sum;
        *ticket = 0u;
    }
}
