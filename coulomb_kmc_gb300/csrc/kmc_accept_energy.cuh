// Part of the kmc_gb300.cu translation unit (included there, in order, inside its
// anonymous namespace unless it says otherwise): the FP64 energy difference of the accepted move (the single-move kernel of the accept).
#pragma once
// ---------------------------------------------------------------------------
// FP64 energy difference of ONE move (accept path): the near sums, expansion
// evaluations, self term and lattice term are split over a few dozen small blocks
// and reduced in a fixed order.  Same arithmetic as the batch kernels
// (direct_new/old, indirect_interactions, self_interaction, long_range_energy,
// diff_lib), summed in a different order.
// ---------------------------------------------------------------------------
constexpr int kSpBlocks = 56, kSpThreads = 128;

__device__ __forceinline__ double block_sum(double v, double *red)
{
    red[threadIdx.x] = v;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

// far-field partial from a staged expansion: column m (< L) of the expansion at the point
__device__ double far_partial(const Sys &S, const double2 *Lc, const int cell, const double px, const double py,
                              const double pz, const int m, const RecTab &T)
{
    if (m < 0 || m >= S.L) return 0.0;
    const int cx = cell % S.n, cy = (cell / S.n) % S.n, cz = cell / (S.n * S.n);
    const double x = px - cell_centre(S, cx), y = py - cell_centre(S, cy), z = pz - cell_centre(S, cz);
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
    double2 Lv = Lc[hidx(m, m)];
    double acc = Lv.x * cre - Lv.y * cim;
    for (int l = m + 1; l < S.L; ++l) {
        const double az = T.a[l * T.L + m] * z;
        const double br = T.b[l * T.L + m] * r2;
        const double nre = az * cre - br * pre;
        const double nim = az * cim - br * pim;
        pre = cre;
        pim = cim;
        cre = nre;
        cim = nim;
        Lv = Lc[hidx(l, m)];
        acc += Lv.x * cre - Lv.y * cim;
    }
    return (m == 0) ? acc : 2.0 * acc;
}

// column m (< L) of q conj(Rg(x)) into out (folded layout)
__device__ void multipole_column(double2 *out, const int L, const int m, const double q, const double x,
                                 const double y, const double z, const RecTab &T)
{
    if (m < 0 || m >= L) return;
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
    out[hidx(m, m)] = make_double2(q * cre, -q * cim);
    for (int l = m + 1; l < L; ++l) {
        const double az = T.a[l * T.L + m] * z;
        const double br = T.b[l * T.L + m] * r2;
        const double nre = az * cre - br * pre;
        const double nim = az * cim - br * pim;
        pre = cre;
        pim = cim;
        cre = nre;
        cim = nim;
        out[hidx(l, m)] = make_double2(q * cre, -q * cim);
    }
}

// Energy difference of an accepted move in FP64, evaluated after the store update
// (k_accept_prep) on the recorded move, spread over kSpBlocks blocks so that its
// FP64 work (issued at a small fraction of the FP32 rate on GB300) runs on as many
// SMs.  Blocks 0-26: the new position's near sum over neighbour cell j of the new
// cell, the mover excluded (it now sits at the new position) and its old position
// added back where that cell is the old cell, which reproduces the pre-move sum of
// propose.  Blocks 27-53: the old position's near sum over neighbour cell j of the
// old cell, and image j of the moved pair's self term.  Block 54: the two cell
// expansions at the two positions, from the snapshot taken before the
// particle-to-local update.  Block 55: the lattice term (pbc), with g from before
// the multipole update that runs beside this kernel.  Each block stores its
// partial; the last block to finish (a ticket, no waiting) adds them in a fixed
// order, adds the difference to the energy (not for a null move), writes it to out
// and resets the ticket.
template <bool STAGE_A>
__global__ void __launch_bounds__(kSpThreads) k_single_post(const Sys S, const AcceptRec *rec, const double2 *snap,
                                                            double *part, unsigned *ticket, double *energy,
                                                            double *out)
{
    __shared__ double red[kSpThreads];
    __shared__ bool last;
    extern __shared__ double2 dsm[];
    if (rec->skip) {
        if (blockIdx.x == 0 && threadIdx.x == 0) *out = 0.0;
        return;
    }
    const AcceptRec r = *rec;
    const int b = blockIdx.x, n = S.n, NH = S.NH;
    const double q = r.q;
    double v = 0.0;
    if (b < 54) {
        const bool nw = b < 27;
        const int j = nw ? b : b - 27, cell = nw ? r.cn : r.co;
        const double x = nw ? r.xn : r.xo, y = nw ? r.yn : r.yo, z = nw ? r.zn : r.zo;
        const int dx = j % 3 - 1, dy = (j / 3) % 3 - 1, dz = j / 9 - 1;
        int nx = cell % n + dx, ny = (cell / n) % n + dy, nz = cell / (n * n) + dz;
        double sx = 0.0, sy = 0.0, sz = 0.0;
        bool ok = true;
        if (nx < 0) { nx += n; sx = -S.E; ok = ok && S.periodic; } else if (nx >= n) { nx -= n; sx = S.E; ok = ok && S.periodic; }
        if (ny < 0) { ny += n; sy = -S.E; ok = ok && S.periodic; } else if (ny >= n) { ny -= n; sy = S.E; ok = ok && S.periodic; }
        if (nz < 0) { nz += n; sz = -S.E; ok = ok && S.periodic; } else if (nz >= n) { nz -= n; sz = S.E; ok = ok && S.periodic; }
        if (ok) {
            const int c = nx + n * (ny + n * nz);
            for (int k = threadIdx.x; k < S.cnt[c]; k += blockDim.x) {
                const size_t a = (size_t)c * S.cap + k;
                if (S.store_pid[a] == r.pid) continue;
                const double4_32a w = S.store[a];
                const double ex = x - (w.x + sx), ey = y - (w.y + sy), ez = z - (w.z + sz);
                v += w.w * rsqrt(ex * ex + ey * ey + ez * ez);
            }
            if (nw && c == r.co && threadIdx.x == 0) {
                const double ex = r.xn - (r.xo + sx), ey = r.yn - (r.yo + sy), ez = r.zn - (r.zo + sz);
                v += q * rsqrt(ex * ex + ey * ey + ez * ez);
            }
        }
        v *= nw ? q : -q;
        if (!nw && S.periodic && threadIdx.x == 0) {
            const double ex = (S.E * dx + r.xo) - r.xn, ey = (S.E * dy + r.yo) - r.yn, ez = (S.E * dz + r.zo) - r.zn;
            v -= q * q * rsqrt(ex * ex + ey * ey + ez * ez);
        }
    } else if (b == 54) {
        // new position on threads 0..L-1, old on 32..32+L-1 (columns in parallel)
        double2 *Lo = dsm, *Ln = dsm + NH;
        const RecTab T = stage_rec(reinterpret_cast<double *>(dsm + 2 * NH), S.L);
        for (int k = threadIdx.x; k < NH; k += blockDim.x) {
            Lo[k] = snap[k];
            Ln[k] = snap[NH + k];
        }
        __syncthreads();
        v = threadIdx.x < 32 ? q * far_partial(S, Ln, r.cn, r.xn, r.yn, r.zn, threadIdx.x, T)
                             : -q * far_partial(S, Lo, r.co, r.xo, r.yo, r.zo, threadIdx.x - 32, T);
        if (!S.periodic && threadIdx.x == 0) {
            const double ex = r.xo - r.xn, ey = r.yo - r.yn, ez = r.zo - r.zn;
            v -= q * q * rsqrt(ex * ex + ey * ey + ez * ez);
        }
    } else if (S.pbc) {
        double2 *dl = dsm, *mo = dsm + NH;
        double *tab = reinterpret_cast<double *>(dsm + 2 * NH);
        const RecTab T = stage_rec(tab, S.L);
        // the upper form (value, column) staged in one parallel round of loads
        const int nru = S.aru_ptr[NH], niu = S.aiu_ptr[NH];
        double *uv = tab + rec_tab_size(S.L);
        int *uc = reinterpret_cast<int *>(uv + (STAGE_A ? nru + niu : 0));
        if (STAGE_A) {
            for (int e = threadIdx.x; e < nru; e += blockDim.x) {
                uv[e] = S.aru_val[e];
                uc[e] = S.aru_col[e];
            }
            for (int e = threadIdx.x; e < niu; e += blockDim.x) {
                uv[nru + e] = S.aiu_val[e];
                uc[nru + e] = S.aiu_col[e];
            }
        }
        __syncthreads();
        if (threadIdx.x < 32)
            multipole_column(dl, S.L, threadIdx.x, q, r.xn, r.yn, r.zn, T);
        else
            multipole_column(mo, S.L, threadIdx.x - 32, q, r.xo, r.yo, r.zo, T);
        __syncthreads();
        for (int k = threadIdx.x; k < NH; k += blockDim.x) dl[k] = make_double2(dl[k].x - mo[k].x, dl[k].y - mo[k].y);
        __syncthreads();
        for (int k = threadIdx.x; k < NH; k += blockDim.x) {
            double t = 0.0, u = 0.0;
            if (STAGE_A) {
                for (int e = S.aru_ptr[k]; e < S.aru_ptr[k + 1]; ++e) t += uv[e] * dl[uc[e]].x;
                for (int e = S.aiu_ptr[k]; e < S.aiu_ptr[k + 1]; ++e) u += uv[nru + e] * dl[uc[nru + e]].y;
            } else {
                for (int e = S.aru_ptr[k]; e < S.aru_ptr[k + 1]; ++e) t += S.aru_val[e] * dl[S.aru_col[e]].x;
                for (int e = S.aiu_ptr[k]; e < S.aiu_ptr[k + 1]; ++e) u += S.aiu_val[e] * dl[S.aiu_col[e]].y;
            }
            const double2 gg = snap[2 * NH + k];  // g before the move
            v += dl[k].x * (gg.x + 0.5 * t) + dl[k].y * (gg.y + 0.5 * u);
        }
    }
    const double bs = block_sum(v, red);
    if (threadIdx.x == 0) {
        part[b] = bs;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x < 32) {
        // the partials in a fixed tree order (warp shuffles): a short FP64 dependency chain
        __threadfence();
        double d = 0.0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += 32) d += *(volatile const double *)&part[i];
        for (int off = 16; off > 0; off >>= 1) d += __shfl_xor_sync(0xffffffffu, d, off);
        if (threadIdx.x == 0) {
            if (S.periodic) d -= q * q * S.dom27;
            out[0] = S.unit * d;
            if (!r.null_move) *energy += S.unit * d;
            *ticket = 0u;
        }
    }
}
