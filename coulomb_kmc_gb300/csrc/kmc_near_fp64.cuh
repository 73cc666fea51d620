// Part of the kmc_gb300.cu translation unit (included there, in order, inside its
// anonymous namespace unless it says otherwise): the FP64 cell-staged near field with the cell-expansion evaluation and the self term (one block per cell).
#pragma once
// ---------------------------------------------------------------------------
// cell-staged near field + expansion evaluation, one CTA per finest cell:
//   old side for the moving charges stored in the cell   -> u0p[pid]
//   new side for the proposals whose target is the cell  -> pnew[p]
// The 27 neighbour cells (shifted across periodic faces) are staged in
// shared memory in chunks, and the cell's expansion once; every thread then
// runs the same loop (direct_new/direct_old kmc_local.py:956-1019,
// indirect_interactions kmc_octal.py:591-691, self_interaction
// kmc_fmm_self_interaction.py:204-242).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double far_eval_shared(const double2 *Lc, const int L, const double x, const double y,
                                                  const double z)
{
    const double r2 = x * x + y * y + z * z;
    double dre = 1.0, dim = 0.0;
    double total = 0.0;
    for (int m = 0; m < L; ++m) {
        if (m > 0) {
            const double t = c_rec_d[m];
            const double nre = t * (dre * x - dim * y);
            const double nim = t * (dre * y + dim * x);
            dre = nre;
            dim = nim;
        }
        double pre = 0.0, pim = 0.0, cre = dre, cim = dim;
        double2 Lv = Lc[hidx(m, m)];
        double acc = Lv.x * cre - Lv.y * cim;
        for (int l = m + 1; l < L; ++l) {
            const double az = c_rec_a[l * KMC_LMAX + m] * z;
            const double br = c_rec_b[l * KMC_LMAX + m] * r2;
            const double nre = az * cre - br * pre;
            const double nim = az * cim - br * pim;
            pre = cre;
            pim = cim;
            cre = nre;
            cim = nim;
            Lv = Lc[hidx(l, m)];
            acc += Lv.x * cre - Lv.y * cim;
        }
        total += (m == 0) ? acc : 2.0 * acc;
    }
    return total;
}

constexpr int kNearThreads = 64;
constexpr int kNearChunk = 256;

// kept: the moving charges' near-field potentials are taken from S.phin (kept by
// every accept), so they only evaluate the cell expansion
__global__ void __launch_bounds__(kNearThreads) k_near_cell(const Sys S, Props P, const bool kept)
{
    extern __shared__ double4_32a nsm[];
    double4_32a *stg = nsm;                                    // [kNearChunk]
    double2 *lc = reinterpret_cast<double2 *>(stg + kNearChunk); // [NH]
    int *spid = reinterpret_cast<int *>(lc + S.NH);            // [kNearChunk]
    __shared__ int nb_cell[27], nb_off[28];
    __shared__ double nb_s[27][3];
    const int c = blockIdx.x;
    const int tid = threadIdx.x;
    const int n_old = S.cnt[c];
    const int p0 = P.cstart[c];
    const int np = P.cstart[c + 1] - p0;
    if (n_old + np == 0) return;
    const int n = S.n;
    const int cx = c % n, cy = (c / n) % n, cz = c / (n * n);
    if (tid < 27) {
        const int dx = tid % 3 - 1, dy = (tid / 3) % 3 - 1, dz = tid / 9 - 1;
        int nx = cx + dx, ny = cy + dy, nz = cz + dz;
        double sx = 0.0, sy = 0.0, sz = 0.0;
        bool ok = true;
        if (nx < 0) { nx += n; sx = -S.E; ok = ok && S.periodic; } else if (nx >= n) { nx -= n; sx = S.E; ok = ok && S.periodic; }
        if (ny < 0) { ny += n; sy = -S.E; ok = ok && S.periodic; } else if (ny >= n) { ny -= n; sy = S.E; ok = ok && S.periodic; }
        if (nz < 0) { nz += n; sz = -S.E; ok = ok && S.periodic; } else if (nz >= n) { nz -= n; sz = S.E; ok = ok && S.periodic; }
        const int cc = nx + n * (ny + n * nz);
        nb_cell[tid] = cc;
        nb_off[tid + 1] = ok ? S.cnt[cc] : 0;
        nb_s[tid][0] = sx;
        nb_s[tid][1] = sy;
        nb_s[tid][2] = sz;
    }
    for (int k = tid; k < S.NH; k += blockDim.x) lc[k] = S.lexp[(size_t)c * S.NH + k];
    __syncthreads();
    if (tid == 0) {
        nb_off[0] = 0;
        for (int j = 0; j < 27; ++j) nb_off[j + 1] += nb_off[j];
    }
    __syncthreads();
    const int total_nb = nb_off[27];
    const double ccx = cell_centre(S, cx), ccy = cell_centre(S, cy), ccz = cell_centre(S, cz);
    const int n_po = kept ? 0 : n_old;  // moving charges among the pair loop's items
    if (kept)
        for (int o = tid; o < n_old; o += blockDim.x) {
            const int pidx = S.store_pid[(size_t)c * S.cap + o];
            if (P.cnt[pidx] <= 0) continue;
            const double x = S.pos[3 * (size_t)pidx], y = S.pos[3 * (size_t)pidx + 1], z = S.pos[3 * (size_t)pidx + 2];
            const double q = S.q[pidx];
            P.u0p[pidx] = q * S.phin[pidx] + q * far_eval_shared(lc, S.L, x - ccx, y - ccy, z - ccz);
        }
    const int nitems = n_po + np;
    for (int base = 0; base < nitems; base += blockDim.x) {
        const int item = base + tid;
        bool act = item < nitems;
        double x = 0.0, y = 0.0, z = 0.0, q = 0.0;
        int self = -1, pidx = -1, p = -1;
        if (act) {
            if (item < n_po) {
                pidx = S.store_pid[(size_t)c * S.cap + item];
                act = P.cnt[pidx] > 0;  // only charges with proposals need their old-side energy
                self = pidx;
                x = S.pos[3 * (size_t)pidx];
                y = S.pos[3 * (size_t)pidx + 1];
                z = S.pos[3 * (size_t)pidx + 2];
                q = S.q[pidx];
            } else {
                p = P.cprops[p0 + item - n_po];
                x = P.ppos[3 * (size_t)p];
                y = P.ppos[3 * (size_t)p + 1];
                z = P.ppos[3 * (size_t)p + 2];
                q = P.pq[p];
            }
        }
        double acc = 0.0;
        for (int k0 = 0; k0 < total_nb; k0 += kNearChunk) {
            const int kn = min(kNearChunk, total_nb - k0);
            __syncthreads();
            for (int k = tid; k < kn; k += blockDim.x) {
                const int kk = k0 + k;
                int j = 0;
                while (nb_off[j + 1] <= kk) ++j;
                const size_t a = (size_t)nb_cell[j] * S.cap + (kk - nb_off[j]);
                const double4_32a v = S.store[a];
                stg[k] = make_double4_32a(v.x + nb_s[j][0], v.y + nb_s[j][1], v.z + nb_s[j][2], v.w);
                spid[k] = S.store_pid[a];
            }
            __syncthreads();
            if (act) {
                if (self >= 0) {
                    for (int k = 0; k < kn; ++k) {
                        const double4_32a v = stg[k];
                        if (spid[k] == self) continue;
                        const double ddx = x - v.x, ddy = y - v.y, ddz = z - v.z;
                        acc += v.w * rsqrt(ddx * ddx + ddy * ddy + ddz * ddz);
                    }
                } else {
                    for (int k = 0; k < kn; ++k) {
                        const double4_32a v = stg[k];
                        const double ddx = x - v.x, ddy = y - v.y, ddz = z - v.z;
                        acc += v.w * rsqrt(ddx * ddx + ddy * ddy + ddz * ddz);
                    }
                }
            }
        }
        if (act) {
            const double ff = far_eval_shared(lc, S.L, x - ccx, y - ccy, z - ccz);
            if (self >= 0) {
                P.u0p[pidx] = q * acc + q * ff;
            } else {
                const int px = P.old_pid[P.owner[p]];
                const double qo = S.q[px];
                const double usi = qo * qo * self_term(S, S.pos[3 * (size_t)px], S.pos[3 * (size_t)px + 1],
                                                       S.pos[3 * (size_t)px + 2], x, y, z);
                P.pnew[p] = (q * acc + q * ff) - usi;
            }
        }
    }
}
