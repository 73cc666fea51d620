// Part of the kmc_gb300.cu translation unit (included there, in order, inside its
// anonymous namespace unless it says otherwise): eval_field, the per-charge energies and the energy of a set of charges (insertion / removal).
#pragma once
// ---------------------------------------------------------------------------
// eval_field (kmc_fmm.py:544-567): potential of all charges at arbitrary points
//   near:  sum over the 27 neighbour cells of q_j / |x - x_j|   (kmc_local.py:1033-1182)
//   far:   the local expansion of the point's cell                (kmc_octal.py:1417-1440)
//   pbc:   the far-lattice term, d/dq of the lattice energy for a unit charge at x:
//          a(x) . g with g = A M                                   (kmc_full_long_range.py:341-390)
// No energy_unit factor (as in the reference).
// ---------------------------------------------------------------------------
// E_LR(M) = 1/2 (ReM^T A_re ReM + ImM^T A_im ImM) for the multipole S.mpole, block reduction
__device__ double lr_energy_block(const Sys &S, double *red)
{
    double e = 0.0;
    for (int r = threadIdx.x; r < S.NH; r += blockDim.x) {
        double t = 0.0, u = 0.0;
        for (int k = S.ar_ptr[r]; k < S.ar_ptr[r + 1]; ++k) t += S.ar_val[k] * S.mpole[S.ar_col[k]].x;
        for (int k = S.ai_ptr[r]; k < S.ai_ptr[r + 1]; ++k) u += S.ai_val[k] * S.mpole[S.ai_col[k]].y;
        e += S.mpole[r].x * t + S.mpole[r].y * u;
    }
    red[threadIdx.x] = e;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    const double v = 0.5 * red[0];
    __syncthreads();
    return v;
}

// lattice term of the potential at x: a(x) . g for the unit-charge multipole a = (Re Rg, -Im Rg)
__device__ double lattice_potential(const Sys &S, const double2 *__restrict__ g, const double x, const double y,
                                    const double z)
{
    const double r2 = x * x + y * y + z * z;
    double dre = 1.0, dim = 0.0, lr = 0.0;
    for (int m = 0; m < S.L; ++m) {
        if (m > 0) {
            const double t = c_rec_d[m];
            const double nre = t * (dre * x - dim * y), nim = t * (dre * y + dim * x);
            dre = nre;
            dim = nim;
        }
        double pre = 0.0, pim = 0.0, cre = dre, cim = dim;
        for (int l = m; l < S.L; ++l) {
            if (l > m) {
                const double az = c_rec_a[l * KMC_LMAX + m] * z, br = c_rec_b[l * KMC_LMAX + m] * r2;
                const double nre = az * cre - br * pre, nim = az * cim - br * pim;
                pre = cre;
                pim = cim;
                cre = nre;
                cim = nim;
            }
            const double2 gg = g[hidx(l, m)];
            lr += cre * gg.x - cim * gg.y;
        }
    }
    return lr;
}

__global__ void k_eval_field(const Sys S, const double2 *__restrict__ g, const int n, const double *__restrict__ pts,
                             double *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = pts[3 * (size_t)i], y = pts[3 * (size_t)i + 1], z = pts[3 * (size_t)i + 2];
    const int cell = bin_cell(x, y, z, S);
    const int cx = cell % S.n, cy = (cell / S.n) % S.n, cz = cell / (S.n * S.n);
    double phi = near_sum_fp64<false>(S, x, y, z, cx, cy, cz, -1) + far_at(S, cell, x, y, z);
    if (S.pbc) phi += lattice_potential(S, g, x, y, z);
    out[i] = phi;
}

// InjectorExtractor.get_energy (kmc_inject_extract.py:82-123): per listed charge
// q_i times its potential without itself -- near field excluding the charge (by
// id), its cell's expansion and, for pbc, the lattice term -- times the energy unit
__global__ void k_energy_ids(const Sys S, const double2 *__restrict__ g, const int n, const long long *__restrict__ ids,
                             double *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int px = (int)ids[i];
    const double x = S.pos[3 * (size_t)px], y = S.pos[3 * (size_t)px + 1], z = S.pos[3 * (size_t)px + 2];
    const int cell = S.pcell[px];
    const int cx = cell % S.n, cy = (cell / S.n) % S.n, cz = cell / (S.n * S.n);
    double phi = near_sum_fp64<true>(S, x, y, z, cx, cy, cz, px) + far_at(S, cell, x, y, z);
    if (S.pbc) phi += lattice_potential(S, g, x, y, z);
    out[i] = S.unit * S.q[px] * phi;
}

// Energy of a set of charges alone in the box, the quantity of the reference's
// direct solvers (kmc_inject_extract.py:145-166: FreeSpaceDirect, NearestDirect,
// PBCDirect) in this library's energy definition: pair terms (over the 3x3x3 image
// block for '27' and pbc), the self-image terms 1/2 q^2 sum_{o != 0} 1/|oE|, and for
// pbc the lattice term 1/2 M^T A M of the set's multipole.  One block; gm is
// scratch [NH].
__global__ void k_group_energy(Sys S, const int n, const double *__restrict__ pos, const double *__restrict__ q,
                               double2 *gm, double *out)
{
    __shared__ double red[256];
    double e = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double xi = pos[3 * (size_t)i], yi = pos[3 * (size_t)i + 1], zi = pos[3 * (size_t)i + 2];
        for (int j = i + 1; j < n; ++j) {
            const double dx = xi - pos[3 * (size_t)j], dy = yi - pos[3 * (size_t)j + 1], dz = zi - pos[3 * (size_t)j + 2];
            double acc = 0.0;
            if (S.periodic) {
                for (int o = 0; o < 27; ++o) {
                    const double ex = dx + (o % 3 - 1) * S.E, ey = dy + ((o / 3) % 3 - 1) * S.E,
                                 ez = dz + (o / 9 - 1) * S.E;
                    acc += rsqrt(ex * ex + ey * ey + ez * ez);
                }
            } else {
                acc = rsqrt(dx * dx + dy * dy + dz * dz);
            }
            e += q[i] * q[j] * acc;
        }
        if (S.periodic) e -= 0.5 * q[i] * q[i] * S.dom27;  // dom27 = -sum_{o != 0} 1/|oE|
    }
    red[threadIdx.x] = e;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
        __syncthreads();
    }
    double tot = red[0];
    __syncthreads();
    if (S.pbc) {
        for (int h = threadIdx.x; h < S.NH; h += blockDim.x) {
            int l = 0;
            while (hidx(l + 1, 0) <= h) ++l;
            const int m = h - hidx(l, 0);
            double mr = 0.0, mi = 0.0;
            for (int i = 0; i < n; ++i) {
                const double x = pos[3 * (size_t)i], y = pos[3 * (size_t)i + 1], z = pos[3 * (size_t)i + 2];
                const double r2 = x * x + y * y + z * z;
                double dre = 1.0, dim = 0.0;
                for (int k = 1; k <= m; ++k) {
                    const double t = c_rec_d[k];
                    const double nre = t * (dre * x - dim * y), nim = t * (dre * y + dim * x);
                    dre = nre;
                    dim = nim;
                }
                double pre = 0.0, pim = 0.0, cre = dre, cim = dim;
                for (int k = m + 1; k <= l; ++k) {
                    const double az = c_rec_a[k * KMC_LMAX + m] * z, br = c_rec_b[k * KMC_LMAX + m] * r2;
                    const double nre = az * cre - br * pre, nim = az * cim - br * pim;
                    pre = cre;
                    pim = cim;
                    cre = nre;
                    cim = nim;
                }
                mr += q[i] * cre;
                mi -= q[i] * cim;
            }
            gm[h] = make_double2(mr, mi);
        }
        __syncthreads();
        S.mpole = gm;
        tot += lr_energy_block(S, red);
    }
    if (threadIdx.x == 0) out[0] = S.unit * tot;
}
