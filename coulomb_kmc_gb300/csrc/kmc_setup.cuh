// Part of the kmc_gb300.cu translation unit (included there, in order, inside its
// anonymous namespace unless it says otherwise): move set-up (setup_move as count / scan / scatter), the FP64 old and new sides, the difference assembly and the counting sort of proposals by target cell.
#pragma once
// ---------------------------------------------------------------------------
// move set-up: setup_move (kmc_mpi_decomp.py:489-616) as count / scan / scatter
// ---------------------------------------------------------------------------
__device__ __forceinline__ int count_active(const int px, const int M, const long long *smc, const long long *sites,
                                            const long long *masks)
{
    const long long lim = smc[sites[px]];
    int found = 0;
    for (int mv = 0; mv < M && found < lim; ++mv)
        if (masks[(size_t)px * M + mv] > 0) ++found;
    return found;
}

template <typename T>
__device__ T block_exclusive_scan(T v, T *warp_tot, T &block_total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        T t = lane < nw ? warp_tot[lane] : (T)0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) warp_tot[lane] = t;
    }
    __syncthreads();
    const T warp_off = wid > 0 ? warp_tot[wid - 1] : (T)0;
    block_total = warp_tot[nw - 1];
    __syncthreads();
    return warp_off + x - v;
}

__global__ void k_count_scan(const int N, const int M, const long long *smc, const long long *sites,
                             const long long *masks, Props P)
{
    __shared__ unsigned long long wt[32];
    const int px = blockIdx.x * blockDim.x + threadIdx.x;
    int c = 0;
    if (px < N) c = count_active(px, M, smc, sites, masks);
    const unsigned long long v = (unsigned long long)c | ((unsigned long long)(c > 0) << 32);
    unsigned long long tot;
    const unsigned long long ex = block_exclusive_scan(v, wt, tot);
    if (px < N) {
        P.cnt[px] = c;
        P.scan[px] = ex;
    }
    if (threadIdx.x == 0) P.part[blockIdx.x] = tot;
}


// check_move, kmc_mpi_decomp.py:460-486 (same operation sequence)
__device__ __forceinline__ int check_move(const Sys &S, const double *p, const double *pp)
{
    int err = 0;
    for (int d = 0; d < 3; ++d) {
        if (pp[d] < -0.5 * S.E) ++err;
        if (pp[d] > 0.5 * S.E) ++err;
    }
    for (int d = 0; d < 3; ++d) {
        double dd = p[d] - pp[d];
        if (S.periodic) {
            if (dd < (0.5 * S.E)) dd += S.E;
            if (dd > (0.5 * S.E)) dd -= S.E;
        }
        if ((dd * dd) > S.max_move2) ++err;
    }
    return err;
}

__global__ void k_scan_part(const int nb, Props P)
{
    __shared__ unsigned long long wt[32];
    __shared__ unsigned long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const unsigned long long v = i < nb ? P.part[i] : 0ull;
        unsigned long long tot;
        const unsigned long long ex = block_exclusive_scan(v, wt, tot);
        if (i < nb) P.part[i] = ex + carry;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int nump = (int)(carry >> 32);
        const int total = (int)(carry & 0xffffffffull);
        P.totals[0] = nump;
        P.totals[1] = total;
        P.es[nump] = total;
    }
}

// one thread per (charge, move slot): the slot's rank among the charge's first
// cnt active slots gives its place in the compacted proposal arrays
// CHECK: apply the reference's move checks (check_move); off for moves that are
// valid by construction (the device driver's hops and displacements)
template <bool CHECK>
__global__ void k_scatter(const Sys S, const int N, const int M, const double *prop_pos, const long long *masks,
                          const double *prop_q, const int *prop_cells, Props P, unsigned long long *err)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (long long)N * M) return;
    const int px = (int)(g / M), mv = (int)(g - (long long)px * M);
    if (masks[g] <= 0) return;
    const int c = P.cnt[px];
    int found = 0;
    for (int k = 0; k < mv; ++k) found += masks[(size_t)px * M + k] > 0;
    if (found >= c) return;
    const unsigned long long v = P.scan[px] + P.part[px / kScanBlock];
    const int off = (int)(v & 0xffffffffull);
    const int oind = (int)(v >> 32);
    if (found == 0) {
        P.old_pid[oind] = px;
        P.es[oind] = off;
    }
    const int nind = off + found;
    const double *pp = prop_pos + 3 * (size_t)g;
    const double x = pp[0], y = pp[1], z = pp[2];
    const int bad = CHECK ? check_move(S, S.pos + 3 * (size_t)px, pp) : 0;
    P.owner[nind] = oind;
    P.ppos[3 * (size_t)nind + 0] = x;
    P.ppos[3 * (size_t)nind + 1] = y;
    P.ppos[3 * (size_t)nind + 2] = z;
    P.pq[nind] = prop_q ? prop_q[g] : S.q[px];
    const int cell = prop_cells ? prop_cells[g] : bin_cell(x, y, z, S);  // given: the caller binned them
    P.pc[nind] = cell;
    atomicAdd(&P.ccount[cell], 1);
    P.rloc[nind] = g;
    if (bad) atomicAdd(err, (unsigned long long)bad);
}

// proposals given explicitly (propose(moves) path): fill per-proposal fields
__global__ void k_fill_moves(const Sys S, Props P, const int nump)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nump) return;
    const int px = P.old_pid[o];
    for (int p = P.es[o]; p < P.es[o + 1]; ++p) {
        P.owner[p] = o;
        P.pq[p] = S.q[px];
        P.pc[p] = bin_cell(P.ppos[3 * (size_t)p], P.ppos[3 * (size_t)p + 1], P.ppos[3 * (size_t)p + 2], S);
        P.rloc[p] = p;
    }
}


// ---------------------------------------------------------------------------
// old side: U0 = q (near excluding self + far) per moving charge; with `all`
// (initialisation), every charge, and its near-field potential is kept in S.phin
// ---------------------------------------------------------------------------
__global__ void k_old(const Sys S, Props P, const int all)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    const int nump = all ? S.N : P.totals[0];
    if (o >= nump) return;
    const int px = all ? o : P.old_pid[o];
    const double x = S.pos[3 * (size_t)px], y = S.pos[3 * (size_t)px + 1], z = S.pos[3 * (size_t)px + 2];
    const int cell = S.pcell[px];
    const int cx = cell % S.n, cy = (cell / S.n) % S.n, cz = cell / (S.n * S.n);
    const double nf = near_sum_fp64<true>(S, x, y, z, cx, cy, cz, px);
    const double ff = far_at(S, cell, x, y, z);
    P.u0p[px] = S.q[px] * nf + S.q[px] * ff;
    if (all) S.phin[px] = nf;  // the near-field potential kept between moves
}

// self / moved-pair term  kmc_fmm_self_interaction.py:163-242
__device__ __forceinline__ double self_term(const Sys &S, const double ox, const double oy, const double oz,
                                            const double nx, const double ny, const double nz)
{
    if (!S.periodic) {
        const double dx = ox - nx, dy = oy - ny, dz = oz - nz;
        return rsqrt(dx * dx + dy * dy + dz * dz);
    }
    double e = S.dom27;
    for (int c = -1; c <= 1; ++c)
        for (int b = -1; b <= 1; ++b)
            for (int a = -1; a <= 1; ++a) {
                const double dx = (S.E * a + ox) - nx;
                const double dy = (S.E * b + oy) - ny;
                const double dz = (S.E * c + oz) - nz;
                e += rsqrt(dx * dx + dy * dy + dz * dz);
            }
    return e;
}

// ---------------------------------------------------------------------------
// new side: near + far + self, and the difference (diff_lib, kmc_fmm.py:607-655)
// ---------------------------------------------------------------------------
__global__ void k_new(const Sys S, Props P, double *out)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.totals[1]) return;
    const int o = P.owner[p];
    const int px = P.old_pid[o];
    const double x = P.ppos[3 * (size_t)p], y = P.ppos[3 * (size_t)p + 1], z = P.ppos[3 * (size_t)p + 2];
    const int cell = P.pc[p];
    const int cx = cell % S.n, cy = (cell / S.n) % S.n, cz = cell / (S.n * S.n);
    const double qn = P.pq[p];
    const double nf = near_sum_fp64<false>(S, x, y, z, cx, cy, cz, -1);
    const double ff = far_at(S, cell, x, y, z);
    const double qo = S.q[px];
    const double usi = qo * qo * self_term(S, S.pos[3 * (size_t)px], S.pos[3 * (size_t)px + 1],
                                           S.pos[3 * (size_t)px + 2], x, y, z);
    P.pnew[p] = (qn * nf + qn * ff) - usi;
    (void)o;
    (void)out;
}

// difference assembly: near + cell expansion parts, plus the lattice part for pbc
// (diff_lib, kmc_fmm.py:607-655)
__global__ void k_diff(const Sys S, Props P, double *out)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.totals[1]) return;
    const int px = P.old_pid[P.owner[p]];
    const double lr = S.pbc ? P.elr[p] : 0.0;
    out[P.rloc[p]] = S.unit * ((P.pnew[p] - P.u0p[px]) + lr);
}

// ---------------------------------------------------------------------------
// proposals grouped by target cell (counting sort)
// ---------------------------------------------------------------------------

__global__ void k_cell_scan(const int ncell, Props P)
{
    __shared__ int wt[32];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < ncell; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < ncell ? P.ccount[i] : 0;
        int tot;
        const int ex = block_exclusive_scan(v, wt, tot);
        if (i < ncell) {
            P.cstart[i] = ex + carry;
            P.ccount[i] = 0;
        }
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) P.cstart[ncell] = carry;
}

__global__ void k_cell_place(Props P)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.totals[1]) return;
    const int c = P.pc[p];
    const int k = atomicAdd(&P.ccount[c], 1);
    P.cprops[P.cstart[c] + k] = p;
}
