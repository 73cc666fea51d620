// Part of the kmc_gb300.cu translation unit (included there, in order, inside its
// anonymous namespace unless it says otherwise): error macros, the device-side views of a system (Sys) and of its compacted proposals (Props), the accept record, binning, the FP64 near-field sum and the warp-cooperative FP64 helpers.
#pragma once
thread_local std::string g_err;

#define KMC_CUDA(call)                                                                                             \
    do {                                                                                                           \
        cudaError_t e_ = (call);                                                                                   \
        if (e_ != cudaSuccess) {                                                                                   \
            g_err = std::string(#call) + ": " + cudaGetErrorString(e_);                                            \
            return KMC_ECUDA;                                                                                      \
        }                                                                                                          \
    } while (0)

#define KMC_LAUNCH_CHECK()                                                                                         \
    do {                                                                                                           \
        cudaError_t e_ = cudaGetLastError();                                                                       \
        if (e_ != cudaSuccess) {                                                                                   \
            g_err = std::string("kernel launch: ") + cudaGetErrorString(e_);                                       \
            return KMC_ECUDA;                                                                                      \
        }                                                                                                          \
    } while (0)

constexpr int kScanBlock = 1024;

// Everything a kernel needs to read the system, passed by value.
struct Sys {
    int n;        // cells per side
    int ncell;    // n^3
    int cap;      // store slots per cell
    int L, NH;    // expansion terms, folded coefficient count
    int periodic; // 1 for '27' and pbc: wrap neighbour cells
    int nimg;     // images in the accept / initial solve: 1 (free space) or 27
    int pbc;      // far-field lattice term present
    int N;        // charges
    double E, w, inv_w, start, max_move2, dom27, unit;
    float w_hi, w_lo, iw_hi, iw_lo;  // cell width and its inverse as df32
    double4_32a *store;
    int *store_pid;
    int *cnt;
    double *pos;
    double *q;
    int *pcell;
    int *pslot;
    double *phin;  // [N] near-field potential of each charge at its position (sum over the 27
                   // cells around it, itself excluded), set at initialisation, kept by every accept
    double2 *lexp;
    double2 *mpole;
    // folded lattice quadratic form (pbc)
    const int *ar_ptr;
    const int *ar_col;
    const double *ar_val;
    const int *ai_ptr;
    const int *ai_col;
    const double *ai_val;
    // upper triangles with doubled off-diagonal entries: x^T A x = sum_{i<=j} U_ij x_i x_j
    const int *aru_ptr;
    const int *aru_col;
    const double *aru_val;
    const int *aiu_ptr;
    const int *aiu_col;
    const double *aiu_val;
    // mixed precision (KMC_PREC_MIXED): FP32 double-word copies
    int mixed;
    int accept_df32;             // accept contributions in double-FP32 (KMC_PREC_MIXED)
    float4 *st_hi, *st_lo;       // [ncell][cap] near-field copy: position relative to the slot's cell
                                 // centre in cell widths (grid_split), charge as df32
    float4 *lexp32;              // [ncell][NH] (re_hi, im_hi, re_lo, im_lo)
    const float2 *a2_val;        // the folded form in box units, A E^(l + l' + 1), as FP32 pairs (pattern of ar / ai)
    const float2 *ai2_val;
    const float *ar32_val;       // full folded lattice form in FP32 (pattern of ar / ai)
    const float *ai32_val;
    // far-lattice self term F(x) = 1/2 a(x)^T A a(x) of a unit charge (lattice_self_program)
    const int *fprog_i;
    const double *fprog_d;
    const float *fprog_f;        // in box units: F(x) = F_hat(x / E) / E
    // mixed lattice path in box units: a(x / E), A E^(l + l' + 1), g E^(l + 1)
    double inv_E;
    const double *escale;        // [NH] E^(l + 1)
    const double *p2lsc;         // [NH] C_lm w^-(l+1): scale of the double-FP32 accept's sums
};

// Compacted proposals (the reference's host_data dictionary, kmc_mpi_decomp.py:122-158).
struct Props {
    int *cnt;                  // [N] active proposals per charge
    unsigned long long *scan;  // [N] packed (charges-with-moves << 32 | proposals) prefix within a block
    unsigned long long *part;  // [nblocks] block totals, scanned in place
    int *old_pid;              // [N] moving charge of each old index
    int *es;                   // [N+1] exclusive_sum
    int *owner;                // [N*M] old index of each proposal
    double *ppos;              // [N*M*3] proposed positions
    double *pq;                // [N*M] proposed charges
    int *pc;                   // [N*M] proposed cells
    long long *rloc;           // [N*M] rate_location
    double *u0p;               // [N] old-side energy q (near + far), indexed by particle
    double *pnew;              // [N*M] new-side energy q'(near + far) - self term, per proposal
    double *dout;              // [N*M] differences in proposal order (explicit-moves path)
    int *ccount;               // [ncell] proposals per target cell (count, then fill cursor)
    int *cstart;               // [ncell+1] first proposal of each cell in cprops
    int *cprops;               // [N*M] proposal ids grouped by target cell
    double2 *g;                // [NH] A M (pbc)
    double2 *h;                // [N*NH] A b per moving charge (pbc)
    double *co;                // [N] per moving charge constant of the lattice difference (pbc)
    double *coq;               // [N] mixed: its quadratic part alone, b.h / 2 (box units / E), for
                               // proposals whose lattice term is formed from the harmonics' difference
    double *elr;               // [N*M] lattice part of each proposal's difference (pbc)
    double *upot;              // [N*M] mixed near field: potential at a proposal position, by its leader
    float4 *ugrid;             // [2 N*M] mixed near field: the leader's grid copy (high words, low words)
    float4 *obox;              // [2 N] mixed pbc: moving charge's old position in box units, double-FP32
                               // (high words xyz, low words xyz), for the self term of its proposals
    int *totals;               // [2] num_particles, total_movs
};

struct AcceptRec {
    double q, xo, yo, zo, xn, yn, zn;
    int to[3], tn[3];
    int skip;       // device-selected accept with pid < 0: no move this round
    int null_move;  // new position == old position: the energy does not change (kmc_fmm.py:1094-1095)
    int pid, co, cn;
    int pad;
};

__device__ __forceinline__ int bin_axis(const double x, const Sys &S)
{
    // get_cell, kmc_mpi_decomp.py:400-420
    long long c = (long long)((x + 0.5 * S.E) * S.inv_w);
    if (c >= S.n) c = S.n - 1;
    if (c < 0) c = 0;  // memory safety only: valid positions never bin below 0 (NaN converts to a negative)
    return (int)c;
}

__device__ __forceinline__ int bin_cell(const double x, const double y, const double z, const Sys &S)
{
    return bin_axis(x, S) + S.n * (bin_axis(y, S) + S.n * bin_axis(z, S));
}

// Near-field sum  sum_j q_j / |x - x_j|  over the 27 cells around cell (cx,cy,cz)
// (direct_new / direct_old, kmc_local.py:956-1019).  EXCL skips particle `self`.
template <bool EXCL>
__device__ double near_sum_fp64(const Sys &S, const double x, const double y, const double z, const int cx,
                                const int cy, const int cz, const int self)
{
    double acc = 0.0;
    for (int dz = -1; dz <= 1; ++dz) {
        int nz = cz + dz;
        double sz = 0.0;
        if (nz < 0) {
            if (!S.periodic) continue;
            nz += S.n;
            sz = -S.E;
        } else if (nz >= S.n) {
            if (!S.periodic) continue;
            nz -= S.n;
            sz = S.E;
        }
        for (int dy = -1; dy <= 1; ++dy) {
            int ny = cy + dy;
            double sy = 0.0;
            if (ny < 0) {
                if (!S.periodic) continue;
                ny += S.n;
                sy = -S.E;
            } else if (ny >= S.n) {
                if (!S.periodic) continue;
                ny -= S.n;
                sy = S.E;
            }
            for (int dx = -1; dx <= 1; ++dx) {
                int nx = cx + dx;
                double sx = 0.0;
                if (nx < 0) {
                    if (!S.periodic) continue;
                    nx += S.n;
                    sx = -S.E;
                } else if (nx >= S.n) {
                    if (!S.periodic) continue;
                    nx -= S.n;
                    sx = S.E;
                }
                const int c = nx + S.n * (ny + S.n * nz);
                const int k = S.cnt[c];
                const double4_32a *st = S.store + (size_t)c * S.cap;
                const int *sp = S.store_pid + (size_t)c * S.cap;
                for (int j = 0; j < k; ++j) {
                    const double4_32a v = st[j];
                    if (EXCL && sp[j] == self) continue;
                    const double ddx = x - (v.x + sx);
                    const double ddy = y - (v.y + sy);
                    const double ddz = z - (v.z + sz);
                    acc += v.w * rsqrt(ddx * ddx + ddy * ddy + ddz * ddz);
                }
            }
        }
    }
    return acc;
}

__device__ __forceinline__ double cell_centre(const Sys &S, const int c)
{
    // kmc_octal.py:397-428: starts + c * widths
    return S.start + c * S.w;
}

// Near-field coordinates: u = (x - cell centre) / cell width, |u| <= 1/2, split
// as u = hi + lo with hi on the 2^-10 grid and lo = u - hi rounded to FP32
// (|lo| <= 2^-11, about 2^-35 absolute error).  In a cell's frame a neighbour's
// hi + d (d = -1, 0, 1) stays on the grid with |.| <= 3/2, so for an item
// (|hi| <= 1/2) and a neighbour the differences s = hi_i - hi_j (|s| <= 2, 12
// bits) and s_x^2 + s_y^2 + s_z^2 (<= 12 on the 2^-20 grid, 24 bits) are exact
// in FP32.
constexpr double kGrid = 1024.0;

__device__ __forceinline__ float2 grid_split(const double u)
{
    const double hi = rint(u * kGrid) * (1.0 / kGrid);
    return make_float2((float)hi, (float)(u - hi));
}


__device__ __forceinline__ double far_at(const Sys &S, const int cell, const double x, const double y,
                                         const double z)
{
    const int cx = cell % S.n, cy = (cell / S.n) % S.n, cz = cell / (S.n * S.n);
    return far_eval_fp64(S.lexp + (size_t)cell * S.NH, S.L, x - cell_centre(S, cx), y - cell_centre(S, cy),
                         z - cell_centre(S, cz));
}

// Warp-cooperative FP64 helpers (one warp per point; lane m owns column m, L <= 32).
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// The regular solid harmonic diagonal Rg_m^m (x + i y) for the lane's column m.
__device__ __forceinline__ void rg_diag(const int m, const double x, const double y, double &re, double &im)
{
    re = 1.0;
    im = 0.0;
    for (int k = 1; k <= m; ++k) {
        const double t = c_rec_d[k];
        const double nre = t * (re * x - im * y);
        const double nim = t * (re * y + im * x);
        re = nre;
        im = nim;
    }
}

// Warp-parallel far_eval_fp64: lane m sums column m, the warp adds the columns.
__device__ double far_eval_warp(const double2 *__restrict__ Lc, const int L, const double x, const double y,
                                const double z)
{
    const int m = threadIdx.x & 31;
    double acc = 0.0;
    if (m < L) {
        const double r2 = x * x + y * y + z * z;
        double cre, cim, pre = 0.0, pim = 0.0;
        rg_diag(m, x, y, cre, cim);
        double2 Lv = Lc[hidx(m, m)];
        acc = Lv.x * cre - Lv.y * cim;
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
        if (m > 0) acc *= 2.0;
    }
    return warp_sum(acc);
}

// Warp-parallel multipole change: d[h(l,m)] += s q conj(Rg_l^m(x)), lane m writes column m.
__device__ void multipole_warp_add(double2 *d, const int L, const double sq, const double x, const double y,
                                   const double z, const bool first)
{
    const int m = threadIdx.x & 31;
    if (m < L) {
        const double r2 = x * x + y * y + z * z;
        double cre, cim, pre = 0.0, pim = 0.0;
        rg_diag(m, x, y, cre, cim);
        for (int l = m; l < L; ++l) {
            if (l > m) {
                const double az = c_rec_a[l * KMC_LMAX + m] * z;
                const double br = c_rec_b[l * KMC_LMAX + m] * r2;
                const double nre = az * cre - br * pre;
                const double nim = az * cim - br * pim;
                pre = cre;
                pim = cim;
                cre = nre;
                cim = nim;
            }
            const double2 v = make_double2(sq * cre, -sq * cim);
            double2 &o = d[hidx(l, m)];
            o = first ? v : make_double2(o.x + v.x, o.y + v.y);
        }
    }
    __syncwarp();
}
