// Part of the kmc_gb300.cu translation unit (included there, in order, inside its
// anonymous namespace unless it says otherwise): the allocation-free explicit-moves kernels (fixed device scratch, validated inputs).
#pragma once
// ---------------------------------------------------------------------------
// Allocation-free variant of the explicit-moves path (kmc_propose_moves_noalloc).
// Its scratch is a fixed file-scope device array instead of handle buffers:
//   g    [NHMAX] double2   far-field lattice vector A M (pbc)
//   u0   [MAX_MOVERS]      old-side energy of each moving charge
//   flag [1] int           0: the call's ids and offsets are valid
// Every element a call reads is written earlier in the same call.  Inputs are
// validated on the device before anything is read through them: ids outside
// [0, N), offsets that do not start at 0, decrease or end at another total than
// `total` make every output NaN; a proposed position outside the box, not
// finite or beyond max_move makes that proposal's output NaN.  Each rejected
// call or proposal is counted in the handle's bad-move counter (kmc_get_error).
// One warp per proposal: the near field over the 27 cells, the cell expansion
// (one m column per lane) and, for pbc, the moved charge's multipole change in
// shared memory with the lattice form's rows split over the lanes.
// ---------------------------------------------------------------------------
#define KMC_NOALLOC_MAX_MOVERS 4096
#define KMC_NOALLOC_MAX_PROPOSALS 16384
#define KMC_NOALLOC_NHMAX (KMC_LMAX * (KMC_LMAX + 1) / 2)
#define KMC_NOALLOC_G_OFF 0
#define KMC_NOALLOC_U0_OFF (KMC_NOALLOC_NHMAX * 16)
#define KMC_NOALLOC_FLAG_OFF (KMC_NOALLOC_U0_OFF + KMC_NOALLOC_MAX_MOVERS * 8)
#define KMC_NOALLOC_BYTES (KMC_NOALLOC_FLAG_OFF + 256)
constexpr int kNaWarps = 4;  // warps (proposals) per block of k_na_new

static __device__ __align__(256) unsigned char g_noalloc_scratch[KMC_NOALLOC_BYTES];

// Validation of the ids and offsets (one block), then g = A M (pbc) by the same block.
__global__ void k_na_prep(const Sys S, const int nump, const int total, const long long *__restrict__ pids,
                          const long long *__restrict__ es, double2 *g, int *flag, unsigned long long *err)
{
    int bad = 0;
    for (int o = threadIdx.x; o < nump; o += blockDim.x) {
        const long long px = pids[o];
        if (px < 0 || px >= S.N) bad = 1;
        if (es[o + 1] < es[o]) bad = 1;
    }
    if (threadIdx.x == 0 && (es[0] != 0 || es[nump] != total)) bad = 1;
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) {
        *flag = bad;
        if (bad) atomicAdd(err, 1ull);
    }
    if (bad || !S.pbc) return;
    for (int r = threadIdx.x; r < S.NH; r += blockDim.x) {
        double t = 0.0, u = 0.0;
        for (int k = S.ar_ptr[r]; k < S.ar_ptr[r + 1]; ++k) t += S.ar_val[k] * S.mpole[S.ar_col[k]].x;
        for (int k = S.ai_ptr[r]; k < S.ai_ptr[r + 1]; ++k) u += S.ai_val[k] * S.mpole[S.ai_col[k]].y;
        g[r] = make_double2(t, u);
    }
}

__global__ void k_na_old(const Sys S, const int nump, const long long *pids, double *u0, const int *flag)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nump || *flag) return;
    const int px = (int)pids[o];
    const double x = S.pos[3 * (size_t)px], y = S.pos[3 * (size_t)px + 1], z = S.pos[3 * (size_t)px + 2];
    const int cell = S.pcell[px];
    const int cx = cell % S.n, cy = (cell / S.n) % S.n, cz = cell / (S.n * S.n);
    u0[o] = S.q[px] * near_sum_fp64<true>(S, x, y, z, cx, cy, cz, px) + S.q[px] * far_at(S, cell, x, y, z);
}

// check_move with non-finite coordinates counted as outside the box.
__device__ __forceinline__ int na_check_move(const Sys &S, const double *p, const double *pp)
{
    int bad = 0;
    for (int d = 0; d < 3; ++d)
        if (!(pp[d] >= -0.5 * S.E && pp[d] <= 0.5 * S.E)) ++bad;
    return bad ? bad : check_move(S, p, pp);
}

__global__ void __launch_bounds__(kNaWarps * 32) k_na_new(const Sys S, const int nump, const int total,
                                                           const long long *__restrict__ pids,
                                                           const long long *__restrict__ es,
                                                           const double *__restrict__ newpos,
                                                           const double *__restrict__ u0,
                                                           const double2 *__restrict__ g, const int *flag,
                                                           unsigned long long *err, double *out)
{
    extern __shared__ double2 na_sh[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int p = blockIdx.x * kNaWarps + wid;
    if (p >= total) return;
    if (*flag) {
        if (lane == 0) out[p] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    int lo = 0, hi = nump - 1;  // owner: es[o] <= p < es[o+1] (offsets validated)
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (es[mid] <= p) lo = mid; else hi = mid - 1;
    }
    const int o = lo;
    const int px = (int)pids[o];
    const double *pp = newpos + 3 * (size_t)p;
    const double *op = S.pos + 3 * (size_t)px;
    const int bad = na_check_move(S, op, pp);
    if (bad) {
        if (lane == 0) {
            out[p] = __longlong_as_double(0x7ff8000000000000ll);
            atomicAdd(err, (unsigned long long)bad);
        }
        return;
    }
    const double x = pp[0], y = pp[1], z = pp[2];
    const double ox = op[0], oy = op[1], oz = op[2];
    const int cell = bin_cell(x, y, z, S);
    const int cx = cell % S.n, cy = (cell / S.n) % S.n, cz = cell / (S.n * S.n);
    const double q = S.q[px];
    // near field: the lanes split each neighbour cell's charges
    double nf = 0.0;
    for (int k = 0; k < 27; ++k) {
        int nx = cx + (k % 3) - 1, ny = cy + ((k / 3) % 3) - 1, nz = cz + (k / 9) - 1;
        double sx = 0.0, sy = 0.0, sz = 0.0;
        if (nx < 0 || nx >= S.n || ny < 0 || ny >= S.n || nz < 0 || nz >= S.n) {
            if (!S.periodic) continue;
            if (nx < 0) { nx += S.n; sx = -S.E; } else if (nx >= S.n) { nx -= S.n; sx = S.E; }
            if (ny < 0) { ny += S.n; sy = -S.E; } else if (ny >= S.n) { ny -= S.n; sy = S.E; }
            if (nz < 0) { nz += S.n; sz = -S.E; } else if (nz >= S.n) { nz -= S.n; sz = S.E; }
        }
        const int c = nx + S.n * (ny + S.n * nz);
        const int cn = S.cnt[c];
        const double4_32a *st = S.store + (size_t)c * S.cap;
        for (int j = lane; j < cn; j += 32) {
            const double4_32a v = st[j];
            const double dx = x - (v.x + sx), dy = y - (v.y + sy), dz = z - (v.z + sz);
            nf += v.w * rsqrt(dx * dx + dy * dy + dz * dz);
        }
    }
    nf = warp_sum(nf);
    const double ff = far_eval_warp(S.lexp + (size_t)cell * S.NH, S.L, x - cell_centre(S, cx),
                                    y - cell_centre(S, cy), z - cell_centre(S, cz));
    // moved-pair self term: lane k < 27 takes image k
    double st = 0.0;
    if (!S.periodic) {
        if (lane == 0) {
            const double dx = ox - x, dy = oy - y, dz = oz - z;
            st = rsqrt(dx * dx + dy * dy + dz * dz);
        }
    } else if (lane < 27) {
        const int a = lane % 3 - 1, b = (lane / 3) % 3 - 1, c = lane / 9 - 1;
        const double dx = (S.E * a + ox) - x, dy = (S.E * b + oy) - y, dz = (S.E * c + oz) - z;
        st = rsqrt(dx * dx + dy * dy + dz * dz);
    }
    st = warp_sum(st);
    if (S.periodic) st += S.dom27;
    double d = (q * nf + q * ff) - q * q * st - u0[o];
    if (S.pbc) {
        // dE_LR = delta.g + 1/2 delta^T A delta, delta = q m(x_new) - q m(x_old)
        double2 *a = na_sh + (size_t)wid * S.NH;
        multipole_warp_add(a, S.L, q, x, y, z, true);
        multipole_warp_add(a, S.L, -q, ox, oy, oz, false);
        double lin = 0.0, quad = 0.0;
        for (int r = lane; r < S.NH; r += 32) {
            const double2 ar = a[r];
            lin += ar.x * g[r].x + ar.y * g[r].y;
            double t = 0.0, u = 0.0;
            for (int k = S.aru_ptr[r]; k < S.aru_ptr[r + 1]; ++k) t += S.aru_val[k] * a[S.aru_col[k]].x;
            for (int k = S.aiu_ptr[r]; k < S.aiu_ptr[r + 1]; ++k) u += S.aiu_val[k] * a[S.aiu_col[k]].y;
            quad += ar.x * t + ar.y * u;
        }
        d += warp_sum(lin) + 0.5 * warp_sum(quad);
    }
    if (lane == 0) out[p] = S.unit * d;
}
