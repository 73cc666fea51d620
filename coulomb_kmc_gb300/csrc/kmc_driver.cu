// Device-side KMC driver around one kmc_system: proposal generation,
// selection and lattice occupancy on the GPU, so that a full KMC step
// (generate -> propose_with_dats -> select -> accept) runs without a host
// round trip and can be captured as one CUDA graph.
//
// It replaces the host bookkeeping of the reference's example driver
// (examples/propose_with_dats_example.py:218-446: hop proposals to the six
// nearest-neighbour sites, occupied-site masks, rates exp(-beta dE / 2),
// cumulative-sum selection) and the Metropolis loops of its tests
// (tests/host/test_free_space_1.py).
//
// Random numbers: Philox4x32-10 keyed by the seed; counter words
// (step low, step high, index, attempt << 4 | tag), so every draw is a pure
// function of (seed, step, index) and independent of launch shapes.
#include "kmc_gb300.h"
#include "kmc_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <new>
#include <thread>
#include <vector>

// a failed CUDA call: its name and error string for kmc_last_error, then KMC_ECUDA
#define DRV_CUDA(call)                                                                                             \
    do {                                                                                                           \
        const cudaError_t e_ = (call);                                                                             \
        if (e_ != cudaSuccess) {                                                                                   \
            kmc_int_set_error(#call, (int)e_);                                                                     \
            return KMC_ECUDA;                                                                                      \
        }                                                                                                          \
    } while (0)

namespace {

constexpr int kGenThreads = 128;
// Entries per partial sum, one per thread of a selection block.  256 spreads the
// FP64 exp (about 19 SM cycles per warp instruction on this part) evenly: a
// 165,888-entry step makes 648 blocks, 4.3 per SM.
constexpr int kSelChunk = 256;
constexpr int kPickThreads = kSelChunk;
constexpr int kMaxAttempts = 32;                      // re-draws of an off-lattice move that left the box

enum { TAG_DISP_XY = 1, TAG_DISP_Z = 2, TAG_SELECT = 3 };

struct P4 {
    uint32_t v[4];
};

// Philox4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC11): ten rounds, each two 32x32->64-bit products of the
// counter words 0 and 2 with the published multipliers, the key bumped by the
// published Weyl constants between rounds.
__host__ __device__ inline P4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return P4{{c0, c1, c2, c3}};
}

// uniform in [0, 1) with 53 random bits
__host__ __device__ inline double u53(const uint32_t a, const uint32_t b)
{
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

struct Key {
    uint32_t k0, k1;
};

__device__ __forceinline__ P4 draw(const Key k, const long long step, const uint32_t index, const uint32_t word3)
{
    return philox((uint32_t)step, (uint32_t)((unsigned long long)step >> 32), index, word3, k.k0, k.k1);
}

// ---------------------------------------------------------------------------
// proposal generation
// ---------------------------------------------------------------------------
// hop order +x, -x, +y, -y, +z, -z (examples/propose_with_dats_example.py:265-290);
// periodic systems wrap, a free-space lattice masks hops that leave it
// one thread per (charge, hop): the six nearest-neighbour sites of each charge,
// the hop's mask (target inside the box, vacant) and the target's centre
// every site's centre (explicit roundings, no contraction, so that host code
// reproduces the positions bit for bit)
__global__ void k_site_centres(const int nsites, const int side, const double spacing, const double half_e,
                               double *centre)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsites) return;
    const int t[3] = {s % side, (s / side) % side, s / (side * side)};
    for (int a = 0; a < 3; ++a)
        centre[3 * (size_t)s + a] =
            __dadd_rn(__dsub_rn(__dmul_rn((double)t[a], spacing), half_e), __dmul_rn(0.5, spacing));
}

// hop h of charge i: target site, mask (vacant and inside the box), the site's
// centre and cell from the tables built at creation
__global__ void k_lat_gen(const int N, const int side, const int wrap, const int *__restrict__ site_of,
                          const int *__restrict__ occ, const double *__restrict__ site_centre,
                          const int *__restrict__ site_cell, double *ppos, long long *masks, int *tsite, int *pcell)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= 6 * N) return;
    const int i = g / 6, h = g - 6 * i;
    const int s = site_of[i];
    int t[3] = {s % side, (s / side) % side, s / (side * side)};
    const int ax = h >> 1, dir = (h & 1) ? -1 : 1;
    t[ax] += dir;
    bool ok = true;
    if (t[ax] < 0 || t[ax] >= side) {
        if (wrap)
            t[ax] = (t[ax] + side) % side;
        else
            ok = false;
    }
    const int ts = ok ? t[0] + side * (t[1] + side * t[2]) : s;
    tsite[g] = ts;
    masks[g] = (ok && occ[ts] < 0) ? 1 : 0;
    double *o = ppos + 3 * (size_t)g;
    o[0] = site_centre[3 * (size_t)ts];
    o[1] = site_centre[3 * (size_t)ts + 1];
    o[2] = site_centre[3 * (size_t)ts + 2];
    pcell[g] = site_cell[ts];
}

// one displacement uniform in [-step, step]^3 per charge, re-drawn while it
// leaves the box (at most kMaxAttempts draws, else a null move)
__global__ void k_off_gen(const int N, const double half_e, const double step, const double *__restrict__ pos,
                          const Key key, const long long *__restrict__ counters, double *ppos)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const long long st = counters[0];
    const double x0 = pos[3 * (size_t)i], y0 = pos[3 * (size_t)i + 1], z0 = pos[3 * (size_t)i + 2];
    double nx = x0, ny = y0, nz = z0;
    for (int a = 0; a < kMaxAttempts; ++a) {
        const P4 A = draw(key, st, (uint32_t)i, ((uint32_t)a << 4) | TAG_DISP_XY);
        const P4 B = draw(key, st, (uint32_t)i, ((uint32_t)a << 4) | TAG_DISP_Z);
        // x0 + (2u - 1) step with explicit roundings (reproducible on the host)
        const double tx = __dadd_rn(x0, __dmul_rn(__dsub_rn(__dmul_rn(2.0, u53(A.v[0], A.v[1])), 1.0), step));
        const double ty = __dadd_rn(y0, __dmul_rn(__dsub_rn(__dmul_rn(2.0, u53(A.v[2], A.v[3])), 1.0), step));
        const double tz = __dadd_rn(z0, __dmul_rn(__dsub_rn(__dmul_rn(2.0, u53(B.v[0], B.v[1])), 1.0), step));
        if (fabs(tx) <= half_e && fabs(ty) <= half_e && fabs(tz) <= half_e) {
            nx = tx;
            ny = ty;
            nz = tz;
            break;
        }
    }
    ppos[3 * (size_t)i] = nx;
    ppos[3 * (size_t)i + 1] = ny;
    ppos[3 * (size_t)i + 2] = nz;
}

__global__ void k_fill_i64(long long *p, const long long n, const long long v)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

// ---------------------------------------------------------------------------
// rejection-free selection: rate_e = exp(-beta dE_e / 2) on unmasked entries,
// pick the first entry whose running sum exceeds u * total
// ---------------------------------------------------------------------------
__device__ __forceinline__ double rate_of(const long long e, const long long n, const double *diffs,
                                          const long long *masks, const double hb)
{
    return (e < n && masks[e]) ? exp(-hb * diffs[e]) : 0.0;
}

// inclusive scan of v[0..kPickThreads) in place: shuffle scans within warps, then
// over the warp totals (fixed order, deterministic)
__device__ void block_scan(double *v)
{
    __shared__ double wsum[kPickThreads / 32];
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    double x = v[t];
    for (int off = 1; off < 32; off <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
        double w = lane < kPickThreads / 32 ? wsum[lane] : 0.0;
        for (int off = 1; off < 32; off <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        if (lane < kPickThreads / 32) wsum[lane] = w;
    }
    __syncthreads();
    if (wid > 0) x += wsum[wid - 1];
    v[t] = x;
    __syncthreads();
}

struct SelOut {
    long long *pid;     // [1]
    double *pos;        // [3]
    double *de;         // [1]
    long long *counters;  // [0] steps, [1] accepted, [2] proposals evaluated
    long long *log_pid, *log_tgt;
    double *log_de;
    long long log_cap;
};

__device__ void log_step(const SelOut &o, const long long st, const long long pid, const long long tgt, const double de)
{
    if (o.log_cap > 0) {
        const long long k = st % o.log_cap;
        o.log_pid[k] = pid;
        o.log_tgt[k] = tgt;
        o.log_de[k] = de;
    }
}

// The pick, run by the last selection block to finish: the partial sums and the
// rates of the other blocks are read through L2 (__ldcg), after their writers'
// __threadfence.
__device__ void rate_pick(const long long n, const int nb, const int M, const double *__restrict__ diffs,
                          const double *rates, const double *part, const double *__restrict__ ppos, const Key key,
                          const SelOut &o, int *site_of, int *occ, const int *__restrict__ tsite)
{
    __shared__ double sc[kPickThreads];
    __shared__ double s_target, s_base;
    __shared__ int s_blk, s_first, s_last;
    const int t = threadIdx.x;
    const long long st = o.counters[0];
    // runs of partial sums, one contiguous run per thread
    const int per = (nb + kPickThreads - 1) / kPickThreads;
    const int b0 = min(nb, t * per), b1 = min(nb, b0 + per);
    double run = 0.0;
    for (int b = b0; b < b1; ++b) run += __ldcg(part + b);
    sc[t] = run;
    if (t == 0) {
        s_blk = -1;
        s_first = 0x7fffffff;
        s_last = -1;
    }
    __syncthreads();
    block_scan(sc);
    const double total = sc[kPickThreads - 1];
    if (t == 0) {
        const P4 r = draw(key, st, 0u, TAG_SELECT);
        s_target = __dmul_rn(u53(r.v[0], r.v[1]), total);
    }
    __syncthreads();
    const double target = s_target;
    {
        const double excl = t ? sc[t - 1] : 0.0;
        if (b1 > b0 && excl <= target && target < sc[t]) {
            double acc = excl;
            for (int b = b0; b < b1; ++b) {
                const double pb = __ldcg(part + b);
                if (acc + pb > target && pb > 0.0) {
                    s_blk = b;
                    s_base = acc;
                    break;
                }
                acc += pb;
            }
        }
    }
    __syncthreads();
    if (s_blk < 0 && t == 0) {
        // target at or beyond the rounded total: the last block with a non-zero rate
        double acc = 0.0;
        for (int b = 0; b < nb; ++b) {
            const double pb = __ldcg(part + b);
            if (pb > 0.0) {
                s_blk = b;
                s_base = acc;
            }
            acc += pb;
        }
        if (s_blk < 0) s_blk = 0;
    }
    __syncthreads();
    const long long e = (long long)s_blk * kSelChunk + t;
    const double r = e < n ? __ldcg(rates + e) : 0.0;
    __syncthreads();
    sc[t] = r;
    __syncthreads();
    block_scan(sc);
    if (r > 0.0 && s_base + sc[t] > target) atomicMin(&s_first, t);
    if (r > 0.0) atomicMax(&s_last, t);
    __syncthreads();
    if (t == 0) {
        const int pick = (s_first != 0x7fffffff) ? s_first : s_last;
        if (pick < 0) {
            // no unmasked proposal at all: no move this step
            o.pid[0] = -1;
            o.de[0] = 0.0;
            log_step(o, st, -1, -1, 0.0);
        } else {
            const long long idx = (long long)s_blk * kSelChunk + pick;
            const int pid = (int)(idx / M);
            o.pid[0] = pid;
            o.pos[0] = ppos[3 * idx];
            o.pos[1] = ppos[3 * idx + 1];
            o.pos[2] = ppos[3 * idx + 2];
            o.de[0] = diffs[idx];
            if (site_of) {
                const int ns = tsite[idx];
                occ[site_of[pid]] = -1;
                occ[ns] = pid;
                site_of[pid] = ns;
                log_step(o, st, pid, ns, diffs[idx]);
            } else {
                log_step(o, st, pid, -1, diffs[idx]);
            }
            o.counters[1] += 1;
        }
        o.counters[0] = st + 1;
    }
}

// Rejection-free selection in one launch: block b computes rate_e =
// exp(-beta dE_e / 2) for its kSelChunk entries (0 where masked), stores them and
// their sum part[b] (fixed-order reduction); the last block to finish (ticket)
// scans the partial sums and picks.  No block waits on another.
__global__ void __launch_bounds__(kSelChunk) k_rate_select(const long long n, const int M,
                                                           const double *__restrict__ diffs,
                                                           const long long *__restrict__ masks, const double hb,
                                                           double *part, double *rates, const double *__restrict__ ppos,
                                                           const Key key, SelOut o, int *site_of, int *occ,
                                                           const int *__restrict__ tsite, unsigned int *ticket)
{
    __shared__ double wsum[kSelChunk / 32];
    __shared__ bool last;
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    const int nb = gridDim.x;
    const long long e = (long long)blockIdx.x * kSelChunk + t;
    const bool on = e < n && masks[e] > 0;
    const double r = on ? exp(-hb * diffs[e]) : 0.0;
    if (e < n) rates[e] = r;
    __threadfence();
    const int na = __syncthreads_count(on);
    double x = r;
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    if (lane == 0) wsum[wid] = x;
    __syncthreads();
    if (t == 0) {
        double b = 0.0;
        for (int w = 0; w < kSelChunk / 32; ++w) b += wsum[w];
        part[blockIdx.x] = b;
        atomicAdd((unsigned long long *)&o.counters[2], (unsigned long long)na);
        __threadfence();
        const unsigned int k = atomicAdd(ticket, 1u);
        last = (k == (unsigned int)nb - 1);
        if (last) *ticket = 0u;  // every block has taken its ticket: reset for the next step
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    rate_pick(n, nb, M, diffs, rates, part, ppos, key, o, site_of, occ, tsite);
}

// Metropolis on one uniformly chosen charge: accept its proposal with
// probability min(1, exp(-beta dE))
__global__ void k_metropolis(const int N, const double beta, const double *__restrict__ diffs,
                             const double *__restrict__ ppos, const Key key, SelOut o)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const long long st = o.counters[0];
    const P4 r = draw(key, st, 0u, TAG_SELECT);
    int i = (int)__dmul_rn(u53(r.v[0], r.v[1]), (double)N);
    if (i >= N) i = N - 1;
    const double de = diffs[i];
    const bool acc = de <= 0.0 || u53(r.v[2], r.v[3]) < exp(-beta * de);
    o.pid[0] = acc ? i : -1;
    o.pos[0] = ppos[3 * (size_t)i];
    o.pos[1] = ppos[3 * (size_t)i + 1];
    o.pos[2] = ppos[3 * (size_t)i + 2];
    o.de[0] = de;
    log_step(o, st, acc ? i : -1, i, de);
    if (acc) o.counters[1] += 1;
    o.counters[2] += N;
    o.counters[0] = st + 1;
}

template <typename T>
bool dmalloc(T **p, size_t n)
{
    return cudaMalloc((void **)p, sizeof(T) * (n ? n : 1)) == cudaSuccess;
}

} // namespace

struct kmc_driver {
    kmc_system *sys = nullptr;
    kmc_driver_params prm{};
    int N = 0, M = 1, side = 0, wrap = 0;
    double E = 0.0, spacing = 1.0;
    Key key{};
    double *ppos = nullptr, *diffs = nullptr, *part = nullptr, *rates = nullptr;
    long long *masks = nullptr, *smc = nullptr, *sites = nullptr;
    int *tsite = nullptr, *site_of = nullptr, *occ = nullptr;
    double *site_centre = nullptr;   // lattice: [nsites][3] site centres
    int *site_cell = nullptr;        // lattice: the system's cell of each site
    int *pcell = nullptr;            // lattice: [N * 6] cell of each hop's target
    unsigned int *ticket = nullptr;  // selection blocks finished this step (k_rate_select)
    bool prepared = false;           // proposals of the current state generated and set up
    int64_t seen = -1;               // the system's launch count when they were
    bool graph_pipelined = false;    // the captured step is the pipelined form
    long long *sel_pid = nullptr, *counters = nullptr, *log_pid = nullptr, *log_tgt = nullptr;
    double *sel_pos = nullptr, *sel_de = nullptr, *log_de = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<void *> owned;
    // store headroom: a step moves one charge, so a cell's occupancy grows by at most
    // one per step; `budget` steps may run before the occupancy is read again (< 0:
    // the store can never overflow, e.g. a lattice whose cells hold fewer sites than
    // the store has slots)
    int64_t budget = 0;
    int64_t layout = -1;            // the system's buffer layout the captured graph reads
    int64_t graph_version = 0;      // advances at every capture (size-bucket graphs embed the step)
    cudaEvent_t ev_last = nullptr;  // after the driver's last enqueued step
    bool ev_recorded = false;
    cudaStream_t own_stream = nullptr;  // for re-capturing the step after a store growth
};

namespace {

template <typename T>
bool own(kmc_driver *d, T **p, size_t n)
{
    if (!dmalloc(p, n)) return false;
    d->owned.push_back((void *)*p);
    return true;
}

// Proposal generation and set-up for the next step on stream st: the hops (or
// displacements) of the current state, compacted and grouped by target cell.
int enqueue_prepare(kmc_driver *d, cudaStream_t st)
{
    const int N = d->N;
    const double half_e = 0.5 * d->E;
    if (d->prm.kind == KMC_DRIVE_LATTICE)
        k_lat_gen<<<(unsigned)((6 * (long long)N + kGenThreads - 1) / kGenThreads), kGenThreads, 0, st>>>(
            N, d->side, d->wrap, d->site_of, d->occ, d->site_centre, d->site_cell, d->ppos, d->masks, d->tsite,
            d->pcell);
    else
        k_off_gen<<<(unsigned)((N + kGenThreads - 1) / kGenThreads), kGenThreads, 0, st>>>(
            N, half_e, d->prm.step, kmc_int_positions(d->sys), d->key, d->counters, d->ppos);
    DRV_CUDA(cudaGetLastError());
    return kmc_int_propose_prepare(d->sys, (void *)st, N, d->M, (const int64_t *)d->smc, (const int64_t *)d->sites,
                                   d->ppos, (const int64_t *)d->masks, d->pcell);
}

int prepare_branch(void *ctx, void *stream) { return enqueue_prepare((kmc_driver *)ctx, (cudaStream_t)stream); }

// Pipelined steps (the default beside the double-FP32 accept): the next step's
// set-up runs beside the accept.  Plain order for FP64 accepts, whose
// particle-to-local blocks fill whole SMs with shared memory: set-up kernels
// interleaved with them delay them (0.73 -> 0.95 ms per step on the 48^3
// lattice), while beside the double-FP32 accept they hide (0.38 -> 0.31 ms).
bool pipelined(const kmc_driver *d)
{
    const int t = kmc_int_tuning(d->sys, KMC_TUNE_DRIVER_SERIAL);
    return t == 2 || (t == 0 && kmc_int_accept_df32(d->sys));
}

// before a replay or capture of a pipelined step: it expects prepared proposals
int ensure_prepared(kmc_driver *d, cudaStream_t st)
{
    if (d->prepared && d->seen == kmc_int_launches(d->sys)) return KMC_OK;
    const int rc = enqueue_prepare(d, st);
    if (rc) return rc;
    d->prepared = true;
    d->seen = kmc_int_launches(d->sys);
    return KMC_OK;
}

// One step, software-pipelined: the proposals of this step were prepared at the
// end of the previous one (or are prepared here when anything else has launched
// work on the system since); evaluate, select, then accept with the next step's
// generation and set-up beside the accept's expansion updates.  Every kernel
// sees the same inputs as in the plain order generate -> propose -> select ->
// accept, so the results are the same.
int enqueue_step(kmc_driver *d, cudaStream_t st)
{
    const int N = d->N;
    SelOut o{d->sel_pid, d->sel_pos, d->sel_de, d->counters, d->log_pid, d->log_tgt, d->log_de, d->prm.log_capacity};
    int rc;
    const bool pipe = pipelined(d);
    if (!pipe || !d->prepared || d->seen != kmc_int_launches(d->sys))
        if ((rc = enqueue_prepare(d, st))) return rc;
    if ((rc = kmc_int_propose_evaluate(d->sys, N, d->M, d->diffs))) return rc;
    if (d->prm.kind == KMC_DRIVE_LATTICE) {
        const long long n = (long long)N * d->M;
        const int nb = (int)((n + kSelChunk - 1) / kSelChunk);
        const double hb = 0.5 * d->prm.beta;
        k_rate_select<<<nb, kSelChunk, 0, st>>>(n, d->M, d->diffs, d->masks, hb, d->part, d->rates, d->ppos, d->key,
                                                o, d->site_of, d->occ, d->tsite, d->ticket);
    } else {
        k_metropolis<<<1, 32, 0, st>>>(N, d->prm.beta, d->diffs, d->ppos, d->key, o);
    }
    DRV_CUDA(cudaGetLastError());
    d->prepared = false;
    if (!pipe) {
        // plain order: the next step prepares at its start
        return kmc_accept_device(d->sys, (const int64_t *)d->sel_pid, d->sel_pos, d->sel_de);
    }
    // lattice hops: the next step's set-up reads only the driver's buffers (updated by
    // the selection) and the charges, so it can start beside k_accept_prep
    if ((rc = kmc_int_accept_device_branch(d->sys, (const int64_t *)d->sel_pid, d->sel_pos, d->sel_de,
                                           prepare_branch, d, d->prm.kind == KMC_DRIVE_LATTICE)))
        return rc;
    d->prepared = true;
    d->seen = kmc_int_launches(d->sys);
    return KMC_OK;
}

void release(kmc_driver *d)
{
    if (d->exec) cudaGraphExecDestroy(d->exec);
    if (d->graph) cudaGraphDestroy(d->graph);
    if (d->ev_last) cudaEventDestroy(d->ev_last);
    if (d->own_stream) cudaStreamDestroy(d->own_stream);
    for (void *p : d->owned) cudaFree(p);
    delete d;
}

int capture_on(kmc_driver *d, cudaStream_t st);

// Before enqueuing n steps: make sure no cell store can fill during them.  When the
// budget is spent, wait for the driver's queued steps, read the largest cell
// occupancy and, if fewer than n free slots remain in some cell, grow the store
// (the reference grows it when a cell fills, kmc_local.py:318-326; growing earlier
// changes no result); a captured step reads the store's buffers, so it is captured
// again after a growth.
int ensure_headroom(kmc_driver *d, int64_t n)
{
    if (d->budget < 0) return KMC_OK;
    if (d->budget >= n) {
        d->budget -= n;
        return KMC_OK;
    }
    if (d->ev_recorded) DRV_CUDA(cudaEventSynchronize(d->ev_last));
    int64_t mx = 0, cap = 0;
    int rc = kmc_max_occupancy(d->sys, &mx, &cap);
    if (rc) return rc;
    if (cap - mx < n) {
        if ((rc = kmc_store_reserve(d->sys, mx + (n > cap ? n : cap)))) return rc;
        if ((rc = kmc_max_occupancy(d->sys, &mx, &cap))) return rc;
    }
    d->budget = cap - mx - n;
    if (d->exec && d->layout != kmc_int_layout_gen(d->sys)) return capture_on(d, d->own_stream);
    return KMC_OK;
}

// the step enqueued on st (stream-ordered with the driver's previous work): for the
// headroom check
int mark_enqueued(kmc_driver *d, cudaStream_t st)
{
    DRV_CUDA(cudaEventRecord(d->ev_last, st));
    d->ev_recorded = true;
    return KMC_OK;
}

} // namespace

int kmc_driver_create(kmc_system *s, const kmc_driver_params *p, kmc_driver **out)
{
    if (!s || !p || !out) return KMC_EINVAL;
    *out = nullptr;
    if (!kmc_int_initialised(s)) return KMC_ESTATE;
    if ((p->kind != KMC_DRIVE_LATTICE && p->kind != KMC_DRIVE_OFFLATTICE) || !(p->beta >= 0.0) ||
        p->log_capacity < 0)
        return KMC_EINVAL;
    const int N = kmc_int_n(s);
    const double E = kmc_int_extent(s), max_move = kmc_int_max_move(s);
    kmc_driver *d = new (std::nothrow) kmc_driver;
    if (!d) return KMC_ENOMEM;
    d->sys = s;
    d->prm = *p;
    d->prm.lattice_sites = nullptr;
    d->N = N;
    d->E = E;
    d->key = Key{(uint32_t)p->seed, (uint32_t)(p->seed >> 32)};
    cudaStream_t st = kmc_int_stream(s);
    if (p->kind == KMC_DRIVE_LATTICE) {
        if (p->lattice_side < 2 || !p->lattice_sites) {
            delete d;
            return KMC_EINVAL;
        }
        d->M = 6;
        d->side = p->lattice_side;
        d->spacing = E / p->lattice_side;
        d->wrap = kmc_int_boundary(s) != KMC_BC_FREE_SPACE;
        if (d->spacing > max_move) {
            delete d;
            return KMC_EINVAL;
        }
        // the charges must sit on the sites given; every site holds at most one
        const long long nsites = (long long)d->side * d->side * d->side;
        std::vector<int> occ((size_t)nsites, -1), so(N);
        std::vector<double> pos(3 * (size_t)N);
        if (cudaMemcpyAsync(pos.data(), kmc_int_positions(s), sizeof(double) * pos.size(), cudaMemcpyDeviceToHost,
                            st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            delete d;
            return KMC_ECUDA;
        }
        for (int i = 0; i < N; ++i) {
            const long long site = p->lattice_sites[i];
            if (site < 0 || site >= nsites || occ[(size_t)site] >= 0) {
                delete d;
                return KMC_EINVAL;
            }
            occ[(size_t)site] = i;
            so[i] = (int)site;
            const long long c[3] = {site % d->side, (site / d->side) % d->side, site / ((long long)d->side * d->side)};
            for (int a = 0; a < 3; ++a) {
                const double want = ((double)c[a] * d->spacing - 0.5 * E) + 0.5 * d->spacing;
                if (fabs(pos[3 * (size_t)i + a] - want) > 1e-9 * (1.0 + fabs(E))) {
                    delete d;
                    return KMC_EINVAL;
                }
            }
        }
        if (!own(d, &d->site_of, N) || !own(d, &d->occ, (size_t)nsites) || !own(d, &d->tsite, 6 * (size_t)N) ||
            !own(d, &d->site_centre, 3 * (size_t)nsites) || !own(d, &d->site_cell, (size_t)nsites) ||
            !own(d, &d->pcell, 6 * (size_t)N)) {
            release(d);
            return KMC_ENOMEM;
        }
        k_site_centres<<<(unsigned)((nsites + 255) / 256), 256, 0, st>>>((int)nsites, d->side, d->spacing, 0.5 * E,
                                                                         d->site_centre);
        if (cudaGetLastError() != cudaSuccess ||
            kmc_int_bin_cells(s, (void *)st, nsites, d->site_centre, d->site_cell) != KMC_OK) {
            release(d);
            return KMC_ECUDA;
        }
        std::vector<int> scell((size_t)nsites);
        if (cudaMemcpyAsync(d->site_of, so.data(), sizeof(int) * N, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaMemcpyAsync(d->occ, occ.data(), sizeof(int) * occ.size(), cudaMemcpyHostToDevice, st) !=
                cudaSuccess ||
            cudaMemcpyAsync(scell.data(), d->site_cell, sizeof(int) * scell.size(), cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            release(d);
            return KMC_ECUDA;
        }
        // a cell never holds more charges than it has sites: with that many slots the
        // store cannot overflow and no step needs an occupancy check
        std::vector<int> per((size_t)kmc_int_ncell(s), 0);
        int most = 0;
        for (int c : scell) most = std::max(most, ++per[(size_t)c]);
        int64_t mx = 0, cap = 0;
        int rc0 = kmc_max_occupancy(s, &mx, &cap);
        if (!rc0 && cap < most) rc0 = kmc_store_reserve(s, most);
        if (rc0) {
            release(d);
            return rc0;
        }
        d->budget = -1;
    } else {
        if (!(p->step > 0.0) || p->step > max_move) {
            delete d;
            return KMC_EINVAL;
        }
        d->M = 1;
    }
    const size_t nm = (size_t)N * d->M;
    const int nb = (int)((nm + kSelChunk - 1) / kSelChunk);
    const size_t lc = (size_t)p->log_capacity;
    if (!own(d, &d->ppos, 3 * nm) || !own(d, &d->diffs, nm) || !own(d, &d->rates, nm) || !own(d, &d->masks, nm) ||
        !own(d, &d->smc, 1) ||
        !own(d, &d->sites, N) || !own(d, &d->part, nb) || !own(d, &d->sel_pid, 1) || !own(d, &d->sel_pos, 3) ||
        !own(d, &d->sel_de, 1) || !own(d, &d->counters, 3) || !own(d, &d->log_pid, lc) || !own(d, &d->log_tgt, lc) ||
        !own(d, &d->log_de, lc) || !own(d, &d->ticket, 1)) {
        release(d);
        return KMC_ENOMEM;
    }
    // stream-ordered on the system's stream only: other threads may be capturing
    // graphs of other systems meanwhile, so nothing here touches the legacy stream
    // or synchronises the device
    const long long smc = d->M;
    bool ok = cudaMemcpyAsync(d->smc, &smc, sizeof(long long), cudaMemcpyHostToDevice, st) == cudaSuccess &&
              cudaMemsetAsync(d->sites, 0, sizeof(long long) * N, st) == cudaSuccess &&
              cudaMemsetAsync(d->counters, 0, sizeof(long long) * 3, st) == cudaSuccess &&
              cudaMemsetAsync(d->ticket, 0, sizeof(unsigned int), st) == cudaSuccess &&
              cudaMemsetAsync(d->diffs, 0, sizeof(double) * nm, st) == cudaSuccess;
    if (ok && p->kind == KMC_DRIVE_OFFLATTICE) {
        k_fill_i64<<<(unsigned)((nm + 255) / 256), 256, 0, st>>>(d->masks, (long long)nm, 1);
        ok = cudaGetLastError() == cudaSuccess;
    }
    ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
    if (!ok) {
        release(d);
        return KMC_ECUDA;
    }
    int rc = kmc_int_reserve(s, N, (int64_t)nm);
    if (rc) {
        release(d);
        return rc;
    }
    if (cudaEventCreateWithFlags(&d->ev_last, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&d->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        release(d);
        return KMC_ECUDA;
    }
    *out = d;
    return KMC_OK;
}

int kmc_driver_step(kmc_driver *d, int64_t nsteps)
{
    if (!d || nsteps < 0) return KMC_EINVAL;
    int rc = ensure_headroom(d, nsteps);
    if (rc) return rc;
    cudaStream_t st = kmc_int_stream(d->sys);
    for (int64_t k = 0; k < nsteps; ++k)
        if ((rc = enqueue_step(d, st))) return rc;
    return nsteps > 0 ? mark_enqueued(d, st) : KMC_OK;
}

int kmc_driver_capture(kmc_driver *d)
{
    if (!d) return KMC_EINVAL;
    cudaStream_t st = kmc_int_stream(d->sys);
    if (!st) return KMC_EINVAL;  // the legacy default stream cannot be captured
    return capture_on(d, st);
}

namespace {
int capture_core(kmc_driver *d, cudaStream_t st)
{
    if (d->exec) {
        cudaGraphExecDestroy(d->exec);
        d->exec = nullptr;
    }
    if (d->graph) {
        cudaGraphDestroy(d->graph);
        d->graph = nullptr;
    }
    d->graph_pipelined = pipelined(d);
    int rc = d->graph_pipelined ? ensure_prepared(d, st) : KMC_OK;
    if (rc) return rc;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return KMC_ECUDA;
    rc = enqueue_step(d, st);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        d->prepared = false;
        return rc ? rc : KMC_ECUDA;
    }
    d->graph = g;
    if (cudaGraphInstantiate(&d->exec, g, 0) != cudaSuccess) return KMC_ECUDA;
    d->layout = kmc_int_layout_gen(d->sys);
    d->graph_version++;
    return KMC_OK;
}

// capture one step on st, with the system bound to st meanwhile (then bound back)
int capture_on(kmc_driver *d, cudaStream_t st)
{
    cudaStream_t prev = kmc_int_stream(d->sys);
    if (st == prev) return capture_core(d, st);
    DRV_CUDA(cudaStreamSynchronize(prev));
    kmc_set_stream(d->sys, (void *)st);
    const int rc = capture_core(d, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    kmc_set_stream(d->sys, (void *)prev);
    if (rc) return rc;
    DRV_CUDA(e);
    return KMC_OK;
}
} // namespace

int kmc_driver_launch(kmc_driver *d, int64_t nsteps, void *stream)
{
    if (!d || nsteps < 0) return KMC_EINVAL;
    if (!d->exec) return KMC_ESTATE;
    int rc = ensure_headroom(d, nsteps);
    if (rc) return rc;
    cudaStream_t st = stream ? (cudaStream_t)stream : kmc_int_stream(d->sys);
    if ((rc = d->graph_pipelined ? ensure_prepared(d, st) : KMC_OK)) return rc;
    for (int64_t k = 0; k < nsteps; ++k)
        if (cudaGraphLaunch(d->exec, st) != cudaSuccess) return KMC_ECUDA;
    return nsteps > 0 ? mark_enqueued(d, st) : KMC_OK;
}

int kmc_driver_counters(kmc_driver *d, int64_t *steps_out, int64_t *accepted_out, int64_t *proposals_out)
{
    if (!d) return KMC_EINVAL;
    long long h[3];
    if (cudaStreamSynchronize(kmc_int_stream(d->sys)) != cudaSuccess) return KMC_ECUDA;
    if (cudaMemcpy(h, d->counters, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return KMC_ECUDA;
    if (steps_out) *steps_out = h[0];
    if (accepted_out) *accepted_out = h[1];
    if (proposals_out) *proposals_out = h[2];
    return KMC_OK;
}

int kmc_driver_log(kmc_driver *d, int64_t max_entries, int64_t *pid_out, int64_t *target_out, double *de_out,
                   int64_t *n_out)
{
    if (!d || max_entries < 0 || !n_out) return KMC_EINVAL;
    int64_t steps = 0;
    int rc = kmc_driver_counters(d, &steps, nullptr, nullptr);
    if (rc) return rc;
    const int64_t cap = d->prm.log_capacity;
    const int64_t have = steps < cap ? steps : cap;
    const int64_t n = have < max_entries ? have : max_entries;
    std::vector<long long> a((size_t)cap), b((size_t)cap);
    std::vector<double> c((size_t)cap);
    if (cap > 0 && (cudaMemcpy(a.data(), d->log_pid, sizeof(long long) * cap, cudaMemcpyDeviceToHost) != cudaSuccess ||
                    cudaMemcpy(b.data(), d->log_tgt, sizeof(long long) * cap, cudaMemcpyDeviceToHost) != cudaSuccess ||
                    cudaMemcpy(c.data(), d->log_de, sizeof(double) * cap, cudaMemcpyDeviceToHost) != cudaSuccess))
        return KMC_ECUDA;
    const int64_t first = steps - have;  // oldest step still in the log
    for (int64_t k = 0; k < n; ++k) {
        const size_t j = (size_t)((first + k) % (cap ? cap : 1));
        if (pid_out) pid_out[k] = a[j];
        if (target_out) target_out[k] = b[j];
        if (de_out) de_out[k] = c[j];
    }
    *n_out = n;
    return KMC_OK;
}

int kmc_driver_sites(kmc_driver *d, int64_t *sites_out)
{
    if (!d || !sites_out) return KMC_EINVAL;
    if (d->prm.kind != KMC_DRIVE_LATTICE) return KMC_EINVAL;
    std::vector<int> so(d->N);
    if (cudaStreamSynchronize(kmc_int_stream(d->sys)) != cudaSuccess) return KMC_ECUDA;
    if (cudaMemcpy(so.data(), d->site_of, sizeof(int) * d->N, cudaMemcpyDeviceToHost) != cudaSuccess)
        return KMC_ECUDA;
    for (int i = 0; i < d->N; ++i) sites_out[i] = so[i];
    return KMC_OK;
}

int kmc_driver_free(kmc_driver *d)
{
    if (!d) return KMC_EINVAL;
    cudaStreamSynchronize(kmc_int_stream(d->sys));
    release(d);
    return KMC_OK;
}

int kmc_host_displacements(int64_t n, const double *pos, double extent, double step, uint64_t seed, int64_t round,
                           double *out, int32_t nthreads)
{
    if (n < 0 || n >= ((int64_t)1 << 32) || (n > 0 && (!pos || !out)) || !(extent > 0.0) || !(step >= 0.0))
        return KMC_EINVAL;
    if (n > 0 && out < pos + 3 * n && pos < out + 3 * n) return KMC_EINVAL;
    const Key key{(uint32_t)seed, (uint32_t)(seed >> 32)};
    const double half_e = 0.5 * extent;
    auto work = [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; ++i) {
            const double x0 = pos[3 * i], y0 = pos[3 * i + 1], z0 = pos[3 * i + 2];
            double nx = x0, ny = y0, nz = z0;
            for (int at = 0; at < kMaxAttempts; ++at) {
                const P4 A = philox((uint32_t)round, (uint32_t)((uint64_t)round >> 32), (uint32_t)i,
                                    ((uint32_t)at << 4) | TAG_DISP_XY, key.k0, key.k1);
                const P4 B = philox((uint32_t)round, (uint32_t)((uint64_t)round >> 32), (uint32_t)i,
                                    ((uint32_t)at << 4) | TAG_DISP_Z, key.k0, key.k1);
                const double tx = x0 + (2.0 * u53(A.v[0], A.v[1]) - 1.0) * step;
                const double ty = y0 + (2.0 * u53(A.v[2], A.v[3]) - 1.0) * step;
                const double tz = z0 + (2.0 * u53(B.v[0], B.v[1]) - 1.0) * step;
                if (std::fabs(tx) <= half_e && std::fabs(ty) <= half_e && std::fabs(tz) <= half_e) {
                    nx = tx;
                    ny = ty;
                    nz = tz;
                    break;
                }
            }
            out[3 * i] = nx;
            out[3 * i + 1] = ny;
            out[3 * i + 2] = nz;
        }
    };
    const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(std::min(nthreads, 256), (n + 4095) / 4096));
    if (nt <= 1) {
        work(0, n);
        return KMC_OK;
    }
    std::vector<std::thread> th;
    try {
        th.reserve(nt);
        for (int t = 1; t < nt; ++t) th.emplace_back(work, n * t / nt, n * (t + 1) / nt);
    } catch (...) {
        // fewer threads than asked (the system refused one): the rest on this thread
        const int started = (int)th.size() + 1;
        work(0, n / nt);
        for (int t = started; t < nt; ++t) work(n * t / nt, n * (t + 1) / nt);
        for (auto &t : th) t.join();
        return KMC_OK;
    }
    work(0, n / nt);
    for (auto &t : th) t.join();
    return KMC_OK;
}

int kmc_stream_create(void **stream_out)
{
    if (!stream_out) return KMC_EINVAL;
    cudaStream_t st = nullptr;
    DRV_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    *stream_out = (void *)st;
    return KMC_OK;
}

int kmc_stream_destroy(void *stream)
{
    if (!stream) return KMC_EINVAL;
    DRV_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    DRV_CUDA(cudaStreamDestroy((cudaStream_t)stream));
    return KMC_OK;
}

int kmc_drivers_launch(kmc_driver **drivers, int64_t n, int64_t steps, void *main_stream, void **worker_streams,
                       int64_t n_workers)
{
    if (!drivers || n < 0 || steps < 0 || !worker_streams || n_workers <= 0) return KMC_EINVAL;
    for (int64_t i = 0; i < n; ++i)
        if (!drivers[i] || !drivers[i]->exec) return KMC_ESTATE;
    for (int64_t i = 0; i < n; ++i) {
        const int rc = ensure_headroom(drivers[i], steps);
        if (rc) return rc;
    }
    // fork/join events, grown on demand and kept for the process
    static std::vector<cudaEvent_t> ev;
    while ((int64_t)ev.size() < n_workers + 1) {
        cudaEvent_t e;
        DRV_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ev.push_back(e);
    }
    cudaStream_t ms = (cudaStream_t)main_stream;
    DRV_CUDA(cudaEventRecord(ev[0], ms));
    const int64_t nw = n_workers < n ? n_workers : n;
    for (int64_t w = 0; w < nw; ++w)
        DRV_CUDA(cudaStreamWaitEvent((cudaStream_t)worker_streams[w], ev[0], 0));
    for (int64_t i = 0; i < n; ++i) {
        const int rc = drivers[i]->graph_pipelined
                           ? ensure_prepared(drivers[i], (cudaStream_t)worker_streams[i % nw])
                           : KMC_OK;
        if (rc) return rc;
    }
    for (int64_t k = 0; k < steps; ++k)
        for (int64_t i = 0; i < n; ++i)
            DRV_CUDA(cudaGraphLaunch(drivers[i]->exec, (cudaStream_t)worker_streams[i % nw]));
    if (steps > 0)
        for (int64_t i = 0; i < n; ++i) {
            const int rc = mark_enqueued(drivers[i], (cudaStream_t)worker_streams[i % nw]);
            if (rc) return rc;
        }
    for (int64_t w = 0; w < nw; ++w) {
        DRV_CUDA(cudaEventRecord(ev[w + 1], (cudaStream_t)worker_streams[w]));
        DRV_CUDA(cudaStreamWaitEvent(ms, ev[w + 1], 0));
    }
    return KMC_OK;
}

// ---------------------------------------------------------------------------
// Size buckets: one CUDA graph holding the captured steps of many systems (child
// graph nodes with no edges between them, so the systems' steps run concurrently
// as the device has room), launched once per round instead of once per system.
// The child graphs are copies: when a member captures its step again (a store
// growth, a new tuning), the bucket graph is rebuilt before its next launch.
// ---------------------------------------------------------------------------
struct kmc_bucket {
    std::vector<kmc_driver *> drv;
    std::vector<int64_t> versions;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {
int bucket_build(kmc_bucket *b)
{
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    DRV_CUDA(cudaGraphCreate(&b->graph, 0));
    b->versions.resize(b->drv.size());
    for (size_t i = 0; i < b->drv.size(); ++i) {
        cudaGraphNode_t node;
        DRV_CUDA(cudaGraphAddChildGraphNode(&node, b->graph, nullptr, 0, b->drv[i]->graph));
        b->versions[i] = b->drv[i]->graph_version;
    }
    DRV_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0));
    return KMC_OK;
}
} // namespace

int kmc_bucket_create(kmc_driver **drivers, int64_t n, kmc_bucket **out)
{
    if (!drivers || n <= 0 || !out) return KMC_EINVAL;
    *out = nullptr;
    for (int64_t i = 0; i < n; ++i)
        if (!drivers[i] || !drivers[i]->graph) return KMC_ESTATE;
    kmc_bucket *b = new (std::nothrow) kmc_bucket;
    if (!b) return KMC_ENOMEM;
    b->drv.assign(drivers, drivers + n);
    const int rc = bucket_build(b);
    if (rc) {
        kmc_bucket_free(b);
        return rc;
    }
    *out = b;
    return KMC_OK;
}

int kmc_bucket_launch(kmc_bucket *b, int64_t steps, void *stream)
{
    if (!b || steps < 0) return KMC_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    int rc;
    bool stale = false;
    for (size_t i = 0; i < b->drv.size(); ++i) {
        kmc_driver *d = b->drv[i];
        if ((rc = ensure_headroom(d, steps))) return rc;
        if (d->graph_pipelined && (rc = ensure_prepared(d, st))) return rc;
        stale = stale || d->graph_version != b->versions[i];
    }
    if (stale && (rc = bucket_build(b))) return rc;
    for (int64_t k = 0; k < steps; ++k) DRV_CUDA(cudaGraphLaunch(b->exec, st));
    if (steps > 0)
        for (kmc_driver *d : b->drv)
            if ((rc = mark_enqueued(d, st))) return rc;
    return KMC_OK;
}

int kmc_bucket_free(kmc_bucket *b)
{
    if (!b) return KMC_EINVAL;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    delete b;
    return KMC_OK;
}
