/*
 * kmc_gb300.h -- C ABI of the GB300 FMM-KMC energy-difference library
 * (libkmc_gb300.so).
 *
 * One handle = one KMC system (one cubic box of point charges) resident on
 * the current CUDA device.  All entry points return KMC_OK (0) or a negative
 * KMC_E* code; no C++ exception crosses this boundary.  A handle is bound to
 * one CUDA stream (kmc_set_stream) and is not thread safe.
 *
 * Each entry point names the reference (ppmd/coulomb_kmc) interface it
 * replaces; paths are relative to the coulomb_kmc project root.
 */
#ifndef KMC_GB300_H
#define KMC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* boundary conditions: coulomb_kmc/common.py:37-50 (BCType) */
#define KMC_BC_FREE_SPACE 0
#define KMC_BC_NEAREST27 1 /* '27': primary box plus its 26 nearest images */
#define KMC_BC_PBC 2

/* arithmetic of the propose path */
#define KMC_PREC_FP64 0  /* plain FP64 drop-in */
/* Mixed precision (propose_with_dats): near field, expansion evaluation, self
 * term and per-proposal lattice term in FP32 / double-FP32 over FP32 copies of
 * the FP64 state; FP64 for the lattice operator applied to the multipole, the
 * final old-minus-new difference and the total energy (the accepted move's
 * difference is recomputed in FP64).  pbc: l <= 20. */
#define KMC_PREC_MIXED 1             /* accept contributions in double-FP32, added to the FP64 master in FP64 */
#define KMC_PREC_MIXED_FP64_ACCEPT 2 /* accept contributions in FP64 */

#define KMC_OK 0
#define KMC_EINVAL -1     /* bad argument */
#define KMC_ECUDA -2      /* CUDA runtime error */
#define KMC_ESTATE -3     /* not initialised */
#define KMC_EBADMOVE -4   /* proposed move outside the box or beyond max_move */
#define KMC_EOVERFLOW -5  /* a cell store overflowed (device-selected accept) */
#define KMC_ENOMEM -6

typedef struct kmc_system kmc_system;

typedef struct kmc_params {
    int32_t boundary;     /* KMC_BC_* */
    int32_t r;            /* FMM levels; the finest level has 2^(r-1) cells per side (r >= 2) */
    int32_t l;            /* number of expansion terms, 2 <= l <= 32 */
    int32_t precision;    /* KMC_PREC_* */
    double extent;        /* cubic box edge; the box is [-extent/2, extent/2]^3 */
    double max_move;      /* maximum per-axis displacement of a proposed move */
    double energy_unit;   /* multiplies every energy */
    /* KMC_BC_PBC only: far-field lattice operator (host memory, copied by kmc_create).
       CSR over the l^2 x l^2 real operator acting on the real and imaginary blocks,
       and the dipole correction -- the interface of ppmd's LongRangeMTL
       (kmc_full_long_range.py:40, linop_data/linop_indptr/linop_indices, dipole_correction). */
    int64_t lr_nnz;
    const double *lr_data;
    const int64_t *lr_indptr;
    const int64_t *lr_indices;
    double lr_dipole[3];
    /* how kmc_initialise builds the finest-level local expansions (KMC_INIT_*):
       the reference runs ppmd's FMM (kmc_fmm.py:956-959); the exact particle-to-local
       sum is the same quantity without the FMM truncation error */
    int32_t initial_solve;
} kmc_params;

#define KMC_INIT_AUTO 0  /* exact up to 1e8 (cells x charges x images), FMM above */
#define KMC_INIT_EXACT 1 /* direct particle-to-local sum over all charges and images */
#define KMC_INIT_FMM 2   /* P2M, M2M, M2L, L2L over the octree (FP64) */

/* Create a system.  Replaces KMCFMM.__init__ (kmc_fmm.py:436-542) and the
 * component constructors it wires (FMMMPIDecomp, LocalParticleData,
 * LocalCellExpansions, FMMSelfInteraction, FullLongRangeEnergy). */
int kmc_create(const kmc_params *params, kmc_system **out);

/* Bind the handle to a CUDA stream (cudaStream_t passed as void*; NULL = legacy default). */
int kmc_set_stream(kmc_system *s, void *stream);

/* Initial solve: bins the charges, builds the cell store, the finest-level
 * local expansions, the level-0 multipole (pbc) and the total energy.
 * positions: host (n,3) f64, charges: host (n) f64.  energy_out: host, may be NULL.
 * Replaces KMCFMM.initialise (kmc_fmm.py:947-993), including the PyFMM solve. */
int kmc_initialise(kmc_system *s, int64_t n, const double *positions, const double *charges, double *energy_out);

/* Energy differences of masked proposals, all pointers device memory.
 * site_max_counts[n_site_types], current_sites[n], prop_positions[n][3*max_prop],
 * prop_masks[n][max_prop], prop_charges[n][max_prop] or NULL,
 * prop_energy_diffs[n][max_prop] (only active slots are written).
 * Move validation errors are counted on the device; read them with
 * kmc_get_error.  Replaces KMCFMM.propose_with_dats (kmc_fmm.py:665-762):
 * setup_move (kmc_mpi_decomp.py:501-616), direct_new/direct_old
 * (kmc_local.py:928-1031), indirect_interactions (kmc_octal.py:569-707),
 * self_interaction (kmc_fmm_self_interaction.py:190-267), long_range_energy
 * (kmc_full_long_range.py:710-858) and diff_lib (kmc_fmm.py:583-663). */
int kmc_propose_with_dats(kmc_system *s, int64_t n, int64_t max_prop, int64_t n_site_types,
                          const int64_t *site_max_counts, const int64_t *current_sites,
                          const double *prop_positions, const int64_t *prop_masks, const double *prop_charges,
                          double *prop_energy_diffs);

/* The same call with every array in host memory, as the reference's
 * propose_with_dats takes its dats: the arrays (prop_energy_diffs too, whose
 * inactive slots keep their values) go to device buffers the handle keeps, the
 * differences come back into prop_energy_diffs, and the call returns when they
 * are there.  errors_out[0] receives the number of invalid moves and errors_out[1]
 * the store overflows counted since the last read (both read and cleared, as
 * kmc_get_error does).  Page-locked host arrays make the copies asynchronous DMA.
 * One library call per propose, so a caller's language runtime takes no part in
 * the copies. */
int kmc_propose_with_dats_host(kmc_system *s, int64_t n, int64_t max_prop, int64_t n_site_types,
                               const int64_t *site_max_counts, const int64_t *current_sites,
                               const double *prop_positions, const int64_t *prop_masks, const double *prop_charges,
                               double *prop_energy_diffs, int64_t *errors_out);

/* Energy differences for explicit moves in CSR form (host memory):
 * particle ids pids[nump], exclusive_sum[nump+1], new_positions[total][3];
 * diffs_out[total] receives dE * energy_unit (host).  Synchronises.
 * Replaces the component calls of KMCFMM._propose (kmc_fmm.py:1001-1105)
 * after FMMMPIDecomp.setup_propose (kmc_mpi_decomp.py:238-310). */
int kmc_propose_moves(kmc_system *s, int64_t nump, const int64_t *pids, const int64_t *exclusive_sum,
                      const double *new_positions, double *diffs_out);

/* Accept one move given on the host (pid, new position): the energy is
 * advanced by that move's energy difference, the charge's position, cell and
 * store slot are updated, every cell's local expansion and (pbc) the level-0
 * multipole are updated.  Does not synchronise.
 * Replaces KMCFMM.accept/_accept (kmc_fmm.py:789-912): LocalParticleData.accept
 * (kmc_local.py:180-371), accept_local_exp (kmc_octal.py:961-1227),
 * FullLongRangeEnergy.accept (kmc_full_long_range.py:270-316). */
int kmc_accept(kmc_system *s, int64_t pid, const double new_position[3]);

/* As kmc_accept, with the move read from device memory written by a device
 * selection step: d_pid[1], d_new_position[3], d_energy_diff[1] (dE already
 * multiplied by energy_unit, as written by kmc_propose_with_dats).  No host
 * synchronisation; usable inside a captured CUDA graph. */
int kmc_accept_device(kmc_system *s, const int64_t *d_pid, const double *d_new_position,
                      const double *d_energy_diff);

/* Allocation-free variant of kmc_propose_moves.  It has no counterpart in the
 * reference.  It serves callers that cannot allocate device memory when they
 * need energy differences: an application whose own memory pool has already
 * claimed the device memory it may use (a cudaMalloc from this library would
 * fail or fragment that pool), or a loop that cannot afford the device
 * synchronisation a cudaFree implies.
 * All pointers are device memory: particle ids d_pids[nump],
 * d_exclusive_sum[nump+1] (proposal offsets), d_new_positions[total][3];
 * d_diffs[total] receives dE * energy_unit, in proposal order.  FP64.
 * Scratch is a fixed file-scope device array of about 41 KB that every device
 * which loads the library holds until exit, not the handle's buffers: limits
 * 4096 moving charges and 16384 proposals per call (larger calls return
 * KMC_EINVAL with a message).  Set-up: the first call on a device (and the
 * first after that device's context was replaced) looks up the array's device
 * address (cudaGetSymbolAddress) with that device current.  Every call on a
 * device shares the array and it
 * keeps the last call's contents, so calls that overlap on the GPU (different
 * streams or handles) race; serialise them.  Each call writes every element of
 * it that the call reads.  Inputs are checked on the device before use: ids
 * outside [0, N) or offsets that do not start at 0, decrease or end at another
 * total than `total` make every output NaN; a proposed position outside the box,
 * not finite or beyond max_move makes its output NaN; both are counted as bad
 * moves (kmc_get_error).  Does not synchronise. */
int kmc_propose_moves_noalloc(kmc_system *s, int64_t nump, int64_t total, const int64_t *d_pids,
                              const int64_t *d_exclusive_sum, const double *d_new_positions, double *d_diffs);

/* Current total energy (synchronises). */
int kmc_get_energy(kmc_system *s, double *energy_out);

/* Read and clear the device error counters (synchronises):
 * bad_moves = invalid proposals since the last call, overflow = store overflows. */
int kmc_get_error(kmc_system *s, int64_t *bad_moves, int64_t *overflow);

/* Cell store capacity.  The reference grows a cell's particle store when an
 * accepted move fills it (LocalParticleData, kmc_local.py:318-326, 558-580);
 * kmc_accept does the same on the host before it launches.  A device-selected
 * accept (kmc_accept_device, the device driver) cannot reallocate: when its new
 * cell is full it leaves the whole state untouched, counts an overflow
 * (kmc_get_error) and keeps the move; every later device-selected accept is
 * refused the same way until kmc_resolve_overflow grows the store and applies
 * the kept move (*applied_out = 1; 0 when nothing was kept).  kmc_accept returns
 * KMC_EOVERFLOW while a move is kept.  The device driver avoids the case: it
 * reads the occupancy before a cell could fill and grows the store first.
 * kmc_store_reserve sets the capacity (slots per cell, rounded up to a multiple
 * of 4) to at least `capacity` and at least the largest occupancy; it may also
 * shrink the store.  Synchronises; captured steps must be captured again after it.
 * kmc_max_occupancy: the largest cell occupancy and the capacity (synchronises). */
int kmc_store_reserve(kmc_system *s, int64_t capacity);
int kmc_max_occupancy(kmc_system *s, int64_t *max_out, int64_t *capacity_out);
int kmc_resolve_overflow(kmc_system *s, int64_t *applied_out);

/* Copy state to host for inspection (synchronises; any pointer may be NULL):
 * positions[n][3], cells[n] (linear finest-level cell, x fastest),
 * occupancy[ncell], local expansions in the reference layout [ncell][2 l^2],
 * multipole[2 l^2] (pbc; reference layout). */
int kmc_read_state(kmc_system *s, double *positions, int64_t *cells, int64_t *occupancy,
                   double *local_expansions, double *multipole);

/* Number of finest-level cells and the current store capacity per cell. */
int kmc_info(kmc_system *s, int64_t *ncell, int64_t *capacity, int64_t *n);

/* Per-kernel timing with CUDA events on the handle's stream (off by default).
 * kmc_profile_read synchronises, and returns for every kernel id
 * (0 <= id < KMC_NKERNELS, names from kmc_kernel_name) the accumulated
 * milliseconds and launch counts since the last reset, and the number of kernel
 * launches issued by this handle.  Counterpart of the reference's per-component
 * timers in the PROFILE dictionary (common.py:136-160, kmc_fmm.py:894-912). */
#define KMC_NKERNELS 19
int kmc_profile(kmc_system *s, int32_t enable);
int kmc_profile_read(kmc_system *s, int32_t reset, double *ms_out, int64_t *count_out, int64_t *launches_out);
/* Diagnostics, no reference counterpart: the launches bracketed since the last
 * read, in launch order, with start and end times (ms, CUDA events) relative to
 * the first one's start, so that concurrent streams show as overlaps.  Consumes
 * them like kmc_profile_read (their durations are added to its totals);
 * synchronises the device. */
int kmc_profile_timeline(kmc_system *s, int64_t max_entries, int32_t *ids_out, double *start_ms, double *end_ms,
                         int64_t *n_out);
const char *kmc_kernel_name(int32_t id);

/* Potential of all charges at n points (device arrays [n][3] and [n]), without
 * the energy unit: near field of the 27 neighbour cells, the cell's local
 * expansion and, for pbc, the far-lattice term.  Points must lie in the box.
 * Replaces KMCFMM.eval_field (kmc_fmm.py:544-567). */
int kmc_eval_field(kmc_system *s, int64_t n, const double *d_points, double *d_out);

/* ------------------------------------------------------------------------
 * Insertion and removal of charges (InjectorExtractor, kmc_inject_extract.py).
 * ------------------------------------------------------------------------ */
/* Energy of each listed charge in the system, q_i times its potential without
 * itself (near field, cell expansion, lattice term), times the energy unit.
 * Device arrays.  Replaces InjectorExtractor.get_energy (kmc_inject_extract.py:82-123). */
int kmc_get_energy_ids(kmc_system *s, int64_t n, const int64_t *d_ids, double *d_out);
/* Energy of n charges alone in the box under the system's boundary condition and
 * energy definition (pair terms over the 3x3x3 image block for '27'/pbc with the
 * self-image terms, and the lattice term for pbc), times the energy unit; device
 * arrays, result in d_out[0].  Replaces compute_energy (kmc_inject_extract.py:145-166,
 * ppmd FreeSpaceDirect / NearestDirect / PBCDirect). */
int kmc_group_energy(kmc_system *s, int64_t n, const double *d_positions, const double *d_charges, double *d_out);
/* Remove the listed charges (host ids): the energy changes by their set energy
 * minus their energies in the system; the expansions lose their contributions;
 * the remaining charges keep their order (higher ids shift down).  Synchronous.
 * Replaces InjectorExtractor.extract (kmc_inject_extract.py:240-301). */
int kmc_extract(kmc_system *s, int64_t n, const int64_t *ids, double *de_out);
/* Add n charges (host arrays), appended with ids N..N+n-1: the energy changes by
 * their set energy plus their charges times the field at their positions.
 * Synchronous.  Replaces InjectorExtractor.inject (kmc_inject_extract.py:304-424).
 * Both calls reallocate the system's charge arrays: a captured driver graph of the
 * system must be recreated afterwards. */
int kmc_inject(kmc_system *s, int64_t n, const double *positions, const double *charges, double *de_out);

/* Launch-shape tuning (no reference counterpart; the reference has fixed
 * OpenMP loops).  key: KMC_TUNE_*; value 0 restores the built-in choice. */
#define KMC_TUNE_P2L_GROUPS 0 /* source groups per block of the double-FP32 accept kernel (1..4) */
#define KMC_TUNE_LR_FUSED 1   /* mixed pbc lattice term: 0 per-charge and per-proposal kernels, 1 one fused kernel */
#define KMC_TUNE_LR_STAGE 2   /* fused lattice kernel: 0 folded form in shared memory (when it fits), 1 read-only cache */
#define KMC_TUNE_NEAR_SCALAR 3 /* mixed near field: 0 two neighbours per packed FP32 instruction, 1 one at a time */
#define KMC_TUNE_NEAR_CHUNK 4  /* mixed near field: neighbours staged per chunk, 0 128, 1 256, 2 64 */
#define KMC_TUNE_LR_NOCACHE 5  /* mixed pbc lattice term: 0 h = A b kept per charge between moves, 1 recomputed each propose */
#define KMC_TUNE_P2L_FP32_FROM 6 /* double-FP32 accept: orders l >= k in FP32 (0: k = 6; k >= l: none) */
#define KMC_TUNE_DRIVER_SERIAL 7 /* device driver: 0 next step's set-up beside a double-FP32 accept, plain order
                                    beside an FP64 one; 1 plain order; 2 set-up beside every accept */
#define KMC_TUNE_FSELF_GENERIC 8 /* mixed pbc lattice self term: 0 unrolled L = 12 cubic evaluator, 1 interpreter */
#define KMC_TUNE_P2L_PAIR 9 /* double-FP32 accept at L = 12, orders from 6 in FP32: 0 column-pair kernel, 1 per-column kernel */
#define KMC_TUNE_P2L64 10 /* FP64 accept at L = 8, 12, 16: 0 column-pair kernel, 1 per-column kernel */
#define KMC_TUNE_P2L64_CELLS 11 /* FP64 column-pair accept: cells per block, 2, 4 or 8 (0: 2) */
#define KMC_TUNE_LR_THREADS 12 /* mixed pbc per-proposal lattice kernels: threads per block, 64, 128 or 256 (0: 128) */
#define KMC_TUNE_NEAR_SPLIT 13 /* mixed near field: blocks per cell, 1, 2 or 4 (0: 1), the cell's item rounds spread over them */
#define KMC_TUNE_NEAR_OLD 14 /* old side of a propose: 0 each charge's near-field potential kept between moves (every
                                accept updates the charges around the moved one), 1 summed afresh on every propose */
#define KMC_TUNE_P2L64_PER_SM 15 /* FP64 column-pair accept: at most 1..4 blocks resident per SM (0: no limit), the rest of
                                    each SM left to other kernels; results unchanged */
#define KMC_TUNE_NEAR_PRIORITY 16 /* mixed near field: 0 default scheduling priority, 1 the device's highest (blocks
                                    dispatched before other kernels' waiting blocks); results unchanged */
#define KMC_NTUNE 17
int kmc_set_tuning(kmc_system *s, int32_t key, int32_t value);
int kmc_get_tuning(kmc_system *s, int32_t key, int32_t *value_out);
/* Autotuner (no reference counterpart; the reference's OpenMP loops and block-256
 * CUDA launches are fixed): times `reps` launches of each candidate of the keys
 * whose variants give bit-identical results and the same total work --
 * KMC_TUNE_LR_THREADS (after a proposal set-up, mixed pbc) and
 * KMC_TUNE_P2L64_CELLS (FP64 accept) -- on this handle and keeps the fastest.
 * KMC_TUNE_NEAR_SPLIT, also bit-identical, repeats each cell's set-up per block:
 * it is tuned on whole rounds of many systems (the Python server), where the
 * device is full, not on one handle alone.  The state is not changed: the lattice kernels
 * rerun the last set-up's proposals into proposal scratch, the accept kernel runs
 * on a copy of the expansions.  chosen_out (may be NULL) receives all KMC_NTUNE
 * values.  Synchronises; allocates scratch for the call. */
int kmc_autotune(kmc_system *s, int32_t reps, int32_t *chosen_out);

/* ------------------------------------------------------------------------
 * Device-side KMC driver: proposal generation, selection and lattice
 * occupancy on the GPU, so that a KMC step (generate, propose_with_dats,
 * select, accept) needs no host round trip and can be captured as one CUDA
 * graph.  Replaces the host bookkeeping of the reference's example driver
 * (examples/propose_with_dats_example.py:218-446: hop proposals, occupied-site
 * masks, rates exp(-beta dE / 2), cumulative-sum selection) and the Metropolis
 * loops of its tests (tests/host/test_free_space_1.py).  Random numbers:
 * Philox4x32-10 keyed by seed, counter (step, index, attempt, stream tag).
 * ------------------------------------------------------------------------ */
#define KMC_DRIVE_LATTICE 0    /* simple-cubic lattice hopping, rejection-free selection */
#define KMC_DRIVE_OFFLATTICE 1 /* one uniform displacement per charge, Metropolis on one random charge */

typedef struct kmc_driver kmc_driver;

typedef struct kmc_driver_params {
    int32_t kind;           /* KMC_DRIVE_* */
    int32_t lattice_side;   /* lattice: sites per side (spacing extent / side, site i at -E/2 + (i + 1/2) spacing) */
    double beta;            /* inverse temperature */
    double step;            /* off-lattice: displacement uniform in [-step, step]^3, re-drawn if it leaves the box */
    uint64_t seed;
    const int64_t *lattice_sites; /* lattice: host array, site index of every charge (x fastest) */
    int64_t log_capacity;   /* steps kept in the selection log (0: none) */
} kmc_driver_params;

int kmc_driver_create(kmc_system *s, const kmc_driver_params *p, kmc_driver **out);
/* enqueue nsteps full KMC steps on the system's stream (no host synchronisation) */
int kmc_driver_step(kmc_driver *d, int64_t nsteps);
/* capture one step as a CUDA graph on the system's stream; kmc_driver_launch replays it */
int kmc_driver_capture(kmc_driver *d);
int kmc_driver_launch(kmc_driver *d, int64_t nsteps, void *stream);
/* steps done, moves accepted, proposals evaluated (synchronises the system's stream; after
   kmc_driver_launch on another stream the caller synchronises that stream first; any pointer may be NULL) */
int kmc_driver_counters(kmc_driver *d, int64_t *steps_out, int64_t *accepted_out, int64_t *proposals_out);
/* selection log, oldest first: particle id (-1 = rejected), target site (lattice) or -1,
   energy difference of the selected proposal; n_out = entries written */
int kmc_driver_log(kmc_driver *d, int64_t max_entries, int64_t *pid_out, int64_t *target_out, double *de_out,
                   int64_t *n_out);
/* lattice: site of every charge (host array of n) */
int kmc_driver_sites(kmc_driver *d, int64_t *sites_out);
int kmc_driver_free(kmc_driver *d);

/* One round over many systems (serving / batched replicas): replay each
 * driver's captured step `steps` times, the drivers spread round-robin over
 * the worker streams, ordered after the work queued on main_stream; main_stream
 * waits for all of them.  No host synchronisation.  Call from one host thread. */
int kmc_drivers_launch(kmc_driver **drivers, int64_t n, int64_t steps, void *main_stream, void **worker_streams,
                       int64_t n_workers);

/* Size buckets (no reference counterpart): one CUDA graph holding the captured
 * steps of n drivers (typically systems of one size class: the same depth, order
 * and boundary condition) as independent child graphs, so that one launch runs a
 * round of all of them and the device overlaps their kernels as it has room.
 * kmc_bucket_launch replays it `steps` times on `stream` after each member's
 * store headroom check (a member that grows its store and captures its step again
 * makes the bucket rebuild its graph first).  Results are those of the members'
 * own launches.  The drivers must outlive the bucket. */
typedef struct kmc_bucket kmc_bucket;
int kmc_bucket_create(kmc_driver **drivers, int64_t n, kmc_bucket **out);
int kmc_bucket_launch(kmc_bucket *b, int64_t steps, void *stream);
int kmc_bucket_free(kmc_bucket *b);

/* A dedicated non-blocking CUDA stream, not taken from any library's stream pool
 * (pooled streams are handed out round-robin and can alias, which breaks stream
 * capture on one of them while another thread launches on its alias); destroy
 * waits for the stream's work.  No reference counterpart. */
int kmc_stream_create(void **stream_out);
int kmc_stream_destroy(void *stream);

/* Host-side proposal generation for the host path (no reference counterpart; the
 * reference's example driver draws these in numpy): out[i] = pos[i] + a uniform
 * displacement in [-step, step]^3, drawn again (up to 32 times, then the old
 * position) while it leaves the box [-extent/2, extent/2]^3 -- the device driver's
 * off-lattice draws (Philox4x32-10 keyed by `seed`, counter (round, index,
 * attempt)), computed on the host with the host's rounding.  n charges, positions
 * [n][3] in and out (host memory, out may not alias pos), `nthreads` host threads
 * (<= 0: one).  A pure function of (seed, round, index): the thread count changes
 * nothing.  Does not touch the GPU. */
int kmc_host_displacements(int64_t n, const double *pos, double extent, double step, uint64_t seed, int64_t round,
                           double *out, int32_t nthreads);

/* Diagnostic (no reference counterpart): measured FMA throughput of the
 * current device's FP64 (fp64 != 0) or FP32 pipe in TFLOP/s (FMA = 2 flops),
 * the denominator of the roofline fraction of the FMA-bound kernels. */
int kmc_diag_fma_rate(int32_t fp64, int32_t iters, double *tflops_out);

/* Release all device memory of the handle.  Replaces KMCFMM.free (kmc_fmm.py:569-577). */
int kmc_free(kmc_system *s);

/* Last CUDA error string of this thread's last failing call (static storage). */
const char *kmc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* KMC_GB300_H */
