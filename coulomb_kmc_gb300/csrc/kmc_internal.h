// Internal interface between the core library (kmc_gb300.cu) and the
// device-side KMC driver (kmc_driver.cu).  Not part of the C ABI.
#pragma once

#include "kmc_gb300.h"

#include <cuda_runtime.h>

extern "C" {

cudaStream_t kmc_int_stream(const kmc_system *s);
int kmc_int_n(const kmc_system *s);
double kmc_int_extent(const kmc_system *s);
int kmc_int_boundary(const kmc_system *s);
double kmc_int_max_move(const kmc_system *s);
const double *kmc_int_positions(const kmc_system *s);  // device [N][3], updated by every accept
// allocate the propose buffers for n movers and nm proposals now, so that a
// later stream capture of propose + accept needs no allocation
int kmc_int_reserve(kmc_system *s, int64_t n, int64_t nm);
bool kmc_int_initialised(const kmc_system *s);
// kmc_propose_with_dats in two parts: the proposal set-up (compaction, cell
// sort) on a given stream, and the evaluation on the system's stream.  The
// set-up skips the per-move checks: it serves the device driver, whose moves are
// valid by construction (spacing / step <= max_move checked at creation,
// positions inside the box); prop_cells (optional, [n * max_prop]) gives each
// proposal's cell as kmc_int_bin_cells computes it
int kmc_int_propose_prepare(kmc_system *s, void *stream, int64_t n, int64_t max_prop, const int64_t *site_max_counts,
                            const int64_t *current_sites, const double *prop_positions, const int64_t *prop_masks,
                            const int *prop_cells);
// records a failed CUDA call for kmc_last_error (the calling thread's message)
void kmc_int_set_error(const char *what, int cuda_error);
// the system's cell of each of n positions (the binning propose applies), on stream
int kmc_int_bin_cells(kmc_system *s, void *stream, int64_t n, const double *d_pos, int *d_cells);
int kmc_int_propose_evaluate(kmc_system *s, int64_t n, int64_t max_prop, double *prop_energy_diffs);
// kmc_accept_device with the caller's work (branch) enqueued on a stream that joins
// with the accept's end and forks after the store / position update, or (early)
// where the accept is enqueued, for a branch that reads nothing the accept writes
// (positions, store, expansions, energy)
int kmc_int_accept_device_branch(kmc_system *s, const int64_t *d_pid, const double *d_new_position,
                                 const double *d_energy_diff, int (*branch)(void *ctx, void *stream), void *ctx,
                                 int early);
// launches made on the system so far (host count; graph replays add none)
int64_t kmc_int_launches(const kmc_system *s);
int kmc_int_tuning(const kmc_system *s, int key);
// advances whenever the system's device buffers that a captured step reads are
// reallocated (store growth): a captured step of an older layout must be captured again
int64_t kmc_int_layout_gen(const kmc_system *s);
int kmc_int_ncell(const kmc_system *s);
bool kmc_int_accept_df32(const kmc_system *s);  // accept contributions in double-FP32 (precision mixed)

} // extern "C"
