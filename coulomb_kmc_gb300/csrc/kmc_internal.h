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

} // extern "C"
