// core_svd.h - SVD and truncation of the 2r x 2r core of the large engines'
// rank-adaptive step on one thread-block cluster (FP32 panels; the SVD runs
// in FP32 sweeps, then double-float).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace lri {

struct CoreSvdArgs {
  int R;              // r_max: panels of 2R columns, core R x R
  const double* F;    // wa x wa core S~ (ld wa), wa = 2 min(R, *rank)
  float* S0;          // out: R x R, diag(sigma_1..sigma_r1), zero elsewhere
  int32_t* rank;      // in: r; out: r1
  double tol;         // truncation: smallest r1 with sum_{j > r1} sigma_j^2 < tol^2
  int rmin;           // then clamped to [rmin, R]
  // scratch: five (2R)^2 blocks of 8-byte values (double-float matrices)
  double* scr[5];
  double* P1;         // out: 2R x R (ld 2R), kept left vectors in the rows of the active columns
  double* Q1;         // out: 2R x R, kept right vectors
  uint32_t* status;   // bits: no convergence, non-finite core
  uint32_t st_noconv, st_nonfinite;
};

// The largest 2r the cluster form takes (r <= 96).
constexpr int CORE_SVD_MAX_WA = 192;

// Launches the cluster SVD on `st`.  Returns the launch error; a device that
// cannot co-schedule the cluster reports cudaErrorClusterOutOfResources or
// similar at launch, never a wrong result.
cudaError_t core_svd_cluster(const CoreSvdArgs& a, cudaStream_t st);

}  // namespace lri
