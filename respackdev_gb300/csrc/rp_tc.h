// rp_tc.h -- tensor-core (tcgen05) chi0 contraction with split-precision operands.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace rp {

// Device scratch of the tensor-core contraction (operand planes, FP32 partials).
struct TcWorkspace {
  void *planes = nullptr;
  size_t planes_bytes = 0;
  void *part = nullptr;
  size_t part_bytes = 0;
  int ng = 0, nen = 0, ndir = 1;
  int ksub = 16;          // K blocks per FP32 accumulation
  double gram_seconds = 0;  // device time of the Gram kernel in the current q
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  size_t bytes() const { return planes_bytes + part_bytes; }
  void release();
};

void tc_begin_q(TcWorkspace &ws, int ng, int nen, int ndir, cudaStream_t st);
// Adds the batch's contribution to chi (FP64, [dir][e][g + ng g']) and, at
// Gamma, to the G=0 rows/columns of directions 2 and 3 (rowcol).
// rho: FP32 pair densities [pair][k][g]; or rho64 (FP64, rounded to float here) when not null.
int tc_contract_batch(TcWorkspace &ws, const float2 *rho, const double2 *rho64, const double2 *w, const double2 *head,
                      int npair, int ntk, int ng, int nen, int g0, int precision, double2 *chi, double2 *rowcol,
                      int *err, cudaStream_t st);
int tc_end_q(TcWorkspace &ws, double2 *chi, double2 *rowcol, cudaStream_t st);

}  // namespace rp
