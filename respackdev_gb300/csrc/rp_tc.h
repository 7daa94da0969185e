// rp_tc.h -- tensor-core (tcgen05) chi0 contraction with split-precision operands.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace rp {

// Device scratch of the tensor-core contraction of one q point (or of one
// problem of a ragged batch): the prepared operands of the current pair batch
// and the float-pair Gram sums of every batch of the q.
struct TcWorkspace {
  void *planes = nullptr;
  size_t planes_bytes = 0;
  void *part = nullptr;
  size_t part_bytes = 0;
  int ng = 0, nen = 0, ndir = 1;
  int ksub = 16;            // K blocks per FP32 accumulation
  int split_req = 0;        // K splits requested (0 = the tuner's choice)
  int nsplit = 1;           // K splits of the Gram launches of this q
  int nslice = 1;           // float-pair sum slices allocated (>= nsplit)
  int tune_pending = 0;     // the first batch of this q times the launch-shape candidates
  int tune_split = 0, tune_pair = 0;  // ... over the K split, over single CTAs / CTA pairs
  int pair_req = 0;         // 0 the tuner's choice, 1 single CTAs, 2 CTA pairs (cta_group::2)
  int pair = 0;             // the Gram launches of this q run CTA pairs
  // the prepared pair batch (tc_prepare)
  const float *Yt = nullptr, *sB = nullptr, *sA = nullptr;
  const float2 *wt = nullptr;
  const unsigned char *Bp = nullptr;
  int Mp = 0, Kp = 0, precision = 0, ready = 0;
  double gram_seconds = 0;  // device time of the Gram kernel in the current q
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  size_t bytes() const { return planes_bytes + part_bytes; }
  void release();
};

// Allocates and zeroes the Gram sums of a q point.  split_req > 0 fixes the
// number of K splits and ws.pair_req != 0 the CTA shape; otherwise the tuner's
// cached choice for this shape or, for a shape it has not seen, the fastest
// candidate, timed on the first batch.
void tc_begin_q(TcWorkspace &ws, int ng, int nen, int ndir, int split_req, long k_estimate, int precision,
                cudaStream_t st);
// Transposes and splits one pair batch into the workspace's operands and, at
// Gamma, adds the batch to the G=0 rows/columns of directions 2 and 3
// (rowcol).  rho: FP32 pair densities [pair][k][g]; or rho64 (FP64, rounded to
// float here) when not null.  Runs the split tuner when it is pending.
int tc_prepare(TcWorkspace &ws, const float2 *rho, const double2 *rho64, const double2 *w, const double2 *head,
               int npair, int ntk, int ng, int nen, int g0, int precision, double2 *rowcol, int *err,
               cudaStream_t st);
// One launch of the Gram kernel over the prepared batches of n workspaces
// (a ragged group: each its own G sphere, K and frequencies; one precision).
// Adds into each workspace's sums; returns the kernel launches made.
int tc_gram_group(TcWorkspace *const *ws, int n, int *err, cudaStream_t st);
// tc_prepare + tc_gram_group of one workspace (the single-q path).
int tc_contract_batch(TcWorkspace &ws, const float2 *rho, const double2 *rho64, const double2 *w, const double2 *head,
                      int npair, int ntk, int ng, int nen, int g0, int precision, double2 *chi, double2 *rowcol,
                      int *err, cudaStream_t st);
// Adds the q's Gram sums to chi (FP64, [e][g + ng g']).
int tc_end_q(TcWorkspace &ws, double2 *chi, double2 *rowcol, cudaStream_t st);
// A ragged group end to end: one Gram launch over the prepared batches of n
// workspaces, then each workspace's sums into its chi (chis[i], which several
// workspaces may share).  With graph, the launch and the assemblies are
// captured into one CUDA graph and that graph is launched.  Waits for the
// result; returns the device seconds and adds the kernel launches to *launches.
double tc_group_run(TcWorkspace *const *ws, int n, double2 *const *chis, int *err, cudaStream_t st, bool graph,
                    long long *launches);

// The launch-shape tuner's cache: number of shapes decided, and a reset (tests).
int tc_tuned_shapes();
void tc_reset_tuner();

}  // namespace rp
