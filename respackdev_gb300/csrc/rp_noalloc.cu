// rp_noalloc.cu -- batched complex matrix inverse that allocates no device memory.
//
// Some callers of this library cannot allocate GPU memory themselves or let a
// library do it: a Fortran driver whose device arrays come from a framework
// that owns every byte of the GPU, or a host application that reserves the whole
// device for its own pool.  They hand over device buffers for the input and the
// output and need the inverse without a single cudaMalloc behind the call.  This
// file gives them the dielectric-matrix inversion (the Gauss-Jordan kernels of
// rp_epsinv_q) with its scratch -- pivot rows, pivot columns, pivot indices and
// an error word -- in one file-scope device array of fixed size.
//
// The scratch array exists once per GPU on which this file's device code is
// loaded, and it stays allocated until the process exits.  CUDA loads modules
// lazily by default, so the array is reserved at the first call on a device
// (unless CUDA_MODULE_LOADING=EAGER): a host that hands all device memory to
// its own pool should make that first call before it reserves the pool.
// Every call shares the array and it keeps the last call's contents: the
// error word is cleared at the start of each call, the other parts are fully
// rewritten before they are read.  Calls that overlap on the GPU (on
// different streams or threads) race on it and give wrong results.  The first
// call on a device looks up the array's device address with
// cudaGetSymbolAddress; make that first call before any stream capture.  Each
// call waits for its stream to finish the work before it returns.
#include <mutex>

#include "rp_dev.cuh"
#include "rp_host.h"

namespace {

using rp::cmul;
using rp::csub;

constexpr int kMaxRows = 1 << 17;   // n * nmat of one call
constexpr int kMaxMats = 1024;      // nmat of one call

struct NoAllocScratch {
  double2 prow[kMaxRows];   // pivot row of each matrix
  double2 fcol[kMaxRows];   // pivot column of each matrix
  double2 dinv[kMaxMats];   // reciprocal of each pivot
  int piv[kMaxRows];        // row exchanged with row k at step k
  int err;                  // 3: singular matrix
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// host copies of the array's device address, one per device
std::mutex g_mu;
NoAllocScratch *g_addr[64] = {nullptr};

NoAllocScratch *scratch_for(int dev) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (dev < 0 || dev >= 64) rp::fail(1, "device ordinal %d out of range", dev);
  if (!g_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) rp::fail(-1, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_addr[dev] = (NoAllocScratch *)p;
  }
  return g_addr[dev];
}

__device__ __forceinline__ double2 recip(double2 b) {
  if (fabs(b.x) >= fabs(b.y)) {
    double t = b.y / b.x, d = b.x + b.y * t;
    return make_double2(1.0 / d, -t / d);
  }
  double t = b.x / b.y, d = b.x * t + b.y;
  return make_double2(t / d, -1.0 / d);
}

// step k: pick the pivot of column k among rows k..n-1 (largest |re|+|im|, first
// on ties), exchange it with row k, copy the pivot row and column
__global__ void noalloc_select_swap(double2 *__restrict__ A, int n, int k, NoAllocScratch *s) {
  const int m = blockIdx.x;
  double2 *Am = A + (size_t)m * n * n;
  __shared__ double sv[256];
  __shared__ int si[256];
  double best = -1.0;
  int bi = k;
  for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
    const double2 v = Am[i + (size_t)n * k];
    const double a = fabs(v.x) + fabs(v.y);
    if (a > best) { best = a; bi = i; }
  }
  sv[threadIdx.x] = best;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int st = blockDim.x / 2; st; st >>= 1) {
    if (threadIdx.x < st) {
      const double ob = sv[threadIdx.x + st];
      const int oi = si[threadIdx.x + st];
      if (ob > sv[threadIdx.x] || (ob == sv[threadIdx.x] && oi < si[threadIdx.x])) {
        sv[threadIdx.x] = ob;
        si[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  const int p = (si[0] >= k && si[0] < n) ? si[0] : k;
  if (p != k)
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      const double2 t = Am[k + (size_t)n * j];
      Am[k + (size_t)n * j] = Am[p + (size_t)n * j];
      Am[p + (size_t)n * j] = t;
    }
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    s->prow[(size_t)m * n + j] = Am[k + (size_t)n * j];
    s->fcol[(size_t)m * n + j] = Am[j + (size_t)n * k];
  }
  if (threadIdx.x == 0) {
    s->piv[(size_t)m * n + k] = p;
    const double2 pk = Am[k + (size_t)n * k];
    if (!(sv[0] > 0.0)) atomicExch(&s->err, 3);
    s->dinv[m] = (pk.x == 0.0 && pk.y == 0.0) ? make_double2(0.0, 0.0) : recip(pk);
  }
}

__global__ void noalloc_update(double2 *__restrict__ A, int n, int k, const NoAllocScratch *__restrict__ s) {
  const int m = blockIdx.z;
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= n || j >= n) return;
  const double2 d = s->dinv[m];
  if (d.x == 0.0 && d.y == 0.0) return;
  double2 *a = A + (size_t)m * n * n + i + (size_t)n * j;
  const double2 pj = s->prow[(size_t)m * n + j];
  if (i == k) {
    *a = (j == k) ? d : cmul(pj, d);
  } else {
    const double2 f = cmul(s->fcol[(size_t)m * n + i], d);
    if (j == k) *a = make_double2(-f.x, -f.y);
    else *a = csub(*a, cmul(f, pj));
  }
}

// undo the row exchanges as column exchanges, last step first
__global__ void noalloc_colswap(double2 *__restrict__ A, int n, const NoAllocScratch *__restrict__ s) {
  const int m = blockIdx.x;
  double2 *Am = A + (size_t)m * n * n;
  for (int k = n - 1; k >= 0; k--) {
    const int p = s->piv[(size_t)m * n + k];
    if (p != k)
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double2 t = Am[i + (size_t)n * k];
        Am[i + (size_t)n * k] = Am[i + (size_t)n * p];
        Am[i + (size_t)n * p] = t;
      }
    __syncthreads();
  }
}

}  // namespace

extern "C" int rp_zinv_batched_noalloc(const double *a, double *ainv, int n, int nmat, void *stream) {
  try {
    if (!a || !ainv) rp::fail(1, "rp_zinv_batched_noalloc: null pointer");
    if (n < 1 || nmat < 1) rp::fail(1, "rp_zinv_batched_noalloc: n and nmat must be positive");
    if ((long)n * nmat > kMaxRows || nmat > kMaxMats)
      rp::fail(1, "rp_zinv_batched_noalloc: n*nmat = %ld exceeds the fixed scratch (n*nmat <= %d, nmat <= %d)",
               (long)n * nmat, kMaxRows, kMaxMats);
    if (((uintptr_t)a | (uintptr_t)ainv) & 15) rp::fail(1, "rp_zinv_batched_noalloc: buffers must be 16-byte aligned");
    {
      // the input and output must be the same buffer or not overlap at all
      const uintptr_t lo_a = (uintptr_t)a, lo_b = (uintptr_t)ainv;
      const uintptr_t len = (uintptr_t)sizeof(double2) * (uintptr_t)n * (uintptr_t)n * (uintptr_t)nmat;
      if (lo_a != lo_b && lo_a < lo_b + len && lo_b < lo_a + len)
        rp::fail(1, "rp_zinv_batched_noalloc: a and ainv overlap without being the same buffer");
    }
    int dev = 0;
    RP_CUDA(cudaGetDevice(&dev));
    NoAllocScratch *s = scratch_for(dev);
    cudaStream_t st = (cudaStream_t)stream;
    const size_t bytes = sizeof(double2) * (size_t)n * n * nmat;
    double2 *A = (double2 *)ainv;
    if (a != ainv) RP_CUDA(cudaMemcpyAsync(A, a, bytes, cudaMemcpyDeviceToDevice, st));
    RP_CUDA(cudaMemsetAsync(&s->err, 0, sizeof(int), st));
    dim3 ublk(32, 8), ugrid((n + 31) / 32, (n + 7) / 8, nmat);
    for (int k = 0; k < n; k++) {
      noalloc_select_swap<<<nmat, 256, 0, st>>>(A, n, k, s);
      noalloc_update<<<ugrid, ublk, 0, st>>>(A, n, k, s);
    }
    noalloc_colswap<<<nmat, 256, 0, st>>>(A, n, s);
    RP_CUDA(cudaGetLastError());
    int err = 0;
    RP_CUDA(cudaMemcpyAsync(&err, &s->err, sizeof(int), cudaMemcpyDeviceToHost, st));
    RP_CUDA(cudaStreamSynchronize(st));
    if (err) rp::fail(3, "rp_zinv_batched_noalloc: singular matrix");
    return 0;
  } catch (const rp::Error &e) {
    rp::set_global_error(e.msg);
    return e.code;
  }
}
