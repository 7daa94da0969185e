// rp_wfn.cu -- full-k coefficients and real-space periodic parts (once per context).
//
// For every full-mesh k and band b this kernel
//   1. rotates the irreducible coefficients to k (make_C0, chiqw_sub.F:264-322:
//      gather through the packing table, phase e^{-2 pi i G.pg/nnp}, conjugation
//      for time-reversed k), keeping the result in `cfull` (used by the Gamma
//      head, calc_VMab), and
//   2. evaluates u_{b,k}(r) = sum_G c(G) e^{+2 pi i G.r/N} on the FFT box
//      (fft3_bw, m_fft3d_20150826.f90:1662-1720: e^{+i}, unscaled) and rounds
//      it to single precision, as the reference's kindless CMPLX() does
//      (chiqw_sub.F:143,162).
// The reference repeats this for every band pair and k; here it runs once and
// the result stays resident in HBM (float2, x fastest, per (k, b) one box).
//
// The transform is three separable DFT passes over one output z-slab at a
// time, staged in shared memory: the plane-wave sphere sits in a compact
// (2R+1)^3 cube, so the z pass touches only the sphere's bounding box.
//
// The split precisions run the three passes in FP32 (WfnSlots::fp32): the
// result is rounded to single either way, and a pass of at most n terms in
// FP32 moves it by about a unit of that rounding, while GB300 runs FP32 at
// many times its FP64 rate (the transform of every virtual band per pair batch
// dominated the large workload's pair stage in FP64).  The FP64 precision and
// pair_fp64 keep the FP64 passes.
//
// When the real-space functions of every band do not fit in HBM (1000 k x
// 1000 bands on a 48^3 box would take 885 GB), the context keeps the occupied
// bands resident and transforms each pair batch's virtual bands into a window
// of slots when the batch starts (WfnSlots: a band list, their slots, and
// rotate = false to start from the rotated coefficients kept in cfull).
#include "rp_dev.cuh"
#include "rp_host.h"

namespace rp {

__device__ __forceinline__ int modp(int a, int n) { int m = a % n; return m < 0 ? m + n : m; }

template <typename T>
__global__ void __launch_bounds__(256) wfn_realspace_kernel(
    const double2 *__restrict__ coef_irr, const int *__restrict__ numirr, const int *__restrict__ trs,
    const int *__restrict__ src, const double2 *__restrict__ phase, const int *__restrict__ ng0,
    const int *__restrict__ kg0, int ncb, int ntg, int n1, int n2, int n3, int R1, int R2, int R3,
    double2 *__restrict__ cfull, float2 *__restrict__ ur, int k_begin, WfnSlots sl) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int b = sl.bands ? sl.bands[blockIdx.x] : blockIdx.x;
  const int k = k_begin + blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
  // the slot of (k, b) in ur; a band without a slot only gets its coefficients
  const int slot = sl.slot_of ? sl.slot_of[b] : b;
  const size_t ur_at = (size_t)k * (sl.slot_of ? sl.nslot : ncb) + slot;
  const bool c1 = 2 * R1 + 1 <= n1, c2 = 2 * R2 + 1 <= n2, c3 = 2 * R3 + 1 <= n3;
  const int D1 = c1 ? 2 * R1 + 1 : n1, D2 = c2 ? 2 * R2 + 1 : n2, D3 = c3 ? 2 * R3 + 1 : n3;
  using T2 = typename C2<T>::t;
  T2 *cube = (T2 *)smem;                           // D1*D2*D3, index c1 + D1*(c2 + D2*c3)
  T2 *A = cube + D1 * D2 * D3;                     // D1*D2
  T2 *B = A + D1 * D2;                             // D1*n2
  T2 *tw1 = B + D1 * n2, *tw2 = tw1 + n1, *tw3 = tw2 + n2;
  int *f1 = (int *)(tw3 + n3), *f2 = f1 + D1, *f3 = f2 + D2;
  const T2 zero = mk<T>(0, 0);
  for (int i = tid; i < D1 * D2 * D3; i += nt) cube[i] = zero;
  // twiddles from FP64 sincospi, rounded once to T
  for (int j = tid; j < n1; j += nt) { double s, c; sincospi(2.0 * j / n1, &s, &c); tw1[j] = mk<T>((T)c, (T)s); }
  for (int j = tid; j < n2; j += nt) { double s, c; sincospi(2.0 * j / n2, &s, &c); tw2[j] = mk<T>((T)c, (T)s); }
  for (int j = tid; j < n3; j += nt) { double s, c; sincospi(2.0 * j / n3, &s, &c); tw3[j] = mk<T>((T)c, (T)s); }
  for (int j = tid; j < D1; j += nt) f1[j] = c1 ? modp(j - R1, n1) : j;
  for (int j = tid; j < D2; j += nt) f2[j] = c2 ? modp(j - R2, n2) : j;
  for (int j = tid; j < D3; j += nt) f3[j] = c3 ? modp(j - R3, n3) : j;
  __syncthreads();
  // 1. rotate (or take the rotated coefficients) + scatter into the cube
  const int ikir = numirr[k], t = trs[k], ng = ng0[k];
  const double2 *cirr = coef_irr + ((size_t)ikir * ncb + b) * ntg;
  double2 *cf = cfull + ((size_t)k * ncb + b) * ntg;
  for (int ig = tid; ig < ntg; ig += nt) {
    double2 v = make_double2(0, 0);
    if (ig < ng) {
      if (sl.rotate) {
        int s = src[(size_t)k * ntg + ig];
        v = cmul(cirr[s], phase[(size_t)k * ntg + ig]);
        if (t == -1) v.y = -v.y;
      } else {
        v = cf[ig];
      }
      const int *g = kg0 + ((size_t)k * ntg + ig) * 3;
      int i1 = c1 ? g[0] + R1 : modp(g[0], n1);
      int i2 = c2 ? g[1] + R2 : modp(g[1], n2);
      int i3 = c3 ? g[2] + R3 : modp(g[2], n3);
      cube[i1 + D1 * (i2 + D2 * i3)] = mk<T>((T)v.x, (T)v.y);
    }
    if (sl.rotate) cf[ig] = v;
  }
  if (slot < 0) return;  // uniform over the block: no barrier is skipped by part of it
  __syncthreads();
  float2 *out = ur + ur_at * (size_t)n1 * n2 * n3;
  for (int z = 0; z < n3; z++) {
    // pass z: A[c1,c2] = sum_c3 cube e^{+2 pi i f3 z / n3}.  The frequencies f
    // of consecutive c are consecutive mod n, so the twiddle index f z mod n
    // steps by z: one modulo per sum instead of one per term (all passes).
    const int z0 = (f3[0] * z) % n3;
    for (int o = tid; o < D1 * D2; o += nt) {
      T2 acc = zero;
      int ix = z0;
      for (int cc = 0; cc < D3; cc++) {
        const T2 v = cube[o + D1 * D2 * cc];
        cfma(acc, v, tw3[ix]);
        ix += z;
        if (ix >= n3) ix -= n3;
      }
      A[o] = acc;
    }
    __syncthreads();
    // pass y: B[c1,y] = sum_c2 A e^{+2 pi i f2 y / n2}
    for (int o = tid; o < D1 * n2; o += nt) {
      int cc1 = o % D1, y = o / D1;
      T2 acc = zero;
      int ix = (f2[0] * y) % n2;
      for (int cc = 0; cc < D2; cc++) {
        cfma(acc, A[cc1 + D1 * cc], tw2[ix]);
        ix += y;
        if (ix >= n2) ix -= n2;
      }
      B[o] = acc;
    }
    __syncthreads();
    // pass x: u[x,y] = sum_c1 B e^{+2 pi i f1 x / n1}
    for (int o = tid; o < n1 * n2; o += nt) {
      int x = o % n1, y = o / n1;
      T2 acc = zero;
      int ix = (f1[0] * x) % n1;
      for (int cc = 0; cc < D1; cc++) {
        cfma(acc, B[cc + D1 * y], tw1[ix]);
        ix += x;
        if (ix >= n1) ix -= n1;
      }
      out[(size_t)z * n1 * n2 + o] = make_float2((float)acc.x, (float)acc.y);
    }
    __syncthreads();
  }
}

int launch_wfn_realspace(const double2 *coef_irr, const int *numirr, const int *trs, const int *src,
                         const double2 *phase, const int *ng0, const int *kg0, int ntk, int ncb, int ntg,
                         int n1, int n2, int n3, int R1, int R2, int R3, double2 *cfull, float2 *ur,
                         int k_begin, int k_end, cudaStream_t st, const WfnSlots &sl) {
  (void)ntk;
  const int nb = sl.bands ? sl.nbands : ncb;
  if (nb == 0 || k_end <= k_begin) return 0;
  const int D1 = 2 * R1 + 1 <= n1 ? 2 * R1 + 1 : n1, D2 = 2 * R2 + 1 <= n2 ? 2 * R2 + 1 : n2,
            D3 = 2 * R3 + 1 <= n3 ? 2 * R3 + 1 : n3;
  auto run = [&](auto kern, size_t cplx) {
    const size_t smem = cplx * ((size_t)D1 * D2 * D3 + D1 * D2 + D1 * n2 + n1 + n2 + n3) + sizeof(int) * (D1 + D2 + D3);
    const int cap = smem_cap(kern);
    if (smem > (size_t)cap) fail(1, "plane-wave sphere too large for the shared-memory cube (%zu bytes)", smem);
    RP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, cap));
    dim3 grid(nb, k_end - k_begin);
    kern<<<grid, 256, smem, st>>>(coef_irr, numirr, trs, src, phase, ng0, kg0, ncb, ntg, n1, n2, n3, R1, R2, R3, cfull,
                                  ur, k_begin, sl);
  };
  if (sl.fp32) run(wfn_realspace_kernel<float>, sizeof(float2));
  else run(wfn_realspace_kernel<double>, sizeof(double2));
  RP_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace rp
