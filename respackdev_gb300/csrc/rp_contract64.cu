// rp_contract64.cu -- plain FP64 chi0 contraction (the reference kernel of the
// precision study) and the Gamma head rows/columns.
//
// chiqw.F:1397-1410 (q != 0) and :1862-1875 (Gamma) accumulate
//     chi(G,G',w) += xow(k,w) conj(rho_k(G)) rho_k(G') / NTK (1 - P_occ P_vir)
// over band pairs and k.  Here K = (pair, k) is one long reduction axis and
// w(K, w) already carries the occupation factor and 1/NTK, so per frequency
// this is chi = rho^H diag(w) rho.  Each CTA owns a 32x32 tile of one
// frequency for the whole K range (fixed summation order, no atomics).
#include "rp_dev.cuh"
#include "rp_host.h"

namespace rp {

__global__ void __launch_bounds__(256) contract_fp64_kernel(const double2 *__restrict__ rho,
                                                            const double2 *__restrict__ w, int npair, int ntk,
                                                            int ng, int nen, double2 *__restrict__ chi) {
  __shared__ double2 As[16][33], Bs[16][33];
  const int g0 = blockIdx.x * 32, h0 = blockIdx.y * 32, e = blockIdx.z;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 16 + tx;
  double2 acc[2][2];
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) acc[i][j] = make_double2(0, 0);
  const long K = (long)npair * ntk;
  for (long kb = 0; kb < K; kb += 16) {
    for (int i = tid; i < 512; i += 256) {
      const int kk = i >> 5, c = i & 31;
      const long Kx = kb + kk;
      double2 a = make_double2(0, 0), b = make_double2(0, 0);
      if (Kx < K) {
        const int p = (int)(Kx / ntk), k = (int)(Kx % ntk);
        const double2 ww = w[((size_t)p * nen + e) * ntk + k];
        if (g0 + c < ng) a = cmul(ww, cconj(rho[(size_t)Kx * ng + g0 + c]));
        if (h0 + c < ng) b = rho[(size_t)Kx * ng + h0 + c];
      }
      As[kk][c] = a;
      Bs[kk][c] = b;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < 16; kk++) {
      const double2 a0 = As[kk][2 * tx], a1 = As[kk][2 * tx + 1];
      const double2 b0 = Bs[kk][2 * ty], b1 = Bs[kk][2 * ty + 1];
      cfma(acc[0][0], a0, b0);
      cfma(acc[0][1], a0, b1);
      cfma(acc[1][0], a1, b0);
      cfma(acc[1][1], a1, b1);
    }
    __syncthreads();
  }
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++) {
      const int g = g0 + 2 * tx + i, h = h0 + 2 * ty + j;
      if (g < ng && h < ng) {
        double2 *d = chi + (size_t)e * ng * ng + g + (size_t)ng * h;
        *d = cadd(*d, acc[i][j]);
      }
    }
}

int launch_contract_fp64(const double2 *rho, const double2 *w, int npair, int ntk, int ng, int nen, double2 *chi,
                         cudaStream_t st) {
  if (npair == 0) return 0;
  dim3 grid((ng + 31) / 32, (ng + 31) / 32, nen), block(16, 16);
  contract_fp64_kernel<<<grid, block, 0, st>>>(rho, w, npair, ntk, ng, nen, chi);
  RP_CUDA(cudaGetLastError());
  return 1;
}

// Gamma: the three head directions differ only in the G=0 entry of rho
// (chiqw.F:1800-1806), so directions 2 and 3 need only the G=0 row and column.
__global__ void __launch_bounds__(256) gamma_rowcol_kernel(const double2 *__restrict__ rho,
                                                           const double2 *__restrict__ w,
                                                           const double2 *__restrict__ head, int npair, int ntk,
                                                           int ng, int nen, int g0, double2 *__restrict__ rowcol) {
  const int g = blockIdx.x, e = blockIdx.y, ix = blockIdx.z + 1;
  const long K = (long)npair * ntk;
  double2 r = make_double2(0, 0), c = make_double2(0, 0);
  for (long Kx = threadIdx.x; Kx < K; Kx += blockDim.x) {
    const int p = (int)(Kx / ntk), k = (int)(Kx % ntk);
    const double2 ww = w[((size_t)p * nen + e) * ntk + k];
    const double2 h = head[(size_t)Kx * 3 + ix];
    const double2 v = g == g0 ? h : rho[(size_t)Kx * ng + g];
    cfma(r, cmul(ww, cconj(h)), v);   // row G0:  w conj(h) rho(g)
    cfma(c, cmul(ww, cconj(v)), h);   // column:  w conj(rho(g)) h
  }
  __shared__ double2 sr[256], sc[256];
  sr[threadIdx.x] = r;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int s = 128; s; s >>= 1) {
    if (threadIdx.x < s) {
      sr[threadIdx.x] = cadd(sr[threadIdx.x], sr[threadIdx.x + s]);
      sc[threadIdx.x] = cadd(sc[threadIdx.x], sc[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double2 *o = rowcol + ((size_t)(ix - 1) * nen + e) * 2 * ng;
    o[g] = cadd(o[g], sr[0]);
    o[ng + g] = cadd(o[ng + g], sc[0]);
  }
}

int launch_gamma_rowcol(const double2 *rho, const double2 *w, const double2 *head, int npair, int ntk, int ng,
                        int nen, int g0, double2 *rowcol, cudaStream_t st) {
  if (npair == 0) return 0;
  dim3 grid(ng, nen, 2);
  gamma_rowcol_kernel<<<grid, 256, 0, st>>>(rho, w, head, npair, ntk, ng, nen, g0, rowcol);
  RP_CUDA(cudaGetLastError());
  return 1;
}

// x /= s (chiqw.F:1476 divides by VOLUME)
__global__ void scale_kernel(double2 *x, size_t n, double s) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { x[i].x /= s; x[i].y /= s; }
}
int launch_scale(double2 *x, size_t n, double s, cudaStream_t st) {
  if (!n) return 0;
  scale_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, n, s);
  RP_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace rp
