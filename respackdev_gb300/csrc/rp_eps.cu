// rp_eps.cu -- dielectric matrix and its inverse in FP64 (K6).
//
// calc_eps_rpa (src/chiqw/chiqw_sub.F:386-457): chi0 *= 2 (spin), then
//     eps(G,G') = delta - chi0 2 tpi / (|q+G| |q+G'|)
// and calc_eps_rpa_q_0 (:459-568) at Gamma: head 1 - chi0 2 tpi plus the Drude
// term cmplx(-wd^2/(w^2+delt^2), delt wd^2/(w^3+w delt^2)) (single precision,
// w = Re(em), 1e-5 when zero), wings divided by one |q+G| only.
// invZGE (invZGE.F90:1-22) inverts with LAPACK zgetrf + zgetri; here every
// (frequency, direction) matrix is inverted by Gauss-Jordan elimination with
// partial pivoting on |re|+|im| (izamax's norm), one kernel pair per pivot
// column over all matrices at once, and the row/column permutation undone at
// the end.  The select kernel scales the pivot column by the pivot's
// reciprocal once, so the update is four FP64 FMAs per element.
#include "rp_dev.cuh"
#include "rp_host.h"

namespace rp {

__global__ void eps_build_kernel(const double2 *__restrict__ chi, EpsArgs a, double2 *__restrict__ A) {
  const int mat = blockIdx.y;              // d*nen + e
  const int d = mat / a.nen, e = mat % a.nen;
  const int n = a.ng;
  const size_t nn = (size_t)n * n;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nn; idx += (size_t)gridDim.x * blockDim.x) {
    const int ig = (int)(idx % n), jg = (int)(idx / n);
    double2 c = chi[(size_t)mat * nn + idx];
    c.x = 2.0 * c.x; c.y = 2.0 * c.y;
    const double qi = a.qglen[ig], qj = a.qglen[jg];
    const double tpi = 2.0 * 3.14159265358979323846;
    double2 r;
    // e = -c*2*tpi/qi/qj  (left to right as the reference)
    auto mul = [](double2 v, double s) { return make_double2(v.x * s, v.y * s); };
    auto dv = [](double2 v, double s) { return make_double2(v.x / s, v.y / s); };
    if (!a.gamma) {
      double2 t = dv(dv(mul(mul(c, 2.0), tpi), qi), qj);
      r = ig == jg ? make_double2(1.0 - t.x, -t.y) : make_double2(-t.x, -t.y);
    } else {
      if (ig == jg && ig == a.g0) {
        double w = a.em[e].x;
        if (w == 0.0) w = 1.0e-5;
        const double wd = a.wd[d], dl = a.delt;
        double dr = (double)(float)(-wd * wd / (w * w + dl * dl));
        double di = (double)(float)(dl * wd * wd / (w * w * w + w * dl * dl));
        double2 t = mul(mul(c, 2.0), tpi);
        r = make_double2((1.0 - t.x) + dr, (0.0 - t.y) + di);
      } else if (ig == jg) {
        double2 t = dv(dv(mul(mul(c, 2.0), tpi), qi), qj);
        r = make_double2(1.0 - t.x, -t.y);
      } else if (ig == a.g0) {
        double2 t = dv(mul(mul(c, 2.0), tpi), qj);
        r = make_double2(-t.x, -t.y);
      } else if (jg == a.g0) {
        double2 t = dv(mul(mul(c, 2.0), tpi), qi);
        r = make_double2(-t.x, -t.y);
      } else {
        double2 t = dv(dv(mul(mul(c, 2.0), tpi), qi), qj);
        r = make_double2(-t.x, -t.y);
      }
    }
    A[(size_t)mat * nn + idx] = r;
  }
}

template <typename T>
__device__ __forceinline__ typename C2<T>::t crecip(typename C2<T>::t b) {
  // 1/b by Smith's algorithm
  if (fabs(b.x) >= fabs(b.y)) {
    const T t = b.y / b.x, d = b.x + b.y * t;
    return mk<T>((T)1 / d, -t / d);
  }
  const T t = b.x / b.y, d = b.x * t + b.y;
  return mk<T>(t / d, (T)-1 / d);
}

// T = double: the inverse itself; T = float: the first approximation of the
// mixed-precision inverse below
template <typename T>
__global__ void gj_select_kernel(typename C2<T>::t *__restrict__ A, int n, int k, typename C2<T>::t *__restrict__ prow,
                                 typename C2<T>::t *__restrict__ fcol, int *__restrict__ piv, int *__restrict__ used,
                                 typename C2<T>::t *__restrict__ dinv, int *__restrict__ err) {
  using T2 = typename C2<T>::t;
  const int m = blockIdx.x;
  const size_t nn = (size_t)n * n;
  T2 *Am = A + m * nn;
  int *um = used + (size_t)m * n;
  __shared__ T sv[256];
  __shared__ int si[256];
  T best = -1;
  int bi = 0x7fffffff;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    if (um[i]) continue;
    T2 v = Am[i + (size_t)n * k];
    T s = fabs(v.x) + fabs(v.y);
    if (s > best || (s == best && i < bi)) { best = s; bi = i; }
  }
  sv[threadIdx.x] = best;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int s = blockDim.x / 2; s; s >>= 1) {
    if (threadIdx.x < s) {
      T ob = sv[threadIdx.x + s];
      int oi = si[threadIdx.x + s];
      if (ob > sv[threadIdx.x] || (ob == sv[threadIdx.x] && oi < si[threadIdx.x])) { sv[threadIdx.x] = ob; si[threadIdx.x] = oi; }
    }
    __syncthreads();
  }
  // NaN entries never win the comparison: fall back to row k's slot and flag
  const int p = (si[0] >= 0 && si[0] < n) ? si[0] : k;
  __shared__ T2 sd;
  if (threadIdx.x == 0) {
    if (!(sv[0] > (T)0) || si[0] != p) atomicExch(err, 3);
    piv[(size_t)m * n + k] = p;
    um[p] = 1;
    const T2 pk = Am[p + (size_t)n * k];
    sd = (pk.x == (T)0 && pk.y == (T)0) ? mk<T>(0, 0) : crecip<T>(pk);
    dinv[m] = sd;
  }
  __syncthreads();
  const T2 d = sd;
  // prow: the pivot row; fcol: the pivot column times the pivot's reciprocal
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    prow[(size_t)m * n + j] = Am[p + (size_t)n * j];
    fcol[(size_t)m * n + j] = cmul(Am[j + (size_t)n * k], d);
  }
}

// one pivot step on all matrices: block (32 rows x 8 columns) of matrix blockIdx.z
template <typename T>
__global__ void __launch_bounds__(256) gj_update_kernel(typename C2<T>::t *__restrict__ A, int n, int k,
                                                        const typename C2<T>::t *__restrict__ prow,
                                                        const typename C2<T>::t *__restrict__ fcol,
                                                        const int *__restrict__ piv,
                                                        const typename C2<T>::t *__restrict__ dinv) {
  using T2 = typename C2<T>::t;
  const int m = blockIdx.z;
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= n || j >= n) return;
  const int p = piv[(size_t)m * n + k];
  const T2 d = dinv[m];
  if (d.x == (T)0 && d.y == (T)0) return;  // singular: flagged by the select kernel
  T2 *a = A + (size_t)m * n * n + i + (size_t)n * j;
  const T2 pj = prow[(size_t)m * n + j];
  if (i == p) {
    *a = (j == k) ? d : cmul(pj, d);
  } else {
    const T2 f = fcol[(size_t)m * n + i];
    if (j == k) {
      *a = mk<T>(-f.x, -f.y);
    } else {
      T2 v = *a;  // a - f pj in four FMAs
      v.x = fma(-f.x, pj.x, v.x); v.x = fma(f.y, pj.y, v.x);
      v.y = fma(-f.x, pj.y, v.y); v.y = fma(-f.y, pj.x, v.y);
      *a = v;
    }
  }
}

// inv(r, c) = A(piv[r], ipiv[c]) with ipiv[piv[k]] = k
template <typename T2>
__global__ void gj_unscramble_kernel(const T2 *__restrict__ A, int n, const int *__restrict__ piv,
                                     int *__restrict__ ipiv, T2 *__restrict__ out) {
  const int m = blockIdx.y;
  const size_t nn = (size_t)n * n;
  const int *pm = piv + (size_t)m * n;
  int *ip = ipiv + (size_t)m * n;
  // every block rebuilds the inverse permutation it needs in shared memory
  extern __shared__ int sip[];
  for (int k = threadIdx.x; k < n; k += blockDim.x) sip[pm[k]] = k;
  __syncthreads();
  if (blockIdx.x == 0)
    for (int k = threadIdx.x; k < n; k += blockDim.x) ip[k] = sip[k];
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < nn; idx += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(idx % n), c = (int)(idx / n);
    out[m * nn + idx] = A[m * nn + pm[r] + (size_t)n * sip[c]];
  }
}

int launch_eps_build(const double2 *chi, const EpsArgs &a, double2 *A, cudaStream_t st) {
  const size_t nn = (size_t)a.ng * a.ng;
  dim3 grid((unsigned)std::min<size_t>((nn + 255) / 256, 4096), a.ndir * a.nen);
  eps_build_kernel<<<grid, 256, 0, st>>>(chi, a, A);
  RP_CUDA(cudaGetLastError());
  return 1;
}

template <typename T>
static int gauss_jordan(typename C2<T>::t *A, int n, int nmat, typename C2<T>::t *prow, typename C2<T>::t *fcol,
                        int *piv, int *used, typename C2<T>::t *out, int *err, cudaStream_t st) {
  int launches = 0;
  RP_CUDA(cudaMemsetAsync(used, 0, sizeof(int) * (size_t)n * nmat, st));
  const size_t nn = (size_t)n * n;
  // reciprocals of the pivots live after the pivot column copies
  typename C2<T>::t *dinv = fcol + (size_t)nmat * n;
  dim3 ublk(32, 8), ugrid2((n + 31) / 32, (n + 7) / 8, nmat);
  dim3 ugrid((unsigned)std::min<size_t>((nn + 255) / 256, 2048), nmat);
  for (int k = 0; k < n; k++) {
    gj_select_kernel<T><<<nmat, 256, 0, st>>>(A, n, k, prow, fcol, piv, used, dinv, err);
    gj_update_kernel<T><<<ugrid2, ublk, 0, st>>>(A, n, k, prow, fcol, piv, dinv);
    launches += 2;
  }
  RP_CUDA(cudaGetLastError());
  // `used` doubles as the inverse-permutation scratch of the unscramble step
  gj_unscramble_kernel<<<ugrid, 256, sizeof(int) * n, st>>>(A, n, piv, used, out);
  RP_CUDA(cudaGetLastError());
  return launches + 1;
}

int launch_gauss_jordan(double2 *A, int n, int nmat, double2 *prow, double2 *fcol, int *piv, int *used,
                        double2 *out, int *err, cudaStream_t st) {
  return gauss_jordan<double>(A, n, nmat, prow, fcol, piv, used, out, err, st);
}

// ---------------------------------------------------------------------------
// Mixed-precision inverse (fast path).  GB300's FP32 rate is many times its
// FP64 rate, so the O(n^3) work runs on FP32 instructions:
//   X0 = FP32 Gauss-Jordan of fl32(A);
//   R  = I - A X0, every product exact (A = a_hi + a_lo, a_hi x as a rounded
//        product plus its FMA remainder) and the sums kept as float pairs
//        (TwoSum), so R is accurate to a few units of FP32 in its own size;
//   X  = X0 + X0 R  (the product in FP32, the sum in FP64).
// One Newton step squares the residual: |A^-1 - X| / |A^-1| <= |R|^2 plus the
// FP32 error of X0 R (about 1e-11 here).  The caller checks |R|_F per matrix
// and falls back to the FP64 Gauss-Jordan when it exceeds 1e-3.

// A split once into float pairs: hl = (re hi, im hi, re lo, im lo); b = the high parts
// (the Gauss-Jordan works on b in place)
__global__ void split_f32_kernel(const double2 *__restrict__ a, size_t n, float2 *__restrict__ b,
                                 float4 *__restrict__ hl) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double2 v = a[i];
    const float hr = (float)v.x, hi = (float)v.y;
    b[i] = make_float2(hr, hi);
    hl[i] = make_float4(hr, hi, (float)(v.x - (double)hr), (float)(v.y - (double)hi));
  }
}

constexpr int MT = 32;  // output tile of the complex GEMMs below (MT x MT per CTA, 2 x 2 per thread)

// s + c += a x: a = ah + al, ah x = p + e exactly (TwoProd), s + p = t + er exactly
// (TwoSum); the _rn intrinsics keep the compiler from fusing the steps
__device__ __forceinline__ void ff_acc(float &s, float &c, float ah, float al, float x) {
  const float p = __fmul_rn(ah, x), e = fmaf(ah, x, -p);
  const float t = __fadd_rn(s, p), z = __fsub_rn(t, s);
  const float er = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
  s = t;
  c = fmaf(al, x, c + (er + e));
}

// R = I - A X0 per matrix (column-major n x n), A in FP64 split into float
// pairs, X0 in FP32; R in FP32 and sum |R|^2 per matrix into rn
__global__ void __launch_bounds__(256) resid_ff_kernel(const float4 *__restrict__ A, const float2 *__restrict__ X,
                                                       int n, float2 *__restrict__ R, float *__restrict__ rn) {
  const int m = blockIdx.z, i0 = blockIdx.x * MT, j0 = blockIdx.y * MT;
  const size_t nn = (size_t)n * n;
  const float4 *Am = A + m * nn;
  const float2 *Xm = X + m * nn;
  __shared__ float4 As[MT][MT];       // [k][row]: (re hi, im hi, re lo, im lo)
  __shared__ float2 Bs[MT][MT + 1];   // [k][col]
  const int tid = threadIdx.x, ti = tid & 15, tj = tid >> 4;
  float sr[2][2], cr[2][2], si[2][2], ci[2][2];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) sr[a][b] = cr[a][b] = si[a][b] = ci[a][b] = 0.f;
  for (int k0 = 0; k0 < n; k0 += MT) {
    for (int l = tid; l < MT * MT; l += 256) {
      const int r = l % MT, kk = l / MT;          // A: rows fastest (coalesced)
      As[kk][r] = (i0 + r < n && k0 + kk < n) ? Am[(i0 + r) + (size_t)n * (k0 + kk)] : make_float4(0.f, 0.f, 0.f, 0.f);
      const int kx = l % MT, c = l / MT;          // X: k fastest (coalesced)
      float2 x = make_float2(0.f, 0.f);
      if (k0 + kx < n && j0 + c < n) x = Xm[(k0 + kx) + (size_t)n * (j0 + c)];
      Bs[kx][c] = x;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < MT; kk++) {
      float4 av[2];
      float2 bv[2];
#pragma unroll
      for (int a = 0; a < 2; a++) av[a] = As[kk][ti + 16 * a];
#pragma unroll
      for (int b = 0; b < 2; b++) bv[b] = Bs[kk][tj + 16 * b];
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) {
          // (ar + i ai)(xr + i xi): re = ar xr - ai xi, im = ar xi + ai xr
          ff_acc(sr[a][b], cr[a][b], av[a].x, av[a].z, bv[b].x);
          ff_acc(sr[a][b], cr[a][b], -av[a].y, -av[a].w, bv[b].y);
          ff_acc(si[a][b], ci[a][b], av[a].x, av[a].z, bv[b].y);
          ff_acc(si[a][b], ci[a][b], av[a].y, av[a].w, bv[b].x);
        }
    }
    __syncthreads();
  }
  float ss = 0.f;
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) {
      const int i = i0 + ti + 16 * a, j = j0 + tj + 16 * b;
      if (i >= n || j >= n) continue;
      // (delta - s) is exact near 1 (Sterbenz), then the pair's low part
      const float re = ((i == j ? 1.f : 0.f) - sr[a][b]) - cr[a][b];
      const float im = -si[a][b] - ci[a][b];
      R[m * nn + i + (size_t)n * j] = make_float2(re, im);
      ss = fmaf(re, re, fmaf(im, im, ss));
    }
  for (int o = 16; o; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  if ((tid & 31) == 0) atomicAdd(&rn[m], ss);
}

// out = X0 + X0 R: the product in FP32, the sum in FP64
__global__ void __launch_bounds__(256) correct_kernel(const float2 *__restrict__ X, const float2 *__restrict__ R,
                                                      int n, double2 *__restrict__ out) {
  const int m = blockIdx.z, i0 = blockIdx.x * MT, j0 = blockIdx.y * MT;
  const size_t nn = (size_t)n * n;
  const float2 *Xm = X + m * nn, *Rm = R + m * nn;
  __shared__ float2 As[MT][MT];
  __shared__ float2 Bs[MT][MT + 1];
  const int tid = threadIdx.x, ti = tid & 15, tj = tid >> 4;
  float2 acc[2][2];
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) acc[a][b] = make_float2(0.f, 0.f);
  for (int k0 = 0; k0 < n; k0 += MT) {
    for (int l = tid; l < MT * MT; l += 256) {
      const int r = l % MT, kk = l / MT;
      As[kk][r] = (i0 + r < n && k0 + kk < n) ? Xm[(i0 + r) + (size_t)n * (k0 + kk)] : make_float2(0.f, 0.f);
      const int kx = l % MT, c = l / MT;
      Bs[kx][c] = (k0 + kx < n && j0 + c < n) ? Rm[(k0 + kx) + (size_t)n * (j0 + c)] : make_float2(0.f, 0.f);
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < MT; kk++) {
      float2 av[2], bv[2];
#pragma unroll
      for (int a = 0; a < 2; a++) av[a] = As[kk][ti + 16 * a];
#pragma unroll
      for (int b = 0; b < 2; b++) bv[b] = Bs[kk][tj + 16 * b];
#pragma unroll
      for (int a = 0; a < 2; a++)
#pragma unroll
        for (int b = 0; b < 2; b++) cfma(acc[a][b], av[a], bv[b]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) {
      const int i = i0 + ti + 16 * a, j = j0 + tj + 16 * b;
      if (i >= n || j >= n) continue;
      const float2 x = Xm[i + (size_t)n * j];
      out[m * nn + i + (size_t)n * j] =
          make_double2((double)x.x + (double)acc[a][b].x, (double)x.y + (double)acc[a][b].y);
    }
}

size_t epsinv_mixed_bytes(int n, int nmat) {
  const size_t nn = (size_t)n * n * nmat;
  return sizeof(float4) * nn + sizeof(float2) * (3 * nn + 2 * (size_t)n * nmat + nmat);
}

int launch_epsinv_mixed(const double2 *A, int n, int nmat, void *ws, int *piv, int *used, double2 *out,
                        float *rnorm, int *err, cudaStream_t st) {
  const size_t nn = (size_t)n * n * nmat;
  float4 *Ahl = (float4 *)ws;
  float2 *A32 = (float2 *)(Ahl + nn), *X0 = A32 + nn, *R = X0 + nn;
  float2 *prow = R + nn, *fcol = prow + (size_t)n * nmat;  // fcol holds nmat reciprocals after the columns
  int launches = 0;
  split_f32_kernel<<<2048, 256, 0, st>>>(A, nn, A32, Ahl);
  launches++;
  launches += gauss_jordan<float>(A32, n, nmat, prow, fcol, piv, used, X0, err, st);
  RP_CUDA(cudaMemsetAsync(rnorm, 0, sizeof(float) * nmat, st));
  dim3 g((n + MT - 1) / MT, (n + MT - 1) / MT, nmat);
  resid_ff_kernel<<<g, 256, 0, st>>>(Ahl, X0, n, R, rnorm);
  correct_kernel<<<g, 256, 0, st>>>(X0, R, n, out);
  launches += 3;
  RP_CUDA(cudaGetLastError());
  return launches;
}

}  // namespace rp
