// rp_eps.cu -- dielectric matrix and its inverse in FP64 (K6).
//
// calc_eps_rpa (src/chiqw/chiqw_sub.F:386-457): chi0 *= 2 (spin), then
//     eps(G,G') = delta - chi0 2 tpi / (|q+G| |q+G'|)
// and calc_eps_rpa_q_0 (:459-568) at Gamma: head 1 - chi0 2 tpi plus the Drude
// term cmplx(-wd^2/(w^2+delt^2), delt wd^2/(w^3+w delt^2)) (single precision,
// w = Re(em), 1e-5 when zero), wings divided by one |q+G| only.
// invZGE (invZGE.F90:1-22) inverts with LAPACK zgetrf + zgetri; here every
// (frequency, direction) matrix is inverted by Gauss-Jordan elimination with
// partial pivoting on |re|+|im| (izamax's norm), all matrices at once, and the
// row/column permutation undone at the end.  The pivot steps run in panels of
// b columns: a panel's steps in shared memory (one CTA per matrix), then one
// rank-b update of every other column (blocked_gauss_jordan below).
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

// ---------------------------------------------------------------------------
// Blocked Gauss-Jordan.  The b pivot steps k0 .. k0 + b - 1 touch every column,
// but only the panel's own columns decide the pivots.  So the panel runs its b
// steps alone (gj_panel_kernel), and the other columns T take the b steps at
// once: with P the panel's pivot rows, GJ leaves in panel column t the image
// of the unit vector e_{P_t} under the b steps, and every column x transforms
// as x <- x - (E_P - Pan) x_P, i.e.
//   A[:,T] <- (A[:,T] with rows P zeroed) + Pan A_old[P,T]
// (gj_trail_kernel, A_old[P,T] copied by gj_prows_kernel before the update).
// Per element the same operations as the one-step-at-a-time elimination up to
// the order of the b-term sums; the matrices are read and written once per
// panel instead of once per pivot.

// widest panel: 32 columns in FP32, 16 in FP64 (the trailing update's 64-row
// tiles of the panel and the pivot rows stay within 32 KB of shared memory)
template <typename T>
__host__ __device__ constexpr int panel_max() { return sizeof(T) == 4 ? 32 : 16; }

// panel width for n: the panel (b columns), the scaled pivot column and the
// row flags in shared memory
template <typename T>
int panel_width(int n) {
  const long avail = 200L * 1024 - (long)n * (sizeof(typename C2<T>::t) + sizeof(int));
  long b = avail / ((long)n * (long)sizeof(typename C2<T>::t));
  b = b > panel_max<T>() ? panel_max<T>() : b;
  return b < 1 ? 1 : (int)b;
}

template <typename T>
__global__ void __launch_bounds__(512) gj_panel_kernel(typename C2<T>::t *__restrict__ A, int n, int k0, int b,
                                                       int *__restrict__ piv, int *__restrict__ used,
                                                       typename C2<T>::t *__restrict__ prows, int *__restrict__ err) {
  using T2 = typename C2<T>::t;
  const int m = blockIdx.x, tid = threadIdx.x, nth = blockDim.x;
  const size_t nn = (size_t)n * n;
  T2 *Am = A + m * nn;
  int *um = used + (size_t)m * n;
  int *pm = piv + (size_t)m * n;
  extern __shared__ __align__(16) unsigned char smem[];
  T2 *pan = (T2 *)smem;                 // [t][i]: panel column t
  T2 *fc = pan + (size_t)b * n;         // the pivot column times the pivot's reciprocal
  int *us = (int *)(fc + n);            // rows used as pivots
  __shared__ T sv[32];
  __shared__ int si[32];
  __shared__ T2 prow[panel_max<T>()], sd;
  __shared__ int sp;
  for (int t = 0; t < b; t++)
    for (int i = tid; i < n; i += nth) pan[(size_t)t * n + i] = Am[i + (size_t)n * (k0 + t)];
  for (int i = tid; i < n; i += nth) us[i] = um[i];
  __syncthreads();
  for (int t = 0; t < b; t++) {
    // pivot: the largest |re|+|im| of column t among unused rows, lowest row on ties
    T best = -1;
    int bi = 0x7fffffff;
    for (int i = tid; i < n; i += nth) {
      if (us[i]) continue;
      const T2 v = pan[(size_t)t * n + i];
      const T s = fabs(v.x) + fabs(v.y);
      if (s > best || (s == best && i < bi)) { best = s; bi = i; }
    }
    for (int o = 16; o; o >>= 1) {
      const T ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if ((tid & 31) == 0) { sv[tid >> 5] = best; si[tid >> 5] = bi; }
    __syncthreads();
    if (tid == 0) {
      for (int w = 1; w < (nth >> 5); w++)
        if (sv[w] > best || (sv[w] == best && si[w] < bi)) { best = sv[w]; bi = si[w]; }
      // NaN entries never win the comparison: fall back to row k's slot and flag
      const int k = k0 + t;
      const int p = (bi >= 0 && bi < n) ? bi : k;
      if (!(best > (T)0) || bi != p) atomicExch(err, 3);
      pm[k] = p;
      us[p] = 1;
      const T2 pk = pan[(size_t)t * n + p];
      sd = (pk.x == (T)0 && pk.y == (T)0) ? mk<T>(0, 0) : crecip<T>(pk);
      sp = p;
    }
    __syncthreads();
    const T2 d = sd;
    const int p = sp;
    if (d.x == (T)0 && d.y == (T)0) continue;  // singular: flagged above
    if (tid < b) prow[tid] = pan[(size_t)tid * n + p];
    for (int i = tid; i < n; i += nth) fc[i] = cmul(pan[(size_t)t * n + i], d);
    __syncthreads();
    // columns outer, rows inner (no index division); a thread keeps its rows'
    // scaled pivot-column values in registers across the columns
    for (int i0 = 0; i0 < n; i0 += nth) {
      const int i = i0 + tid;
      if (i >= n) continue;
      const T2 f = fc[i];
      for (int j = 0; j < b; j++) {
        T2 &a = pan[(size_t)j * n + i];
        const T2 pj = prow[j];
        if (i == p) {
          a = (j == t) ? d : cmul(pj, d);
        } else if (j == t) {
          a = mk<T>(-f.x, -f.y);
        } else {
          a.x = fma(-f.x, pj.x, a.x); a.x = fma(f.y, pj.y, a.x);
          a.y = fma(-f.x, pj.y, a.y); a.y = fma(-f.y, pj.x, a.y);
        }
      }
    }
    __syncthreads();
  }
  for (int t = 0; t < b; t++)
    for (int i = tid; i < n; i += nth) Am[i + (size_t)n * (k0 + t)] = pan[(size_t)t * n + i];
  for (int i = tid; i < n; i += nth) um[i] = us[i];
}

// The panel's pivot rows outside the panel, before the trailing update:
// prows[m][t][j] = A[P_t, j].  Row reads of column-major matrices are one
// sector per element, so they run as their own grid (matrix, panel column)
// for the memory parallelism.
template <typename T>
__global__ void __launch_bounds__(256) gj_prows_kernel(const typename C2<T>::t *__restrict__ A, int n, int k0, int b,
                                                       const int *__restrict__ piv,
                                                       typename C2<T>::t *__restrict__ prows) {
  const int t = blockIdx.x, m = blockIdx.y;
  const size_t nn = (size_t)n * n;
  const int p = piv[(size_t)m * n + k0 + t];
  const typename C2<T>::t *Am = A + m * nn;
  typename C2<T>::t *pr = prows + ((size_t)m * b + t) * n;
  for (int j = threadIdx.x; j < n; j += blockDim.x)
    if (j < k0 || j >= k0 + b) pr[j] = Am[p + (size_t)n * j];
}

constexpr int TT = 64;  // trailing-update tile (TT x TT per CTA, 4 x 4 per thread)

// A[:,T] <- (A[:,T] with the panel's pivot rows zeroed) + Pan A_old[P,T]
template <typename T>
__global__ void __launch_bounds__(256) gj_trail_kernel(typename C2<T>::t *__restrict__ A, int n, int k0, int b,
                                                       const int *__restrict__ piv,
                                                       const typename C2<T>::t *__restrict__ prows) {
  using T2 = typename C2<T>::t;
  const int m = blockIdx.z, i0 = blockIdx.x * TT, j0 = blockIdx.y * TT, tid = threadIdx.x;
  // a tile of panel columns only: nothing to do
  if (j0 >= k0 && j0 + TT <= k0 + b) return;
  const size_t nn = (size_t)n * n;
  T2 *Am = A + m * nn;
  const T2 *pr = prows + (size_t)m * b * n;
  __shared__ T2 Ps[panel_max<T>()][TT];   // panel rows i0 .., column t
  __shared__ T2 Rs[panel_max<T>()][TT];   // pivot row t, columns j0 ..
  __shared__ int isp[TT];
  if (tid < TT) isp[tid] = 0;
  __syncthreads();
  if (tid < b) {
    const int p = piv[(size_t)m * n + k0 + tid];
    if (p >= i0 && p < i0 + TT) isp[p - i0] = 1;
  }
  for (int l = tid; l < b * TT; l += 256) {
    const int r = l % TT, t = l / TT;
    Ps[t][r] = (i0 + r < n) ? Am[(i0 + r) + (size_t)n * (k0 + t)] : mk<T>(0, 0);
    Rs[t][r] = (j0 + r < n) ? pr[(size_t)t * n + j0 + r] : mk<T>(0, 0);
  }
  __syncthreads();
  const int ti = tid & 15, tj = tid >> 4;
  T2 acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int c = 0; c < 4; c++) acc[a][c] = mk<T>(0, 0);
  for (int t = 0; t < b; t++) {
    T2 pv[4], rv[4];
#pragma unroll
    for (int a = 0; a < 4; a++) pv[a] = Ps[t][ti + 16 * a];
#pragma unroll
    for (int c = 0; c < 4; c++) rv[c] = Rs[t][tj + 16 * c];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
      for (int c = 0; c < 4; c++) cfma(acc[a][c], pv[a], rv[c]);
  }
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const int j = j0 + tj + 16 * c;
    if (j >= n || (j >= k0 && j < k0 + b)) continue;
#pragma unroll
    for (int a = 0; a < 4; a++) {
      const int r = ti + 16 * a, i = i0 + r;
      if (i >= n) continue;
      T2 *x = Am + i + (size_t)n * j;
      const T2 v = isp[r] ? mk<T>(0, 0) : *x;
      *x = mk<T>(v.x + acc[a][c].x, v.y + acc[a][c].y);
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

// Blocked Gauss-Jordan of nmat matrices (n x n, column-major, consecutive) in
// place, then the unscrambled inverse into out.  prows: nmat * panel_width(n) * n scratch.
template <typename T>
static int blocked_gauss_jordan(typename C2<T>::t *A, int n, int nmat, typename C2<T>::t *prows, int *piv, int *used,
                                typename C2<T>::t *out, int *err, cudaStream_t st) {
  using T2 = typename C2<T>::t;
  int launches = 0;
  RP_CUDA(cudaMemsetAsync(used, 0, sizeof(int) * (size_t)n * nmat, st));
  const int bw = panel_width<T>(n);
  const size_t psmem = ((size_t)bw + 1) * n * sizeof(T2) + sizeof(int) * (size_t)n;
  if (psmem > 227 * 1024) fail(1, "Gauss-Jordan panel of n = %d does not fit in shared memory", n);
  RP_CUDA(cudaFuncSetAttribute(gj_panel_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               smem_cap(gj_panel_kernel<T>)));
  dim3 tgrid((n + TT - 1) / TT, (n + TT - 1) / TT, nmat);
  for (int k0 = 0; k0 < n; k0 += bw) {
    const int b = std::min(bw, n - k0);
    gj_panel_kernel<T><<<nmat, 512, psmem, st>>>(A, n, k0, b, piv, used, prows, err);
    gj_prows_kernel<T><<<dim3(b, nmat), 256, 0, st>>>(A, n, k0, b, piv, prows);
    gj_trail_kernel<T><<<tgrid, 256, 0, st>>>(A, n, k0, b, piv, prows);
    launches += 3;
  }
  RP_CUDA(cudaGetLastError());
  // `used` doubles as the inverse-permutation scratch of the unscramble step
  const size_t nn = (size_t)n * n;
  dim3 ugrid((unsigned)std::min<size_t>((nn + 255) / 256, 2048), nmat);
  gj_unscramble_kernel<<<ugrid, 256, sizeof(int) * n, st>>>(A, n, piv, used, out);
  RP_CUDA(cudaGetLastError());
  return launches + 1;
}

size_t gauss_jordan_scratch_bytes(int n, int nmat) {
  return sizeof(double2) * (size_t)nmat * panel_width<double>(n) * n;
}

int launch_gauss_jordan(double2 *A, int n, int nmat, double2 *prows, int *piv, int *used, double2 *out, int *err,
                        cudaStream_t st) {
  return blocked_gauss_jordan<double>(A, n, nmat, prows, piv, used, out, err, st);
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
  return sizeof(float4) * nn + sizeof(float2) * (3 * nn + (size_t)nmat * panel_width<float>(n) * n);
}

int launch_epsinv_mixed(const double2 *A, int n, int nmat, void *ws, int *piv, int *used, double2 *out,
                        float *rnorm, int *err, cudaStream_t st) {
  const size_t nn = (size_t)n * n * nmat;
  float4 *Ahl = (float4 *)ws;
  float2 *A32 = (float2 *)(Ahl + nn), *X0 = A32 + nn, *R = X0 + nn;
  float2 *prows = R + nn;  // the panels' pivot rows
  int launches = 0;
  split_f32_kernel<<<2048, 256, 0, st>>>(A, nn, A32, Ahl);
  launches++;
  launches += blocked_gauss_jordan<float>(A32, n, nmat, prows, piv, used, X0, err, st);
  RP_CUDA(cudaMemsetAsync(rnorm, 0, sizeof(float) * nmat, st));
  dim3 g((n + MT - 1) / MT, (n + MT - 1) / MT, nmat);
  resid_ff_kernel<<<g, 256, 0, st>>>(Ahl, X0, n, R, rnorm);
  correct_kernel<<<g, 256, 0, st>>>(X0, R, n, out);
  launches += 3;
  RP_CUDA(cudaGetLastError());
  return launches;
}

}  // namespace rp
