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

__device__ __forceinline__ double2 crecip(double2 b) {
  // 1/b by Smith's algorithm
  if (fabs(b.x) >= fabs(b.y)) {
    double t = b.y / b.x, d = b.x + b.y * t;
    return make_double2(1.0 / d, -t / d);
  }
  double t = b.x / b.y, d = b.x * t + b.y;
  return make_double2(t / d, -1.0 / d);
}

__global__ void gj_select_kernel(double2 *__restrict__ A, int n, int k, double2 *__restrict__ prow,
                                 double2 *__restrict__ fcol, int *__restrict__ piv, int *__restrict__ used,
                                 double2 *__restrict__ dinv, int *__restrict__ err) {
  const int m = blockIdx.x;
  const size_t nn = (size_t)n * n;
  double2 *Am = A + m * nn;
  int *um = used + (size_t)m * n;
  __shared__ double sv[256];
  __shared__ int si[256];
  double best = -1.0;
  int bi = 0x7fffffff;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    if (um[i]) continue;
    double2 v = Am[i + (size_t)n * k];
    double s = fabs(v.x) + fabs(v.y);
    if (s > best || (s == best && i < bi)) { best = s; bi = i; }
  }
  sv[threadIdx.x] = best;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int s = blockDim.x / 2; s; s >>= 1) {
    if (threadIdx.x < s) {
      double ob = sv[threadIdx.x + s];
      int oi = si[threadIdx.x + s];
      if (ob > sv[threadIdx.x] || (ob == sv[threadIdx.x] && oi < si[threadIdx.x])) { sv[threadIdx.x] = ob; si[threadIdx.x] = oi; }
    }
    __syncthreads();
  }
  // NaN entries never win the comparison: fall back to row k's slot and flag
  const int p = (si[0] >= 0 && si[0] < n) ? si[0] : k;
  __shared__ double2 sd;
  if (threadIdx.x == 0) {
    if (!(sv[0] > 0.0) || si[0] != p) atomicExch(err, 3);
    piv[(size_t)m * n + k] = p;
    um[p] = 1;
    const double2 pk = Am[p + (size_t)n * k];
    sd = (pk.x == 0.0 && pk.y == 0.0) ? make_double2(0.0, 0.0) : crecip(pk);
    dinv[m] = sd;
  }
  __syncthreads();
  const double2 d = sd;
  // prow: the pivot row; fcol: the pivot column times the pivot's reciprocal
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    prow[(size_t)m * n + j] = Am[p + (size_t)n * j];
    fcol[(size_t)m * n + j] = cmul(Am[j + (size_t)n * k], d);
  }
}

// one pivot step on all matrices: block (32 rows x 8 columns) of matrix blockIdx.z
__global__ void __launch_bounds__(256) gj_update_kernel(double2 *__restrict__ A, int n, int k,
                                                        const double2 *__restrict__ prow,
                                                        const double2 *__restrict__ fcol, const int *__restrict__ piv,
                                                        const double2 *__restrict__ dinv) {
  const int m = blockIdx.z;
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= n || j >= n) return;
  const int p = piv[(size_t)m * n + k];
  const double2 d = dinv[m];
  if (d.x == 0.0 && d.y == 0.0) return;  // singular: flagged by the select kernel
  double2 *a = A + (size_t)m * n * n + i + (size_t)n * j;
  const double2 pj = prow[(size_t)m * n + j];
  if (i == p) {
    *a = (j == k) ? d : cmul(pj, d);
  } else {
    const double2 f = fcol[(size_t)m * n + i];
    if (j == k) {
      *a = make_double2(-f.x, -f.y);
    } else {
      double2 v = *a;  // a - f pj in four FMAs
      v.x = fma(-f.x, pj.x, v.x); v.x = fma(f.y, pj.y, v.x);
      v.y = fma(-f.x, pj.y, v.y); v.y = fma(-f.y, pj.x, v.y);
      *a = v;
    }
  }
}

// inv(r, c) = A(piv[r], ipiv[c]) with ipiv[piv[k]] = k
__global__ void gj_unscramble_kernel(const double2 *__restrict__ A, int n, const int *__restrict__ piv,
                                     int *__restrict__ ipiv, double2 *__restrict__ out) {
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

int launch_gauss_jordan(double2 *A, int n, int nmat, double2 *prow, double2 *fcol, int *piv, int *used,
                        double2 *out, int *err, cudaStream_t st) {
  int launches = 0;
  RP_CUDA(cudaMemsetAsync(used, 0, sizeof(int) * (size_t)n * nmat, st));
  const size_t nn = (size_t)n * n;
  // reciprocals of the pivots live after the pivot column copies
  double2 *dinv = fcol + (size_t)nmat * n;
  dim3 ublk(32, 8), ugrid2((n + 31) / 32, (n + 7) / 8, nmat);
  dim3 ugrid((unsigned)std::min<size_t>((nn + 255) / 256, 2048), nmat);
  for (int k = 0; k < n; k++) {
    gj_select_kernel<<<nmat, 256, 0, st>>>(A, n, k, prow, fcol, piv, used, dinv, err);
    gj_update_kernel<<<ugrid2, ublk, 0, st>>>(A, n, k, prow, fcol, piv, dinv);
    launches += 2;
  }
  RP_CUDA(cudaGetLastError());
  // `used` doubles as the inverse-permutation scratch of the unscramble step
  gj_unscramble_kernel<<<ugrid, 256, sizeof(int) * n, st>>>(A, n, piv, used, out);
  RP_CUDA(cudaGetLastError());
  return launches + 1;
}

}  // namespace rp
