// rp_int.cu -- kernels of the Wannier-basis interaction integrals (calc_int):
// bare and screened Coulomb V, W (src/calc_int/calc_intW.F) and exchange X, J
// (src/calc_int/calc_intJ.F).
//
// Per q point the pair densities of Wannier functions (calc_InterStateMatrix,
// calc_int_sub.F:102-220) come from the chiqw pair-density kernel, one value per
// (pair, k, G) in single precision as the reference rounds them.  The kernels
// here then
//   int_reduce_kernel   sum over k:  rho_p(R, q+G) = sum_k e^{-2 pi i k.R} rho_pk(G) / |q+G| / NTK
//                       (calc_intW.F:680-767, calc_intJ.F:641-677 and :748-791);
//   int_eps_kernel      T_v(G) = sum_G' eps^-1_q(G,G') conj(rho_v(G')), eps^-1 of the
//                       irreducible q rotated on the fly (make_eps, calc_int_sub.F:222-311)
//                       and rounded to complex(4) as the reference stores it;
//   int_quad_kernel     func / funcw: sums over G of rho_a conj(rho_b) and rho_a T_b,
//                       plus the bare shell beyond the eps sphere (calc_intW.F:833-912);
//   int_fourier_kernel  V(R) = 4 pi / (Omega NTQ) sum_q func(q) e^{-2 pi i q.R} + head
//                       (calc_intW.F:942-985) and the plain q sums of X, J (calc_intJ.F:849-873).
// Everything after the pair densities is FP64, like the reference.
#include <algorithm>

#include "rp_dev.cuh"
#include "rp_host.h"
#include "rp_int.h"

namespace rp {

// rho_out[(r*np + p)*ngp + g]: sum over k of rho_pk(G) times the phase of
// lattice vector r, divided by |q+G| and NTK in the order of the reference:
// j_order = 0 (V/W): (sum_k rho) / |q+G| / NTK; j_order = 1 (X/J): sum_k (rho pf / |q+G|) / NTK,
// at Gamma (sum_k rho pf) / |G| / NTK.  G = 0 at Gamma is zero.
__global__ void int_reduce_kernel(const float2 *__restrict__ rho_pk, const double2 *__restrict__ pf /* [r][k] */,
                                  const double *__restrict__ len, int np, int ntk, int ngp, int g0, int gamma,
                                  int j_order, double2 *__restrict__ rho_out) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x, p = blockIdx.y, r = blockIdx.z;
  if (g >= ngp) return;
  double2 *dst = rho_out + ((size_t)r * np + p) * ngp + g;
  if (gamma && g == g0) { *dst = make_double2(0, 0); return; }
  const double L = len[g];
  const float2 *src = rho_pk + (size_t)p * ntk * ngp + g;
  const double2 *ph = pf + (size_t)r * ntk;
  double2 acc = make_double2(0, 0);
  if (!j_order) {
    for (int k = 0; k < ntk; k++) {
      const float2 v = src[(size_t)k * ngp];
      acc.x += (double)v.x; acc.y += (double)v.y;
    }
    acc = make_double2(acc.x / L / (double)ntk, acc.y / L / (double)ntk);
  } else if (gamma) {
    for (int k = 0; k < ntk; k++) {
      const float2 v = src[(size_t)k * ngp];
      acc = cadd(acc, cmul(make_double2(v.x, v.y), ph[k]));
    }
    acc = make_double2(acc.x / L / (double)ntk, acc.y / L / (double)ntk);
  } else {
    for (int k = 0; k < ntk; k++) {
      const float2 v = src[(size_t)k * ngp];
      const double2 t = cmul(make_double2(v.x, v.y), ph[k]);
      acc.x += t.x / L; acc.y += t.y / L;
    }
    acc = make_double2(acc.x / (double)ntk, acc.y / (double)ntk);
  }
  *dst = acc;
}

// T[(e*nv + v)*nge + g] = sum_{g'} eps(g, g', e) conj(V[v*ngp + g']), eps taken
// from the irreducible array: element (idx[g], idx[g']) (or transposed for a
// time-reversed q) times p1[g] p2[g'], rounded to complex(4).
constexpr int EB_G = 64, EB_V = 8, EB_K = 32;
__global__ void __launch_bounds__(256) int_eps_kernel(const float2 *__restrict__ eps_irr /* [e][NTGQ][NTGQ], col-major */,
                                                      int ntgq, const int *__restrict__ idx,
                                                      const double2 *__restrict__ p1, const double2 *__restrict__ p2,
                                                      int trs, const double2 *__restrict__ V, int nv, int nge, int ngp,
                                                      double2 *__restrict__ T) {
  const int e = blockIdx.z, g0 = blockIdx.x * EB_G, v0 = blockIdx.y * EB_V;
  __shared__ double2 sE[EB_K][EB_G + 1];
  __shared__ double2 sV[EB_V][EB_K];
  const int tid = threadIdx.x;
  const int tg = tid % EB_G, tv = tid / EB_G;  // 64 x 4 threads; each thread 2 columns
  double2 acc[EB_V / 4];
  for (int i = 0; i < EB_V / 4; i++) acc[i] = make_double2(0, 0);
  const float2 *E = eps_irr + (size_t)e * ntgq * ntgq;
  for (int k0 = 0; k0 < nge; k0 += EB_K) {
    for (int i = tid; i < EB_K * EB_G; i += blockDim.x) {
      const int kk = i / EB_G, gg = i % EB_G, g = g0 + gg, gp = k0 + kk;
      double2 val = make_double2(0, 0);
      if (g < nge && gp < nge) {
        const int a = idx[g], b = idx[gp];
        if (a >= 0 && b >= 0) {
          const float2 s = trs == 1 ? E[(size_t)b * ntgq + a] : E[(size_t)a * ntgq + b];
          const double2 w = cmul(cmul(make_double2(s.x, s.y), p1[g]), p2[gp]);
          val = make_double2((double)(float)w.x, (double)(float)w.y);
        }
      }
      sE[kk][gg] = val;
    }
    for (int i = tid; i < EB_V * EB_K; i += blockDim.x) {
      const int vv = i / EB_K, kk = i % EB_K, v = v0 + vv, gp = k0 + kk;
      double2 x = make_double2(0, 0);
      if (v < nv && gp < nge) { x = V[(size_t)v * ngp + gp]; x.y = -x.y; }
      sV[vv][kk] = x;
    }
    __syncthreads();
    for (int kk = 0; kk < EB_K; kk++) {
      const double2 ev = sE[kk][tg];
#pragma unroll
      for (int i = 0; i < EB_V / 4; i++) cfma(acc[i], ev, sV[tv + 4 * i][kk]);
    }
    __syncthreads();
  }
  const int g = g0 + tg;
  if (g < nge)
    for (int i = 0; i < EB_V / 4; i++) {
      const int v = v0 + tv + 4 * i;
      if (v < nv) T[((size_t)e * nv + v) * nge + g] = acc[i];
    }
}

// out[o] for pair o = (a[o], b[o]):
//   screened (T != null): sum_{g<nge} V_a(g) T_b(g) + sum_{nge<=g<ngp} V_a(g) conj(V_b(g))
//   bare     (T == null): sum_{g<ngp} V_a(g) conj(V_b(g))
// out[e*ostride + o]; one warp per output.
__global__ void int_quad_kernel(const double2 *__restrict__ V, const double2 *__restrict__ T, const int *__restrict__ pa,
                                const int *__restrict__ pb, int nout, int nv, int nge, int ngp, int ne,
                                double2 *__restrict__ out, size_t ostride) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nout * ne) return;
  const int o = warp % nout, e = warp / nout;
  const double2 *va = V + (size_t)pa[o] * ngp, *vb = V + (size_t)pb[o] * ngp;
  double2 s = make_double2(0, 0);
  if (T) {
    const double2 *tb = T + ((size_t)e * nv + pb[o]) * nge;
    for (int g = lane; g < nge; g += 32) cfma(s, va[g], tb[g]);
    for (int g = nge + lane; g < ngp; g += 32) cfma(s, va[g], cconj(vb[g]));
  } else {
    for (int g = lane; g < ngp; g += 32) cfma(s, va[g], cconj(vb[g]));
  }
  for (int off = 16; off; off >>= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, off);
    s.y += __shfl_xor_sync(0xffffffffu, s.y, off);
  }
  if (lane == 0) out[(size_t)e * ostride + o] = s;
}

// out[((e*nbox + R)*nwf + j)*nwf + i] = scale * sum_q f[((e*ntq + q)*nwf + j)*nwf + i] * pf[q*nbox + R] + head[e]
__global__ void int_fourier_kernel(const double2 *__restrict__ f, const double2 *__restrict__ pf, int ntq, int nbox,
                                   int nwf, int ne, double scale, const double *__restrict__ head,
                                   double2 *__restrict__ out) {
  const size_t n = (size_t)ne * nbox * nwf * nwf;
  for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int ij = (int)(t % ((size_t)nwf * nwf));
    const int R = (int)((t / ((size_t)nwf * nwf)) % nbox);
    const int e = (int)(t / ((size_t)nwf * nwf * nbox));
    double2 s = make_double2(0, 0);
    for (int q = 0; q < ntq; q++) s = cadd(s, cmul(f[((size_t)e * ntq + q) * nwf * nwf + ij], pf[(size_t)q * nbox + R]));
    out[t] = make_double2(scale * s.x + head[e], scale * s.y);
  }
}

int launch_int_reduce(const float2 *rho_pk, const double2 *pf, const double *len, int np, int ntk, int ngp, int g0,
                      int gamma, int j_order, int nr, double2 *rho_out, cudaStream_t st) {
  if (ngp <= 0 || np <= 0 || nr <= 0) return 0;
  if (np > 65535 || nr > 65535) fail(1, "k sum: %d pairs x %d lattice vectors exceed the grid", np, nr);
  dim3 grid((ngp + 127) / 128, np, nr);
  int_reduce_kernel<<<grid, 128, 0, st>>>(rho_pk, pf, len, np, ntk, ngp, g0, gamma, j_order, rho_out);
  RP_CUDA(cudaGetLastError());
  return 1;
}

int launch_int_eps(const float2 *eps_irr, int ntgq, const int *idx, const double2 *p1, const double2 *p2, int trs,
                   const double2 *V, int nv, int nge, int ngp, int ne, double2 *T, cudaStream_t st) {
  if (nge <= 0 || nv <= 0 || ne <= 0) return 0;
  if ((nv + EB_V - 1) / EB_V > 65535 || ne > 65535) fail(1, "eps product: %d vectors x %d frequencies exceed the grid", nv, ne);
  dim3 grid((nge + EB_G - 1) / EB_G, (nv + EB_V - 1) / EB_V, ne);
  int_eps_kernel<<<grid, 256, 0, st>>>(eps_irr, ntgq, idx, p1, p2, trs, V, nv, nge, ngp, T);
  RP_CUDA(cudaGetLastError());
  return 1;
}

int launch_int_quad(const double2 *V, const double2 *T, const int *pa, const int *pb, int nout, int nv, int nge,
                    int ngp, int ne, double2 *out, size_t ostride, cudaStream_t st) {
  if (nout <= 0 || ne <= 0) return 0;
  const long threads = (long)nout * ne * 32;
  int_quad_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(V, T, pa, pb, nout, nv, nge, ngp, ne, out,
                                                                    ostride);
  RP_CUDA(cudaGetLastError());
  return 1;
}

int launch_int_fourier(const double2 *f, const double2 *pf, int ntq, int nbox, int nwf, int ne, double scale,
                       const double *head, double2 *out, cudaStream_t st) {
  const size_t n = (size_t)ne * nbox * nwf * nwf;
  if (n == 0) return 0;
  const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 4096);
  int_fourier_kernel<<<blocks, 256, 0, st>>>(f, pf, ntq, nbox, nwf, ne, scale, head, out);
  RP_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace rp
