// rp_tail.cu -- the band-tail correction applied inside rp_chi0_q (no
// reference counterpart).
//
// A chi0 summed over the bands up to N_CALC_BAND misses the bands above it.  A
// context given a band-tail network file (&param_gpu tail_model) adds the
// network's prediction of that tail to the diagonal of chi0 on the device:
//   1. features per (frequency, |q+G| shell): the shell's mean |q+G|, the shell
//      mean of v chi0 on the diagonal (v = 4 pi / |q+G|^2), the frequency, the
//      lowest and mean energy of the excluded bands above E_F and the
//      excluded/included band ratio, the shell's position (tail_features_kernel);
//   2. the network's forward pass (rp_mlp.cu's kernels);
//   3. chi0(G, G, w) += prediction(w, shell(G)) / tscale |q+G|^2 / (4 pi) for
//      every G but the head at Gamma, in every Gamma direction (tail_apply_kernel).
// The shells are equal-count quantiles of |q+G|; the feature order, the scale
// and the shells are those of respackdev_gb300/tail.py, which trains the network.
#include "rp_dev.cuh"
#include "rp_host.h"

namespace rp {

// one block per frequency, one thread per shell: sums in G order (deterministic)
__global__ void tail_features_kernel(const double2 *__restrict__ chi, int ng, int nen, const int *__restrict__ sh,
                                     const double *__restrict__ qglen, int nshell, const double2 *__restrict__ em,
                                     float e_lo, float e_mean, float ratio, float *__restrict__ X) {
  const int e = blockIdx.x;
  for (int s = threadIdx.x; s < nshell; s += blockDim.x) {
    double sr = 0.0, si = 0.0, sq = 0.0;
    int n = 0;
    const double2 *c = chi + (size_t)e * ng * ng;
    for (int g = 0; g < ng; g++) {
      if (sh[g] != s) continue;
      const double ql = qglen[g], v = 4.0 * 3.14159265358979323846 / (ql * ql);
      const double2 d = c[g + (size_t)ng * g];
      sr += v * d.x;
      si += v * d.y;
      sq += ql;
      n++;
    }
    float *x = X + ((size_t)e * nshell + s) * 9;
    const double inv = n ? 1.0 / n : 0.0;
    x[0] = (float)(sq * inv);
    x[1] = (float)(sr * inv);
    x[2] = (float)(si * inv);
    x[3] = (float)em[e].x;
    x[4] = (float)em[e].y;
    x[5] = e_lo;
    x[6] = e_mean;
    x[7] = ratio;
    x[8] = n ? ((float)s + 0.5f) / (float)nshell : 0.f;  // an empty shell keeps zeros, as tail.features
  }
}

__global__ void tail_apply_kernel(double2 *__restrict__ chi, int ng, int nen, int ndir, const int *__restrict__ sh,
                                  const double *__restrict__ qglen, int nshell, const float *__restrict__ Y,
                                  float tscale) {
  const size_t n = (size_t)ndir * nen * ng;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int g = (int)(i % ng);
    const int e = (int)((i / ng) % nen);
    const int dir = (int)(i / ((size_t)ng * nen));
    const int s = sh[g];
    if (s < 0) continue;
    const double ql = qglen[g], f = ql * ql / (4.0 * 3.14159265358979323846) / (double)tscale;
    const float *y = Y + ((size_t)e * nshell + s) * 2;
    double2 *d = chi + ((size_t)dir * nen + e) * ng * ng + g + (size_t)ng * g;
    d->x += (double)y[0] * f;
    d->y += (double)y[1] * f;
  }
}

int launch_tail_features(const double2 *chi, int ng, int nen, const int *sh, const double *qglen, int nshell,
                         const double2 *em, const float *stats, float *X, cudaStream_t st) {
  tail_features_kernel<<<nen, 64, 0, st>>>(chi, ng, nen, sh, qglen, nshell, em, stats[0], stats[1], stats[2], X);
  RP_CUDA(cudaGetLastError());
  return 1;
}

int launch_tail_apply(double2 *chi, int ng, int nen, int ndir, const int *sh, const double *qglen, int nshell,
                      const float *Y, float tscale, cudaStream_t st) {
  const size_t n = (size_t)ndir * nen * ng;
  tail_apply_kernel<<<(unsigned)std::min<size_t>((n + 255) / 256, 1024), 256, 0, st>>>(chi, ng, nen, ndir, sh, qglen,
                                                                                      nshell, Y, tscale);
  RP_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace rp
