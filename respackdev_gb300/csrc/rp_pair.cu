// rp_pair.cu -- band-pair densities on the dielectric G sphere (K3) and the
// Gamma-point k.p head.
//
// calc_InterStateMatrix (src/chiqw/chiqw_sub.F:97-205) forms, per pair (i vir,
// j occ) and k,
//     f(r) = conj(u_{i,k+q}(r) e^{-2 pi i s.r/N}) u_{j,k}(r)
//     rho(G) = FFT_fw[f](-G)          (scaled by 1/N, e^{-i}; fft3_fw)
// with s the reciprocal-lattice shift that folds k+q back into the mesh
// (search_kq), and rounds rho to single precision (chiqw_sub.F:201).  The
// shift phase and the -G read-out combine into one forward DFT of
// conj(u_i) u_j at the frequencies (-G - s) mod N, so this kernel evaluates a
// pruned DFT: per z-slab of the product an x pass (only the x frequencies of
// the sphere), a y pass (only its (x,y) frequency pairs), then each G's z term
// is accumulated.  One CTA owns one k and up to JMAX pairs that share the same
// virtual band, so u_{i,k+q} is read from HBM once per slab and reused.
#include "rp_dev.cuh"
#include "rp_host.h"

namespace rp {

__device__ __forceinline__ int modp2(int a, int n) { int m = a % n; return m < 0 ? m + n : m; }

struct PairArgs {
  int ntk, ncb, n1, n2, n3, ng, R1, R2;
  const int *kpq, *shift, *lg0;
  const int *chunk_vir, *chunk_first, *chunk_count, *pair_list, *pair_occ;
  int jmax;
};

template <typename T> struct ToT2;
template <> struct ToT2<float> {
  __device__ static float2 cvt(float2 v) { return v; }
  __device__ static float2 tw(int j, int n) { float s, c; sincospif(-2.0f * j / n, &s, &c); return make_float2(c, s); }
};
template <> struct ToT2<double> {
  __device__ static double2 cvt(float2 v) { return make_double2(v.x, v.y); }
  __device__ static double2 tw(int j, int n) { double s, c; sincospi(-2.0 * j / n, &s, &c); return make_double2(c, s); }
};

template <typename T>
__global__ void __launch_bounds__(256) pair_density_kernel(const float2 *__restrict__ ur, PairArgs a,
                                                           typename C2<T>::t *__restrict__ out) {
  using T2 = typename C2<T>::t;
  extern __shared__ __align__(16) unsigned char smem[];
  const int k = blockIdx.x, ch = blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
  const int n1 = a.n1, n2 = a.n2, n3 = a.n3, n12 = n1 * n2, ng = a.ng;
  const bool c1 = 2 * a.R1 + 1 <= n1, c2 = 2 * a.R2 + 1 <= n2;
  const int D1 = c1 ? 2 * a.R1 + 1 : n1, D2 = c2 ? 2 * a.R2 + 1 : n2;
  const int kq = a.kpq[k];
  const int s1 = a.shift[3 * k], s2 = a.shift[3 * k + 1], s3 = a.shift[3 * k + 2];
  const int vir = a.chunk_vir[ch], first = a.chunk_first[ch], cnt = a.chunk_count[ch];
  // twiddle tables TW1[x][c1] = e^{-2 pi i f1(c1) x / n1}, TW2[y][c2] likewise: the
  // lanes of a warp read consecutive entries, and no index arithmetic per term
  T2 *TW1 = (T2 *)smem, *TW2 = TW1 + (size_t)n1 * D1, *tw3 = TW2 + (size_t)n2 * D2;
  T2 *ui = tw3 + n3;              // n12
  T2 *P = ui + n12;               // n12
  T2 *X = P + n12;                // D1*n2
  T2 *Y = X + D1 * n2;            // D1*D2
  T2 *acc = Y + D1 * D2;          // jmax*ng
  int *f1 = (int *)(acc + (size_t)a.jmax * ng), *f2 = f1 + D1;
  int *gsel = f2 + D2;            // ng: c1 | c2 << 10 | f3 << 20
  for (int j = tid; j < n3; j += nt) tw3[j] = ToT2<T>::tw(j, n3);
  for (int j = tid; j < D1; j += nt) f1[j] = c1 ? modp2(-(j - a.R1) - s1, n1) : j;
  for (int j = tid; j < D2; j += nt) f2[j] = c2 ? modp2(-(j - a.R2) - s2, n2) : j;
  __syncthreads();
  for (int i = tid; i < n1 * D1; i += nt) { const int x = i / D1, c = i % D1; TW1[i] = ToT2<T>::tw((f1[c] * x) % n1, n1); }
  for (int i = tid; i < n2 * D2; i += nt) { const int y = i / D2, c = i % D2; TW2[i] = ToT2<T>::tw((f2[c] * y) % n2, n2); }
  for (int g = tid; g < ng; g += nt) {
    const int *l = a.lg0 + 3 * g;
    int i1 = c1 ? l[0] + a.R1 : modp2(-l[0] - s1, n1);
    int i2 = c2 ? l[1] + a.R2 : modp2(-l[1] - s2, n2);
    int i3 = modp2(-l[2] - s3, n3);
    gsel[g] = i1 | (i2 << 10) | (i3 << 20);
  }
  for (int i = tid; i < a.jmax * ng; i += nt) acc[i] = mk<T>(0, 0);
  __syncthreads();
  const float2 *ui_g = ur + ((size_t)kq * a.ncb + vir) * (size_t)n12 * n3;
  for (int z = 0; z < n3; z++) {
    for (int i = tid; i < n12; i += nt) ui[i] = ToT2<T>::cvt(ui_g[(size_t)z * n12 + i]);
    __syncthreads();
    for (int jj = 0; jj < cnt; jj++) {
      const int occ = a.pair_occ[a.pair_list[first + jj]];
      const float2 *uj_g = ur + ((size_t)k * a.ncb + occ) * (size_t)n12 * n3 + (size_t)z * n12;
      for (int i = tid; i < n12; i += nt) P[i] = cmul(cconj(ui[i]), ToT2<T>::cvt(uj_g[i]));
      __syncthreads();
      // x pass: X[c1,y] = sum_x P[x,y] TW1[x][c1], two c1 (cc, cc + H1) per thread
      const int H1 = (D1 + 1) / 2, H2 = (D2 + 1) / 2;
      for (int o = tid; o < H1 * n2; o += nt) {
        const int cc = o % H1, y = o / H1, cb = min(cc + H1, D1 - 1);
        T2 sa = mk<T>(0, 0), sb = mk<T>(0, 0);
        const T2 *pr = P + (size_t)n1 * y;
        for (int x = 0; x < n1; x++) {
          const T2 pv = pr[x];
          cfma(sa, pv, TW1[(size_t)x * D1 + cc]);
          cfma(sb, pv, TW1[(size_t)x * D1 + cb]);
        }
        X[cc + D1 * y] = sa;
        if (cc + H1 < D1) X[cc + H1 + D1 * y] = sb;
      }
      __syncthreads();
      // y pass: Y[c1,c2] = sum_y X[c1,y] TW2[y][c2], two c2 (c, c + H2) per thread
      for (int o = tid; o < D1 * H2; o += nt) {
        const int cc1 = o % D1, cc2 = o / D1, cb = min(cc2 + H2, D2 - 1);
        T2 sa = mk<T>(0, 0), sb = mk<T>(0, 0);
        for (int y = 0; y < n2; y++) {
          const T2 xv = X[cc1 + D1 * y];
          cfma(sa, xv, TW2[(size_t)y * D2 + cc2]);
          cfma(sb, xv, TW2[(size_t)y * D2 + cb]);
        }
        Y[cc1 + D1 * cc2] = sa;
        if (cc2 + H2 < D2) Y[cc1 + D1 * (cc2 + H2)] = sb;
      }
      __syncthreads();
      // z term of each G
      T2 *ac = acc + (size_t)jj * ng;
      for (int g = tid; g < ng; g += nt) {
        const int sel = gsel[g];
        const int i1 = sel & 1023, i2 = (sel >> 10) & 1023, i3 = sel >> 20;
        cfma(ac[g], Y[i1 + D1 * i2], tw3[(i3 * z) % n3]);
      }
    }
    __syncthreads();
  }
  const T inv = (T)(1.0 / ((double)n12 * n3));
  for (int jj = 0; jj < cnt; jj++) {
    const int p = a.pair_list[first + jj];
    T2 *dst = out + ((size_t)p * a.ntk + k) * ng;
    for (int g = tid; g < ng; g += nt) {
      T2 v = acc[(size_t)jj * ng + g];
      // single-precision rounding of the reference's CMPLX (chiqw_sub.F:201)
      dst[g] = mk<T>((T)(float)(v.x * inv), (T)(float)(v.y * inv));
    }
  }
}

size_t pair_density_smem(const PairGeom &g, int jmax, bool fp64) {
  const int D1 = 2 * g.R1 + 1 <= g.n1 ? 2 * g.R1 + 1 : g.n1, D2 = 2 * g.R2 + 1 <= g.n2 ? 2 * g.R2 + 1 : g.n2;
  const size_t elt = fp64 ? sizeof(double2) : sizeof(float2);
  return elt * ((size_t)g.n1 * D1 + (size_t)g.n2 * D2 + g.n3 + 2 * (size_t)g.n1 * g.n2 + (size_t)D1 * g.n2 +
                (size_t)D1 * D2 + (size_t)jmax * g.ng) +
         sizeof(int) * ((size_t)D1 + D2 + g.ng);
}

template <typename T>
static int launch_pd(const float2 *ur, const PairGeom &g, const PairChunks &c, typename C2<T>::t *out,
                     cudaStream_t st) {
  using T2 = typename C2<T>::t;
  if (c.nchunk == 0) return 0;
  if (g.n1 > 1023 || g.n2 > 1023 || g.n3 > 1023) fail(1, "FFT box dimension above 1023");
  const size_t smem = pair_density_smem(g, c.jmax, sizeof(T2) == sizeof(double2));
  if (smem > 227 * 1024) fail(1, "pair-density tile needs %zu bytes of shared memory", smem);
  RP_CUDA(cudaFuncSetAttribute(pair_density_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  PairArgs a;
  a.ntk = g.ntk; a.ncb = g.ncb; a.n1 = g.n1; a.n2 = g.n2; a.n3 = g.n3; a.ng = g.ng; a.R1 = g.R1; a.R2 = g.R2;
  a.kpq = g.kpq; a.shift = g.shift; a.lg0 = g.lg0;
  a.chunk_vir = c.chunk_vir; a.chunk_first = c.chunk_first; a.chunk_count = c.chunk_count;
  a.pair_list = c.pair_list; a.pair_occ = c.pair_occ; a.jmax = c.jmax;
  dim3 grid(g.ntk, c.nchunk);
  pair_density_kernel<T><<<grid, 256, smem, st>>>(ur, a, out);
  RP_CUDA(cudaGetLastError());
  return 1;
}

int launch_pair_density_fp64(const float2 *ur, const PairGeom &g, const PairChunks &c, double2 *out,
                             cudaStream_t st) {
  return launch_pd<double>(ur, g, c, out, st);
}
int launch_pair_density_fp32(const float2 *ur, const PairGeom &g, const PairChunks &c, float2 *out,
                             cudaStream_t st) {
  return launch_pd<float>(ur, g, c, out, st);
}

// ---------------------------------------------------------------------------
// Gamma head (chiqw.F:1786-1806, calc_VMab chiqw_sub.F:207-232): one warp per
// (pair, k); vm = i sum_G G conj(C_vir) C_occ, head = -i vm / del_eps, set to
// zero when |del_eps| <= delt (del_eps floored at delt first).
__global__ void gamma_head_kernel(const double2 *__restrict__ cfull, const int *__restrict__ ng0,
                                  const int *__restrict__ kg0, int ntk, int ncb, int ntg, const double *__restrict__ b9,
                                  const double *__restrict__ energy, int ntb, const int *__restrict__ numirr,
                                  const int *__restrict__ pvir, const int *__restrict__ pocc, int npair, double delt,
                                  double2 *__restrict__ head) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= npair * ntk) return;
  const int p = warp / ntk, k = warp % ntk;
  const int bv = pvir[p], bo = pocc[p];
  const double2 *cv = cfull + ((size_t)k * ncb + bv) * ntg, *co = cfull + ((size_t)k * ncb + bo) * ntg;
  double2 s[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
  for (int ig = lane; ig < ng0[k]; ig += 32) {
    const int *g = kg0 + ((size_t)k * ntg + ig) * 3;
    double2 pr = cmul(cconj(cv[ig]), co[ig]);
    for (int d = 0; d < 3; d++) {
      double G = (double)g[0] * b9[d] + (double)g[1] * b9[3 + d] + (double)g[2] * b9[6 + d];
      s[d].x += G * pr.x;
      s[d].y += G * pr.y;
    }
  }
  for (int d = 0; d < 3; d++)
    for (int o = 16; o; o >>= 1) {
      s[d].x += __shfl_xor_sync(0xffffffffu, s[d].x, o);
      s[d].y += __shfl_xor_sync(0xffffffffu, s[d].y, o);
    }
  if (lane == 0) {
    double del = energy[(size_t)numirr[k] * ntb + bv] - energy[(size_t)numirr[k] * ntb + bo];
    if (fabs(del) < delt) del = delt;
    for (int d = 0; d < 3; d++) {
      // vm = i*S ; head = -i*vm/del = S/del
      double2 h = make_double2(s[d].x / del, s[d].y / del);
      if (fabs(del) <= delt) h = make_double2(0, 0);
      head[((size_t)p * ntk + k) * 3 + d] = h;
    }
  }
}

int launch_gamma_head(const double2 *cfull, const int *ng0, const int *kg0, int ntk, int ncb, int ntg,
                      const double *bvec9, const double *energy, int ntb, const int *numirr,
                      const int *pair_vir, const int *pair_occ, int npair, double delt, double2 *head,
                      cudaStream_t st) {
  long nw = (long)npair * ntk;
  if (nw == 0) return 0;
  int blocks = (int)((nw * 32 + 255) / 256);
  gamma_head_kernel<<<blocks, 256, 0, st>>>(cfull, ng0, kg0, ntk, ncb, ntg, bvec9, energy, ntb, numirr, pair_vir,
                                            pair_occ, npair, delt, head);
  RP_CUDA(cudaGetLastError());
  return 1;
}

__global__ void set_head_kernel(double2 *rho, const double2 *head, long nK, int ng, int g0, int ix) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nK) rho[i * ng + g0] = head[i * 3 + ix];
}
int launch_set_head(double2 *rho, const double2 *head, int npair, int ntk, int ng, int g0, int ix, cudaStream_t st) {
  long nK = (long)npair * ntk;
  if (!nK) return 0;
  set_head_kernel<<<(unsigned)((nK + 255) / 256), 256, 0, st>>>(rho, head, nK, ng, g0, ix);
  RP_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace rp
