// rp_dev.cuh -- device helpers and kernel launchers of the GB300 chiqw library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/respack_gb300.h"

namespace rp {

// ---- complex arithmetic on float2/double2 (device code only) ----------------
#ifdef __CUDACC__
template <typename T> struct C2;
template <> struct C2<float> { using t = float2; };
template <> struct C2<double> { using t = double2; };

template <typename T> __host__ __device__ inline typename C2<T>::t mk(T re, T im) {
  typename C2<T>::t r; r.x = re; r.y = im; return r;
}
__host__ __device__ inline double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ inline double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ inline double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__host__ __device__ inline double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__host__ __device__ inline float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ inline float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

// a += b*c
__device__ inline void cfma(double2 &a, double2 b, double2 c) {
  a.x = fma(b.x, c.x, a.x); a.x = fma(-b.y, c.y, a.x);
  a.y = fma(b.x, c.y, a.y); a.y = fma(b.y, c.x, a.y);
}
__device__ inline void cfma(float2 &a, float2 b, float2 c) {
  a.x = fmaf(b.x, c.x, a.x); a.x = fmaf(-b.y, c.y, a.x);
  a.y = fmaf(b.x, c.y, a.y); a.y = fmaf(b.y, c.x, a.y);
}
#endif  // __CUDACC__

#define RP_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t _e = (call);                                                           \
    if (_e != cudaSuccess) ::rp::fail(-1, "%s: %s (%s:%d)", #call, cudaGetErrorString(_e), __FILE__, __LINE__); \
  } while (0)

// Opt-in shared memory per block of the current device.  Kernels with large
// tiles get this as their cap once and for all (the launch's own size decides
// occupancy), so launches from several host threads never see a smaller cap
// that another thread set for its own launch.
inline int smem_optin_bytes() {
  static int v = 0;
  if (!v) {
    int d = 0, x = 0;
    if (cudaGetDevice(&d) != cudaSuccess ||
        cudaDeviceGetAttribute(&x, cudaDevAttrMaxSharedMemoryPerBlockOptin, d) != cudaSuccess)
      return 48 * 1024;  // the launch that follows reports the error
    v = x;
  }
  return v;
}
// the largest dynamic shared memory a kernel may be given: the opt-in total
// less the kernel's static shared memory
template <typename K> inline int smem_cap(K kern) {
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, (const void *)kern) != cudaSuccess) return 48 * 1024;
  return smem_optin_bytes() - (int)fa.sharedSizeBytes;
}

// ---- launchers (each returns the number of kernels it launched) -------------

// Full-k coefficients and real-space periodic parts (K1 + K2):
//   cfull[(k*ncb + b)*ntg + ig] = rotated coefficients (make_C0),
//   ur[((k*ncb + b)*n3 + z)*n2*n1 + y*n1 + x] = float(bw FFT) (fft3_bw, unscaled).
// Which (k, band) real-space functions to make and where they go: bands (device
// list of nbands absolute bands; null = every band), slot_of (device table band
// -> slot, -1 = none; null = slot b with a stride of ncb bands), nslot (slots
// per k), rotate (apply make_C0 to coef_irr and write cfull; false: read cfull),
// fp32 (the transform's passes in FP32 instead of FP64; the rotation and cfull
// stay FP64).
struct WfnSlots {
  const int *bands = nullptr;
  int nbands = 0;
  const int *slot_of = nullptr;
  int nslot = 0;
  bool rotate = true;
  bool fp32 = false;
};
int launch_wfn_realspace(const double2 *coef_irr, const int *numirr, const int *trs, const int *src,
                         const double2 *phase, const int *ng0, const int *kg0, int ntk, int ncb, int ntg,
                         int n1, int n2, int n3, int R1, int R2, int R3, double2 *cfull, float2 *ur,
                         int k_begin, int k_end, cudaStream_t st, const WfnSlots &sl = WfnSlots());

// Pair densities rho(pair, k, g) = (1/N) DFT[conj(u_vir(k+q)) u_occ(k)] at -G-shift (K3).
struct PairChunks {
  const int *chunk_vir;    // absolute vir band of each chunk
  const int *chunk_first;  // first entry into pair_list
  const int *chunk_count;  // <= jmax
  const int *pair_list;    // pair indices (into the batch) grouped by vir band
  const int *pair_occ;     // absolute occ band of each pair
  int nchunk, jmax;
};
struct PairGeom {
  int ntk, ncb, n1, n2, n3, ng;
  const int *kpq, *shift, *lg0;  // device
  int R1, R2, R3;                // eps-sphere extent per dimension
  // real-space functions held in slots: (k, band) at k * nslot + slot_of[band]
  // (device table); null: every band resident at k * ncb + band
  const int *slot_of = nullptr;
  int nslot = 0;
};
// out64: rho[(pair*ntk + k)*ng + g] (double2, FP32-rounded values, plain path)
int launch_pair_density_fp64(const float2 *ur, const PairGeom &g, const PairChunks &c, double2 *out,
                             cudaStream_t st);
// shared memory of a pair-density CTA holding jmax pairs (callers size their chunks by it)
size_t pair_density_smem(const PairGeom &g, int jmax, bool fp64);
// FP32 path; writes the same layout in float2
int launch_pair_density_fp32(const float2 *ur, const PairGeom &g, const PairChunks &c, float2 *out,
                             cudaStream_t st);

// Gamma head: h[(pair*ntk + k)*3 + ix] = -i (i sum_G G conj(C_vir) C_occ)/del_eps  (calc_VMab)
int launch_gamma_head(const double2 *cfull, const int *ng0, const int *kg0, int ntk, int ncb, int ntg,
                      const double *bvec9, const double *energy, int ntb, const int *numirr,
                      const int *pair_vir, const int *pair_occ, int npair, double delt, double2 *head,
                      cudaStream_t st);

// Tetrahedron weights (K4): w[(pair*nen + e)*ntk + k] = xow(k,e) (1 - P_occ P_vir)/NTK.
struct TetraArgs {
  int ntk, nen, ntb;
  const int *imt1;        // 4*6*ntk mesh slots
  const int *index_kpt;   // [0,ntk): mesh slot -> k ; [ntk,2ntk): k -> mesh slot
  const int *numirr, *kpq;
  const double *energy;   // e_eigi [ik*ntb + ib]
  const double2 *prob;    // [k*ntb + ib]
  const double2 *em;
  const int *pair_vir, *pair_occ;
  int npair;
  double efermi, delt, dmna, dmnr;
  int *err;               // device error word
  // the FP32-series kernel: tetrahedra around each mesh slot (CSR: slot m owns
  // inc[inc_off[m] .. inc_off[m+1]), entries 4*tetrahedron + vertex position),
  // and whether any tetrahedron can be cut by the Fermi level (a partially
  // occupied band exists)
  const int *inc_off = nullptr, *inc = nullptr;
  int may_cut = 1;
};
// series = false: the reference's closed forms in FP64 for every tetrahedron
// (the plain FP64 path); true: the FP32 series wherever it converges, the
// closed forms in FP64 elsewhere (the split-precision paths)
int launch_tetra_weights(const TetraArgs &a, double2 *w, cudaStream_t st, bool series = false);
// Intraband plasma frequency at Gamma (ttrhdrn_simple + calc_VMaa): accumulates
// pwpl[3] (complex) for each band in bands[].
int launch_intraband(const TetraArgs &a, const double2 *cfull, const int *ng0, const int *kg0, int ncb,
                     int ntg, const double *bvec9, const double *sk0, const int *bands, int nb,
                     double2 *pwpl, cudaStream_t st);

// Plain FP64 contraction (K5): chi[(d*nen + e)*ng*ng + g + ng*g'] += sum_K w conj(rho_g) rho_g'
int launch_contract_fp64(const double2 *rho, const double2 *w, int npair, int ntk, int ng, int nen,
                         double2 *chi, cudaStream_t st);
// Gamma: rows/columns of G=0 for the head directions ix=1,2 (accumulating).
int launch_gamma_rowcol(const double2 *rho, const double2 *w, const double2 *head, int npair, int ntk,
                        int ng, int nen, int g0, double2 *rowcol /* [2][nen][2][ng] */, cudaStream_t st);
int launch_set_head(double2 *rho, const double2 *head, int npair, int ntk, int ng, int g0, int ix,
                    cudaStream_t st);

// eps build + inversion (K6)
struct EpsArgs {
  int ng, nen, ndir, gamma, g0;
  const double *qglen;    // device
  const double2 *em;      // device
  double wd[3], delt;
};
int launch_eps_build(const double2 *chi, const EpsArgs &a, double2 *A, cudaStream_t st);
// FP64 blocked Gauss-Jordan of the nmat matrices A (n x n, column-major, in
// place; the unscrambled inverse into out); prows holds
// gauss_jordan_scratch_bytes, piv and used n ints per matrix.
size_t gauss_jordan_scratch_bytes(int n, int nmat);
int launch_gauss_jordan(double2 *A, int n, int nmat, double2 *prows, int *piv, int *used, double2 *out, int *err,
                        cudaStream_t st);
// Mixed-precision inverse of the nmat matrices A (n x n, column-major): FP32
// Gauss-Jordan, a float-pair residual R = I - A X0 and one Newton step.
// rnorm[m] receives |R|_F^2 of matrix m (device); ws holds epsinv_mixed_bytes.
size_t epsinv_mixed_bytes(int n, int nmat);
int launch_epsinv_mixed(const double2 *A, int n, int nmat, void *ws, int *piv, int *used, double2 *out,
                        float *rnorm, int *err, cudaStream_t st);
int launch_scale(double2 *x, size_t n, double divisor, cudaStream_t st);  // x /= divisor

// band-tail correction (rp_tail.cu): X[(e*nshell + s)*9 + j] features of shell s
// at frequency e from the diagonal of chi (direction 0); sh[g] = shell of G (-1:
// none); stats = {lowest, mean excluded band energy above E_F, excluded/included}
int launch_tail_features(const double2 *chi, int ng, int nen, const int *sh, const double *qglen, int nshell,
                         const double2 *em, const float *stats, float *X, cudaStream_t st);
// chi(G,G,w) += Y[(e*nshell + sh[G])*2 + {0,1}] / tscale |q+G|^2 / (4 pi), every direction
int launch_tail_apply(double2 *chi, int ng, int nen, int ndir, const int *sh, const double *qglen, int nshell,
                      const float *Y, float tscale, cudaStream_t st);
// the network's forward pass on device inputs X (B x nin) on stream st; returns
// the device outputs (B x nout), valid until the network's next call
const float *mlp_forward_device(rp_mlp *m, const float *X, int B, cudaStream_t st);

}  // namespace rp
