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
//
// Two kernels: pair_density_kernel (FP64 arithmetic, the plain path: x pass,
// y pass, z term) and pair_slab_kernel (FP32, the fast path), which runs the y
// pass first with the lanes along x so that every thread streams its own
// column of the product straight from global memory and keeps two pairs and up
// to 16 output frequencies in registers.
#include "rp_dev.cuh"
#include "rp_host.h"

namespace rp {

__device__ __forceinline__ int modp2(int a, int n) { int m = a % n; return m < 0 ? m + n : m; }

struct PairArgs {
  int ntk, ncb, n1, n2, n3, ng, R1, R2;
  // resident real-space functions: (k, band) at slot (k * nslot + slot_of[band]),
  // or (k * ncb + band) when slot_of is null
  const int *slot_of;
  int nslot;
  const int *kpq, *shift, *lg0;
  const int *chunk_vir, *chunk_first, *chunk_count, *pair_list, *pair_occ;
  int jmax;
};

__device__ __forceinline__ size_t ur_slot(const PairArgs &a, int k, int band) {
  return a.slot_of ? (size_t)k * a.nslot + a.slot_of[band] : (size_t)k * a.ncb + band;
}

template <typename T> struct ToT2;
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
  const float2 *ui_g = ur + ur_slot(a, kq, vir) * (size_t)n12 * n3;
  for (int z = 0; z < n3; z++) {
    for (int i = tid; i < n12; i += nt) ui[i] = ToT2<T>::cvt(ui_g[(size_t)z * n12 + i]);
    __syncthreads();
    for (int jj = 0; jj < cnt; jj++) {
      const int occ = a.pair_occ[a.pair_list[first + jj]];
      const float2 *uj_g = ur + ur_slot(a, k, occ) * (size_t)n12 * n3 + (size_t)z * n12;
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

// ---------------------------------------------------------------------------
// FP32 path.  One CTA per (chunk of <= jmax pairs sharing a virtual band, k);
// the chunks of one k are consecutive in the grid, so the occupied bands of k
// stay in L2 while every virtual band is read from HBM once.  Per z slab:
//   pass 1 (y):  X[q][x][c2] = sum_y P_{2q}[x,y] TW2[y][c2], and the same for
//                pair 2q+1 in the other half of the float4.  Thread (pair, x)
//                loads conj(u_vir) and u_occ of its column from global memory
//                (32 lanes = 32 consecutive x: coalesced; u_vir shared in L1 by
//                the chunk's pairs) and keeps up to 16 frequencies in
//                registers; the twiddle rows are warp-uniform (broadcast)
//                16-byte loads.  One pair per thread keeps the registers low
//                enough for 18 warps per SM.
//   pass 2 (x):  Y[j][c2][c1] = sum_x X[j][x][c2] TW1[x][c1], thread
//                (pair, tile) with a tile = (c2, group of 4 c1) holding at
//                least one G of the sphere (about 30 of the 52 tiles of a
//                13x13 square).
//   z term:      acc[j][g] += Y[j][c2(g)][c1(g)] e^{-2 pi i f3(g) z / n3}.
// Y and acc hold the two pairs of a couple side by side (float4), so the z
// term moves both with one 16-byte access.
constexpr int PD_THREADS = 288;  // one pass-1 row (pair, x) per thread for 8 pairs on a 36-point line
constexpr int PD_CGMAX = 16;  // pass-1 output frequencies per register group, at most

// pass-1 register group for D2 output frequencies: an even count (the twiddles
// are read in 16-byte pairs) from a few compiled widths; above 14 frequencies
// the groups are 16 wide, so every group starts at a multiple of 4
__host__ __device__ inline int pd_group(int D2) {
  const int need = (D2 + 1) & ~1;
  return need <= 8 ? 8 : need <= 12 ? 12 : need <= 14 ? 14 : 16;
}

struct PdLayout {
  int D1, D2, D1P, D2P, D2X, SQ, nq, ntl;
  size_t oTW1, oTZ, oX, oY, oAcc, oSel, oF, oTile, total;
};

__host__ __device__ inline size_t pd_up16(size_t b) { return (b + 15) & ~(size_t)15; }

// Shared-memory carve-up of pair_slab_kernel (host and device agree on it).
//   TW2 [n2][D2P] float2, zero beyond D2 (direct y pass), or, split y pass:
//       [n2/4][D2P] twiddles e^{+2 pi i c b / n2} then the n2 phases e^{-2 pi i f0 y / n2}
//   TW1 [n1][D1P] float2, zero beyond D1, or, split x pass: [n1/4][D1P] then n1 phases
//   TZ  [2][n3]  float2 (z twiddles of the slab, double-buffered by slab parity)
//   X   [nq][SQ] float4: row x at x*D2X, column c2 -> (pair 2q, pair 2q+1)
//   Y   [nq][D2][D1] float4          acc [nq][ng] float4 (pair 2q, pair 2q+1)
//   sel [ng] int: c1 | c2 << 10 | f3 << 20          f1 [D1], f2 [D2] int
//   tile flags [ntl] and tile list [ntl + 1] int, ntl = (D1P / 4) D2, tile = grp D2 + c2
// D2X is odd and SQ = D2X (mod 8), so the 16-byte column stores of pass 1 and
// the (q, c2)-consecutive loads of pass 2 hit distinct bank quads.
__host__ __device__ inline PdLayout pd_layout(int n1, int n2, int n3, int R1, int R2, int ng, int jmax) {
  PdLayout L;
  L.D1 = 2 * R1 + 1 <= n1 ? 2 * R1 + 1 : n1;
  L.D2 = 2 * R2 + 1 <= n2 ? 2 * R2 + 1 : n2;
  const int cg = pd_group(L.D2);
  L.D2P = (L.D2 + cg - 1) / cg * cg;
  L.D1P = (L.D1 + 3) / 4 * 4;
  L.D2X = L.D2 | 1;
  L.nq = (jmax + 1) / 2;
  int sq = n1 * L.D2X;
  while ((sq - L.D2X) % 8) sq++;
  L.SQ = sq;
  size_t o = pd_up16(sizeof(float2) * (size_t)n2 * L.D2P);
  L.oTW1 = o; o += pd_up16(sizeof(float2) * (size_t)n1 * L.D1P);
  L.oTZ = o;  o += pd_up16(sizeof(float2) * 2 * (size_t)n3);
  L.oX = o;   o += sizeof(float4) * (size_t)L.nq * L.SQ;
  L.oY = o;   o += sizeof(float4) * (size_t)L.nq * L.D1 * L.D2;
  L.oAcc = o; o += sizeof(float4) * (size_t)L.nq * ng;
  L.oSel = o; o += pd_up16(sizeof(int) * (size_t)ng);
  L.oF = o;   o += pd_up16(sizeof(int) * (size_t)(L.D1 + L.D2));
  L.ntl = (L.D1P / 4) * L.D2;
  L.oTile = o; o += sizeof(int) * (2 * (size_t)L.ntl + 1);
  L.total = o;
  return L;
}

__device__ __forceinline__ float2 tw32(int j, int n) {
  float s, c;
  sincospif(-2.0f * j / n, &s, &c);
  return make_float2(c, s);
}
// L2 prefetch of a contiguous range (16-byte aligned, a multiple of 16 bytes)
__device__ __forceinline__ void l2_prefetch_bulk(const void *p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
// Q[r] = sum_a i^{r a} P[a], a, r = 0..3
__device__ __forceinline__ void bfly4(const float2 *P, float2 *Q) {
  const float2 t0 = make_float2(P[0].x + P[2].x, P[0].y + P[2].y);
  const float2 t1 = make_float2(P[0].x - P[2].x, P[0].y - P[2].y);
  const float2 t2 = make_float2(P[1].x + P[3].x, P[1].y + P[3].y);
  const float2 t3 = make_float2(P[1].x - P[3].x, P[1].y - P[3].y);
  Q[0] = make_float2(t0.x + t2.x, t0.y + t2.y);
  Q[2] = make_float2(t0.x - t2.x, t0.y - t2.y);
  Q[1] = make_float2(t1.x - t3.y, t1.y + t3.x);  // t1 + i t3
  Q[3] = make_float2(t1.x + t3.y, t1.y - t3.x);  // t1 - i t3
}
// conj(a) * b
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.x, b.y, -a.y * b.x));
}

// The y and x passes, direct (SPLIT false) or split (SPLIT true: n1 and n2
// multiples of 4, the sphere inside the box).  The split form writes
// y = s a + b (s = n2/4); the output frequencies of the register group are
// f0 - c (c = 0 .. D2-1), so
//   X[c] = sum_b e^{+2 pi i c b / n2} Q_b[c mod 4],
//   Q_b[r] = sum_a i^{r a} P[s a + b] e^{-2 pi i f0 (s a + b) / n2},
// a radix-4 butterfly of additions per b instead of four twiddle products per
// frequency: about 2.6 times fewer FP32 instructions than the direct sum.  The
// x pass is split the same way; its phase e^{-2 pi i f1_0 x / n1} is applied
// when pass 1 stores X.
template <int CG, bool SPLIT>
__global__ void __launch_bounds__(PD_THREADS, 2) pair_slab_kernel(const float2 *__restrict__ ur, PairArgs a,
                                                                   float2 *__restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ch = blockIdx.x, k = blockIdx.y, tid = threadIdx.x;
  const int n1 = a.n1, n2 = a.n2, n3 = a.n3, n12 = n1 * n2, ng = a.ng;
  const PdLayout L = pd_layout(n1, n2, n3, a.R1, a.R2, ng, a.jmax);
  const int D1 = L.D1, D2 = L.D2;
  const bool c1 = 2 * a.R1 + 1 <= n1, c2 = 2 * a.R2 + 1 <= n2;
  const int kq = a.kpq[k];
  const int s1 = a.shift[3 * k], s2 = a.shift[3 * k + 1], s3 = a.shift[3 * k + 2];
  const int vir = a.chunk_vir[ch], first = a.chunk_first[ch], cnt = a.chunk_count[ch];
  const int nq = (cnt + 1) / 2;
  float2 *TW2 = (float2 *)smem, *TW1 = (float2 *)(smem + L.oTW1), *TZ = (float2 *)(smem + L.oTZ);
  float4 *X = (float4 *)(smem + L.oX);
  float4 *Y = (float4 *)(smem + L.oY), *acc = (float4 *)(smem + L.oAcc);
  int *gsel = (int *)(smem + L.oSel), *f1 = (int *)(smem + L.oF), *f2 = f1 + D1;
  int *tflag = (int *)(smem + L.oTile), *tlist = tflag + L.ntl;  // tlist[0] = count
  for (int i = tid; i < L.ntl; i += PD_THREADS) tflag[i] = 0;
  for (int j = tid; j < D1; j += PD_THREADS) f1[j] = c1 ? modp2(-(j - a.R1) - s1, n1) : j;
  for (int j = tid; j < D2; j += PD_THREADS) f2[j] = c2 ? modp2(-(j - a.R2) - s2, n2) : j;
  __syncthreads();
  const int rows4 = n2 / 4;  // split y pass: rows per residue class
  float2 *PH = TW2 + (size_t)rows4 * L.D2P;
  if (SPLIT) {
    for (int i = tid; i < rows4 * L.D2P; i += PD_THREADS) {
      const int b = i / L.D2P, c = i % L.D2P;
      TW2[i] = c < D2 ? tw32((n2 - (c * b) % n2) % n2, n2) : make_float2(0.f, 0.f);
    }
    for (int y = tid; y < n2; y += PD_THREADS) PH[y] = tw32((f2[0] * y) % n2, n2);
  } else {
    for (int i = tid; i < n2 * L.D2P; i += PD_THREADS) {
      const int y = i / L.D2P, c = i % L.D2P;
      TW2[i] = c < D2 ? tw32((f2[c] * y) % n2, n2) : make_float2(0.f, 0.f);
    }
  }
  const int cols4 = n1 / 4;  // split x pass: columns per residue class
  float2 *PH1 = TW1 + (size_t)cols4 * L.D1P;
  if (SPLIT) {
    for (int i = tid; i < cols4 * L.D1P; i += PD_THREADS) {
      const int b = i / L.D1P, c = i % L.D1P;
      TW1[i] = c < D1 ? tw32((n1 - (c * b) % n1) % n1, n1) : make_float2(0.f, 0.f);
    }
    for (int x = tid; x < n1; x += PD_THREADS) PH1[x] = tw32((f1[0] * x) % n1, n1);
  } else {
    for (int i = tid; i < n1 * L.D1P; i += PD_THREADS) {
      const int x = i / L.D1P, c = i % L.D1P;
      TW1[i] = c < D1 ? tw32((f1[c] * x) % n1, n1) : make_float2(0.f, 0.f);
    }
  }
  for (int g = tid; g < ng; g += PD_THREADS) {
    const int *l = a.lg0 + 3 * g;
    const int i1 = c1 ? l[0] + a.R1 : modp2(-l[0] - s1, n1);
    const int i2 = c2 ? l[1] + a.R2 : modp2(-l[1] - s2, n2);
    const int i3 = modp2(-l[2] - s3, n3);
    gsel[g] = i1 | (i2 << 10) | (i3 << 20);
    tflag[(i1 >> 2) * D2 + i2] = 1;
  }
  for (int i = tid; i < nq * ng; i += PD_THREADS) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  __syncthreads();
  if (tid < 32) {  // compact the flagged tiles in (group, c2) order; read after pass 1's barrier
    int n = 0;
    for (int b = 0; b < L.ntl; b += 32) {
      const bool f = b + tid < L.ntl && tflag[b + tid];
      const unsigned m = __ballot_sync(0xffffffffu, f);
      if (f) tlist[1 + n + __popc(m & ((1u << tid) - 1u))] = b + tid;
      n += __popc(m);
    }
    if (tid == 0) tlist[0] = n;
  }
  const size_t bstride = (size_t)n12 * n3;
  const float2 *uvir = ur + ur_slot(a, kq, vir) * bstride;
  // the virtual band is read by this CTA alone, straight from HBM: its slab two
  // ahead is pulled into L2 by one bulk prefetch per slab (16-byte multiples)
  const bool pf = (n12 % 2) == 0;
  if (pf && tid == 0)
    for (int z = 0; z < min(2, n3); z++) l2_prefetch_bulk(uvir + (size_t)z * n12, (unsigned)(n12 * sizeof(float2)));
  for (int z = 0; z < n3; z++) {
    float2 *tz = TZ + (z & 1) * n3;
    for (int i = tid; i < n3; i += PD_THREADS) tz[i] = tw32((i * z) % n3, n3);
    if (pf && tid == 0 && z + 2 < n3) l2_prefetch_bulk(uvir + (size_t)(z + 2) * n12, (unsigned)(n12 * sizeof(float2)));
    // pass 1: row = (pair j1, column x1); one row per thread when cnt n1 <= PD_THREADS
    for (int row = tid; row < cnt * n1; row += PD_THREADS) {
      const int j1 = row / n1, x1 = row - j1 * n1;
      const float2 *pv = uvir + x1;
      const float2 *pa = ur + ur_slot(a, k, a.pair_occ[a.pair_list[first + j1]]) * bstride + x1;
      const size_t zo = (size_t)z * n12;
      for (int cg = 0; cg < D2; cg += CG) {
        float2 sa[CG];
#pragma unroll
        for (int c = 0; c < CG; c++) sa[c] = make_float2(0.f, 0.f);
        if (SPLIT) {
          // four rows (s a + b, a = 0..3) per step; the next step's rows in flight
          float2 nv[4], na[4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const size_t o = zo + (size_t)(u * rows4) * n1;
            nv[u] = __ldg(pv + o); na[u] = __ldg(pa + o);
          }
          for (int b = 0; b < rows4; b++) {
            float2 PA[4];
            const int bn = min(b + 1, rows4 - 1);
#pragma unroll
            for (int u = 0; u < 4; u++) {
              const float2 v = cmulc(nv[u], PH[u * rows4 + b]), va = na[u];
              const size_t o = zo + (size_t)(u * rows4 + bn) * n1;
              nv[u] = __ldg(pv + o); na[u] = __ldg(pa + o);
              PA[u] = cmul(v, va);
            }
            float2 QA[4];
            bfly4(PA, QA);
            const float4 *t = (const float4 *)(TW2 + (size_t)b * L.D2P + cg);
#pragma unroll
            for (int c = 0; c < CG / 2; c++) {
              const float4 w = t[c];
              cfma(sa[2 * c], QA[(2 * c) & 3], make_float2(w.x, w.y));
              cfma(sa[2 * c + 1], QA[(2 * c + 1) & 3], make_float2(w.z, w.w));
            }
          }
        } else {
          const float4 *twr = (const float4 *)(TW2 + cg);
          auto step = [&](float2 v, float2 va, int y) {
            const float2 PA = cmulc(v, va);
            const float4 *t = twr + (size_t)y * (L.D2P / 2);
#pragma unroll
            for (int c = 0; c < CG / 2; c++) {
              const float4 w = t[c];
              cfma(sa[2 * c], PA, make_float2(w.x, w.y));
              cfma(sa[2 * c + 1], PA, make_float2(w.z, w.w));
            }
          };
          // four rows in flight: each row's registers are refilled with the row
          // four ahead as soon as they are consumed (row index clamped to the
          // slab, so the loads need no guard)
          const int n2f = n2 & ~3;
          float2 nv[4], na[4];
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const size_t o = zo + (size_t)min(u, n2 - 1) * n1;
            nv[u] = __ldg(pv + o); na[u] = __ldg(pa + o);
          }
          for (int y0 = 0; y0 < n2f; y0 += 4) {
#pragma unroll
            for (int u = 0; u < 4; u++) {
              const float2 cv = nv[u], ca = na[u];
              const size_t o = zo + (size_t)min(y0 + 4 + u, n2 - 1) * n1;
              nv[u] = __ldg(pv + o); na[u] = __ldg(pa + o);
              step(cv, ca, y0 + u);
            }
          }
#pragma unroll
          for (int u = 0; u < 3; u++)
            if (n2f + u < n2) step(nv[u], na[u], n2f + u);
        }
        // this pair's half of the couple's float4 (pair 2q in .xy, 2q + 1 in .zw)
        float2 *xr = (float2 *)(X + (size_t)(j1 >> 1) * L.SQ + (size_t)x1 * L.D2X + cg) + (j1 & 1);
        const float2 ph1 = SPLIT ? PH1[x1] : make_float2(1.f, 0.f);
#pragma unroll
        for (int c = 0; c < CG; c++)
          if (cg + c < D2) xr[2 * c] = SPLIT ? cmul(sa[c], ph1) : sa[c];
      }
    }
    __syncthreads();
    // pass 2: item = (pair, tile); the pair's half of the couple's float4
    const int ntile = tlist[0];
    for (int it = tid; it < ntile * cnt; it += PD_THREADS) {
      const int j = it / ntile, t = tlist[1 + it - j * ntile], grp = t / D2, cc2 = t - grp * D2;
      float2 ya[4];
#pragma unroll
      for (int c = 0; c < 4; c++) ya[c] = make_float2(0.f, 0.f);
      const float2 *xc = (const float2 *)(X + (size_t)(j >> 1) * L.SQ + cc2) + (j & 1);
      if (SPLIT) {
        // x = s a + b; residue r of c1 = 4 grp + r is r
        for (int b = 0; b < cols4; b++) {
          float2 PA[4];
#pragma unroll
          for (int u = 0; u < 4; u++) PA[u] = xc[2 * (size_t)(u * cols4 + b) * L.D2X];
          float2 QA[4];
          bfly4(PA, QA);
          const float4 *tw = (const float4 *)(TW1 + (size_t)b * L.D1P + 4 * grp);
          const float4 t0 = tw[0], t1 = tw[1];
          cfma(ya[0], QA[0], make_float2(t0.x, t0.y));
          cfma(ya[1], QA[1], make_float2(t0.z, t0.w));
          cfma(ya[2], QA[2], make_float2(t1.x, t1.y));
          cfma(ya[3], QA[3], make_float2(t1.z, t1.w));
        }
      } else {
        const float4 *tw = (const float4 *)(TW1 + 4 * grp);
#pragma unroll 4
        for (int x = 0; x < n1; x++) {
          const float2 va = xc[2 * (size_t)x * L.D2X];
          const float4 t0 = tw[(size_t)x * (L.D1P / 2)], t1 = tw[(size_t)x * (L.D1P / 2) + 1];
          cfma(ya[0], va, make_float2(t0.x, t0.y));
          cfma(ya[1], va, make_float2(t0.z, t0.w));
          cfma(ya[2], va, make_float2(t1.x, t1.y));
          cfma(ya[3], va, make_float2(t1.z, t1.w));
        }
      }
      float2 *yq = (float2 *)(Y + (size_t)(j >> 1) * D1 * D2 + (size_t)cc2 * D1 + 4 * grp) + (j & 1);
#pragma unroll
      for (int c = 0; c < 4; c++)
        if (4 * grp + c < D1) yq[2 * c] = ya[c];
    }
    __syncthreads();
    // z term (overlaps the next slab's pass 1, which touches neither Y nor this tz)
    for (int g = tid; g < ng; g += PD_THREADS) {
      const int sel = gsel[g];
      const int yi = (sel & 1023) + D1 * ((sel >> 10) & 1023);
      const float2 t = tz[sel >> 20];
      for (int q = 0; q < nq; q++) {
        const float4 yv = Y[(size_t)q * D1 * D2 + yi];
        float4 &av = acc[(size_t)q * ng + g];
        float2 sA = make_float2(av.x, av.y), sB = make_float2(av.z, av.w);
        cfma(sA, make_float2(yv.x, yv.y), t);
        cfma(sB, make_float2(yv.z, yv.w), t);
        av = make_float4(sA.x, sA.y, sB.x, sB.y);
      }
    }
  }
  __syncthreads();
  const float inv = (float)(1.0 / ((double)n12 * n3));
  for (int jj = 0; jj < cnt; jj++) {
    const int p = a.pair_list[first + jj];
    float2 *dst = out + ((size_t)p * a.ntk + k) * ng;
    const float4 *src = acc + (size_t)(jj >> 1) * ng;
    for (int g = tid; g < ng; g += PD_THREADS) {
      const float4 v4 = src[g];
      const float2 v = (jj & 1) ? make_float2(v4.z, v4.w) : make_float2(v4.x, v4.y);
      dst[g] = make_float2(v.x * inv, v.y * inv);
    }
  }
}

size_t pair_density_smem(const PairGeom &g, int jmax, bool fp64) {
  if (!fp64) return pd_layout(g.n1, g.n2, g.n3, g.R1, g.R2, g.ng, jmax).total;
  const int D1 = 2 * g.R1 + 1 <= g.n1 ? 2 * g.R1 + 1 : g.n1, D2 = 2 * g.R2 + 1 <= g.n2 ? 2 * g.R2 + 1 : g.n2;
  const size_t elt = sizeof(double2);
  return elt * ((size_t)g.n1 * D1 + (size_t)g.n2 * D2 + g.n3 + 2 * (size_t)g.n1 * g.n2 + (size_t)D1 * g.n2 +
                (size_t)D1 * D2 + (size_t)jmax * g.ng) +
         sizeof(int) * ((size_t)D1 + D2 + g.ng);
}

static PairArgs pair_args(const PairGeom &g, const PairChunks &c) {
  PairArgs a;
  a.ntk = g.ntk; a.ncb = g.ncb; a.n1 = g.n1; a.n2 = g.n2; a.n3 = g.n3; a.ng = g.ng; a.R1 = g.R1; a.R2 = g.R2;
  a.slot_of = g.slot_of; a.nslot = g.nslot;
  a.kpq = g.kpq; a.shift = g.shift; a.lg0 = g.lg0;
  a.chunk_vir = c.chunk_vir; a.chunk_first = c.chunk_first; a.chunk_count = c.chunk_count;
  a.pair_list = c.pair_list; a.pair_occ = c.pair_occ; a.jmax = c.jmax;
  return a;
}

int launch_pair_density_fp64(const float2 *ur, const PairGeom &g, const PairChunks &c, double2 *out,
                             cudaStream_t st) {
  if (c.nchunk == 0) return 0;
  if (g.n1 > 1023 || g.n2 > 1023 || g.n3 > 1023) fail(1, "FFT box dimension above 1023");
  const size_t smem = pair_density_smem(g, c.jmax, true);
  if (smem > 227 * 1024) fail(1, "pair-density tile needs %zu bytes of shared memory", smem);
  RP_CUDA(cudaFuncSetAttribute(pair_density_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_cap(pair_density_kernel<double>)));
  dim3 grid(g.ntk, c.nchunk);
  pair_density_kernel<double><<<grid, 256, smem, st>>>(ur, pair_args(g, c), out);
  RP_CUDA(cudaGetLastError());
  return 1;
}

int launch_pair_density_fp32(const float2 *ur, const PairGeom &g, const PairChunks &c, float2 *out,
                             cudaStream_t st) {
  if (c.nchunk == 0) return 0;
  if (g.n1 > 1023 || g.n2 > 1023 || g.n3 > 1023) fail(1, "FFT box dimension above 1023");
  if (g.ntk > 65535) fail(1, "more than 65535 k points in one pair-density launch");
  const size_t smem = pair_density_smem(g, c.jmax, false);
  if (smem > 227 * 1024) fail(1, "pair-density tile needs %zu bytes of shared memory", smem);
  const bool inside = 2 * g.R2 + 1 <= g.n2;
  const int D2 = inside ? 2 * g.R2 + 1 : g.n2;
  // split y and x passes when both box lengths divide by 4 and the sphere fits in the box
  const bool split = inside && 2 * g.R1 + 1 <= g.n1 && g.n2 % 4 == 0 && g.n1 % 4 == 0;
  auto kern = split ? pair_slab_kernel<16, true> : pair_slab_kernel<16, false>;
  switch (pd_group(D2)) {
    case 8: kern = split ? pair_slab_kernel<8, true> : pair_slab_kernel<8, false>; break;
    case 12: kern = split ? pair_slab_kernel<12, true> : pair_slab_kernel<12, false>; break;
    case 14: kern = split ? pair_slab_kernel<14, true> : pair_slab_kernel<14, false>; break;
    default: break;
  }
  RP_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_cap(kern)));
  dim3 grid(c.nchunk, g.ntk);
  kern<<<grid, PD_THREADS, smem, st>>>(ur, pair_args(g, c), out);
  RP_CUDA(cudaGetLastError());
  return 1;
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
