// rp_tc.cu -- chi0 contraction on the 5th-generation tensor cores (tcgen05).
//
// Per frequency w the contraction of chiqw.F:1397-1410 is
//     chi_w = rho^H diag(x_w) rho,   x_w(K) = xow(k,w) (1 - P P)/NTK,  K = (pair, k).
// With Y the real matrix whose rows are Re rho(G) (rows 0..Gp) and Im rho(G)
// (rows Gp..2Gp), and M_x = Y diag(x) Y^T,
//     Re chi = Mr.rr + Mr.ii - Mi.ri + Mi.ir,   Im chi = Mi.rr + Mi.ii + Mr.ri - Mr.ir
// (Mr, Mi: x = Re / Im of the weight; rr, ri, ir, ii: quadrants of M).  M is
// symmetric, so only tiles on or above the diagonal are computed.
//
// Precision.  Every row of both operands gets a power-of-two scale from its
// largest value.  RP_PREC_FP16X2 splits a scaled value into two FP16 terms
// (products hi.hi + hi.lo + lo.hi, about 22 bits).  The three-term variants
// (RP_PREC_FP16X3, RP_PREC_BF16X3) make the leading term an integer of at most
// 8 bits (row scale maps the row maximum to 128) and carry the remainder in two
// 16-bit floating terms of the same row units, keeping the six products with
// plane(A) + plane(B) <= 2.  The tensor core's FP32 accumulator does not round
// to nearest, so the products of integer leading terms go to their own
// accumulator: their partial sums are integers of at most 2^24 over a
// sub-chunk of up to 1024 K; the five correction products, about 2^-7
// smaller, go to a second accumulator.  On single CTAs the
// accumulators are double-buffered in tensor memory: while the tensor core
// fills one pair for sub-chunk s + 1, the epilogue warps take sub-chunk s out
// of the other, unscale it (powers of two: exact) and add it with TwoSum into
// a float-pair copy of the tile in
// global memory (tile-blocked, rows contiguous, so a warp's 32 rows are one
// coalesced access), converted to FP64 once when chi is assembled.
//
// Kernel layout: one CTA of 704 threads per work item -- (problem, upper tile,
// frequency, Re/Im weight, K split) -- of a work list.  A q point is a group of
// one problem; a ragged batch (several q points of several cells) is one
// launch over all its problems.  Small problems split K across CTAs, each
// split into its own slice of the sums, added when chi is assembled.  Work
// items can also run as CTA pairs (tcgen05.mma.cta_group::2 on 2 x 2 tile
// blocks; see tc_gram_kernel).  The K split and the CTA shape of a problem
// shape are measured once and cached (tc_begin_q, tune_shape).
//   warps 0-15  producers (8 rows each): read the FP32 rows of the A operand (prefetched one K
//               block ahead in registers), multiply by the weights, split into
//               planes and store them into shared memory in the 128-byte-swizzled
//               K-major layout the tensor core reads;
//   warps 16-19 epilogue: drain the FP32 accumulators from tensor memory
//               (tcgen05.ld) into the float-pair tile in global memory (in a
//               CTA pair the producer warps help: drain_sub);
//   warp 20     allocates tensor memory and issues tcgen05.mma (one thread);
//   warp 21     loader (one thread): bulk-copies (cp.async.bulk) the B operand
//               planes -- split once per batch by bplanes_kernel and shared by
//               every channel -- and the block's weights into the stage.
// Two operand stages overlap loading, production and MMA.  Every mbarrier wait
// is bounded; on timeout the CTA raises the error word, waits (bounded) for its
// own MMAs and bulk copies and frees tensor memory before returning.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <vector>

#include "rp_dev.cuh"
#include "rp_host.h"
#include "rp_tc.h"

namespace rp {

namespace {

constexpr int BM = 128;          // tile rows (a) = TMEM lanes
constexpr int BN = 128;          // tile columns (b)
constexpr int BK = 64;           // K per stage (one 128-byte swizzle row of 16-bit values)
constexpr int NSTAGE = 2;        // operand stages
constexpr int TILE_BYTES = BM * BK * 2;  // 16 KB per operand plane tile
constexpr int NPROD = 512, NEPI = 128;    // 16 producer warps, 4 epilogue warps, MMA warp, loader warp
constexpr int PROWS = BM / (NPROD / 32); // A rows per producer warp
constexpr int MMA_WARP = (NPROD + NEPI) / 32;
constexpr int NTHREADS = NPROD + NEPI + 64;
constexpr int WCHUNK = 16;                 // K blocks per weight chunk
// accumulator columns of a CTA (a CTA pair: both column tiles of its 2 x 2
// block) and tensor-memory buffers of them (a pair: one, its two accumulators
// of 256 columns fill the 512)
__host__ __device__ constexpr int nb_of(bool pair) { return pair ? 2 * BN : BN; }
__host__ __device__ constexpr int nbuf_of(bool pair) { return pair ? 1 : 2; }
constexpr long WAIT_LIMIT = 1L << 28;    // polls before a wait gives up

// One problem of a (possibly ragged) group: a prepared pair batch of one q.
struct TcArgs {
  const float *Yt;        // [Mp][Kp] rows: Re rho (0..Gp), Im rho (Gp..2Gp)
  const float *sB;        // [Mp] row scales of the unweighted operand
  const float *sA;        // [2 nen][Mp] row scales of the weighted operand per channel
  const float2 *wt;       // [nen][Re/Im][Kp] weights as float pairs (hi, lo)
  // float-pair tiles, one slice per K split: [split][nen][2][ta][tb][col][row]
  // (128 x 128 per tile, ta <= tb); `slice` elements per split
  float2 *Macc;
  const unsigned char *Bp;  // B operand planes, [tb][kb][plane] tiles of TILE_BYTES
  size_t slice;
  int Mp, Kp, nen, ntile_side, ksub_blocks;
  int kb_split;           // K blocks per split (the last split takes the rest)
};

// A grouped launch: CTA i takes work item work[i] = (problem, ta | tb << 16,
// channel 2e + Re/Im, split).
struct TcGroup {
  const TcArgs *probs;
  const int4 *work;
  int *err;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *b, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t *b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// try_wait with cluster-scope acquire: for barriers the peer CTA of a pair arrives on
__device__ __forceinline__ bool mbar_try_cluster(uint64_t *b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
// the shared::cluster address of a local shared variable's copy in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t cluster_addr(const void *p, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}
__device__ __forceinline__ void mbar_arrive_remote(uint32_t cluster_bar) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_bar) : "memory");
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// The CTA's abort flag; in a CTA pair raising it also raises the peer's, so
// both halves of the pair leave their waits.
struct Abort {
  volatile int *flag;
  uint32_t peer;  // the peer's flag (shared::cluster address), 0 without a pair
  __device__ __forceinline__ bool up() const { return *flag != 0; }
  __device__ __forceinline__ void raise() const {
    *flag = 1;
    if (peer) asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(peer), "r"(1) : "memory");
  }
};

// bounded wait; returns false (and raises the abort flag) when it gives up
template <bool CLUSTER = false>
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, const Abort &ab) {
  for (long i = 0; i < WAIT_LIMIT; i++) {
    if (CLUSTER ? mbar_try_cluster(b, parity) : mbar_try(b, parity)) return true;
    if (ab.up()) return false;
    if (i > 64) __nanosleep(32);
  }
  ab.raise();
  return false;
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms of 1024 bytes
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);       // start address
  d |= (uint64_t)1 << 16;                         // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;               // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                         // descriptor version
  d |= (uint64_t)2 << 61;                         // SWIZZLE_128B
  return d;
}
// instruction descriptor of kind::f16: D f32, A/B f16 (0) or bf16 (1), both K-major
__host__ __device__ constexpr uint32_t make_idesc(int bf16, int M, int N) {
  return (1u << 4) | ((uint32_t)bf16 << 7) | ((uint32_t)bf16 << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// COLL: the A operand's collector buffer -- 0 not kept, 1 fill (read A, keep
// it), 2 use (the kept A, keep it), 3 last use (the kept A, release it).  The
// products that share an A plane run back to back, so that plane is read from
// shared memory once per K step instead of once per product.  CG: 1 one CTA
// (128 x N), 2 a CTA pair (256 x N: each CTA its 128 rows of A, N/2 rows of B
// and its 128 rows of D), issued by the pair's first CTA.
#define RP_MMA_F16(CGS, COLLS)                                                                    \
  asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"                                 \
               "tcgen05.mma.cta_group::" CGS ".kind::f16" COLLS " [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem), \
               "l"(ad), "l"(bd), "r"(idesc), "r"(accum))
template <int COLL, int CG>
__device__ __forceinline__ void mma_f16(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, int accum) {
  if (CG == 1) {
    if (COLL == 1) RP_MMA_F16("1", ".collector::a::fill");
    else if (COLL == 2) RP_MMA_F16("1", ".collector::a::use");
    else if (COLL == 3) RP_MMA_F16("1", ".collector::a::lastuse");
    else RP_MMA_F16("1", "");
  } else {
    if (COLL == 1) RP_MMA_F16("2", ".collector::a::fill");
    else if (COLL == 2) RP_MMA_F16("2", ".collector::a::use");
    else if (COLL == 3) RP_MMA_F16("2", ".collector::a::lastuse");
    else RP_MMA_F16("2", "");
  }
}
#undef RP_MMA_F16
// the collector mode of product pb of an A plane that has npb products
template <int PB, int NPB, int CG>
__device__ __forceinline__ void mma_plane(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, int accum) {
  if (NPB == 1) mma_f16<0, CG>(dtmem, ad, bd, idesc, accum);
  else if (PB == 0) mma_f16<1, CG>(dtmem, ad, bd, idesc, accum);
  else if (PB == NPB - 1) mma_f16<3, CG>(dtmem, ad, bd, idesc, accum);
  else mma_f16<2, CG>(dtmem, ad, bd, idesc, accum);
}
// arrive on barrier b when this thread's MMAs are done: in this CTA, or (CG 2)
// on the barrier at the same offset in both CTAs of the pair
template <int CG>
__device__ __forceinline__ void mma_commit(uint64_t *b) {
  if (CG == 1)
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(b))
                 : "memory");
  else
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
            smem_u32(b)),
        "h"((unsigned short)3)
        : "memory");
}


__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float *v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// power-of-two scale that maps |v| <= vmax below 2^top (m 2^e -> m 2^top)
__device__ __forceinline__ float scale_for(float vmax, int top) {
  if (!(vmax > 0.f)) return 1.f;
  int e;
  frexpf(vmax, &e);  // vmax = m 2^e, m in [0.5, 1)
  return ldexpf(1.f, top - e);
}

// byte offset of element (row, k) of a 128 x 64 16-bit tile in the 128B-swizzled K-major layout
__device__ __forceinline__ uint32_t swz(int row, int chunk16) {
  return (uint32_t)(row * 128 + ((chunk16 ^ (row & 7)) << 4));
}

// Split two values (each a float pair v + l, l joining after the leading term)
// into NP planes, packed two per 32-bit word.  Built from full-rate FP32
// operations; the only conversions are the packed cvt.rn.{f16,bf16}x2 stores:
//   integer leading plane: round to nearest even by adding and removing 1.5 * 2^23
//     (exact for |v| < 2^22);
//   16-bit planes: Veltkamp splitting (t = v (2^s + 1); h = t - (t - v)) rounds v
//     to the 11 (FP16) or 8 (BF16) significant bits the plane holds, so v - h is
//     exact; __fmul_rn / __fsub_rn keep the compiler from fusing the steps;
//   last plane: the remainder itself, rounded by the conversion.
template <bool BF16>
__device__ __forceinline__ float round_to_plane(float v) {
  const float t = __fmul_rn(v, BF16 ? 65537.0f : 8193.0f);
  return __fsub_rn(t, __fsub_rn(t, v));
}
template <bool BF16>
__device__ __forceinline__ uint32_t pack2(float a, float b) {
  if (BF16) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *(const uint32_t *)&h;
  }
  const __half2 h = __floats2half2_rn(a, b);
  return *(const uint32_t *)&h;
}
template <int NP, bool EXACT, bool BF16>
__device__ __forceinline__ void split2(float v0, float l0, float v1, float l1, uint32_t (&w)[NP]) {
  float r0 = v0, r1 = v1;
#pragma unroll
  for (int p = 0; p < NP; p++) {
    if (p == 1) { r0 = r0 + l0; r1 = r1 + l1; }
    float h0, h1;
    if (p == NP - 1) {
      h0 = r0; h1 = r1;
    } else if (p == 0 && EXACT) {
      const float M = 12582912.0f;  // 1.5 * 2^23
      h0 = __fsub_rn(__fadd_rn(r0, M), M);
      h1 = __fsub_rn(__fadd_rn(r1, M), M);
    } else {
      h0 = round_to_plane<BF16>(r0);
      h1 = round_to_plane<BF16>(r1);
    }
    w[p] = pack2<BF16>(h0, h1);
    if (p < NP - 1) { r0 = __fsub_rn(r0, h0); r1 = __fsub_rn(r1, h1); }
  }
}

// B operand planes of the batch, once for every channel: Bp[((tb*nkb + kb)*NP + p)*TILE_BYTES]
// holds rows tb*128.. of plane p for K block kb in the swizzled layout the
// tensor core reads (the same split as the A operand, without a weight).
template <int NP, bool EXACT, bool BF16>
__global__ void __launch_bounds__(256) bplanes_kernel(const float *__restrict__ Yt, const float *__restrict__ sB, int Kp,
                                                      int nkb, unsigned char *__restrict__ Bp) {
  const int tb = blockIdx.y, kb = blockIdx.x, tid = threadIdx.x;
  const int r = tid & (BM - 1), half = tid >> 7;
  const float s = sB[tb * BM + r];
  const float *y = Yt + (size_t)(tb * BM + r) * Kp + (size_t)kb * BK;
  unsigned char *dst = Bp + ((size_t)tb * nkb + kb) * NP * TILE_BYTES;
#pragma unroll 1
  for (int cc = 0; cc < 4; cc++) {
    const int c = 4 * half + cc;
    const float4 v0 = __ldg((const float4 *)(y + 8 * c)), v1 = __ldg((const float4 *)(y + 8 * c) + 1);
    const float bv[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
    uint32_t wb[NP][4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      uint32_t t[NP];
      split2<NP, EXACT, BF16>(bv[2 * j] * s, 0.f, bv[2 * j + 1] * s, 0.f, t);
#pragma unroll
      for (int p = 0; p < NP; p++) wb[p][j] = t[p];
    }
    const uint32_t off = swz(r, c);
#pragma unroll
    for (int p = 0; p < NP; p++)
      *(uint4 *)(dst + (size_t)p * TILE_BYTES + off) = make_uint4(wb[p][0], wb[p][1], wb[p][2], wb[p][3]);
  }
}

__device__ __forceinline__ void mbar_arrive_tx(uint64_t *b, uint32_t bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(b)),
               "r"(bytes)
               : "memory");
}
// L2 prefetch hints: a line for the producers' plain loads, a range for the loader's bulk copies
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
__device__ __forceinline__ void bulk_prefetch_l2(const void *p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
constexpr int PF_AHEAD = 4;  // K blocks between an L2 prefetch and its use

// bulk copy global -> shared, completion counted in bytes on mbarrier b
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(b))
               : "memory");
}

// A warp's view of the accumulator drain: its 32 rows of the float-pair tile(s)
// in global memory, the column scales, its row scale, its tensor-memory lanes.
struct DrainCtx {
  float2 *dst0;      // row rl of column 0 of the first tile; column c at (c / BN) BN BM + (c mod BN) BM
  const float *rB;   // 1 / column scales (NB)
  float ia;          // 1 / row scale
  uint32_t base;     // tensor memory: this warp's lane quarter, column 0
  uint64_t *accfull, *accempty;
  Abort ab;
};

// Drains sub-chunk sc: TMEM columns of buffer b hold [main][corr (exact
// scheme)] at b * NACC * NB.  The sub-chunk's sum (main exact, corr small) is
// unscaled by powers of two and added with an error-free TwoSum into (hi, lo)
// in global memory, so the running sum keeps about 48 bits with FP32
// arithmetic only.  Worker j of the W warps of a lane quarter takes the
// 8-column groups j, j + W, ...; the running sums of its next group are loaded
// while this one is added.
template <int NB, int NBUF, int NACC>
__device__ __forceinline__ bool drain_body(const DrainCtx &dc, int sc, int j, int W) {
  const int b = sc % NBUF;
  if (!mbar_wait(&dc.accfull[b], (sc / NBUF) & 1, dc.ab)) return false;
  tc_fence_after();
  auto dst_of = [&](int c) { return dc.dst0 + (size_t)(c / BN) * BN * BM + (size_t)(c % BN) * BM; };
  const uint32_t base = dc.base + (uint32_t)(b * NACC * NB);
  float2 g[8], gn[8] = {};
  if (8 * j < NB) {
#pragma unroll
    for (int jj = 0; jj < 8; jj++) g[jj] = dst_of(8 * j + jj)[0];
  }
#pragma unroll 1
  for (int c0 = 8 * j; c0 < NB; c0 += 8 * W) {
    if (c0 + 8 * W < NB) {
#pragma unroll
      for (int jj = 0; jj < 8; jj++) gn[jj] = dst_of(c0 + 8 * W + jj)[0];
    }
    float m[8], cr[8];
    tmem_ld8(base + c0, m);
    if (NACC == 2) tmem_ld8(base + NB + c0, cr);
    tmem_wait_ld();
#pragma unroll
    for (int jj = 0; jj < 8; jj++) {
      const float f = dc.ia * dc.rB[c0 + jj];
      const float x = m[jj] * f, l = (NACC == 2 ? cr[jj] : 0.f) * f;
      const float sm = g[jj].x + x, bb = sm - g[jj].x;
      const float err = (g[jj].x - (sm - bb)) + (x - bb);
      dst_of(c0 + jj)[0] = make_float2(sm, g[jj].y + err + l);
      g[jj] = gn[jj];
    }
  }
  tc_fence_before();
  mbar_arrive(&dc.accempty[b]);
  return true;
}
// out of line, for the producer warps that help drain in a CTA pair: they keep
// their registers for the production loop
template <int NB, int NBUF, int NACC>
__device__ __noinline__ bool drain_sub(const DrainCtx &dc, int sc, int j, int W) {
  return drain_body<NB, NBUF, NACC>(dc, sc, j, W);
}

// NP operand planes, EXACT integer leading plane, BF16 or FP16.  One CTA per
// work item (problem, upper tile, frequency, Re/Im weight, K split); see the
// file comment for the roles.
//
// PAIR: a cluster of two CTAs computes a 2 x 2 block of tiles, rows 2 tpa,
// 2 tpa + 1 and columns 2 tpb, 2 tpb + 1 (work items 2i, 2i + 1), with
// tcgen05.mma.cta_group::2 of 256 x 256: CTA r produces row tile 2 tpa + r of
// the weighted operand and bulk-copies column tile 2 tpb + r of B, and each
// CTA's tensor memory takes its row tile against both column tiles.  So a
// produced A plane and a loaded B plane each serve twice the products of a
// single CTA, and one thread issues the MMAs of both CTAs.  The two
// accumulators of 256 columns fill tensor memory, so the MMAs of a sub-chunk
// wait for the drain of the previous one.  The first CTA (rank 0)
// issues; its commits arrive on the barriers of both CTAs.  The second CTA's
// MMA warp relays to the first: lane 0 that a stage of its operands is ready
// (pready), lane 1 that its epilogue has drained the accumulators (paccempty).
template <int NP, bool EXACT, bool BF16, bool PAIR>
// 22 warps: at most 6 on one SM sub-partition, whose 16K registers allow 85 per thread
__global__ void __maxnreg__(80) tc_gram_kernel(TcGroup grp) {
  __shared__ TcArgs sh_args;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr int CG = PAIR ? 2 : 1;
  constexpr int NACC = EXACT ? 2 : 1;               // accumulators
  constexpr int NST = NSTAGE, WCH = WCHUNK, WB = WCH * BK * 8;
  constexpr int NB = nb_of(PAIR), NBUF = nbuf_of(PAIR);  // accumulator columns, buffers
  // warps that drain the accumulators: the epilogue warps, and in a CTA pair,
  // whose single-buffered MMAs wait for every drain, the producer warps too
  // (five warps per tensor-memory lane quarter)
  constexpr int DRAIN_THREADS = PAIR ? NEPI + NPROD : NEPI, DRAIN_W = DRAIN_THREADS / NEPI;
  constexpr int AOFF = 0, BOFF = NP * TILE_BYTES;
  constexpr int STAGE = 2 * NP * TILE_BYTES;        // A planes, B planes
  unsigned char *stage_base = smem;
  unsigned char *wring = smem + (size_t)NST * STAGE;  // two weight chunks
  uint64_t *bars = (uint64_t *)(wring + 2 * WB);
  // per stage: full (producers), bfull (loader), empty (MMAs done), pready (the
  // pair's second CTA ready, used in rank 0); per accumulator buffer: accfull,
  // accempty, paccempty (the second CTA's drain, rank 0); per weight chunk slot:
  // wready, wfree
  uint64_t *full = bars, *bfull = bars + 3, *empty = bars + 6, *pready = bars + 9, *accfull = bars + 12,
           *accempty = bars + 14, *paccempty = bars + 16, *wready = bars + 18, *wfree = bars + 20, *fin = bars + 22;
  volatile int *abort_word = (volatile int *)(bars + 23);
  uint32_t *tmem_slot = (uint32_t *)(bars + 24);
  float *sA_s = (float *)(bars + 32);               // row scales of this CTA's A rows (128)
  float *rB_s = sA_s + BM;                          // 1 / column scales of the accumulator columns (NB)

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t rank = PAIR ? cluster_rank() : 0;
  const Abort ab{abort_word, PAIR ? cluster_addr((const void *)abort_word, rank ^ 1u) : 0u};
  // the work list has channels fastest, so the CTAs running together share their operand rows in L2
  const int4 wk = grp.work[blockIdx.x];
  const TcArgs &a = sh_args;
  const int ta = wk.y & 0xffff, tb = wk.y >> 16;     // this CTA's row tile and B tile
  const int tb0 = PAIR ? (tb & ~1) : tb;               // the first column tile of the accumulators
  const int cidx = wk.z, e = cidx >> 1, ch = cidx & 1;  // frequency, channel (0 = Re weight, 1 = Im weight)
  {
    // empty K range (the host makes none): the whole CTA leaves, and so does
    // its peer, whose work item has the same K range
    const TcArgs &p = grp.probs[wk.x];
    if (wk.w * p.kb_split >= p.Kp / BK) return;
  }

  if (tid == 0) {
    sh_args = grp.probs[wk.x];
    for (int s = 0; s < NST; s++) {
      mbar_init(&full[s], NPROD);
      mbar_init(&bfull[s], 1);
      mbar_init(&empty[s], 1);
      mbar_init(&pready[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&accfull[b], 1);
      mbar_init(&accempty[b], DRAIN_THREADS);
      mbar_init(&paccempty[b], 1);
      mbar_init(&wready[b], 1);
      mbar_init(&wfree[b], NPROD);
    }
    mbar_init(fin, 1);
    *abort_word = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == MMA_WARP) {
    if (PAIR) {
      asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                   "r"(512));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    } else {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                   "r"(512));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
  }
  tc_fence_before();
  __syncthreads();
  // both CTAs of a pair: barriers initialised and tensor memory allocated before either uses the other's
  if (PAIR) cluster_sync();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  // this CTA's K range: blocks kb0 .. kb0 + nkb - 1 of the problem
  const int nkb_all = a.Kp / BK, kb0 = wk.w * a.kb_split;
  const int nkb = min(nkb_all - kb0, a.kb_split);
  const int ksub = a.ksub_blocks;
  const int nsub = (nkb + ksub - 1) / ksub;
  for (int i = tid; i < BM; i += NTHREADS) sA_s[i] = a.sA[(size_t)cidx * a.Mp + ta * BM + i];
  for (int i = tid; i < NB; i += NTHREADS) rB_s[i] = 1.0f / a.sB[tb0 * BN + i];  // exact: a power of two
  __syncthreads();

  // ---------------- draining a sub-chunk into the float-pair tile(s) ----------------
  // (drain_sub below; its state is fixed per warp)
  DrainCtx dc;
  {
    const int qd = warp & 3, rl = 32 * qd + lane;  // row within the tile
    const int nt = a.ntile_side;
    dc.dst0 = a.Macc + (size_t)wk.w * a.slice + (((((size_t)e * 2 + ch) * nt + ta) * nt + tb0) * BN) * BM + rl;
    dc.rB = rB_s;
    dc.ia = 1.0f / sA_s[rl];  // exact: a power of two
    dc.base = tmem + ((uint32_t)(32 * qd) << 16);
    dc.accfull = accfull;
    dc.accempty = accempty;
    dc.ab = ab;
  }
  auto drain = [&](int sc, int j, int W) { return drain_sub<NB, NBUF, NACC>(dc, sc, j, W); };
  auto drain_inline = [&](int sc, int j, int W) { return drain_body<NB, NBUF, NACC>(dc, sc, j, W); };

  if (warp < NPROD / 32) {
    // ---------------- producers: the weighted A operand ----------------
    // warp pw owns rows PROWS pw .. PROWS (pw + 1) - 1; lane l the K pair 2l, 2l+1 of every
    // block, so the global reads are coalesced (one 256-byte row per instruction),
    // the lane's two weights serve all the warp's rows, and each plane store writes one
    // full 128-byte swizzled row.
    const int pw = warp, r0 = PROWS * pw;
    const float2 *ya = (const float2 *)(a.Yt + (size_t)(ta * BM + r0) * a.Kp + (size_t)kb0 * BK) + lane;
    const size_t rstride = (size_t)a.Kp / 2;  // float2 per row
    float2 cur[PROWS], nxt[PROWS];
#pragma unroll
    for (int i = 0; i < PROWS; i++) cur[i] = __ldg(ya + i * rstride);
    const uint32_t cofs = (uint32_t)(lane & 3) * 4, chunk = (uint32_t)(lane >> 2);
    int drained = 0;  // sub-chunks this warp has helped drain (CTA pairs)
    bool ok = true;
    for (int kb = 0; kb < nkb; kb++) {
      const int s = kb % NST, use = kb / NST;
      // CTA pairs: before waiting for the stage of block kb, whose MMAs of block
      // kb - NST run only once every sub-chunk before that block's is drained,
      // help drain those (their MMAs have all been issued: their blocks are
      // produced)
      if (PAIR && kb >= NST) {
        const int target = (kb - NST) / ksub;
        for (; ok && drained < target; drained++) ok = drain(drained, 1 + warp / 4, DRAIN_W);
        if (!ok) break;
      }
      if (kb + 1 < nkb) {
#pragma unroll
        for (int i = 0; i < PROWS; i++) nxt[i] = __ldg(ya + i * rstride + (size_t)(kb + 1) * (BK / 2));
      }
      // DRAM -> L2 a few blocks ahead, one line per lane group: lanes 0 and 16 cover a row's 256 bytes
      if (kb + PF_AHEAD < nkb && (lane & 15) == 0) {
#pragma unroll
        for (int i = 0; i < PROWS; i++) prefetch_l2(ya + i * rstride + (size_t)(kb + PF_AHEAD) * (BK / 2));
      }
      const int wc = kb / WCH, kin = kb % WCH;
      if (kin == 0 && !mbar_wait(&wready[wc & 1], (wc >> 1) & 1, ab)) break;  // this chunk's weights
      if (use > 0 && !mbar_wait(&empty[s], (use - 1) & 1, ab)) break;
      unsigned char *st = stage_base + (size_t)s * STAGE;
      // (hi, lo) of K = 2 lane and 2 lane + 1
      const float4 wv = *(const float4 *)(wring + (size_t)(wc & 1) * WB + ((size_t)kin * BK + 2 * lane) * 8);
      const float x0h = wv.x, x0l = wv.y, x1h = wv.z, x1l = wv.w;
#pragma unroll
      for (int i = 0; i < PROWS; i++) {
        const int row = r0 + i;
        // (wh + wl) * y * s as a float pair: rounded head product plus its exact remainder
        const float sa = sA_s[r0 + i];
        const float xs0 = x0h * sa, xl0 = x0l * sa, xs1 = x1h * sa, xl1 = x1l * sa;
        const float zh0 = xs0 * cur[i].x, zl0 = fmaf(xl0, cur[i].x, fmaf(xs0, cur[i].x, -zh0));
        const float zh1 = xs1 * cur[i].y, zl1 = fmaf(xl1, cur[i].y, fmaf(xs1, cur[i].y, -zh1));
        uint32_t t[NP];
        split2<NP, EXACT, BF16>(zh0, zl0, zh1, zl1, t);
        const uint32_t off = (uint32_t)row * 128 + ((chunk ^ (uint32_t)(row & 7)) << 4) + cofs;
#pragma unroll
        for (int p = 0; p < NP; p++) *(uint32_t *)(st + AOFF + (size_t)p * TILE_BYTES + off) = t[p];
      }
      fence_proxy_async();
      mbar_arrive(&full[s]);
      if (kin == WCH - 1 || kb == nkb - 1) mbar_arrive(&wfree[wc & 1]);  // done with this chunk's weights
#pragma unroll
      for (int i = 0; i < PROWS; i++) cur[i] = nxt[i];
    }
    // the sub-chunks not drained inside the loop (at least the last)
    if (PAIR && ok)
      for (; drained < nsub; drained++)
        if (!drain(drained, 1 + warp / 4, DRAIN_W)) break;
  } else if (warp < MMA_WARP) {
    // ---------------- epilogue: every sub-chunk into the float-pair tile(s) ----------------
    for (int sc = 0; sc < nsub; sc++)
      if (!drain_inline(sc, 0, DRAIN_W)) break;
  } else if (warp == MMA_WARP) {
    if (PAIR && rank == 1) {
      // ---------------- the second CTA of a pair: relays to the issuer ----------------
      if (lane == 0) {
        const uint32_t rp0 = cluster_addr(&pready[0], 0);  // pready[s] is rp0 + 8 s
        for (int kb = 0; kb < nkb; kb++) {
          const int s = kb % NST, use = kb / NST;
          if (!mbar_wait(&bfull[s], use & 1, ab) || !mbar_wait(&full[s], use & 1, ab)) break;
          mbar_arrive_remote(rp0 + 8u * (uint32_t)s);
        }
      } else if (lane == 1) {
        const uint32_t ra0 = cluster_addr(&paccempty[0], 0);  // paccempty[b] is ra0 + 8 b
        // the issuer waits for the drains of sub-chunks 0 .. nsub - 1 - NBUF only
        for (int sc = 0; sc + NBUF < nsub; sc++) {
          const int b = sc % NBUF;
          if (!mbar_wait(&accempty[b], (sc / NBUF) & 1, ab)) break;
          mbar_arrive_remote(ra0 + 8u * (uint32_t)b);
        }
      }
    } else if (lane == 0) {
      // ---------------- MMA issuer ----------------
      const uint32_t idesc = make_idesc(BF16 ? 1 : 0, PAIR ? 2 * BM : BM, NB);
      // descriptors of every plane tile of stage 0, built once: per MMA the
      // issuing thread only adds the stage and the K step (32 bytes = 2 units of
      // the start address, which stays below 2^14 units), since it shares its
      // sub-partition with busy producer warps
      uint64_t dA[NP], dB[NP];
      const uint32_t sb0 = smem_u32(stage_base);
#pragma unroll
      for (int p = 0; p < NP; p++) {
        dA[p] = make_desc(sb0 + (uint32_t)(AOFF + p * TILE_BYTES));
        dB[p] = make_desc(sb0 + (uint32_t)(BOFF + p * TILE_BYTES));
      }
      // the MMAs of one K block in stage s: products of planes pa (A) and pb (B)
      // with pa + pb <= NP - 1, grouped by A plane (collector reuse); with the
      // exact scheme the leading product has its own accumulator.  The first
      // product into each accumulator of a sub-chunk overwrites it.
      auto issue = [&](int s, bool fresh_block, uint32_t tacc) {
        const uint64_t soff = (uint64_t)((uint32_t)s * (uint32_t)(STAGE >> 4));
#pragma unroll
        for (int kk = 0; kk < BK / 16; kk++) {
          const bool fresh = fresh_block && kk == 0;
          auto prod = [&](auto PA_, auto PB_) {
            constexpr int pa = decltype(PA_)::value, pb = decltype(PB_)::value;
            const uint64_t ad = dA[pa] + soff + (uint64_t)(2 * kk);
            const uint64_t bd = dB[pb] + soff + (uint64_t)(2 * kk);
            constexpr bool main_acc = (EXACT && pa == 0 && pb == 0) || !EXACT;
            constexpr bool first = main_acc ? (pa == 0 && pb == 0) : (pa == 0 && pb == 1);
            mma_plane<pb, NP - pa, CG>(main_acc ? tacc : tacc + NB, ad, bd, idesc, (first && fresh) ? 0 : 1);
          };
          prod(std::integral_constant<int, 0>{}, std::integral_constant<int, 0>{});
          prod(std::integral_constant<int, 0>{}, std::integral_constant<int, 1>{});
          if constexpr (NP == 3) prod(std::integral_constant<int, 0>{}, std::integral_constant<int, 2>{});
          prod(std::integral_constant<int, 1>{}, std::integral_constant<int, 0>{});
          if constexpr (NP == 3) {
            prod(std::integral_constant<int, 1>{}, std::integral_constant<int, 1>{});
            prod(std::integral_constant<int, 2>{}, std::integral_constant<int, 0>{});
          }
        }
      };
      for (int sc = 0; sc < nsub && !ab.up(); sc++) {
        // accumulator buffer b; the epilogues must have drained it (sub-chunk sc - NBUF)
        const int b = sc % NBUF;
        if (sc >= NBUF) {
          const uint32_t par = ((sc - NBUF) / NBUF) & 1;
          if (!mbar_wait(&accempty[b], par, ab)) break;
          if (PAIR && !mbar_wait<true>(&paccempty[b], par, ab)) break;
        }
        tc_fence_after();
        const uint32_t tacc = tmem + (uint32_t)(b * NACC * NB);
        const int kbeg = sc * ksub, kend = min(nkb, kbeg + ksub);
        bool ok = true;
        for (int kb = kbeg; kb < kend; kb++) {
          const int s = kb % NST, use = kb / NST;
          if (!mbar_wait(&bfull[s], use & 1, ab) || !mbar_wait(&full[s], use & 1, ab) ||
              (PAIR && !mbar_wait<true>(&pready[s], use & 1, ab))) {
            ok = false;
            break;
          }
          tc_fence_after();
          issue(s, kb == kbeg, tacc);
          mma_commit<CG>(&empty[s]);
        }
        if (!ok) break;
        mma_commit<CG>(&accfull[b]);
      }
      // wait for every MMA this thread issued before tensor memory is released
      mma_commit<CG>(fin);
      mbar_wait(fin, 0, ab);
    }
  } else if (lane == 0) {
    // ---------------- loader: B planes per K block, weights per chunk, by bulk copy ----------------
    const unsigned char *bsrc = a.Bp + ((size_t)tb * nkb_all + kb0) * NP * TILE_BYTES;
    const float2 *wsrc = a.wt + (size_t)cidx * a.Kp + (size_t)kb0 * BK;
    const int nchunk = (nkb + WCH - 1) / WCH;
    auto issue_w = [&](int c) {
      const uint32_t bytes = (uint32_t)min(WCH, nkb - c * WCH) * BK * 8;
      mbar_arrive_tx(&wready[c & 1], bytes);
      bulk_g2s(wring + (size_t)(c & 1) * WB, wsrc + (size_t)c * WCH * BK, bytes, &wready[c & 1]);
    };
    issue_w(0);
    if (nchunk > 1) issue_w(1);
    int wnext = 2, issued = 0;
    for (int kb = 0; kb < nkb; kb++) {
      const int s = kb % NST, use = kb / NST;
      if (use > 0 && !mbar_wait(&empty[s], (use - 1) & 1, ab)) break;
      unsigned char *st = stage_base + (size_t)s * STAGE;
      if (kb + PF_AHEAD < nkb) bulk_prefetch_l2(bsrc + (size_t)(kb + PF_AHEAD) * NP * TILE_BYTES, NP * TILE_BYTES);
      mbar_arrive_tx(&bfull[s], (uint32_t)(NP * TILE_BYTES));
#pragma unroll
      for (int p = 0; p < NP; p++)
        bulk_g2s(st + BOFF + p * TILE_BYTES, bsrc + ((size_t)kb * NP + p) * TILE_BYTES, TILE_BYTES, &bfull[s]);
      issued = kb + 1;
      // chunk wnext reuses the slot of chunk wnext - 2 once the producers have left it
      if (wnext < nchunk && kb >= (wnext - 1) * WCH) {
        if (!mbar_wait(&wfree[wnext & 1], ((wnext - 2) >> 1) & 1, ab)) break;
        issue_w(wnext);
        wnext++;
      }
    }
    // after an abort, wait (bounded) for the copies still in flight before the CTA exits
    if (ab.up()) {
      for (int kb = max(0, issued - NST); kb < issued; kb++)
        for (long i = 0; i < WAIT_LIMIT && !mbar_try(&bfull[kb % NST], (kb / NST) & 1); i++) __nanosleep(32);
      for (int c = max(0, wnext - 2); c < wnext; c++)
        for (long i = 0; i < WAIT_LIMIT && !mbar_try(&wready[c & 1], (c >> 1) & 1); i++) __nanosleep(32);
    }
  }
  __syncwarp();
  if (tid == 0 && ab.up()) atomicExch(grp.err, 4);
  tc_fence_before();
  __syncthreads();
  // a pair: the issuer's MMAs (which read both CTAs' shared memory and write
  // both CTAs' tensor memory) are complete before either CTA frees or leaves
  if (PAIR) cluster_sync();
  if (warp == MMA_WARP) {
    tc_fence_after();
    if (PAIR) asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
    else asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
  }
}

// ---------------------------------------------------------------------------
// helpers: transpose the batch's pair densities and weights into the GEMM's
// K-major operands, batch maxima, Gamma rows/columns, final assembly.

__device__ __forceinline__ void atomic_max_pos(float *addr, float v) {
  atomicMax((int *)addr, __float_as_int(v));  // valid for non-negative floats
}

// Yt[g][K] = Re rho, Yt[Gp+g][K] = Im rho, K = k*npair + p (rho is [p][k][g],
// float2 or, with FP64 pair densities, double2 rounded to float as chiqw_sub.F:201),
// and the rows' maxima over K (rowmax, zeroed beforehand).  A tiled transpose:
// a CTA reads 32 K x 64 g coalesced along g, keeps the tile in shared memory
// and writes 64 rows of 32 consecutive K (128-byte segments).
constexpr int YT_K = 32, YT_G = 64;
template <typename R>
__global__ void __launch_bounds__(256) yt_kernel(const R *__restrict__ rho, int npair, int ntk, int ng, int Gp, int Kp,
                                                 long Kn, float *__restrict__ Yt, const double2 *__restrict__ head,
                                                 int g0, float *__restrict__ rowmax) {
  __shared__ float2 tile[YT_G][YT_K + 1];
  const long K0 = (long)blockIdx.x * YT_K;
  const int gb = blockIdx.y * YT_G, tid = threadIdx.x;
  // load: thread (g = tid mod 64, K rows tid / 64, +4, ...)
  {
    const int gl = tid & (YT_G - 1), g = gb + gl;
    for (int kk = tid >> 6; kk < YT_K; kk += 256 / YT_G) {
      const long K = K0 + kk;
      float2 v = make_float2(0.f, 0.f);
      if (K < Kn && g < ng) {
        const int k = (int)(K / npair), p = (int)(K % npair);
        const R x = rho[((size_t)p * ntk + k) * ng + g];
        v = make_float2((float)x.x, (float)x.y);
        if (head && g == g0) {
          const double2 h = head[((size_t)p * ntk + k) * 3];
          v = make_float2((float)h.x, (float)h.y);
        }
      }
      tile[gl][kk] = v;
    }
  }
  __syncthreads();
  // store: a warp writes 32 consecutive K of one row (Re, then Im); lane 0 keeps the row's maxima
  const int kk = tid & (YT_K - 1);
  for (int gl = tid >> 5; gl < YT_G; gl += 256 / YT_K) {
    const int g = gb + gl;
    if (g >= ng) break;
    const long K = K0 + kk;
    const float2 v = tile[gl][kk];
    float mr = 0.f, mi = 0.f;
    if (K < Kn) {
      Yt[(size_t)g * Kp + K] = v.x;
      Yt[(size_t)(Gp + g) * Kp + K] = v.y;
      mr = fabsf(v.x);
      mi = fabsf(v.y);
    }
    for (int o = 16; o; o >>= 1) {
      mr = fmaxf(mr, __shfl_xor_sync(0xffffffffu, mr, o));
      mi = fmaxf(mi, __shfl_xor_sync(0xffffffffu, mi, o));
    }
    if (kk == 0) {
      atomic_max_pos(&rowmax[g], mr);
      atomic_max_pos(&rowmax[Gp + g], mi);
    }
  }
}

// wt[e][K] = w[(p*nen + e)*ntk + k] as float pairs: hi = float(v), lo = float(v - hi)
__global__ void wt_kernel(const double2 *__restrict__ w, int npair, int ntk, int nen, int Kp, float2 *__restrict__ wt) {
  const long K = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (K >= (long)npair * ntk) return;
  const int k = (int)(K / npair), p = (int)(K % npair);
  for (int e = 0; e < nen; e++) {
    double2 v = w[((size_t)p * nen + e) * ntk + k];
    const float rh = (float)v.x, ih = (float)v.y;
    wt[(size_t)(2 * e) * Kp + K] = make_float2(rh, (float)(v.x - (double)rh));
    wt[(size_t)(2 * e + 1) * Kp + K] = make_float2(ih, (float)(v.y - (double)ih));
  }
}


// per-channel maxima of the weights (hi words) over the batch's K: out[1 + c]
__global__ void maxes_kernel(const float2 *__restrict__ wt, int nen, int Kp, long Kn, float *__restrict__ out) {
  for (int e = 0; e < nen; e++) {
    float mr = 0.f, mi = 0.f;
    for (long K = (long)blockIdx.x * blockDim.x + threadIdx.x; K < Kn; K += (long)gridDim.x * blockDim.x) {
      mr = fmaxf(mr, fabsf(wt[(size_t)(2 * e) * Kp + K].x));
      mi = fmaxf(mi, fabsf(wt[(size_t)(2 * e + 1) * Kp + K].x));
    }
    for (int o = 16; o; o >>= 1) {
      mr = fmaxf(mr, __shfl_xor_sync(0xffffffffu, mr, o));
      mi = fmaxf(mi, __shfl_xor_sync(0xffffffffu, mi, o));
    }
    if ((threadIdx.x & 31) == 0) { atomic_max_pos(&out[1 + 2 * e], mr); atomic_max_pos(&out[2 + 2 * e], mi); }
  }
}

// row scales: B rows from the row maximum, A rows from row maximum x channel maximum
__global__ void scales_kernel(const float *__restrict__ rowmax, const float *__restrict__ maxes, int Mp, int nen,
                              int top, float *__restrict__ sB, float *__restrict__ sA) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= Mp) return;
  sB[a] = scale_for(rowmax[a], top);
  for (int c = 0; c < 2 * nen; c++) sA[(size_t)c * Mp + a] = scale_for(rowmax[a] * maxes[1 + c], top);
}

// Gamma, directions 2 and 3: G=0 row and column in FP64 from the FP32 densities
__global__ void gamma_rowcol_f32_kernel(const float2 *__restrict__ rho, const double2 *__restrict__ w,
                                        const double2 *__restrict__ head, int npair, int ntk, int ng, int nen, int g0,
                                        double2 *__restrict__ rowcol) {
  const int g = blockIdx.x, e = blockIdx.y, ix = blockIdx.z + 1;
  const long K = (long)npair * ntk;
  double2 r = make_double2(0, 0), c = make_double2(0, 0);
  for (long Kx = threadIdx.x; Kx < K; Kx += blockDim.x) {
    const int p = (int)(Kx / ntk), k = (int)(Kx % ntk);
    const double2 ww = w[((size_t)p * nen + e) * ntk + k];
    const double2 h = head[(size_t)Kx * 3 + ix];
    double2 v;
    if (g == g0) v = h;
    else { float2 f = rho[(size_t)Kx * ng + g]; v = make_double2(f.x, f.y); }
    cfma(r, cmul(ww, cconj(h)), v);
    cfma(c, cmul(ww, cconj(v)), h);
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

// element (i, j) of a symmetric matrix stored in its upper tiles (tile-blocked,
// rows contiguous) as float pairs, summed over the K-split slices
__device__ __forceinline__ double mget(const float2 *M, size_t slice, int nslice, int nt, int i, int j) {
  if (i / BM > j / BN) { const int t = i; i = j; j = t; }
  const size_t o = (((size_t)(i / BM) * nt + j / BN) * BN + (j % BN)) * BM + (i % BM);
  double v = 0;
  for (int s = 0; s < nslice; s++) {
    const float2 x = M[s * slice + o];
    v += (double)x.x + (double)x.y;
  }
  return v;
}

// chi[e][g + ng h] += (Mr.rr + Mr.ii - Mi.ri + Mi.ir) + i (Mi.rr + Mi.ii + Mr.ri - Mr.ir)
__global__ void assemble_kernel(const float2 *__restrict__ Macc, size_t slice, int nslice, int Mp, int Gp, int ng,
                                double2 *__restrict__ chi) {
  const int e = blockIdx.y;
  const float2 *Mr = Macc + ((size_t)e * 2 + 0) * Mp * Mp, *Mi = Macc + ((size_t)e * 2 + 1) * Mp * Mp;
  const int nt = Mp / BM;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < (size_t)ng * ng;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int g = (int)(idx % ng), h = (int)(idx / ng);
    const double rr_r = mget(Mr, slice, nslice, nt, g, h), ii_r = mget(Mr, slice, nslice, nt, Gp + g, Gp + h);
    const double ri_r = mget(Mr, slice, nslice, nt, g, Gp + h), ir_r = mget(Mr, slice, nslice, nt, Gp + g, h);
    const double rr_i = mget(Mi, slice, nslice, nt, g, h), ii_i = mget(Mi, slice, nslice, nt, Gp + g, Gp + h);
    const double ri_i = mget(Mi, slice, nslice, nt, g, Gp + h), ir_i = mget(Mi, slice, nslice, nt, Gp + g, h);
    double2 *d = chi + (size_t)e * ng * ng + idx;
    d->x += rr_r + ii_r - ri_i + ir_i;
    d->y += rr_i + ii_i + ri_r - ir_r;
  }
}

}  // namespace

void TcWorkspace::release() {
  if (planes) cudaFree(planes);
  if (part) cudaFree(part);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  planes = part = nullptr;
  ev0 = ev1 = nullptr;
  planes_bytes = part_bytes = 0;
}

static void *grow(void *&p, size_t &have, size_t need) {
  if (need <= have) return p;
  if (p) cudaFree(p);
  p = nullptr;
  have = 0;
  RP_CUDA(cudaMalloc(&p, need));
  have = need;
  return p;
}


static int Gp_of(int ng) { return ((ng + BM - 1) / BM) * BM; }
static int nplanes_of(int precision) { return (precision == RP_PREC_BF16X3 || precision == RP_PREC_FP16X3) ? 3 : 2; }
static size_t smem_of(int precision, bool pair) {
  // per stage: A planes, B planes; the weight ring; then the barriers and the
  // row and column scales
  const size_t np = (size_t)nplanes_of(precision);
  return 1024 + (size_t)NSTAGE * np * 2 * TILE_BYTES + 2 * (size_t)WCHUNK * BK * 8 + 256 +
         sizeof(float) * (BM + (size_t)nb_of(pair));
}
static size_t slice_of(int Mp, int nen) { return (size_t)nen * 2 * Mp * Mp; }
// K blocks per FP32 sub-chunk: 1024 K by default, and at most that for the
// 8-bit integer leading plane (its partial sums stay integers of at most
// 2^24).  The tensor core's FP32 accumulation also loses accuracy in
// proportion to the length of a sum (chi against the FP64 oracle, FP16x3 with
// a 7-bit leading plane: 2.4e-7 at 256 K, 8.3e-7 at 1024 K, 3.4e-6 at 4096 K),
// so longer sub-chunks would not pay even where the integers allowed them; a
// CTA pair takes the same length.
static int ksub_of(const TcWorkspace &ws, bool pair = false) {
  (void)pair;
  const int k = ws.ksub > 0 ? ws.ksub : 16;
  return nplanes_of(ws.precision) == 3 ? std::min(k, 16) : k;
}

// ---------------------------------------------------------------------------
// Launch-shape tuner.  A q point whose upper tiles x channels give fewer than
// two CTAs per SM leaves SMs idle; splitting K across CTAs (each split into
// its own float-pair slice, summed when chi is assembled) fills them at the
// cost of more sums to drain.  CTA pairs (cta_group::2) read less shared
// memory per product but compute the row tiles below the diagonal that pair
// with the diagonal ones.  The best (split, pair) of a shape (precision, Mp,
// nen, K order of magnitude) is measured once on the first batch of that shape
// and cached for the process.

namespace {
constexpr int SPLIT_MAX = 16;
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, std::pair<int, int>> g_tuned;  // -> (split, pair)

int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    RP_CUDA(cudaGetDevice(&dev));
    RP_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  }
  return n;
}
int kbits(long nkb) {
  int b = 0;
  while ((2L << b) <= nkb) b++;
  return b;
}
// K blocks per split for `split` splits of nkb blocks: whole sub-chunks
int kb_split_of(int nkb, int split, int ksub) {
  int per = (nkb + split - 1) / split;
  per = ((per + ksub - 1) / ksub) * ksub;
  return std::max(per, 1);
}
}  // namespace

int tc_tuned_shapes() {
  std::lock_guard<std::mutex> g(g_tune_mu);
  return (int)g_tuned.size();
}
void tc_reset_tuner() {
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tuned.clear();
}

void tc_begin_q(TcWorkspace &ws, int ng, int nen, int ndir, int split_req, long k_estimate, int precision,
                cudaStream_t st) {
  ws.ng = ng; ws.nen = nen; ws.ndir = ndir;
  ws.gram_seconds = 0;
  ws.ready = 0;
  if (!ws.ev0) { RP_CUDA(cudaEventCreate(&ws.ev0)); RP_CUDA(cudaEventCreate(&ws.ev1)); }
  const int Mp = 2 * Gp_of(ng), nt = Mp / BM;
  const long nkb = std::max(1L, (k_estimate + BK - 1) / BK);
  const long ctas = (long)nt * (nt + 1) / 2 * 2 * nen;
  ws.tune_pending = 0;
  ws.tune_split = ws.tune_pair = 0;
  ws.precision = precision;
  const bool split_fixed = split_req > 0 || ctas >= 2L * num_sms() || nkb < 2L * ksub_of(ws);
  const bool pair_fixed = ws.pair_req != 0;
  ws.nsplit = split_req > 0 ? std::min(split_req, SPLIT_MAX) : 1;
  ws.pair = ws.pair_req == 2 ? 1 : 0;
  if (!split_fixed || !pair_fixed) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tuned.find(std::make_tuple(precision, Mp, nen, kbits(nkb)));
    if (it != g_tuned.end()) {
      if (!split_fixed) ws.nsplit = it->second.first;
      if (!pair_fixed) ws.pair = it->second.second;
    } else {
      ws.tune_pending = 1;
      ws.tune_split = split_fixed ? 0 : 1;
      ws.tune_pair = pair_fixed ? 0 : 1;
    }
  }
  ws.nslice = ws.tune_pending && ws.tune_split ? SPLIT_MAX : ws.nsplit;
  const size_t mbytes = sizeof(float2) * slice_of(Mp, nen) * ws.nslice;
  grow(ws.part, ws.part_bytes, mbytes);
  RP_CUDA(cudaMemsetAsync(ws.part, 0, mbytes, st));
  ws.precision = precision;
  ws.Mp = Mp;
  ws.Kp = (int)(nkb * BK);  // the tuner's key until a batch is prepared
}

// ---------------------------------------------------------------------------
// grouped launch

namespace {
struct GroupScratch {
  void *dev = nullptr;
  size_t bytes = 0;
  ~GroupScratch() {
    if (dev) cudaFree(dev);
  }
};
thread_local GroupScratch g_scratch;

// The problem table and the work list of a group, uploaded to `dev`.
struct GroupPlan {
  const TcArgs *probs = nullptr;
  const int4 *work = nullptr;
  int nwork = 0, precision = 0, pair = 0;
  size_t smem = 0;
};

bool pairs_available(int precision);

GroupPlan plan_group(TcWorkspace *const *wss, int n, cudaStream_t st, void *&dev, size_t &have) {
  GroupPlan P;
  if (n <= 0) return P;
  P.precision = wss[0]->precision;
  // CTA pairs when every problem of the group takes them
  P.pair = 1;
  for (int i = 0; i < n; i++) P.pair &= wss[i]->pair ? 1 : 0;
  std::vector<TcArgs> probs(n);
  // larger problems first, so the short ones fill the tail of the launch
  std::vector<int> order(n);
  std::vector<double> cost(n);
  for (int i = 0; i < n; i++) {
    const TcWorkspace &ws = *wss[i];
    if (!ws.ready) fail(1, "tensor-core group: problem %d has no prepared batch", i);
    if (ws.precision != P.precision) fail(1, "tensor-core group: mixed precisions");
    const int nt = ws.Mp / BM;
    cost[i] = (double)nt * (nt + 1) / 2 * ws.nen * ((double)ws.Kp / BK);
    order[i] = i;
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  std::vector<int4> work;
  for (int oi = 0; oi < n; oi++) {
    const int i = order[oi];
    const TcWorkspace &ws = *wss[i];
    TcArgs &a = probs[i];
    const int nt = ws.Mp / BM, nkb = ws.Kp / BK;
    const int ksub = ksub_of(ws, P.pair);
    a.Yt = ws.Yt; a.sB = ws.sB; a.sA = ws.sA; a.wt = ws.wt; a.Bp = ws.Bp;
    a.Macc = (float2 *)ws.part;
    a.slice = slice_of(ws.Mp, ws.nen);
    a.Mp = ws.Mp; a.Kp = ws.Kp; a.nen = ws.nen; a.ntile_side = nt; a.ksub_blocks = ksub;
    a.kb_split = kb_split_of(nkb, std::min(ws.nsplit, ws.nslice), ksub);
    const int nsp = (nkb + a.kb_split - 1) / a.kb_split;
    if (nsp > ws.nslice) fail(1, "tensor-core group: %d K splits for %d slices", nsp, ws.nslice);
    if (P.pair) {
      // 2 x 2 blocks (tpa, tpb >= tpa) of tiles, the pair's two CTAs adjacent
      // (nt is even: Mp = 2 Gp): CTA r takes row tile 2 tpa + r and loads
      // column tile 2 tpb + r; tile (2 tpa + 1, 2 tpa) of a diagonal block is
      // below the diagonal and never read
      for (int tpa = 0; tpa < nt / 2; tpa++)
        for (int tpb = tpa; tpb < nt / 2; tpb++)
          for (int sp = 0; sp < nsp; sp++)
            for (int c = 0; c < 2 * ws.nen; c++)
              for (int r = 0; r < 2; r++)
                work.push_back(make_int4(i, (2 * tpa + r) | ((2 * tpb + r) << 16), c, sp));
    } else {
      for (int ta = 0; ta < nt; ta++)
        for (int tb = ta; tb < nt; tb++)
          for (int sp = 0; sp < nsp; sp++)
            for (int c = 0; c < 2 * ws.nen; c++) work.push_back(make_int4(i, ta | (tb << 16), c, sp));
    }
  }
  if (work.size() > 0x7fffffffu) fail(1, "tensor-core group: too many work items");
  const size_t pbytes = ((sizeof(TcArgs) * n + 255) / 256) * 256, wbytes = sizeof(int4) * work.size();
  grow(dev, have, pbytes + wbytes);
  RP_CUDA(cudaMemcpyAsync(dev, probs.data(), sizeof(TcArgs) * n, cudaMemcpyHostToDevice, st));
  RP_CUDA(cudaMemcpyAsync((unsigned char *)dev + pbytes, work.data(), wbytes, cudaMemcpyHostToDevice, st));
  note_transfer((long long)(sizeof(TcArgs) * n + wbytes), 0);
  P.probs = (const TcArgs *)dev;
  P.work = (const int4 *)((unsigned char *)dev + pbytes);
  P.nwork = (int)work.size();
  P.smem = smem_of(P.precision, P.pair);
  if (P.smem > 227 * 1024) fail(1, "tensor-core stage layout needs %zu bytes", P.smem);
  if (P.pair && !pairs_available(P.precision))
    fail(1, "tensor-core CTA pairs requested (tc_pair=2) but the device holds no cluster of two %zu-byte CTAs",
         P.smem);
  if (P.pair && P.nwork % 2) fail(1, "tensor-core group: odd work list for CTA pairs");
  return P;
}

void (*kernel_of(int precision, bool pair))(TcGroup) {
  if (pair) {
    if (precision == RP_PREC_FP16X3) return tc_gram_kernel<3, true, false, true>;
    if (precision == RP_PREC_BF16X3) return tc_gram_kernel<3, true, true, true>;
    return tc_gram_kernel<2, false, false, true>;
  }
  if (precision == RP_PREC_FP16X3) return tc_gram_kernel<3, true, false, false>;
  if (precision == RP_PREC_BF16X3) return tc_gram_kernel<3, true, true, false>;
  return tc_gram_kernel<2, false, false, false>;
}

int launch_group(const GroupPlan &P, int *err, cudaStream_t st) {
  if (P.nwork == 0) return 0;
  void (*kern)(TcGroup) = kernel_of(P.precision, P.pair);
  TcGroup g{P.probs, P.work, err};
  if (P.pair) {
    // clusters of two adjacent CTAs: work items 2i and 2i + 1
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)P.nwork);
    cfg.blockDim = dim3(NTHREADS);
    cfg.dynamicSmemBytes = P.smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    RP_CUDA(cudaLaunchKernelEx(&cfg, kern, g));
  } else {
    kern<<<(unsigned)P.nwork, NTHREADS, P.smem, st>>>(g);
  }
  RP_CUDA(cudaGetLastError());
  return 1;
}

// clusters of the CTA-pair kernel of each precision the device can hold at once
// (0: CTA pairs unavailable), set by set_kernel_smem
thread_local int g_pair_clusters[4] = {-1, -1, -1, -1};

void set_kernel_smem(int precision) {
  const int idx = precision & 3;
  if (g_pair_clusters[idx] >= 0) return;
  for (int pair = 0; pair < 2; pair++) {
    RP_CUDA(cudaFuncSetAttribute(kernel_of(precision, pair), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem_cap(kernel_of(precision, pair))));
    RP_CUDA(cudaFuncSetAttribute(kernel_of(precision, pair), cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared));
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2 * (unsigned)num_sms());
  cfg.blockDim = dim3(NTHREADS);
  cfg.dynamicSmemBytes = smem_of(precision, true);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, kernel_of(precision, true), &cfg) != cudaSuccess) {
    cudaGetLastError();  // not a sticky error: the pairs are just not offered
    n = 0;
  }
  g_pair_clusters[idx] = n;
}

bool pairs_available(int precision) {
  set_kernel_smem(precision);
  return g_pair_clusters[precision & 3] > 0;
}

// times every candidate (split, pair) of the prepared batch, keeps the fastest
void tune_shape(TcWorkspace &ws, int *err, cudaStream_t st) {
  const int nkb = ws.Kp / BK, ksub = ksub_of(ws);
  std::vector<int> splits;
  if (ws.tune_split) {
    int last_nsp = 0;
    for (int s = 1; s <= SPLIT_MAX; s *= 2) {
      const int kbs = kb_split_of(nkb, s, ksub), nsp = (nkb + kbs - 1) / kbs;
      if (nsp != last_nsp && nsp <= ws.nslice) splits.push_back(s);
      last_nsp = nsp;
    }
  } else {
    splits.push_back(ws.nsplit);
  }
  std::vector<int> pairs;
  if (ws.tune_pair && pairs_available(ws.precision)) pairs = {0, 1};
  else pairs.push_back(ws.tune_pair ? 0 : ws.pair);
  TcWorkspace *one = &ws;
  int best_s = splits[0], best_p = pairs[0];
  float best_ms = 1e30f;
  for (int rep = 0; rep < 2; rep++)  // the first pass warms up
    for (int p : pairs)
      for (int s : splits) {
        ws.nsplit = s;
        ws.pair = p;
        GroupPlan P = plan_group(&one, 1, st, g_scratch.dev, g_scratch.bytes);
        RP_CUDA(cudaEventRecord(ws.ev0, st));
        launch_group(P, err, st);
        RP_CUDA(cudaEventRecord(ws.ev1, st));
        RP_CUDA(cudaEventSynchronize(ws.ev1));
        float ms = 0;
        RP_CUDA(cudaEventElapsedTime(&ms, ws.ev0, ws.ev1));
        if (rep == 1 && ms < best_ms) { best_ms = ms; best_s = s; best_p = p; }
      }
  ws.nsplit = best_s;
  ws.pair = best_p;
  ws.tune_pending = 0;
  // the candidates' sums are discarded
  RP_CUDA(cudaMemsetAsync(ws.part, 0, sizeof(float2) * slice_of(ws.Mp, ws.nen) * ws.nslice, st));
}
}  // namespace

int tc_prepare(TcWorkspace &ws, const float2 *rho, const double2 *rho64, const double2 *w, const double2 *head,
               int npair, int ntk, int ng, int nen, int g0, int precision, double2 *rowcol, int *err,
               cudaStream_t st) {
  ws.ready = 0;
  if (npair == 0) return 0;
  if (ng != ws.ng || nen != ws.nen) fail(1, "tc_prepare: workspace begun for another q");
  int launches = 0;
  const int Gp = Gp_of(ng), Mp = 2 * Gp;
  const long Kn = (long)npair * ntk;
  const int Kp = (int)(((Kn + BK - 1) / BK) * BK);
  const int nplanes = nplanes_of(precision);
  // workspace: Yt [Mp][Kp] float, wt [nen][Kp] float4, maxes, scales, B planes
  const size_t ybytes = sizeof(float) * (size_t)Mp * Kp, wbytes = sizeof(float2) * 2 * (size_t)nen * Kp;
  const size_t mxbytes = sizeof(float) * (1 + 2 * (size_t)nen);
  const size_t sbytes = sizeof(float) * (size_t)Mp * (2 + 2 * (size_t)nen);  // rowmax, sB, sA
  const size_t bpbytes = (size_t)nplanes * 2 * Mp * Kp;
  const size_t sboff = ((ybytes + wbytes + ((mxbytes + 255) / 256) * 256 + sbytes + 1023) / 1024) * 1024;
  unsigned char *base = (unsigned char *)grow(ws.planes, ws.planes_bytes, sboff + bpbytes + 1024);
  float *Yt = (float *)base;
  float2 *wt = (float2 *)(base + ybytes);
  float *maxes = (float *)(base + ybytes + wbytes);
  float *rowmax = (float *)(base + ybytes + wbytes + ((mxbytes + 255) / 256) * 256);
  float *sBv = rowmax + Mp, *sAv = sBv + Mp;
  unsigned char *Bp = base + sboff;
  RP_CUDA(cudaMemsetAsync(base, 0, ybytes + wbytes + mxbytes, st));
  if (Kn > 0x7fffffffL) fail(1, "batch too large");
  RP_CUDA(cudaMemsetAsync(rowmax, 0, sizeof(float) * (size_t)Mp, st));
  {
    const dim3 g((unsigned)((Kn + YT_K - 1) / YT_K), (unsigned)((ng + YT_G - 1) / YT_G));
    if (rho64) yt_kernel<double2><<<g, 256, 0, st>>>(rho64, npair, ntk, ng, Gp, Kp, Kn, Yt, head, g0, rowmax);
    else yt_kernel<float2><<<g, 256, 0, st>>>(rho, npair, ntk, ng, Gp, Kp, Kn, Yt, head, g0, rowmax);
  }
  wt_kernel<<<(unsigned)((Kn + 255) / 256), 256, 0, st>>>(w, npair, ntk, nen, Kp, wt);
  maxes_kernel<<<1024, 256, 0, st>>>(wt, nen, Kp, Kn, maxes);
  const int exact = nplanes == 3 ? 1 : 0;
  scales_kernel<<<(Mp + 127) / 128, 128, 0, st>>>(rowmax, maxes, Mp, nen, exact ? 7 : 14, sBv, sAv);
  launches += 4;
  RP_CUDA(cudaGetLastError());
  if (head && rowcol && !rho64) {
    dim3 g(ng, nen, 2);
    gamma_rowcol_f32_kernel<<<g, 256, 0, st>>>(rho, w, head, npair, ntk, ng, nen, g0, rowcol);
    launches++;
    RP_CUDA(cudaGetLastError());
  }
  // B operand planes, shared by every (frequency, Re/Im) channel
  const int nt = Mp / BM, nkb = Kp / BK;
  {
    dim3 g((unsigned)nkb, nt);
    if (precision == RP_PREC_FP16X3) bplanes_kernel<3, true, false><<<g, 256, 0, st>>>(Yt, sBv, Kp, nkb, Bp);
    else if (precision == RP_PREC_BF16X3) bplanes_kernel<3, true, true><<<g, 256, 0, st>>>(Yt, sBv, Kp, nkb, Bp);
    else bplanes_kernel<2, false, false><<<g, 256, 0, st>>>(Yt, sBv, Kp, nkb, Bp);
    launches++;
    RP_CUDA(cudaGetLastError());
  }
  ws.Yt = Yt; ws.sB = sBv; ws.sA = sAv; ws.wt = wt; ws.Bp = Bp;
  ws.Mp = Mp; ws.precision = precision; ws.ready = 1;
  set_kernel_smem(precision);
  if (ws.tune_pending) {
    const int kp_key = ws.Kp;  // the q's K estimate keys the cache
    ws.Kp = Kp;
    tune_shape(ws, err, st);
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tuned[std::make_tuple(precision, Mp, nen, kbits(kp_key / BK))] = std::make_pair(ws.nsplit, ws.pair);
  }
  ws.Kp = Kp;
  return launches;
}

int tc_gram_group(TcWorkspace *const *wss, int n, int *err, cudaStream_t st) {
  for (int i = 0; i < n; i++) set_kernel_smem(wss[i]->precision);
  GroupPlan P = plan_group(wss, n, st, g_scratch.dev, g_scratch.bytes);
  return launch_group(P, err, st);
}

int tc_contract_batch(TcWorkspace &ws, const float2 *rho, const double2 *rho64, const double2 *w, const double2 *head,
                      int npair, int ntk, int ng, int nen, int g0, int precision, double2 *chi, double2 *rowcol,
                      int *err, cudaStream_t st) {
  (void)chi;
  if (npair == 0) return 0;
  int launches = tc_prepare(ws, rho, rho64, w, head, npair, ntk, ng, nen, g0, precision, rowcol, err, st);
  TcWorkspace *one = &ws;
  RP_CUDA(cudaEventRecord(ws.ev0, st));
  launches += tc_gram_group(&one, 1, err, st);
  RP_CUDA(cudaEventRecord(ws.ev1, st));
  RP_CUDA(cudaStreamSynchronize(st));  // the workspace (and work list) is reused by the next batch
  float ms = 0;
  RP_CUDA(cudaEventElapsedTime(&ms, ws.ev0, ws.ev1));
  ws.gram_seconds += ms * 1e-3;
  ws.ready = 0;
  return launches;
}

int tc_end_q(TcWorkspace &ws, double2 *chi, double2 *rowcol, cudaStream_t st) {
  (void)rowcol;
  const int Gp = Gp_of(ws.ng), Mp = 2 * Gp;
  dim3 grid((unsigned)std::min<size_t>(((size_t)ws.ng * ws.ng + 255) / 256, 2048), ws.nen);
  assemble_kernel<<<grid, 256, 0, st>>>((const float2 *)ws.part, slice_of(Mp, ws.nen), ws.nslice, Mp, Gp, ws.ng,
                                         chi);
  RP_CUDA(cudaGetLastError());
  return 1;
}

double tc_group_run(TcWorkspace *const *wss, int n, double2 *const *chis, int *err, cudaStream_t st, bool graph,
                    long long *launches) {
  if (n <= 0) return 0.0;
  for (int i = 0; i < n; i++) set_kernel_smem(wss[i]->precision);
  // the problem table and work list go up before any capture (host copies are not captured)
  GroupPlan P = plan_group(wss, n, st, g_scratch.dev, g_scratch.bytes);
  long long nl = 0;
  auto enqueue = [&] {
    nl += launch_group(P, err, st);
    for (int i = 0; i < n; i++) nl += tc_end_q(*wss[i], chis[i], nullptr, st);
  };
  cudaEvent_t e0 = wss[0]->ev0, e1 = wss[0]->ev1;
  if (graph) {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    RP_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      enqueue();
    } catch (...) {
      cudaStreamEndCapture(st, &g);  // leave the stream usable
      if (g) cudaGraphDestroy(g);
      throw;
    }
    RP_CUDA(cudaStreamEndCapture(st, &g));
    const cudaError_t ie = cudaGraphInstantiate(&x, g, 0);
    if (ie != cudaSuccess) {
      cudaGraphDestroy(g);
      fail(-1, "CUDA graph of the ragged group: %s", cudaGetErrorString(ie));
    }
    RP_CUDA(cudaEventRecord(e0, st));
    const cudaError_t le = cudaGraphLaunch(x, st);
    RP_CUDA(cudaEventRecord(e1, st));
    const cudaError_t se = cudaStreamSynchronize(st);
    cudaGraphExecDestroy(x);
    cudaGraphDestroy(g);
    if (le != cudaSuccess) fail(-1, "CUDA graph launch: %s", cudaGetErrorString(le));
    if (se != cudaSuccess) fail(-1, "ragged group: %s", cudaGetErrorString(se));
  } else {
    RP_CUDA(cudaEventRecord(e0, st));
    enqueue();
    RP_CUDA(cudaEventRecord(e1, st));
    RP_CUDA(cudaStreamSynchronize(st));
  }
  float ms = 0;
  RP_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  for (int i = 0; i < n; i++) wss[i]->ready = 0;
  if (launches) *launches += nl;
  return ms * 1e-3;
}

}  // namespace rp
