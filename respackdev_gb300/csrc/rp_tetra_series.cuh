// rp_tetra_series.cuh -- well-conditioned vertex weights of one tetrahedron,
// FP32, for host and device.
//
// For a tetrahedron with linear g (vertex values g_v = dsgn (gr_v + i delt),
// all with the same imaginary part), the linear-tetrahedron weight of vertex v
// for frequency w is a confluent divided difference.  The closed forms of
// m_tetrahedron_20170325.F:304-451 (sub2normal / sub1normal) evaluate it as
// sums of terms g^2 log g / prod(g_i - g_j).  Those terms cancel by up to
// (|w + g| / |g_i - g_j|)^3, which costs FP64 about 1e-6 of the per-k weights
// on dense meshes.  Expanded about the mean gbar instead:
//   c_v = sum_n (-1)^n n!/(n+4)! h_n(d_0..d_3, d_v) / z^(n+1),
//   z = w + gbar,  d_i = g_i - gbar (real),
// where h_n is the complete homogeneous polynomial of degree n in the five
// values d_0..d_3 and d_v again.  The terms fall off like r^n with
// r = max|d| / |z|.  For r <= 0.5 the series in FP32 is closer to the exact
// weights than the closed forms in FP64.  Larger r (near resonance) is left
// to the closed forms, which are well conditioned there.
//
// The h_n are generated in ascending n by the recurrences
//   H1_n = d0 H1_{n-1},  Hm_n = H(m-1)_n + d(m-1) Hm_{n-1}  (m = 2..4),
//   Hv_n = H4_n + d_v Hv_{n-1},
// so no arrays are kept: eight running values and four complex sums.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define RP_TS_HD __host__ __device__ __forceinline__
#else
#define RP_TS_HD inline
#endif

namespace rp {

struct TsCplx {
  float r, i;
};

// the largest r the series takes, and its term cap
constexpr float TS_RMAX = 0.5f;
constexpr int TS_NMAX = 30;

// Vertex weights x[v] (v = 0..3, the order of gr) of one tetrahedron for one
// sign (dsgn = +-1) and frequency w = (wr, wi), in the closed forms'
// normalisation (all four equal: x = 1 / (24 (w + g))).  Returns false, with x
// untouched, when r > TS_RMAX or z = 0.
RP_TS_HD bool tetra_series_weights(const double (&gr)[4], double dsgn, double delt, double wr, double wi,
                                   TsCplx (&x)[4]) {
  const double mean = 0.25 * ((gr[0] + gr[1]) + (gr[2] + gr[3]));
  // z = w + gbar in double (one subtraction's worth of care), the rest in FP32
  const double zr = wr + dsgn * mean, zi = wi + dsgn * delt;
  const double zz = zr * zr + zi * zi;
  if (!(zz > 0.0)) return false;
  float d[4];
  float dmax = 0.f;
  for (int v = 0; v < 4; v++) {
    d[v] = (float)(dsgn * (gr[v] - mean));
    dmax = fmaxf(dmax, fabsf(d[v]));
  }
  const float r = dmax / (float)sqrt(zz);
  if (!(r <= TS_RMAX)) return false;
  // terms to FP32 rounding: term n is at most r^n times the first
  // (a_n h_n <= max|d|^n / 24), so r^N <= 2^-24 suffices
  int nterm = 1;
  if (r > 1e-30f) {
    const float n = 1.f + ceilf(-24.f * 0.6931472f / logf(r));
    nterm = n < (float)TS_NMAX ? (int)n : TS_NMAX;
  }
  // u = 1 / z
  const float ur = (float)(zr / zz), ui = (float)(-zi / zz);
  float h1 = 1.f, h2 = 1.f, h3 = 1.f, h4 = 1.f;   // H1_0 .. H4_0
  float hv[4] = {1.f, 1.f, 1.f, 1.f};
  float sr[4], si[4];
  // n = 0: a_0 = 1/24, u^1
  float pr = ur, pi = ui;                           // u^(n+1)
  float an = 1.f / 24.f;
  for (int v = 0; v < 4; v++) {
    sr[v] = an * pr;
    si[v] = an * pi;
  }
  for (int n = 1; n < nterm; n++) {
    h1 = d[0] * h1;
    h2 = h1 + d[1] * h2;
    h3 = h2 + d[2] * h3;
    h4 = h3 + d[3] * h4;
    an = -an * (float)n / (float)(n + 4);
    const float qr = pr * ur - pi * ui, qi = pr * ui + pi * ur;
    pr = qr;
    pi = qi;
    for (int v = 0; v < 4; v++) {
      hv[v] = h4 + d[v] * hv[v];
      const float t = an * hv[v];
      sr[v] += t * pr;
      si[v] += t * pi;
    }
  }
  for (int v = 0; v < 4; v++) x[v] = TsCplx{sr[v], si[v]};
  return true;
}

// a_n = (-1)^n n!/(n+4)! without its sign: 1 / ((n+1)(n+2)(n+3)(n+4))
#define RP_TS_A(n) (1.0f / ((float)((n) + 1) * (float)((n) + 2) * (float)((n) + 3) * (float)((n) + 4)))
#define RP_TS_A5(n) RP_TS_A(n), RP_TS_A(n + 1), RP_TS_A(n + 2), RP_TS_A(n + 3), RP_TS_A(n + 4)
#if defined(__CUDA_ARCH__)
static __constant__ float kTsA[TS_NMAX] = {RP_TS_A5(0), RP_TS_A5(5), RP_TS_A5(10), RP_TS_A5(15), RP_TS_A5(20),
                                           RP_TS_A5(25)};
#else
static const float kTsA[TS_NMAX] = {RP_TS_A5(0), RP_TS_A5(5), RP_TS_A5(10), RP_TS_A5(15), RP_TS_A5(20),
                                    RP_TS_A5(25)};
#endif

// Products and sums that the compiler must not contract into FMAs, so that
// every caller that decides whether the series is taken for a (tetrahedron,
// sign, frequency) decides the same way.
#if defined(__CUDA_ARCH__)
#define RP_TS_MUL(a, b) __fmul_rn((a), (b))
#define RP_TS_ADD(a, b) __fadd_rn((a), (b))
#else
#define RP_TS_MUL(a, b) ((a) * (b))
#define RP_TS_ADD(a, b) ((a) + (b))
#endif

// (ah + al) + (bh + bl) for two float pairs, rounded once to float: TwoSum of
// the heads, then the tails (z = w + gbar to about one rounding, without FP64)
RP_TS_HD float ts_pair_sum(float ah, float al, float bh, float bl) {
  const float s = RP_TS_ADD(ah, bh);
  const float bp = RP_TS_ADD(s, -ah);
  const float err = RP_TS_ADD(RP_TS_ADD(ah, -RP_TS_ADD(s, -bp)), RP_TS_ADD(bh, -bp));
  return RP_TS_ADD(s, RP_TS_ADD(err, RP_TS_ADD(al, bl)));
}

// Whether the series is taken at z (r = dmax / |z| <= TS_RMAX, z != 0), and 1 / |z|^2.
RP_TS_HD void ts_decide(float zr, float zi, float dmax, bool &ok, float &inv) {
  const float zz = RP_TS_ADD(RP_TS_MUL(zr, zr), RP_TS_MUL(zi, zi));
  ok = zz > 0.f && RP_TS_MUL(dmax, dmax) <= RP_TS_MUL(TS_RMAX * TS_RMAX, zz);
  inv = ok ? 1.f / zz : 0.f;
}

// The weight of one vertex for both signs at once, given each sign's z and
// decision (ts_decide).  d[i] = g_i - gbar (FP32) for the sign +1, with g_i the
// tetrahedron's points (near-degenerate vertices already replaced by their
// average, as the reference's calc() does) and gbar their mean; dv = d of the
// vertex; dmax = max |d|.  The sign -1 negates every d, so it shares the h_n
// and its terms carry (-1)^n.  x[s] = 0 where ok[s] is false.  Values in the
// closed forms' normalisation (before the factor fk = dsgn).
//
// Near resonance |z| is of order delt and u^n alone would overflow FP32 (and
// h_n underflow) long before their product, which r^n bounds, is small.  So
// with sc = 1/min|z| over the signs taken, the recurrences run on d sc
// (|d sc| <= r) and u / sc (|u / sc| <= 1): h_n(d) u^n = h_n(d sc) (u / sc)^n.
RP_TS_HD void tetra_series_core(const float (&d)[4], float dv, float dmax, const float (&zr)[2], const float (&zi)[2],
                                const bool (&ok)[2], const float (&inv)[2], TsCplx (&x)[2]) {
  x[0] = x[1] = TsCplx{0.f, 0.f};
  if (!ok[0] && !ok[1]) return;
  float sc = 0.f;
  for (int s = 0; s < 2; s++)
    if (ok[s]) sc = fmaxf(sc, sqrtf(inv[s]));
  // scaled u = conj(z) / |z|^2 / sc of each sign, and the scaled deviations
  const float is = 1.f / sc;
  const float ur0 = zr[0] * inv[0] * is, ui0 = -zi[0] * inv[0] * is;
  const float ur1 = zr[1] * inv[1] * is, ui1 = -zi[1] * inv[1] * is;
  const float e0 = d[0] * sc, e1 = d[1] * sc, e2 = d[2] * sc, e3 = d[3] * sc, ev = dv * sc;
  const float rmax = dmax * sc;
  // S_s = sum_n a_n h_n(d sc) (u_s / sc)^n; n = 0 term a_0
  float pr0 = 1.f, pi0 = 0.f, pr1 = 1.f, pi1 = 0.f;
  float sr0 = kTsA[0], si0 = 0.f, sr1 = kTsA[0], si1 = 0.f;
  float h1 = 1.f, h2 = 1.f, h3 = 1.f, h4 = 1.f, hv = 1.f;
  // term n is at most r^n times the first: take terms while r^(n-1) > 2^-24
  float rprev = 1.f;
  float sgn = 1.f;
  for (int n = 1; n < TS_NMAX && rprev > 5.9604645e-8f; n++) {
    h1 = e0 * h1;
    h2 = h1 + e1 * h2;
    h3 = h2 + e2 * h3;
    h4 = h3 + e3 * h4;
    hv = h4 + ev * hv;
    sgn = -sgn;
    const float t = sgn * kTsA[n] * hv;
    float q = pr0 * ur0 - pi0 * ui0;
    pi0 = pr0 * ui0 + pi0 * ur0;
    pr0 = q;
    sr0 += t * pr0;
    si0 += t * pi0;
    q = pr1 * ur1 - pi1 * ui1;
    pi1 = pr1 * ui1 + pi1 * ur1;
    pr1 = q;
    // sign -1: its d are negated, so its h_n carry (-1)^n
    const float t1 = (n & 1) ? -t : t;
    sr1 += t1 * pr1;
    si1 += t1 * pi1;
    rprev *= rmax;
  }
  // x_s = u_s S_s, u_s = conj(z_s) / |z_s|^2
  if (ok[0]) {
    const float ar = zr[0] * inv[0], ai = -zi[0] * inv[0];
    x[0] = TsCplx{ar * sr0 - ai * si0, ar * si0 + ai * sr0};
  }
  if (ok[1]) {
    const float ar = zr[1] * inv[1], ai = -zi[1] * inv[1];
    x[1] = TsCplx{ar * sr1 - ai * si1, ar * si1 + ai * sr1};
  }
}

// a double as a float pair (hi + lo to about 2^-48 relative)
RP_TS_HD void ts_split(double v, float &hi, float &lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// z_s = w + s (gbar + i delt) of sign s (s = 0: +1, s = 1: -1) from float pairs,
// and its decision: the one formation the gather and the fallback pass share.
RP_TS_HD void ts_z(float wrh, float wrl, float wih, float wil, float mh, float ml, float dh, float dl, float dmax,
                   float (&zr)[2], float (&zi)[2], bool (&ok)[2], float (&inv)[2]) {
  zr[0] = ts_pair_sum(wrh, wrl, mh, ml);
  zi[0] = ts_pair_sum(wih, wil, dh, dl);
  zr[1] = ts_pair_sum(wrh, wrl, -mh, -ml);
  zi[1] = ts_pair_sum(wih, wil, -dh, -dl);
  ts_decide(zr[0], zi[0], dmax, ok[0], inv[0]);
  ts_decide(zr[1], zi[1], dmax, ok[1], inv[1]);
}

// The same from double inputs (the host tests' interface), with z formed as
// the device forms it.  ok[s] says whether the series was taken for sign s.
RP_TS_HD void tetra_series_vertex2(const float (&d)[4], float dv, float dmax, double mean, double delt, double wr,
                                   double wi, bool (&ok)[2], TsCplx (&x)[2]) {
  float wrh, wrl, wih, wil, mh, ml, dh, dl;
  ts_split(wr, wrh, wrl);
  ts_split(wi, wih, wil);
  ts_split(mean, mh, ml);
  ts_split(delt, dh, dl);
  float zr[2], zi[2], inv[2];
  ts_z(wrh, wrl, wih, wil, mh, ml, dh, dl, dmax, zr, zi, ok, inv);
  tetra_series_core(d, dv, dmax, zr, zi, ok, inv, x);
}

}  // namespace rp
