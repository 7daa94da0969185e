// rp_tetra.cu -- generalized tetrahedron weights in FP64 (K4).
//
// Follows src/chiqw/m_tetrahedron_20170325.F (MIT-licensed Fujiwara et al.
// generalized tetrahedron method): ttrhdrn_chi0 (:99-141) splits every
// tetrahedron of the k mesh at the Fermi level (ttct, :143-207), classifies
// near-degenerate vertex energies (chk1, :457-503) and evaluates the closed
// forms (:304-451) per frequency, scattering them to the four vertices (calc,
// :209-302).  chiqw.F:1371-1383 calls it for dsgn = +1 and -1 with the pair's
// energies rounded to single precision (kindless CMPLX, chiqw.F:1354,1357).
//
// One CTA per (band pair, frequency chunk).  The weights of the chunk live in
// shared memory (ntk x nchunk complex) and every thread walks tetrahedra,
// adding its vertex terms with shared-memory FP64 atomics.  Tetrahedra that the
// Fermi level does not cut (all of them for an insulator) skip ttct.
#include "rp_dev.cuh"
#include "rp_host.h"
#include "rp_tetra_series.cuh"

namespace rp {

struct cx {
  double r, i;
  __device__ cx() : r(0), i(0) {}
  __device__ cx(double a, double b = 0) : r(a), i(b) {}
};
__device__ __forceinline__ cx operator+(cx a, cx b) { return cx(a.r + b.r, a.i + b.i); }
__device__ __forceinline__ cx operator-(cx a, cx b) { return cx(a.r - b.r, a.i - b.i); }
__device__ __forceinline__ cx operator-(cx a) { return cx(-a.r, -a.i); }
__device__ __forceinline__ cx operator*(cx a, cx b) { return cx(a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r); }
__device__ __forceinline__ cx operator*(cx a, double s) { return cx(a.r * s, a.i * s); }
__device__ __forceinline__ cx operator*(double s, cx a) { return cx(a.r * s, a.i * s); }
__device__ __forceinline__ cx operator/(cx a, cx b) {
  // Smith's algorithm
  if (fabs(b.r) >= fabs(b.i)) {
    double t = b.i / b.r, d = b.r + b.i * t;
    return cx((a.r + a.i * t) / d, (a.i - a.r * t) / d);
  }
  double t = b.r / b.i, d = b.r * t + b.i;
  return cx((a.r * t + a.i) / d, (a.i * t - a.r) / d);
}
__device__ __forceinline__ cx operator/(cx a, double s) { return cx(a.r / s, a.i / s); }
__device__ __forceinline__ cx operator/(double s, cx b) { return cx(s, 0) / b; }
__device__ __forceinline__ double cabs_(cx a) { return hypot(a.r, a.i); }
// log z = log|z| + i arg z, with log|z| = log(|z|^2) / 2 (|z| of order one here)
__device__ __forceinline__ cx clog_(cx a) { return cx(0.5 * log(fma(a.r, a.r, a.i * a.i)), atan2(a.i, a.r)); }

// ---- closed forms (m_tetrahedron_20170325.F:304-451), one frequency w ----
__device__ cx s1g30g21(cx g0, cx g1, cx w) {
  cx d = g0 - g1;
  cx v = (0.5 * (g0 + g1) + w) / (d * d);
  return v - clog_((g0 + w) / (g1 + w)) * (g0 + w) * (g1 + w) / (d * d * d);
}
__device__ cx s1g30g20(cx g0, cx g1, cx w) {
  cx d = g0 - g1;
  cx v = (g0 - 3.0 * g1 - 2.0 * w) * 0.25 / (d * d);
  return v + (g1 + w) * (g1 + w) * clog_((g0 + w) / (g1 + w)) * 0.5 / (d * d * d);
}
__device__ cx s1g30(cx g0, cx g1, cx g2, cx w) {
  cx v = 0.5 / (g0 - g2);
  cx t = (g0 - g2) * (g0 - g1);
  v = v - 0.5 / (t * t) * (g0 + w) * (-2.0 * (g1 + w) * (g2 + w) + (g0 + w) * (g1 + g2 + 2.0 * w)) *
              clog_((g0 + w) / (g1 + w));
  v = v + 0.5 / ((g0 - g2) * (g0 - g2)) * (g2 + w) * (g2 + w) * clog_((g1 + w) / (g2 + w)) / (g1 - g2);
  return v + 0.5 / ((g0 - g2) * (g0 - g1)) * (g1 + w);
}
__device__ cx s1normal(cx g0, cx g1, cx g2, cx g3, cx w) {
  cx L10 = clog_((g1 + w) / (g0 + w)), L20 = clog_((g2 + w) / (g0 + w)), L30 = clog_((g3 + w) / (g0 + w));
  cx v = (-(g1 + w) * (g1 + w) * L10) / ((g0 - g2) * (g0 - g3) * (g0 - g1)) * 0.5;
  v = v - ((g1 + w) * (g1 + w) * L10 - (g2 + w) * (g2 + w) * L20) / ((g0 - g2) * (g1 - g2) * (g2 - g3)) * 0.5;
  return v + ((g1 + w) * (g1 + w) * L10 - (g3 + w) * (g3 + w) * L30) / ((g1 - g3) * (g0 - g3) * (g2 - g3)) * 0.5;
}
__device__ cx s2simple(cx g0, cx w) { return 1.0 / ((g0 + w) * 24.0); }
__device__ cx s2g30g20(cx g0, cx g1, cx w) {
  cx d = g0 - g1;
  cx v = ((g0 - g1) * (g0 + 2.0 * g1 + 3.0 * w) - 6.0 * (g0 + w) * (g1 + w)) / (12.0 * (d * d * d));
  return v + (g0 + w) * (g1 + w) * (g1 + w) * clog_((g0 + w) / (g1 + w)) / (d * d * d * d) * 0.5;
}
__device__ cx s2g30g10(cx g0, cx g2, cx w) {
  cx d = g0 - g2;
  cx v = (2.0 * (g0 + w) * (g0 + w) - 7.0 * (g0 + w) * (g2 + w) + 11.0 * (g2 + w) * (g2 + w)) / (36.0 * (d * d * d));
  return v - (g2 + w) * (g2 + w) * (g2 + w) * clog_((g0 + w) / (g2 + w)) / (6.0 * (d * d * d * d));
}
__device__ cx s2g10(cx g0, cx g2, cx g3, cx w) {
  cx d2 = g0 - g2, d3 = g0 - g3;
  cx v = (g0 + w) * ((g0 + w) * (g0 + w) + 5.0 * (g2 + w) * (g3 + w) - 3.0 * (g0 + w) * (g2 + g3 + 2.0 * w)) /
         (12.0 * (d2 * d2) * (d3 * d3));
  v = v - (g2 + w) * (g2 + w) * (g2 + w) * clog_((g2 + w) / (g0 + w)) / (6.0 * (d2 * d2 * d2) * (g2 - g3));
  return v + (g3 + w) * (g3 + w) * (g3 + w) * clog_((g3 + w) / (g0 + w)) / (6.0 * (d3 * d3 * d3) * (g2 - g3));
}
__device__ cx s2g30(cx g0, cx g1, cx g2, cx w) {
  cx d01 = g0 - g1, d02 = g0 - g2, d12 = g1 - g2;
  cx v = ((g0 + w) * (g0 + w) * (g1 - g2) + (g1 + w) * (g1 + w) * (g0 - g2)) / (6.0 * d02 * (d01 * d01) * d12);
  v = v - (g0 + w) * (g0 + w) * (2.0 * (g1 + w) * (g0 - g2) + (g2 + w) * (g0 - g1)) * clog_((g0 + w) / (g2 + w)) /
              (6.0 * (d02 * d02) * (d01 * d01 * d01));
  return v + (g1 + w) * (g1 + w) * (2.0 * (g0 + w) * (g1 - g2) - (g2 + w) * (g0 - g1)) * clog_((g1 + w) / (g2 + w)) /
                 (6.0 * (d01 * d01 * d01) * (d12 * d12));
}
__device__ cx s2normal(cx g0, cx g1, cx g2, cx g3, cx w) {
  cx v = -(g1 + w) * (g1 + w) / (6.0 * (g0 - g1) * (g1 - g2) * (g1 - g3));
  v = v - (g2 + w) * (g2 + w) * (g2 + w) * clog_((g2 + w) / (g1 + w)) / (6.0 * (g0 - g2) * ((g1 - g2) * (g1 - g2)) * (g2 - g3));
  v = v + (g3 + w) * (g3 + w) * (g3 + w) * clog_((g3 + w) / (g1 + w)) / (6.0 * (g0 - g3) * ((g1 - g3) * (g1 - g3)) * (g2 - g3));
  return v + (g0 + w) * (g0 + w) * (g0 + w) * clog_((g0 + w) / (g1 + w)) / (6.0 * ((g0 - g1) * (g0 - g1)) * (g0 - g2) * (g0 - g3));
}

// chk1 on positions 0..3 (ia1 = identity); returns case (sum ia2) and i3
struct Chk { int s, i3; int ia3[4], ia4[4]; };
__device__ Chk chk1(double dmna, double dmnr, const cx *gk) {
  Chk c;
  int ia2[4] = {0, 0, 0, 0}, i3 = 0, i4 = 0;
  for (int a = 0; a < 4; a++) { c.ia3[a] = 0; c.ia4[a] = 0; }
  for (int i1 = 1; i1 <= 3; i1++)
    for (int i2 = i1 + 1; i2 <= 4; i2++) {
      int p = i1 % 4, r = i2 % 4;
      double d1 = cabs_(gk[p] - gk[r]);
      double d2 = cabs_(gk[p] + gk[r]) * 0.5;
      if (d1 < dmna || d1 / d2 < dmnr) {
        i3++;
        if (ia2[p] == 0) { c.ia3[i4++] = p; ia2[p] = 1; }
        if (ia2[r] == 0) { c.ia3[i4++] = r; ia2[r] = 1; }
      }
    }
  int i5 = 0;
  for (int i1 = 1; i1 <= 4; i1++) { int p = i1 % 4; if (ia2[p] == 0) c.ia4[i5++] = p; }
  c.s = ia2[0] + ia2[1] + ia2[2] + ia2[3];
  c.i3 = i3;
  return c;
}

// calc() for one frequency: vertex terms x[0..3] (positions), fk per position
__device__ bool calc_w(const Chk &c, const cx *fk, const cx *gk, cx w, cx *x) {
  x[0] = x[1] = x[2] = x[3] = cx(0, 0);
  switch (c.s) {
  case 0: {
    const int *a = c.ia4;
    cx c1 = s2normal(gk[a[1]], gk[a[0]], gk[a[2]], gk[a[3]], w);
    cx c2 = s2normal(gk[a[0]], gk[a[1]], gk[a[2]], gk[a[3]], w);
    cx c3 = s2normal(gk[a[0]], gk[a[2]], gk[a[1]], gk[a[3]], w);
    cx c4 = s1normal(gk[a[0]], gk[a[3]], gk[a[1]], gk[a[2]], w);
    x[a[0]] = fk[a[0]] * c1;
    x[a[1]] = fk[a[1]] * c2;
    x[a[2]] = fk[a[2]] * c3;
    x[a[3]] = fk[a[3]] * (c4 - c3 - c2 - c1);
    return true;
  }
  case 2: {
    cx geq1 = (gk[c.ia3[0]] + gk[c.ia3[1]]) / 2.0;
    cx c1 = s2g10(geq1, gk[c.ia4[0]], gk[c.ia4[1]], w);
    cx c2 = s2g30(geq1, gk[c.ia4[0]], gk[c.ia4[1]], w);
    cx c3 = s1g30(geq1, gk[c.ia4[1]], gk[c.ia4[0]], w);
    x[c.ia3[0]] = fk[c.ia3[0]] * c1;
    x[c.ia3[1]] = fk[c.ia3[1]] * c1;
    x[c.ia4[0]] = fk[c.ia4[0]] * c2;
    x[c.ia4[1]] = fk[c.ia4[1]] * (c3 - c2 - c1 - c1);
    return true;
  }
  case 3: {
    cx geq1 = (gk[c.ia3[0]] + gk[c.ia3[1]] + gk[c.ia3[2]]) / 3.0;
    cx c1 = s2g30g10(geq1, gk[c.ia4[0]], w);
    cx c2 = s1g30g20(geq1, gk[c.ia4[0]], w);
    x[c.ia3[0]] = fk[c.ia3[0]] * c1;
    x[c.ia3[1]] = fk[c.ia3[1]] * c1;
    x[c.ia3[2]] = fk[c.ia3[2]] * c1;
    x[c.ia4[0]] = fk[c.ia4[0]] * (c2 - c1 - c1 - c1);
    return true;
  }
  case 4:
    if (c.i3 == 2) {
      cx geq1 = (gk[c.ia3[0]] + gk[c.ia3[1]]) / 2.0, geq2 = (gk[c.ia3[2]] + gk[c.ia3[3]]) / 2.0;
      cx c1 = s2g30g20(geq1, geq2, w);  // ttrhdrn_sub2g30g21(geq2,geq1,...) = sub2g30g20(geq1,geq2)
      cx c2 = s1g30g21(geq1, geq2, w);
      x[c.ia3[0]] = fk[c.ia3[0]] * c1;
      x[c.ia3[1]] = fk[c.ia3[1]] * c1;
      x[c.ia3[2]] = fk[c.ia3[2]] * (c2 - c1 - c1) * 0.5;
      x[c.ia3[3]] = fk[c.ia3[3]] * (c2 - c1 - c1) * 0.5;
      return true;
    } else if (c.i3 >= 3 && c.i3 <= 6) {
      cx geq1 = (gk[c.ia3[0]] + gk[c.ia3[1]] + gk[c.ia3[2]] + gk[c.ia3[3]]) / 4.0;
      cx c1 = s2simple(geq1, w);
      for (int a = 0; a < 4; a++) x[c.ia3[a]] = c1 * fk[c.ia3[a]];
      return true;
    }
    return false;
  default:
    return false;
  }
}

#define TT_NMAX 64

// ttct (:143-207) on local arrays; returns false when more than TT_NMAX pieces
__device__ bool ttct(double dval, const double *dvtx, int imod, int &ntet, double (*dwgt)[4][4], double *dvol) {
  unsigned char bvtx[TT_NMAX][4];
  bool btsk[TT_NMAX];
  for (int t = 0; t < TT_NMAX; t++) { btsk[t] = false; bvtx[t][0] = bvtx[t][1] = bvtx[t][2] = bvtx[t][3] = 0; }
  int itet = 0;
  while (itet < ntet) {
    itet++;
    const int t = itet - 1;
    double d0[4];
    for (int i1 = 0; i1 < 4; i1++) {
      double s = 0;
      for (int v = 0; v < 4; v++) s += dwgt[t][i1][v] * dvtx[v];
      d0[i1] = s;
    }
    bool b1 = false;
    int i1, i2 = 0;
    for (i1 = 0; i1 < 3; i1++) {
      if (bvtx[t][i1]) continue;
      for (i2 = i1 + 1; i2 < 4; i2++) {
        if (bvtx[t][i2]) continue;
        b1 = (d0[i1] - dval) * (dval - d0[i2]) > 0.0;
        if (b1) break;
      }
      if (b1) break;
    }
    if (b1) {
      double dd1 = (d0[i2] - dval) / (d0[i2] - d0[i1]);
      double dd2 = (dval - d0[i1]) / (d0[i2] - d0[i1]);
      ntet++;
      if (ntet > TT_NMAX) return false;
      const int nt = ntet - 1;
      for (int a = 0; a < 4; a++) {
        bvtx[nt][a] = bvtx[t][a];
        for (int v = 0; v < 4; v++) dwgt[nt][a][v] = dwgt[t][a][v];
      }
      bvtx[nt][i1] = 1;
      for (int v = 0; v < 4; v++) dwgt[nt][i1][v] = dwgt[t][i1][v] * dd1 + dwgt[t][i2][v] * dd2;
      dvol[nt] = dvol[t] * dd1;
      bvtx[t][i2] = 1;
      for (int v = 0; v < 4; v++) dwgt[t][i2][v] = dwgt[t][i1][v] * dd1 + dwgt[t][i2][v] * dd2;
      dvol[t] = dvol[t] * dd2;
      itet--;
    } else {
      for (int a = 0; a < 4; a++) {
        if (bvtx[t][a]) continue;
        btsk[t] = btsk[t] || ((double)imod * (d0[a] - dval) > 0.0);
      }
    }
  }
  int k = 0;
  for (int a = 0; a < ntet; a++) {
    if (!btsk[a]) continue;
    for (int i = 0; i < 4; i++)
      for (int v = 0; v < 4; v++) dwgt[k][i][v] = dwgt[a][i][v];
    dvol[k] = dvol[a];
    k++;
  }
  ntet = k;
  return true;
}

__device__ __forceinline__ void sadd(double2 *xo, cx v) {
  atomicAdd(&xo->x, v.r);
  atomicAdd(&xo->y, v.i);
}

// one (sub)tetrahedron: add its terms for frequencies [e0, e0+ne) into xo[slot*stride + e]
__device__ bool tetra_terms(double dmna, double dmnr, const cx *ffk, const cx *ggk, const double2 *em, int e0,
                            int ne, int stride, const int *slot, const double (*wgt)[4], double2 *xo) {
  Chk c = chk1(dmna, dmnr, ggk);
  for (int e = 0; e < ne; e++) {
    cx w(em[e0 + e].x, em[e0 + e].y);
    cx x[4];
    if (!calc_w(c, ffk, ggk, w, x)) return false;
    if (wgt == nullptr) {
      for (int a = 0; a < 4; a++) sadd(&xo[slot[a] * stride + e], x[a]);
    } else {
      for (int i5 = 0; i5 < 4; i5++) {
        cx s = x[0] * wgt[0][i5] + x[1] * wgt[1][i5] + x[2] * wgt[2][i5] + x[3] * wgt[3][i5];
        sadd(&xo[slot[i5] * stride + e], s);
      }
    }
  }
  return true;
}

// Normal case of calc() (chk1 finds no near-degenerate pair, so ia4 holds the
// positions 1, 2, 3, 0: m_tetrahedron_20170325.F:457-503, calc :209-235) with
// shared vertex logs.  All four g share the imaginary part delt*dsgn, so
// g_a - g_b is real and log(z_a / z_b) = L_a - L_b with L = log(g + w) (z_a,
// z_b in the same half plane).  The closed forms sub2normal / sub1normal
// (:346-363, :435-451) then need only real reciprocal differences
// id(a,b) = 1/(gr_a - gr_b), computed once per tetrahedron for every frequency
// and both signs: the sign -1 negates every gr, which flips the coefficients
// of odd degree in id and leaves the others.  Every vertex index below is a
// compile-time constant, so all per-vertex values stay in registers.
struct NormalCoef {
  double A[3], B[3], C[3], D[3];   // sub2normal forms c1, c2, c3
  double S1a, S1b, S1c;            // sub1normal form c4
};

// id(i,j) from r = {id01, id02, id03, id12, id13, id23}; i, j constants after inlining
__device__ __forceinline__ double idr(const double (&r)[6], int i, int j) {
  const bool neg = i > j;
  const int a = neg ? j : i, b = neg ? i : j;
  const int k = a == 0 ? b - 1 : (a == 1 ? b + 1 : 5);
  return neg ? -r[k] : r[k];
}

template <int P, int Q, int R, int S>
__device__ __forceinline__ void coef2(const double (&r)[6], double &A, double &B, double &C, double &D) {
  A = idr(r, P, Q) * idr(r, Q, R) * idr(r, Q, S) / 6.0;
  B = idr(r, P, R) * idr(r, Q, R) * idr(r, Q, R) * idr(r, R, S) / 6.0;
  C = idr(r, P, S) * idr(r, Q, S) * idr(r, Q, S) * idr(r, R, S) / 6.0;
  D = idr(r, P, Q) * idr(r, P, Q) * idr(r, P, R) * idr(r, P, S) / 6.0;
}

// sign +1 coefficients: c1 = sub2normal(g2, g1, g3, g0), c2 = sub2normal(g1, g2, g3, g0),
// c3 = sub2normal(g1, g3, g2, g0), c4 = sub1normal(g1, g0, g2, g3)
__device__ __forceinline__ void normal_coef(const double (&gr)[4], NormalCoef &c) {
  const double d01 = gr[0] - gr[1], d02 = gr[0] - gr[2], d03 = gr[0] - gr[3];
  const double d12 = gr[1] - gr[2], d13 = gr[1] - gr[3], d23 = gr[2] - gr[3];
  const double r[6] = {1.0 / d01, 1.0 / d02, 1.0 / d03, 1.0 / d12, 1.0 / d13, 1.0 / d23};
  coef2<2, 1, 3, 0>(r, c.A[0], c.B[0], c.C[0], c.D[0]);
  coef2<1, 2, 3, 0>(r, c.A[1], c.B[1], c.C[1], c.D[1]);
  coef2<1, 3, 2, 0>(r, c.A[2], c.B[2], c.C[2], c.D[2]);
  c.S1a = 0.5 * idr(r, 1, 2) * idr(r, 1, 3) * idr(r, 1, 0);
  c.S1b = 0.5 * idr(r, 1, 2) * idr(r, 0, 2) * idr(r, 2, 3);
  c.S1c = 0.5 * idr(r, 0, 3) * idr(r, 1, 3) * idr(r, 2, 3);
}

template <int P, int Q, int R, int S>
__device__ __forceinline__ cx s2term(const cx (&z2)[4], const cx (&z3)[4], const cx (&L)[4], double A, double B,
                                     double C, double D) {
  return -(z2[Q] * A) - z3[R] * (L[R] - L[Q]) * B + z3[S] * (L[S] - L[Q]) * C + z3[P] * (L[P] - L[Q]) * D;
}

// vertex terms x (positions 0..3) of one sign: z_a = g_a + w, L_a = log z_a; sg = +1 or -1
__device__ __forceinline__ void normal_terms(const NormalCoef &c, double sg, const cx (&z)[4], const cx (&L)[4],
                                             cx (&x)[4]) {
  cx z2[4], z3[4];
#pragma unroll
  for (int v = 0; v < 4; v++) { z2[v] = z[v] * z[v]; z3[v] = z2[v] * z[v]; }
  const cx F0 = s2term<2, 1, 3, 0>(z2, z3, L, c.A[0] * sg, c.B[0], c.C[0], c.D[0]);
  const cx F1 = s2term<1, 2, 3, 0>(z2, z3, L, c.A[1] * sg, c.B[1], c.C[1], c.D[1]);
  const cx F2 = s2term<1, 3, 2, 0>(z2, z3, L, c.A[2] * sg, c.B[2], c.C[2], c.D[2]);
  // sub1normal(g1, g0, g2, g3): p = 1, q = 0, r = 2, s = 3
  const cx lq = z2[0] * (L[0] - L[1]), lr = z2[2] * (L[2] - L[1]), ls = z2[3] * (L[3] - L[1]);
  const cx F4 = -(lq * (c.S1a * sg)) - (lq - lr) * (c.S1b * sg) + (lq - ls) * (c.S1c * sg);
  // fk = dsgn on every vertex
  x[1] = F0 * sg;
  x[2] = F1 * sg;
  x[3] = F2 * sg;
  x[0] = (F4 - F2 - F1 - F0) * sg;
}

// Tetrahedron categories: the normal closed forms, the near-degenerate forms of
// chk1's cases 2, 3, 4 (i3 = 2) and 4 (i3 = 3..6) on an uncut tetrahedron, and
// the rest (cut by the Fermi level, or a case calc() does not know).
enum { TC_NORMAL = 0, TC_S2, TC_S3, TC_S4A, TC_S4B, TC_OTHER, TC_NCAT, TC_SKIP = 255 };

// One uncut near-degenerate (tetrahedron, sign) of category cat: the reference's
// special forms (sub1g30g21 ... sub2simple, m_tetrahedron_20170325.F:304-451)
// at the averaged points of calc() (:243-296).  All points share the imaginary
// part delt*dsgn, so every energy difference is real and log(z_a / z_b) =
// L_a - L_b: vertex logs come from the shared table, only the averages need a
// log of their own.  Every real difference of the tetrahedron is turned into a
// product of a few reciprocals once, outside the frequency loop: per frequency
// only complex products and the averaged points' logs remain.
__device__ void degen_tetra(const TetraArgs &a, int code, int cat, const double *e1m, const double *e2m,
                            const double2 *Lt, int e0, int ne, int nec, double2 *xo) {
  const int t = code >> 1, sg = code & 1;
  const double dsgn = sg == 0 ? 1.0 : -1.0, dg = a.delt * dsgn;
  int slot[4];
  double g[4];
  cx ffk[4], ggk[4];
  for (int v = 0; v < 4; v++) {
    slot[v] = a.imt1[4 * t + v];
    ggk[v] = cx(-(e2m[slot[v]] - e1m[slot[v]]), a.delt) * dsgn;
    ffk[v] = cx(dsgn, 0);
    g[v] = ggk[v].r;
  }
  const Chk c = chk1(a.dmna, a.dmnr, ggk);
  // the permuted vertices as scalars: slots (output rows), energies and log rows
  const int i0 = c.ia3[0], i1 = c.ia3[1], i2 = c.ia3[2], i3 = c.ia3[3], j0 = c.ia4[0], j1 = c.ia4[1];
  const int sa0 = slot[i0], sa1 = slot[i1], sa2 = slot[i2], sa3 = slot[i3], sb0 = slot[j0], sb1 = slot[j1];
  const double ga0 = g[i0], ga1 = g[i1], ga2 = g[i2], ga3 = g[i3], gb0 = g[j0], gb1 = g[j1];
  const double2 *Lb0 = Lt + ((size_t)sg * a.ntk + sb0) * nec, *Lb1 = Lt + ((size_t)sg * a.ntk + sb1) * nec;
  auto put = [&](int sl, int e, cx v) { sadd(&xo[sl * nec + e], v); };
  // z on the real axis: the reference's ratio logs through calc()
  auto on_axis = [&](cx w, int e) {
    cx x[4];
    if (!calc_w(c, ffk, ggk, w, x)) { atomicExch(a.err, 2); return; }
    for (int v = 0; v < 4; v++) put(slot[v], e, x[v]);
  };
  if (cat == TC_S2) {
    const double qg = (ga0 + ga1) / 2.0;
    const double d2 = qg - gb0, d3 = qg - gb1, d23 = gb0 - gb1;
    const double r2 = 1.0 / d2, r3 = 1.0 / d3, r23 = 1.0 / d23;
    const double r22 = r2 * r2, r33 = r3 * r3;
    // sub2g10 (c1), sub2g30 (c2), sub1g30 (c3) of calc's case 2
    const double K1 = r22 * r33 / 12.0, K2 = r22 * r2 * r23 / 6.0, K3 = r33 * r3 * r23 / 6.0;
    const double K4 = r3 * r22 * r23 / 6.0, K5 = r33 * r22 * r2 / 6.0, K6 = r22 * r2 * r23 * r23 / 6.0;
    const double K7 = 0.5 * r2, K8 = 0.5 * r22 * r33, K9 = -0.5 * r22 * r23, K10 = 0.5 * r2 * r3;
    for (int e = 0; e < ne; e++) {
      const cx w(a.em[e0 + e].x, a.em[e0 + e].y);
      if (dg + w.i == 0.0) { on_axis(w, e); continue; }
      const cx Zq(qg + w.r, dg + w.i), Z0(gb0 + w.r, dg + w.i), Z1(gb1 + w.r, dg + w.i);
      const cx Lq = clog_(Zq), L0(Lb0[e].x, Lb0[e].y), L1(Lb1[e].x, Lb1[e].y);
      const cx Zq2 = Zq * Zq, Z02 = Z0 * Z0, Z12 = Z1 * Z1, Z01 = Z0 * Z1;
      const cx c1 = Zq * (Zq2 + 5.0 * Z01 - 3.0 * Zq * (Z0 + Z1)) * K1 - Z02 * Z0 * (L0 - Lq) * K2 +
                    Z12 * Z1 * (L1 - Lq) * K3;
      const cx c2 = (Zq2 * d23 + Z02 * d3) * K4 - Zq2 * (2.0 * Z0 * d3 + Z1 * d2) * (Lq - L1) * K5 +
                    Z02 * (2.0 * Zq * d23 - Z1 * d2) * (L0 - L1) * K6;
      const cx c3 = cx(K7, 0.0) - Zq * (-2.0 * Z01 + Zq * (Z1 + Z0)) * (Lq - L1) * K8 + Z02 * (L1 - L0) * K9 +
                    Z1 * K10;
      put(sa0, e, c1 * dsgn);
      put(sa1, e, c1 * dsgn);
      put(sb0, e, c2 * dsgn);
      put(sb1, e, (c3 - c2 - c1 - c1) * dsgn);
    }
  } else if (cat == TC_S3) {
    const double qg = (ga0 + ga1 + ga2) / 3.0;
    const double r = 1.0 / (qg - gb0), r2 = r * r, r3 = r2 * r;
    // sub2g30g10 (c1), sub1g30g20 (c2)
    const double K1 = r3 / 36.0, K2 = r3 * r / 6.0, K3 = 0.25 * r2, K4 = 0.5 * r3;
    for (int e = 0; e < ne; e++) {
      const cx w(a.em[e0 + e].x, a.em[e0 + e].y);
      if (dg + w.i == 0.0) { on_axis(w, e); continue; }
      const cx Zq(qg + w.r, dg + w.i), Zp(gb0 + w.r, dg + w.i);
      const cx dL = clog_(Zq) - cx(Lb0[e].x, Lb0[e].y), Zp2 = Zp * Zp;
      const cx c1 = (2.0 * Zq * Zq - 7.0 * Zq * Zp + 11.0 * Zp2) * K1 - Zp2 * Zp * dL * K2;
      const cx c2 = (Zq - 3.0 * Zp) * K3 + Zp2 * dL * K4;
      put(sa0, e, c1 * dsgn);
      put(sa1, e, c1 * dsgn);
      put(sa2, e, c1 * dsgn);
      put(sb0, e, (c2 - c1 - c1 - c1) * dsgn);
    }
  } else if (cat == TC_S4A) {
    const double q1g = (ga0 + ga1) / 2.0, q2g = (ga2 + ga3) / 2.0;
    const double d = q1g - q2g, r = 1.0 / d, r2 = r * r, r3 = r2 * r;
    // sub2g30g20 (c1), sub1g30g21 (c2)
    const double K1 = r3 / 12.0, K2 = 0.5 * r3 * r, K3 = 0.5 * r2;
    for (int e = 0; e < ne; e++) {
      const cx w(a.em[e0 + e].x, a.em[e0 + e].y);
      if (dg + w.i == 0.0) { on_axis(w, e); continue; }
      const cx Z1(q1g + w.r, dg + w.i), Z2(q2g + w.r, dg + w.i);
      const cx dL = clog_(Z1) - clog_(Z2), Z12 = Z1 * Z2;
      const cx c1 = (d * (Z1 + 2.0 * Z2) - 6.0 * Z12) * K1 + Z12 * Z2 * dL * K2;
      const cx c2 = (Z1 + Z2) * K3 - dL * Z12 * r3;
      const cx h = (c2 - c1 - c1) * 0.5 * dsgn;
      put(sa0, e, c1 * dsgn);
      put(sa1, e, c1 * dsgn);
      put(sa2, e, h);
      put(sa3, e, h);
    }
  } else {  // TC_S4B: sub2simple at the average of all four
    const double s4 = (ga0 + ga1 + ga2 + ga3) / 4.0;
    for (int e = 0; e < ne; e++) {
      const cx w(a.em[e0 + e].x, a.em[e0 + e].y);
      if (dg + w.i == 0.0) { on_axis(w, e); continue; }
      const cx c1 = 1.0 / (cx(s4 + w.r, dg + w.i) * 24.0) * dsgn;
      put(sa0, e, c1);
      put(sa1, e, c1);
      put(sa2, e, c1);
      put(sa3, e, c1);
    }
  }
}

// One (tetrahedron, sign) that is cut by the Fermi level (or of a chk1 case
// the other paths do not know): ttct and the reference's closed forms
// (m_tetrahedron_20170325.F:99-302).  Out of line, so that its large local
// arrays do not weigh on the other paths.
__device__ __noinline__ void other_tetra(const TetraArgs &a, int code, const double *e1m, const double *e2m, int e0,
                                         int ne, int nec, double2 *xo) {
  const double f = a.efermi, delt = a.delt;
  const int t = code >> 1, sg = code & 1;
  const double dsgn = sg == 0 ? 1.0 : -1.0;
  int slot[4];
  double ee1[4], ee2[4];
  for (int v = 0; v < 4; v++) { slot[v] = a.imt1[4 * t + v]; ee1[v] = e1m[slot[v]]; ee2[v] = e2m[slot[v]]; }
  const double mn2 = fmin(fmin(ee2[0], ee2[1]), fmin(ee2[2], ee2[3]));
  const double mx1 = fmax(fmax(ee1[0], ee1[1]), fmax(ee1[2], ee1[3]));
  if (mn2 > f && mx1 < f) {
    cx ffk[4], ggk[4];
    for (int v = 0; v < 4; v++) {
      ffk[v] = cx(dsgn, 0);
      ggk[v] = cx(-(ee2[v] - ee1[v]), delt) * dsgn;
    }
    if (!tetra_terms(a.dmna, a.dmnr, ffk, ggk, a.em, e0, ne, nec, slot, nullptr, xo)) atomicExch(a.err, 2);
    return;
  }
  double dwgt[TT_NMAX][4][4], dvol[TT_NMAX];
  for (int i = 0; i < 4; i++)
    for (int v = 0; v < 4; v++) dwgt[0][i][v] = (i == v) ? 1.0 : 0.0;
  dvol[0] = 1.0;
  int nt = 1;
  if (!ttct(f, ee2, +1, nt, dwgt, dvol) || !ttct(f, ee1, -1, nt, dwgt, dvol)) { atomicExch(a.err, 1); return; }
  for (int i3 = 0; i3 < nt; i3++) {
    cx ffk[4], ggk[4];
    for (int i4 = 0; i4 < 4; i4++) {
      double sm = 0;
      for (int v = 0; v < 4; v++) sm += (ee2[v] - ee1[v]) * dwgt[i3][i4][v];
      ffk[i4] = cx(dvol[i3], 0) * dsgn;
      ggk[i4] = cx(-sm, delt) * dsgn;
    }
    double w4[4][4];
    for (int i4 = 0; i4 < 4; i4++)
      for (int v = 0; v < 4; v++) w4[i4][v] = dwgt[i3][i4][v];
    if (!tetra_terms(a.dmna, a.dmnr, ffk, ggk, a.em, e0, ne, nec, slot, w4, xo)) atomicExch(a.err, 2);
  }
}

// Tetrahedra are first sorted into shared-memory lists by the work they need --
// normal (the shared-log closed forms), near-degenerate (the reference's special
// forms) and Fermi-cut (ttct) -- so the threads of a warp run the same code.
__global__ void __launch_bounds__(256) tetra_weights_kernel(TetraArgs a, int nec, double2 *__restrict__ wout) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int p = blockIdx.x, e0 = blockIdx.y * nec, ntk = a.ntk;
  const int ne = min(nec, a.nen - e0);
  const int ntet = 6 * ntk;
  double2 *xo = (double2 *)smem;               // ntk * nec
  double2 *Lt = xo + (size_t)ntk * nec;        // [sign][mesh slot][e] log(g + w)
  double *e1m = (double *)(Lt + 2 * (size_t)ntk * nec), *e2m = e1m + ntk;
  int *lists = (int *)(e2m + ntk);             // 2*ntet entries, one segment per category
  unsigned char *tcat = (unsigned char *)(lists + 2 * (size_t)ntet);  // category of each tetrahedron
  __shared__ int ncat[TC_NCAT], cbeg[TC_NCAT + 1], cur[TC_NCAT];
  const int bv = a.pair_vir[p], bo = a.pair_occ[p];
  if (threadIdx.x < TC_NCAT) ncat[threadIdx.x] = 0;
  for (int i = threadIdx.x; i < ntk * nec; i += blockDim.x) xo[i] = make_double2(0, 0);
  for (int m = threadIdx.x; m < ntk; m += blockDim.x) {
    int k = a.index_kpt[m];
    e1m[m] = (double)(float)a.energy[(size_t)a.numirr[k] * a.ntb + bo];
    e2m[m] = (double)(float)a.energy[(size_t)a.numirr[a.kpq[k]] * a.ntb + bv];
  }
  __syncthreads();
  const double f = a.efermi, delt = a.delt;
  // log(g_k + w) per mesh vertex, sign and frequency of the chunk
  for (int i = threadIdx.x; i < 2 * ntk * ne; i += blockDim.x) {
    const int sg = i / (ntk * ne), rem = i % (ntk * ne), m = rem / ne, e = rem % ne;
    const double dsgn = sg == 0 ? 1.0 : -1.0;
    const cx g = cx(-(e2m[m] - e1m[m]), delt) * dsgn;
    const cx z = g + cx(a.em[e0 + e].x, a.em[e0 + e].y);
    const cx L = clog_(z);
    Lt[((size_t)sg * ntk + m) * nec + e] = make_double2(L.r, L.i);
  }
  // classify every tetrahedron.  chk1 sees |g_a - g_b| and |g_a + g_b|, which
  // the sign does not change, so one test covers both signs.
  for (int t = threadIdx.x; t < ntet; t += blockDim.x) {
    double ee1[4], ee2[4];
    for (int v = 0; v < 4; v++) { const int sl = a.imt1[4 * t + v]; ee1[v] = e1m[sl]; ee2[v] = e2m[sl]; }
    const double mn2 = fmin(fmin(ee2[0], ee2[1]), fmin(ee2[2], ee2[3]));
    const double mx2 = fmax(fmax(ee2[0], ee2[1]), fmax(ee2[2], ee2[3]));
    const double mx1 = fmax(fmax(ee1[0], ee1[1]), fmax(ee1[2], ee1[3]));
    int cat = TC_OTHER;
    if (mx2 <= f) {
      cat = TC_SKIP;  // ttct(+1) drops the whole tetrahedron
    } else if (mn2 > f && mx1 < f) {
      cx ggk[4];
      for (int v = 0; v < 4; v++) ggk[v] = cx(-(ee2[v] - ee1[v]), delt);
      const Chk c = chk1(a.dmna, a.dmnr, ggk);
      cat = c.s == 0 ? TC_NORMAL : c.s == 2 ? TC_S2 : c.s == 3 ? TC_S3
          : c.s == 4 && c.i3 == 2 ? TC_S4A : c.s == 4 && c.i3 >= 3 && c.i3 <= 6 ? TC_S4B : TC_OTHER;
    }
    tcat[t] = (unsigned char)cat;
    if (cat != TC_SKIP) atomicAdd(&ncat[cat], 1);
  }
  __syncthreads();
  // segments: the normal tetrahedra once (both signs in one pass), the others once per sign
  if (threadIdx.x == 0) {
    cbeg[0] = 0;
    for (int c = 0; c < TC_NCAT; c++) {
      cbeg[c + 1] = cbeg[c] + ncat[c] * (c == TC_NORMAL ? 1 : 2);
      cur[c] = cbeg[c];
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < ntet; t += blockDim.x) {
    const int cat = tcat[t];
    if (cat == TC_SKIP) continue;
    if (cat == TC_NORMAL) {
      lists[atomicAdd(&cur[cat], 1)] = t;
    } else {
      const int o = atomicAdd(&cur[cat], 2);
      lists[o] = 2 * t;
      lists[o + 1] = 2 * t + 1;
    }
  }
  __syncthreads();
  const int n_normal = ncat[TC_NORMAL];
  // normal tetrahedra: shared logs, real reciprocal differences, both signs
  for (int idx = threadIdx.x; idx < n_normal; idx += blockDim.x) {
    const int t = lists[idx];
    int slot[4];
    double gr[4];
#pragma unroll
    for (int v = 0; v < 4; v++) {
      slot[v] = a.imt1[4 * t + v];
      gr[v] = -(e2m[slot[v]] - e1m[slot[v]]);
    }
    NormalCoef nc;
    normal_coef(gr, nc);
    for (int e = 0; e < ne; e++) {
      const cx w(a.em[e0 + e].x, a.em[e0 + e].y);
      cx acc[4];
#pragma unroll 1
      for (int sg = 0; sg < 2; sg++) {
        const double dsgn = sg == 0 ? 1.0 : -1.0;
        cx x[4];
        if (delt * dsgn + w.i == 0.0) {
          // z on the real axis: keep the ratio logs of the reference
          Chk c;
          c.s = 0; c.i3 = 0;
          c.ia4[0] = 1; c.ia4[1] = 2; c.ia4[2] = 3; c.ia4[3] = 0;
          c.ia3[0] = c.ia3[1] = c.ia3[2] = c.ia3[3] = 0;
          cx ffk[4], ggk[4];
          for (int v = 0; v < 4; v++) { ffk[v] = cx(dsgn, 0); ggk[v] = cx(gr[v], delt) * dsgn; }
          if (!calc_w(c, ffk, ggk, w, x)) { atomicExch(a.err, 2); x[0] = x[1] = x[2] = x[3] = cx(0, 0); }
        } else {
          cx z[4], L[4];
#pragma unroll
          for (int v = 0; v < 4; v++) {
            z[v] = cx(gr[v] * dsgn + w.r, delt * dsgn + w.i);
            const double2 l = Lt[((size_t)sg * ntk + slot[v]) * nec + e];
            L[v] = cx(l.x, l.y);
          }
          normal_terms(nc, dsgn, z, L, x);
        }
#pragma unroll
        for (int v = 0; v < 4; v++) acc[v] = sg == 0 ? x[v] : acc[v] + x[v];
      }
#pragma unroll
      for (int v = 0; v < 4; v++) sadd(&xo[slot[v] * nec + e], acc[v]);
    }
  }
  // near-degenerate tetrahedra, one category at a time so a warp runs one form
  for (int cat = TC_S2; cat <= TC_S4B; cat++)
    for (int idx = cbeg[cat] + threadIdx.x; idx < cbeg[cat + 1]; idx += blockDim.x)
      degen_tetra(a, lists[idx], cat, e1m, e2m, Lt, e0, ne, nec, xo);
  // Fermi-cut tetrahedra and unknown cases: the reference's ttct and forms
  for (int idx = cbeg[TC_OTHER] + threadIdx.x; idx < cbeg[TC_OTHER + 1]; idx += blockDim.x)
    other_tetra(a, lists[idx], e1m, e2m, e0, ne, nec, xo);
  __syncthreads();
  // w[(p*nen + e)*ntk + k] = xow(mesh(k), e) * (1 - P_occ(bo,k) P_vir(bv,k+q)) / NTK
  for (int i = threadIdx.x; i < ntk * ne; i += blockDim.x) {
    const int e = i / ntk, k = i % ntk;
    const int m = a.index_kpt[ntk + k];  // second half holds k -> mesh slot
    double2 x = xo[(size_t)m * nec + e];
    double2 po = a.prob[(size_t)k * a.ntb + bo], pv = a.prob[(size_t)a.kpq[k] * a.ntb + bv];
    double2 pp = make_double2(1.0 - (po.x * pv.x - po.y * pv.y), -(po.x * pv.y + po.y * pv.x));
    double2 r = cmul(x, pp);
    wout[((size_t)p * a.nen + e0 + e) * ntk + k] = make_double2(r.x / (double)ntk, r.y / (double)ntk);
  }
}

// ---------------------------------------------------------------------------
// Split-precision path: the FP32 series of rp_tetra_series.cuh for every
// uncut tetrahedron where it converges, gathered per mesh vertex.
//
// Every tetrahedron is classified once, as the reference's calc() does (chk1:
// normal, or near-degenerate with some vertices replaced by their average,
// m_tetrahedron_20170325.F:209-302, 457-503), and its points' mean (a float
// pair) and deviations (FP32) go to shared memory.  Then one thread per (mesh
// slot, frequency) walks the tetrahedra that touch the slot (24 on a cubic
// mesh) and sums its vertex's weight over them and both signs in float pairs:
// no FP64 and no atomics in the hot loop, one fixed summation order.  The
// weight is the confluent divided difference of the tetrahedron's (averaged)
// points -- the quantity the reference's closed forms (:304-451) evaluate.
// For each (tetrahedron, sign, frequency) where the series does not converge
// (r > 1/2, near resonance: the Lindhard denominators of near-degenerate band
// pairs) a second pass, over a compacted list, runs the reference's closed
// forms in FP64 once for all four vertices and adds them to the outputs with
// FP64 atomics.  Tetrahedra cut by the Fermi level take ttct and the closed
// forms in FP64 (other_tetra) with shared-memory sums; they exist only when a
// band is partially occupied.

// A tetrahedron's code: its category in the low byte, then for each vertex
// position (2 bits each) the position whose point it takes -- the first member
// of its group of near-degenerate vertices, which share their average.
__device__ __forceinline__ unsigned short tetra_code(int cat, const Chk &c) {
  int rep[4] = {0, 1, 2, 3};
  if (cat == TC_S2) {
    rep[c.ia3[1]] = c.ia3[0];
  } else if (cat == TC_S3) {
    rep[c.ia3[1]] = c.ia3[0];
    rep[c.ia3[2]] = c.ia3[0];
  } else if (cat == TC_S4A) {
    rep[c.ia3[1]] = c.ia3[0];
    rep[c.ia3[3]] = c.ia3[2];
  } else if (cat == TC_S4B) {
    rep[c.ia3[1]] = rep[c.ia3[2]] = rep[c.ia3[3]] = c.ia3[0];
  }
  return (unsigned short)(cat | (rep[0] << 8) | (rep[1] << 10) | (rep[2] << 12) | (rep[3] << 14));
}

// the points of calc(): each vertex's value, or its group's average (:243-296)
__device__ __forceinline__ void tetra_points(unsigned code, const double (&gr)[4], double (&gp)[4]) {
  const double inv[5] = {0.0, 1.0, 0.5, 1.0 / 3.0, 0.25};
#pragma unroll
  for (int v = 0; v < 4; v++) {
    const unsigned rv = (code >> (8 + 2 * v)) & 3u;
    double s = 0.0;
    int n = 0;
#pragma unroll
    for (int u = 0; u < 4; u++)
      if (((code >> (8 + 2 * u)) & 3u) == rv) { s += gr[u]; n++; }
    gp[v] = n == 1 ? s : s * inv[n];
  }
}

// all four vertex weights of tetrahedron t by the reference's closed forms for
// one sign (fk = dsgn) at frequency w, FP64
__device__ __noinline__ bool closed_form_tetra(const TetraArgs &a, int t, const double *e1m, const double *e2m,
                                               double dsgn, double wr, double wi, cx (&x)[4]) {
  cx ffk[4], ggk[4];
  for (int v = 0; v < 4; v++) {
    const int sl = a.imt1[4 * t + v];
    ffk[v] = cx(dsgn, 0);
    ggk[v] = cx(-(e2m[sl] - e1m[sl]), a.delt) * dsgn;
  }
  const Chk c = chk1(a.dmna, a.dmnr, ggk);
  return calc_w(c, ffk, ggk, cx(wr, wi), x);
}

// (1 - P_occ(bo,k) P_vir(bv,k+q)) / NTK of mesh slot m
__device__ __forceinline__ double2 occ_factor(const TetraArgs &a, int m, int bo, int bv) {
  const int k = a.index_kpt[m];
  const double2 po = a.prob[(size_t)k * a.ntb + bo], pv = a.prob[(size_t)a.kpq[k] * a.ntb + bv];
  const double s = 1.0 / (double)a.ntk;
  return make_double2((1.0 - (po.x * pv.x - po.y * pv.y)) * s, -(po.x * pv.y + po.y * pv.x) * s);
}

// s += v for a float pair s = (h, l) (TwoSum of the heads, tails summed)
__device__ __forceinline__ void pair_acc(float &h, float &l, float v) {
  const float t = h + v;
  const float bp = t - h;
  l += (h - (t - bp)) + (v - bp);
  h = t;
}

// the fallback list of one pass: entries 2 * item + sign, items (e, t) with
// item = e * ntet + t
#define TS_FB_CAP 4096

// two CTAs per SM: the smem of a 512-k mesh allows two, and the register cap
// leaves the hot gather loop unspilled
__global__ void __launch_bounds__(256, 2) tetra_series_kernel(TetraArgs a, int nec, double2 *__restrict__ wout) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int p = blockIdx.x, e0 = blockIdx.y * nec, ntk = a.ntk;
  const int ne = min(nec, a.nen - e0);
  const int ntet = 6 * ntk;
  // per tetrahedron: the FP32 deviations d of its points from their mean, the
  // mean as a float pair and the code; per slot the pair's energies; per
  // frequency w as float pairs; the fallback list; for metals the sums of the
  // cut tetrahedra and their list
  float4 *td = (float4 *)smem;
  float2 *tm = (float2 *)(td + ntet);
  double *e1m = (double *)(tm + ntet), *e2m = e1m + ntk;
  float4 *wsp = (float4 *)(e2m + ntk);
  double2 *xo = (double2 *)(wsp + nec);
  int *olist = (int *)(xo + (a.may_cut ? (size_t)ntk * nec : 0));
  int *fbl = olist + (a.may_cut ? 2 * (size_t)ntet : 0);
  unsigned short *tcode = (unsigned short *)(fbl + TS_FB_CAP);
  __shared__ int ncut, nfb;
  const int bv = a.pair_vir[p], bo = a.pair_occ[p];
  if (threadIdx.x == 0) ncut = 0;
  for (int m = threadIdx.x; m < ntk; m += blockDim.x) {
    const int k = a.index_kpt[m];
    e1m[m] = (double)(float)a.energy[(size_t)a.numirr[k] * a.ntb + bo];
    e2m[m] = (double)(float)a.energy[(size_t)a.numirr[a.kpq[k]] * a.ntb + bv];
  }
  for (int e = threadIdx.x; e < ne; e += blockDim.x) {
    const double2 w = a.em[e0 + e];
    float4 f;
    ts_split(w.x, f.x, f.y);
    ts_split(w.y, f.z, f.w);
    wsp[e] = f;
  }
  if (a.may_cut)
    for (int i = threadIdx.x; i < ntk * nec; i += blockDim.x) xo[i] = make_double2(0, 0);
  __syncthreads();
  const double f = a.efermi, delt = a.delt;
  float dh, dl;
  ts_split(delt, dh, dl);
  // classify every tetrahedron (chk1 sees |g_a - g_b| and |g_a + g_b|, which the
  // sign does not change, so one test covers both signs) and keep its points
  for (int t = threadIdx.x; t < ntet; t += blockDim.x) {
    double ee1[4], ee2[4];
    for (int v = 0; v < 4; v++) { const int sl = a.imt1[4 * t + v]; ee1[v] = e1m[sl]; ee2[v] = e2m[sl]; }
    const double mn2 = fmin(fmin(ee2[0], ee2[1]), fmin(ee2[2], ee2[3]));
    const double mx2 = fmax(fmax(ee2[0], ee2[1]), fmax(ee2[2], ee2[3]));
    const double mx1 = fmax(fmax(ee1[0], ee1[1]), fmax(ee1[2], ee1[3]));
    unsigned short code = TC_OTHER;
    if (mx2 <= f) {
      code = TC_SKIP;  // ttct(+1) drops the whole tetrahedron
    } else if (mn2 > f && mx1 < f) {
      cx ggk[4];
      double gr[4];
      for (int v = 0; v < 4; v++) {
        gr[v] = -(ee2[v] - ee1[v]);
        ggk[v] = cx(gr[v], delt);
      }
      const Chk c = chk1(a.dmna, a.dmnr, ggk);
      const int cat = c.s == 0 ? TC_NORMAL : c.s == 2 ? TC_S2 : c.s == 3 ? TC_S3
                    : c.s == 4 && c.i3 == 2 ? TC_S4A : c.s == 4 && c.i3 >= 3 && c.i3 <= 6 ? TC_S4B : TC_OTHER;
      if (cat != TC_OTHER) {
        code = tetra_code(cat, c);
        double gp[4];
        tetra_points(code, gr, gp);
        const double mean = 0.25 * ((gp[0] + gp[1]) + (gp[2] + gp[3]));
        float2 mp;
        ts_split(mean, mp.x, mp.y);
        tm[t] = mp;
        td[t] = make_float4((float)(gp[0] - mean), (float)(gp[1] - mean), (float)(gp[2] - mean), (float)(gp[3] - mean));
      }
    }
    tcode[t] = code;
    if (code == TC_OTHER) {
      if (a.may_cut) {
        const int o = atomicAdd(&ncut, 2);
        olist[o] = 2 * t;
        olist[o + 1] = 2 * t + 1;
      } else {
        atomicExch(a.err, 5);  // a cut tetrahedron although no band is partially occupied
      }
    }
  }
  __syncthreads();
  if (a.may_cut) {
    for (int idx = threadIdx.x; idx < ncut; idx += blockDim.x) other_tetra(a, olist[idx], e1m, e2m, e0, ne, nec, xo);
    __syncthreads();
  }
  // one thread per (slot, frequency): the slot's vertex weight summed over the
  // tetrahedra around it and both signs, in FP32 with float-pair sums
  for (int it = threadIdx.x; it < ntk * ne; it += blockDim.x) {
    const int m = it % ntk, e = it / ntk;
    const float4 w = wsp[e];
    float arh = 0.f, arl = 0.f, aih = 0.f, ail = 0.f;
    const int j1 = __ldg(a.inc_off + m + 1);
    for (int j = __ldg(a.inc_off + m); j < j1; j++) {
      const int ent = __ldg(a.inc + j), t = ent >> 2, pos = ent & 3;
      const int cat = tcode[t] & 0xff;
      if (cat == TC_SKIP || cat == TC_OTHER) continue;
      const float4 d4 = td[t];
      const float2 mp = tm[t];
      const float d[4] = {d4.x, d4.y, d4.z, d4.w};
      const float dmax = fmaxf(fmaxf(fabsf(d4.x), fabsf(d4.y)), fmaxf(fabsf(d4.z), fabsf(d4.w)));
      const float dv = pos == 0 ? d4.x : pos == 1 ? d4.y : pos == 2 ? d4.z : d4.w;
      float zr[2], zi[2], inv[2];
      bool ok[2];
      ts_z(w.x, w.y, w.z, w.w, mp.x, mp.y, dh, dl, dmax, zr, zi, ok, inv);
      TsCplx x[2];
      tetra_series_core(d, dv, dmax, zr, zi, ok, inv, x);
      // fk = dsgn: the sign -1 enters negated
      pair_acc(arh, arl, x[0].r - x[1].r);
      pair_acc(aih, ail, x[0].i - x[1].i);
    }
    const int k = a.index_kpt[m];
    const double2 pp = occ_factor(a, m, bo, bv);
    double2 x = make_double2((double)arh + (double)arl, (double)aih + (double)ail);
    if (a.may_cut) x = cadd(x, xo[(size_t)m * nec + e]);
    // w[(p*nen + e)*ntk + k] = xow(m, e) * (1 - P_occ(bo,k) P_vir(bv,k+q)) / NTK
    wout[((size_t)p * a.nen + e0 + e) * ntk + k] = cmul(x, pp);
  }
  __syncthreads();
  // the (tetrahedron, sign, frequency) where the series was not taken (the same
  // decision, from the same float inputs): the closed forms in FP64 for all
  // four vertices at once, added to the CTA's own outputs
  const int nitem = ntet * ne;
  for (int base = 0; base < nitem; base += TS_FB_CAP / 2) {
    if (threadIdx.x == 0) nfb = 0;
    __syncthreads();
    const int iend = min(nitem, base + TS_FB_CAP / 2);
    for (int i = base + threadIdx.x; i < iend; i += blockDim.x) {
      const int t = i % ntet, e = i / ntet;
      const int cat = tcode[t] & 0xff;
      if (cat == TC_SKIP || cat == TC_OTHER) continue;
      const float4 d4 = td[t];
      const float2 mp = tm[t];
      const float4 w = wsp[e];
      const float dmax = fmaxf(fmaxf(fabsf(d4.x), fabsf(d4.y)), fmaxf(fabsf(d4.z), fabsf(d4.w)));
      float zr[2], zi[2], inv[2];
      bool ok[2];
      ts_z(w.x, w.y, w.z, w.w, mp.x, mp.y, dh, dl, dmax, zr, zi, ok, inv);
      for (int sg = 0; sg < 2; sg++)
        if (!ok[sg]) fbl[atomicAdd(&nfb, 1)] = 2 * i + sg;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nfb; j += blockDim.x) {
      const int ent = fbl[j], i = ent >> 1, sg = ent & 1;
      const int t = i % ntet, e = i / ntet;
      const double2 w = a.em[e0 + e];
      cx x[4];
      if (!closed_form_tetra(a, t, e1m, e2m, sg ? -1.0 : 1.0, w.x, w.y, x)) {
        atomicExch(a.err, 2);
        continue;
      }
      for (int v = 0; v < 4; v++) {
        const int m = a.imt1[4 * t + v];
        const double2 r = cmul(make_double2(x[v].r, x[v].i), occ_factor(a, m, bo, bv));
        double2 *o = wout + ((size_t)p * a.nen + e0 + e) * ntk + a.index_kpt[m];
        atomicAdd(&o->x, r.x);
        atomicAdd(&o->y, r.y);
      }
    }
    __syncthreads();
  }
}

int launch_tetra_weights(const TetraArgs &a, double2 *w, cudaStream_t st, bool series) {
  if (a.npair == 0) return 0;
  if (series) {
    if (!a.inc_off || !a.inc) fail(1, "tetrahedron series kernel: no vertex incidence lists");
    // the tetrahedra's deviations, means and codes, e1m and e2m, the fallback
    // list, plus for metals the cut-tetrahedron list and the sums of a
    // frequency chunk; per frequency its float pairs
    const size_t ntk = (size_t)a.ntk, ntet = 6 * ntk;
    const size_t fixed = (sizeof(float4) + sizeof(float2) + sizeof(unsigned short)) * ntet + 2 * sizeof(double) * ntk +
                         sizeof(int) * TS_FB_CAP + (a.may_cut ? 2 * sizeof(int) * ntet : 0);
    const size_t per_e = sizeof(float4) + (a.may_cut ? sizeof(double2) * ntk : 0);
    int nec = a.nen;
    while (nec > 1 && fixed + per_e * nec > 210 * 1024) nec--;
    const size_t smem = fixed + per_e * nec;
    if (smem > 227 * 1024) fail(1, "k mesh too large for the tetrahedron tile (%zu bytes)", smem);
    RP_CUDA(cudaFuncSetAttribute(tetra_series_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem_cap(tetra_series_kernel)));
    dim3 grid(a.npair, (a.nen + nec - 1) / nec);
    tetra_series_kernel<<<grid, 256, smem, st>>>(a, nec, w);
    RP_CUDA(cudaGetLastError());
    return 1;
  }
  // weights (ntk x nec) and vertex logs (2 x ntk x nec) of a frequency chunk in shared memory
  int nec = a.nen;
  const size_t fixed = 2 * sizeof(double) * (size_t)a.ntk + 2 * 6 * sizeof(int) * (size_t)a.ntk + 6 * (size_t)a.ntk;
  const size_t budget = 210 * 1024 - fixed;
  while (nec > 1 && (size_t)a.ntk * nec * 3 * sizeof(double2) > budget) nec--;
  size_t smem = (size_t)a.ntk * nec * 3 * sizeof(double2) + fixed;
  if (smem > 227 * 1024) fail(1, "k mesh too large for the tetrahedron tile (%zu bytes)", smem);
  RP_CUDA(cudaFuncSetAttribute(tetra_weights_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_cap(tetra_weights_kernel)));
  dim3 grid(a.npair, (a.nen + nec - 1) / nec);
  tetra_weights_kernel<<<grid, 256, smem, st>>>(a, nec, w);
  RP_CUDA(cudaGetLastError());
  return 1;
}

// ---------------------------------------------------------------------------
// Intraband plasma frequency at Gamma for metals (chiqw.F:1639-1733): for each
// partially occupied band b, pk(k) = sum_G (k+G) |C_b(k,G)|^2 (calc_VMaa) and
// xo = ttrhdrn_simple(fk=1, gk = E_b(k) - E_F - i delt) at w = 0;
// pwpl += Im(xo) pk^2.
__global__ void __launch_bounds__(256) intraband_kernel(TetraArgs a, const double2 *__restrict__ cfull,
                                                        const int *__restrict__ ng0, const int *__restrict__ kg0,
                                                        int ncb, int ntg, const double *__restrict__ b9,
                                                        const double *__restrict__ sk0, const int *__restrict__ bands,
                                                        double2 *__restrict__ pwpl) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int ntk = a.ntk, b = bands[blockIdx.x];
  double2 *xo = (double2 *)smem;           // ntk (mesh slots)
  double *pk = (double *)(xo + ntk);       // 3*ntk (by k)
  cx *gk = (cx *)(pk + 3 * ntk);           // ntk (mesh slots)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int m = threadIdx.x; m < ntk; m += blockDim.x) {
    xo[m] = make_double2(0, 0);
    int k = a.index_kpt[m];
    double e = a.energy[(size_t)a.numirr[k] * a.ntb + b] - a.efermi;
    gk[m] = cx((double)(float)e, (double)(float)(-a.delt));
  }
  for (int k = warp; k < ntk; k += nw) {
    double s[3] = {0, 0, 0};
    const double2 *c = cfull + ((size_t)k * ncb + b) * ntg;
    for (int ig = lane; ig < ng0[k]; ig += 32) {
      const int *g = kg0 + ((size_t)k * ntg + ig) * 3;
      double w = c[ig].x * c[ig].x + c[ig].y * c[ig].y;
      for (int d = 0; d < 3; d++) {
        double G = (sk0[3 * k] + g[0]) * b9[d] + (sk0[3 * k + 1] + g[1]) * b9[3 + d] + (sk0[3 * k + 2] + g[2]) * b9[6 + d];
        s[d] += G * w;
      }
    }
    for (int d = 0; d < 3; d++)
      for (int o = 16; o; o >>= 1) s[d] += __shfl_xor_sync(0xffffffffu, s[d], o);
    if (lane == 0)
      for (int d = 0; d < 3; d++) pk[3 * k + d] = s[d];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < 6 * ntk; t += blockDim.x) {
    int slot[4];
    cx ffk[4], ggk[4];
    for (int v = 0; v < 4; v++) { slot[v] = a.imt1[4 * t + v]; ffk[v] = cx(1, 0); ggk[v] = gk[slot[v]]; }
    Chk c = chk1(a.dmna, a.dmnr, ggk);
    cx x[4];
    if (!calc_w(c, ffk, ggk, cx(0, 0), x)) { atomicExch(a.err, 2); continue; }
    for (int v = 0; v < 4; v++) sadd(&xo[slot[v]], x[v]);
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    const int d = threadIdx.x;
    double s = 0;
    for (int m = 0; m < ntk; m++) {
      int k = a.index_kpt[m];
      s += xo[m].y * pk[3 * k + d] * pk[3 * k + d];
    }
    atomicAdd(&pwpl[d].x, s);
  }
}

int launch_intraband(const TetraArgs &a, const double2 *cfull, const int *ng0, const int *kg0, int ncb, int ntg,
                     const double *bvec9, const double *sk0, const int *bands, int nb, double2 *pwpl,
                     cudaStream_t st) {
  if (nb == 0) return 0;
  size_t smem = (size_t)a.ntk * (sizeof(double2) + 3 * sizeof(double) + sizeof(cx));
  if (smem > 227 * 1024) fail(1, "k mesh too large for the intraband tile");
  RP_CUDA(cudaFuncSetAttribute(intraband_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_cap(intraband_kernel)));
  intraband_kernel<<<nb, 256, smem, st>>>(a, cfull, ng0, kg0, ncb, ntg, bvec9, sk0, bands, pwpl);
  RP_CUDA(cudaGetLastError());
  return 1;
}

}  // namespace rp
