// rp_setup.cpp -- host setup of a calc_chiqw run.
//
// Restates (file:line of RESPACK's src/chiqw):
//   readers                      chiqw.F:87-329, :870-906, :1100-1160
//   Ecut_for_psi / eps defaults  chiqw.F:331-352
//   FFT grid rule                chiqw.F:389-416, est_nwx2.f90:1-41
//   unfolding (est_NTK + loop)   est_NTK.f90:42-98, chiqw.F:419-545, kcheck(_trs) chiqw_sub.F:668-771
//   mesh size, index_kpt         est_NTK.f90:1-39, chiqw_sub.F:324-384
//   q list + resume              chiqw.F:587-655 ; search_list chiqw_sub.F:77-95
//   eps G sphere                 make_KG0 chiqw_sub.F:773-812 (same triple-loop order)
//   k+q map                      search_kq chiqw_sub.F:1-75
//   band classification, pairs   judge_FermiInside chiqw_sub.F:570-613, chiqw.F:943-967,
//                                :1270-1294 (q != 0), :1589-1629 (Gamma)
//   frequency grid               gen_grid.f90:1-39
//   tetrahedra                   libtetrabzinitialize m_tetrahedron_20170325.F:523-584
//   make_C0 map                  chiqw_sub.F:264-322
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "rp_host.h"

namespace rp {

static void cross(const double *x, const double *y, double *z) {
  z[0] = x[1] * y[2] - x[2] * y[1];
  z[1] = x[2] * y[0] - x[0] * y[2];
  z[2] = x[0] * y[1] - x[1] * y[0];
}

int algn235(int n) {
  auto bad = [](int v) {
    while (v != 1) {
      if (v % 2 == 0) v /= 2;
      else if (v % 3 == 0) v /= 3;
      else if (v % 5 == 0) v /= 5;
      else return true;
    }
    return false;
  };
  while (bad(n)) n++;
  return n;
}

void gen_grid(int nt, double e, std::vector<cd> &em) {
  em.assign(nt, cd(0, 0));
  if (nt == 1) return;
  const double dlt = 0.05 / kAu, ratio = 0.1, eps = 1.0e-6;
  int m = (int)(ratio * (double)nt), n = nt - m;
  double alp = e / dlt, x = 1.5, dl = 1.0;
  while (dl > eps) {
    double f = std::pow(x, n - 1) - alp * x + alp - 1.0;
    double g = (double)(n - 1) * std::pow(x, n - 2) - alp;
    double x1 = x - f / g;
    dl = std::fabs(x1 - x);
    x = x1;
  }
  double a = dlt / (x - 1.0), b = std::log(x);
  for (int i = 1; i <= n; i++) em[i - 1] = cd(a * std::exp(b * (double)(i - 1)) - a, 0);
  double c = e * std::exp(-std::log(2.0) * (double)n / (double)m), d = std::log(2.0) / (double)m;
  for (int i = n + 1; i <= n + m; i++) em[i - 1] = cd(c * std::exp(d * (double)i), 0);
}

void search_list(const double *in, double *sq) {
  const double d = 1.0e-6;
  for (int i = 0; i < 3; i++) sq[i] = in[i];
  for (int i = 0; i < 2; i++) {
    if (sq[i] > 1.5 + d) sq[i] -= 2.0;
    if (sq[i] > 0.5 + d) sq[i] -= 1.0;
    if (sq[i] <= -1.5 + d) sq[i] += 2.0;
    if (sq[i] <= -0.5 + d) sq[i] += 1.0;
  }
  // the reference tests the third component at -0.5 before -1.5
  if (sq[2] > 1.5 + d) sq[2] -= 2.0;
  if (sq[2] > 0.5 + d) sq[2] -= 1.0;
  if (sq[2] <= -0.5 + d) sq[2] += 1.0;
  if (sq[2] <= -1.5 + d) sq[2] += 2.0;
}

static void kcheck(double *k, int *rw, bool trs) {
  for (int i = 0; i < 3; i++) {
    if (!trs) {
      const double d = 1.0e-6;
      if (k[i] > 1.5 + d) { k[i] -= 2.0; rw[i] = -2; }
      if (k[i] > 0.5 + d) { k[i] -= 1.0; rw[i] = -1; }
      if (k[i] <= -1.5 + d) { k[i] += 2.0; rw[i] = 2; }
      if (k[i] <= -0.5 + d) { k[i] += 1.0; rw[i] = 1; }
    } else {
      const double d = -1.0e-6;
      if (k[i] >= 1.5 + d) { k[i] -= 2.0; rw[i] = -2; }
      if (k[i] >= 0.5 + d) { k[i] -= 1.0; rw[i] = -1; }
      if (k[i] < -1.5 + d) { k[i] += 2.0; rw[i] = 2; }
      if (k[i] < -0.5 + d) { k[i] += 1.0; rw[i] = 1; }
    }
  }
}

// make_KG0: points with |q+G|^2 <= gcut in the igL1-outer order.  The reference
// scans -100..100; the scan is narrowed to indices that can pass the cutoff.
void make_kg0(const double b[3][3], double gcut, const double q[3], int ntg_max, std::vector<int> &kg, int &ng) {
  int lim[3];
  for (int i = 0; i < 3; i++) {
    double c[3];
    cross(b[(i + 1) % 3], b[(i + 2) % 3], c);
    double vol = b[i][0] * c[0] + b[i][1] * c[1] + b[i][2] * c[2];
    double alen = kTpi * std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) / std::fabs(vol);
    lim[i] = std::min(100, (int)(std::sqrt(gcut) * alen / kTpi + std::fabs(q[i])) + 2);
  }
  kg.clear();
  ng = 0;
  for (int i1 = -lim[0]; i1 <= lim[0]; i1++)
    for (int i2 = -lim[1]; i2 <= lim[1]; i2++)
      for (int i3 = -lim[2]; i3 <= lim[2]; i3++) {
        double g[3];
        for (int d = 0; d < 3; d++)
          g[d] = (q[0] + i1) * b[0][d] + (q[1] + i2) * b[1][d] + (q[2] + i3) * b[2][d];
        if (g[0] * g[0] + g[1] * g[1] + g[2] * g[2] <= gcut) {
          if (ntg_max > 0 && ng >= ntg_max) fail(1, "make_KG0: more than NTG=%d points", ntg_max);
          kg.push_back(i1); kg.push_back(i2); kg.push_back(i3);
          ng++;
        }
      }
}

void read_dir_wfn(Setup &s, const std::string &root) {
  const std::string d = root + "/dir-wfn/";
  {
    ListReader r(d + "dat.bandcalc");
    s.ecut_psi = r.read_real();
    s.efermi = r.read_real();
  }
  {
    ListReader r(d + "dat.lattice");
    for (int i = 0; i < 3; i++) r.read(3, s.a[i]);
  }
  double c[3];
  cross(s.a[1], s.a[2], c);
  s.volume = s.a[0][0] * c[0] + s.a[0][1] * c[1] + s.a[0][2] * c[2];
  for (int i = 0; i < 3; i++) {
    cross(s.a[(i + 1) % 3], s.a[(i + 2) % 3], s.b[i]);
    for (int d2 = 0; d2 < 3; d2++) s.b[i][d2] = s.b[i][d2] * kTpi / s.volume;
  }
  {
    ListReader r(d + "dat.symmetry");
    s.nsymq = r.read_int();
    s.nnp = r.read_int();
    s.rg.resize(9 * s.nsymq);
    s.pg.resize(3 * s.nsymq);
    s.rginv.resize(9 * s.nsymq);
    for (int iop = 0; iop < s.nsymq; iop++) {
      auto m = r.read_ints(9);
      auto t = r.read_ints(3);
      std::copy(m.begin(), m.end(), s.rg.begin() + 9 * iop);
      std::copy(t.begin(), t.end(), s.pg.begin() + 3 * iop);
      // inverse via the adjugate (exact for the unimodular integer rotations; inv.F90)
      const int *R = &s.rg[9 * iop];
      double A = R[0], B = R[3], C = R[6], D = R[1], E = R[4], F = R[7], G = R[2], H = R[5], K = R[8];
      double det = A * (E * K - F * H) - B * (D * K - F * G) + C * (D * H - E * G);
      if (det == 0) fail(1, "dat.symmetry: singular rotation %d", iop + 1);
      double inv[9] = {(E * K - F * H), -(B * K - C * H), (B * F - C * E),
                       -(D * K - F * G), (A * K - C * G), -(A * F - C * D),
                       (D * H - E * G), -(A * H - B * G), (A * E - B * D)};
      for (int rr = 0; rr < 3; rr++)
        for (int cc = 0; cc < 3; cc++) s.rginv[9 * iop + rr + 3 * cc] = inv[3 * rr + cc] / det;
    }
  }
  {
    ListReader r(d + "dat.sample-k");
    s.nk_irr = r.read_int();
    s.ski.resize(3 * s.nk_irr);
    s.ski_list.resize(3 * s.nk_irr);
    for (int ik = 0; ik < s.nk_irr; ik++) {
      r.read(3, &s.ski[3 * ik]);
      search_list(&s.ski[3 * ik], &s.ski_list[3 * ik]);
    }
  }
  {
    ListReader r(d + "dat.nkm");
    s.ngi.resize(s.nk_irr);
    s.ntg = 0;
    for (int ik = 0; ik < s.nk_irr; ik++) {
      s.ngi[ik] = r.read_int();
      s.ntg = std::max(s.ntg, std::abs(s.ngi[ik]));
    }
  }
  {
    ListReader r(d + "dat.eigenvalue");
    s.ntb = r.read_int();
    s.e_eigi.resize((size_t)s.ntb * s.nk_irr);
    for (int ik = 0; ik < s.nk_irr; ik++)
      for (int ib = 0; ib < s.ntb; ib++) s.e_eigi[(size_t)ik * s.ntb + ib] = r.read_real();
  }
  {
    ListReader r(d + "dat.kg");
    s.kgi.assign((size_t)3 * s.ntg * s.nk_irr, 0);
    for (int ik = 0; ik < s.nk_irr; ik++) {
      int ng = r.read_int();
      if (ng != s.ngi[ik]) fail(1, "ERROR;STOP;NG_for_psi should be NGI(ik): k %d has %d and %d", ik + 1, ng, s.ngi[ik]);
      for (int ig = 0; ig < ng; ig++) {
        auto g = r.read_ints(3);
        for (int dd = 0; dd < 3; dd++) s.kgi[((size_t)ik * s.ntg + ig) * 3 + dd] = g[dd];
      }
    }
  }
}

void read_dir_wan_crpa(Setup &s, const std::string &root) {
  std::vector<int> ns(s.ntk), nb(s.ntk);
  {
    ListReader r(root + "/dir-wan/dat.ns-nb");
    for (int ik = 0; ik < s.ntk; ik++) {
      auto t = r.read_ints(2);
      ns[ik] = t[0];
      nb[ik] = t[1];
    }
  }
  ListReader r(root + "/dir-wan/dat.umat");
  int nwf = r.read_int();
  std::vector<double> row(2 * nwf);
  for (int ik = 0; ik < s.ntk; ik++)
    for (int jb = 0; jb < nb[ik]; jb++) {
      r.read(2 * nwf, row.data());
      cd sum(0, 0);
      for (int iw = 0; iw < nwf; iw++) {
        cd u(row[2 * iw], row[2 * iw + 1]);
        sum += std::conj(u) * u;
      }
      int band = ns[ik] + jb;
      if (band < 0 || band >= s.ntb) fail(1, "dat.ns-nb: band %d out of range", band + 1);
      s.prob[(size_t)ik * s.ntb + band] = sum;
    }
}

void read_wfn_coefficients(Setup &s, const std::string &root) {
  UnformattedReader f(root + "/dir-wfn/dat.wfn");
  int ncomp = 0;
  f.read(&ncomp, 4);
  if (ncomp != 1) fail(1, "This program not suport ncomp/=1; then stop");
  s.coef.assign((size_t)s.nk_irr * s.ncb * s.ntg, cd(0, 0));
  for (int ik = 0; ik < s.nk_irr; ik++)
    for (int ib = 0; ib < s.ntb; ib++) {
      if (ib < s.ncb) {
        size_t len = f.read(&s.coef[((size_t)ik * s.ncb + ib) * s.ntg], sizeof(cd) * s.ngi[ik]);
        if (len < sizeof(cd) * (size_t)s.ngi[ik]) fail(1, "dat.wfn: short record at k %d band %d", ik + 1, ib + 1);
      } else {
        f.read(nullptr, 0);
      }
    }
}

void finish_setup(Setup &s, const std::vector<double> &explicit_em) {
  const rp_params &P = s.params;
  s.efermi += P.shift_ef / kAu;
  s.ncb = P.n_calc_band > 0 ? P.n_calc_band : s.ntb;
  if (s.ncb > s.ntb) fail(1, "N_CALC_BAND (%d) > NTB (%d)", s.ncb, s.ntb);
  // Ecut_psi from the plane-wave lists
  double mx = 0;
  for (int ik = 0; ik < s.nk_irr; ik++)
    for (int ig = 0; ig < s.ngi[ik]; ig++) {
      const int *g = &s.kgi[((size_t)ik * s.ntg + ig) * 3];
      double k[3];
      for (int d = 0; d < 3; d++)
        k[d] = (s.ski[3 * ik] + g[0]) * s.b[0][d] + (s.ski[3 * ik + 1] + g[1]) * s.b[1][d] +
               (s.ski[3 * ik + 2] + g[2]) * s.b[2][d];
      double l = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
      if ((ik == 0 && ig == 0) || l > mx) mx = l;
    }
  s.ecut_psi = mx + 1.0e-8;
  s.ecut_eps = P.ecut_for_eps != 0.0 ? P.ecut_for_eps : s.ecut_psi / 10.0;
  // packing
  for (int d = 0; d < 3; d++) s.L[d] = 0;
  for (size_t i = 0; i < (size_t)s.nk_irr * s.ntg; i++)
    for (int d = 0; d < 3; d++) s.L[d] = std::max(s.L[d], std::abs(s.kgi[3 * i + d]));
  for (int d = 0; d < 3; d++) s.L[d]++;
  const int p1 = 2 * s.L[0] + 1, p2 = 2 * s.L[1] + 1, p3 = 2 * s.L[2] + 1;
  s.packing.assign((size_t)p1 * p2 * p3 * s.nk_irr, 0);
  for (int ik = 0; ik < s.nk_irr; ik++)
    for (int ig = 0; ig < s.ngi[ik]; ig++) {
      const int *g = &s.kgi[((size_t)ik * s.ntg + ig) * 3];
      s.packing[(size_t)ik * p1 * p2 * p3 + (g[0] + s.L[0]) + (size_t)p1 * ((g[1] + s.L[1]) + (size_t)p2 * (g[2] + s.L[2]))] = ig + 1;
    }
  // FFT grid
  if (P.fft_box[0] > 0) {
    for (int i = 0; i < 3; i++) s.nw[i] = P.fft_box[i];
  } else {
    double qwf = 2.0 * std::sqrt(s.ecut_psi);
    for (int i = 0; i < 3; i++) {
      double h = std::sqrt(s.a[i][0] * s.a[i][0] + s.a[i][1] * s.a[i][1] + s.a[i][2] * s.a[i][2]);
      double dd = std::fabs(s.b[i][0] * s.a[i][0] / h + s.b[i][1] * s.a[i][1] / h + s.b[i][2] * s.a[i][2] / h);
      s.nw[i] = algn235((int)(qwf / dd) + 1);
    }
  }
  // unfold
  s.sk0.clear(); s.numirr.clear(); s.numrot.clear(); s.trs.clear(); s.rw.clear();
  for (int ik = 0; ik < s.nk_irr; ik++)
    for (int iop = 0; iop < s.nsymq; iop++) {
      const int *R = &s.rg[9 * iop];
      const double *k = &s.ski[3 * ik];
      for (int pass = 0; pass < 2; pass++) {
        double kt[3];
        int rwt[3] = {0, 0, 0};
        for (int i = 0; i < 3; i++) kt[i] = (double)R[i] * k[0] + (double)R[i + 3] * k[1] + (double)R[i + 6] * k[2];
        kcheck(kt, rwt, pass == 1);
        const double sg = pass == 0 ? 1.0 : -1.0;
        bool dup = false;
        for (size_t j = 0; j < s.sk0.size() / 3 && !dup; j++)
          dup = std::fabs(s.sk0[3 * j] - sg * kt[0]) < 1e-4 && std::fabs(s.sk0[3 * j + 1] - sg * kt[1]) < 1e-4 &&
                std::fabs(s.sk0[3 * j + 2] - sg * kt[2]) < 1e-4;
        if (dup) continue;
        for (int i = 0; i < 3; i++) { s.sk0.push_back(sg * kt[i]); s.rw.push_back(rwt[i]); }
        s.numirr.push_back(ik);
        s.numrot.push_back(iop);
        s.trs.push_back(pass == 0 ? 1 : -1);
      }
    }
  s.ntk = (int)s.numirr.size();
  for (int d = 0; d < 3; d++) {
    double x = 1.0;
    for (int i = 0; i < s.ntk; i++) {
      double a = std::fabs(s.sk0[3 * i + d]);
      if (a < 1.0e-7) continue;
      x = std::min(x, a);
    }
    s.nkb[d] = (int)llround(1.0 / x);
  }
  if (s.nkb[0] * s.nkb[1] * s.nkb[2] != s.ntk)
    fail(1, "k mesh %dx%dx%d does not match the %d unfolded k points", s.nkb[0], s.nkb[1], s.nkb[2], s.ntk);
  // KG0 per full k
  s.ng0.assign(s.ntk, 0);
  s.kg0.assign((size_t)3 * s.ntg * s.ntk, 0);
  std::vector<int> tmp;
  for (int j = 0; j < s.ntk; j++) {
    int ik = s.numirr[j], iop = s.numrot[j];
    const int *R = &s.rg[9 * iop];
    const double *k = &s.ski[3 * ik];
    double kt[3];
    for (int i = 0; i < 3; i++)
      kt[i] = (double)R[i] * k[0] + (double)R[i + 3] * k[1] + (double)R[i + 6] * k[2] + (double)s.rw[3 * j + i];
    int ng = 0;
    make_kg0(s.b, s.ecut_psi, kt, s.ntg, tmp, ng);
    if (ng != s.ngi[ik]) fail(1, "ERROR;STOP;NG_for_psi should be NGI(ik): full k %d", j + 1);
    s.ng0[j] = ng;
    int sg = s.trs[j] == -1 ? -1 : 1;
    for (int i = 0; i < 3 * ng; i++) s.kg0[(size_t)j * s.ntg * 3 + i] = sg * tmp[i];
  }
  // index_kpt
  s.index_kpt.assign(s.ntk, -1);
  s.mesh_of_k.assign(s.ntk, -1);
  for (int ik = 0; ik < s.ntk; ik++) {
    int ix[3];
    for (int d = 0; d < 3; d++) {
      double x = s.sk0[3 * ik + d] * (double)s.nkb[d];
      if (s.ntk % 2 != 0) ix[d] = (int)llround(x + ((double)s.nkb[d] - 1.0) / 2.0) + 1;
      else ix[d] = (int)llround(x + (double)s.nkb[d] / 2.0);
      if (ix[d] < 1 || ix[d] > s.nkb[d]) fail(1, "make_index_kpt: k %d outside the mesh", ik + 1);
    }
    int m = (ix[0] - 1) + s.nkb[0] * ((ix[1] - 1) + s.nkb[1] * (ix[2] - 1));
    s.index_kpt[m] = ik;
  }
  for (int m = 0; m < s.ntk; m++) {
    if (s.index_kpt[m] < 0) fail(1, "make_index_kpt: mesh slot %d empty", m + 1);
    s.mesh_of_k[s.index_kpt[m]] = m;
  }
  // bands
  s.window_inside.assign(s.ntb, 0); s.tindx.assign(s.ntb, 0);
  s.e_ave.assign(s.ntb, 0); s.band_max.assign(s.ntb, 0); s.band_min.assign(s.ntb, 0);
  for (int ib = 0; ib < s.ntb; ib++) {
    double top = 0, btm = 0;
    int fs = 0;
    for (int ik = 0; ik < s.nk_irr; ik++) {
      double e = s.e_eigi[(size_t)ik * s.ntb + ib];
      if (ik == 0) { top = e; btm = e; }
      btm = std::min(btm, e);
      top = std::max(top, e);
    }
    if (btm > s.efermi) fs = 2;
    if (btm <= s.efermi && top >= s.efermi) { fs = 1; s.tindx[ib] = ib + 1; }
    if (top < s.efermi) fs = 0;
    s.window_inside[ib] = fs;
    s.e_ave[ib] = (top + btm) / 2.0;
    s.band_max[ib] = top;
    s.band_min[ib] = btm;
  }
  s.prob.assign((size_t)s.ntb * s.ntk, cd(0, 0));
  s.n_docc = s.n_pocc = s.n_uocc = 0;
  for (int ib = 0; ib < s.ncb; ib++) {
    if (s.window_inside[ib] == 0) s.n_docc++;
    if (s.window_inside[ib] == 1) s.n_pocc++;
    if (s.window_inside[ib] == 2) s.n_uocc++;
  }
  s.n_occ = s.n_docc + s.n_pocc;
  s.n_vir = s.n_uocc + s.n_pocc;
  // frequency grid
  double bmax = -1e300, bmin = 1e300;
  for (int ib = 0; ib < s.ncb; ib++) { bmax = std::max(bmax, s.band_max[ib]); bmin = std::min(bmin, s.band_min[ib]); }
  if (!explicit_em.empty()) {
    s.em.resize(explicit_em.size() / 2);
    for (size_t i = 0; i < s.em.size(); i++) s.em[i] = cd(explicit_em[2 * i], explicit_em[2 * i + 1]);
  } else {
    gen_grid(P.num_freq_grid, std::fabs(bmax - bmin), s.em);
  }
  // tetrahedra (0-based mesh slots)
  {
    const int ng[3] = {s.nkb[0], s.nkb[1], s.nkb[2]};
    double b2[3][3], b3[4][3], l[4];
    for (int i = 0; i < 3; i++)
      for (int d = 0; d < 3; d++) b2[i][d] = s.b[i][d] / (double)ng[i];
    for (int d = 0; d < 3; d++) {
      b3[0][d] = -b2[0][d] + b2[1][d] + b2[2][d];
      b3[1][d] = b2[0][d] - b2[1][d] + b2[2][d];
      b3[2][d] = b2[0][d] + b2[1][d] - b2[2][d];
      b3[3][d] = b2[0][d] + b2[1][d] + b2[2][d];
    }
    int itype = 0;
    for (int i = 0; i < 4; i++) {
      l[i] = b3[i][0] * b3[i][0] + b3[i][1] * b3[i][1] + b3[i][2] * b3[i][2];
      if (l[i] < l[itype]) itype = i;
    }
    int iv0[4] = {0, 0, 0, 0}, dv[4][4];
    for (int c = 0; c < 4; c++)
      for (int r = 0; r < 4; r++) dv[c][r] = (c == r);
    iv0[itype] = 1;
    dv[itype][itype] = -1;
    int ivv[6][4][3], it = 0;
    for (int i1 = 0; i1 < 3; i1++)
      for (int i2 = 0; i2 < 3; i2++) {
        if (i2 == i1) continue;
        for (int i3 = 0; i3 < 3; i3++) {
          if (i3 == i1 || i3 == i2) continue;
          for (int d = 0; d < 3; d++) {
            ivv[it][0][d] = iv0[d];
            ivv[it][1][d] = ivv[it][0][d] + dv[i1][d];
            ivv[it][2][d] = ivv[it][1][d] + dv[i2][d];
            ivv[it][3][d] = ivv[it][2][d] + dv[i3][d];
          }
          it++;
        }
      }
    s.imt1.assign((size_t)4 * 6 * s.ntk, 0);
    size_t nt = 0;
    for (int i3 = 0; i3 < ng[2]; i3++)
      for (int i2 = 0; i2 < ng[1]; i2++)
        for (int i1 = 0; i1 < ng[0]; i1++)
          for (int t = 0; t < 6; t++, nt++)
            for (int ii = 0; ii < 4; ii++) {
              int kv[3] = {i1 + ivv[t][ii][0], i2 + ivv[t][ii][1], i3 + ivv[t][ii][2]};
              for (int d = 0; d < 3; d++) { kv[d] %= ng[d]; if (kv[d] < 0) kv[d] += ng[d]; }
              s.imt1[4 * nt + ii] = kv[0] + ng[0] * kv[1] + ng[0] * ng[1] * kv[2];
            }
  }
  s.delt = P.green_func_delt / kAu;
  s.delta_ex = P.max_excitation_energy / kAu;
  s.dmna = P.ttrhdrn_dmna;  // used in Hartree units as given (chiqw.F passes it unconverted)
  s.dmnr = P.ttrhdrn_dmnr;
}

void build_unfold_map(const Setup &s, UnfoldMap &m) {
  m.src.assign((size_t)s.ntk * s.ntg, -1);
  m.phase.assign((size_t)s.ntk * s.ntg, cd(0, 0));
  const int p1 = 2 * s.L[0] + 1, p2 = 2 * s.L[1] + 1, p3 = 2 * s.L[2] + 1;
  for (int jk = 0; jk < s.ntk; jk++) {
    int ikir = s.numirr[jk], iop = s.numrot[jk], itrs = s.trs[jk];
    const double *ri = &s.rginv[9 * iop];
    const int *pgt = &s.pg[3 * iop];
    const int *rw = &s.rw[3 * jk];
    const int *pk = &s.packing[(size_t)ikir * p1 * p2 * p3];
    for (int ig = 0; ig < s.ng0[jk]; ig++) {
      const int *g = &s.kg0[((size_t)jk * s.ntg + ig) * 3];
      int i1 = g[0], j1 = g[1], k1 = g[2];
      if (itrs == -1) { i1 = -i1; j1 = -j1; k1 = -k1; }
      int i2 = i1 + rw[0], j2 = j1 + rw[1], k2 = k1 + rw[2];
      int i3 = (int)ri[0] * i2 + (int)ri[3] * j2 + (int)ri[6] * k2;
      int j3 = (int)ri[1] * i2 + (int)ri[4] * j2 + (int)ri[7] * k2;
      int k3 = (int)ri[2] * i2 + (int)ri[5] * j2 + (int)ri[8] * k2;
      int jg = 0;
      if (std::abs(i3) <= s.L[0] && std::abs(j3) <= s.L[1] && std::abs(k3) <= s.L[2])
        jg = pk[(i3 + s.L[0]) + (size_t)p1 * ((j3 + s.L[1]) + (size_t)p2 * (k3 + s.L[2]))];
      if (jg <= 0) fail(1, "make_C0: rotated G (%d,%d,%d) of full k %d not in the plane-wave list", i3, j3, k3, jk + 1);
      double phase = kTpi * ((double)i1 * (double)pgt[0] + (double)j1 * (double)pgt[1] + (double)k1 * (double)pgt[2]);
      cd pf = std::exp(cd(0, -1) * (phase / (double)s.nnp));
      m.src[(size_t)jk * s.ntg + ig] = jg - 1;
      m.phase[(size_t)jk * s.ntg + ig] = pf;
    }
  }
}

std::vector<int> q_list(const Setup &s, const std::string &epsdir) {
  const rp_params &P = s.params;
  std::vector<int> out;
  struct stat st;
  auto done = [&](int ik) {
    char path[4200];
    snprintf(path, sizeof path, "%s/q%03d/dat.log.%03d", epsdir.c_str(), ik + 1, P.file_num_log_start);
    return stat(path, &st) == 0;
  };
  if (P.flg_calc_type == 0) {
    for (int ik = 0; ik < s.nk_irr; ik++) if (!done(ik)) out.push_back(ik);
  } else if (P.flg_calc_type == 1) {
    int ix = -1;
    for (int ik = 0; ik < s.nk_irr; ik++)
      if (std::fabs(s.ski[3 * ik]) < 1e-5 && std::fabs(s.ski[3 * ik + 1]) < 1e-5 && std::fabs(s.ski[3 * ik + 2]) < 1e-5) ix = ik;
    if (ix < 0) fail(1, "flg_calc_type=1 but no Gamma point in dat.sample-k");
    if (!done(ix)) out.push_back(ix);
  } else if (P.flg_calc_type != 2) {
    fail(1, "flg_calc_type must be 0, 1 or 2");
  }
  return out;
}

QTask make_qtask(const Setup &s, int iq_irr, int max_pairs) {
  QTask t;
  if (iq_irr < 0 || iq_irr >= s.nk_irr) fail(1, "q index %d outside dat.sample-k (1..%d)", iq_irr + 1, s.nk_irr);
  t.iq_irr = iq_irr;
  search_list(&s.ski[3 * iq_irr], t.q);
  make_kg0(s.b, s.ecut_eps, t.q, s.ntg, t.lg0, t.ng);
  if (t.ng == 0) fail(1, "empty dielectric G sphere (Ecut_for_eps too small)");
  t.gamma = (t.q[0] == 0.0 && t.q[1] == 0.0 && t.q[2] == 0.0);
  t.qglen.resize(t.ng);
  for (int g = 0; g < t.ng; g++) {
    double v[3];
    for (int d = 0; d < 3; d++)
      v[d] = (t.q[0] + t.lg0[3 * g]) * s.b[0][d] + (t.q[1] + t.lg0[3 * g + 1]) * s.b[1][d] +
             (t.q[2] + t.lg0[3 * g + 2]) * s.b[2][d];
    t.qglen[g] = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (t.lg0[3 * g] == 0 && t.lg0[3 * g + 1] == 0 && t.lg0[3 * g + 2] == 0) t.no_g0 = g;
  }
  if (t.gamma && t.no_g0 < 0) fail(1, "G=0 missing from the dielectric sphere");
  t.kpq.assign(s.ntk, -1);
  t.shift.assign(3 * s.ntk, 0);
  for (int ik = 0; ik < s.ntk; ik++) {
    if (t.gamma) { t.kpq[ik] = ik; continue; }
    double sk[3];
    int *sg = &t.shift[3 * ik];
    const double d = 1.0e-6;
    for (int i = 0; i < 3; i++) {
      sk[i] = s.sk0[3 * ik + i] + t.q[i];
      if (sk[i] > 1.5 + d) { sk[i] -= 2.0; sg[i] = 2; }
      if (sk[i] > 0.5 + d) { sk[i] -= 1.0; sg[i] = 1; }
      if (sk[i] <= -1.5 + d) { sk[i] += 2.0; sg[i] = -2; }
      if (sk[i] <= -0.5 + d) { sk[i] += 1.0; sg[i] = -1; }
    }
    for (int jk = 0; jk < s.ntk; jk++)
      if (std::fabs(s.sk0[3 * jk] - sk[0]) < 1e-6 && std::fabs(s.sk0[3 * jk + 1] - sk[1]) < 1e-6 &&
          std::fabs(s.sk0[3 * jk + 2] - sk[2]) < 1e-6)
        t.kpq[ik] = jk;
    if (t.kpq[ik] < 0) fail(1, "k+q of full k %d is not on the mesh", ik + 1);
  }
  for (int jb = 0; jb < s.n_occ; jb++)
    for (int ib = 0; ib < s.n_vir; ib++) {
      int bv = s.n_docc + ib, bo = jb;
      if (std::fabs(s.e_ave[bv] - s.e_ave[bo]) >= s.delta_ex) continue;
      if (t.gamma && s.tindx[bv] == s.tindx[bo] && s.tindx[bv] != 0) {
        t.intra_band.push_back(bv);
        continue;
      }
      t.pair_vir.push_back(bv);
      t.pair_occ.push_back(bo);
    }
  if (s.params.flg_crpa == 1) t.intra_band.clear();  // chiqw.F:1626-1629
  t.npair_full = (int)t.pair_vir.size();
  if (max_pairs > 0 && (int)t.pair_vir.size() > max_pairs) {
    t.pair_vir.resize(max_pairs);
    t.pair_occ.resize(max_pairs);
  }
  return t;
}

}  // namespace rp
