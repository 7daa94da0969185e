"""The FP32 series form of the tetrahedron vertex weights
(respackdev_gb300/csrc/rp_tetra_series.cuh), compiled for the host with g++
and compared with the closed forms of the reference (sub2normal / sub1normal,
m_tetrahedron_20170325.F:304-451) evaluated in long double, their logs of
ratios taken as log1p so that the reference values themselves are accurate."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HARNESS = r"""
#include <complex>
#include <cstdio>
#include <random>
#include "rp_tetra_series.cuh"
typedef std::complex<long double> C;
// log(a / b) for a close to b without the cancellation of log of a ratio near 1:
// log(1 + t), t = (a - b) / b, as 0.5 log1p(2 Re t + |t|^2) + i atan2(Im t, 1 + Re t)
static C lr(C a, C b) {
  const C t = (a - b) / b;
  return C(0.5L * std::log1p(2.0L * t.real() + std::norm(t)), std::atan2(t.imag(), 1.0L + t.real()));
}
// the reference's closed forms (the oracle's sub2normal / sub1normal) in long double
static C s2(C g0, C g1, C g2, C g3, C w) {
  C v = -(g1 + w) * (g1 + w) / (6.0L * (g0 - g1) * (g1 - g2) * (g1 - g3));
  v -= (g2 + w) * (g2 + w) * (g2 + w) * lr(g2 + w, g1 + w) / (6.0L * (g0 - g2) * ((g1 - g2) * (g1 - g2)) * (g2 - g3));
  v += (g3 + w) * (g3 + w) * (g3 + w) * lr(g3 + w, g1 + w) / (6.0L * (g0 - g3) * ((g1 - g3) * (g1 - g3)) * (g2 - g3));
  v += (g0 + w) * (g0 + w) * (g0 + w) * lr(g0 + w, g1 + w) / (6.0L * ((g0 - g1) * (g0 - g1)) * (g0 - g2) * (g0 - g3));
  return v;
}
static C s1(C g0, C g1, C g2, C g3, C w) {
  C L10 = lr(g1 + w, g0 + w), L20 = lr(g2 + w, g0 + w), L30 = lr(g3 + w, g0 + w);
  C v = (-(g1 + w) * (g1 + w) * L10) / ((g0 - g2) * (g0 - g3) * (g0 - g1)) * 0.5L;
  v -= ((g1 + w) * (g1 + w) * L10 - (g2 + w) * (g2 + w) * L20) / ((g0 - g2) * (g1 - g2) * (g2 - g3)) * 0.5L;
  v += ((g1 + w) * (g1 + w) * L10 - (g3 + w) * (g3 + w) * L30) / ((g1 - g3) * (g0 - g3) * (g2 - g3)) * 0.5L;
  return v;
}
int main() {
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  const double delt = 0.01;
  long n_series = 0, n_total = 0;
  double worst = 0, worst_r = 0;
  for (int it = 0; it < 200000; it++) {
    double gr[4];
    const double c = -1.5 + 3.0 * U(rng), s = std::exp(std::log(2e-3) + (std::log(0.05) - std::log(2e-3)) * U(rng));
    for (int v = 0; v < 4; v++) gr[v] = c + s * (2.0 * U(rng) - 1.0);
    // the normal category: every pair separated (chk1 with dmna = dmnr = 1e-3)
    bool normal = true;
    for (int a = 0; a < 4; a++)
      for (int b = a + 1; b < 4; b++) {
        const double d1 = std::abs(gr[a] - gr[b]);
        const double d2 = std::abs(std::complex<double>(gr[a] + gr[b], 2 * delt)) * 0.5;
        if (d1 < 1e-3 || d1 / d2 < 1e-3) normal = false;
      }
    if (!normal) continue;
    const double dsgn = U(rng) < 0.5 ? 1.0 : -1.0;
    const bool imag = U(rng) < 0.5;
    const double wm = 1.1 * U(rng), wr = imag ? 0.0 : wm, wi = imag ? wm : 0.0;
    rp::TsCplx x[4];
    n_total++;
    if (!rp::tetra_series_weights(gr, dsgn, delt, wr, wi, x)) continue;
    n_series++;
    C g[4], w(wr, wi);
    for (int v = 0; v < 4; v++) g[v] = C(gr[v], delt) * (long double)dsgn;
    C ref[4];
    ref[0] = s2(g[1], g[0], g[2], g[3], w);
    ref[1] = s2(g[0], g[1], g[2], g[3], w);
    ref[2] = s2(g[0], g[2], g[1], g[3], w);
    ref[3] = s1(g[0], g[3], g[1], g[2], w) - ref[2] - ref[1] - ref[0];
    long double den = 0, err = 0;
    for (int v = 0; v < 4; v++) {
      den = std::max(den, std::abs(ref[v]));
      err = std::max(err, std::abs(C(x[v].r, x[v].i) - ref[v]));
    }
    const double e = (double)(err / den);
    double gm = 0.25 * (gr[0] + gr[1] + gr[2] + gr[3]), dmax = 0;
    for (int v = 0; v < 4; v++) dmax = std::max(dmax, std::abs(gr[v] - gm));
    const double r = dmax / std::abs(std::complex<double>(wr + dsgn * gm, wi + dsgn * delt));
    if (e > worst) { worst = e; worst_r = r; }
  }
  // all four values equal: 1 / (24 z)
  double eq[4] = {0.3, 0.3, 0.3, 0.3};
  rp::TsCplx y[4];
  const bool ok = rp::tetra_series_weights(eq, 1.0, delt, 0.1, 0.0, y);
  const std::complex<double> z(0.1 + 0.3, delt), want = 1.0 / (24.0 * z);
  double eqerr = 0;
  for (int v = 0; v < 4; v++) eqerr = std::max(eqerr, std::abs(std::complex<double>(y[v].r, y[v].i) - want) / std::abs(want));
  // near resonance the series declines
  double gres[4] = {-0.40, -0.39, -0.37, -0.42};
  const bool res = rp::tetra_series_weights(gres, 1.0, delt, 0.40, 0.0, y);
  std::printf("%ld %ld %.3e %.3e %d %.3e %d\n", n_total, n_series, worst, worst_r, ok ? 1 : 0, eqerr, res ? 1 : 0);
  return 0;
}
"""


def test_series_weights_match_the_closed_forms(tmp_path):
    src = tmp_path / "h.cpp"
    exe = tmp_path / "h"
    src.write_text(HARNESS)
    r = subprocess.run(["g++", "-O2", "-std=c++17", f"-I{ROOT}/respackdev_gb300/csrc", str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    n_total, n_series = int(out[0]), int(out[1])
    worst, worst_r = float(out[2]), float(out[3])
    ok_eq, eqerr, took_res = int(out[4]), float(out[5]), int(out[6])
    print(f"{n_series}/{n_total} normal (tetra, w) on the series; worst FP32 error {worst:.2e} (r = {worst_r:.3f})")
    assert n_total > 10000 and n_series > 0.9 * n_total
    # FP32 weights within a few units of FP32 rounding of the long-double closed forms
    assert worst < 1e-6
    assert ok_eq == 1 and eqerr < 1e-6
    assert took_res == 0


HARNESS2 = r"""
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include "rp_tetra_series.cuh"
typedef std::complex<long double> C;
static C lr(C a, C b) {
  const C t = (a - b) / b;
  return C(0.5L * std::log1p(2.0L * t.real() + std::norm(t)), std::atan2(t.imag(), 1.0L + t.real()));
}
static C s2(C g0, C g1, C g2, C g3, C w) {
  C v = -(g1 + w) * (g1 + w) / (6.0L * (g0 - g1) * (g1 - g2) * (g1 - g3));
  v -= (g2 + w) * (g2 + w) * (g2 + w) * lr(g2 + w, g1 + w) / (6.0L * (g0 - g2) * ((g1 - g2) * (g1 - g2)) * (g2 - g3));
  v += (g3 + w) * (g3 + w) * (g3 + w) * lr(g3 + w, g1 + w) / (6.0L * (g0 - g3) * ((g1 - g3) * (g1 - g3)) * (g2 - g3));
  v += (g0 + w) * (g0 + w) * (g0 + w) * lr(g0 + w, g1 + w) / (6.0L * ((g0 - g1) * (g0 - g1)) * (g0 - g2) * (g0 - g3));
  return v;
}
static C s1(C g0, C g1, C g2, C g3, C w) {
  C L10 = lr(g1 + w, g0 + w), L20 = lr(g2 + w, g0 + w), L30 = lr(g3 + w, g0 + w);
  C v = (-(g1 + w) * (g1 + w) * L10) / ((g0 - g2) * (g0 - g3) * (g0 - g1)) * 0.5L;
  v -= ((g1 + w) * (g1 + w) * L10 - (g2 + w) * (g2 + w) * L20) / ((g0 - g2) * (g1 - g2) * (g2 - g3)) * 0.5L;
  v += ((g1 + w) * (g1 + w) * L10 - (g3 + w) * (g3 + w) * L30) / ((g1 - g3) * (g0 - g3) * (g2 - g3)) * 0.5L;
  return v;
}
// tetra_series_vertex2 (one vertex, both signs, the kernel's form) against
// tetra_series_weights (all four vertices, one sign) on random points, and on
// near-resonant normal tetrahedra against the closed forms in long double
int main() {
  std::mt19937_64 rng(777);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  const double delt = 0.01;
  long n = 0, n_ok = 0, n_mismatch_flag = 0;
  double worst = 0;
  for (int it = 0; it < 100000; it++) {
    double gr[4];
    const double c = -1.5 + 3.0 * U(rng), s = std::exp(std::log(1e-4) + (std::log(0.1) - std::log(1e-4)) * U(rng));
    for (int v = 0; v < 4; v++) gr[v] = c + s * (2.0 * U(rng) - 1.0);
    if (U(rng) < 0.2) gr[1] = gr[0];                 // averaged (degenerate) points
    if (U(rng) < 0.1) gr[3] = gr[2] = gr[0];
    const bool imag = U(rng) < 0.5;
    double wm = 1.5 * U(rng), wr = imag ? 0.0 : wm, wi = imag ? wm : 0.0;
    const double mean = 0.25 * ((gr[0] + gr[1]) + (gr[2] + gr[3]));
    // a quarter of the cases near resonance: |w + gbar| of order delt, where
    // the unscaled powers of 1/z would overflow FP32
    if (!imag && U(rng) < 0.25) wr = -mean + (2.0 * U(rng) - 1.0) * 0.02;
    float d[4], dmax = 0.f;
    for (int v = 0; v < 4; v++) { d[v] = (float)(gr[v] - mean); dmax = std::fmax(dmax, std::fabs(d[v])); }
    for (int pos = 0; pos < 4; pos++) {
      bool ok[2];
      rp::TsCplx x2[2];
      rp::tetra_series_vertex2(d, d[pos], dmax, mean, delt, wr, wi, ok, x2);
      for (int sgi = 0; sgi < 2; sgi++) {
        rp::TsCplx x4[4];
        const bool ok4 = rp::tetra_series_weights(gr, sgi == 0 ? 1.0 : -1.0, delt, wr, wi, x4);
        n++;
        if (ok4 != ok[sgi]) { n_mismatch_flag++; continue; }
        if (!ok4) continue;
        n_ok++;
        const double den = std::hypot(x4[pos].r, x4[pos].i);
        const double e = std::hypot(x2[sgi].r - x4[pos].r, x2[sgi].i - x4[pos].i) / den;
        if (e > worst) worst = e;
      }
    }
  }
  // near resonance (|w + gbar| a few delt, r up to 1/2: up to 25 terms of
  // (1/z)^n with |z| ~ delt) against the long-double closed forms
  long nonfinite = 0, n_res = 0;
  double worst_res = 0;
  for (int it = 0; it < 20000; it++) {
    double gr[4];
    const double c = -1.0 + 2.0 * U(rng);
    for (int v = 0; v < 4; v++) gr[v] = c + 0.004 * v + 0.003 * U(rng);  // separated: the normal forms apply
    const double mean = 0.25 * ((gr[0] + gr[1]) + (gr[2] + gr[3]));
    const double wr = -mean + (2.0 * U(rng) - 1.0) * 0.03;
    float d[4], dmax = 0.f;
    for (int v = 0; v < 4; v++) { d[v] = (float)(gr[v] - mean); dmax = std::fmax(dmax, std::fabs(d[v])); }
    C g[4], w(wr, 0.0L);
    for (int v = 0; v < 4; v++) g[v] = C(gr[v], delt);
    C ref[4];
    ref[0] = s2(g[1], g[0], g[2], g[3], w);
    ref[1] = s2(g[0], g[1], g[2], g[3], w);
    ref[2] = s2(g[0], g[2], g[1], g[3], w);
    ref[3] = s1(g[0], g[3], g[1], g[2], w) - ref[2] - ref[1] - ref[0];
    long double den = 0;
    for (int v = 0; v < 4; v++) den = std::max(den, std::abs(ref[v]));
    for (int pos = 0; pos < 4; pos++) {
      bool ok[2];
      rp::TsCplx x2[2];
      rp::tetra_series_vertex2(d, d[pos], dmax, mean, delt, wr, 0.0, ok, x2);
      for (int s2i = 0; s2i < 2; s2i++)
        if (!std::isfinite(x2[s2i].r) || !std::isfinite(x2[s2i].i)) nonfinite++;
      if (!ok[0]) continue;
      n_res++;
      const double e = (double)(std::abs(C(x2[0].r, x2[0].i) - ref[pos]) / den);
      if (e > worst_res) worst_res = e;
    }
  }
  std::printf("%ld %ld %ld %.3e %ld %ld %.3e\n", n, n_ok, n_mismatch_flag, worst, nonfinite, n_res, worst_res);
  return 0;
}
"""


def test_vertex_series_both_signs_matches_four_vertex_form(tmp_path):
    """The kernel's form (one vertex, both signs sharing the h_n recurrence, the
    sign -1 through (-1)^n) equals the four-vertex form per sign to FP32
    rounding, and declines the same (tetrahedron, sign, frequency) cases."""
    src = tmp_path / "h2.cpp"
    exe = tmp_path / "h2"
    src.write_text(HARNESS2)
    r = subprocess.run(["g++", "-O2", "-std=c++17", f"-I{ROOT}/respackdev_gb300/csrc", str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    n, n_ok, n_flag, worst, nonfinite, n_res, worst_res = (int(out[0]), int(out[1]), int(out[2]), float(out[3]),
                                                           int(out[4]), int(out[5]), float(out[6]))
    print(f"near resonance: {n_res} vertex weights on the series, worst {worst_res:.2e} of the closed forms")
    print(f"{n_ok}/{n} on the series, {n_flag} decided differently, worst difference {worst:.2e}")
    # the r <= 1/2 test is the same up to rounding at the boundary
    assert n_flag < 1e-4 * n
    assert n_ok > 0.5 * n
    assert worst < 2e-6
    assert nonfinite == 0
    assert n_res > 1000 and worst_res < 2e-6
