// rp_int.cpp -- calc_int on the device: the C ABI of calc_w3d (V, W) and
// calc_j3d (X, J), their readers and their writers.
//
// A context reads dir-wfn (through the chiqw set-up), the Wannier functions of
// dir-wan and the dielectric data of dir-eps, unfolds the q mesh, builds the
// eps/psi G lists of every q (make_LG0) and keeps on the device
//   - the real-space Wannier functions u_w,k(r) (single precision, computed once),
//   - eps^-1 of every irreducible q in complex(4), as the reference stores it.
// Per q point it then runs: pair densities (chiqw's kernel, pairs of Wannier
// functions) -> k sums with the lattice phases -> eps^-1 products -> the
// quadratic forms func / funcw; a last pass Fourier-transforms q -> R.
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cerrno>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "rp_dev.cuh"
#include "rp_host.h"
#include "rp_int.h"

namespace {

using rp::cd;
using rp::fail;

struct Buf {
  void *p = nullptr;
  size_t bytes = 0;
  void ensure(size_t n) {
    if (n <= bytes) return;
    release();
    RP_CUDA(cudaMalloc(&p, n));
    bytes = n;
  }
  template <typename T> T *as() const { return (T *)p; }
  void release() { if (p) cudaFree(p); p = nullptr; bytes = 0; }
};

template <typename T> void put(Buf &b, const std::vector<T> &v, cudaStream_t st) {
  b.ensure(std::max<size_t>(sizeof(T) * v.size(), 16));
  if (!v.empty()) RP_CUDA(cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st));
  rp::note_transfer((long long)(sizeof(T) * v.size()), 0);
}

template <typename T> void get(std::vector<T> &v, const Buf &b, size_t n, cudaStream_t st) {
  v.resize(n);
  if (n) RP_CUDA(cudaMemcpyAsync(v.data(), b.p, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
  RP_CUDA(cudaStreamSynchronize(st));
  rp::note_transfer(0, (long long)(sizeof(T) * n));
}

constexpr double kBohr = 0.529177;  // config_w3d.h

// search_kq (calc_int_sub.F:1-100): k+q folded into the mesh and its shift
void search_kq(const rp::Setup &s, const double q[3], bool gamma, std::vector<int> &kpq, std::vector<int> &shift) {
  kpq.assign(s.ntk, -1);
  shift.assign(3 * s.ntk, 0);
  for (int ik = 0; ik < s.ntk; ik++) {
    if (gamma) { kpq[ik] = ik; continue; }
    double sk[3];
    int *sg = &shift[3 * ik];
    const double d = 1.0e-6;
    for (int i = 0; i < 3; i++) {
      sk[i] = s.sk0[3 * ik + i] + q[i];
      if (sk[i] > 1.5 + d) { sk[i] -= 2.0; sg[i] = 2; }
      if (sk[i] > 0.5 + d) { sk[i] -= 1.0; sg[i] = 1; }
      if (sk[i] <= -1.5 + d) { sk[i] += 2.0; sg[i] = -2; }
      if (sk[i] <= -0.5 + d) { sk[i] += 1.0; sg[i] = -1; }
    }
    for (int jk = 0; jk < s.ntk; jk++)
      if (std::fabs(s.sk0[3 * jk] - sk[0]) < 1e-6 && std::fabs(s.sk0[3 * jk + 1] - sk[1]) < 1e-6 &&
          std::fabs(s.sk0[3 * jk + 2] - sk[2]) < 1e-6)
        kpq[ik] = jk;
    if (kpq[ik] < 0) fail(1, "k+q of full k %d is not on the mesh", ik + 1);
  }
}

// kcheck / kcheck_trs (calc_int_sub.F:356-446)
void kcheck(double *k, int *rw, bool trs) {
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

std::string fmt(const char *f, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, f);
  vsnprintf(buf, sizeof buf, f, ap);
  va_end(ap);
  return buf;
}

// '(2f15.10)' records of dat.wgrid (fixed columns, the two fields may touch)
cd read_2f15(const std::string &line) {
  if (line.size() >= 30) return cd(std::atof(line.substr(0, 15).c_str()), std::atof(line.substr(15, 15).c_str()));
  double a = 0, b = 0;
  if (std::sscanf(line.c_str(), "%lf %lf", &a, &b) != 2) fail(1, "dat.wgrid: bad record '%s'", line.c_str());
  return cd(a, b);
}

}  // namespace

namespace rp {

// dir-wan/dat.wan and dat.wan-center (calc_intW.F:339-370; writer wannier.F:2136-2175)
void read_dir_wan_orbitals(Setup &s, const std::string &root) {
  UnformattedReader r(root + "/dir-wan/dat.wan");
  int nwf = 0;
  if (r.read(&nwf, sizeof nwf) != sizeof nwf || nwf <= 0) fail(1, "dir-wan/dat.wan: bad NWF record");
  s.nwf = nwf;
  s.wan.assign((size_t)s.ntk * nwf * s.ntg, cd(0, 0));
  std::vector<cd> rec((size_t)s.ntg * nwf);
  for (int k = 0; k < s.ntk; k++) {
    const size_t want = sizeof(cd) * (size_t)s.ng0[k] * nwf;
    const size_t got = r.read(rec.data(), want);
    if (got != want) fail(1, "dir-wan/dat.wan: record of k %d has %zu bytes, expected %zu", k + 1, got, want);
    for (int w = 0; w < nwf; w++)
      for (int ig = 0; ig < s.ng0[k]; ig++) s.wan[((size_t)k * nwf + w) * s.ntg + ig] = rec[(size_t)w * s.ng0[k] + ig];
  }
  std::ifstream f(root + "/dir-wan/dat.wan-center");
  if (!f) fail(1, "cannot open dir-wan/dat.wan-center");
  std::string line;
  std::getline(f, line);
  std::getline(f, line);
  s.wan_center.assign(3 * nwf, 0.0);
  for (int w = 0; w < nwf; w++)
    if (!(f >> s.wan_center[3 * w] >> s.wan_center[3 * w + 1] >> s.wan_center[3 * w + 2]))
      fail(1, "dir-wan/dat.wan-center: %d centres, expected %d", w, nwf);
}

}  // namespace rp

struct rp_int {
  rp::Setup S;
  rp_int_params P{};
  std::string root, err;
  int dev = 0;
  cudaStream_t st = nullptr;
  long long launches = 0;
  // dir-eps
  int ne = 0;
  std::vector<cd> em;
  double ecut_eps = 0;
  // q mesh
  int nq_irr = 0, ntq = 0, ntgq = 0, iqgm = -1, nog0 = -1, Lq[3]{};
  std::vector<double> sq;  // 3*ntq
  std::vector<int> numirrq, numrotq, trsq, rwq;
  std::vector<std::vector<int>> lg0;  // per full q: eps sphere, then the psi shell
  std::vector<int> nge, ngp;
  std::vector<int> packingq;          // irreducible q
  std::vector<cd> eps00;              // eps^-1(G=0,G=0) of Gamma per frequency (complex(4) values)
  int Rw[3]{};                        // extent of the psi spheres (real-space transform)
  // device data
  Buf wan, numirr, trs, src, phase, ng0, kg0, cfull, ur, eps;
  Buf kpq, shift, lg, len, pfk, rho_pk, rhoV, T, pa, pb, fw, fq, idx, p1, p2, pfR, out, head, chunk_vir, chunk_first,
      chunk_count, pair_list, pair_occ;
  cudaEvent_t ev[2]{};
  double times[5]{};
  ~rp_int() {
    for (Buf *b : {&wan, &numirr, &trs, &src, &phase, &ng0, &kg0, &cfull, &ur, &eps, &kpq, &shift, &lg, &len, &pfk,
                   &rho_pk, &rhoV, &T, &pa, &pb, &fw, &fq, &idx, &p1, &p2, &pfR, &out, &head, &chunk_vir, &chunk_first,
                   &chunk_count, &pair_list, &pair_occ})
      b->release();
    for (auto &e : ev) if (e) cudaEventDestroy(e);
    if (st) cudaStreamDestroy(st);
  }
};

static thread_local std::string g_int_err;

template <typename F> static int guarded_int(rp_int *c, F &&f) {
  try {
    f();
    return 0;
  } catch (const rp::Error &e) {
    if (c) c->err = e.msg; else g_int_err = e.msg;
    return e.code;
  } catch (const std::bad_alloc &) {
    if (c) c->err = "host out of memory"; else g_int_err = "host out of memory";
    return -2;
  }
}

// make_LG0 (calc_int_sub.F:447-504): the eps sphere in scan order, then the
// points of the psi sphere outside it, in scan order
static void make_lg0(const rp::Setup &s, double ge, double gp, const double q[3], std::vector<int> &lg, int &nge,
                     int &ngp) {
  std::vector<int> pe, pp;
  int ne_ = 0, np_ = 0;
  rp::make_kg0(s.b, ge, q, 0, pe, ne_);
  rp::make_kg0(s.b, gp, q, 0, pp, np_);
  lg = pe;
  for (int i = 0; i < np_; i++) {
    const int *g = &pp[3 * i];
    double v[3];
    for (int d = 0; d < 3; d++) v[d] = (q[0] + g[0]) * s.b[0][d] + (q[1] + g[1]) * s.b[1][d] + (q[2] + g[2]) * s.b[2][d];
    if (v[0] * v[0] + v[1] * v[1] + v[2] * v[2] > ge) lg.insert(lg.end(), g, g + 3);
  }
  nge = ne_;
  ngp = (int)lg.size() / 3;
}

static void int_read_eps_dir(rp_int *c) {
  rp::Setup &S = c->S;
  const std::string d = c->root + "/dir-eps/";
  {
    rp::ListReader r(d + "dat.chi_cutoff");
    c->ecut_eps = r.read_real();
  }
  {
    std::ifstream f(d + "dat.wgrid");
    if (!f) fail(1, "cannot open dir-eps/dat.wgrid");
    std::string line;
    if (!std::getline(f, line)) fail(1, "dir-eps/dat.wgrid is empty");
    c->ne = std::atoi(line.c_str());
    if (c->ne <= 0) fail(1, "dir-eps/dat.wgrid: bad frequency count");
    c->em.resize(c->ne);
    for (int e = 0; e < c->ne; e++) {
      if (!std::getline(f, line)) fail(1, "dir-eps/dat.wgrid: %d of %d frequencies", e, c->ne);
      c->em[e] = read_2f15(line);
    }
  }
  if (c->P.calc_ifreq < 1 || c->P.calc_ifreq > c->ne) fail(1, "calc_ifreq = %d outside 1..%d", c->P.calc_ifreq, c->ne);
  c->nq_irr = S.nk_irr;
  std::vector<double> sqi(3 * c->nq_irr);
  for (int iq = 0; iq < c->nq_irr; iq++) {
    rp::ListReader r(d + fmt("q%03d/dat.sq", iq + 1));
    r.read(3, &sqi[3 * iq]);
  }
  // full q mesh (calc_intW.F:441-510)
  c->sq = sqi;
  c->numirrq.resize(c->nq_irr); c->numrotq.assign(c->nq_irr, 0); c->trsq.assign(c->nq_irr, 1);
  c->rwq.assign(3 * c->nq_irr, 0);
  for (int iq = 0; iq < c->nq_irr; iq++) c->numirrq[iq] = iq;
  for (int iq = 0; iq < c->nq_irr; iq++)
    for (int iop = 0; iop < S.nsymq; iop++) {
      const int *R = &S.rg[9 * iop];
      const double *k = &sqi[3 * iq];
      for (int pass = 0; pass < 2; pass++) {
        double kt[3];
        int rw[3] = {0, 0, 0};
        for (int i = 0; i < 3; i++) kt[i] = (double)R[i] * k[0] + (double)R[i + 3] * k[1] + (double)R[i + 6] * k[2];
        kcheck(kt, rw, pass == 1);
        const double sg = pass == 0 ? 1.0 : -1.0;
        bool dup = false;
        for (size_t j = 0; j < c->sq.size() / 3 && !dup; j++)
          dup = std::fabs(c->sq[3 * j] - sg * kt[0]) < 1e-4 && std::fabs(c->sq[3 * j + 1] - sg * kt[1]) < 1e-4 &&
                std::fabs(c->sq[3 * j + 2] - sg * kt[2]) < 1e-4;
        if (dup) continue;
        for (int i = 0; i < 3; i++) { c->sq.push_back(sg * kt[i]); c->rwq.push_back(rw[i]); }
        c->numirrq.push_back(iq); c->numrotq.push_back(iop); c->trsq.push_back(pass == 0 ? 1 : -1);
      }
    }
  c->ntq = (int)c->sq.size() / 3;
  if (c->ntq != S.ntk) fail(1, "ERROR;STOP;NTQ should be jk (NTQ=%d, NTK=%d)", c->ntq, S.ntk);
  // G lists per full q (calc_intW.F:514-582)
  c->lg0.assign(c->ntq, {});
  c->nge.assign(c->ntq, 0);
  c->ngp.assign(c->ntq, 0);
  for (int iq = 0; iq < c->ntq; iq++) {
    double q[3];
    if (iq < c->nq_irr) {
      for (int dd = 0; dd < 3; dd++) q[dd] = sqi[3 * iq + dd];
    } else {
      const int *R = &S.rg[9 * c->numrotq[iq]];
      const double *k = &sqi[3 * c->numirrq[iq]];
      for (int i = 0; i < 3; i++)
        q[i] = (double)R[i] * k[0] + (double)R[i + 3] * k[1] + (double)R[i + 6] * k[2] + (double)c->rwq[3 * iq + i];
    }
    make_lg0(S, c->ecut_eps, S.ecut_psi, q, c->lg0[iq], c->nge[iq], c->ngp[iq]);
    if (iq >= c->nq_irr && c->trsq[iq] == -1)
      for (auto &x : c->lg0[iq]) x = -x;
  }
  for (int dd = 0; dd < 3; dd++) c->Lq[dd] = 0;
  for (auto &l : c->lg0)
    for (size_t i = 0; i < l.size(); i++) c->Lq[i % 3] = std::max(c->Lq[i % 3], std::abs(l[i]));
  for (int dd = 0; dd < 3; dd++) c->Lq[dd]++;
  const int n1 = 2 * c->Lq[0] + 1, n2 = 2 * c->Lq[1] + 1, n3 = 2 * c->Lq[2] + 1;
  c->packingq.assign((size_t)n1 * n2 * n3 * c->nq_irr, 0);
  for (int iq = 0; iq < c->nq_irr; iq++)
    for (int ig = 0; ig < c->nge[iq]; ig++) {
      const int *g = &c->lg0[iq][3 * ig];
      c->packingq[(size_t)iq * n1 * n2 * n3 + (g[0] + c->Lq[0]) + (size_t)n1 * ((g[1] + c->Lq[1]) + (size_t)n2 * (g[2] + c->Lq[2]))] =
          ig + 1;
    }
  c->ntgq = 0;
  for (int iq = 0; iq < c->ntq; iq++) c->ntgq = std::max(c->ntgq, c->nge[iq]);
  // eps^-1 of the irreducible q as complex(4); Gamma: the mean of files 600-602 (:587-630)
  const size_t nn = (size_t)c->ntgq * c->ntgq;
  c->eps.ensure(sizeof(float2) * nn * c->ne * c->nq_irr);
  RP_CUDA(cudaMemsetAsync(c->eps.p, 0, sizeof(float2) * nn * c->ne * c->nq_irr, c->st));
  std::vector<float2> host(nn * c->ne);
  for (int iq = 0; iq < c->nq_irr; iq++) {
    const double *k = &S.ski[3 * iq];
    const bool gm = std::fabs(k[0]) < 1e-5 && std::fabs(k[1]) < 1e-5 && std::fabs(k[2]) < 1e-5;
    const int NG = c->nge[iq], nf = gm ? 3 : 1;
    if (gm) c->iqgm = iq;
    std::fill(host.begin(), host.end(), make_float2(0.f, 0.f));
    const std::string c4path = d + fmt("q%03d/dat.epsqw.c4", iq + 1);
    struct stat st4;
    if (c->P.read_eps_f32 && stat(c4path.c_str(), &st4) == 0) {
      // the complex(4) side file of rp_write_q (write_eps_f32): the values below, precomputed
      std::vector<float2> b4((size_t)NG * NG * c->ne);
      rp::UnformattedReader r(c4path);
      const size_t got = r.read(b4.data(), sizeof(float2) * b4.size());
      if (got != sizeof(float2) * b4.size())
        fail(1, "dir-eps/q%03d/dat.epsqw.c4: %zu bytes, expected %zu", iq + 1, got, sizeof(float2) * b4.size());
      for (int e = 0; e < c->ne; e++)
        for (int jg = 0; jg < NG; jg++)
          for (int ig = 0; ig < NG; ig++)
            host[((size_t)e * c->ntgq + jg) * c->ntgq + ig] = b4[((size_t)e * NG + jg) * NG + ig];
    } else {
      std::vector<cd> acc((size_t)NG * NG * c->ne, cd(0, 0)), buf(acc.size());
      for (int ix = 0; ix < nf; ix++) {
        rp::UnformattedReader r(d + fmt("q%03d/dat.epsqw.%03d", iq + 1, 600 + ix));
        const size_t got = r.read(buf.data(), sizeof(cd) * buf.size());
        if (got != sizeof(cd) * buf.size()) fail(1, "dir-eps/q%03d/dat.epsqw.%03d: %zu bytes, expected %zu", iq + 1, 600 + ix, got, sizeof(cd) * buf.size());
        for (size_t i = 0; i < acc.size(); i++) acc[i] += buf[i];
      }
      for (int e = 0; e < c->ne; e++)
        for (int jg = 0; jg < NG; jg++)
          for (int ig = 0; ig < NG; ig++) {
            cd v = acc[((size_t)e * NG + jg) * NG + ig];
            if (gm) v = v / 3.0;
            host[((size_t)e * c->ntgq + jg) * c->ntgq + ig] = make_float2((float)v.real(), (float)v.imag());
          }
    }
    RP_CUDA(cudaMemcpyAsync(c->eps.as<float2>() + (size_t)iq * nn * c->ne, host.data(), sizeof(float2) * host.size(),
                            cudaMemcpyHostToDevice, c->st));
    RP_CUDA(cudaStreamSynchronize(c->st));
    rp::note_transfer((long long)(sizeof(float2) * host.size()), 0);
    if (gm) {
      // NoG0: position of G = 0 in the Gamma list (calc_intW.F:707-712)
      for (int ig = 0; ig < c->ngp[iq]; ig++)
        if (c->lg0[iq][3 * ig] == 0 && c->lg0[iq][3 * ig + 1] == 0 && c->lg0[iq][3 * ig + 2] == 0) c->nog0 = ig;
      c->eps00.resize(c->ne);
      for (int e = 0; e < c->ne; e++) {
        const float2 v = host[((size_t)e * c->ntgq + c->nog0) * c->ntgq + c->nog0];
        c->eps00[e] = cd(v.x, v.y);
      }
    }
  }
  if (c->iqgm < 0 || c->nog0 < 0) fail(1, "no Gamma point among the q points of dir-eps");
}

// make_eps (calc_int_sub.F:222-311) as an index map into the irreducible q's
// list plus the two phases; trs = -1 transposes
static void eps_map(const rp_int *c, int iq, bool identity, std::vector<int> &idx, std::vector<cd> &ph1,
                    std::vector<cd> &ph2, int &trs, int &iqir) {
  const rp::Setup &S = c->S;
  const int NG = c->nge[iq];
  idx.assign(NG, -1); ph1.assign(NG, cd(1, 0)); ph2.assign(NG, cd(1, 0));
  if (identity) {
    trs = 1; iqir = iq;
    for (int ig = 0; ig < NG; ig++) idx[ig] = ig;
    return;
  }
  iqir = c->numirrq[iq];
  trs = c->trsq[iq];
  const int iop = c->numrotq[iq];
  const double *ri = &S.rginv[9 * iop];
  const int *pgt = &S.pg[3 * iop], *rw = &c->rwq[3 * iq];
  const int n1 = 2 * c->Lq[0] + 1, n2 = 2 * c->Lq[1] + 1, n3 = 2 * c->Lq[2] + 1;
  const int *pk = &c->packingq[(size_t)iqir * n1 * n2 * n3];
  for (int ig = 0; ig < NG; ig++) {
    const int *g = &c->lg0[iq][3 * ig];
    int i1 = g[0], j1 = g[1], k1 = g[2];
    if (trs == -1) { i1 = -i1; j1 = -j1; k1 = -k1; }
    const int i2 = i1 + rw[0], j2 = j1 + rw[1], k2 = k1 + rw[2];
    const int i3 = (int)ri[0] * i2 + (int)ri[3] * j2 + (int)ri[6] * k2;
    const int j3 = (int)ri[1] * i2 + (int)ri[4] * j2 + (int)ri[7] * k2;
    const int k3 = (int)ri[2] * i2 + (int)ri[5] * j2 + (int)ri[8] * k2;
    int v = 0;
    if (std::abs(i3) <= c->Lq[0] && std::abs(j3) <= c->Lq[1] && std::abs(k3) <= c->Lq[2])
      v = pk[(i3 + c->Lq[0]) + (size_t)n1 * ((j3 + c->Lq[1]) + (size_t)n2 * (k3 + c->Lq[2]))];
    idx[ig] = v - 1;
    const double phase = rp::kTpi * ((double)i1 * (double)pgt[0] + (double)j1 * (double)pgt[1] + (double)k1 * (double)pgt[2]);
    ph1[ig] = std::exp(cd(0, -1) * phase / (double)S.nnp);
    ph2[ig] = std::exp(cd(0, 1) * phase / (double)S.nnp);
  }
}

static void int_create(rp_int *c, const char *root, const rp_int_params *p) {
  c->root = root;
  c->P = *p;
  rp::Setup &S = c->S;
  rp_default_params(&S.params);
  S.params.n_calc_band = 1;
  for (int d = 0; d < 3; d++) S.params.fft_box[d] = p->fft_box[d];
  S.params.device = p->device;
  c->dev = p->device;
  RP_CUDA(cudaSetDevice(c->dev));
  RP_CUDA(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
  for (auto &e : c->ev) RP_CUDA(cudaEventCreate(&e));
  rp::read_dir_wfn(S, c->root);
  rp::finish_setup(S, {});
  rp::read_dir_wan_orbitals(S, c->root);
  int_read_eps_dir(c);
  // real-space Wannier functions: the dat.wan coefficients are already on the
  // full mesh, so the rotation of the chiqw transform is the identity
  const int ntk = S.ntk, nwf = S.nwf, ntg = S.ntg;
  std::vector<int> idk(ntk), one(ntk, 1), srcv((size_t)ntk * ntg);
  std::vector<cd> ph((size_t)ntk * ntg, cd(1, 0));
  for (int k = 0; k < ntk; k++) {
    idk[k] = k;
    for (int ig = 0; ig < ntg; ig++) srcv[(size_t)k * ntg + ig] = ig;
  }
  for (int dd = 0; dd < 3; dd++) c->Rw[dd] = 0;
  for (size_t i = 0; i < S.kg0.size(); i++) c->Rw[i % 3] = std::max(c->Rw[i % 3], std::abs(S.kg0[i]));
  put(c->wan, S.wan, c->st);
  put(c->numirr, idk, c->st);
  put(c->trs, one, c->st);
  put(c->src, srcv, c->st);
  put(c->phase, ph, c->st);
  put(c->ng0, S.ng0, c->st);
  put(c->kg0, S.kg0, c->st);
  const size_t N = (size_t)S.nw[0] * S.nw[1] * S.nw[2];
  c->cfull.ensure(sizeof(cd) * (size_t)ntk * nwf * ntg);
  c->ur.ensure(sizeof(float2) * (size_t)ntk * nwf * N);
  c->launches += rp::launch_wfn_realspace(c->wan.as<double2>(), c->numirr.as<int>(), c->trs.as<int>(), c->src.as<int>(),
                                          c->phase.as<double2>(), c->ng0.as<int>(), c->kg0.as<int>(), ntk, nwf, ntg,
                                          S.nw[0], S.nw[1], S.nw[2], c->Rw[0], c->Rw[1], c->Rw[2],
                                          c->cfull.as<double2>(), c->ur.as<float2>(), 0, ntk, c->st);
  RP_CUDA(cudaStreamSynchronize(c->st));
}

// Pair densities of q point iq for the pairs (vir[p] at k+q, occ[p] at k) and
// their k sums with nr phase sets pf[r*ntk + k]: c->rhoV[(r*np + p)*ngp + g].
static void int_q_rho(rp_int *c, int iq, const std::vector<int> &pv, const std::vector<int> &po, int j_order,
                      const std::vector<cd> &pf, int nr, float *ms_pair, float *ms_red) {
  rp::Setup &S = c->S;
  cudaStream_t st = c->st;
  const double *q = &c->sq[3 * iq];
  const bool gamma = q[0] == 0.0 && q[1] == 0.0 && q[2] == 0.0;
  const int ngp = c->ngp[iq], np = (int)pv.size(), ntk = S.ntk;
  const std::vector<int> &LG = c->lg0[iq];
  std::vector<int> kpq, shift;
  search_kq(S, q, gamma, kpq, shift);
  std::vector<double> len(ngp, 1.0);
  int g0 = -1;
  for (int g = 0; g < ngp; g++) {
    const int *l = &LG[3 * g];
    if (gamma && l[0] == 0 && l[1] == 0 && l[2] == 0) { g0 = g; continue; }
    double v[3];
    for (int d = 0; d < 3; d++) v[d] = (q[0] + (double)l[0]) * S.b[0][d] + (q[1] + (double)l[1]) * S.b[1][d] + (q[2] + (double)l[2]) * S.b[2][d];
    len[g] = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  }
  int ext[3] = {0, 0, 0};
  for (int i = 0; i < 3 * ngp; i++) ext[i % 3] = std::max(ext[i % 3], std::abs(LG[i]));
  // pairs grouped by virtual function, as many per CTA as shared memory allows
  const int n1 = S.nw[0], n2 = S.nw[1], n3 = S.nw[2];
  auto smem_of = [&](int j) {
    rp::PairGeom gq;
    gq.n1 = n1; gq.n2 = n2; gq.n3 = n3; gq.R1 = ext[0]; gq.R2 = ext[1]; gq.ng = ngp;
    return rp::pair_density_smem(gq, j, false);
  };
  int jmax = 8;
  while (jmax > 1 && smem_of(jmax) > 220 * 1024) jmax--;
  if (smem_of(jmax) > 220 * 1024) fail(1, "G list of q %d (%d vectors) too large for the pair-density tile", iq + 1, ngp);
  std::map<int, std::vector<int>> by;
  for (int p = 0; p < np; p++) by[pv[p]].push_back(p);
  std::vector<int> cv, cf, cc, pl;
  for (auto &kv : by)
    for (size_t s0 = 0; s0 < kv.second.size(); s0 += jmax) {
      cv.push_back(kv.first);
      cf.push_back((int)pl.size());
      const size_t n = std::min<size_t>(jmax, kv.second.size() - s0);
      cc.push_back((int)n);
      for (size_t j = 0; j < n; j++) pl.push_back(kv.second[s0 + j]);
    }
  put(c->kpq, kpq, st);
  put(c->shift, shift, st);
  put(c->lg, LG, st);
  put(c->len, len, st);
  put(c->chunk_vir, cv, st);
  put(c->chunk_first, cf, st);
  put(c->chunk_count, cc, st);
  put(c->pair_list, pl, st);
  put(c->pair_occ, po, st);
  c->rho_pk.ensure(sizeof(float2) * (size_t)np * ntk * ngp);
  rp::PairGeom pg;
  pg.ntk = ntk; pg.ncb = S.nwf; pg.n1 = n1; pg.n2 = n2; pg.n3 = n3; pg.ng = ngp;
  pg.kpq = c->kpq.as<int>(); pg.shift = c->shift.as<int>(); pg.lg0 = c->lg.as<int>();
  pg.R1 = ext[0]; pg.R2 = ext[1]; pg.R3 = ext[2];
  rp::PairChunks pc;
  pc.chunk_vir = c->chunk_vir.as<int>(); pc.chunk_first = c->chunk_first.as<int>();
  pc.chunk_count = c->chunk_count.as<int>(); pc.pair_list = c->pair_list.as<int>();
  pc.pair_occ = c->pair_occ.as<int>(); pc.nchunk = (int)cv.size(); pc.jmax = jmax;
  RP_CUDA(cudaEventRecord(c->ev[0], st));
  c->launches += rp::launch_pair_density_fp32(c->ur.as<float2>(), pg, pc, c->rho_pk.as<float2>(), st);
  RP_CUDA(cudaEventRecord(c->ev[1], st));
  RP_CUDA(cudaEventSynchronize(c->ev[1]));
  float ms = 0;
  RP_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
  *ms_pair += ms;
  put(c->pfk, pf, st);
  c->rhoV.ensure(sizeof(double2) * (size_t)nr * np * ngp);
  RP_CUDA(cudaEventRecord(c->ev[0], st));
  c->launches += rp::launch_int_reduce(c->rho_pk.as<float2>(), c->pfk.as<double2>(), c->len.as<double>(), np, ntk, ngp,
                                       g0, gamma ? 1 : 0, j_order, nr, c->rhoV.as<double2>(), st);
  RP_CUDA(cudaEventRecord(c->ev[1], st));
  RP_CUDA(cudaEventSynchronize(c->ev[1]));
  RP_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
  *ms_red += ms;
}

// T = eps^-1_q conj(rhoV) and the quadratic forms of the pairs (pa, pb):
// bare sums into fb[o] and screened sums into fs[e*fstride + o]
static void int_q_forms(rp_int *c, int iq, bool identity_eps, int nv, const std::vector<int> &pa,
                        const std::vector<int> &pb, double2 *fb, double2 *fs, size_t fstride, float *ms) {
  cudaStream_t st = c->st;
  const int nge = c->nge[iq], ngp = c->ngp[iq], nout = (int)pa.size();
  std::vector<int> idx;
  std::vector<cd> ph1, ph2;
  int trs = 1, iqir = 0;
  eps_map(c, iq, identity_eps, idx, ph1, ph2, trs, iqir);
  if (iqir < 0 || iqir >= c->nq_irr) fail(1, "q %d maps outside the irreducible q list", iq + 1);
  put(c->idx, idx, st);
  put(c->p1, ph1, st);
  put(c->p2, ph2, st);
  put(c->pa, pa, st);
  put(c->pb, pb, st);
  c->T.ensure(sizeof(double2) * (size_t)c->ne * nv * std::max(nge, 1));
  RP_CUDA(cudaEventRecord(c->ev[0], st));
  const size_t nn = (size_t)c->ntgq * c->ntgq;
  c->launches += rp::launch_int_quad(c->rhoV.as<double2>(), nullptr, c->pa.as<int>(), c->pb.as<int>(), nout, nv, nge,
                                     ngp, 1, fb, 0, st);
  c->launches += rp::launch_int_eps(c->eps.as<float2>() + (size_t)iqir * nn * c->ne, c->ntgq, c->idx.as<int>(),
                                    c->p1.as<double2>(), c->p2.as<double2>(), trs, c->rhoV.as<double2>(), nv, nge, ngp,
                                    c->ne, c->T.as<double2>(), st);
  c->launches += rp::launch_int_quad(c->rhoV.as<double2>(), c->T.as<double2>(), c->pa.as<int>(), c->pb.as<int>(), nout,
                                     nv, nge, ngp, c->ne, fs, fstride, st);
  RP_CUDA(cudaEventRecord(c->ev[1], st));
  RP_CUDA(cudaEventSynchronize(c->ev[1]));
  float t = 0;
  RP_CUDA(cudaEventElapsedTime(&t, c->ev[0], c->ev[1]));
  *ms += t;
}

static int box_of(const rp_int *c, int na[3]) {
  for (int d = 0; d < 3; d++) na[d] = c->S.nkb[d] / 2;
  return (2 * na[0] + 1) * (2 * na[1] + 1) * (2 * na[2] + 1);
}

static double qsz_of(const rp_int *c) {
  return std::pow(6.0 * (rp::kPi * rp::kPi) / (double)c->ntq / c->S.volume, 1.0 / 3.0);
}

// ---- text writers (calc_intW.F:1006-1158, calc_intJ.F:925-1030, wrt_mvmc_*.f90) ----
static FILE *open_w(const std::string &p) {
  FILE *f = std::fopen(p.c_str(), "w");
  if (!f) fail(1, "cannot write %s", p.c_str());
  return f;
}

// '(i5,i5,2f20.10)' blocks after a list-directed "R1 R2 R3" line
static void wr_matrix(const std::string &path, const char *title, const char *cols, int nwf, const int *na, const int *lo,
                      const int *hi, const std::vector<cd> &M /* (i,j,R) box */) {
  FILE *f = open_w(path);
  const int n1 = 2 * na[0] + 1, n2 = 2 * na[1] + 1;
  std::fprintf(f, "%s\n#1:R1, 2:R2, 3:R3 (lattice vector)\n%s\n", title, cols);
  for (int a1 = lo[0]; a1 <= hi[0]; a1++)
    for (int a2 = lo[1]; a2 <= hi[1]; a2++)
      for (int a3 = lo[2]; a3 <= hi[2]; a3++) {
        std::fprintf(f, " %11d %11d %11d\n", a1, a2, a3);
        const size_t R = (size_t)(a1 + na[0]) + n1 * ((size_t)(a2 + na[1]) + (size_t)n2 * (a3 + na[2]));
        for (int i = 0; i < nwf; i++)
          for (int j = 0; j < nwf; j++) {
            const cd v = M[(R * nwf + j) * nwf + i] * rp::kAu;
            std::fprintf(f, "%5d%5d%20.10f%20.10f\n", i + 1, j + 1, v.real(), v.imag());
          }
        std::fprintf(f, "\n");
      }
  std::fclose(f);
}

static void wr_vs_r(const std::string &dir, const char *stem, const char *title, const char *cols, const rp::Setup &S,
                    const int *na, const std::vector<cd> &M) {
  const int nwf = S.nwf, n1 = 2 * na[0] + 1, n2 = 2 * na[1] + 1;
  for (int i = 0; i < nwf; i++) {
    FILE *f = open_w(dir + fmt("/%s.%03d", stem, i + 1));
    std::fprintf(f, "%s\n%s\n", title, cols);
    for (int a1 = -na[0]; a1 <= na[0]; a1++)
      for (int a2 = -na[1]; a2 <= na[1]; a2++)
        for (int a3 = -na[2]; a3 <= na[2]; a3++)
          for (int j = 0; j < nwf; j++) {
            double r[3];
            for (int d = 0; d < 3; d++)
              r[d] = (double)a1 * S.a[0][d] + (double)a2 * S.a[1][d] + (double)a3 * S.a[2][d] +
                     (S.wan_center[3 * j + d] - S.wan_center[3 * i + d]);
            const double rr = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
            const size_t R = (size_t)(a1 + na[0]) + n1 * ((size_t)(a2 + na[1]) + (size_t)n2 * (a3 + na[2]));
            const cd v = M[(R * nwf + j) * nwf + i] * rp::kAu;
            std::fprintf(f, "%12.5f%12.5f%12.5f\n", rr * kBohr, v.real(), v.imag());
          }
    std::fclose(f);
  }
}

static void wr_vs_e(const std::string &dir, const char *stem, const char *title, const char *cols, const rp_int *c,
                    int box, const std::vector<cd> &M /* box x ne */) {
  const int nwf = c->S.nwf;
  const size_t R0 = (size_t)(box - 1) / 2;
  for (int i = 0; i < nwf; i++)
    for (int j = i; j < nwf; j++) {
      FILE *f = open_w(dir + fmt("/%s.%03d-%03d", stem, i + 1, j + 1));
      std::fprintf(f, "%s\n%s\n", title, cols);
      for (int e = 0; e < c->ne; e++) {
        const cd w = c->em[e] * rp::kAu, v = M[(((size_t)e * box + R0) * nwf + j) * nwf + i] * rp::kAu;
        std::fprintf(f, "%12.5f%12.5f%12.5f%12.5f\n", w.real(), w.imag(), v.real(), v.imag());
      }
      std::fclose(f);
    }
}

static void rwind(int &t, int N, int L, bool even) {
  if (even) { if (t < -N + 1) t += L; if (t > N) t -= L; }
  else { if (t < -N) t += L; if (t > N) t -= L; }
}

// wrt_mvmc (wrt_mvmc_w3d.f90, wrt_mvmc_j3d.f90): the interaction on the
// nkb1 x nkb2 x nkb3 supercell, pairs with |H| >= cut
static void wr_mvmc(const std::string &dir, const rp_int *c, const int *na, double cut, const cd *HR, bool exchange) {
  const rp::Setup &S = c->S;
  const int nwf = S.nwf, L2 = S.nkb[1], L3 = S.nkb[2], Nsite = S.ntk;
  const int n1 = 2 * na[0] + 1, n2 = 2 * na[1] + 1;
  const bool even = Nsite % 2 == 0;
  const int off = even ? 1 : 0;
  std::vector<cd> H((size_t)nwf * nwf * Nsite * Nsite, cd(0, 0));
  auto HH = [&](int a, int b, int is, int js) -> cd & { return H[(((size_t)js * Nsite + is) * nwf + b) * nwf + a]; };
  for (int i1 = -na[0] + off; i1 <= na[0]; i1++)
    for (int i2 = -na[1] + off; i2 <= na[1]; i2++)
      for (int i3 = -na[2] + off; i3 <= na[2]; i3++) {
        const long is = (i3 + na[2] - off) + (long)(i2 + na[1] - off) * L3 + (long)(i1 + na[0] - off) * L3 * L2;
        for (int j1 = -na[0] + off; j1 <= na[0]; j1++)
          for (int j2 = -na[1] + off; j2 <= na[1]; j2++)
            for (int j3 = -na[2] + off; j3 <= na[2]; j3++) {
              const long js = (j3 + na[2] - off) + (long)(j2 + na[1] - off) * L3 + (long)(j1 + na[0] - off) * L3 * L2;
              int t1 = j1 - i1, t2 = j2 - i2, t3 = j3 - i3;
              rwind(t1, na[0], S.nkb[0], even); rwind(t2, na[1], S.nkb[1], even); rwind(t3, na[2], S.nkb[2], even);
              if (is < 0 || is >= Nsite || js < 0 || js >= Nsite) continue;
              if (std::abs(t1) > na[0] || std::abs(t2) > na[1] || std::abs(t3) > na[2]) continue;
              const size_t R = (size_t)(t1 + na[0]) + n1 * ((size_t)(t2 + na[1]) + (size_t)n2 * (t3 + na[2]));
              for (int b = 0; b < nwf; b++)
                for (int a = 0; a < nwf; a++) HH(a, b, (int)is, (int)js) = HR[(R * nwf + b) * nwf + a];
            }
      }
  const char *eq = "==============================";
  if (!exchange) {
    FILE *f = open_w(dir + "/zCoulombIntra.def");
    std::fprintf(f, "%s\n%-13s%17d\n%s\n%s\n%s\n", eq, "NCoulombIntra", Nsite * nwf, eq, eq, eq);
    for (int is = 0; is < Nsite; is++)
      for (int b = 0; b < nwf; b++) std::fprintf(f, "%5d%15.10f\n", b + is * nwf, HH(b, b, is, is).real() * rp::kAu);
    std::fclose(f);
  }
  struct Out { const char *file, *key; int w1, w2; bool pairhop; };
  std::vector<Out> outs;
  if (!exchange) outs.push_back({"zCoulombInter.def", "NCoulombInter", 13, 17, false});
  else {
    outs.push_back({"zHund.def", "NHund", 5, 25, false});
    outs.push_back({"zExchange.def", "NExchange", 9, 21, false});
    outs.push_back({"zPairHop.def", "NPairhop", 8, 22, true});
  }
  for (const Out &o : outs) {
    long cnt = 0;
    for (int pass = 0; pass < 2; pass++) {
      FILE *f = nullptr;
      if (pass == 1) {
        f = open_w(dir + "/" + o.file);
        std::fprintf(f, "%s\n%-*s%*ld\n%s\n%s%10.5f%s\n%s\n", eq, o.w1, o.key, o.w2, cnt, eq,
                     exchange ? "=== Jcut >" : "=== Vcut >", cut * rp::kAu, "eV =======", eq);
      }
      for (int is = 0; is < Nsite; is++)
        for (int b = 0; b < nwf; b++) {
          const int i = b + is * nwf;
          for (int js = 0; js < Nsite; js++)
            for (int cb = 0; cb < nwf; cb++) {
              const int j = cb + js * nwf;
              if (o.pairhop ? (j == i) : (i >= j)) continue;
              const cd h = HH(b, cb, is, js);
              if (std::abs(h) < cut) continue;
              if (pass == 0) cnt++;
              else std::fprintf(f, "%5d%5d%15.10f\n", i, j, h.real() * rp::kAu);
            }
        }
      if (f) std::fclose(f);
    }
  }
}

static void rm_tree(const std::string &dir) {
  const std::string cmd = "rm -rf '" + dir + "'";
  if (std::system(cmd.c_str()) != 0) fail(1, "cannot clear %s", dir.c_str());
}
static void mk_dir(const std::string &dir) {
  if (mkdir(dir.c_str(), 0755) != 0 && errno != EEXIST) fail(1, "cannot create %s", dir.c_str());
}

// calc_w3d: V and W on the R box (calc_intW.F:647-1006)
static void int_w3d(rp_int *c, std::vector<cd> &Vh, std::vector<cd> &Wh) {
  rp::Setup &S = c->S;
  cudaStream_t st = c->st;
  const int nwf = S.nwf, ne = c->ne, ntq = c->ntq, ntk = S.ntk;
  int na[3];
  const int box = box_of(c, na);
  float ms[4] = {0, 0, 0, 0};
  const size_t nw2 = (size_t)nwf * nwf;
  c->fq.ensure(sizeof(double2) * ntq * nw2);
  c->fw.ensure(sizeof(double2) * (size_t)ne * ntq * nw2);
  std::vector<int> pv(nwf), pa(nw2), pb(nw2);
  for (int i = 0; i < nwf; i++) pv[i] = i;
  for (int j = 0; j < nwf; j++)
    for (int i = 0; i < nwf; i++) { pa[(size_t)j * nwf + i] = i; pb[(size_t)j * nwf + i] = j; }
  const std::vector<cd> one(ntk, cd(1, 0));
  for (int iq = 0; iq < ntq; iq++) {
    int_q_rho(c, iq, pv, pv, 0, one, 1, &ms[0], &ms[1]);
    int_q_forms(c, iq, false, nwf, pa, pb, c->fq.as<double2>() + (size_t)iq * nw2,
                c->fw.as<double2>() + (size_t)iq * nw2, (size_t)ntq * nw2, &ms[2]);
  }
  // Hybertsen-Louie heads (calc_intW.F:778-795)
  const double qsz = qsz_of(c);
  std::vector<double> chead(1, (2.0 / rp::kPi) * qsz), cheadw(ne);
  for (int e = 0; e < ne; e++) cheadw[e] = ((2.0 / rp::kPi) * c->eps00[e] * qsz).real();
  // q -> R (calc_intW.F:942-985)
  std::vector<cd> pf((size_t)ntq * box);
  for (int iq = 0; iq < ntq; iq++) {
    const double *q = &c->sq[3 * iq];
    int R = 0;
    for (int a3 = -na[2]; a3 <= na[2]; a3++)
      for (int a2 = -na[1]; a2 <= na[1]; a2++)
        for (int a1 = -na[0]; a1 <= na[0]; a1++, R++) {
          const double phase = rp::kTpi * (q[0] * (double)a1 + q[1] * (double)a2 + q[2] * (double)a3);
          pf[(size_t)iq * box + R] = std::exp(cd(0, -1) * phase);
        }
  }
  put(c->pfR, pf, st);
  std::vector<double> heads(chead);
  heads.insert(heads.end(), cheadw.begin(), cheadw.end());
  put(c->head, heads, st);
  c->out.ensure(sizeof(double2) * (size_t)(1 + ne) * box * nw2);
  const double scale = 2.0 * rp::kTpi / S.volume / (double)ntq;
  RP_CUDA(cudaEventRecord(c->ev[0], st));
  c->launches += rp::launch_int_fourier(c->fq.as<double2>(), c->pfR.as<double2>(), ntq, box, nwf, 1, scale,
                                        c->head.as<double>(), c->out.as<double2>(), st);
  c->launches += rp::launch_int_fourier(c->fw.as<double2>(), c->pfR.as<double2>(), ntq, box, nwf, ne, scale,
                                        c->head.as<double>() + 1, c->out.as<double2>() + (size_t)box * nw2, st);
  RP_CUDA(cudaEventRecord(c->ev[1], st));
  RP_CUDA(cudaEventSynchronize(c->ev[1]));
  RP_CUDA(cudaEventElapsedTime(&ms[3], c->ev[0], c->ev[1]));
  std::vector<cd> all;
  get(all, c->out, (size_t)(1 + ne) * box * nw2, st);
  Vh.assign(all.begin(), all.begin() + (size_t)box * nw2);
  Wh.assign(all.begin() + (size_t)box * nw2, all.end());
  for (int i = 0; i < 4; i++) c->times[i] = ms[i] * 1e-3;
  c->times[4] = c->times[0] + c->times[1] + c->times[2] + c->times[3];
  if (c->P.write_files) {
    const std::string dir = c->root + "/dir-intW";
    rm_tree(dir);
    mk_dir(dir);
    const int lo[3] = {-na[0], -na[1], -na[2]};
    const std::vector<cd> Wi(Wh.begin() + (size_t)(c->P.calc_ifreq - 1) * box * nw2,
                             Wh.begin() + (size_t)c->P.calc_ifreq * box * nw2);
    wr_matrix(dir + "/dat.Vmat", "#Bare Coulomb: V", "#1:i, 2:j, 3:Re(V_ij) [eV], 4:Im(V_ij) [eV]", nwf, na, lo, na, Vh);
    wr_matrix(dir + "/dat.Wmat", "#Screened Coulomb: W at omega=calc_ifreq", "#1:i, 2:j, 3:Re(W_ij) [eV], 4:Im(W_ij) [eV]",
              nwf, na, lo, na, Wi);
    wr_vs_r(dir, "dat.VvsR", "#R dependence of bare Coulomb", "#1:R [AA], 2:Re[V(R)] [eV], 3:Im[V(R)] [eV]", S, na, Vh);
    wr_vs_r(dir, "dat.WvsR", "#R dependence of screened Coulomb at omega=calc_ifreq",
            "#1:R [AA], 2:Re[W(R)] [eV], 3:Im[W(R)] [eV]", S, na, Wi);
    wr_vs_e(dir, "dat.UvsE", "#Omega dependence of onsite Coulomb",
            "#1:Re(w) [eV], 2:Im(w) [eV], 3:Re[U(w)] [eV], 4:Im[U(w)] [eV]", c, box, Wh);
    const std::string mv = c->root + "/dir-mvmc";
    mk_dir(mv);
    wr_mvmc(mv, c, na, c->P.wcut_mvmc / rp::kAu, Wi.data(), false);
  }
}

// calc_j3d: X and J on the IX/IY/IZ range of R (calc_intJ.F:609-905)
static void int_j3d(rp_int *c, std::vector<cd> &Xh, std::vector<cd> &Jh) {
  rp::Setup &S = c->S;
  cudaStream_t st = c->st;
  const int nwf = S.nwf, ne = c->ne, ntq = c->ntq, ntk = S.ntk;
  int na[3];
  const int box = box_of(c, na);
  const int lo[3] = {c->P.ix_intj_min, c->P.iy_intj_min, c->P.iz_intj_min};
  const int hi[3] = {c->P.ix_intj_max, c->P.iy_intj_max, c->P.iz_intj_max};
  for (int d = 0; d < 3; d++)
    if (lo[d] > hi[d] || lo[d] < -na[d] || hi[d] > na[d])
      fail(1, "intJ range %d..%d of direction %d is outside -%d..%d", lo[d], hi[d], d + 1, na[d], na[d]);
  std::vector<int> Rs;
  for (int a1 = lo[0]; a1 <= hi[0]; a1++)
    for (int a2 = lo[1]; a2 <= hi[1]; a2++)
      for (int a3 = lo[2]; a3 <= hi[2]; a3++) { Rs.push_back(a1); Rs.push_back(a2); Rs.push_back(a3); }
  const int nr = (int)Rs.size() / 3, np = nwf * nwf, nv = nr * np;
  std::vector<cd> pf((size_t)nr * ntk);
  for (int r = 0; r < nr; r++)
    for (int k = 0; k < ntk; k++) {
      const double *sk = &S.sk0[3 * k];
      pf[(size_t)r * ntk + k] =
          std::exp(cd(0, -1) * rp::kTpi * (sk[0] * (double)Rs[3 * r] + sk[1] * (double)Rs[3 * r + 1] + sk[2] * (double)Rs[3 * r + 2]));
    }
  // pair p = j*nwf + i: rho of w_i at k+q against w_j at k (calc_intJ.F:651-664)
  std::vector<int> pv(np), po(np), pa(nv);
  for (int j = 0; j < nwf; j++)
    for (int i = 0; i < nwf; i++) { pv[(size_t)j * nwf + i] = i; po[(size_t)j * nwf + i] = j; }
  for (int v = 0; v < nv; v++) pa[v] = v;
  c->fq.ensure(sizeof(double2) * nv);
  c->fw.ensure(sizeof(double2) * (size_t)ne * nv);
  std::vector<cd> fsum(nv, cd(0, 0)), fwsum((size_t)ne * nv, cd(0, 0)), tmp;
  float ms[4] = {0, 0, 0, 0};
  for (int iq = 0; iq < ntq; iq++) {
    const double *q = &c->sq[3 * iq];
    const bool gamma = q[0] == 0.0 && q[1] == 0.0 && q[2] == 0.0;
    if (gamma && iq >= c->nq_irr) fail(1, "Gamma is not among the irreducible q points");
    int_q_rho(c, iq, pv, po, 1, pf, nr, &ms[0], &ms[1]);
    // Gamma reads eps^-1 of the same index directly (calc_intJ.F:818)
    int_q_forms(c, iq, gamma, nv, pa, pa, c->fq.as<double2>(), c->fw.as<double2>(), (size_t)nv, &ms[2]);
    get(tmp, c->fq, nv, st);
    for (int v = 0; v < nv; v++) fsum[v] += tmp[v];
    get(tmp, c->fw, (size_t)ne * nv, st);
    for (size_t x = 0; x < tmp.size(); x++) fwsum[x] += tmp[x];
  }
  const size_t nw2 = (size_t)nwf * nwf;
  Xh.assign((size_t)box * nw2, cd(0, 0));
  Jh.assign((size_t)ne * box * nw2, cd(0, 0));
  const int n1 = 2 * na[0] + 1, n2 = 2 * na[1] + 1;
  for (int r = 0; r < nr; r++) {
    const size_t R = (size_t)(Rs[3 * r] + na[0]) + n1 * ((size_t)(Rs[3 * r + 1] + na[1]) + (size_t)n2 * (Rs[3 * r + 2] + na[2]));
    for (int p = 0; p < np; p++) {
      Xh[R * nw2 + p] = 2.0 * rp::kTpi * fsum[(size_t)r * np + p] / S.volume / (double)ntq;
      for (int e = 0; e < ne; e++)
        Jh[((size_t)e * box + R) * nw2 + p] = 2.0 * rp::kTpi * fwsum[(size_t)e * nv + (size_t)r * np + p] / S.volume / (double)ntq;
    }
  }
  // Hybertsen-Louie head on the R = 0 diagonal (calc_intJ.F:876-905)
  const double qsz = qsz_of(c), chead = (2.0 / rp::kPi) * qsz;
  const size_t R0 = (size_t)(box - 1) / 2;
  for (int i = 0; i < nwf; i++) {
    Xh[R0 * nw2 + (size_t)i * nwf + i] += chead;
    for (int e = 0; e < ne; e++)
      Jh[((size_t)e * box + R0) * nw2 + (size_t)i * nwf + i] += ((2.0 / rp::kPi) * c->eps00[e] * qsz).real();
  }
  for (int i = 0; i < 4; i++) c->times[i] = ms[i] * 1e-3;
  c->times[4] = c->times[0] + c->times[1] + c->times[2] + c->times[3];
  if (c->P.write_files) {
    const std::string dir = c->root + "/dir-intJ";
    rm_tree(dir);
    mk_dir(dir);
    const std::vector<cd> Ji(Jh.begin() + (size_t)(c->P.calc_ifreq - 1) * box * nw2,
                             Jh.begin() + (size_t)c->P.calc_ifreq * box * nw2);
    wr_matrix(dir + "/dat.Xmat", "#Bare exchamge: X", "#1:i, 2:j, 3:Re(X_ij) [eV], 4:Im(X_ij) [eV]", nwf, na, lo, hi, Xh);
    wr_matrix(dir + "/dat.Jmat", "#Screened exchamge: J at omega=calc_ifreq", "#1:i, 2:j, 3:Re(J_ij) [eV], 4:Im(J_ij) [eV]",
              nwf, na, lo, hi, Ji);
    wr_vs_e(dir, "dat.JvsE", "#Omega dependence of screened exchange J",
            "#Re(w) [eV], Im(w) [eV], Re[J(w)] [eV], Im[J(w)] [eV]", c, box, Jh);
    const std::string mv = c->root + "/dir-mvmc";
    mk_dir(mv);
    wr_mvmc(mv, c, na, c->P.jcut_mvmc / rp::kAu, Ji.data(), true);
  }
}

// ---- C ABI ----
extern "C" {

void rp_int_default_params(rp_int_params *p) {
  std::memset(p, 0, sizeof *p);
  p->calc_ifreq = 1;  // m_rdinput.f90 (calc_int):20-29
  p->wcut_mvmc = 2.0;
  p->jcut_mvmc = 0.3;
  p->write_files = 1;
  p->read_eps_f32 = 1;
}

int rp_int_parse_namelist(const char *text, rp_int_params *p) {
  return guarded_int(nullptr, [&] { rp::parse_calc_int_namelist(text ? text : "", p); });
}

int rp_int_create(rp_int **out, const char *root, const rp_int_params *p) {
  *out = nullptr;
  rp_int *c = new rp_int();
  int rc = guarded_int(c, [&] { int_create(c, root, p); });
  if (rc) {
    g_int_err = c->err;
    delete c;
    return rc;
  }
  *out = c;
  return 0;
}

int rp_int_dims(const rp_int *c, int *nwf, int *ne, int *ntq, int *na3) {
  if (!c) return 1;
  if (nwf) *nwf = c->S.nwf;
  if (ne) *ne = c->ne;
  if (ntq) *ntq = c->ntq;
  if (na3) for (int d = 0; d < 3; d++) na3[d] = c->S.nkb[d] / 2;
  return 0;
}

int rp_int_w3d(rp_int *c, double *V, double *W) {
  return guarded_int(c, [&] {
    std::vector<cd> Vh, Wh;
    int_w3d(c, Vh, Wh);
    if (V) std::memcpy(V, Vh.data(), sizeof(cd) * Vh.size());
    if (W) std::memcpy(W, Wh.data(), sizeof(cd) * Wh.size());
  });
}

int rp_int_j3d(rp_int *c, double *X, double *J) {
  return guarded_int(c, [&] {
    std::vector<cd> Xh, Jh;
    int_j3d(c, Xh, Jh);
    if (X) std::memcpy(X, Xh.data(), sizeof(cd) * Xh.size());
    if (J) std::memcpy(J, Jh.data(), sizeof(cd) * Jh.size());
  });
}

int rp_int_stage_times(const rp_int *c, double *t5) {
  if (!c) return 1;
  for (int i = 0; i < 5; i++) t5[i] = c->times[i];
  return 0;
}

const char *rp_int_last_error(const rp_int *c) { return c ? c->err.c_str() : g_int_err.c_str(); }

void rp_int_destroy(rp_int *c) { delete c; }

static int run_program(const char *root, const char *text, bool j) {
  rp_int_params p;
  rp_int_default_params(&p);
  int rc = rp_int_parse_namelist(text, &p);
  if (rc) return rc;
  rp_int *c = nullptr;
  rc = rp_int_create(&c, root, &p);
  if (rc) return rc;
  rc = j ? rp_int_j3d(c, nullptr, nullptr) : rp_int_w3d(c, nullptr, nullptr);
  if (rc) g_int_err = c->err;
  rp_int_destroy(c);
  return rc;
}

int rp_calc_w3d(const char *root, const char *namelist_text) { return run_program(root, namelist_text, false); }
int rp_calc_j3d(const char *root, const char *namelist_text) { return run_program(root, namelist_text, true); }

}  // extern "C"
