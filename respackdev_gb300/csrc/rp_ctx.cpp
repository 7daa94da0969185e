// rp_ctx.cpp -- the context behind the C ABI (include/respack_gb300.h).
//
// A context owns one CUDA stream and the device-resident data of a run: the
// irreducible wave-function coefficients, the unfolding map, and -- computed
// once -- the full-mesh coefficients and their real-space periodic parts.  Per
// q point it uploads the small task tables (G sphere, k+q map, band pairs) and
// runs, in band-pair batches sized for HBM:
//   tetrahedron weights -> pair densities -> contraction (FP64 or tensor-core)
// then the dielectric matrix build and inversion.  Results stay on the device
// until the caller asks for a host copy or the dir-eps files.
#include <sys/stat.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "rp_dev.cuh"
#include "rp_host.h"
#include "rp_tc.h"

namespace {

using rp::cd;

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  void ensure(size_t n) {
    if (n <= bytes) return;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    if (n == 0) return;
    RP_CUDA(cudaMalloc(&p, n));
    bytes = n;
  }
  template <typename T> T *as() const { return (T *)p; }
  void release() { if (p) cudaFree(p); p = nullptr; bytes = 0; }
};

// bytes copied host->device and device->host by the calling thread; the C-ABI
// calls add the change over each call to their context's totals
thread_local long long t_h2d = 0, t_d2h = 0;

template <typename T> void upload(DevBuf &b, const std::vector<T> &v, cudaStream_t st) {
  b.ensure(std::max<size_t>(sizeof(T) * v.size(), 16));
  if (!v.empty()) RP_CUDA(cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st));
  t_h2d += (long long)(sizeof(T) * v.size());
}

}  // namespace

struct rp_ctx {
  rp::Setup S;
  rp::UnfoldMap U;
  std::string root;
  int dev = 0;
  cudaStream_t st = nullptr;
  std::string err;
  long long launches = 0;
  int R[3]{};  // psi-sphere extent per dimension
  // persistent device data
  DevBuf coef, numirr, trs, src, phase, ng0, kg0, cfull, ur, energy, prob, imt1, index2, em, b9, sk0, errw, inc_off,
      inc;
  // real-space functions in slots when every band does not fit: the occupied
  // bands resident (slots 0..n_fixed-1), a window of nwin slots that each pair
  // batch fills with its virtual bands; h_slot_of / slot_of map band -> slot
  bool ur_window = false;
  bool wfn_fp32 = false;  // the real-space transforms run in FP32 (split precisions)
  int n_fixed = 0, nwin = 0, nslot = 0;
  std::vector<int> h_slot_of;
  DevBuf slot_of, win_bands;
  // per-q device data
  DevBuf kpq, shift, lg0, qglen, pvir, pocc, chunk_vir, chunk_first, chunk_count, pair_list, wts, rho, head, chi,
      rowcol, A, eps, prow, piv, used, intra, pwpl, mixws, mixaux;
  rp::TcWorkspace tcw;
  // band-tail network (&param_gpu tail_model): the network, its shell count and
  // target scale, the excluded-band statistics, and the per-q shell map,
  // features and whether the last rp_chi0_q applied it
  rp_mlp *tail = nullptr;
  int tail_nshell = 0;
  float tail_scale = 1.f, tail_stats[3]{};
  DevBuf tail_sh, tail_x;
  bool tail_done = false;
  rp::QTask task;
  int ndir = 1;
  double wd[3]{};
  bool have_chi = false, have_eps = false;
  bool eps_fallback = false;  // the last rp_epsinv_q fell back to the FP64 inversion
  std::vector<cd> h_chi, h_eps;
  static constexpr int NSLOT = 4;  // pinned staging slots of device->host copies (one per host thread)
  void *stage = nullptr;           // NSLOT slots of 8 MB
  cudaEvent_t sev[NSLOT]{};        // completion of each slot's copy
  cudaEvent_t ev[6]{};
  double times[6]{};
  long long h2d = 0, d2h = 0;  // bytes moved between host and device by this context's calls
  ~rp_ctx() {
    for (DevBuf *b : {&coef, &numirr, &trs, &src, &phase, &ng0, &kg0, &cfull, &ur, &energy, &prob, &imt1, &index2, &em,
                      &b9, &sk0, &errw, &inc_off, &inc, &kpq, &shift, &lg0, &qglen, &pvir, &pocc, &chunk_vir, &chunk_first,
                      &chunk_count, &pair_list, &wts, &rho, &head, &chi, &rowcol, &A, &eps, &prow, &piv, &used,
                      &intra, &pwpl, &mixws, &mixaux, &tail_sh, &tail_x, &slot_of, &win_bands})
      b->release();
    tcw.release();
    if (tail) rp_mlp_destroy(tail);
    for (auto &e : ev) if (e) cudaEventDestroy(e);
    for (auto &e : sev) if (e) cudaEventDestroy(e);
    if (stage) cudaFreeHost(stage);
    if (st) cudaStreamDestroy(st);
  }
};

static thread_local std::string g_create_err;

// error text of calls that have no context (read by rp_last_error(NULL))
void rp::set_global_error(const std::string &msg) { g_create_err = msg; }
void rp::note_transfer(long long h2d, long long d2h) { t_h2d += h2d; t_d2h += d2h; }

template <typename F> static int guarded(rp_ctx *ctx, F &&f) {
  const long long h0 = t_h2d, d0 = t_d2h;
  struct Count {
    rp_ctx *c; long long h0, d0;
    ~Count() { if (c) { c->h2d += t_h2d - h0; c->d2h += t_d2h - d0; } }
  } count{ctx, h0, d0};
  try {
    f();
    return 0;
  } catch (const rp::Error &e) {
    if (ctx) ctx->err = e.msg; else g_create_err = e.msg;
    return e.code;
  } catch (const std::bad_alloc &) {
    if (ctx) ctx->err = "host out of memory"; else g_create_err = "host out of memory";
    return -2;
  }
}

static void check_device_error(rp_ctx *c) {
  int e = 0;
  RP_CUDA(cudaMemcpyAsync(&e, c->errw.p, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  RP_CUDA(cudaStreamSynchronize(c->st));
  t_d2h += sizeof(int);
  if (e == 1) rp::fail(-3, "ntet.gt.nmax: a tetrahedron was cut into too many pieces");
  if (e == 2) rp::fail(-3, "tetrahedron degeneracy classification failed (bad i3 / bad sum ia2)");
  if (e == 3) rp::fail(-3, "dielectric matrix is singular");
  if (e == 4) rp::fail(-3, "tensor-core contraction: wait limit reached");
  if (e == 5) rp::fail(-3, "a tetrahedron is cut by the Fermi level although no band is partially occupied");
}

// The band-tail network file written by respackdev_gb300.tail.TailMLP.save:
// int32 magic "RPTL", version 1, nin, nhid, nout, nshell; float32 target scale,
// one float32 of padding; then the nparams float32 parameters in rp_mlp's order.
static void load_tail(rp_ctx *c, const std::string &path) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) rp::fail(1, "cannot open the band-tail network %s", path.c_str());
  int32_t h[6];
  float sc[2];
  const bool ok = fread(h, 4, 6, f) == 6 && fread(sc, 4, 2, f) == 2;
  if (!ok || h[0] != 0x4c545052 || h[1] != 1) { fclose(f); rp::fail(1, "%s is not a band-tail network file", path.c_str()); }
  if (h[2] != 9 || h[4] != 2 || h[5] < 1 || h[5] > 256 || !(sc[0] > 0.f)) {
    fclose(f);
    rp::fail(1, "%s: a band-tail network takes 9 features and gives 2 outputs per shell", path.c_str());
  }
  rp_mlp *m = nullptr;
  int rc = rp_mlp_create(&m, h[2], h[3], h[4], 0, c->dev);
  if (rc) { fclose(f); rp::fail(rc, "band-tail network: %s", rp_last_error(nullptr)); }
  std::vector<float> prm((size_t)rp_mlp_nparams(m));
  if (fread(prm.data(), 4, prm.size(), f) != prm.size()) {
    fclose(f);
    rp_mlp_destroy(m);
    rp::fail(1, "%s: short parameter block", path.c_str());
  }
  fclose(f);
  rc = rp_mlp_set_params(m, prm.data());
  if (rc) { rp_mlp_destroy(m); rp::fail(rc, "band-tail network: cannot upload its parameters"); }
  c->tail = m;
  c->tail_nshell = h[5];
  c->tail_scale = sc[0];
  // the excluded bands (N_CALC_BAND+1 .. NTB) over the listed k points, as tail.band_stats
  const rp::Setup &S = c->S;
  if (S.ncb >= S.ntb) rp::fail(1, "tail_model needs N_CALC_BAND below the number of bands (%d)", S.ntb);
  double lo = 1e300, sum = 0.0;
  long n = 0;
  for (int ib = S.ncb; ib < S.ntb; ib++)
    for (int ik = 0; ik < S.nk_irr; ik++) {
      const double e = S.e_eigi[(size_t)ik * S.ntb + ib] - S.efermi;
      lo = std::min(lo, e);
      sum += e;
      n++;
    }
  c->tail_stats[0] = (float)lo;
  c->tail_stats[1] = (float)(sum / (double)n);
  c->tail_stats[2] = (float)((double)(S.ntb - S.ncb) / (double)std::max(S.ncb, 1));
}

// Shells of the G of a q (equal-count quantiles of |q+G| > 0, -1 for the head)
// and the network's correction of the diagonal of chi0 (rp_tail.cu).
static void tail_apply(rp_ctx *c, const rp::QTask &t, DevBuf &chi, int nen, int ndir) {
  c->tail_done = false;
  if (!c->tail) return;
  const int ng = t.ng, ns = c->tail_nshell;
  std::vector<int> ok, sh(ng, -1);
  std::vector<double> key(ng);
  for (int g = 0; g < ng; g++) {
    if (t.qglen[g] > 0) ok.push_back(g);
    // |q+G| rounded to 2^-30 (to nearest even, as numpy's rint): lengths equal by
    // symmetry tie, and ties keep the G order, as respackdev_gb300.tail.shells
    key[g] = std::nearbyint(t.qglen[g] * 1073741824.0);
  }
  std::stable_sort(ok.begin(), ok.end(), [&](int a, int b) { return key[a] < key[b]; });
  const long n = (long)ok.size();
  for (long i = 0; i < n; i++) sh[ok[i]] = (int)std::min<long>((i * ns) / std::max<long>(n, 1), ns - 1);
  cudaStream_t st = c->st;
  upload(c->tail_sh, sh, st);
  upload(c->qglen, t.qglen, st);  // another q of this context may have replaced it (ragged batches)
  c->tail_x.ensure(sizeof(float) * (size_t)nen * ns * 9);
  c->launches += rp::launch_tail_features(chi.as<double2>(), ng, nen, c->tail_sh.as<int>(), c->qglen.as<double>(), ns,
                                          c->em.as<double2>(), c->tail_stats, c->tail_x.as<float>(), st);
  const float *y = rp::mlp_forward_device(c->tail, c->tail_x.as<float>(), nen * ns, st);
  c->launches += 3;
  c->launches += rp::launch_tail_apply(chi.as<double2>(), ng, nen, ndir, c->tail_sh.as<int>(), c->qglen.as<double>(),
                                       ns, y, c->tail_scale, st);
  c->tail_done = true;
}

static void create_ctx(rp_ctx *c, const char *root, const rp_params *p, const double *em, int nen_explicit) {
  c->root = root ? root : ".";
  c->S.params = *p;
  RP_CUDA(cudaSetDevice(p->device));
  c->dev = p->device;
  RP_CUDA(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
  for (auto &e : c->ev) RP_CUDA(cudaEventCreate(&e));
  std::vector<double> emx;
  for (int i = 0; i < 2 * nen_explicit; i++) emx.push_back(em[i]);
  rp::read_dir_wfn(c->S, c->root);
  rp::finish_setup(c->S, emx);
  rp::read_wfn_coefficients(c->S, c->root);
  if (p->flg_crpa == 1) rp::read_dir_wan_crpa(c->S, c->root);
  rp::build_unfold_map(c->S, c->U);
  rp::Setup &S = c->S;
  for (int d = 0; d < 3; d++) c->R[d] = 0;
  for (int j = 0; j < S.ntk; j++)
    for (int ig = 0; ig < S.ng0[j]; ig++)
      for (int d = 0; d < 3; d++) c->R[d] = std::max(c->R[d], std::abs(S.kg0[((size_t)j * S.ntg + ig) * 3 + d]));
  cudaStream_t st = c->st;
  upload(c->coef, S.coef, st);
  upload(c->numirr, S.numirr, st);
  upload(c->trs, S.trs, st);
  upload(c->src, c->U.src, st);
  upload(c->phase, c->U.phase, st);
  upload(c->ng0, S.ng0, st);
  upload(c->kg0, S.kg0, st);
  upload(c->energy, S.e_eigi, st);
  upload(c->prob, S.prob, st);
  upload(c->imt1, S.imt1, st);
  {
    // the tetrahedra around each mesh slot (4*tetrahedron + vertex position), for
    // the gathered weights of the split precisions
    std::vector<int> off(S.ntk + 1, 0), inc(S.imt1.size());
    for (int sl : S.imt1) off[sl + 1]++;
    for (int m = 0; m < S.ntk; m++) off[m + 1] += off[m];
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (size_t i = 0; i < S.imt1.size(); i++) inc[fill[S.imt1[i]]++] = (int)i;
    upload(c->inc_off, off, st);
    upload(c->inc, inc, st);
  }
  std::vector<int> idx2(S.index_kpt);
  idx2.insert(idx2.end(), S.mesh_of_k.begin(), S.mesh_of_k.end());
  upload(c->index2, idx2, st);
  upload(c->em, S.em, st);
  std::vector<double> b9(9);
  for (int i = 0; i < 3; i++)
    for (int d = 0; d < 3; d++) b9[3 * i + d] = S.b[i][d];
  upload(c->b9, b9, st);
  upload(c->sk0, S.sk0, st);
  c->errw.ensure(16);
  RP_CUDA(cudaMemsetAsync(c->errw.p, 0, 16, st));
  const size_t N = (size_t)S.nw[0] * S.nw[1] * S.nw[2];
  c->cfull.ensure(sizeof(cd) * (size_t)S.ntk * S.ncb * S.ntg);
  // every band's real-space functions when they fit beside a 48 GB working set
  // (pair batches, tensor-core operands, eps); otherwise the occupied bands and
  // a window of virtual bands that each pair batch fills
  const size_t per_band = sizeof(float) * 2 * (size_t)S.ntk * N;
  size_t freeb = 0, totb = 0;
  RP_CUDA(cudaMemGetInfo(&freeb, &totb));
  const size_t reserve = (size_t)48 << 30;
  const size_t avail = freeb > reserve ? freeb - reserve : 0;
  rp::WfnSlots sl;
  // the split precisions transform in FP32 (then round to single, as both
  // paths do); the FP64 precision and pair_fp64 keep the FP64 passes
  sl.fp32 = p->precision != RP_PREC_FP64 && !p->pair_fp64;
  c->wfn_fp32 = sl.fp32;
  if (p->ur_window > 0 || per_band * (size_t)S.ncb > avail) {
    c->ur_window = true;
    c->n_fixed = S.n_occ;
    int nw = p->ur_window;
    if (nw <= 0) {
      // a third of what is left: a window larger than one 24 GB pair batch
      // can use would only take memory
      const size_t fixed = per_band * (size_t)c->n_fixed;
      nw = avail > fixed ? (int)std::min<size_t>((avail - fixed) / 3 / per_band, (size_t)1 << 20) : 0;
    }
    c->nwin = std::min(nw, S.ncb - c->n_fixed);
    if (c->nwin < 1 && S.ncb > c->n_fixed)
      rp::fail(-2, "device memory holds no window of virtual-band real-space functions (%.1f GB free)",
               (double)freeb / 1e9);
    c->nslot = c->n_fixed + std::max(c->nwin, 0);
    c->h_slot_of.assign(S.ncb, -1);
    for (int b = 0; b < c->n_fixed; b++) c->h_slot_of[b] = b;
    upload(c->slot_of, c->h_slot_of, st);
    sl.slot_of = c->slot_of.as<int>();
    sl.nslot = c->nslot;
    c->ur.ensure(per_band * (size_t)c->nslot);
  } else {
    c->ur.ensure(per_band * (size_t)S.ncb);
  }
  c->launches += rp::launch_wfn_realspace(c->coef.as<double2>(), c->numirr.as<int>(), c->trs.as<int>(),
                                          c->src.as<int>(), c->phase.as<double2>(), c->ng0.as<int>(),
                                          c->kg0.as<int>(), S.ntk, S.ncb, S.ntg, S.nw[0], S.nw[1], S.nw[2], c->R[0],
                                          c->R[1], c->R[2], c->cfull.as<double2>(), c->ur.as<float2>(), 0, S.ntk, st,
                                          sl);
  RP_CUDA(cudaStreamSynchronize(st));
  if (p->tail_model[0]) {
    char path[sizeof p->tail_model + 1];
    std::memcpy(path, p->tail_model, sizeof p->tail_model);
    path[sizeof p->tail_model] = 0;
    std::string tp(path);
    if (tp[0] != '/') tp = c->root + "/" + tp;  // relative to the run directory
    load_tail(c, tp);
  }
}

// Band pairs of one batch grouped by virtual band into chunks of <= jmax.
static void build_chunks(const std::vector<int> &pvir, const std::vector<int> &pocc, int jmax,
                         std::vector<int> &cv, std::vector<int> &cf, std::vector<int> &cc, std::vector<int> &plist) {
  std::map<int, std::vector<int>> by;
  for (size_t p = 0; p < pvir.size(); p++) by[pvir[p]].push_back((int)p);
  cv.clear(); cf.clear(); cc.clear(); plist.clear();
  for (auto &kv : by) {
    const auto &v = kv.second;
    for (size_t s = 0; s < v.size(); s += jmax) {
      cv.push_back(kv.first);
      cf.push_back((int)plist.size());
      int n = (int)std::min<size_t>(jmax, v.size() - s);
      cc.push_back(n);
      for (int i = 0; i < n; i++) plist.push_back(v[s + i]);
    }
  }
  (void)pocc;
}

// One q point while its chi0 is computed: the task, where chi0 accumulates,
// the pair batches and the stage timings.  The single-q path keeps these in
// the context; a ragged batch (rp_chi0_batch) keeps one per problem.
struct QRun {
  int iq = 0;
  bool fast = false;
  rp::QTask *t = nullptr;
  DevBuf *chi = nullptr, *rowcol = nullptr;
  int ndir = 1, ng = 0, nen = 0, ntk = 0, jmax = 8, npair = 0;
  int ep[3]{};
  std::vector<int> ord, bstart;
  float tms[4]{};
};

static void upload_qtables(rp_ctx *c, const rp::QTask &t) {
  upload(c->kpq, t.kpq, c->st);
  upload(c->shift, t.shift, c->st);
  upload(c->lg0, t.lg0, c->st);
  upload(c->qglen, t.qglen, c->st);
}

// Tables of the q, chi0 zeroed, the pair batches planned.
static void q_begin(rp_ctx *c, QRun &r) {
  rp::Setup &S = c->S;
  cudaStream_t st = c->st;
  rp::QTask &t = *r.t;
  r.ndir = t.gamma ? 3 : 1;
  r.ng = t.ng; r.nen = (int)S.em.size(); r.ntk = S.ntk;
  const int ng = r.ng, nen = r.nen, ntk = r.ntk;
  upload_qtables(c, t);
  RP_CUDA(cudaMemsetAsync(c->errw.p, 0, 16, st));
  const size_t chisz = (size_t)r.ndir * nen * ng * ng;
  r.chi->ensure(sizeof(cd) * chisz);
  RP_CUDA(cudaMemsetAsync(r.chi->p, 0, sizeof(cd) * chisz, st));
  if (t.gamma) {
    r.rowcol->ensure(sizeof(cd) * 4 * (size_t)nen * ng);
    RP_CUDA(cudaMemsetAsync(r.rowcol->p, 0, sizeof(cd) * 4 * (size_t)nen * ng, st));
  }
  for (int d = 0; d < 3; d++) {
    int m = 0;
    for (int g = 0; g < ng; g++) m = std::max(m, std::abs(t.lg0[3 * g + d]));
    r.ep[d] = m;
  }
  // pair batches: per pair the densities, weights and Gamma heads plus the
  // contraction's operand rows, weights and three planes; one batch per q
  // while that fits in 24 GB (the bench workload needs about 14 GB)
  const int npair = r.npair = (int)t.pair_vir.size();
  const size_t per_pair = (size_t)ntk * (ng * sizeof(cd) + nen * sizeof(cd) + 3 * sizeof(cd) +
                                         2 * (size_t)((ng + 127) / 128 * 128) * (sizeof(float) + 6) +
                                         2 * (size_t)nen * 8);
  const size_t budget = (size_t)24 << 30;
  int bsz = (int)std::max<size_t>(1, std::min<size_t>(npair, budget / std::max<size_t>(per_pair, 1)));
  if (S.params.pair_batch > 0) bsz = std::min(bsz, S.params.pair_batch);
  // shared-memory limit of the pair-density tile decides how many pairs share one virtual band load
  int jmax = 8;
  auto smem_of = [&](int j, size_t elt) {
    rp::PairGeom gq;
    gq.n1 = S.nw[0]; gq.n2 = S.nw[1]; gq.n3 = S.nw[2]; gq.R1 = r.ep[0]; gq.R2 = r.ep[1]; gq.ng = ng;
    return rp::pair_density_smem(gq, j, elt == sizeof(double) * 2);
  };
  const size_t elt = (r.fast && !S.params.pair_fp64) ? sizeof(float) * 2 : sizeof(double) * 2;
  while (jmax > 1 && smem_of(jmax, elt) > 220 * 1024) jmax--;
  if (smem_of(jmax, elt) > 220 * 1024) rp::fail(1, "dielectric sphere (NG=%d) too large for the pair-density tile", ng);
  r.jmax = jmax;
  // pairs grouped by virtual band (stable in the occupied band); a batch takes
  // whole groups while they fit, so every pair-density chunk (pairs sharing a
  // virtual band) is as full as jmax allows.  chi is a sum over pairs: the
  // order changes only the rounding.
  r.ord.resize(npair);
  for (int i = 0; i < npair; i++) r.ord[i] = i;
  std::stable_sort(r.ord.begin(), r.ord.end(), [&](int a, int b) { return t.pair_vir[a] < t.pair_vir[b]; });
  // With a real-space window, a batch also holds at most nwin virtual bands
  // outside the resident ones.
  r.bstart.assign(1, 0);
  int nvb = 0;
  for (int i = 0; i < npair;) {
    int j = i;
    while (j < npair && t.pair_vir[r.ord[j]] == t.pair_vir[r.ord[i]]) j++;  // group [i, j)
    const int cur = i - r.bstart.back();
    const bool windowed = c->ur_window && t.pair_vir[r.ord[i]] >= c->n_fixed;
    if (cur > 0 && (cur + (j - i) > bsz || (windowed && nvb + 1 > c->nwin))) {
      r.bstart.push_back(i);                                                // group starts a new batch
      nvb = 0;
    }
    for (int s0 = i + bsz; s0 < j; s0 += bsz) r.bstart.push_back(s0);      // a group larger than a batch
    if (windowed) nvb = (j - i > bsz) ? 1 : nvb + 1;
    i = j;
  }
  r.bstart.push_back(npair);
  for (float &x : r.tms) x = 0;
}

static int q_nbatch(const QRun &r) { return (int)r.bstart.size() - 1; }
static int q_batch_pairs(const QRun &r, int bi) { return r.bstart[bi + 1] - r.bstart[bi]; }

// Pair batch bi: tetrahedron weights, pair densities and the contraction.  With
// run_gram false (tensor-core precisions only) the batch is prepared in ws and
// its Gram launch is left to the caller.
static void q_batch(rp_ctx *c, QRun &r, int bi, rp::TcWorkspace *ws, bool run_gram) {
  rp::Setup &S = c->S;
  cudaStream_t st = c->st;
  rp::QTask &t = *r.t;
  const int ng = r.ng, nen = r.nen, ntk = r.ntk;
  const int n1 = S.nw[0], n2 = S.nw[1], n3 = S.nw[2];
  const int p0 = r.bstart[bi], nb = r.bstart[bi + 1] - p0;
  if (nb <= 0) return;
  std::vector<int> bv(nb), bo(nb);
  for (int i = 0; i < nb; i++) { bv[i] = t.pair_vir[r.ord[p0 + i]]; bo[i] = t.pair_occ[r.ord[p0 + i]]; }
  std::vector<int> cv, cf, cc, pl;
  build_chunks(bv, bo, r.jmax, cv, cf, cc, pl);
  upload(c->pvir, bv, st);
  upload(c->pocc, bo, st);
  upload(c->chunk_vir, cv, st);
  upload(c->chunk_first, cf, st);
  upload(c->chunk_count, cc, st);
  upload(c->pair_list, pl, st);
  // tetrahedron weights
  rp::TetraArgs ta;
  ta.ntk = ntk; ta.nen = nen; ta.ntb = S.ntb; ta.imt1 = c->imt1.as<int>(); ta.index_kpt = c->index2.as<int>();
  ta.numirr = c->numirr.as<int>(); ta.kpq = c->kpq.as<int>(); ta.energy = c->energy.as<double>();
  ta.prob = c->prob.as<double2>(); ta.em = c->em.as<double2>(); ta.pair_vir = c->pvir.as<int>();
  ta.pair_occ = c->pocc.as<int>(); ta.npair = nb; ta.efermi = S.efermi; ta.delt = S.delt; ta.dmna = S.dmna;
  ta.dmnr = S.dmnr; ta.err = c->errw.as<int>();
  ta.inc_off = c->inc_off.as<int>(); ta.inc = c->inc.as<int>(); ta.may_cut = S.n_pocc > 0 ? 1 : 0;
  c->wts.ensure(sizeof(cd) * (size_t)nb * nen * ntk);
  RP_CUDA(cudaEventRecord(c->ev[0], st));
  // the split precisions take the FP32 series where it converges; the plain
  // FP64 path keeps the reference's closed forms everywhere
  c->launches += rp::launch_tetra_weights(ta, c->wts.as<double2>(), st, r.fast && !S.params.tetra_fp64);
  RP_CUDA(cudaEventRecord(c->ev[1], st));
  rp::PairGeom pg;
  pg.ntk = ntk; pg.ncb = S.ncb; pg.n1 = n1; pg.n2 = n2; pg.n3 = n3; pg.ng = ng;
  pg.kpq = c->kpq.as<int>(); pg.shift = c->shift.as<int>(); pg.lg0 = c->lg0.as<int>();
  pg.R1 = r.ep[0]; pg.R2 = r.ep[1]; pg.R3 = r.ep[2];
  if (c->ur_window) {
    // this batch's virtual bands into the window (counted with the pair densities)
    std::vector<int> wb;
    for (int v : cv)
      if (v >= c->n_fixed && c->h_slot_of[v] < 0 && std::find(wb.begin(), wb.end(), v) == wb.end()) wb.push_back(v);
    for (int b = c->n_fixed; b < S.ncb; b++) c->h_slot_of[b] = -1;
    for (size_t i = 0; i < wb.size(); i++) c->h_slot_of[wb[i]] = c->n_fixed + (int)i;
    if ((int)wb.size() > c->nwin) rp::fail(-2, "pair batch holds %zu virtual bands for %d window slots", wb.size(), c->nwin);
    upload(c->slot_of, c->h_slot_of, st);
    upload(c->win_bands, wb, st);
    rp::WfnSlots sl;
    sl.bands = c->win_bands.as<int>();
    sl.nbands = (int)wb.size();
    sl.slot_of = c->slot_of.as<int>();
    sl.nslot = c->nslot;
    sl.rotate = false;
    sl.fp32 = c->wfn_fp32;
    c->launches += rp::launch_wfn_realspace(c->coef.as<double2>(), c->numirr.as<int>(), c->trs.as<int>(),
                                            c->src.as<int>(), c->phase.as<double2>(), c->ng0.as<int>(),
                                            c->kg0.as<int>(), S.ntk, S.ncb, S.ntg, n1, n2, n3, c->R[0], c->R[1],
                                            c->R[2], c->cfull.as<double2>(), c->ur.as<float2>(), 0, S.ntk, st, sl);
    pg.slot_of = c->slot_of.as<int>();
    pg.nslot = c->nslot;
  }
  rp::PairChunks pc;
  pc.chunk_vir = c->chunk_vir.as<int>(); pc.chunk_first = c->chunk_first.as<int>();
  pc.chunk_count = c->chunk_count.as<int>(); pc.pair_list = c->pair_list.as<int>();
  pc.pair_occ = c->pocc.as<int>(); pc.nchunk = (int)cv.size(); pc.jmax = r.jmax;
  if (t.gamma) {
    c->head.ensure(sizeof(cd) * 3 * (size_t)nb * ntk);
    c->launches += rp::launch_gamma_head(c->cfull.as<double2>(), c->ng0.as<int>(), c->kg0.as<int>(), ntk, S.ncb,
                                         S.ntg, c->b9.as<double>(), c->energy.as<double>(), S.ntb,
                                         c->numirr.as<int>(), c->pvir.as<int>(), c->pocc.as<int>(), nb, S.delt,
                                         c->head.as<double2>(), st);
  }
  double2 *chi = r.chi->as<double2>();
  double2 *rowcol = t.gamma ? r.rowcol->as<double2>() : nullptr;
  if (!r.fast) {
    c->rho.ensure(sizeof(cd) * (size_t)nb * ntk * ng);
    c->launches += rp::launch_pair_density_fp64(c->ur.as<float2>(), pg, pc, c->rho.as<double2>(), st);
    RP_CUDA(cudaEventRecord(c->ev[2], st));
    if (t.gamma) {
      c->launches += rp::launch_gamma_rowcol(c->rho.as<double2>(), c->wts.as<double2>(), c->head.as<double2>(), nb,
                                             ntk, ng, nen, t.no_g0, rowcol, st);
      c->launches += rp::launch_set_head(c->rho.as<double2>(), c->head.as<double2>(), nb, ntk, ng, t.no_g0, 0, st);
    }
    c->launches += rp::launch_contract_fp64(c->rho.as<double2>(), c->wts.as<double2>(), nb, ntk, ng, nen, chi, st);
  } else {
    const bool p64 = S.params.pair_fp64 != 0;
    c->rho.ensure((p64 ? sizeof(cd) : sizeof(float) * 2) * (size_t)nb * ntk * ng);
    if (p64) c->launches += rp::launch_pair_density_fp64(c->ur.as<float2>(), pg, pc, c->rho.as<double2>(), st);
    else c->launches += rp::launch_pair_density_fp32(c->ur.as<float2>(), pg, pc, c->rho.as<float2>(), st);
    RP_CUDA(cudaEventRecord(c->ev[2], st));
    if (p64 && t.gamma)
      c->launches += rp::launch_gamma_rowcol(c->rho.as<double2>(), c->wts.as<double2>(), c->head.as<double2>(), nb,
                                             ntk, ng, nen, t.no_g0, rowcol, st);
    const float2 *rho32 = p64 ? nullptr : c->rho.as<float2>();
    const double2 *rho64 = p64 ? c->rho.as<double2>() : nullptr;
    const double2 *head = t.gamma ? c->head.as<double2>() : nullptr;
    if (run_gram)
      c->launches += rp::tc_contract_batch(*ws, rho32, rho64, c->wts.as<double2>(), head, nb, ntk, ng, nen, t.no_g0,
                                           S.params.precision, chi, rowcol, c->errw.as<int>(), st);
    else
      c->launches += rp::tc_prepare(*ws, rho32, rho64, c->wts.as<double2>(), head, nb, ntk, ng, nen, t.no_g0,
                                    S.params.precision, rowcol, c->errw.as<int>(), st);
  }
  RP_CUDA(cudaEventRecord(c->ev[3], st));
  RP_CUDA(cudaEventSynchronize(c->ev[3]));
  float a = 0, b = 0, d = 0;
  RP_CUDA(cudaEventElapsedTime(&a, c->ev[0], c->ev[1]));
  RP_CUDA(cudaEventElapsedTime(&b, c->ev[1], c->ev[2]));
  RP_CUDA(cudaEventElapsedTime(&d, c->ev[2], c->ev[3]));
  r.tms[0] += a; r.tms[1] += b; r.tms[2] += d;
}

// Gamma's directions 2 and 3, the 1/VOLUME scale and the Drude term.
static void q_end(rp_ctx *c, QRun &r) {
  rp::Setup &S = c->S;
  cudaStream_t st = c->st;
  rp::QTask &t = *r.t;
  const int ng = r.ng, nen = r.nen, ntk = r.ntk;
  const size_t chisz = (size_t)r.ndir * nen * ng * ng;
  // Gamma: directions 2 and 3 share the body of direction 1 and get their own G=0 row/column
  if (t.gamma) {
    const size_t m = (size_t)nen * ng * ng;
    double2 *chi = r.chi->as<double2>();
    RP_CUDA(cudaMemcpyAsync(chi + m, chi, sizeof(cd) * m, cudaMemcpyDeviceToDevice, st));
    RP_CUDA(cudaMemcpyAsync(chi + 2 * m, chi, sizeof(cd) * m, cudaMemcpyDeviceToDevice, st));
    std::vector<cd> rc(4 * (size_t)nen * ng);
    RP_CUDA(cudaMemcpyAsync(rc.data(), r.rowcol->p, sizeof(cd) * rc.size(), cudaMemcpyDeviceToHost, st));
    t_d2h += (long long)(sizeof(cd) * rc.size());
    RP_CUDA(cudaStreamSynchronize(st));
    for (int ix = 1; ix <= 2; ix++)
      for (int e = 0; e < nen; e++) {
        const cd *row = &rc[(((size_t)(ix - 1) * nen + e) * 2) * ng], *col = row + ng;
        double2 *base = chi + (size_t)ix * m + (size_t)e * ng * ng;
        // row G0: element (G0, g') at G0 + ng*g'; column G0: element (g, G0) at g + ng*G0
        std::vector<double2> rr(ng), cl(ng);
        for (int g = 0; g < ng; g++) { rr[g] = make_double2(row[g].real(), row[g].imag()); cl[g] = make_double2(col[g].real(), col[g].imag()); }
        RP_CUDA(cudaMemcpy2DAsync(base + t.no_g0, sizeof(double2) * ng, rr.data(), sizeof(double2), sizeof(double2), ng,
                                  cudaMemcpyHostToDevice, st));
        RP_CUDA(cudaMemcpyAsync(base + (size_t)ng * t.no_g0, cl.data(), sizeof(double2) * ng, cudaMemcpyHostToDevice, st));
        t_h2d += (long long)(2 * sizeof(double2) * ng);
        RP_CUDA(cudaStreamSynchronize(st));
      }
  }
  c->launches += rp::launch_scale(r.chi->as<double2>(), chisz, S.volume, st);
  // Drude plasma frequency from the intraband pairs (metals, fRPA only)
  c->wd[0] = c->wd[1] = c->wd[2] = 0;
  if (t.gamma && !t.intra_band.empty()) {
    upload_qtables(c, t);  // another q of this context may have replaced them (ragged batches)
    upload(c->intra, t.intra_band, st);
    c->pwpl.ensure(sizeof(cd) * 3);
    RP_CUDA(cudaMemsetAsync(c->pwpl.p, 0, sizeof(cd) * 3, st));
    rp::TetraArgs ta;
    ta.ntk = ntk; ta.nen = nen; ta.ntb = S.ntb; ta.imt1 = c->imt1.as<int>(); ta.index_kpt = c->index2.as<int>();
    ta.numirr = c->numirr.as<int>(); ta.kpq = c->kpq.as<int>(); ta.energy = c->energy.as<double>();
    ta.prob = c->prob.as<double2>(); ta.em = c->em.as<double2>(); ta.pair_vir = nullptr; ta.pair_occ = nullptr;
    ta.npair = 0; ta.efermi = S.efermi; ta.delt = S.delt; ta.dmna = S.dmna; ta.dmnr = S.dmnr;
    ta.err = c->errw.as<int>();
    c->launches += rp::launch_intraband(ta, c->cfull.as<double2>(), c->ng0.as<int>(), c->kg0.as<int>(), S.ncb,
                                        S.ntg, c->b9.as<double>(), c->sk0.as<double>(), c->intra.as<int>(),
                                        (int)t.intra_band.size(), c->pwpl.as<double2>(), st);
    cd pw[3];
    RP_CUDA(cudaMemcpyAsync(pw, c->pwpl.p, sizeof(cd) * 3, cudaMemcpyDeviceToHost, st));
    t_d2h += (long long)(sizeof(cd) * 3);
    RP_CUDA(cudaStreamSynchronize(st));
    for (int d = 0; d < 3; d++) {
      cd wpl = 8.0 * pw[d] / S.volume / (double)ntk;
      c->wd[d] = std::sqrt(wpl.real());
    }
  }
  RP_CUDA(cudaEventRecord(c->ev[4], st));
  check_device_error(c);
}

static void chi0_q(rp_ctx *c, int iq, bool fast) {
  rp::Setup &S = c->S;
  c->have_chi = c->have_eps = false;
  c->task = rp::make_qtask(S, iq - 1, S.params.max_pairs);
  QRun r;
  r.iq = iq; r.fast = fast; r.t = &c->task; r.chi = &c->chi; r.rowcol = &c->rowcol;
  q_begin(c, r);
  c->ndir = r.ndir;
  RP_CUDA(cudaEventRecord(c->ev[5], c->st));
  if (fast) {
    c->tcw.ksub = S.params.tc_ksub;
    c->tcw.pair_req = S.params.tc_pair;
    rp::tc_begin_q(c->tcw, r.ng, r.nen, r.ndir, S.params.tc_split, (long)r.npair * r.ntk, S.params.precision, c->st);
  }
  for (int bi = 0; bi < q_nbatch(r); bi++) q_batch(c, r, bi, &c->tcw, true);
  if (fast) c->launches += rp::tc_end_q(c->tcw, c->chi.as<double2>(), nullptr, c->st);
  q_end(c, r);
  tail_apply(c, c->task, c->chi, r.nen, r.ndir);
  float tot = 0;
  RP_CUDA(cudaEventElapsedTime(&tot, c->ev[5], c->ev[4]));
  c->times[0] = r.tms[0] * 1e-3; c->times[1] = r.tms[1] * 1e-3; c->times[2] = r.tms[2] * 1e-3;
  c->times[4] = tot * 1e-3;
  c->times[5] = fast ? c->tcw.gram_seconds : 0.0;
  c->have_chi = true;
}

static void epsinv_run(rp_ctx *c) {
  if (!c->have_chi) rp::fail(1, "rp_epsinv_q needs a preceding rp_chi0_q");
  rp::QTask &t = c->task;
  const int ng = t.ng, nen = (int)c->S.em.size(), nmat = c->ndir * nen;
  const size_t sz = (size_t)nmat * ng * ng;
  cudaStream_t st = c->st;
  c->A.ensure(sizeof(cd) * sz);
  c->eps.ensure(sizeof(cd) * sz);
  c->prow.ensure(rp::gauss_jordan_scratch_bytes(ng, nmat));  // the Gauss-Jordan panels' pivot rows
  c->piv.ensure(sizeof(int) * (size_t)nmat * ng);
  c->used.ensure(sizeof(int) * (size_t)nmat * ng);
  rp::EpsArgs a;
  a.ng = ng; a.nen = nen; a.ndir = c->ndir; a.gamma = t.gamma; a.g0 = t.no_g0; a.qglen = c->qglen.as<double>();
  a.em = c->em.as<double2>(); a.delt = c->S.delt;
  for (int d = 0; d < 3; d++) a.wd[d] = c->wd[d];
  RP_CUDA(cudaEventRecord(c->ev[0], st));
  c->launches += rp::launch_eps_build(c->chi.as<double2>(), a, c->A.as<double2>(), st);
  bool fp64 = c->S.params.precision == RP_PREC_FP64 || c->S.params.eps_fp64 != 0;
  c->eps_fallback = false;
  if (!fp64) {
    // FP32 Gauss-Jordan plus one float-pair Newton step; its own singular flag and
    // per-matrix |R|_F^2 decide whether the FP64 inversion has to run instead
    c->mixws.ensure(rp::epsinv_mixed_bytes(ng, nmat));
    c->mixaux.ensure(sizeof(float) * nmat + sizeof(int));
    float *rn = c->mixaux.as<float>();
    int *ferr = (int *)(rn + nmat);
    RP_CUDA(cudaMemsetAsync(ferr, 0, sizeof(int), st));
    c->launches += rp::launch_epsinv_mixed(c->A.as<double2>(), ng, nmat, c->mixws.p, c->piv.as<int>(),
                                           c->used.as<int>(), c->eps.as<double2>(), rn, ferr, st);
    std::vector<float> h(nmat + 1);
    RP_CUDA(cudaMemcpyAsync(h.data(), rn, sizeof(float) * (nmat + 1), cudaMemcpyDeviceToHost, st));
    RP_CUDA(cudaStreamSynchronize(st));
    t_d2h += (long long)(sizeof(float) * (nmat + 1));
    int fe;
    std::memcpy(&fe, &h[nmat], sizeof(int));
    bool ok = fe == 0;
    for (int m = 0; m < nmat; m++) ok = ok && h[m] <= 1.0e-6f;  // |R|_F <= 1e-3, so |error| <~ 1e-6 |A^-1|
    c->eps_fallback = !ok;
    fp64 = !ok;
  }
  if (fp64)
    c->launches += rp::launch_gauss_jordan(c->A.as<double2>(), ng, nmat, c->prow.as<double2>(), c->piv.as<int>(),
                                           c->used.as<int>(), c->eps.as<double2>(), c->errw.as<int>(), st);
  RP_CUDA(cudaEventRecord(c->ev[1], st));
  check_device_error(c);
  float ms = 0;
  RP_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
  c->times[3] = ms * 1e-3;
  c->have_eps = true;
}

// Device -> host copy of `bytes` into any host memory.  Chunks go through
// pinned slots, one per host thread: thread t copies chunks t, t + T, ... --
// device copy into its slot, then the host copy out of it -- so the host
// copies (and the first touch of fresh pageable pages) run in parallel and
// overlap the device copies of the other threads' chunks.
static void fetch_to(rp_ctx *c, const void *src, void *dst, size_t bytes) {
  constexpr size_t CH = (size_t)8 << 20;
  if (!c->stage) {
    RP_CUDA(cudaMallocHost(&c->stage, rp_ctx::NSLOT * CH));
    for (auto &e : c->sev) RP_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  const size_t n = (bytes + CH - 1) / CH;
  const int T = (int)std::min<size_t>(rp_ctx::NSLOT, n);
  std::exception_ptr errs[rp_ctx::NSLOT];
  auto worker = [&](int t) {
    try {
      RP_CUDA(cudaSetDevice(c->dev));
      char *slot = (char *)c->stage + (size_t)t * CH;
      for (size_t j = (size_t)t; j < n; j += (size_t)T) {
        const size_t o = j * CH, len = std::min(CH, bytes - o);
        RP_CUDA(cudaMemcpyAsync(slot, (const char *)src + o, len, cudaMemcpyDeviceToHost, c->st));
        RP_CUDA(cudaEventRecord(c->sev[t], c->st));
        RP_CUDA(cudaEventSynchronize(c->sev[t]));
        std::memcpy((char *)dst + o, slot, len);
      }
    } catch (...) {
      errs[t] = std::current_exception();
    }
  };
  {
    std::vector<std::thread> th;
    for (int t = 1; t < T; t++) th.emplace_back(worker, t);
    if (T > 0) worker(0);
    for (auto &x : th) x.join();
  }
  for (int t = 0; t < T; t++)
    if (errs[t]) std::rethrow_exception(errs[t]);
  t_d2h += (long long)bytes;
}

static size_t result_elems(const rp_ctx *c) { return (size_t)c->ndir * c->S.em.size() * c->task.ng * c->task.ng; }

static void fetch(rp_ctx *c, DevBuf &b, std::vector<cd> &h) {
  h.resize(result_elems(c));
  fetch_to(c, b.p, h.data(), sizeof(cd) * h.size());
}

static void mkdir_p(const std::string &p) { mkdir(p.c_str(), 0755); }

static void write_q(rp_ctx *c, const std::string &root) {
  if (!c->have_eps) rp::fail(1, "rp_write_q needs rp_chi0_q and rp_epsinv_q first");
  rp::Setup &S = c->S;
  rp::QTask &t = c->task;
  const int ng = t.ng, nen = (int)S.em.size();
  fetch(c, c->eps, c->h_eps);
  int qnum = -1;
  for (int ik = 0; ik < S.nk_irr; ik++)
    if (std::fabs(S.ski_list[3 * ik] - t.q[0]) < 1e-6 && std::fabs(S.ski_list[3 * ik + 1] - t.q[1]) < 1e-6 &&
        std::fabs(S.ski_list[3 * ik + 2] - t.q[2]) < 1e-6)
      qnum = ik + 1;
  char buf[64];
  snprintf(buf, sizeof buf, "q%03d", qnum);
  const std::string epsdir = root + "/dir-eps", qdir = epsdir + "/" + buf;
  mkdir_p(epsdir);
  mkdir_p(qdir);
  if (S.params.dump_chi) {
    fetch(c, c->chi, c->h_chi);
    FILE *f = fopen((qdir + "/dat.chi0").c_str(), "wb");
    if (!f) rp::fail(1, "cannot write %s/dat.chi0", qdir.c_str());
    int32_t hdr[4] = {ng, nen, c->ndir, (int32_t)t.pair_vir.size()};
    fwrite(hdr, 4, 4, f);
    fwrite(c->h_chi.data(), sizeof(cd), c->h_chi.size(), f);
    fclose(f);
  }
  {
    FILE *f = fopen((qdir + "/dat.sq").c_str(), "w");
    if (!f) rp::fail(1, "cannot write %s/dat.sq", qdir.c_str());
    fprintf(f, " %24.16E %24.16E %24.16E\n", t.q[0], t.q[1], t.q[2]);
    fclose(f);
  }
  const size_t m = (size_t)nen * ng * ng;
  for (int ix = 0; ix < c->ndir; ix++) {
    const int base = S.params.file_num_eps_base_start + ix * 1000;
    for (int e = 0; e < nen; e++) {
      snprintf(buf, sizeof buf, "/dat.epsqw.%06d", base + e + 1);
      FILE *f = fopen((qdir + buf).c_str(), "w");
      if (!f) rp::fail(1, "cannot write %s%s", qdir.c_str(), buf);
      fprintf(f, "#epsqw diagonal term\n#1:q+G [au], 2:Re(eps-1), 3:Im(eps-1)\n");
      const cd *E = &c->h_eps[ix * m + (size_t)e * ng * ng];
      for (int g = 0; g < ng; g++)
        fprintf(f, "%20.10f%20.10f%20.10f\n", t.qglen[g], E[g + (size_t)ng * g].real(), E[g + (size_t)ng * g].imag());
      fclose(f);
    }
    snprintf(buf, sizeof buf, "/dat.epsqw.%03d", S.params.file_num_eps_start + ix);
    rp::write_unformatted_record(qdir + buf, &c->h_eps[ix * m], sizeof(cd) * m);
  }
  if (S.params.write_eps_f32) {
    // what calc_int keeps of eps^-1 (epsirr, complex(4); calc_intW.F:587-630):
    // at Gamma the mean of the three directions, summed and divided in the
    // order its reader uses, so reading this file gives the same values at
    // half the bytes of one FP64 record
    std::vector<float> c4(2 * m);
    for (size_t i = 0; i < m; i++) {
      cd acc(0.0, 0.0);
      for (int ix = 0; ix < c->ndir; ix++) acc += c->h_eps[ix * m + i];
      if (c->ndir == 3) acc = acc / 3.0;
      c4[2 * i] = (float)acc.real();
      c4[2 * i + 1] = (float)acc.imag();
    }
    rp::write_unformatted_record(qdir + "/dat.epsqw.c4", c4.data(), sizeof(float) * c4.size());
  }
  // the completion flag is written last, so an interrupted run resumes at this q
  snprintf(buf, sizeof buf, "/dat.log.%03d", S.params.file_num_log_start);
  FILE *f = fopen((qdir + buf).c_str(), "w");
  if (!f) rp::fail(1, "cannot write %s%s", qdir.c_str(), buf);
  fprintf(f, " #\n #finish chi0 evaluation for %11d\n #\n", qnum);
  fclose(f);
}

extern "C" {

int rp_ctx_create(rp_ctx **out, const char *root, const rp_params *p, const double *em, int nen_explicit) {
  if (!out || !p) return 1;
  *out = nullptr;
  std::unique_ptr<rp_ctx> c(new rp_ctx());
  int rc = guarded(nullptr, [&] { create_ctx(c.get(), root, p, em, nen_explicit); });
  if (rc) return rc;
  *out = c.release();
  return 0;
}

int rp_ctx_info(const rp_ctx *c, rp_info *info) {
  if (!c || !info) return 1;
  const rp::Setup &S = c->S;
  info->ntk = S.ntk; info->nk_irr = S.nk_irr; info->ntg = S.ntg; info->ntb = S.ntb; info->ncb = S.ncb;
  for (int d = 0; d < 3; d++) { info->nkb[d] = S.nkb[d]; info->fft_box[d] = S.nw[d]; }
  info->nen = (int)S.em.size();
  info->n_occ = S.n_occ; info->n_vir = S.n_vir; info->n_docc = S.n_docc; info->n_pocc = S.n_pocc; info->n_uocc = S.n_uocc;
  info->volume = S.volume; info->efermi = S.efermi; info->ecut_psi = S.ecut_psi; info->ecut_eps = S.ecut_eps;
  double bytes = 0;
  for (const DevBuf *b : {&c->coef, &c->cfull, &c->ur, &c->wts, &c->rho, &c->chi, &c->A, &c->eps, &c->src, &c->phase,
                          &c->kg0})
    bytes += (double)b->bytes;
  info->device_bytes = bytes + (double)c->tcw.bytes();
  return 0;
}

int rp_num_qirr(const rp_ctx *c) { return c ? c->S.nk_irr : 0; }

int rp_chi0_q(rp_ctx *c, int iq, double *chi, int *ng_out, int *ndir_out) {
  if (!c) return 1;
  return guarded(c, [&] {
    RP_CUDA(cudaSetDevice(c->dev));
    chi0_q(c, iq, c->S.params.precision != RP_PREC_FP64);
    if (ng_out) *ng_out = c->task.ng;
    if (ndir_out) *ndir_out = c->ndir;
    if (chi) {
      fetch_to(c, c->chi.p, chi, sizeof(cd) * result_elems(c));
    }
  });
}

int rp_chi0_batch(rp_ctx *const *ctxs, const int *iqs, int n, int use_graph, double *const *chi, int *ng_out,
                  int *ndir_out, double *seconds) {
  if (!ctxs || !iqs || n <= 0 || !ctxs[0]) return 1;
  rp_ctx *c0 = ctxs[0];
  return guarded(c0, [&] {
    struct Prob {
      rp_ctx *c = nullptr;
      rp::QTask task;
      DevBuf chi, rowcol;
      QRun r;
      std::vector<std::unique_ptr<rp::TcWorkspace>> ws;
      ~Prob() {
        chi.release();
        rowcol.release();
        for (auto &w : ws) w->release();
      }
    };
    const int prec = c0->S.params.precision;
    if (prec == RP_PREC_FP64) rp::fail(1, "rp_chi0_batch needs a tensor-core precision");
    for (int i = 0; i < n; i++) {
      rp_ctx *c = ctxs[i];
      if (!c) rp::fail(1, "rp_chi0_batch: context %d is NULL", i);
      if (c->dev != c0->dev) rp::fail(1, "rp_chi0_batch: contexts on different devices");
      if (c->S.params.precision != prec) rp::fail(1, "rp_chi0_batch: contexts with different precisions");
      if (iqs[i] < 1 || iqs[i] > c->S.nk_irr) rp::fail(1, "q index %d outside dat.sample-k (1..%d)", iqs[i], c->S.nk_irr);
    }
    RP_CUDA(cudaSetDevice(c0->dev));
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    std::vector<std::unique_ptr<Prob>> P(n);
    for (int i = 0; i < n; i++) {
      P[i] = std::make_unique<Prob>();
      P[i]->c = ctxs[i];
    }
    // preparation: the problems of one context in order on its stream (they
    // share its pair-density buffers), the contexts concurrently, one host
    // thread each, so small problems of different cells overlap on the GPU
    std::vector<rp_ctx *> uniq;
    for (int i = 0; i < n; i++)
      if (std::find(uniq.begin(), uniq.end(), ctxs[i]) == uniq.end()) uniq.push_back(ctxs[i]);
    std::vector<std::exception_ptr> errs(uniq.size());
    std::vector<long long> h2d(uniq.size(), 0), d2h(uniq.size(), 0);
    auto prepare = [&](size_t u) {
      rp_ctx *c = uniq[u];
      const long long h0 = t_h2d, d0 = t_d2h;
      try {
        RP_CUDA(cudaSetDevice(c->dev));
        c->have_chi = c->have_eps = false;
        for (int i = 0; i < n; i++) {
          if (ctxs[i] != c) continue;
          Prob &p = *P[i];
          p.task = rp::make_qtask(c->S, iqs[i] - 1, c->S.params.max_pairs);
          p.r.iq = iqs[i]; p.r.fast = true; p.r.t = &p.task; p.r.chi = &p.chi; p.r.rowcol = &p.rowcol;
          q_begin(c, p.r);
          for (int bi = 0; bi < q_nbatch(p.r); bi++) {
            auto ws = std::make_unique<rp::TcWorkspace>();
            ws->ksub = c->S.params.tc_ksub;
            ws->pair_req = c->S.params.tc_pair;
            rp::tc_begin_q(*ws, p.r.ng, p.r.nen, p.r.ndir, c->S.params.tc_split,
                           (long)q_batch_pairs(p.r, bi) * p.r.ntk, prec, c->st);
            p.ws.push_back(std::move(ws));
            q_batch(c, p.r, bi, p.ws.back().get(), false);
          }
          check_device_error(c);
        }
      } catch (...) {
        errs[u] = std::current_exception();
      }
      h2d[u] = t_h2d - h0;
      d2h[u] = t_d2h - d0;
    };
    {
      std::vector<std::thread> th;
      for (size_t u = 1; u < uniq.size(); u++) th.emplace_back(prepare, u);
      prepare(0);
      for (auto &x : th) x.join();
    }
    for (size_t u = 1; u < uniq.size(); u++) { t_h2d += h2d[u]; t_d2h += d2h[u]; }
    for (auto &e : errs)
      if (e) std::rethrow_exception(e);
    RP_CUDA(cudaSetDevice(c0->dev));
    const auto t1 = clk::now();
    // one grouped Gram launch over every prepared batch, then each batch into its problem's chi
    std::vector<rp::TcWorkspace *> wl;
    std::vector<double2 *> cl;
    for (auto &p : P)
      for (auto &w : p->ws)
        if (w->ready) { wl.push_back(w.get()); cl.push_back(p->chi.as<double2>()); }
    const double gsec = rp::tc_group_run(wl.data(), (int)wl.size(), cl.data(), c0->errw.as<int>(), c0->st,
                                         use_graph != 0, &c0->launches);
    check_device_error(c0);
    const auto t2 = clk::now();
    for (int i = 0; i < n; i++) {
      Prob &p = *P[i];
      q_end(p.c, p.r);
      tail_apply(p.c, p.task, p.chi, p.r.nen, p.r.ndir);
      if (ng_out) ng_out[i] = p.r.ng;
      if (ndir_out) ndir_out[i] = p.r.ndir;
      if (chi && chi[i]) fetch_to(p.c, p.chi.p, chi[i], sizeof(cd) * (size_t)p.r.ndir * p.r.nen * p.r.ng * p.r.ng);
    }
    const auto t3 = clk::now();
    if (seconds) {
      seconds[0] = std::chrono::duration<double>(t1 - t0).count();
      seconds[1] = gsec;
      seconds[2] = std::chrono::duration<double>(t3 - t2).count();
    }
  });
}

int rp_tuned_shapes(void) { return rp::tc_tuned_shapes(); }
void rp_reset_tuner(void) { rp::tc_reset_tuner(); }

int rp_epsinv_q(rp_ctx *c, double *epsinv) {
  if (!c) return 1;
  return guarded(c, [&] {
    RP_CUDA(cudaSetDevice(c->dev));
    epsinv_run(c);
    if (epsinv) {
      fetch_to(c, c->eps.p, epsinv, sizeof(cd) * result_elems(c));
    }
  });
}

int rp_epsinv_chi_q(rp_ctx *c, const double *chi, double *epsinv) {
  if (!c) return 1;
  return guarded(c, [&] {
    if (!c->have_chi) rp::fail(1, "rp_epsinv_chi_q needs a preceding rp_chi0_q (its q point)");
    if (!chi) rp::fail(1, "rp_epsinv_chi_q: chi is NULL");
    RP_CUDA(cudaSetDevice(c->dev));
    const size_t bytes = sizeof(cd) * result_elems(c);
    RP_CUDA(cudaMemcpyAsync(c->chi.p, chi, bytes, cudaMemcpyHostToDevice, c->st));
    t_h2d += (long long)bytes;
    epsinv_run(c);
    if (epsinv) fetch_to(c, c->eps.p, epsinv, bytes);
  });
}

int rp_tail_applied(const rp_ctx *c) { return c && c->tail_done ? 1 : 0; }

int rp_write_q(rp_ctx *c, const char *root) {
  if (!c) return 1;
  return guarded(c, [&] { write_q(c, root ? root : c->root); });
}

int rp_stage_times(const rp_ctx *c, double *t6) {
  if (!c || !t6) return 1;
  for (int i = 0; i < 6; i++) t6[i] = c->times[i];
  return 0;
}

int rp_q_dims(const rp_ctx *c, int iq, int *ng, int *ndir) {
  if (!c) return 1;
  return guarded(const_cast<rp_ctx *>(c), [&] {
    rp::QTask t = rp::make_qtask(c->S, iq - 1, 1);
    if (ng) *ng = t.ng;
    if (ndir) *ndir = t.gamma ? 3 : 1;
  });
}

long long rp_kernel_launches(const rp_ctx *c) { return c ? c->launches : 0; }

int rp_eps_fallback(const rp_ctx *c) { return c && c->eps_fallback ? 1 : 0; }

int rp_transfer_bytes(const rp_ctx *c, long long *h2d, long long *d2h) {
  if (!c) return 1;
  if (h2d) *h2d = c->h2d;
  if (d2h) *d2h = c->d2h;
  return 0;
}

const char *rp_last_error(const rp_ctx *c) { return c ? c->err.c_str() : g_create_err.c_str(); }

void rp_ctx_destroy(rp_ctx *c) { delete c; }

// q points (0-based) that a calc_chiqw run with parameters p computes in root:
// the manual list or every q without dat.log (chiqw.F:593-608), then this
// process's shard of them (qshard_index of qshard_count, taken modulo).
static std::vector<int> plan_q(const rp::Setup &S, const rp_params &p, const std::vector<int> &qlist,
                               const std::string &root) {
  const std::string epsdir = root + "/dir-eps";
  char buf[64];
  std::vector<int> todo;
  if (p.flg_calc_type == 2) {
    struct stat stt;
    for (int ik : qlist) {
      if (ik < 1 || ik > S.nk_irr) rp::fail(1, "q index %d outside dat.sample-k", ik);
      snprintf(buf, sizeof buf, "/q%03d/dat.log.%03d", ik, p.file_num_log_start);
      if (stat((epsdir + buf).c_str(), &stt) != 0) todo.push_back(ik - 1);
    }
  } else {
    todo = rp::q_list(S, epsdir);
  }
  const int ns = std::max(1, p.qshard_count), si = p.qshard_index;
  if (si < 0 || si >= ns) rp::fail(1, "qshard_index %d outside 0..%d", si, ns - 1);
  std::vector<int> mine;
  for (size_t i = 0; i < todo.size(); i++)
    if ((int)(i % ns) == si) mine.push_back(todo[i]);
  return mine;
}

int rp_plan_q(const char *root, const char *namelist_text, int *qlist, int cap, int *n) {
  return guarded(nullptr, [&] {
    rp_params p;
    rp_default_params(&p);
    std::vector<int> ql;
    std::vector<double> em;
    rp::parse_namelist_text(namelist_text ? namelist_text : "", &p, &ql, &em);
    rp::Setup S;
    S.params = p;
    rp::read_dir_wfn(S, root);
    const std::vector<int> mine = plan_q(S, p, ql, root);
    if (n) *n = (int)mine.size();
    for (int i = 0; i < (int)mine.size() && i < cap && qlist; i++) qlist[i] = mine[i] + 1;
  });
}

int rp_calc_chiqw(const char *root, const char *namelist_text) {
  rp_params p;
  rp_default_params(&p);
  std::vector<int> qlist;
  std::vector<double> em;
  int rc = guarded(nullptr, [&] { rp::parse_namelist_text(namelist_text ? namelist_text : "", &p, &qlist, &em); });
  if (rc) return rc;
  rp_ctx *c = nullptr;
  rc = rp_ctx_create(&c, root, &p, em.data(), (int)em.size() / 2);
  if (rc) return rc;
  rc = guarded(c, [&] {
    rp::Setup &S = c->S;
    const std::string epsdir = std::string(root) + "/dir-eps";
    mkdir_p(epsdir);
    char buf[64];
    for (int ik = 0; ik < S.nk_irr; ik++) { snprintf(buf, sizeof buf, "/q%03d", ik + 1); mkdir_p(epsdir + buf); }
    const std::vector<int> mine = plan_q(S, p, qlist, root);
    // shared files (chiqw.F:1206-1215)
    FILE *f = fopen((epsdir + "/dat.chi_cutoff").c_str(), "w");
    if (f) { fprintf(f, " %24.16E\n", S.ecut_eps); fclose(f); }
    f = fopen((epsdir + "/dat.wgrid").c_str(), "w");
    if (f) {
      fprintf(f, " %11d\n", (int)S.em.size());
      for (auto &e : S.em) fprintf(f, "%15.10f%15.10f\n", e.real(), e.imag());
      fclose(f);
    }
    for (int iq : mine) {
      chi0_q(c, iq + 1, p.precision != RP_PREC_FP64);
      epsinv_run(c);
      write_q(c, root);
    }
  });
  if (rc) g_create_err = c->err;
  rp_ctx_destroy(c);
  return rc;
}

}  // extern "C"
