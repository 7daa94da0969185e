// rp_host.h -- host-side data of the GB300 chiqw library (C++17).
//
// The host part restates RESPACK's setup in chiqw.F (readers :87-329, Brillouin
// zone unfolding :437-545, q list :587-655, band classification :817-967,
// frequency grid :1184-1218) as plain C++ over std::vector, and prepares the
// per-q task (G sphere, k+q map, band pairs) that the CUDA kernels consume.
#pragma once

#include <complex>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/respack_gb300.h"

namespace rp {

using cd = std::complex<double>;

constexpr double kAu = 27.21151;                 // src/chiqw/config.h:19
constexpr double kPi = 3.14159265358979323846;
constexpr double kTpi = 2.0 * kPi;

struct Error : std::exception {
  int code;
  std::string msg;
  Error(int c, std::string m) : code(c), msg(std::move(m)) {}
  const char *what() const noexcept override { return msg.c_str(); }
};
[[noreturn]] void fail(int code, const char *fmt, ...);
void set_global_error(const std::string &msg);  // text of rp_last_error(NULL)
// count bytes a helper copied between host and device for the calling context
void note_transfer(long long h2d, long long d2h);

// ---- Fortran list-directed text and unformatted sequential files ----------
class ListReader {
 public:
  explicit ListReader(const std::string &path);
  // one READ statement: starts on a new record; "(a,b)" complex tokens give 2 values
  void read(int n, double *out);
  int read_int();
  std::vector<int> read_ints(int n);
  double read_real();
 private:
  std::vector<std::string> lines_;
  size_t next_ = 0;
  std::string path_;
};

// whole-record read of a sequential unformatted file (gfortran markers, subrecords)
class UnformattedReader {
 public:
  explicit UnformattedReader(const std::string &path);
  ~UnformattedReader();
  size_t read(void *buf, size_t want);  // returns record length, copies min(want,len)
 private:
  void *f_ = nullptr;
  std::string path_;
};
void write_unformatted_record(const std::string &path, const void *buf, size_t nbytes);

// ---- namelist (&param_chiqw, &param_gpu) -----------------------------------
void parse_namelist_text(const std::string &text, rp_params *p, std::vector<int> *qlist,
                         std::vector<double> *explicit_em);
void parse_calc_int_namelist(const std::string &text, rp_int_params *p);

// ---- the host model of one run ----------------------------------------------
struct Setup {
  // lattice (chiqw.F:148-184)
  double a[3][3]{}, b[3][3]{}, volume = 0;
  // symmetry (:186-202)
  int nsymq = 0, nnp = 1;
  std::vector<int> rg;        // rg[iop*9 + i + 3j] = rg(i,j,iop)
  std::vector<int> pg;        // pg[iop*3 + i]
  std::vector<double> rginv;  // like rg
  // irreducible k and plane waves (:252-329)
  int nk_irr = 0, ntg = 0, ntb = 0, ncb = 0;
  std::vector<double> ski, ski_list;  // 3*nk_irr
  std::vector<int> ngi;               // nk_irr
  std::vector<int> kgi;               // 3*ntg*nk_irr
  std::vector<double> e_eigi;         // [ik*ntb + ib] (Hartree)
  double efermi = 0, ecut_psi = 0, ecut_eps = 0;
  int L[3]{};
  std::vector<int> packing;           // per irreducible k box (2L+1)^3 -> 1-based ig
  int nw[3]{};                        // FFT box
  // full mesh (:419-545)
  int ntk = 0, nkb[3]{};
  std::vector<double> sk0;            // 3*ntk
  std::vector<int> numirr, numrot, trs, rw;
  std::vector<int> ng0, kg0;          // kg0[(jk*ntg + ig)*3 + d]
  std::vector<int> index_kpt;         // mesh slot -> full k (0-based)
  std::vector<int> mesh_of_k;         // full k -> mesh slot
  // bands (:817-967)
  std::vector<int> window_inside, tindx;
  std::vector<double> e_ave, band_max, band_min;
  std::vector<cd> prob;               // [ik*ntb + ib], full k
  int n_docc = 0, n_pocc = 0, n_uocc = 0, n_occ = 0, n_vir = 0;
  // frequencies (:1184-1192), Hartree
  std::vector<cd> em;
  // tetrahedra (ttrhdrn_mkidx), 0-based mesh slots, 4 per tetrahedron
  std::vector<int> imt1;
  // coefficients of the irreducible k, bands 0..ncb-1: [(ik*ncb + ib)*ntg + ig]
  std::vector<cd> coef;
  // run parameters (converted)
  double delt = 0, delta_ex = 0, dmna = 0, dmnr = 0;
  rp_params params{};
  // Wannier (calc_int) inputs, optional
  int nwf = 0;
  std::vector<cd> wan;                // [(jk*nwf + iw)*ntg + ig] on the full-mesh KG0 lists
  std::vector<double> wan_center;     // 3*nwf
};

// Unfold rotation/time-reversal map of full k jk into the irreducible list:
// src[jk*ntg + ig] = index into coef of numirr[jk] (or -1), with the phase and
// conjugation of make_C0 (chiqw_sub.F:264-322).
struct UnfoldMap {
  std::vector<int> src;   // ntk*ntg
  std::vector<cd> phase;  // ntk*ntg
};

struct QTask {
  int iq_irr = -1;      // 0-based index into dat.sample-k
  double q[3]{};        // SQ (search_list)
  bool gamma = false;
  int ng = 0, no_g0 = -1;
  std::vector<int> lg0;       // 3*ng
  std::vector<double> qglen;  // |q+G|
  std::vector<int> kpq;       // ntk
  std::vector<int> shift;     // 3*ntk
  std::vector<int> pair_vir, pair_occ;    // absolute 0-based bands, reference order
  std::vector<int> intra_band;            // Gamma: absolute band of intraband pairs
  int npair_full = 0;
};

// setup.cpp
void read_dir_wfn(Setup &s, const std::string &root);
void read_dir_wan_crpa(Setup &s, const std::string &root);
void read_dir_wan_orbitals(Setup &s, const std::string &root);
void read_wfn_coefficients(Setup &s, const std::string &root);
void finish_setup(Setup &s, const std::vector<double> &explicit_em);
void build_unfold_map(const Setup &s, UnfoldMap &m);
void make_kg0(const double b[3][3], double gcut, const double q[3], int ntg_max, std::vector<int> &kg, int &ng);
void search_list(const double *in, double *out);
QTask make_qtask(const Setup &s, int iq_irr, int max_pairs);
std::vector<int> q_list(const Setup &s, const std::string &epsdir);
int algn235(int n);
void gen_grid(int nt, double e, std::vector<cd> &em);

}  // namespace rp
