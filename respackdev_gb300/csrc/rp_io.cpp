// rp_io.cpp -- Fortran file formats and the namelist parser.
//
// List-directed reads follow the Fortran rule the reference relies on: each
// READ statement starts on a new record and may continue over several lines.
// Unformatted sequential records use gfortran's 4-byte length markers and its
// subrecord scheme above 2 GiB (dat.wfn is read as chiqw.F:1106-1158 does,
// dat.epsqw.600 is written as chiqw.F:1531-1538).
#include <cctype>
#include <cerrno>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "rp_host.h"

namespace rp {

void fail(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  throw Error(code, buf);
}

// ---------------------------------------------------------------------------
static void split_tokens(const std::string &line, std::vector<std::string> &tok) {
  size_t i = 0, n = line.size();
  while (i < n) {
    char c = line[i];
    if (c == ' ' || c == '\t' || c == ',' || c == '\r' || c == '\n') { i++; continue; }
    if (c == '/' || c == '!') break;
    if (c == '(') {
      size_t j = line.find(')', i);
      if (j == std::string::npos) break;
      tok.push_back(line.substr(i, j - i + 1));
      i = j + 1;
      continue;
    }
    size_t j = i;
    while (j < n && line[j] != ' ' && line[j] != '\t' && line[j] != ',' && line[j] != '\r' && line[j] != '\n') j++;
    tok.push_back(line.substr(i, j - i));
    i = j;
  }
}

static double to_num(std::string t) {
  for (auto &c : t)
    if (c == 'd' || c == 'D') c = 'e';
  char *end = nullptr;
  double v = strtod(t.c_str(), &end);
  if (end == t.c_str()) fail(1, "not a number: '%s'", t.c_str());
  return v;
}

ListReader::ListReader(const std::string &path) : path_(path) {
  std::ifstream f(path);
  if (!f) fail(1, "cannot open %s", path.c_str());
  std::string l;
  while (std::getline(f, l)) lines_.push_back(l);
}

void ListReader::read(int n, double *out) {
  int got = 0;
  while (got < n) {
    if (next_ >= lines_.size()) fail(1, "%s: unexpected end of file", path_.c_str());
    std::vector<std::string> tok;
    split_tokens(lines_[next_++], tok);
    for (size_t i = 0; i < tok.size() && got < n; i++) {
      const std::string &t = tok[i];
      if (t[0] == '(') {
        size_t c = t.find(',');
        if (c == std::string::npos) fail(1, "%s: bad complex '%s'", path_.c_str(), t.c_str());
        out[got++] = to_num(t.substr(1, c - 1));
        if (got < n) out[got++] = to_num(t.substr(c + 1, t.size() - c - 2));
      } else {
        out[got++] = to_num(t);
      }
    }
  }
}
int ListReader::read_int() { double v; read(1, &v); return (int)llround(v); }
double ListReader::read_real() { double v; read(1, &v); return v; }
std::vector<int> ListReader::read_ints(int n) {
  std::vector<double> v(n);
  read(n, v.data());
  std::vector<int> r(n);
  for (int i = 0; i < n; i++) r[i] = (int)llround(v[i]);
  return r;
}

// ---------------------------------------------------------------------------
UnformattedReader::UnformattedReader(const std::string &path) : path_(path) {
  f_ = fopen(path.c_str(), "rb");
  if (!f_) fail(1, "cannot open %s", path.c_str());
}
UnformattedReader::~UnformattedReader() { if (f_) fclose((FILE *)f_); }

size_t UnformattedReader::read(void *buf, size_t want) {
  FILE *f = (FILE *)f_;
  size_t total = 0, copied = 0;
  bool cont = true;
  while (cont) {
    int32_t m1;
    if (fread(&m1, 4, 1, f) != 1) fail(1, "%s: end of file", path_.c_str());
    cont = m1 < 0;
    size_t n = (size_t)(m1 < 0 ? -(int64_t)m1 : m1);
    size_t take = copied < want ? std::min(want - copied, n) : 0;
    if (take && fread((char *)buf + copied, 1, take, f) != take) fail(1, "%s: short record", path_.c_str());
    if (n > take) fseek(f, (long)(n - take), SEEK_CUR);
    copied += take;
    total += n;
    int32_t m2;
    if (fread(&m2, 4, 1, f) != 1) fail(1, "%s: missing record marker", path_.c_str());
  }
  return total;
}

void write_unformatted_record(const std::string &path, const void *buf, size_t n) {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) fail(1, "cannot write %s", path.c_str());
  const size_t maxsub = 2147483639u;
  size_t off = 0;
  bool first = true;
  do {
    size_t len = n - off;
    bool more = false;
    if (len > maxsub) { len = maxsub; more = true; }
    int32_t head = more ? -(int32_t)len : (int32_t)len;
    int32_t tail = first ? (int32_t)len : -(int32_t)len;
    bool ok = fwrite(&head, 4, 1, f) == 1 && (len == 0 || fwrite((const char *)buf + off, 1, len, f) == len) &&
              fwrite(&tail, 4, 1, f) == 1;
    if (!ok) { fclose(f); fail(1, "write error on %s", path.c_str()); }
    off += len;
    first = false;
  } while (off < n);
  if (fclose(f) != 0) fail(1, "close error on %s", path.c_str());
}

// ---------------------------------------------------------------------------
// namelist: &group name = value[, value...] ... /   (case-insensitive, ! comments)
struct NlGroup {
  std::vector<std::pair<std::string, std::vector<std::string>>> items;
  size_t end_pos = 0;  // text offset after the closing '/'
};

static std::string lower(std::string s) {
  for (auto &c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

static bool find_group(const std::string &text, const std::string &name, NlGroup &g) {
  std::string lt = lower(text);
  size_t p = 0;
  while (true) {
    p = lt.find("&" + name, p);
    if (p == std::string::npos) return false;
    size_t after = p + 1 + name.size();
    if (after < lt.size() && (std::isalnum((unsigned char)lt[after]) || lt[after] == '_')) { p = after; continue; }
    p = after;
    break;
  }
  // strip comments, collect until an unquoted '/'
  std::string body;
  size_t i = p;
  bool quote = false;
  char qc = 0;
  for (; i < text.size(); i++) {
    char c = text[i];
    if (quote) { if (c == qc) quote = false; body += c; continue; }
    if (c == '\'' || c == '"') { quote = true; qc = c; body += c; continue; }
    if (c == '!') { while (i < text.size() && text[i] != '\n') i++; body += ' '; continue; }
    if (c == '/') { i++; break; }
    if (c == '&' && lower(text.substr(i, 4)) == "&end") { i += 4; break; }
    body += c;
  }
  g.end_pos = i;
  // tokenize "name = v, v, ..." entries
  size_t k = 0;
  std::string cur;
  std::vector<std::string> toks;
  auto flush = [&]() { if (!cur.empty()) { toks.push_back(cur); cur.clear(); } };
  quote = false;
  for (; k < body.size(); k++) {
    char c = body[k];
    if (quote) { cur += c; if (c == qc) { quote = false; flush(); } continue; }
    if (c == '\'' || c == '"') { flush(); quote = true; qc = c; cur += c; continue; }
    if (c == '=') { flush(); toks.push_back("="); continue; }
    if (c == ',' || std::isspace((unsigned char)c)) { flush(); continue; }
    cur += c;
  }
  flush();
  for (size_t t = 0; t < toks.size(); t++) {
    if (t + 1 < toks.size() && toks[t + 1] == "=") {
      std::string key = lower(toks[t]);
      // strip an array subscript like name(1)
      size_t par = key.find('(');
      if (par != std::string::npos) key = key.substr(0, par);
      g.items.push_back({key, {}});
      t++;
      continue;
    }
    if (g.items.empty()) fail(1, "namelist &%s: value without a name", name.c_str());
    std::string v = toks[t];
    if (v.size() >= 2 && (v[0] == '\'' || v[0] == '"')) v = v.substr(1, v.size() - 2);
    g.items.back().second.push_back(v);
  }
  return true;
}

static int nl_int(const std::vector<std::string> &v, const std::string &key) {
  if (v.empty()) fail(1, "namelist: %s has no value", key.c_str());
  return (int)llround(to_num(v[0]));
}
static double nl_real(const std::vector<std::string> &v, const std::string &key) {
  if (v.empty()) fail(1, "namelist: %s has no value", key.c_str());
  return to_num(v[0]);
}

void parse_namelist_text(const std::string &text, rp_params *p, std::vector<int> *qlist,
                         std::vector<double> *explicit_em) {
  NlGroup g;
  if (!find_group(text, "param_chiqw", g)) fail(1, "namelist &param_chiqw not found");
  for (auto &kv : g.items) {
    const std::string &k = kv.first;
    const auto &v = kv.second;
    if (k == "n_calc_band") p->n_calc_band = nl_int(v, k);
    else if (k == "ecut_for_eps") p->ecut_for_eps = nl_real(v, k);
    else if (k == "shift_ef") p->shift_ef = nl_real(v, k);
    else if (k == "max_excitation_energy") p->max_excitation_energy = nl_real(v, k);
    else if (k == "green_func_delt") p->green_func_delt = nl_real(v, k);
    else if (k == "ttrhdrn_dmna") p->ttrhdrn_dmna = nl_real(v, k);
    else if (k == "ttrhdrn_dmnr") p->ttrhdrn_dmnr = nl_real(v, k);
    else if (k == "num_freq_grid") p->num_freq_grid = nl_int(v, k);
    else if (k == "lower_bound_energy_window") p->lower_bound_energy_window = nl_real(v, k);
    else if (k == "upper_bound_energy_window") p->upper_bound_energy_window = nl_real(v, k);
    else if (k == "flg_crpa") p->flg_crpa = nl_int(v, k);
    else if (k == "flg_calc_type") p->flg_calc_type = nl_int(v, k);
    else if (k == "file_num_log_start") p->file_num_log_start = nl_int(v, k);
    else if (k == "file_num_eps_start") p->file_num_eps_start = nl_int(v, k);
    else if (k == "file_num_eps_base_start") p->file_num_eps_base_start = nl_int(v, k);
    else if (k == "n_calc_q") p->n_calc_q = nl_int(v, k);
    else if (k == "mpi_num_qcomm") p->mpi_num_qcomm = nl_int(v, k);
    else if (k == "mpi_io_rank" || k == "mpi_num_proc_per_qcomm" || k == "file_num_chi_start" ||
             k == "file_num_chi_base_start") { /* accepted; no effect on one device */ }
    else fail(1, "namelist &param_chiqw: unknown name '%s'", k.c_str());
  }
  // the q index list follows the namelist (m_rdinput.f90:97-103)
  if (p->flg_calc_type == 2 && p->n_calc_q == 0) fail(1, "n_calc_q should not be zero");
  if (p->n_calc_q > 0 && qlist) {
    std::istringstream rest(text.substr(g.end_pos));
    std::string tok;
    qlist->clear();
    while ((int)qlist->size() < p->n_calc_q && rest >> tok) {
      if (tok[0] == '&') break;
      std::vector<std::string> parts;
      split_tokens(tok, parts);
      for (auto &t : parts) if ((int)qlist->size() < p->n_calc_q) qlist->push_back((int)llround(to_num(t)));
    }
    if ((int)qlist->size() < p->n_calc_q) fail(1, "q index list shorter than n_calc_q");
  }
  NlGroup gg;
  if (find_group(text, "param_gpu", gg)) {
    std::vector<double> fre, fim;
    for (auto &kv : gg.items) {
      const std::string &k = kv.first;
      const auto &v = kv.second;
      if (k == "precision") {
        std::string s = lower(v.empty() ? "" : v[0]);
        if (s == "fp64") p->precision = RP_PREC_FP64;
        else if (s == "fp16x2") p->precision = RP_PREC_FP16X2;
        else if (s == "bf16x3") p->precision = RP_PREC_BF16X3;
        else if (s == "fp16x3") p->precision = RP_PREC_FP16X3;
        else fail(1, "&param_gpu precision: unknown '%s'", s.c_str());
      } else if (k == "fft_box") {
        if (v.size() != 3) fail(1, "&param_gpu fft_box needs 3 integers");
        for (int i = 0; i < 3; i++) p->fft_box[i] = (int)llround(to_num(v[i]));
      } else if (k == "dump_chi") p->dump_chi = nl_int(v, k);
      else if (k == "device") p->device = nl_int(v, k);
      else if (k == "max_pairs") p->max_pairs = nl_int(v, k);
      else if (k == "qshard_index") p->qshard_index = nl_int(v, k);
      else if (k == "qshard_count") p->qshard_count = nl_int(v, k);
      else if (k == "pair_fp64") p->pair_fp64 = nl_int(v, k);
      else if (k == "tc_ksub") p->tc_ksub = nl_int(v, k);
      else if (k == "pair_batch") p->pair_batch = nl_int(v, k);
      else if (k == "tc_split") p->tc_split = nl_int(v, k);
      else if (k == "tc_pair") p->tc_pair = nl_int(v, k);
      else if (k == "write_eps_f32") p->write_eps_f32 = nl_int(v, k);
      else if (k == "eps_fp64") p->eps_fp64 = nl_int(v, k);
      else if (k == "ur_window") p->ur_window = nl_int(v, k);
      else if (k == "tetra_fp64") p->tetra_fp64 = nl_int(v, k);
      else if (k == "tail_model") {
        const std::string path = v.empty() ? "" : v[0];
        if (path.size() >= sizeof p->tail_model) fail(1, "&param_gpu tail_model: path longer than %zu characters",
                                                      sizeof p->tail_model - 1);
        std::memset(p->tail_model, 0, sizeof p->tail_model);
        std::memcpy(p->tail_model, path.data(), path.size());
      }
      else if (k == "freq_re_ev") for (auto &x : v) fre.push_back(to_num(x));
      else if (k == "freq_im_ev") for (auto &x : v) fim.push_back(to_num(x));
      else fail(1, "namelist &param_gpu: unknown name '%s'", k.c_str());
    }
    if (!fre.empty() && explicit_em) {
      if (!fim.empty() && fim.size() != fre.size()) fail(1, "freq_im_ev and freq_re_ev differ in length");
      explicit_em->clear();
      for (size_t i = 0; i < fre.size(); i++) {
        explicit_em->push_back(fre[i] / kAu);
        explicit_em->push_back(fim.empty() ? 0.0 : fim[i] / kAu);
      }
    }
  }
}

}  // namespace rp

extern "C" void rp_default_params(rp_params *p) {
  std::memset(p, 0, sizeof *p);
  p->n_calc_band = 0;
  p->ecut_for_eps = 0.0;
  p->shift_ef = 0.0;
  p->max_excitation_energy = 200.0;
  p->green_func_delt = 0.1;
  p->ttrhdrn_dmna = 0.001;
  p->ttrhdrn_dmnr = 0.001;
  p->num_freq_grid = 70;
  p->flg_crpa = 0;
  p->flg_calc_type = 0;
  p->file_num_log_start = 400;
  p->file_num_eps_start = 600;
  p->file_num_eps_base_start = 600000;
  p->precision = RP_PREC_FP64;
  p->qshard_count = 1;
}

namespace rp {

// &param_calc_int (src/calc_int/m_rdinput.f90:7-29) and the &param_gpu keys that apply
void parse_calc_int_namelist(const std::string &text, rp_int_params *p) {
  NlGroup g;
  if (!find_group(text, "param_calc_int", g)) fail(1, "namelist &param_calc_int not found");
  for (auto &kv : g.items) {
    const std::string &k = kv.first;
    const auto &v = kv.second;
    if (k == "calc_ifreq") p->calc_ifreq = nl_int(v, k);
    else if (k == "ix_intj_min") p->ix_intj_min = nl_int(v, k);
    else if (k == "ix_intj_max") p->ix_intj_max = nl_int(v, k);
    else if (k == "iy_intj_min") p->iy_intj_min = nl_int(v, k);
    else if (k == "iy_intj_max") p->iy_intj_max = nl_int(v, k);
    else if (k == "iz_intj_min") p->iz_intj_min = nl_int(v, k);
    else if (k == "iz_intj_max") p->iz_intj_max = nl_int(v, k);
    else if (k == "wcut_mvmc") p->wcut_mvmc = nl_real(v, k);
    else if (k == "jcut_mvmc") p->jcut_mvmc = nl_real(v, k);
    else fail(1, "namelist &param_calc_int: unknown name '%s'", k.c_str());
  }
  NlGroup gg;
  if (find_group(text, "param_gpu", gg)) {
    for (auto &kv : gg.items) {
      const std::string &k = kv.first;
      const auto &v = kv.second;
      if (k == "fft_box") {
        if (v.size() != 3) fail(1, "&param_gpu fft_box needs 3 integers");
        for (int i = 0; i < 3; i++) p->fft_box[i] = (int)llround(to_num(v[i]));
      } else if (k == "device") p->device = nl_int(v, k);
      else if (k == "write_files") p->write_files = nl_int(v, k);
      else if (k == "read_eps_f32") p->read_eps_f32 = nl_int(v, k);
      else fail(1, "namelist &param_gpu: unknown name '%s' for calc_int", k.c_str());
    }
  }
}

}  // namespace rp

static thread_local std::string g_parse_err;

extern "C" int rp_parse_namelist(const char *text, rp_params *p, int *qlist, int qcap, int *nq, double *em,
                                 int emcap, int *nen_explicit) {
  try {
    std::vector<int> q;
    std::vector<double> e;
    rp::parse_namelist_text(text ? text : "", p, &q, &e);
    if (nq) *nq = (int)q.size();
    for (int i = 0; i < (int)q.size() && i < qcap && qlist; i++) qlist[i] = q[i];
    int ne = (int)e.size() / 2;
    if (nen_explicit) *nen_explicit = ne;
    for (int i = 0; i < 2 * ne && i < 2 * emcap && em; i++) em[i] = e[i];
    return 0;
  } catch (const rp::Error &ex) {
    g_parse_err = ex.msg;
    return ex.code;
  }
}

extern "C" const char *rp_parse_error(void) { return g_parse_err.c_str(); }
