// rp_calc_chiqw -- drop-in for RESPACK's calc_chiqw executable
// (src/chiqw/chiqw.F, PROGRAM DIELECTRIC): reads the &param_chiqw namelist (and
// the optional q list and &param_gpu group) from standard input, runs in the
// current directory (dir-wfn, dir-wan in; dir-eps out) on one GPU.
#include <cstdio>
#include <iostream>
#include <iterator>
#include <string>

#include "../../include/respack_gb300.h"

int main(int argc, char **argv) {
  std::string text((std::istreambuf_iterator<char>(std::cin)), std::istreambuf_iterator<char>());
  const char *root = argc > 1 ? argv[1] : ".";
  int rc = rp_calc_chiqw(root, text.c_str());
  if (rc != 0) {
    std::fprintf(stderr, "rp_calc_chiqw: %s\n", rp_last_error(nullptr));
    return rc > 0 ? 2 : 3;
  }
  return 0;
}
