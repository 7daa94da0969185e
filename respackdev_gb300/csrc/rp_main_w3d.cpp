// rp_calc_w3d -- drop-in for RESPACK's calc_w3d executable
// (src/calc_int/calc_intW.F): reads &param_calc_int (and the optional
// &param_gpu group) from standard input and runs in the current directory
// (dir-wfn, dir-wan, dir-eps in; dir-intW and dir-mvmc out) on one GPU.
#include <cstdio>
#include <iostream>
#include <iterator>
#include <string>

#include "../../include/respack_gb300.h"

int main(int argc, char **argv) {
  std::string text((std::istreambuf_iterator<char>(std::cin)), std::istreambuf_iterator<char>());
  const char *root = argc > 1 ? argv[1] : ".";
  int rc = rp_calc_w3d(root, text.c_str());
  if (rc != 0) {
    std::fprintf(stderr, "rp_calc_w3d: %s\n", rp_int_last_error(nullptr));
    return rc > 0 ? 2 : 3;
  }
  return 0;
}
