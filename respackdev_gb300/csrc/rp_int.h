// rp_int.h -- launchers of the calc_int kernels (rp_int.cu).
#pragma once

#include <cuda_runtime.h>

namespace rp {

// rho_out[(r*np + p)*ngp + g] = k sum of the pair densities rho_pk[(p*ntk + k)*ngp + g]
// with the lattice phases pf[r*ntk + k]; j_order selects the reference's
// operation order of calc_intJ (1) or calc_intW (0).
int launch_int_reduce(const float2 *rho_pk, const double2 *pf, const double *len, int np, int ntk, int ngp, int g0,
                      int gamma, int j_order, int nr, double2 *rho_out, cudaStream_t st);
// T[(e*nv + v)*nge + g] = sum_g' eps(g,g',e) conj(V[v*ngp + g']), eps from the
// irreducible complex(4) array through the make_eps map (idx, p1, p2, trs).
int launch_int_eps(const float2 *eps_irr, int ntgq, const int *idx, const double2 *p1, const double2 *p2, int trs,
                   const double2 *V, int nv, int nge, int ngp, int ne, double2 *T, cudaStream_t st);
// out[e*ostride + o]: screened (T) or bare (T == nullptr) quadratic forms of the pairs (pa[o], pb[o]).
int launch_int_quad(const double2 *V, const double2 *T, const int *pa, const int *pb, int nout, int nv, int nge,
                    int ngp, int ne, double2 *out, size_t ostride, cudaStream_t st);
// out[((e*nbox + R)*nwf + j)*nwf + i] = scale sum_q f[((e*ntq + q)*nwf + j)*nwf + i] pf[q*nbox + R] + head[e]
int launch_int_fourier(const double2 *f, const double2 *pf, int ntq, int nbox, int nwf, int ne, double scale,
                       const double *head, double2 *out, cudaStream_t st);

}  // namespace rp
