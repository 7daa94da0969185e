/*
 * respack_gb300.h -- C ABI of the GB300 (sm_103a) cRPA polarization library.
 *
 * Drop-in for RESPACK's chiqw path (src/chiqw).  RESPACK has no plugin or FFI
 * layer; its boundaries are the calc_chiqw executable (stdin namelist +
 * dir-wfn/dir-wan in, dir-eps out) and the subroutine seam inside the q loop of
 * src/chiqw/chiqw.F.  Each entry point below names the reference code it
 * replaces.  All arrays are caller-owned host memory, column-major (Fortran
 * order), complex numbers as interleaved (re, im) doubles.  Every call returns
 * 0 on success, >0 for an input error and <0 for a device error; the message is
 * available from rp_last_error().  One context owns one CUDA stream; calls on a
 * context must not overlap.
 */
#ifndef RESPACK_GB300_H
#define RESPACK_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* Arithmetic of the path.  RP_PREC_FP64 is FP64 throughout, as the reference.
 * The split precisions take FP32 pair densities and real-space transforms,
 * the FP32 tetrahedron series (FP64 closed forms where it does not converge;
 * tetra_fp64 = 1: everywhere), the tensor-core contraction below, and the
 * mixed-precision eps inverse (eps_fp64 = 1: FP64); eps is built in FP64. */
enum rp_precision {
  RP_PREC_FP64 = 0,    /* plain FP64 everywhere (pair densities, contraction)      */
  RP_PREC_FP16X2 = 1,  /* FP32 pair densities; tcgen05 contraction, 2-term FP16
                          split (3 products), FP32 accumulate, FP64 chunk reduce  */
  RP_PREC_BF16X3 = 2,  /* as FP16X2 with a 3-term BF16 split (6 products)        */
  RP_PREC_FP16X3 = 3   /* as FP16X2 with a 3-term FP16 split (6 products)        */
};

/* &param_chiqw (src/chiqw/m_rdinput.f90:41-45, defaults :52-73) in the
 * namelist's units (eV, Ry), plus extensions (&param_gpu). */
typedef struct rp_params {
  int    n_calc_band;
  double ecut_for_eps;
  double shift_ef;
  double max_excitation_energy;
  double green_func_delt;
  double ttrhdrn_dmna;
  double ttrhdrn_dmnr;
  int    num_freq_grid;
  double lower_bound_energy_window;
  double upper_bound_energy_window;
  int    flg_crpa;
  int    flg_calc_type;
  int    file_num_log_start;
  int    file_num_eps_start;
  int    file_num_eps_base_start;
  int    n_calc_q;
  int    mpi_num_qcomm;        /* q communities: here the number of q shards */
  /* --- &param_gpu extensions --- */
  int    precision;            /* enum rp_precision                          */
  int    fft_box[3];           /* 0 0 0: reference rule (chiqw.F:389-401)    */
  int    dump_chi;             /* also write dir-eps/qNNN/dat.chi0           */
  int    device;               /* CUDA device ordinal                        */
  int    max_pairs;            /* >0: keep only the first pairs (timing)     */
  int    qshard_index;         /* this process's shard of the q list        */
  int    qshard_count;         /* number of shards (1 = all q here)          */
  int    pair_fp64;            /* tensor-core precisions: pair densities in FP64
                                  (as the reference) instead of FP32          */
  int    tc_ksub;              /* K blocks (of 64) per FP32 accumulation in
                                  tensor memory before it joins the float-pair
                                  sums (0 = 16; at most 16 for the three-plane
                                  precisions, whose integer sums stay exact)  */
  int    pair_batch;           /* at most this many band pairs per batch of a
                                  q (0 = as many as fit in 24 GB)             */
  int    tc_split;             /* K splits of the tensor-core Gram launch (0 =
                                  measured per shape by the launch tuner)     */
  int    tc_pair;              /* tensor-core Gram CTAs: 1 single CTAs, 2 CTA
                                  pairs (cta_group::2), 0 measured per shape
                                  by the launch tuner                         */
  int    write_eps_f32;        /* 1: rp_write_q also writes dat.epsqw.c4, the
                                  complex(4) eps^-1 calc_int reads (Gamma: the
                                  mean of the three directions)              */
  int    eps_fp64;             /* 1: the split precisions also invert eps with
                                  the FP64 Gauss-Jordan (0: FP32 Gauss-Jordan
                                  plus one float-pair Newton step, FP64 only
                                  as its fallback)                            */
  int    tetra_fp64;           /* 1: the split precisions also take the
                                  reference's FP64 closed forms for every
                                  tetrahedron weight (0: the FP32 series where
                                  it converges)                               */
  int    ur_window;            /* real-space functions of the virtual bands
                                  held for one pair batch at a time in this
                                  many slots (0: every band resident when it
                                  fits in HBM, else as many slots as fit)     */
  char   tail_model[256];      /* band-tail network file (written by
                                  respackdev_gb300.tail.TailMLP.save); when set,
                                  rp_chi0_q adds the network's prediction of
                                  the bands above N_CALC_BAND to the diagonal
                                  of chi0.  Empty: no correction.             */
} rp_params;

/* Defaults of m_rdinput.f90:52-73 (Num_freq_grid=70, Green_func_delt=0.1 eV, ...). */
void rp_default_params(rp_params *p);

/* Parse a namelist text holding &param_chiqw (and optionally the q index list
 * that follows it, m_rdinput.f90:97-103, and &param_gpu).  qlist receives up to
 * qcap indices, em up to emcap explicit frequencies (complex, Hartree).
 * Replaces read_input (m_rdinput.f90:47-129). */
int rp_parse_namelist(const char *text, rp_params *p, int *qlist, int qcap, int *nq,
                      double *em, int emcap, int *nen_explicit);

typedef struct rp_ctx rp_ctx;

/* Size/geometry report of a context. */
typedef struct rp_info {
  int ntk, nk_irr, nkb[3], ntg, ntb, ncb, nen;
  int n_occ, n_vir, n_docc, n_pocc, n_uocc;
  int fft_box[3];
  double volume, efermi, ecut_psi, ecut_eps;
  double device_bytes;         /* HBM held by the context */
} rp_info;

/* Build a context from a run directory holding dir-wfn (and dir-wan for
 * band-cRPA): reads the files like chiqw.F:87-329 and :870-906, unfolds the
 * Brillouin zone (:419-545), classifies bands (:817-967), makes the frequency
 * grid (:1184-1192, or the explicit grid em/nen_explicit when nen_explicit>0),
 * uploads the wave functions and computes their real-space periodic parts on
 * the device once (the reference recomputes them for every band pair,
 * chiqw_sub.F:128-163). */
int rp_ctx_create(rp_ctx **out, const char *root, const rp_params *p, const double *em,
                  int nen_explicit);

int rp_ctx_info(const rp_ctx *ctx, rp_info *info);

/* Number of entries of dat.sample-k (= candidate q points). */
int rp_num_qirr(const rp_ctx *ctx);

/* Sizes of q point iq without computing it: ng (dielectric G sphere of
 * make_KG0, chiqw_sub.F:773-812) and ndir (3 at Gamma, else 1). */
int rp_q_dims(const rp_ctx *ctx, int iq, int *ng, int *ndir);

/* chi0(G,G',w) of irreducible point iq (1-based index of dat.sample-k), after
 * /VOLUME and before the spin factor: the array chiqw of chiqw.F:1476 (q != 0,
 * layout (ng, ng, nen)) or chiqwgm of :1989 (Gamma, (ng, ng, nen, 3)).
 * Replaces the pair loop chiqw.F:1264-1472 (q != 0) and :1578-1985 (Gamma):
 * pair densities (calc_InterStateMatrix), tetrahedron weights (ttrhdrn_chi0)
 * and the contraction.  chi may be NULL (result stays on the device for
 * rp_epsinv_q).  ng_out / ndir_out report the sizes. */
int rp_chi0_q(rp_ctx *ctx, int iq, double *chi, int *ng_out, int *ndir_out);

/* chi0 of a ragged batch of problems: problem i is q point iqs[i] of context
 * ctxs[i] (one cell per context; a context may appear several times, and the
 * cells may differ in mesh, bands, G sphere and frequencies).  Every problem is
 * prepared first (tetrahedron weights, pair densities, split operands); then
 * ONE tensor-core Gram launch covers every (problem, tile, frequency, K split)
 * of the batch, and it and the assembly of each problem's chi0 run as one CUDA
 * graph (use_graph != 0) or as plain launches.  No reference counterpart: the
 * reference computes one q at a time (chiqw.F:1264-1472 per q); each chi[i]
 * (may be NULL) receives what rp_chi0_q(ctxs[i], iqs[i]) would give, up to the
 * rounding of the K splits.  All contexts: one device, one tensor-core
 * precision (not RP_PREC_FP64).  ng_out / ndir_out (may be NULL) get each
 * problem's sizes; seconds (may be NULL) gets [preparation wall time, device
 * time of the graph (Gram launch + assembly), finishing wall time].  The
 * contexts have no current q afterwards (rp_epsinv_q needs rp_chi0_q). */
int rp_chi0_batch(rp_ctx *const *ctxs, const int *iqs, int n, int use_graph, double *const *chi, int *ng_out,
                  int *ndir_out, double *seconds);

/* Shapes (K split and CTA shape) the tensor-core launch tuner has measured in
 * this process, and a reset of its cache (for tests). */
int rp_tuned_shapes(void);
void rp_reset_tuner(void);

/* eps^-1(G,G',w) of the last rp_chi0_q: calc_eps_rpa / calc_eps_rpa_q_0 and
 * invZGE (chiqw_sub.F:386-568, invZGE.F90:1-22), FP64 on the device.
 * Layout as chi.  epsinv may be NULL. */
int rp_epsinv_q(rp_ctx *ctx, double *epsinv);

/* eps^-1 of the q point of the last rp_chi0_q from a chi0 the caller supplies
 * in rp_chi0_q's layout (for instance a chi0 the caller corrected): the device
 * chi0 of that q is replaced by chi, then rp_epsinv_q runs.  No reference
 * counterpart (the reference inverts only its own chi, chiqw.F:1515-1525). */
int rp_epsinv_chi_q(rp_ctx *ctx, const double *chi, double *epsinv);

/* 1 if the last rp_chi0_q added the band-tail network's correction (a context
 * created with tail_model), else 0. */
int rp_tail_applied(const rp_ctx *ctx);

/* Write dir-eps/qNNN for the last rp_chi0_q/rp_epsinv_q: dat.sq,
 * dat.epsqw.600(-602), dat.epsqw.6NN0MM text diagonals and dat.log.400 last
 * (chiqw.F:1493-1548, :2012-2076). */
int rp_write_q(rp_ctx *ctx, const char *root);

/* Whole calc_chiqw run (PROGRAM DIELECTRIC, chiqw.F:1-2100) in directory
 * root with the namelist text (stdin content of the reference).  With
 * &param_gpu qshard_index/qshard_count, one process per GPU takes every
 * qshard_count-th q point still to do (the reference's MPI_num_qcomm
 * q communities, chiqw.F:662-687); no data is exchanged. */
int rp_calc_chiqw(const char *root, const char *namelist_text);

/* The 1-based q points rp_calc_chiqw would compute in root with this namelist
 * (host only, no device): the q list or every q without dat.log.400
 * (chiqw.F:593-608), then this process's shard.  Fills up to cap entries and
 * the count *n. */
int rp_plan_q(const char *root, const char *namelist_text, int *qlist, int cap, int *n);

/* Seconds spent in each stage of the last rp_chi0_q + rp_epsinv_q (device
 * time from CUDA events): [0] tetrahedron weights, [1] pair densities,
 * [2] contraction, [3] eps build + inversion, [4] total chi0_q, [5] the
 * tensor-core Gram kernel alone (0 on the FP64 path). */
int rp_stage_times(const rp_ctx *ctx, double *t6);

/* Number of kernel launches issued by this context so far. */
long long rp_kernel_launches(const rp_ctx *ctx);

/* Bytes this context's calls copied host->device and device->host so far
 * (task tables, Gamma rows, results fetched into host buffers). */
int rp_transfer_bytes(const rp_ctx *ctx, long long *h2d, long long *d2h);

/* 1 if the last rp_epsinv_q used the FP64 Gauss-Jordan inversion although the
 * precision is a split (fast) one: the FP32 inverse had a zero pivot or a
 * residual |I - eps X0|_F above 1e-3 in some matrix.  0 when the
 * mixed-precision inverse (FP32 Gauss-Jordan plus one float-pair Newton step)
 * was kept, and on the FP64 precision, which always inverts in FP64. */
int rp_eps_fallback(const rp_ctx *ctx);

const char *rp_last_error(const rp_ctx *ctx);
void rp_ctx_destroy(rp_ctx *ctx);

/* ---- calc_int: Wannier-basis interaction integrals --------------------------
 * calc_w3d (bare Coulomb V, screened W: src/calc_int/calc_intW.F) and calc_j3d
 * (bare exchange X, screened exchange J: src/calc_int/calc_intJ.F).  Inputs:
 * dir-wfn, dir-wan/dat.wan and dat.wan-center (Wannier functions on the full
 * k mesh), dir-eps from calc_chiqw (dat.chi_cutoff, dat.wgrid, qNNN/dat.sq and
 * dat.epsqw.600-602). */

/* &param_calc_int (src/calc_int/m_rdinput.f90:7-29) plus &param_gpu extensions. */
typedef struct rp_int_params {
  int    calc_ifreq;           /* 1-based frequency written to dat.Wmat / dat.Jmat */
  int    ix_intj_min, ix_intj_max, iy_intj_min, iy_intj_max, iz_intj_min, iz_intj_max;
  double wcut_mvmc, jcut_mvmc; /* eV */
  /* --- &param_gpu extensions --- */
  int    fft_box[3];           /* 0 0 0: reference rule (calc_intW.F:150-185) */
  int    device;
  int    write_files;          /* 1: write dir-intW / dir-intJ / dir-mvmc */
  int    read_eps_f32;         /* 1: read dir-eps/qNNN/dat.epsqw.c4 where it
                                  exists instead of dat.epsqw.600(-602)       */
} rp_int_params;

void rp_int_default_params(rp_int_params *p);
/* Replaces read_input of src/calc_int/m_rdinput.f90:15-35. */
int rp_int_parse_namelist(const char *text, rp_int_params *p);

typedef struct rp_int rp_int;

/* Reads every input like calc_intW.F:1-630 (k and q unfolding, make_LG0,
 * eps^-1 of the irreducible q as complex(4)) and computes the real-space
 * Wannier functions on the device once. */
int rp_int_create(rp_int **out, const char *root, const rp_int_params *p);
/* nwf, ne, number of q points, and Na (the R box is -Na..Na, Na = nkb/2). */
int rp_int_dims(const rp_int *c, int *nwf, int *ne, int *ntq, int *na3);

/* calc_w3d: V (nwf, nwf, 2Na1+1, 2Na2+1, 2Na3+1) and W (..., ne), complex
 * interleaved, column-major, R1 fastest (V_MAT / W_MAT of calc_intW.F:942-985,
 * heads included).  Writes dir-intW and dir-mvmc when write_files.  V, W may
 * be NULL. */
int rp_int_w3d(rp_int *c, double *V, double *W);
/* calc_j3d: X and J on the same box (zero outside the IX/IY/IZ range;
 * calc_intJ.F:609-905).  Writes dir-intJ and dir-mvmc when write_files. */
int rp_int_j3d(rp_int *c, double *X, double *J);
/* Device seconds of the last rp_int_w3d / rp_int_j3d: [0] pair densities,
 * [1] k sums, [2] eps^-1 products, [3] q -> R sums, [4] total. */
int rp_int_stage_times(const rp_int *c, double *t5);
const char *rp_int_last_error(const rp_int *c);
void rp_int_destroy(rp_int *c);

/* Whole programs (stdin namelist text of the reference) in directory root. */
int rp_calc_w3d(const char *root, const char *namelist_text);
int rp_calc_j3d(const char *root, const char *namelist_text);

/* Batched inverse of nmat complex n x n matrices (column-major, interleaved
 * re/im doubles, matrix m at a + 2*m*n*n) that allocates no device memory.
 * It has no counterpart in the reference.  It is the inversion step of
 * rp_epsinv_q (partial pivoting on |re|+|im|) offered on its own for callers
 * that cannot allocate GPU memory or let a library do so -- a Fortran or C++
 * host whose device memory belongs to its own allocator or pool, or code that
 * runs where cudaMalloc is not allowed.  a and ainv are device pointers,
 * 16-byte aligned, either the same buffer (the inverse overwrites it) or not
 * overlapping at all (a is left unchanged); a partial overlap is rejected.  The
 * work is queued on `stream` (a cudaStream_t, NULL = legacy default stream) and
 * the call synchronizes that stream before it returns.
 *
 * Scratch lives in one fixed device array of the library (about 4.6 MB per
 * GPU): n*nmat <= 131072 and nmat <= 1024, larger requests are rejected with
 * code 1 before any work.  CUDA loads the library's device code lazily by
 * default, so the array is reserved on a device at the first call there (or
 * when the program starts, with CUDA_MODULE_LOADING=EAGER): make that first
 * call before the host reserves its own pool.  Nothing in the array has to
 * start at zero; the error word is cleared by each call.  The first call on
 * each device also looks the array up (cudaGetSymbolAddress) with that device
 * current; make it before any stream capture.  Calls whose work overlaps on the
 * GPU (different streams or host threads) share the array and race: serialise
 * them.  Returns 0, 1 (bad arguments or size), 3 (singular matrix) or -1 (CUDA
 * error); rp_last_error(NULL) gives the text. */
int rp_zinv_batched_noalloc(const double *a, double *ainv, int n, int nmat, void *stream);

/* ---- band-tail MLP (no reference counterpart) ----------------------------
 * A fully connected network nin -> nhid -> nhid -> nout (ReLU between layers)
 * that predicts the chi0 contribution of the bands above a truncation per
 * |q+G| shell (features and targets: respackdev_gb300/tail.py).  Trained and
 * run on the GPU by the library's own kernels: FP32 master weights updated by
 * Adam, a BF16 copy read by the forward and backward passes, FP32
 * accumulation.  Loss: mean squared error over samples and outputs.  Arrays
 * are host, row-major: x [n][nin], t and y [n][nout]; parameters in the order
 * W1 [nhid][nin], b1 [nhid], W2 [nhid][nhid], b2 [nhid], W3 [nout][nhid],
 * b3 [nout].  Sizes are at most 256.  Status codes as the calls above. */
typedef struct rp_mlp rp_mlp;
int rp_mlp_create(rp_mlp **out, int nin, int nhid, int nout, unsigned long long seed, int device);
int rp_mlp_nparams(const rp_mlp *m);
int rp_mlp_get_params(rp_mlp *m, float *params);
int rp_mlp_set_params(rp_mlp *m, const float *params);   /* also resets Adam */
int rp_mlp_forward(rp_mlp *m, const float *x, int n, float *y);
/* loss and its gradient with respect to every parameter, for one batch */
int rp_mlp_gradients(rp_mlp *m, const float *x, const float *t, int n, float *loss, float *grad);
/* `steps` Adam steps on minibatches of `batch` samples taken in order
 * (wrapping at n); losses[s] = minibatch loss before step s (may be NULL) */
int rp_mlp_train(rp_mlp *m, const float *x, const float *t, int n, int steps, int batch, float lr, float *losses);
const char *rp_mlp_last_error(const rp_mlp *m);
void rp_mlp_destroy(rp_mlp *m);

#ifdef __cplusplus
}
#endif
#endif
