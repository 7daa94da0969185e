/*
 * rp_oracle.h -- CPU restatement (FP64) of RESPACK's cRPA polarization path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the tests, the
 * smoke check and the CPU-baseline leg of bench.py call it; the product
 * (respackdev_gb300) never links, loads or calls it.
 *
 * Parity status: unpinned by the reference.  RESPACK ships no tests, no golden
 * outputs and no dir-wfn fixtures, and it cannot be compiled here (Fortran 77/90
 * + MPI + MKL, no Fortran compiler in this image).  This restatement is
 * cross-checked against numpy (FFT, inversion), brute-force plane-wave sums and
 * analytic tetrahedron integrals in tests/.
 *
 * Every routine cites the reference file:line it restates (paths relative to
 * the RESPACK source tree).
 */
#ifndef RP_ORACLE_H
#define RP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Values of the &param_chiqw namelist (src/chiqw/m_rdinput.f90:41-45), already
 * parsed, in the namelist's own units (eV for energies, Ry for the cutoff),
 * plus the extensions the GPU library also supports. */
typedef struct orc_params {
    int    n_calc_band;            /* N_CALC_BAND (0 = all bands)            */
    double ecut_for_eps;           /* Ecut_for_eps (Ry; 0 = Ecut_psi/10)     */
    double shift_ef;               /* shift_ef (eV)                          */
    double max_excitation_energy;  /* Max_excitation_energy (eV)             */
    double green_func_delt;        /* Green_func_delt (eV)                   */
    double ttrhdrn_dmna;           /* used as-is (no eV->Ha conversion, as chiqw.F) */
    double ttrhdrn_dmnr;
    int    num_freq_grid;          /* Num_freq_grid                          */
    double lower_bound_energy_window, upper_bound_energy_window;
    int    flg_crpa;               /* 0 fRPA, 1 band-cRPA                    */
    int    flg_calc_type;          /* 0 all q, 1 Gamma only, 2 manual list   */
    int    file_num_log_start;     /* 400    */
    int    file_num_eps_start;     /* 600    */
    int    file_num_eps_base_start;/* 600000 */
    int    n_calc_q;
    const int *calc_num_k;         /* n_calc_q entries, 1-based irreducible k */
    /* --- extensions --- */
    int    nen_explicit;           /* >0: use this explicit grid instead of gen_grid */
    const double *em_explicit;     /* complex (re,im) pairs in Hartree       */
    int    fft_box[3];             /* 0,0,0 = reference rule (chiqw.F:389-401) */
    int    dump_chi;               /* write dir-eps/qNNN/dat.chi0 (chiqw after /VOLUME) */
    int    write_eps;              /* 1: write the dir-eps files             */
    int    nthreads;               /* OpenMP threads (0 = runtime default)   */
    int    max_pairs;              /* >0: bounded sample of the first pairs (CPU timing) */
    int    max_q;                  /* >0: stop after this many q             */
    int    max_k;                  /* >0: timing sample: pair densities and the
                                      contraction over the first max_k k points
                                      only (chi is then incomplete)            */
} orc_params;

/* Per-run timing/size report. */
typedef struct orc_report {
    int    nq_done;
    int    ntk, ng_last, npair_last, npair_full_last, nen;
    int    fft_box[3];
    double seconds_total;
    double seconds_last_q;
    int    nk_used_last;           /* k points of the pair densities and contraction */
} orc_report;

void orc_default_params(orc_params *p);

/* Full calc_chiqw run in directory `root` (which holds dir-wfn, dir-wan). */
int orc_calc_chiqw(const char *root, const orc_params *p, orc_report *rep);

/* ---- unit entry points used by the tests ---- */
/* 3D complex FFT on an n1 x n2 x n3 box, x fastest.  fw: e^{-i}, scaled 1/N;
 * bw: e^{+i}, unscaled (m_fft3d_20150826.f90:1598-1720). */
void orc_fft3(int n1, int n2, int n3, double *re_im /* interleaved */, int forward);
/* gen_grid (src/chiqw/gen_grid.f90:1-39); em is complex interleaved. */
void orc_gen_grid(int nt, double e, double *em);
int  orc_algn235(int n);
/* In-place inverse of a complex n x n column-major matrix (zgetrf+zgetri). */
int  orc_zinv(int n, double *a);
/* ttrhdrn_mkidx (m_tetrahedron_20170325.F:505-584) */
void orc_ttrhdrn_mkidx(int n1, int n2, int n3, const double *b1, const double *b2,
                       const double *b3, int *imt1 /* 4*n1*n2*n3*6, 1-based */);
/* ttrhdrn_chi0 (m_tetrahedron_20170325.F:99-141), accumulating into xo(ne, nk). */
int  orc_ttrhdrn_chi0(double dmna, double dmnr, int n1, int n2, int n3, const int *imt1,
                      const double *e1, const double *e2, double f1, double f2,
                      double delt, double dsgn, int ne, const double *em, double *xo);
/* ttrhdrn_simple (m_tetrahedron_20170325.F:63-76), fk/gk complex, xo(nk) complex. */
/* one tetrahedron of ttrhdrn_chi0 with vertices 0..3; xo4 complex (4, ne) */
int  orc_tt_one(double dmna, double dmnr, const double *ee1, const double *ee2, double f1, double f2,
                double delt, double dsgn, int ne, const double *em, double *xo4);
int  orc_ttrhdrn_simple(double dmna, double dmnr, int n1, int n2, int n3, const int *imt1,
                        const double *fk, const double *gk, double *xo);

/* ---- calc_int: calc_w3d (V, W) and calc_j3d (X, J) ---- */
/* &param_calc_int (src/calc_int/m_rdinput.f90:7-13) plus extensions */
typedef struct orc_int_params {
    int    calc_ifreq;                   /* 1-based frequency of dat.Wmat / dat.Jmat */
    int    ix_min, ix_max, iy_min, iy_max, iz_min, iz_max;   /* IX_INTJ_MIN ... */
    double wcut_mvmc, jcut_mvmc;         /* eV */
    /* --- extensions --- */
    int    fft_box[3];                   /* 0,0,0 = reference rule */
    int    nthreads;
    int    write_files;                  /* dir-intW / dir-intJ / dir-mvmc */
    int    do_w, do_j;                   /* run calc_w3d / calc_j3d */
} orc_int_params;

typedef struct orc_int_dims {
    int nwf, ne, ntq, na[3], nkb[3], box, fft_box[3];
    double seconds;
} orc_int_dims;

void orc_int_default_params(orc_int_params *p);
/* V (nwf, nwf, box) and W (nwf, nwf, box, ne), X and J likewise (zero outside
 * the IX/IY/IZ range), complex interleaved, box = (2Na1+1)(2Na2+1)(2Na3+1)
 * with R1 fastest; any pointer may be NULL. */
int orc_calc_int(const char *root, const orc_int_params *p, orc_int_dims *dims, double *V, double *W,
                 double *X, double *J);

#ifdef __cplusplus
}
#endif
#endif
