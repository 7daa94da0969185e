/*
 * rp_oracle.c -- CPU restatement (FP64) of RESPACK's chiqw (cRPA polarization).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for respackdev_gb300.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
 *
 * Parity unpinned by the reference (no reference tests, fixtures or compiler);
 * cross-checked against numpy and analytic integrals in tests/.
 *
 * Restates, with file:line of the RESPACK source tree:
 *   src/chiqw/chiqw.F           driver, readers, unfold, q loop (q!=0 :1257-1554, q=0 :1557-2085)
 *   src/chiqw/chiqw_sub.F       search_kq, search_list, calc_InterStateMatrix, calc_VMab/aa,
 *                               make_C0, make_index_kpt, calc_eps_rpa(_q_0), judge_*, kcheck*,
 *                               make_KG0
 *   src/chiqw/m_tetrahedron_20170325.F   generalized tetrahedron weights
 *   src/chiqw/gen_grid.f90, est_nwx2.f90, est_NTK.f90, invZGE.F90, inv.F90
 * Kindless Fortran CMPLX() calls round to single precision; those sites
 * (chiqw.F:1354,1357,1672,1813,1814; chiqw_sub.F:143,162,201,510) are
 * reproduced with a float round trip (SGL below).
 */
#define _GNU_SOURCE
#include "rp_oracle.h"

#include <complex.h>
#include <errno.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

static const double AU = 27.21151;          /* config.h:19 */
#define PI_ 3.14159265358979323846
static const double TPI = 2.0 * PI_;        /* config.h:21 (2*dacos(-1)) */

static inline double SGL(double x) { return (double)(float)x; }
static inline cplx SGLC(double re, double im) { return SGL(re) + I * SGL(im); }

static double now_s(void) {
    struct timeval tv; gettimeofday(&tv, NULL);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
}

static char g_err[512];
static int fail(const char *fmt, ...) {
    va_list ap; va_start(ap, fmt); vsnprintf(g_err, sizeof g_err, fmt, ap); va_end(ap);
    fprintf(stderr, "rp_oracle: %s\n", g_err);
    return 1;
}

/* ========================================================================= */
/* list-directed text reading: every READ statement starts on a new record   */
/* ========================================================================= */
typedef struct { FILE *f; char *line; size_t cap; } ldr;

static int ld_open(ldr *r, const char *path) {
    r->f = fopen(path, "r"); r->line = NULL; r->cap = 0;
    return r->f ? 0 : fail("cannot open %s", path);
}
static void ld_close(ldr *r) { if (r->f) fclose(r->f); free(r->line); r->f = NULL; }

/* split one line into tokens; "(a,b)" stays one token */
static int ld_tokens(char *s, char **tok, int maxt) {
    int n = 0;
    char *p = s;
    while (*p && n < maxt) {
        while (*p == ' ' || *p == '\t' || *p == ',' || *p == '\n' || *p == '\r') p++;
        if (!*p) break;
        if (*p == '/') break;
        if (*p == '(') {
            char *q = strchr(p, ')');
            if (!q) break;
            tok[n++] = p; p = q + 1;
            if (*p) { *p = 0; p++; }
            continue;
        }
        tok[n++] = p;
        while (*p && *p != ' ' && *p != '\t' && *p != ',' && *p != '\n' && *p != '\r') p++;
        if (*p) { *p = 0; p++; }
    }
    return n;
}
static double ld_num(const char *t) {
    char buf[64]; size_t i;
    for (i = 0; t[i] && i < sizeof buf - 1; i++) buf[i] = (t[i] == 'd' || t[i] == 'D') ? 'e' : t[i];
    buf[i] = 0;
    return strtod(buf, NULL);
}
/* read n real numbers (complex tokens "(a,b)" give two) starting on a new line */
static int ld_read(ldr *r, int n, double *out) {
    int got = 0;
    while (got < n) {
        ssize_t len = getline(&r->line, &r->cap, r->f);
        if (len < 0) return fail("unexpected end of file");
        char *tok[256];
        int nt = ld_tokens(r->line, tok, 256);
        for (int i = 0; i < nt && got < n; i++) {
            if (tok[i][0] == '(') {
                char *c = strchr(tok[i], ',');
                if (!c) return fail("bad complex token %s", tok[i]);
                *c = 0;
                out[got++] = ld_num(tok[i] + 1);
                if (got < n) out[got++] = ld_num(c + 1);
            } else {
                out[got++] = ld_num(tok[i]);
            }
        }
    }
    return 0;
}
static int ld_int(ldr *r, int n, int *out) {
    double tmp[64];
    if (n > 64) return fail("ld_int too many");
    if (ld_read(r, n, tmp)) return 1;
    for (int i = 0; i < n; i++) out[i] = (int)lround(tmp[i]);
    return 0;
}

/* ========================================================================= */
/* Fortran unformatted sequential files (gfortran 4-byte markers, subrecords) */
/* ========================================================================= */
static int fu_read_record(FILE *f, void *buf, size_t want, size_t *got) {
    size_t total = 0; int cont = 1;
    while (cont) {
        int32_t m1;
        if (fread(&m1, 4, 1, f) != 1) return fail("unformatted: eof");
        cont = m1 < 0;
        size_t n = (size_t)(m1 < 0 ? -(int64_t)m1 : m1);
        size_t take = 0;
        if (total < want) take = (want - total < n) ? want - total : n;
        if (take && fread((char *)buf + total, 1, take, f) != take) return fail("unformatted: short");
        if (n > take) fseek(f, (long)(n - take), SEEK_CUR);
        total += take;
        int32_t m2;
        if (fread(&m2, 4, 1, f) != 1) return fail("unformatted: no tail marker");
    }
    if (got) *got = total;
    return 0;
}
/* gfortran splits records above 2147483639 bytes into subrecords: the head
 * marker is negative when more subrecords follow, the tail marker is negative
 * when a subrecord continues an earlier one. */
static int fu_write_record(FILE *f, const void *buf, size_t n) {
    const size_t maxsub = 2147483639u;
    size_t off = 0; int first = 1;
    do {
        size_t len = n - off; int more = 0;
        if (len > maxsub) { len = maxsub; more = 1; }
        int32_t head = more ? -(int32_t)len : (int32_t)len;
        int32_t tail = first ? (int32_t)len : -(int32_t)len;
        if (fwrite(&head, 4, 1, f) != 1) return 1;
        if (len && fwrite((const char *)buf + off, 1, len, f) != len) return 1;
        if (fwrite(&tail, 4, 1, f) != 1) return 1;
        off += len; first = 0;
    } while (off < n);
    return 0;
}

/* ========================================================================= */
/* small helpers restated from the reference                                  */
/* ========================================================================= */
/* est_nwx2.f90:1-41 */
static int fctck(int n) {
    int i = n;
    while (i != 1) {
        if (i % 2 == 0) i /= 2; else if (i % 3 == 0) i /= 3; else if (i % 5 == 0) i /= 5;
        else return 1;
    }
    return 0;
}
int orc_algn235(int inr) { int nr = inr; while (fctck(nr)) nr++; return nr; }

/* gen_grid.f90:1-39 */
void orc_gen_grid(int Nt, double E, double *em) {
    const double au = 27.21151, dlt = 0.05 / au, ratio = 0.1, eps = 1.0e-6;
    if (Nt == 1) { em[0] = 0; em[1] = 0; return; }
    int M = (int)(ratio * (double)Nt);
    int N = Nt - M;
    double alp = E / dlt, x = 1.5, dl = 1.0;
    while (dl > eps) {
        double f = pow(x, N - 1) - alp * x + alp - 1.0;
        double g = (double)(N - 1) * pow(x, N - 2) - alp;
        double x1 = x - f / g;
        dl = fabs(x1 - x);
        x = x1;
    }
    double a = dlt / (x - 1.0), b = log(x);
    for (int i = 1; i <= N; i++) { em[2 * (i - 1)] = a * exp(b * (double)(i - 1)) - a; em[2 * (i - 1) + 1] = 0; }
    double c = E * exp(-log(2.0) * (double)N / (double)M);
    double d = log(2.0) / (double)M;
    for (int i = N + 1; i <= N + M; i++) { em[2 * (i - 1)] = c * exp(d * (double)i); em[2 * (i - 1) + 1] = 0; }
}

/* kcheck / kcheck_trs (chiqw_sub.F:668-771) */
static void kcheck(double *k, int *RW) {
    const double d = 1.0e-6;
    for (int i = 0; i < 3; i++) {
        if (k[i] > 1.5 + d) { k[i] -= 2.0; RW[i] = -2; }
        if (k[i] > 0.5 + d) { k[i] -= 1.0; RW[i] = -1; }
        if (k[i] <= -1.5 + d) { k[i] += 2.0; RW[i] = 2; }
        if (k[i] <= -0.5 + d) { k[i] += 1.0; RW[i] = 1; }
    }
}
static void kcheck_trs(double *k, int *RW) {
    const double d = -1.0e-6;
    for (int i = 0; i < 3; i++) {
        if (k[i] >= 1.5 + d) { k[i] -= 2.0; RW[i] = -2; }
        if (k[i] >= 0.5 + d) { k[i] -= 1.0; RW[i] = -1; }
        if (k[i] < -1.5 + d) { k[i] += 2.0; RW[i] = 2; }
        if (k[i] < -0.5 + d) { k[i] += 1.0; RW[i] = 1; }
    }
}
/* search_list (chiqw_sub.F:77-95); note the z component tests -0.5 before -1.5 */
static void search_list(const double *SQI, double *SQ) {
    const double d = 1.0e-6;
    SQ[0] = SQI[0]; SQ[1] = SQI[1]; SQ[2] = SQI[2];
    for (int i = 0; i < 2; i++) {
        if (SQ[i] > 1.5 + d) SQ[i] -= 2.0;
        if (SQ[i] > 0.5 + d) SQ[i] -= 1.0;
        if (SQ[i] <= -1.5 + d) SQ[i] += 2.0;
        if (SQ[i] <= -0.5 + d) SQ[i] += 1.0;
    }
    if (SQ[2] > 1.5 + d) SQ[2] -= 2.0;
    if (SQ[2] > 0.5 + d) SQ[2] -= 1.0;
    if (SQ[2] <= -0.5 + d) SQ[2] += 1.0;
    if (SQ[2] <= -1.5 + d) SQ[2] += 2.0;
}
/* search_kq (chiqw_sub.F:1-75): last match wins */
static void search_kq(int NTK, const double *SK0, const double *q, int ik, int *ikq, int *sG) {
    const double d = 1.0e-6;
    double s[3];
    for (int i = 0; i < 3; i++) {
        s[i] = SK0[3 * ik + i] + q[i];
        if (s[i] > 1.5 + d) { s[i] -= 2.0; sG[i] = 2; }
        if (s[i] > 0.5 + d) { s[i] -= 1.0; sG[i] = 1; }
        if (s[i] <= -1.5 + d) { s[i] += 2.0; sG[i] = -2; }
        if (s[i] <= -0.5 + d) { s[i] += 1.0; sG[i] = -1; }
    }
    for (int jk = 0; jk < NTK; jk++)
        if (fabs(SK0[3 * jk] - s[0]) < 1e-6 && fabs(SK0[3 * jk + 1] - s[1]) < 1e-6 &&
            fabs(SK0[3 * jk + 2] - s[2]) < 1e-6)
            *ikq = jk;
}

/* make_KG0 (chiqw_sub.F:773-812): sphere in the igL1-outer triple loop order.
 * The loop bounds -100..100 are narrowed to the indices that can satisfy the
 * cutoff, which keeps the order of the accepted points. */
static int make_KG0(int NTG, const double *b1, const double *b2, const double *b3, double Gcut,
                    double q1, double q2, double q3, int *KG, int *NG) {
    /* |n_i| <= sqrt(Gcut)*|a_i|/(2 pi) + |q_i| + 1, a_i from the reciprocal basis */
    double bb[3][3] = {{b1[0], b1[1], b1[2]}, {b2[0], b2[1], b2[2]}, {b3[0], b3[1], b3[2]}};
    int lim[3];
    for (int i = 0; i < 3; i++) {
        const double *u = bb[(i + 1) % 3], *v = bb[(i + 2) % 3];
        double c[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
        double vol = bb[i][0] * c[0] + bb[i][1] * c[1] + bb[i][2] * c[2];
        double alen = TPI * sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) / fabs(vol);
        double qi = (i == 0 ? q1 : i == 1 ? q2 : q3);
        lim[i] = (int)(sqrt(Gcut) * alen / TPI + fabs(qi)) + 2;
        if (lim[i] > 100) lim[i] = 100;
    }
    int n = 0;
    for (int i1 = -lim[0]; i1 <= lim[0]; i1++)
        for (int i2 = -lim[1]; i2 <= lim[1]; i2++)
            for (int i3 = -lim[2]; i3 <= lim[2]; i3++) {
                double g[3];
                for (int d = 0; d < 3; d++)
                    g[d] = (q1 + (double)i1) * b1[d] + (q2 + (double)i2) * b2[d] + (q3 + (double)i3) * b3[d];
                double g2 = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
                if (g2 <= Gcut) {
                    if (n >= NTG) return fail("make_KG0: more than NTG=%d points", NTG);
                    KG[3 * n] = i1; KG[3 * n + 1] = i2; KG[3 * n + 2] = i3;
                    n++;
                }
            }
    *NG = n;
    return 0;
}

/* 3x3 real inverse of an integer matrix (inv.F90); exact for |det| = 1 */
static void inv3(const int *m /* column-major m(i,j)=m[i+3j] */, double *out) {
    double a = m[0], b = m[3], c = m[6], d = m[1], e = m[4], f = m[7], g = m[2], h = m[5], k = m[8];
    double det = a * (e * k - f * h) - b * (d * k - f * g) + c * (d * h - e * g);
    double inv[9] = {(e * k - f * h), -(b * k - c * h), (b * f - c * e),
                     -(d * k - f * g), (a * k - c * g), -(a * f - c * d),
                     (d * h - e * g), -(a * h - b * g), (a * e - b * d)};
    /* inv[] is row-major (row r, col c at 3r+c); store column-major */
    for (int r = 0; r < 3; r++)
        for (int cc = 0; cc < 3; cc++) out[r + 3 * cc] = inv[3 * r + cc] / det;
}

/* ========================================================================= */
/* FFT (any algorithm may be used; semantics of m_fft3d:1598-1720)           */
/* ========================================================================= */
typedef struct { int n; cplx *w; } fft_plan1;

static void fft_rec(int n, const cplx *in, int stride, cplx *out, const cplx *w, int wstep, cplx *scratch) {
    if (n == 1) { out[0] = in[0]; return; }
    int p = 2;
    while (n % p) p++;
    int m = n / p;
    for (int r = 0; r < p; r++) fft_rec(m, in + r * stride, stride * p, out + r * m, w, wstep * p, scratch);
    /* combine: X[k + q m] = sum_r Y_r[k] w^{r (k + q m)} (w = e^{s 2 pi i / n}) */
    for (int k = 0; k < m; k++) {
        cplx y[16];
        cplx *yy = (p <= 16) ? y : scratch;
        for (int r = 0; r < p; r++) yy[r] = out[r * m + k];
        for (int q = 0; q < p; q++) {
            cplx acc = 0;
            int idx = k + q * m;
            for (int r = 0; r < p; r++) {
                long e = ((long)r * idx) % n;
                acc += yy[r] * w[e * wstep];
            }
            out[k + q * m] = acc;    /* reads of this k were copied to yy first */
        }
    }
}

static void fft1d(int n, cplx *x, int stride, int sign, cplx *tmpin, cplx *tmpout, cplx *scratch) {
    static __thread int wn = 0, ws = 0;
    static __thread cplx *w = NULL;
    if (wn != n || ws != sign) {
        free(w);
        w = (cplx *)malloc(sizeof(cplx) * n);
        for (int j = 0; j < n; j++) {
            double ang = sign * TPI * (double)j / (double)n;
            w[j] = cos(ang) + I * sin(ang);
        }
        wn = n; ws = sign;
    }
    for (int j = 0; j < n; j++) tmpin[j] = x[(long)j * stride];
    fft_rec(n, tmpin, 1, tmpout, w, 1, scratch);
    for (int j = 0; j < n; j++) x[(long)j * stride] = tmpout[j];
}

/* box x fastest: index ix + n1*(iy + n2*iz) */
static void fft3(int n1, int n2, int n3, cplx *a, int forward) {
    int nmax = n1 > n2 ? n1 : n2; if (n3 > nmax) nmax = n3;
    cplx *ti = (cplx *)malloc(sizeof(cplx) * nmax), *to = (cplx *)malloc(sizeof(cplx) * nmax);
    cplx *sc = (cplx *)malloc(sizeof(cplx) * nmax);
    int sign = forward ? -1 : +1;
    for (int iz = 0; iz < n3; iz++)
        for (int iy = 0; iy < n2; iy++) fft1d(n1, a + (long)n1 * (iy + (long)n2 * iz), 1, sign, ti, to, sc);
    for (int iz = 0; iz < n3; iz++)
        for (int ix = 0; ix < n1; ix++) fft1d(n2, a + ix + (long)n1 * n2 * iz, n1, sign, ti, to, sc);
    for (int iy = 0; iy < n2; iy++)
        for (int ix = 0; ix < n1; ix++) fft1d(n3, a + ix + (long)n1 * iy, n1 * n2, sign, ti, to, sc);
    if (forward) {
        double scl = 1.0 / ((double)n1 * n2 * n3);
        long N = (long)n1 * n2 * n3;
        for (long i = 0; i < N; i++) a[i] *= scl;
    }
    free(ti); free(to); free(sc);
}
void orc_fft3(int n1, int n2, int n3, double *re_im, int forward) { fft3(n1, n2, n3, (cplx *)re_im, forward); }

/* ========================================================================= */
/* LU inverse (zgetrf + zgetri semantics, izamax pivot on |re|+|im|)         */
/* ========================================================================= */
static int zinv(int n, cplx *a) {
    int *piv = (int *)malloc(sizeof(int) * n);
    /* LU with partial pivoting, column-major a[i + n*j] */
    for (int j = 0; j < n; j++) {
        int p = j; double best = -1;
        for (int i = j; i < n; i++) {
            double v = fabs(creal(a[i + (long)n * j])) + fabs(cimag(a[i + (long)n * j]));
            if (v > best) { best = v; p = i; }
        }
        piv[j] = p;
        if (best == 0.0) { free(piv); return fail("singular matrix in zinv (column %d)", j + 1); }
        if (p != j)
            for (int c = 0; c < n; c++) { cplx t = a[j + (long)n * c]; a[j + (long)n * c] = a[p + (long)n * c]; a[p + (long)n * c] = t; }
        cplx d = 1.0 / a[j + (long)n * j];
        for (int i = j + 1; i < n; i++) a[i + (long)n * j] *= d;
        for (int c = j + 1; c < n; c++) {
            cplx f = a[j + (long)n * c];
            if (f != 0)
                for (int i = j + 1; i < n; i++) a[i + (long)n * c] -= a[i + (long)n * j] * f;
        }
    }
    /* inverse of U (upper) in place */
    for (int j = 0; j < n; j++) {
        a[j + (long)n * j] = 1.0 / a[j + (long)n * j];
        cplx ajj = -a[j + (long)n * j];
        for (int i = 0; i < j; i++) {
            cplx s = 0;
            for (int k = i; k < j; k++) s += a[i + (long)n * k] * a[k + (long)n * j];
            a[i + (long)n * j] = s;
        }
        for (int i = 0; i < j; i++) a[i + (long)n * j] *= ajj;
    }
    /* solve inv(A)*L = inv(U) for inv(A) */
    cplx *work = (cplx *)malloc(sizeof(cplx) * n);
    for (int j = n - 1; j >= 0; j--) {
        for (int i = j + 1; i < n; i++) { work[i] = a[i + (long)n * j]; a[i + (long)n * j] = 0; }
        for (int i = j + 1; i < n; i++) {
            cplx w = work[i];
            for (int r = 0; r < n; r++) a[r + (long)n * j] -= a[r + (long)n * i] * w;
        }
    }
    free(work);
    for (int j = n - 2; j >= 0; j--) {
        int p = piv[j];
        if (p != j)
            for (int r = 0; r < n; r++) { cplx t = a[r + (long)n * j]; a[r + (long)n * j] = a[r + (long)n * p]; a[r + (long)n * p] = t; }
    }
    free(piv);
    return 0;
}
int orc_zinv(int n, double *a) { return zinv(n, (cplx *)a); }

/* ========================================================================= */
/* generalized tetrahedron method (m_tetrahedron_20170325.F)                 */
/* ========================================================================= */
#define TT_NMAX 99

/* libtetrabzinitialize (:523-584); imt1 1-based, 4 per tetrahedron */
void orc_ttrhdrn_mkidx(int n1, int n2, int n3, const double *bv1, const double *bv2,
                       const double *bv3, int *idx1) {
    int ng[3] = {n1, n2, n3};
    double bvec[3][3]; /* bvec[i] = column i */
    for (int d = 0; d < 3; d++) { bvec[0][d] = bv1[d]; bvec[1][d] = bv2[d]; bvec[2][d] = bv3[d]; }
    double bvec2[3][3], bvec3[4][3], l[4];
    for (int i = 0; i < 3; i++)
        for (int d = 0; d < 3; d++) bvec2[i][d] = bvec[i][d] / (double)ng[i];
    for (int d = 0; d < 3; d++) {
        bvec3[0][d] = -bvec2[0][d] + bvec2[1][d] + bvec2[2][d];
        bvec3[1][d] = bvec2[0][d] - bvec2[1][d] + bvec2[2][d];
        bvec3[2][d] = bvec2[0][d] + bvec2[1][d] - bvec2[2][d];
        bvec3[3][d] = bvec2[0][d] + bvec2[1][d] + bvec2[2][d];
    }
    int itype = 0;
    for (int i = 0; i < 4; i++) {
        l[i] = bvec3[i][0] * bvec3[i][0] + bvec3[i][1] * bvec3[i][1] + bvec3[i][2] * bvec3[i][2];
        if (l[i] < l[itype]) itype = i;
    }
    int ivvec0[4] = {0, 0, 0, 0}, divvec[4][4]; /* divvec[col][row] */
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) divvec[c][r] = (c == r);
    ivvec0[itype] = 1;
    divvec[itype][itype] = -1;
    int ivvec[6][4][3];
    int it = 0;
    for (int i1 = 0; i1 < 3; i1++)
        for (int i2 = 0; i2 < 3; i2++) {
            if (i2 == i1) continue;
            for (int i3 = 0; i3 < 3; i3++) {
                if (i3 == i1 || i3 == i2) continue;
                for (int d = 0; d < 3; d++) {
                    ivvec[it][0][d] = ivvec0[d];
                    ivvec[it][1][d] = ivvec[it][0][d] + divvec[i1][d];
                    ivvec[it][2][d] = ivvec[it][1][d] + divvec[i2][d];
                    ivvec[it][3][d] = ivvec[it][2][d] + divvec[i3][d];
                }
                it++;
            }
        }
    long nt = 0;
    for (int i3 = 1; i3 <= n3; i3++)
        for (int i2 = 1; i2 <= n2; i2++)
            for (int i1 = 1; i1 <= n1; i1++)
                for (int t = 0; t < 6; t++) {
                    for (int ii = 0; ii < 4; ii++) {
                        int kv[3] = {i1 + ivvec[t][ii][0] - 1, i2 + ivvec[t][ii][1] - 1, i3 + ivvec[t][ii][2] - 1};
                        for (int d = 0; d < 3; d++) { kv[d] %= ng[d]; if (kv[d] < 0) kv[d] += ng[d]; }
                        idx1[4 * nt + ii] = 1 + kv[0] + ng[0] * kv[1] + ng[0] * ng[1] * kv[2];
                    }
                    nt++;
                }
}

/* ttct (:143-207).  dwgt[t][col i][vertex v] = dwgt(v, i, t) */
static int ttct(double dval, const double *dvtx, int imod, int *ntet, double (*dwgt)[4][4], double *dvol) {
    int bvtx[TT_NMAX][4], btsk[TT_NMAX];
    memset(bvtx, 0, sizeof bvtx); memset(btsk, 0, sizeof btsk);
    int itet = 0;
    while (itet < *ntet) {
        itet++;
        int t = itet - 1;
        double dvtx0[4];
        for (int i1 = 0; i1 < 4; i1++) {
            double s = 0;
            for (int v = 0; v < 4; v++) s += dwgt[t][i1][v] * dvtx[v];
            dvtx0[i1] = s;
        }
        int b1 = 0, i1, i2 = 0;
        for (i1 = 0; i1 < 3; i1++) {
            if (bvtx[t][i1]) continue;
            for (i2 = i1 + 1; i2 < 4; i2++) {
                if (bvtx[t][i2]) continue;
                b1 = (dvtx0[i1] - dval) * (dval - dvtx0[i2]) > 0.0;
                if (b1) break;
            }
            if (b1) break;
        }
        if (b1) {
            double d1 = (dvtx0[i2] - dval) / (dvtx0[i2] - dvtx0[i1]);
            double d2 = (dval - dvtx0[i1]) / (dvtx0[i2] - dvtx0[i1]);
            (*ntet)++;
            if (*ntet > TT_NMAX) return fail("ntet.gt.nmax");
            int nt = *ntet - 1;
            memcpy(bvtx[nt], bvtx[t], sizeof bvtx[t]);
            memcpy(dwgt[nt], dwgt[t], sizeof dwgt[t]);
            bvtx[nt][i1] = 1;
            for (int v = 0; v < 4; v++) dwgt[nt][i1][v] = dwgt[t][i1][v] * d1 + dwgt[t][i2][v] * d2;
            dvol[nt] = dvol[t] * d1;
            bvtx[t][i2] = 1;
            for (int v = 0; v < 4; v++) dwgt[t][i2][v] = dwgt[t][i1][v] * d1 + dwgt[t][i2][v] * d2;
            dvol[t] = dvol[t] * d2;
            itet--;
        } else {
            for (int a = 0; a < 4; a++) {
                if (bvtx[t][a]) continue;
                btsk[t] = btsk[t] || ((double)imod * (dvtx0[a] - dval) > 0.0);
            }
        }
    }
    int k = 0;
    for (int a = 0; a < *ntet; a++) {
        if (!btsk[a]) continue;
        memcpy(dwgt[k], dwgt[a], sizeof dwgt[a]);
        dvol[k] = dvol[a];
        k++;
    }
    *ntet = k;
    return 0;
}

/* closed forms (:304-451); x0(ne) */
static void sub1simple(cplx g0, int ne, const cplx *em, cplx *x) {
    for (int e = 0; e < ne; e++) x[e] = 1.0 / ((g0 + em[e]) * 6.0);
}
static void sub1g30g21(cplx g0, cplx g1, int ne, const cplx *em, cplx *x) {
    for (int e = 0; e < ne; e++) {
        cplx w = em[e], d = g0 - g1;
        cplx v = (0.5 * (g0 + g1) + w) / (d * d);
        v = v - clog((g0 + w) / (g1 + w)) * (g0 + w) * (g1 + w) / (d * d * d);
        x[e] = v;
    }
}
static void sub1g30g20(cplx g0, cplx g1, int ne, const cplx *em, cplx *x) {
    for (int e = 0; e < ne; e++) {
        cplx w = em[e], d = g0 - g1;
        cplx v = (g0 - 3.0 * g1 - 2.0 * w) * 0.25 / (d * d);
        v = v + (g1 + w) * (g1 + w) * clog((g0 + w) / (g1 + w)) * 0.5 / (d * d * d);
        x[e] = v;
    }
}
static void sub1g30(cplx g0, cplx g1, cplx g2, int ne, const cplx *em, cplx *x) {
    for (int e = 0; e < ne; e++) {
        cplx w = em[e];
        cplx v = 0.5 / (g0 - g2);
        cplx t = (g0 - g2) * (g0 - g1);
        v = v - 0.5 / (t * t) * (g0 + w) * (-2.0 * (g1 + w) * (g2 + w) + (g0 + w) * (g1 + g2 + 2.0 * w)) *
                    clog((g0 + w) / (g1 + w));
        v = v + 0.5 / ((g0 - g2) * (g0 - g2)) * (g2 + w) * (g2 + w) * clog((g1 + w) / (g2 + w)) / (g1 - g2);
        v = v + 0.5 / ((g0 - g2) * (g0 - g1)) * (g1 + w);
        x[e] = v;
    }
}
static void sub1normal(cplx g0, cplx g1, cplx g2, cplx g3, int ne, const cplx *em, cplx *x) {
    for (int e = 0; e < ne; e++) {
        cplx w = em[e];
        cplx L10 = clog((g1 + w) / (g0 + w)), L20 = clog((g2 + w) / (g0 + w)), L30 = clog((g3 + w) / (g0 + w));
        cplx v = (-(g1 + w) * (g1 + w) * L10) / ((g0 - g2) * (g0 - g3) * (g0 - g1)) * 0.5;
        v = v - ((g1 + w) * (g1 + w) * L10 - (g2 + w) * (g2 + w) * L20) / ((g0 - g2) * (g1 - g2) * (g2 - g3)) * 0.5;
        v = v + ((g1 + w) * (g1 + w) * L10 - (g3 + w) * (g3 + w) * L30) / ((g1 - g3) * (g0 - g3) * (g2 - g3)) * 0.5;
        x[e] = v;
    }
}
static void sub2simple(cplx g0, int ne, const cplx *em, cplx *x) {
    for (int e = 0; e < ne; e++) x[e] = 1.0 / ((g0 + em[e]) * 24.0);
}
static void sub2g30g20(cplx g0, cplx g1, int ne, const cplx *em, cplx *x) {
    for (int e = 0; e < ne; e++) {
        cplx w = em[e], d = g0 - g1;
        cplx v = ((g0 - g1) * (g0 + 2.0 * g1 + 3.0 * w) - 6.0 * (g0 + w) * (g1 + w)) / (12.0 * (d * d * d));
        v = v + (g0 + w) * (g1 + w) * (g1 + w) * clog((g0 + w) / (g1 + w)) / (d * d * d * d) * 0.5;
        x[e] = v;
    }
}
static void sub2g30g21(cplx g0, cplx g1, int ne, const cplx *em, cplx *x) { sub2g30g20(g1, g0, ne, em, x); }
static void sub2g30g10(cplx g0, cplx g2, int ne, const cplx *em, cplx *x) {
    for (int e = 0; e < ne; e++) {
        cplx w = em[e], d = g0 - g2;
        cplx v = (2.0 * (g0 + w) * (g0 + w) - 7.0 * (g0 + w) * (g2 + w) + 11.0 * (g2 + w) * (g2 + w)) / (36.0 * (d * d * d));
        v = v - (g2 + w) * (g2 + w) * (g2 + w) * clog((g0 + w) / (g2 + w)) / (6.0 * (d * d * d * d));
        x[e] = v;
    }
}
static void sub2g10(cplx g0, cplx g2, cplx g3, int ne, const cplx *em, cplx *x) {
    for (int e = 0; e < ne; e++) {
        cplx w = em[e], d2 = g0 - g2, d3 = g0 - g3;
        cplx v = (g0 + w) * ((g0 + w) * (g0 + w) + 5.0 * (g2 + w) * (g3 + w) - 3.0 * (g0 + w) * (g2 + g3 + 2.0 * w)) /
                 (12.0 * (d2 * d2) * (d3 * d3));
        v = v - (g2 + w) * (g2 + w) * (g2 + w) * clog((g2 + w) / (g0 + w)) / (6.0 * (d2 * d2 * d2) * (g2 - g3));
        v = v + (g3 + w) * (g3 + w) * (g3 + w) * clog((g3 + w) / (g0 + w)) / (6.0 * (d3 * d3 * d3) * (g2 - g3));
        x[e] = v;
    }
}
static void sub2g30(cplx g0, cplx g1, cplx g2, int ne, const cplx *em, cplx *x) {
    for (int e = 0; e < ne; e++) {
        cplx w = em[e];
        cplx d01 = g0 - g1, d02 = g0 - g2, d12 = g1 - g2;
        cplx v = ((g0 + w) * (g0 + w) * (g1 - g2) + (g1 + w) * (g1 + w) * (g0 - g2)) / (6.0 * d02 * (d01 * d01) * d12);
        v = v - (g0 + w) * (g0 + w) * (2.0 * (g1 + w) * (g0 - g2) + (g2 + w) * (g0 - g1)) * clog((g0 + w) / (g2 + w)) /
                    (6.0 * (d02 * d02) * (d01 * d01 * d01));
        v = v + (g1 + w) * (g1 + w) * (2.0 * (g0 + w) * (g1 - g2) - (g2 + w) * (g0 - g1)) * clog((g1 + w) / (g2 + w)) /
                    (6.0 * (d01 * d01 * d01) * (d12 * d12));
        x[e] = v;
    }
}
static void sub2normal(cplx g0, cplx g1, cplx g2, cplx g3, int ne, const cplx *em, cplx *x) {
    for (int e = 0; e < ne; e++) {
        cplx w = em[e];
        cplx v = -(g1 + w) * (g1 + w) / (6.0 * (g0 - g1) * (g1 - g2) * (g1 - g3));
        v = v - (g2 + w) * (g2 + w) * (g2 + w) * clog((g2 + w) / (g1 + w)) / (6.0 * (g0 - g2) * ((g1 - g2) * (g1 - g2)) * (g2 - g3));
        v = v + (g3 + w) * (g3 + w) * (g3 + w) * clog((g3 + w) / (g1 + w)) / (6.0 * (g0 - g3) * ((g1 - g3) * (g1 - g3)) * (g2 - g3));
        v = v + (g0 + w) * (g0 + w) * (g0 + w) * clog((g0 + w) / (g1 + w)) / (6.0 * ((g0 - g1) * (g0 - g1)) * (g0 - g2) * (g0 - g3));
        x[e] = v;
    }
}

/* chk1 (:457-503).  positions 0..3; ia1 maps position -> vertex id */
static int chk1(double dmna, double dmnr, const cplx *gk, const int *ia1, int *ia2, int *ia3, int *ia4, int *i3out) {
    int i3 = 0, i4 = 0;
    for (int a = 0; a < 4; a++) { ia2[a] = 0; ia3[a] = 0; ia4[a] = 0; }
    for (int i1 = 1; i1 <= 3; i1++)
        for (int i2 = i1 + 1; i2 <= 4; i2++) {
            int p = i1 % 4, r = i2 % 4; /* mod(i,4)+1, 0-based */
            double d1 = cabs(gk[ia1[p]] - gk[ia1[r]]);
            double d2 = cabs(gk[ia1[p]] + gk[ia1[r]]) * 0.5;
            if (d1 < dmna || d1 / d2 < dmnr) {
                i3++;
                if (ia2[p] == 0) { ia3[i4++] = ia1[p]; ia2[p] = 1; }
                if (ia2[r] == 0) { ia3[i4++] = ia1[r]; ia2[r] = 1; }
            }
        }
    int i5 = 0;
    for (int i1 = 1; i1 <= 4; i1++) {
        int p = i1 % 4;
        if (ia2[p] == 0) ia4[i5++] = ia1[p];
    }
    int s = ia2[0] + ia2[1] + ia2[2] + ia2[3];
    if (s != i4) return fail("bad ia2 and i4");
    if (i4 + i5 != 4) return fail("bad i4 and i5");
    *i3out = i3;
    return 0;
}

/* calc (:209-302).  fk, gk, xo are indexed by vertex id; xo[id*ne + e] */
static int tt_calc(double dmna, double dmnr, const int *ia1, const cplx *fk, const cplx *gk, int ne,
                   const cplx *em, cplx *ca1 /* 4*ne */, cplx *xo) {
    int ia2[4], ia3[4], ia4[4], i3 = 0;
    if (chk1(dmna, dmnr, gk, ia1, ia2, ia3, ia4, &i3)) return 1;
    cplx *c1 = ca1, *c2 = ca1 + ne, *c3 = ca1 + 2 * ne, *c4 = ca1 + 3 * ne;
    int s = ia2[0] + ia2[1] + ia2[2] + ia2[3];
    switch (s) {
    case 0:
        sub2normal(gk[ia4[1]], gk[ia4[0]], gk[ia4[2]], gk[ia4[3]], ne, em, c1);
        sub2normal(gk[ia4[0]], gk[ia4[1]], gk[ia4[2]], gk[ia4[3]], ne, em, c2);
        sub2normal(gk[ia4[0]], gk[ia4[2]], gk[ia4[1]], gk[ia4[3]], ne, em, c3);
        sub1normal(gk[ia4[0]], gk[ia4[3]], gk[ia4[1]], gk[ia4[2]], ne, em, c4);
        for (int e = 0; e < ne; e++) {
            xo[(long)ia4[0] * ne + e] += fk[ia4[0]] * c1[e];
            xo[(long)ia4[1] * ne + e] += fk[ia4[1]] * c2[e];
            xo[(long)ia4[2] * ne + e] += fk[ia4[2]] * c3[e];
            xo[(long)ia4[3] * ne + e] += fk[ia4[3]] * (c4[e] - c3[e] - c2[e] - c1[e]);
        }
        break;
    case 2: {
        cplx geq1 = (gk[ia3[0]] + gk[ia3[1]]) / 2.0;
        sub2g10(geq1, gk[ia4[0]], gk[ia4[1]], ne, em, c1);
        sub2g30(geq1, gk[ia4[0]], gk[ia4[1]], ne, em, c2);
        sub1g30(geq1, gk[ia4[1]], gk[ia4[0]], ne, em, c3);
        for (int e = 0; e < ne; e++) {
            xo[(long)ia3[0] * ne + e] += fk[ia3[0]] * c1[e];
            xo[(long)ia3[1] * ne + e] += fk[ia3[1]] * c1[e];
            xo[(long)ia4[0] * ne + e] += fk[ia4[0]] * c2[e];
            xo[(long)ia4[1] * ne + e] += fk[ia4[1]] * (c3[e] - c2[e] - c1[e] - c1[e]);
        }
        break;
    }
    case 3: {
        cplx geq1 = (gk[ia3[0]] + gk[ia3[1]] + gk[ia3[2]]) / 3.0;
        sub2g30g10(geq1, gk[ia4[0]], ne, em, c1);
        sub1g30g20(geq1, gk[ia4[0]], ne, em, c2);
        for (int e = 0; e < ne; e++) {
            xo[(long)ia3[0] * ne + e] += fk[ia3[0]] * c1[e];
            xo[(long)ia3[1] * ne + e] += fk[ia3[1]] * c1[e];
            xo[(long)ia3[2] * ne + e] += fk[ia3[2]] * c1[e];
            xo[(long)ia4[0] * ne + e] += fk[ia4[0]] * (c2[e] - c1[e] - c1[e] - c1[e]);
        }
        break;
    }
    case 4:
        if (i3 == 2) {
            cplx geq1 = (gk[ia3[0]] + gk[ia3[1]]) / 2.0, geq2 = (gk[ia3[2]] + gk[ia3[3]]) / 2.0;
            /* sub2g30g21(geq2, geq1, geq1, geq2) = sub2g30g20(geq1, geq2, ...) */
            sub2g30g21(geq2, geq1, ne, em, c1);
            sub1g30g21(geq1, geq2, ne, em, c2);
            for (int e = 0; e < ne; e++) {
                xo[(long)ia3[0] * ne + e] += fk[ia3[0]] * c1[e];
                xo[(long)ia3[1] * ne + e] += fk[ia3[1]] * c1[e];
                xo[(long)ia3[2] * ne + e] += fk[ia3[2]] * (c2[e] - c1[e] - c1[e]) * 0.5;
                xo[(long)ia3[3] * ne + e] += fk[ia3[3]] * (c2[e] - c1[e] - c1[e]) * 0.5;
            }
        } else if (i3 >= 3 && i3 <= 6) {
            cplx geq1 = (gk[ia3[0]] + gk[ia3[1]] + gk[ia3[2]] + gk[ia3[3]]) / 4.0;
            sub2simple(geq1, ne, em, c1);
            for (int e = 0; e < ne; e++)
                for (int a = 0; a < 4; a++) xo[(long)ia3[a] * ne + e] += c1[e] * fk[ia3[a]];
        } else {
            return fail("bad i3");
        }
        break;
    default:
        return fail("bad sum ia2");
    }
    (void)sub1simple;
    return 0;
}

/* body of the ttrhdrn_chi0 tetrahedron loop (:119-136) for one tetrahedron
 * whose vertices carry ee1/ee2; accumulates into xo4[vertex*ne + e] */
static int tt_one(double dmna, double dmnr, const double *ee1, const double *ee2, double f1, double f2,
                  double delt, double dsgn, int ne, const cplx *em, double (*dwgt)[4][4], double *dvol,
                  cplx *ca1, cplx *xxo, const int *vmap, cplx *xo4) {
    const int ia1[4] = {0, 1, 2, 3};
    memset(dwgt[0], 0, sizeof dwgt[0]);
    for (int a = 0; a < 4; a++) dwgt[0][a][a] = 1.0;
    dvol[0] = 1.0;
    int ntet = 1;
    if (ttct(f2, ee2, +1, &ntet, dwgt, dvol)) return 1;
    if (ttct(f1, ee1, -1, &ntet, dwgt, dvol)) return 1;
    for (int i3 = 0; i3 < ntet; i3++) {
        cplx ffk[4], ggk[4];
        memset(xxo, 0, sizeof(cplx) * 4 * ne);
        for (int a = 0; a < 4; a++) ffk[a] = dvol[i3];
        for (int i4 = 0; i4 < 4; i4++) {
            double sm = 0;
            for (int vv = 0; vv < 4; vv++) sm += (ee2[vv] - ee1[vv]) * dwgt[i3][i4][vv];
            ggk[i4] = -(sm - I * delt);
        }
        for (int a = 0; a < 4; a++) { ffk[a] *= dsgn; ggk[a] *= dsgn; }
        if (tt_calc(dmna, dmnr, ia1, ffk, ggk, ne, em, ca1, xxo)) return 1;
        for (int i4 = 0; i4 < 4; i4++)
            for (int i5 = 0; i5 < 4; i5++) {
                double wgt = dwgt[i3][i4][i5];
                long dst = (long)(vmap ? vmap[i5] : i5) * ne;
                for (int e = 0; e < ne; e++) xo4[dst + e] += xxo[i4 * ne + e] * wgt;
            }
    }
    return 0;
}

/* ttrhdrn_chi0 (:99-141): e1, e2 real energies on the mesh; xo[(k)*ne + e] */
static int ttrhdrn_chi0(double dmna, double dmnr, int nk, const int *imt1, const double *e1, const double *e2,
                        double f1, double f2, double delt, double dsgn, int ne, const cplx *em, cplx *xo) {
    static __thread double (*dwgt)[4][4] = NULL;
    static __thread double *dvol = NULL;
    if (!dwgt) { dwgt = malloc(sizeof(double) * 16 * TT_NMAX); dvol = malloc(sizeof(double) * TT_NMAX); }
    cplx *ca1 = (cplx *)malloc(sizeof(cplx) * 4 * ne);
    cplx *xxo = (cplx *)malloc(sizeof(cplx) * 4 * ne);
    long ntet_all = (long)nk * 6;
    int rc = 0;
    for (long t = 0; t < ntet_all && !rc; t++) {
        const int *v = imt1 + 4 * t;
        double ee2[4], ee1[4];
        int vm0[4];
        for (int a = 0; a < 4; a++) { ee2[a] = e2[v[a] - 1]; ee1[a] = e1[v[a] - 1]; vm0[a] = v[a] - 1; }
        rc = tt_one(dmna, dmnr, ee1, ee2, f1, f2, delt, dsgn, ne, em, dwgt, dvol, ca1, xxo, vm0, xo);
    }
    free(ca1); free(xxo);
    return rc;
}

int orc_tt_one(double dmna, double dmnr, const double *ee1, const double *ee2, double f1, double f2, double delt,
               double dsgn, int ne, const double *em, double *xo4) {
    double (*dwgt)[4][4] = malloc(sizeof(double) * 16 * TT_NMAX);
    double *dvol = malloc(sizeof(double) * TT_NMAX);
    cplx *ca1 = malloc(sizeof(cplx) * 4 * ne), *xxo = malloc(sizeof(cplx) * 4 * ne);
    int rc = tt_one(dmna, dmnr, ee1, ee2, f1, f2, delt, dsgn, ne, (const cplx *)em, dwgt, dvol, ca1, xxo, NULL, (cplx *)xo4);
    free(dwgt); free(dvol); free(ca1); free(xxo);
    return rc;
}

int orc_ttrhdrn_chi0(double dmna, double dmnr, int n1, int n2, int n3, const int *imt1, const double *e1,
                     const double *e2, double f1, double f2, double delt, double dsgn, int ne, const double *em,
                     double *xo) {
    return ttrhdrn_chi0(dmna, dmnr, n1 * n2 * n3, imt1, e1, e2, f1, f2, delt, dsgn, ne, (const cplx *)em, (cplx *)xo);
}

/* ttrhdrn_simple / ttrhdrn_sum (:63-97): ne = 1, em = 0 */
int orc_ttrhdrn_simple(double dmna, double dmnr, int n1, int n2, int n3, const int *imt1, const double *fk,
                       const double *gk, double *xo) {
    long nt = (long)n1 * n2 * n3 * 6;
    cplx em0 = 0, ca1[4];
    for (long t = 0; t < nt; t++) {
        int ia1[4];
        for (int a = 0; a < 4; a++) ia1[a] = imt1[4 * t + a] - 1;
        if (tt_calc(dmna, dmnr, ia1, (const cplx *)fk, (const cplx *)gk, 1, &em0, ca1, (cplx *)xo)) return 1;
    }
    return 0;
}

/* ========================================================================= */
/* the calc_chiqw driver                                                      */
/* ========================================================================= */
typedef struct {
    /* lattice */
    double a1[3], a2[3], a3[3], b1[3], b2[3], b3[3], VOLUME;
    /* symmetry */
    int nsymq, nnp; int *rg; /* rg[iop*9 + i + 3j] */ int *pg; double *rginv;
    /* k */
    int Nk_irr; double *SKI, *SKI_list;
    int NTG, NTB, *NGI, *KGI; /* KGI[(ik*NTG + ig)*3 + d] */
    double *E_EIGI; /* [ik*NTB + ib] */
    double Ecut_psi, Ecut_eps, FermiEnergy;
    int L1, L2, L3; int *packing; /* [ik][i1+L1][j1+L2][k1+L3] */
    int nw[3];
    int NTK; double *SK0; int *numirr, *numrot, *trs, *RW;
    int nkb[3]; int *NG0, *KG0; /* KG0[(jk*NTG+ig)*3+d] */
    int *index_kpt; /* [ix + nkb1*(iy + nkb2*iz)] -> 0-based k */
    int *WindowInside, *Tindx; double *E_AVE, *band_max, *band_min;
    cplx *prob; /* [ik*NTB + ib] (full k) */
    int NCB, N_docc, N_pocc, N_uocc, N_occ, N_vir;
    cplx *C; /* coefficients [(ik*NCB + ib)*NTG + ig] for bands 0..NCB-1 */
    int nen; cplx *em;
    int *imt1;
    double delt, delta_ex, dmna, dmnr;
} orc_state;

static void free_state(orc_state *s) {
    free(s->rg); free(s->pg); free(s->rginv); free(s->SKI); free(s->SKI_list); free(s->NGI); free(s->KGI);
    free(s->E_EIGI); free(s->packing); free(s->SK0); free(s->numirr); free(s->numrot); free(s->trs); free(s->RW);
    free(s->NG0); free(s->KG0); free(s->index_kpt); free(s->WindowInside); free(s->Tindx); free(s->E_AVE);
    free(s->band_max); free(s->band_min); free(s->prob); free(s->C); free(s->em); free(s->imt1);
}

static void outer(const double *x, const double *y, double *z) {
    z[0] = x[1] * y[2] - x[2] * y[1]; z[1] = x[2] * y[0] - x[0] * y[2]; z[2] = x[0] * y[1] - x[1] * y[0];
}

static int path_join(char *out, size_t n, const char *a, const char *b) {
    int r = snprintf(out, n, "%s/%s", a, b);
    return (r < 0 || (size_t)r >= n) ? fail("path too long") : 0;
}

/* judge_FermiInside / judge_WindowInside (chiqw_sub.F:570-666) */
static void judge(orc_state *s, int window, double EL, double EU) {
    for (int ib = 0; ib < s->NTB; ib++) {
        double top = 0, btm = 0; int fsv = 0;
        for (int ik = 0; ik < s->Nk_irr; ik++) {
            double e = s->E_EIGI[(long)ik * s->NTB + ib];
            if (ik == 0) { top = e; btm = e; }
            if (e < btm) btm = e;
            if (e > top) top = e;
        }
        s->Tindx[ib] = 0;
        if (!window) {
            if (btm > s->FermiEnergy) fsv = 2;
            if (btm <= s->FermiEnergy && top >= s->FermiEnergy) { fsv = 1; s->Tindx[ib] = ib + 1; }
            if (top < s->FermiEnergy) fsv = 0;
        } else {
            if (top < EL) fsv = 0;
            if (EL <= top && top < EU && btm < EL) fsv = 0;
            if (EL <= top && top < EU && EL <= btm && btm < EU) { fsv = 1; s->Tindx[ib] = ib + 1; }
            if (btm < EL && top > EU) { fsv = 1; s->Tindx[ib] = ib + 1; }
            if (EL < btm && btm < EU && top > EU) fsv = 2;
            if (btm > EU) fsv = 2;
        }
        s->WindowInside[ib] = fsv;
        s->E_AVE[ib] = (top + btm) / 2.0;
        s->band_max[ib] = top;
        s->band_min[ib] = btm;
    }
}

/* make_C0 (chiqw_sub.F:264-322): rotate band `band` of irreducible k into full k jk */
static void make_C0(const orc_state *s, int jk, int band, cplx *out) {
    int ikir = s->numirr[jk], iop = s->numrot[jk], itrs = s->trs[jk];
    const double *ri = s->rginv + 9 * iop;
    const int *pgt = s->pg + 3 * iop;
    const int *RWt = s->RW + 3 * jk;
    const cplx *src = s->C + ((long)ikir * s->NCB + band) * s->NTG;
    int n1 = 2 * s->L1 + 1, n2 = 2 * s->L2 + 1, n3 = 2 * s->L3 + 1;
    const int *pk = s->packing + (long)ikir * n1 * n2 * n3;
    int NG = s->NG0[jk];
    for (int ig = 0; ig < s->NTG; ig++) out[ig] = 0;
    for (int ig = 0; ig < NG; ig++) {
        const int *g = s->KG0 + ((long)jk * s->NTG + ig) * 3;
        int i1 = g[0], j1 = g[1], k1 = g[2];
        if (itrs == -1) { i1 = -i1; j1 = -j1; k1 = -k1; }
        int i2 = i1 + RWt[0], j2 = j1 + RWt[1], k2 = k1 + RWt[2];
        int i3 = (int)ri[0] * i2 + (int)ri[3] * j2 + (int)ri[6] * k2;
        int j3 = (int)ri[1] * i2 + (int)ri[4] * j2 + (int)ri[7] * k2;
        int k3 = (int)ri[2] * i2 + (int)ri[5] * j2 + (int)ri[8] * k2;
        int jg = 0;
        if (abs(i3) <= s->L1 && abs(j3) <= s->L2 && abs(k3) <= s->L3)
            jg = pk[(i3 + s->L1) + n1 * ((j3 + s->L2) + (long)n2 * (k3 + s->L3))];
        double phase = TPI * ((double)i1 * (double)pgt[0] + (double)j1 * (double)pgt[1] + (double)k1 * (double)pgt[2]);
        cplx pf = cexp(-I * phase / (double)s->nnp);
        cplx v = jg > 0 ? src[jg - 1] : 0;
        out[ig] = v * pf;
    }
    if (itrs == -1)
        for (int ig = 0; ig < NG; ig++) out[ig] = conj(out[ig]);
}

static inline int wrapidx(int g, int n) { int m = g % n; return m < 0 ? m + n : m; }

/* calc_InterStateMatrix (chiqw_sub.F:97-205) */
static void interstate(const orc_state *s, int ik, int ikq, const cplx *C0K, const cplx *C0KQ, const int *LG0, int NG,
                       const int *shiftG, cplx *wk, cplx *wkq, cplx *m_tmp) {
    int n1 = s->nw[0], n2 = s->nw[1], n3 = s->nw[2];
    long N = (long)n1 * n2 * n3;
    for (long i = 0; i < N; i++) { wk[i] = 0; wkq[i] = 0; }
    for (int ig = 0; ig < s->NG0[ik]; ig++) {
        const int *g = s->KG0 + ((long)ik * s->NTG + ig) * 3;
        long ind = wrapidx(g[0], n1) + n1 * (wrapidx(g[1], n2) + (long)n2 * wrapidx(g[2], n3));
        wk[ind] = C0K[ig];
    }
    fft3(n1, n2, n3, wk, 0);
    for (long i = 0; i < N; i++) wk[i] = SGLC(creal(wk[i]), cimag(wk[i]));
    for (int ig = 0; ig < s->NG0[ikq]; ig++) {
        const int *g = s->KG0 + ((long)ikq * s->NTG + ig) * 3;
        long ind = wrapidx(g[0], n1) + n1 * (wrapidx(g[1], n2) + (long)n2 * wrapidx(g[2], n3));
        wkq[ind] = C0KQ[ig];
    }
    fft3(n1, n2, n3, wkq, 0);
    for (long i = 0; i < N; i++) wkq[i] = SGLC(creal(wkq[i]), cimag(wkq[i]));
    double dG1 = shiftG[0], dG2 = shiftG[1], dG3 = shiftG[2];
    for (int r3 = 0; r3 < n3; r3++)
        for (int r2 = 0; r2 < n2; r2++)
            for (int r1 = 0; r1 < n1; r1++) {
                long ir = r1 + n1 * (r2 + (long)n2 * r3);
                double phase = TPI * ((double)r1 * dG1 / (double)n1 + (double)r2 * dG2 / (double)n2 +
                                      (double)r3 * dG3 / (double)n3);
                cplx pf = cexp(-I * phase);
                wkq[ir] = wkq[ir] * pf;
            }
    for (long i = 0; i < N; i++) wk[i] = conj(wkq[i]) * wk[i];
    fft3(n1, n2, n3, wk, 1);
    for (int igL = 0; igL < NG; igL++) {
        int i1 = wrapidx(-LG0[3 * igL], n1), i2 = wrapidx(-LG0[3 * igL + 1], n2), i3 = wrapidx(-LG0[3 * igL + 2], n3);
        cplx v = wk[i1 + n1 * (i2 + (long)n2 * i3)];
        m_tmp[igL] = SGLC(creal(v), cimag(v));
    }
}

/* calc_VMab / calc_VMaa (chiqw_sub.F:207-262); skt == NULL for VMab */
static void calc_vm(const orc_state *s, int ik, const cplx *C0K, const cplx *C0KQ, const double *skt, cplx *vm) {
    cplx S[3] = {0, 0, 0};
    for (int ig = 0; ig < s->NG0[ik]; ig++) {
        const int *g = s->KG0 + ((long)ik * s->NTG + ig) * 3;
        double G[3];
        double x1 = g[0], x2 = g[1], x3 = g[2];
        if (skt) { x1 += skt[0]; x2 += skt[1]; x3 += skt[2]; }
        for (int d = 0; d < 3; d++) G[d] = x1 * s->b1[d] + x2 * s->b2[d] + x3 * s->b3[d];
        cplx pr = conj(C0KQ[ig]) * C0K[ig];
        for (int d = 0; d < 3; d++) S[d] += G[d] * pr;
    }
    for (int d = 0; d < 3; d++) vm[d] = S[d] * I;
}

static double qg_len(const orc_state *s, const double *q, const int *g) {
    double v[3];
    for (int d = 0; d < 3; d++)
        v[d] = (q[0] + (double)g[0]) * s->b1[d] + (q[1] + (double)g[1]) * s->b2[d] + (q[2] + (double)g[2]) * s->b3[d];
    return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
}

/* calc_eps_rpa (chiqw_sub.F:386-457) and calc_eps_rpa_q_0 (:459-568).
 * chi0 is overwritten by eps^-1.  Writes the diagonal text file if fp. */
static int eps_rpa(const orc_state *s, const double *q, const int *LG0, int NG, cplx *chi0, int gamma, int No_G_0,
                   double wd, double delt, cplx wcmplx, FILE *fp) {
    double *ql = (double *)malloc(sizeof(double) * NG);
    for (int ig = 0; ig < NG; ig++) ql[ig] = qg_len(s, q, LG0 + 3 * ig);
    for (long i = 0; i < (long)NG * NG; i++) chi0[i] = 2.0 * chi0[i];
    double w = creal(wcmplx);
    if (gamma && w == 0.0) w = 1.0e-5;
    for (int jg = 0; jg < NG; jg++)
        for (int ig = 0; ig < NG; ig++) {
            cplx c = chi0[ig + (long)NG * jg], e;
            double qi = ql[ig], qj = ql[jg];
            if (!gamma) {
                if (ig == jg) e = 1.0 - c * 2.0 * TPI / qi / qj;
                else e = -c * 2.0 * TPI / qi / qj;
            } else {
                if (ig == jg && ig == No_G_0) {
                    cplx drude = SGLC(-wd * wd / (w * w + delt * delt), delt * wd * wd / (w * w * w + w * delt * delt));
                    e = 1.0 - c * 2.0 * TPI + drude;
                } else if (ig == jg) e = 1.0 - c * 2.0 * TPI / qi / qj;
                else if (ig == No_G_0) e = -c * 2.0 * TPI / qj;
                else if (jg == No_G_0) e = -c * 2.0 * TPI / qi;
                else e = -c * 2.0 * TPI / qi / qj;
            }
            chi0[ig + (long)NG * jg] = e;
        }
    if (zinv(NG, chi0)) { free(ql); return 1; }
    if (fp)
        for (int ig = 0; ig < NG; ig++) {
            cplx f = chi0[ig + (long)NG * ig];
            fprintf(fp, "%20.10f%20.10f%20.10f\n", ql[ig], creal(f), cimag(f));
        }
    free(ql);
    return 0;
}

static int mkdir_p(const char *p) {
    if (mkdir(p, 0755) && errno != EEXIST) return fail("mkdir %s", p);
    return 0;
}

static int read_inputs(orc_state *s, const char *root, const orc_params *P) {
    char path[4096], d[4096];
    ldr r;
    if (path_join(d, sizeof d, root, "dir-wfn")) return 1;
    /* dat.bandcalc (chiqw.F:87-97) */
    snprintf(path, sizeof path, "%s/dat.bandcalc", d);
    if (ld_open(&r, path)) return 1;
    double v[3];
    if (ld_read(&r, 1, v) || ld_read(&r, 1, v + 1) || ld_read(&r, 1, v + 2)) { ld_close(&r); return 1; }
    ld_close(&r);
    s->Ecut_psi = v[0];
    s->FermiEnergy = v[1] + P->shift_ef / AU;
    /* dat.lattice (:148-161) */
    snprintf(path, sizeof path, "%s/dat.lattice", d);
    if (ld_open(&r, path)) return 1;
    if (ld_read(&r, 3, s->a1) || ld_read(&r, 3, s->a2) || ld_read(&r, 3, s->a3)) { ld_close(&r); return 1; }
    ld_close(&r);
    outer(s->a2, s->a3, s->b1);
    s->VOLUME = s->a1[0] * s->b1[0] + s->a1[1] * s->b1[1] + s->a1[2] * s->b1[2];
    for (int i = 0; i < 3; i++) s->b1[i] = s->b1[i] * TPI / s->VOLUME;
    outer(s->a3, s->a1, s->b2);
    for (int i = 0; i < 3; i++) s->b2[i] = s->b2[i] * TPI / s->VOLUME;
    outer(s->a1, s->a2, s->b3);
    for (int i = 0; i < 3; i++) s->b3[i] = s->b3[i] * TPI / s->VOLUME;
    /* dat.symmetry (:186-202) */
    snprintf(path, sizeof path, "%s/dat.symmetry", d);
    if (ld_open(&r, path)) return 1;
    if (ld_int(&r, 1, &s->nsymq) || ld_int(&r, 1, &s->nnp)) { ld_close(&r); return 1; }
    s->rg = calloc(9 * s->nsymq, sizeof(int)); s->pg = calloc(3 * s->nsymq, sizeof(int));
    s->rginv = calloc(9 * s->nsymq, sizeof(double));
    for (int iop = 0; iop < s->nsymq; iop++) {
        if (ld_int(&r, 9, s->rg + 9 * iop) || ld_int(&r, 3, s->pg + 3 * iop)) { ld_close(&r); return 1; }
        inv3(s->rg + 9 * iop, s->rginv + 9 * iop);
    }
    ld_close(&r);
    /* dat.sample-k (:252-270) */
    snprintf(path, sizeof path, "%s/dat.sample-k", d);
    if (ld_open(&r, path)) return 1;
    if (ld_int(&r, 1, &s->Nk_irr)) { ld_close(&r); return 1; }
    s->SKI = calloc(3 * s->Nk_irr, sizeof(double)); s->SKI_list = calloc(3 * s->Nk_irr, sizeof(double));
    for (int ik = 0; ik < s->Nk_irr; ik++) {
        if (ld_read(&r, 3, s->SKI + 3 * ik)) { ld_close(&r); return 1; }
        search_list(s->SKI + 3 * ik, s->SKI_list + 3 * ik);
    }
    ld_close(&r);
    /* dat.nkm (:276-287) */
    snprintf(path, sizeof path, "%s/dat.nkm", d);
    if (ld_open(&r, path)) return 1;
    s->NGI = calloc(s->Nk_irr, sizeof(int));
    s->NTG = 0;
    for (int ik = 0; ik < s->Nk_irr; ik++) {
        if (ld_int(&r, 1, s->NGI + ik)) { ld_close(&r); return 1; }
        if (abs(s->NGI[ik]) > s->NTG) s->NTG = abs(s->NGI[ik]);
    }
    ld_close(&r);
    /* dat.eigenvalue (:289-305) */
    snprintf(path, sizeof path, "%s/dat.eigenvalue", d);
    if (ld_open(&r, path)) return 1;
    if (ld_int(&r, 1, &s->NTB)) { ld_close(&r); return 1; }
    s->E_EIGI = calloc((long)s->NTB * s->Nk_irr, sizeof(double));
    for (int ik = 0; ik < s->Nk_irr; ik++)
        for (int ib = 0; ib < s->NTB; ib++)
            if (ld_read(&r, 1, s->E_EIGI + (long)ik * s->NTB + ib)) { ld_close(&r); return 1; }
    ld_close(&r);
    s->NCB = P->n_calc_band > 0 ? P->n_calc_band : s->NTB;
    if (s->NCB > s->NTB) return fail("N_CALC_BAND > NTB");
    /* dat.kg (:314-329) */
    snprintf(path, sizeof path, "%s/dat.kg", d);
    if (ld_open(&r, path)) return 1;
    s->KGI = calloc((long)3 * s->NTG * s->Nk_irr, sizeof(int));
    for (int ik = 0; ik < s->Nk_irr; ik++) {
        int ng;
        if (ld_int(&r, 1, &ng)) { ld_close(&r); return 1; }
        if (ng != s->NGI[ik]) { ld_close(&r); return fail("NG_for_psi should be NGI(ik)"); }
        for (int ig = 0; ig < ng; ig++)
            if (ld_int(&r, 3, s->KGI + ((long)ik * s->NTG + ig) * 3)) { ld_close(&r); return 1; }
    }
    ld_close(&r);
    return 0;
}

static int setup(orc_state *s, const char *root, const orc_params *P) {
    if (read_inputs(s, root, P)) return 1;
    /* Ecut_psi from the plane-wave lists (:331-352) */
    double mx = 0;
    for (int ik = 0; ik < s->Nk_irr; ik++)
        for (int ig = 0; ig < s->NGI[ik]; ig++) {
            const int *g = s->KGI + ((long)ik * s->NTG + ig) * 3;
            double k[3];
            for (int d = 0; d < 3; d++)
                k[d] = (s->SKI[3 * ik] + g[0]) * s->b1[d] + (s->SKI[3 * ik + 1] + g[1]) * s->b2[d] +
                       (s->SKI[3 * ik + 2] + g[2]) * s->b3[d];
            double l = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
            if ((ik == 0 && ig == 0) || l > mx) mx = l;
        }
    s->Ecut_psi = mx + 1.0e-8;
    s->Ecut_eps = P->ecut_for_eps != 0.0 ? P->ecut_for_eps : s->Ecut_psi / 10.0;
    /* packing (:364-378) */
    s->L1 = s->L2 = s->L3 = 0;
    for (long i = 0; i < (long)s->Nk_irr * s->NTG; i++) {
        if (abs(s->KGI[3 * i]) > s->L1) s->L1 = abs(s->KGI[3 * i]);
        if (abs(s->KGI[3 * i + 1]) > s->L2) s->L2 = abs(s->KGI[3 * i + 1]);
        if (abs(s->KGI[3 * i + 2]) > s->L3) s->L3 = abs(s->KGI[3 * i + 2]);
    }
    s->L1++; s->L2++; s->L3++;
    int n1 = 2 * s->L1 + 1, n2 = 2 * s->L2 + 1, n3 = 2 * s->L3 + 1;
    s->packing = calloc((long)n1 * n2 * n3 * s->Nk_irr, sizeof(int));
    for (int ik = 0; ik < s->Nk_irr; ik++)
        for (int ig = 0; ig < s->NGI[ik]; ig++) {
            const int *g = s->KGI + ((long)ik * s->NTG + ig) * 3;
            s->packing[(long)ik * n1 * n2 * n3 + (g[0] + s->L1) + n1 * ((g[1] + s->L2) + (long)n2 * (g[2] + s->L3))] = ig + 1;
        }
    /* FFT grid (:389-416) */
    if (P->fft_box[0] > 0) {
        for (int i = 0; i < 3; i++) s->nw[i] = P->fft_box[i];
    } else {
        const double *av[3] = {s->a1, s->a2, s->a3}, *bv[3] = {s->b1, s->b2, s->b3};
        double qwf = 2.0 * sqrt(s->Ecut_psi);
        for (int i = 0; i < 3; i++) {
            double h = sqrt(av[i][0] * av[i][0] + av[i][1] * av[i][1] + av[i][2] * av[i][2]);
            double dd = fabs(bv[i][0] * av[i][0] / h + bv[i][1] * av[i][1] / h + bv[i][2] * av[i][2] / h);
            s->nw[i] = orc_algn235((int)(qwf / dd) + 1);
        }
    }
    /* est_NTK + unfold (est_NTK.f90:42-98, chiqw.F:437-480) */
    int Nmax = s->Nk_irr * s->nsymq * 2;
    s->SK0 = calloc(3 * Nmax, sizeof(double)); s->numirr = calloc(Nmax, sizeof(int));
    s->numrot = calloc(Nmax, sizeof(int)); s->trs = calloc(Nmax, sizeof(int)); s->RW = calloc(3 * Nmax, sizeof(int));
    int jk = 0;
    for (int ik = 0; ik < s->Nk_irr; ik++)
        for (int iop = 0; iop < s->nsymq; iop++) {
            const int *R = s->rg + 9 * iop;
            const double *k = s->SKI + 3 * ik;
            for (int pass = 0; pass < 2; pass++) {
                double kt[3]; int RWt[3] = {0, 0, 0};
                for (int i = 0; i < 3; i++)
                    kt[i] = (double)R[i] * k[0] + (double)R[i + 3] * k[1] + (double)R[i + 6] * k[2];
                if (pass == 0) kcheck(kt, RWt); else kcheck_trs(kt, RWt);
                double sgn = pass == 0 ? 1.0 : -1.0;
                int dup = 0;
                for (int iik = 0; iik < jk; iik++)
                    if (fabs(s->SK0[3 * iik] - sgn * kt[0]) < 1e-4 && fabs(s->SK0[3 * iik + 1] - sgn * kt[1]) < 1e-4 &&
                        fabs(s->SK0[3 * iik + 2] - sgn * kt[2]) < 1e-4) { dup = 1; break; }
                if (dup) continue;
                for (int i = 0; i < 3; i++) { s->SK0[3 * jk + i] = sgn * kt[i]; s->RW[3 * jk + i] = RWt[i]; }
                s->numirr[jk] = ik; s->numrot[jk] = iop; s->trs[jk] = pass == 0 ? 1 : -1;
                jk++;
            }
        }
    s->NTK = jk;
    /* est_nkbi (est_NTK.f90:1-39) */
    for (int d = 0; d < 3; d++) {
        double x = 1.0;
        for (int i = 0; i < s->NTK; i++) {
            double a = fabs(s->SK0[3 * i + d]);
            if (a < 1.0e-7) continue;
            if (a < x) x = a;
        }
        s->nkb[d] = (int)lround(1.0 / x);
    }
    if (s->nkb[0] * s->nkb[1] * s->nkb[2] != s->NTK) return fail("k mesh %dx%dx%d does not match NTK=%d", s->nkb[0], s->nkb[1], s->nkb[2], s->NTK);
    /* KG0 per full k (chiqw.F:509-545) */
    s->NG0 = calloc(s->NTK, sizeof(int)); s->KG0 = calloc((long)3 * s->NTG * s->NTK, sizeof(int));
    for (int j = 0; j < s->NTK; j++) {
        int ik = s->numirr[j], iop = s->numrot[j];
        const int *R = s->rg + 9 * iop;
        const double *k = s->SKI + 3 * ik;
        double kt[3];
        for (int i = 0; i < 3; i++)
            kt[i] = (double)R[i] * k[0] + (double)R[i + 3] * k[1] + (double)R[i + 6] * k[2] + (double)s->RW[3 * j + i];
        int ng;
        int *dst = s->KG0 + (long)j * s->NTG * 3;
        if (make_KG0(s->NTG, s->b1, s->b2, s->b3, s->Ecut_psi, kt[0], kt[1], kt[2], dst, &ng)) return 1;
        if (ng != s->NGI[ik]) return fail("NG_for_psi should be NGI(ik) (full k %d)", j + 1);
        s->NG0[j] = ng;
        if (s->trs[j] == -1)
            for (int i = 0; i < 3 * ng; i++) dst[i] = -dst[i];
    }
    /* index_kpt (chiqw_sub.F:324-384) */
    s->index_kpt = calloc(s->NTK, sizeof(int));
    for (int ik = 0; ik < s->NTK; ik++) {
        int ix[3];
        for (int d = 0; d < 3; d++) {
            double x = s->SK0[3 * ik + d] * (double)s->nkb[d];
            if (s->NTK % 2 != 0) { x += ((double)s->nkb[d] - 1.0) / 2.0; ix[d] = (int)lround(x) + 1; }
            else { x += (double)s->nkb[d] / 2.0; ix[d] = (int)lround(x); }
            if (ix[d] < 1 || ix[d] > s->nkb[d]) return fail("index_kpt out of range");
        }
        s->index_kpt[(ix[0] - 1) + s->nkb[0] * ((ix[1] - 1) + s->nkb[1] * (ix[2] - 1))] = ik;
    }
    /* band classification (chiqw.F:817-837) */
    s->WindowInside = calloc(s->NTB, sizeof(int)); s->Tindx = calloc(s->NTB, sizeof(int));
    s->E_AVE = calloc(s->NTB, sizeof(double)); s->band_max = calloc(s->NTB, sizeof(double));
    s->band_min = calloc(s->NTB, sizeof(double));
    s->prob = calloc((long)s->NTB * s->NTK, sizeof(cplx));
    judge(s, 0, 0, 0);
    /* band-cRPA probabilities (:869-906) */
    if (P->flg_crpa == 1) {
        char path[4096]; ldr r;
        snprintf(path, sizeof path, "%s/dir-wan/dat.ns-nb", root);
        if (ld_open(&r, path)) return 1;
        int *Ns = calloc(s->NTK, sizeof(int)), *Nb = calloc(s->NTK, sizeof(int));
        int Mb = 0;
        for (int ik = 0; ik < s->NTK; ik++) {
            int t[2];
            if (ld_int(&r, 2, t)) { ld_close(&r); free(Ns); free(Nb); return 1; }
            Ns[ik] = t[0]; Nb[ik] = t[1]; if (t[1] > Mb) Mb = t[1];
        }
        ld_close(&r);
        snprintf(path, sizeof path, "%s/dir-wan/dat.umat", root);
        if (ld_open(&r, path)) { free(Ns); free(Nb); return 1; }
        int NWF;
        if (ld_int(&r, 1, &NWF)) { ld_close(&r); free(Ns); free(Nb); return 1; }
        double *row = malloc(sizeof(double) * 2 * NWF);
        for (int ik = 0; ik < s->NTK; ik++)
            for (int jb = 0; jb < Nb[ik]; jb++) {
                if (ld_read(&r, 2 * NWF, row)) { ld_close(&r); free(Ns); free(Nb); free(row); return 1; }
                cplx sum = 0;
                for (int iw = 0; iw < NWF; iw++) {
                    cplx u = row[2 * iw] + I * row[2 * iw + 1];
                    sum += conj(u) * u;
                }
                int band = Ns[ik] + jb;
                if (band < 0 || band >= s->NTB) { ld_close(&r); free(Ns); free(Nb); free(row); return fail("dat.ns-nb band out of range"); }
                s->prob[(long)ik * s->NTB + band] = sum;
            }
        ld_close(&r); free(Ns); free(Nb); free(row);
    }
    /* occupied / virtual counts (:943-967) */
    s->N_docc = s->N_pocc = s->N_uocc = 0;
    for (int ib = 0; ib < s->NCB; ib++) {
        if (s->WindowInside[ib] == 0) s->N_docc++;
        if (s->WindowInside[ib] == 1) s->N_pocc++;
        if (s->WindowInside[ib] == 2) s->N_uocc++;
    }
    s->N_occ = s->N_docc + s->N_pocc;
    s->N_vir = s->N_uocc + s->N_pocc;
    /* wave functions (:1100-1160): keep bands 1..N_CALC_BAND of every k */
    {
        char path[4096];
        snprintf(path, sizeof path, "%s/dir-wfn/dat.wfn", root);
        FILE *f = fopen(path, "rb");
        if (!f) return fail("cannot open %s", path);
        int ncomp; size_t got;
        if (fu_read_record(f, &ncomp, 4, &got)) { fclose(f); return 1; }
        if (ncomp != 1) { fclose(f); return fail("This program not suport ncomp/=1"); }
        s->C = calloc((long)s->Nk_irr * s->NCB * s->NTG, sizeof(cplx));
        for (int ik = 0; ik < s->Nk_irr; ik++)
            for (int ib = 0; ib < s->NTB; ib++) {
                if (ib < s->NCB) {
                    if (fu_read_record(f, s->C + ((long)ik * s->NCB + ib) * s->NTG, sizeof(cplx) * s->NGI[ik], &got)) { fclose(f); return 1; }
                } else if (fu_read_record(f, NULL, 0, &got)) { fclose(f); return 1; }
            }
        fclose(f);
    }
    /* frequency grid (:1184-1192) */
    double bmax = -1e300, bmin = 1e300;
    for (int ib = 0; ib < s->NCB; ib++) { if (s->band_max[ib] > bmax) bmax = s->band_max[ib]; if (s->band_min[ib] < bmin) bmin = s->band_min[ib]; }
    double emax = fabs(bmax - bmin);
    if (P->nen_explicit > 0) {
        s->nen = P->nen_explicit;
        s->em = malloc(sizeof(cplx) * s->nen);
        for (int i = 0; i < s->nen; i++) s->em[i] = P->em_explicit[2 * i] + I * P->em_explicit[2 * i + 1];
    } else {
        s->nen = P->num_freq_grid;
        s->em = malloc(sizeof(cplx) * s->nen);
        orc_gen_grid(s->nen, emax, (double *)s->em);
    }
    s->imt1 = malloc(sizeof(int) * 4 * 6 * (long)s->NTK);
    orc_ttrhdrn_mkidx(s->nkb[0], s->nkb[1], s->nkb[2], s->b1, s->b2, s->b3, s->imt1);
    s->delt = P->green_func_delt / AU;
    s->delta_ex = P->max_excitation_energy / AU;
    s->dmna = P->ttrhdrn_dmna;
    s->dmnr = P->ttrhdrn_dmnr;
    return 0;
}

void orc_default_params(orc_params *p) {
    memset(p, 0, sizeof *p);
    p->n_calc_band = 0; p->ecut_for_eps = 0.0; p->shift_ef = 0.0; p->max_excitation_energy = 200.0;
    p->green_func_delt = 0.1; p->ttrhdrn_dmna = 0.001; p->ttrhdrn_dmnr = 0.001; p->num_freq_grid = 70;
    p->flg_crpa = 0; p->flg_calc_type = 0; p->file_num_log_start = 400; p->file_num_eps_start = 600;
    p->file_num_eps_base_start = 600000; p->write_eps = 1;
}

/* per-thread work buffers */
typedef struct {
    cplx *wk, *wkq, *m_tmp, *ism, *C0K, *C0KQ, *xow; double *e1, *e2;
    cplx *pc; /* accumulator NG*NG*nen*ndir */
} tbuf;

static int pair_loop(const orc_state *s, const double *q, const int *LG0, int NG, int gamma, int No_G_0,
                     const int *ipair, const int *jpair, int npair, const int *kpq, const int *sG, cplx *chi,
                     int nthreads, int nk_use) {
    int ndir = gamma ? 3 : 1;
    int nen = s->nen, NTK = s->NTK;
    long chisz = (long)NG * NG * nen * ndir;
    int err = 0;
    int nt = nthreads > 0 ? nthreads : 1;
#ifdef _OPENMP
    if (nthreads <= 0) nt = omp_get_max_threads();
#endif
    if (nt > npair && npair > 0) nt = npair;
    if (nt < 1) nt = 1;
    cplx **acc = calloc(nt, sizeof(cplx *));
#pragma omp parallel num_threads(nt)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        long N = (long)s->nw[0] * s->nw[1] * s->nw[2];
        tbuf b;
        b.wk = malloc(sizeof(cplx) * N); b.wkq = malloc(sizeof(cplx) * N);
        b.m_tmp = malloc(sizeof(cplx) * NG); b.ism = malloc(sizeof(cplx) * (long)NTK * NG * ndir);
        b.C0K = malloc(sizeof(cplx) * s->NTG); b.C0KQ = malloc(sizeof(cplx) * s->NTG);
        b.xow = malloc(sizeof(cplx) * (long)NTK * nen);
        b.e1 = malloc(sizeof(double) * NTK); b.e2 = malloc(sizeof(double) * NTK);
        b.pc = calloc(chisz, sizeof(cplx));
        acc[tid] = b.pc;
        cplx *xo1 = malloc(sizeof(cplx) * (long)NTK * nen);
        /* static contiguous blocks of pairs: deterministic for a given thread count */
        int lo = (int)((long)npair * tid / nt), hi = (int)((long)npair * (tid + 1) / nt);
        for (int ij = lo; ij < hi && !err; ij++) {
            int ib = ipair[ij], jb = jpair[ij];          /* 0-based vir / occ index */
            int bandv = s->N_docc + ib, bando = jb;      /* absolute band (0-based) */
            for (int ik = 0; ik < nk_use; ik++) {
                int ikq = kpq[ik];
                make_C0(s, ik, bando, b.C0K);
                make_C0(s, ikq, bandv, b.C0KQ);
                interstate(s, ik, ikq, b.C0K, b.C0KQ, LG0, NG, sG + 3 * ik, b.wk, b.wkq, b.m_tmp);
                if (!gamma) {
                    for (int g = 0; g < NG; g++) b.ism[(long)g * NTK + ik] = b.m_tmp[g];
                } else {
                    cplx vm[3];
                    calc_vm(s, ik, b.C0K, b.C0KQ, NULL, vm);
                    double del = s->E_EIGI[(long)s->numirr[ikq] * s->NTB + bandv] - s->E_EIGI[(long)s->numirr[ik] * s->NTB + bando];
                    if (fabs(del) < s->delt) del = s->delt;
                    for (int d = 0; d < 3; d++) vm[d] = -I * (vm[d] - 0.0) / del;
                    for (int ix = 0; ix < 3; ix++) {
                        b.m_tmp[No_G_0] = vm[ix];
                        if (fabs(del) <= s->delt) b.m_tmp[No_G_0] = 0;
                        for (int g = 0; g < NG; g++) b.ism[((long)ix * NG + g) * NTK + ik] = b.m_tmp[g];
                    }
                }
            }
            /* energies on the mesh (float rounding of cmplx(), chiqw.F:1354/1357, 1813/1814) */
            for (int ik = 0; ik < NTK; ik++) {
                b.e1[ik] = SGL(s->E_EIGI[(long)s->numirr[ik] * s->NTB + bando]);
                b.e2[ik] = SGL(s->E_EIGI[(long)s->numirr[kpq[ik]] * s->NTB + bandv]);
            }
            double *e1m = malloc(sizeof(double) * NTK), *e2m = malloc(sizeof(double) * NTK);
            for (int m = 0; m < NTK; m++) { e1m[m] = b.e1[s->index_kpt[m]]; e2m[m] = b.e2[s->index_kpt[m]]; }
            memset(xo1, 0, sizeof(cplx) * (long)NTK * nen);
            if (ttrhdrn_chi0(s->dmna, s->dmnr, NTK, s->imt1, e1m, e2m, s->FermiEnergy, s->FermiEnergy, s->delt, 1.0, nen, s->em, xo1) ||
                ttrhdrn_chi0(s->dmna, s->dmnr, NTK, s->imt1, e1m, e2m, s->FermiEnergy, s->FermiEnergy, s->delt, -1.0, nen, s->em, xo1)) {
#pragma omp atomic write
                err = 1;
            }
            free(e1m); free(e2m);
            /* xow_1D(ik, ie) */
            for (int m = 0; m < NTK; m++) {
                int ik = s->index_kpt[m];
                for (int e = 0; e < nen; e++) b.xow[(long)e * NTK + ik] = xo1[(long)m * nen + e];
            }
            /* contraction (chiqw.F:1397-1410 / 1862-1875) */
            for (int ix = 0; ix < ndir; ix++)
                for (int e = 0; e < nen; e++)
                    for (int jg = 0; jg < NG; jg++)
                        for (int ig = 0; ig < NG; ig++) {
                            const cplx *ri = b.ism + ((long)ix * NG + ig) * NTK, *rj = b.ism + ((long)ix * NG + jg) * NTK;
                            const cplx *xw = b.xow + (long)e * NTK;
                            cplx sacc = b.pc[((long)ix * nen + e) * NG * NG + ig + (long)NG * jg];
                            for (int ik = 0; ik < nk_use; ik++) {
                                int ikq = kpq[ik];
                                cplx pp = 1.0 - s->prob[(long)ik * s->NTB + bando] * s->prob[(long)ikq * s->NTB + bandv];
                                sacc = sacc + xw[ik] * conj(ri[ik]) * rj[ik] / (double)NTK * pp;
                            }
                            b.pc[((long)ix * nen + e) * NG * NG + ig + (long)NG * jg] = sacc;
                        }
        }
        free(b.wk); free(b.wkq); free(b.m_tmp); free(b.ism); free(b.C0K); free(b.C0KQ); free(b.xow); free(b.e1); free(b.e2);
        free(xo1);
    }
    for (long i = 0; i < chisz; i++) chi[i] = 0;
    for (int t = 0; t < nt; t++) {
        if (!acc[t]) continue;
        for (long i = 0; i < chisz; i++) chi[i] += acc[t][i];
        free(acc[t]);
    }
    free(acc);
    return err ? fail("tetrahedron failure: %s", g_err) : 0;
}

int orc_calc_chiqw(const char *root, const orc_params *P, orc_report *rep) {
    orc_state S; memset(&S, 0, sizeof S);
    orc_state *s = &S;
    double t0 = now_s();
    if (rep) memset(rep, 0, sizeof *rep);
    if (setup(s, root, P)) { free_state(s); return 1; }
    char epsdir[4096], path[4096];
    snprintf(epsdir, sizeof epsdir, "%s/dir-eps", root);
    if (mkdir_p(epsdir)) { free_state(s); return 1; }
    for (int ik = 0; ik < s->Nk_irr; ik++) {
        snprintf(path, sizeof path, "%s/q%03d", epsdir, ik + 1);
        if (mkdir_p(path)) { free_state(s); return 1; }
    }
    /* q list (chiqw.F:587-655) */
    int *qlist = calloc(s->Nk_irr + (P->n_calc_q > 0 ? P->n_calc_q : 0), sizeof(int));
    int nq = 0;
    struct stat st;
    if (P->flg_calc_type == 0) {
        for (int ik = 0; ik < s->Nk_irr; ik++) {
            snprintf(path, sizeof path, "%s/q%03d/dat.log.%03d", epsdir, ik + 1, P->file_num_log_start);
            if (stat(path, &st) == 0) continue;
            qlist[nq++] = ik;
        }
    } else if (P->flg_calc_type == 1) {
        int ix = -1;
        for (int ik = 0; ik < s->Nk_irr; ik++)
            if (fabs(s->SKI[3 * ik]) < 1e-5 && fabs(s->SKI[3 * ik + 1]) < 1e-5 && fabs(s->SKI[3 * ik + 2]) < 1e-5) ix = ik;
        if (ix < 0) { free(qlist); free_state(s); return fail("no Gamma point in dat.sample-k"); }
        snprintf(path, sizeof path, "%s/q%03d/dat.log.%03d", epsdir, ix + 1, P->file_num_log_start);
        if (stat(path, &st) != 0) qlist[nq++] = ix;
    } else if (P->flg_calc_type == 2) {
        if (P->n_calc_q <= 0) { free(qlist); free_state(s); return fail("n_calc_q should not be zero"); }
        for (int i = 0; i < P->n_calc_q; i++) {
            int ik = P->calc_num_k[i] - 1;
            if (ik < 0 || ik >= s->Nk_irr) { free(qlist); free_state(s); return fail("calc_num_k out of range"); }
            snprintf(path, sizeof path, "%s/q%03d/dat.log.%03d", epsdir, ik + 1, P->file_num_log_start);
            if (stat(path, &st) == 0) continue;
            qlist[nq++] = ik;
        }
    }
    /* dat.chi_cutoff, dat.wgrid (:1203-1218) */
    if (P->write_eps) {
        snprintf(path, sizeof path, "%s/dat.chi_cutoff", epsdir);
        FILE *f = fopen(path, "w"); if (f) { fprintf(f, " %24.16E\n", s->Ecut_eps); fclose(f); }
        snprintf(path, sizeof path, "%s/dat.wgrid", epsdir);
        f = fopen(path, "w");
        if (f) {
            fprintf(f, " %11d\n", s->nen);
            for (int e = 0; e < s->nen; e++) fprintf(f, "%15.10f%15.10f\n", creal(s->em[e]), cimag(s->em[e]));
            fclose(f);
        }
    }
    int *LG0 = malloc(sizeof(int) * 3 * s->NTG);
    int *kpq = malloc(sizeof(int) * s->NTK), *sG = malloc(sizeof(int) * 3 * s->NTK);
    int *ip = malloc(sizeof(int) * (long)s->NCB * s->NCB), *jp = malloc(sizeof(int) * (long)s->NCB * s->NCB);
    int rc = 0;
    int nq_run = nq;
    if (P->max_q > 0 && nq_run > P->max_q) nq_run = P->max_q;
    for (int iq = 0; iq < nq_run && !rc; iq++) {
        double tq = now_s();
        double q[3];
        search_list(s->SKI + 3 * qlist[iq], q);
        int NG;
        if (make_KG0(s->NTG, s->b1, s->b2, s->b3, s->Ecut_eps, q[0], q[1], q[2], LG0, &NG)) { rc = 1; break; }
        int gamma = (q[0] == 0.0 && q[1] == 0.0 && q[2] == 0.0);
        int No_G_0 = -1;
        if (gamma)
            for (int g = 0; g < NG; g++) if (LG0[3 * g] == 0 && LG0[3 * g + 1] == 0 && LG0[3 * g + 2] == 0) No_G_0 = g;
        if (gamma && No_G_0 < 0) { rc = fail("G=0 not in the dielectric sphere"); break; }
        for (int ik = 0; ik < s->NTK; ik++) {
            sG[3 * ik] = sG[3 * ik + 1] = sG[3 * ik + 2] = 0;
            if (gamma) kpq[ik] = ik;
            else { kpq[ik] = -1; search_kq(s->NTK, s->SK0, q, ik, kpq + ik, sG + 3 * ik); }
            if (kpq[ik] < 0) { rc = fail("k+q not found on the mesh"); break; }
        }
        if (rc) break;
        /* pair lists (:1270-1294, :1589-1629) */
        int np = 0, nintra = 0;
        int *ii = malloc(sizeof(int) * (long)s->NCB * s->NCB), *jj = malloc(sizeof(int) * (long)s->NCB * s->NCB);
        for (int jb = 0; jb < s->N_occ; jb++)
            for (int ib = 0; ib < s->N_vir; ib++) {
                int bv = s->N_docc + ib, bo = jb;
                if (fabs(s->E_AVE[bv] - s->E_AVE[bo]) >= s->delta_ex) continue;
                if (gamma && s->Tindx[bv] == s->Tindx[bo] && s->Tindx[bv] != 0) {
                    ii[nintra] = ib; jj[nintra] = jb; nintra++;
                    continue;
                }
                ip[np] = ib; jp[np] = jb; np++;
            }
        if (P->flg_crpa == 1) nintra = 0;
        int npair_full = np;
        if (P->max_pairs > 0 && np > P->max_pairs) np = P->max_pairs;
        int ndir = gamma ? 3 : 1;
        long chisz = (long)NG * NG * s->nen * ndir;
        cplx *chi = malloc(sizeof(cplx) * chisz);
        const int nk_use = (P->max_k > 0 && P->max_k < s->NTK) ? P->max_k : s->NTK;
        rc = pair_loop(s, q, LG0, NG, gamma, No_G_0, ip, jp, np, kpq, sG, chi, P->nthreads, nk_use);
        /* intraband plasma frequency at Gamma (:1639-1733, :1989-1994) */
        double wd[3] = {0, 0, 0};
        if (!rc && gamma && nintra > 0) {
            cplx pwpl[3] = {0, 0, 0};
            cplx *C0K = malloc(sizeof(cplx) * s->NTG), *C0KQ = malloc(sizeof(cplx) * s->NTG);
            cplx *pk = malloc(sizeof(cplx) * 3 * s->NTK), *fk = malloc(sizeof(cplx) * s->NTK), *gk = malloc(sizeof(cplx) * s->NTK);
            cplx *xo = malloc(sizeof(cplx) * s->NTK);
            for (int t = 0; t < nintra && !rc; t++) {
                int bv = s->N_docc + ii[t], bo = jj[t];
                cplx pk1[3];
                for (int ik = 0; ik < s->NTK; ik++) {
                    make_C0(s, ik, bo, C0K);
                    make_C0(s, ik, bv, C0KQ);
                    calc_vm(s, ik, C0K, C0KQ, s->SK0 + 3 * ik, pk1);
                    int m = -1;
                    (void)m;
                    for (int d = 0; d < 3; d++) pk[3 * ik + d] = -I * (pk1[d] - 0.0);
                    fk[ik] = 1.0;
                    gk[ik] = SGLC(s->E_EIGI[(long)s->numirr[ik] * s->NTB + bo] - s->FermiEnergy, -s->delt);
                }
                /* to the 3D mesh */
                cplx *fk3 = malloc(sizeof(cplx) * s->NTK), *gk3 = malloc(sizeof(cplx) * s->NTK);
                for (int m = 0; m < s->NTK; m++) { fk3[m] = fk[s->index_kpt[m]]; gk3[m] = gk[s->index_kpt[m]]; xo[m] = 0; }
                if (orc_ttrhdrn_simple(s->dmna, s->dmnr, s->nkb[0], s->nkb[1], s->nkb[2], s->imt1, (double *)fk3, (double *)gk3, (double *)xo)) rc = 1;
                for (int m = 0; m < s->NTK; m++) {
                    int ik = s->index_kpt[m];
                    for (int d = 0; d < 3; d++) pwpl[d] = pwpl[d] + cimag(xo[m]) * pk[3 * ik + d] * pk[3 * ik + d];
                }
                free(fk3); free(gk3);
            }
            for (int d = 0; d < 3; d++) {
                cplx wpl = 8.0 * pwpl[d] / s->VOLUME / (double)s->NTK;
                wd[d] = sqrt(creal(wpl));
            }
            free(C0K); free(C0KQ); free(pk); free(fk); free(gk); free(xo);
        }
        free(ii); free(jj);
        if (rc) { free(chi); break; }
        for (long i = 0; i < chisz; i++) chi[i] = chi[i] / s->VOLUME;
        /* output (:1475-1553, :1988-2081) */
        int qnum = -1;
        for (int ik = 0; ik < s->Nk_irr; ik++)
            if (fabs(s->SKI_list[3 * ik] - q[0]) < 1e-6 && fabs(s->SKI_list[3 * ik + 1] - q[1]) < 1e-6 &&
                fabs(s->SKI_list[3 * ik + 2] - q[2]) < 1e-6) qnum = ik + 1;
        char qdir[4096];
        snprintf(qdir, sizeof qdir, "%s/q%03d", epsdir, qnum);
        if (P->dump_chi) {
            snprintf(path, sizeof path, "%s/dat.chi0", qdir);
            FILE *f = fopen(path, "wb");
            if (f) {
                int32_t hdr[4] = {NG, s->nen, ndir, np};
                fwrite(hdr, 4, 4, f);
                fwrite(chi, sizeof(cplx), chisz, f);
                fclose(f);
            }
        }
        if (P->write_eps) {
            snprintf(path, sizeof path, "%s/dat.sq", qdir);
            FILE *f = fopen(path, "w");
            if (f) { fprintf(f, " %24.16E %24.16E %24.16E\n", q[0], q[1], q[2]); fclose(f); }
            cplx *work = malloc(sizeof(cplx) * (long)NG * NG);
            cplx *epsall = malloc(sizeof(cplx) * chisz);
            for (int ix = 0; ix < ndir && !rc; ix++) {
                int base = P->file_num_eps_base_start + ix * 1000;
                for (int e = 0; e < s->nen && !rc; e++) {
                    snprintf(path, sizeof path, "%s/dat.epsqw.%06d", qdir, base + e + 1);
                    FILE *ft = fopen(path, "w");
                    if (ft) fprintf(ft, "#epsqw diagonal term\n#1:q+G [au], 2:Re(eps-1), 3:Im(eps-1)\n");
                    memcpy(work, chi + ((long)ix * s->nen + e) * NG * NG, sizeof(cplx) * (long)NG * NG);
                    rc = eps_rpa(s, q, LG0, NG, work, gamma, No_G_0, wd[ix], s->delt, s->em[e], ft);
                    if (ft) fclose(ft);
                    memcpy(epsall + ((long)ix * s->nen + e) * NG * NG, work, sizeof(cplx) * (long)NG * NG);
                }
                snprintf(path, sizeof path, "%s/dat.epsqw.%03d", qdir, P->file_num_eps_start + ix);
                FILE *fb = fopen(path, "wb");
                if (fb) { fu_write_record(fb, epsall + (long)ix * s->nen * NG * NG, sizeof(cplx) * (long)s->nen * NG * NG); fclose(fb); }
            }
            free(work); free(epsall);
            snprintf(path, sizeof path, "%s/dat.log.%03d", qdir, P->file_num_log_start);
            f = fopen(path, "w");
            if (f && !rc) { fprintf(f, " #\n #finish chi0 evaluation for %11d\n #\n", qnum); }
            if (f) fclose(f);
        }
        free(chi);
        if (rep) {
            rep->nq_done++; rep->ntk = s->NTK; rep->ng_last = NG; rep->npair_last = np; rep->npair_full_last = npair_full;
            rep->nen = s->nen; rep->fft_box[0] = s->nw[0]; rep->fft_box[1] = s->nw[1]; rep->fft_box[2] = s->nw[2];
            rep->seconds_last_q = now_s() - tq;
            rep->nk_used_last = nk_use;
        }
    }
    free(LG0); free(kpq); free(sG); free(ip); free(jp); free(qlist);
    free_state(s);
    if (rep) rep->seconds_total = now_s() - t0;
    return rc;
}

const char *orc_last_error(void) { return g_err; }

/* calc_int (V, W, X, J): shares the readers, unfold, FFT and pair density above */
#include "rp_oracle_int.c"
