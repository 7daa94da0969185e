/*
 * rp_oracle_int.c -- CPU restatement (FP64) of RESPACK's calc_int programs:
 * calc_w3d (bare V and screened W, src/calc_int/calc_intW.F) and calc_j3d
 * (bare X and screened J exchange, src/calc_int/calc_intJ.F), with
 * src/calc_int/calc_int_sub.F (make_LG0, make_eps, search_kq,
 * calc_InterStateMatrix) and the mvmc writers (wrt_mvmc_w3d.f90,
 * wrt_mvmc_j3d.f90).
 *
 * TEST INFRASTRUCTURE ONLY (the checker), like rp_oracle.c, which includes
 * this file so that it shares the dir-wfn readers, the Brillouin-zone unfold,
 * the FFT and the pair-density routine.  Parity unpinned by the reference.
 */

void orc_int_default_params(orc_int_params *p) {
    memset(p, 0, sizeof *p);
    /* m_rdinput.f90 (calc_int):20-29 */
    p->calc_ifreq = 1;
    p->wcut_mvmc = 2.0;
    p->jcut_mvmc = 0.3;
    p->write_files = 1;
    p->do_w = 1;
    p->do_j = 1;
}

typedef struct {
    int NWF, ne, NTQ, Nq_irr, NTGQ, iqgm, NoG0, Lq[3];
    cplx *C0;                 /* [(k*NWF + w)*NTG + ig] */
    double *coord;            /* [w*3 + d] */
    double Ecut_eps;
    cplx *em;
    double *SQI, *SQ;         /* [iq*3 + d] */
    int *numirrq, *numrotq, *trsq, *RWq;
    int *LG0;                 /* [(iq*NTG2 + ig)*3 + d], NTG2 = room per q */
    int NTG2;
    int *NGQ_eps, *NGQ_psi;
    int *packingq;            /* [iq][i+Lq1][j+Lq2][k+Lq3] (irreducible q), 1-based */
    float complex *epsirr;    /* [((iq*ne + e)*NTGQ + jg)*NTGQ + ig] */
} int_state;

static void free_int(int_state *t) {
    free(t->C0); free(t->coord); free(t->em); free(t->SQI); free(t->SQ); free(t->numirrq); free(t->numrotq);
    free(t->trsq); free(t->RWq); free(t->LG0); free(t->NGQ_eps); free(t->NGQ_psi); free(t->packingq); free(t->epsirr);
}

/* make_LG0 (calc_int_sub.F:447-504): the eps sphere, then the shell up to the psi cutoff */
static int make_LG0(int cap, const double *b1, const double *b2, const double *b3, double Ge, double Gp,
                    const double *q, int *LG, int *nge, int *ngp) {
    const int N = 100;
    int n = 0;
    for (int pass = 0; pass < 2; pass++) {
        for (int i1 = -N; i1 <= N; i1++)
            for (int i2 = -N; i2 <= N; i2++)
                for (int i3 = -N; i3 <= N; i3++) {
                    double v[3];
                    for (int d = 0; d < 3; d++)
                        v[d] = (q[0] + i1) * b1[d] + (q[1] + i2) * b2[d] + (q[2] + i3) * b3[d];
                    double l = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
                    int take = pass == 0 ? (l <= Ge) : (l > Ge && l <= Gp);
                    if (!take) continue;
                    if (n >= cap) return fail("make_LG0: more than %d G vectors", cap);
                    LG[3 * n] = i1; LG[3 * n + 1] = i2; LG[3 * n + 2] = i3;
                    n++;
                }
        if (pass == 0) *nge = n;
    }
    *ngp = n;
    return 0;
}

/* '(2f15.10)' fixed-width pair */
static int read_2f15(const char *line, double *a, double *b) {
    char buf[16];
    size_t L = strlen(line);
    if (L < 30) {
        return sscanf(line, "%lf %lf", a, b) == 2 ? 0 : fail("bad (2f15.10) record: %s", line);
    }
    memcpy(buf, line, 15); buf[15] = 0; *a = atof(buf);
    memcpy(buf, line + 15, 15); buf[15] = 0; *b = atof(buf);
    return 0;
}

static int int_read(orc_state *s, int_state *t, const char *root, const orc_int_params *P) {
    char path[4096];
    /* dat.wan (calc_intW.F:339-348) */
    snprintf(path, sizeof path, "%s/dir-wan/dat.wan", root);
    FILE *f = fopen(path, "rb");
    if (!f) return fail("cannot open %s", path);
    size_t got;
    if (fu_read_record(f, &t->NWF, 4, &got)) { fclose(f); return 1; }
    if (t->NWF <= 0) { fclose(f); return fail("dat.wan: NWF = %d", t->NWF); }
    t->C0 = calloc((long)s->NTK * t->NWF * s->NTG, sizeof(cplx));
    cplx *rec = malloc(sizeof(cplx) * (long)s->NTG * t->NWF);
    for (int k = 0; k < s->NTK; k++) {
        long want = (long)s->NG0[k] * t->NWF;
        if (fu_read_record(f, rec, sizeof(cplx) * want, &got)) { fclose(f); free(rec); return 1; }
        if (got != sizeof(cplx) * want) { fclose(f); free(rec); return fail("dat.wan record %d: %zu bytes, expected %ld", k + 1, got, (long)(sizeof(cplx) * want)); }
        for (int w = 0; w < t->NWF; w++)
            for (int ig = 0; ig < s->NG0[k]; ig++)
                t->C0[((long)k * t->NWF + w) * s->NTG + ig] = rec[(long)w * s->NG0[k] + ig];
    }
    free(rec);
    fclose(f);
    /* dat.wan-center (:362-370) */
    snprintf(path, sizeof path, "%s/dir-wan/dat.wan-center", root);
    ldr r;
    if (ld_open(&r, path)) return 1;
    if (getline(&r.line, &r.cap, r.f) < 0 || getline(&r.line, &r.cap, r.f) < 0) { ld_close(&r); return fail("dat.wan-center: header"); }
    t->coord = calloc(3 * t->NWF, sizeof(double));
    for (int w = 0; w < t->NWF; w++)
        if (ld_read(&r, 3, t->coord + 3 * w)) { ld_close(&r); return 1; }
    ld_close(&r);
    /* dat.chi_cutoff, dat.wgrid (:398-411) */
    snprintf(path, sizeof path, "%s/dir-eps/dat.chi_cutoff", root);
    if (ld_open(&r, path) || ld_read(&r, 1, &t->Ecut_eps)) { ld_close(&r); return 1; }
    ld_close(&r);
    snprintf(path, sizeof path, "%s/dir-eps/dat.wgrid", root);
    if (ld_open(&r, path) || ld_int(&r, 1, &t->ne)) { ld_close(&r); return 1; }
    t->em = calloc(t->ne, sizeof(cplx));
    for (int e = 0; e < t->ne; e++) {
        double a, b;
        if (getline(&r.line, &r.cap, r.f) < 0) { ld_close(&r); return fail("dat.wgrid: %d of %d frequencies", e, t->ne); }
        if (read_2f15(r.line, &a, &b)) { ld_close(&r); return 1; }
        t->em[e] = a + I * b;
    }
    ld_close(&r);
    if (P->calc_ifreq < 1 || P->calc_ifreq > t->ne) return fail("calc_ifreq = %d outside 1..%d", P->calc_ifreq, t->ne);
    /* dat.sq of every irreducible q (:413-439) */
    t->Nq_irr = s->Nk_irr;
    t->SQI = calloc(3 * t->Nq_irr, sizeof(double));
    for (int iq = 0; iq < t->Nq_irr; iq++) {
        snprintf(path, sizeof path, "%s/dir-eps/q%03d/dat.sq", root, iq + 1);
        if (ld_open(&r, path) || ld_read(&r, 3, t->SQI + 3 * iq)) { ld_close(&r); return 1; }
        ld_close(&r);
    }
    return 0;
}

/* full q mesh (calc_intW.F:441-510): the irreducible q first, then their new images */
static int int_unfold_q(orc_state *s, int_state *t) {
    int cap = t->Nq_irr * (1 + 2 * s->nsymq);
    t->SQ = calloc(3 * cap, sizeof(double));
    t->numirrq = calloc(cap, sizeof(int)); t->numrotq = calloc(cap, sizeof(int));
    t->trsq = calloc(cap, sizeof(int)); t->RWq = calloc(3 * cap, sizeof(int));
    for (int iq = 0; iq < t->Nq_irr; iq++) {
        for (int d = 0; d < 3; d++) t->SQ[3 * iq + d] = t->SQI[3 * iq + d];
        t->numirrq[iq] = iq; t->numrotq[iq] = 0; t->trsq[iq] = 1;
    }
    int jk = t->Nq_irr;
    for (int iq = 0; iq < t->Nq_irr; iq++)
        for (int iop = 0; iop < s->nsymq; iop++) {
            const int *R = s->rg + 9 * iop;
            const double *k = t->SQI + 3 * iq;
            for (int pass = 0; pass < 2; pass++) {
                double kt[3]; int RWt[3] = {0, 0, 0};
                for (int i = 0; i < 3; i++)
                    kt[i] = (double)R[i] * k[0] + (double)R[i + 3] * k[1] + (double)R[i + 6] * k[2];
                if (pass == 0) kcheck(kt, RWt); else kcheck_trs(kt, RWt);
                double sg = pass == 0 ? 1.0 : -1.0;
                int dup = 0;
                for (int i = 0; i < jk; i++)
                    if (fabs(t->SQ[3 * i] - sg * kt[0]) < 1e-4 && fabs(t->SQ[3 * i + 1] - sg * kt[1]) < 1e-4 &&
                        fabs(t->SQ[3 * i + 2] - sg * kt[2]) < 1e-4) { dup = 1; break; }
                if (dup) continue;
                for (int i = 0; i < 3; i++) { t->SQ[3 * jk + i] = sg * kt[i]; t->RWq[3 * jk + i] = RWt[i]; }
                t->numirrq[jk] = iq; t->numrotq[jk] = iop; t->trsq[jk] = pass == 0 ? 1 : -1;
                jk++;
            }
        }
    t->NTQ = jk;
    if (t->NTQ != s->NTK) return fail("NTQ should be NTK (NTQ=%d, NTK=%d)", t->NTQ, s->NTK);
    /* LG0 per full q (:514-582) */
    t->NTG2 = 2 * s->NTG + 64;
    t->LG0 = calloc((long)3 * t->NTG2 * t->NTQ, sizeof(int));
    t->NGQ_eps = calloc(t->NTQ, sizeof(int)); t->NGQ_psi = calloc(t->NTQ, sizeof(int));
    for (int iq = 0; iq < t->NTQ; iq++) {
        double q[3];
        int *dst = t->LG0 + (long)3 * t->NTG2 * iq;
        if (iq < t->Nq_irr) {
            for (int d = 0; d < 3; d++) q[d] = t->SQI[3 * iq + d];
        } else {
            const int *R = s->rg + 9 * t->numrotq[iq];
            const double *k = t->SQI + 3 * t->numirrq[iq];
            for (int i = 0; i < 3; i++)
                q[i] = (double)R[i] * k[0] + (double)R[i + 3] * k[1] + (double)R[i + 6] * k[2] + (double)t->RWq[3 * iq + i];
        }
        if (make_LG0(t->NTG2, s->b1, s->b2, s->b3, t->Ecut_eps, s->Ecut_psi, q, dst, t->NGQ_eps + iq, t->NGQ_psi + iq))
            return 1;
        if (iq >= t->Nq_irr && t->trsq[iq] == -1)
            for (int i = 0; i < 3 * t->NGQ_psi[iq]; i++) dst[i] = -dst[i];
    }
    for (int d = 0; d < 3; d++) t->Lq[d] = 0;
    for (int iq = 0; iq < t->NTQ; iq++)
        for (int ig = 0; ig < t->NTG2; ig++)
            for (int d = 0; d < 3; d++) {
                int v = abs(t->LG0[((long)t->NTG2 * iq + ig) * 3 + d]);
                if (v > t->Lq[d]) t->Lq[d] = v;
            }
    for (int d = 0; d < 3; d++) t->Lq[d]++;
    int n1 = 2 * t->Lq[0] + 1, n2 = 2 * t->Lq[1] + 1, n3 = 2 * t->Lq[2] + 1;
    t->packingq = calloc((long)n1 * n2 * n3 * t->Nq_irr, sizeof(int));
    t->NTGQ = 0;
    for (int iq = 0; iq < t->Nq_irr; iq++)
        for (int ig = 0; ig < t->NGQ_eps[iq]; ig++) {
            const int *g = t->LG0 + ((long)t->NTG2 * iq + ig) * 3;
            t->packingq[(long)iq * n1 * n2 * n3 + (g[0] + t->Lq[0]) + n1 * ((g[1] + t->Lq[1]) + (long)n2 * (g[2] + t->Lq[2]))] = ig + 1;
        }
    for (int iq = 0; iq < t->NTQ; iq++) if (t->NGQ_eps[iq] > t->NTGQ) t->NTGQ = t->NGQ_eps[iq];
    return 0;
}

/* eps^-1 of the irreducible q as complex(4); Gamma: mean of the three directions (:587-630) */
static int int_read_eps(orc_state *s, int_state *t, const char *root) {
    long nn = (long)t->NTGQ * t->NTGQ;
    t->epsirr = calloc(nn * t->ne * t->Nq_irr, sizeof(float complex));
    t->iqgm = -1;
    for (int iq = 0; iq < t->Nq_irr; iq++) {
        const double *k = s->SKI + 3 * iq;
        int gm = fabs(k[0]) < 1e-5 && fabs(k[1]) < 1e-5 && fabs(k[2]) < 1e-5;
        int NG = t->NGQ_eps[iq], nf = gm ? 3 : 1;
        if (gm) t->iqgm = iq;
        cplx *acc = calloc((long)NG * NG * t->ne, sizeof(cplx));
        cplx *buf = malloc(sizeof(cplx) * (long)NG * NG * t->ne);
        for (int ix = 0; ix < nf; ix++) {
            char path[4096];
            snprintf(path, sizeof path, "%s/dir-eps/q%03d/dat.epsqw.%03d", root, iq + 1, 600 + ix);
            FILE *f = fopen(path, "rb");
            size_t got;
            if (!f) { free(acc); free(buf); return fail("cannot open %s", path); }
            int rc = fu_read_record(f, buf, sizeof(cplx) * (long)NG * NG * t->ne, &got);
            fclose(f);
            if (rc) { free(acc); free(buf); return 1; }
            if (got != sizeof(cplx) * (size_t)NG * NG * t->ne) { free(acc); free(buf); return fail("%s: %zu bytes", path, got); }
            for (long i = 0; i < (long)NG * NG * t->ne; i++) acc[i] += buf[i];
        }
        for (int e = 0; e < t->ne; e++)
            for (int jg = 0; jg < NG; jg++)
                for (int ig = 0; ig < NG; ig++) {
                    cplx v = acc[((long)e * NG + jg) * NG + ig];
                    if (gm) v = v / 3.0;
                    t->epsirr[(((long)iq * t->ne + e) * t->NTGQ + jg) * t->NTGQ + ig] = (float complex)v;
                }
        free(acc); free(buf);
    }
    return 0;
}

/* make_eps (calc_int_sub.F:222-311): eps^-1 of full q iq from its irreducible image, complex(4) */
static void make_eps(const orc_state *s, const int_state *t, int iq, float complex *epsmk /* [(e*NG + jg)*NG + ig] */) {
    int NG = t->NGQ_eps[iq], iqir = t->numirrq[iq], iop = t->numrotq[iq], itrs = t->trsq[iq];
    const double *ri = s->rginv + 9 * iop;
    const int *pgt = s->pg + 3 * iop, *RWt = t->RWq + 3 * iq;
    int n1 = 2 * t->Lq[0] + 1, n2 = 2 * t->Lq[1] + 1, n3 = 2 * t->Lq[2] + 1;
    const int *pk = t->packingq + (long)iqir * n1 * n2 * n3;
    int *idx = malloc(sizeof(int) * NG);
    cplx *p1 = malloc(sizeof(cplx) * NG), *p2 = malloc(sizeof(cplx) * NG);
    for (int ig = 0; ig < NG; ig++) {
        const int *g = t->LG0 + ((long)t->NTG2 * iq + ig) * 3;
        int i1 = g[0], j1 = g[1], k1 = g[2];
        if (itrs == -1) { i1 = -i1; j1 = -j1; k1 = -k1; }
        int i2 = i1 + RWt[0], j2 = j1 + RWt[1], k2 = k1 + RWt[2];
        int i3 = (int)ri[0] * i2 + (int)ri[3] * j2 + (int)ri[6] * k2;
        int j3 = (int)ri[1] * i2 + (int)ri[4] * j2 + (int)ri[7] * k2;
        int k3 = (int)ri[2] * i2 + (int)ri[5] * j2 + (int)ri[8] * k2;
        int v = 0;
        if (abs(i3) <= t->Lq[0] && abs(j3) <= t->Lq[1] && abs(k3) <= t->Lq[2])
            v = pk[(i3 + t->Lq[0]) + n1 * ((j3 + t->Lq[1]) + (long)n2 * (k3 + t->Lq[2]))];
        idx[ig] = v - 1;
        double phase = TPI * ((double)i1 * (double)pgt[0] + (double)j1 * (double)pgt[1] + (double)k1 * (double)pgt[2]);
        p1[ig] = cexp(-I * phase / (double)s->nnp);
        p2[ig] = cexp(I * phase / (double)s->nnp);
    }
    for (int e = 0; e < t->ne; e++)
        for (int jg = 0; jg < NG; jg++)
            for (int ig = 0; ig < NG; ig++) {
                int a = idx[ig], b = idx[jg];
                cplx v = 0;
                if (a >= 0 && b >= 0) {
                    float complex src = itrs == 1 ? t->epsirr[(((long)iqir * t->ne + e) * t->NTGQ + b) * t->NTGQ + a]
                                                  : t->epsirr[(((long)iqir * t->ne + e) * t->NTGQ + a) * t->NTGQ + b];
                    v = (cplx)src * p1[ig] * p2[jg];
                }
                epsmk[((long)e * NG + jg) * NG + ig] = (float complex)v;
            }
    free(idx); free(p1); free(p2);
}

/* rho_w(q+G) of calc_intW.F:647-767 for every full q: [(iq*NWF + w)*NTG2 + g] */
static void int_rho_w(const orc_state *s, int_state *t, cplx *rho) {
    const int NWF = t->NWF;
    long N = (long)s->nw[0] * s->nw[1] * s->nw[2];
    for (int iq = 0; iq < t->NTQ; iq++) {
        const double *q = t->SQ + 3 * iq;
        const int *LG = t->LG0 + (long)3 * t->NTG2 * iq;
        int ngp = t->NGQ_psi[iq];
        int gamma = q[0] == 0.0 && q[1] == 0.0 && q[2] == 0.0;
        double *len = calloc(ngp, sizeof(double));
        int nog0 = -1;
        for (int g = 0; g < ngp; g++) {
            if (gamma && LG[3 * g] == 0 && LG[3 * g + 1] == 0 && LG[3 * g + 2] == 0) { nog0 = g; continue; }
            len[g] = qg_len(s, q, LG + 3 * g);
        }
        if (gamma) t->NoG0 = nog0;
        cplx *acc = calloc((long)NWF * ngp, sizeof(cplx));
#pragma omp parallel
        {
            cplx *wk = malloc(sizeof(cplx) * N), *wkq = malloc(sizeof(cplx) * N), *m = malloc(sizeof(cplx) * ngp);
            cplx *part = calloc((long)NWF * ngp, sizeof(cplx));
#pragma omp for schedule(static)
            for (int k = 0; k < s->NTK; k++)
                for (int w = 0; w < NWF; w++) {
                    int ikq = k, sG[3] = {0, 0, 0};
                    if (!gamma) search_kq(s->NTK, s->SK0, q, k, &ikq, sG);
                    interstate(s, k, ikq, t->C0 + ((long)k * NWF + w) * s->NTG, t->C0 + ((long)ikq * NWF + w) * s->NTG,
                               LG, ngp, sG, wk, wkq, m);
                    if (gamma && nog0 >= 0) m[nog0] = 0;
                    for (int g = 0; g < ngp; g++) part[(long)w * ngp + g] += m[g];
                }
#pragma omp critical
            for (long i = 0; i < (long)NWF * ngp; i++) acc[i] += part[i];
            free(wk); free(wkq); free(m); free(part);
        }
        for (int w = 0; w < NWF; w++)
            for (int g = 0; g < ngp; g++) {
                cplx v = acc[(long)w * ngp + g];
                if (!(gamma && g == nog0)) v = v / len[g];
                rho[((long)iq * NWF + w) * t->NTG2 + g] = v / (double)s->NTK;
            }
        free(acc); free(len);
    }
}

/* Hybertsen-Louie head (calc_intW.F:778-795) */
static double int_qsz(const orc_state *s, const int_state *t) {
    return pow(6.0 * (PI_ * PI_) / (double)t->NTQ / s->VOLUME, 1.0 / 3.0);
}

/* sum over G, G' of a(G) eps(G,G') conj(b(G')) on the eps sphere plus the bare
 * shell (calc_intW.F:880-900), in the reference's loop order */
static cplx int_quad(const cplx *a, const cplx *b, const float complex *eps, int nge, int ngp) {
    cplx sum = 0;
    for (int ig = 0; ig < nge; ig++)
        for (int jg = 0; jg < nge; jg++) sum = sum + a[ig] * (cplx)eps[(long)jg * nge + ig] * conj(b[jg]);
    for (int ig = nge; ig < ngp; ig++) sum = sum + a[ig] * conj(b[ig]);
    return sum;
}

static void int_fourier(const int_state *t, const orc_state *s, const cplx *f /* [iq][j][i] */, int ne_f,
                        const int *na, double head, const double *headw, cplx *out) {
    const int NWF = t->NWF, n1 = 2 * na[0] + 1, n2 = 2 * na[1] + 1, n3 = 2 * na[2] + 1;
    for (int e = 0; e < ne_f; e++)
        for (int a3 = -na[2]; a3 <= na[2]; a3++)
            for (int a2 = -na[1]; a2 <= na[1]; a2++)
                for (int a1 = -na[0]; a1 <= na[0]; a1++)
                    for (int j = 0; j < NWF; j++)
                        for (int i = 0; i < NWF; i++) {
                            cplx sum = 0;
                            for (int iq = 0; iq < t->NTQ; iq++) {
                                const double *q = t->SQ + 3 * iq;
                                double phase = TPI * (q[0] * (double)a1 + q[1] * (double)a2 + q[2] * (double)a3);
                                cplx pf = cexp(-I * phase);
                                sum = sum + f[(((long)e * t->NTQ + iq) * NWF + j) * NWF + i] * pf;
                            }
                            long R = (a1 + na[0]) + n1 * ((a2 + na[1]) + (long)n2 * (a3 + na[2]));
                            out[(((long)e * n3 * n2 * n1 + R) * NWF + j) * NWF + i] =
                                2.0 * TPI * sum / s->VOLUME / (double)t->NTQ + (headw ? headw[e] : head);
                        }
}

/* rho_ij(q+G) of calc_intJ.F:641-677 (q != 0) and :748-791 (q = 0) for one R:
 * [(j*NWF + i)*ngp + g] */
static void int_rho_ij(const orc_state *s, int_state *t, int iq, const int *R, cplx *rho) {
    const int NWF = t->NWF;
    long N = (long)s->nw[0] * s->nw[1] * s->nw[2];
    const double *q = t->SQ + 3 * iq;
    const int *LG = t->LG0 + (long)3 * t->NTG2 * iq;
    int ngp = t->NGQ_psi[iq];
    int gamma = q[0] == 0.0 && q[1] == 0.0 && q[2] == 0.0;
    double *len = calloc(ngp, sizeof(double));
    int nog0 = -1;
    for (int g = 0; g < ngp; g++) {
        if (gamma && LG[3 * g] == 0 && LG[3 * g + 1] == 0 && LG[3 * g + 2] == 0) { nog0 = g; continue; }
        len[g] = qg_len(s, q, LG + 3 * g);
    }
    if (gamma) t->NoG0 = nog0;
    cplx *acc = calloc((long)NWF * NWF * ngp, sizeof(cplx));
#pragma omp parallel
    {
        cplx *wk = malloc(sizeof(cplx) * N), *wkq = malloc(sizeof(cplx) * N), *m = malloc(sizeof(cplx) * ngp);
        cplx *part = calloc((long)NWF * NWF * ngp, sizeof(cplx));
#pragma omp for schedule(static)
        for (int k = 0; k < s->NTK; k++)
            for (int i = 0; i < NWF; i++)
                for (int j = 0; j < NWF; j++) {
                    const double *sk = s->SK0 + 3 * k;
                    cplx pf = cexp(-I * TPI * (sk[0] * (double)R[0] + sk[1] * (double)R[1] + sk[2] * (double)R[2]));
                    int ikq = k, sG[3] = {0, 0, 0};
                    if (!gamma) search_kq(s->NTK, s->SK0, q, k, &ikq, sG);
                    interstate(s, k, ikq, t->C0 + ((long)k * NWF + j) * s->NTG, t->C0 + ((long)ikq * NWF + i) * s->NTG,
                               LG, ngp, sG, wk, wkq, m);
                    cplx *dst = part + ((long)j * NWF + i) * ngp;
                    if (gamma) {
                        if (nog0 >= 0) m[nog0] = 0;
                        for (int g = 0; g < ngp; g++) dst[g] += m[g] * pf;
                    } else {
                        for (int g = 0; g < ngp; g++) dst[g] += m[g] * pf / len[g];
                    }
                }
#pragma omp critical
        for (long x = 0; x < (long)NWF * NWF * ngp; x++) acc[x] += part[x];
        free(wk); free(wkq); free(m); free(part);
    }
    for (long p = 0; p < (long)NWF * NWF; p++)
        for (int g = 0; g < ngp; g++) {
            cplx v = acc[p * ngp + g];
            if (gamma && g != nog0) v = v / len[g] / (double)s->NTK;
            else v = v / (double)s->NTK;
            rho[p * ngp + g] = v;
        }
    free(acc); free(len);
}

/* ---- text writers (calc_intW.F:1006-1158, calc_intJ.F:925-1030) ---- */
static void wr_ints(FILE *f, int a, int b, int c) { fprintf(f, " %11d %11d %11d\n", a, b, c); }

static int wr_matrix(const char *path, const char *title, const char *row3, const orc_state *s, const int_state *t,
                     const int *na, const int *lo, const int *hi, const cplx *M /* (i,j,R) box */) {
    FILE *f = fopen(path, "w");
    if (!f) return fail("cannot write %s", path);
    const int NWF = t->NWF, n1 = 2 * na[0] + 1, n2 = 2 * na[1] + 1;
    fprintf(f, "%s\n#1:R1, 2:R2, 3:R3 (lattice vector)\n%s\n", title, row3);
    for (int a1 = lo[0]; a1 <= hi[0]; a1++)
        for (int a2 = lo[1]; a2 <= hi[1]; a2++)
            for (int a3 = lo[2]; a3 <= hi[2]; a3++) {
                wr_ints(f, a1, a2, a3);
                long R = (a1 + na[0]) + n1 * ((a2 + na[1]) + (long)n2 * (a3 + na[2]));
                for (int i = 0; i < NWF; i++)
                    for (int j = 0; j < NWF; j++) {
                        cplx v = M[(R * NWF + j) * NWF + i] * AU;
                        fprintf(f, "%5d%5d%20.10f%20.10f\n", i + 1, j + 1, creal(v), cimag(v));
                    }
                fprintf(f, "\n");
            }
    fclose(f);
    (void)s;
    return 0;
}

static const double BOHR = 0.529177; /* config_w3d.h */

static int wr_vs_r(const char *dir, const char *stem, const char *title, const char *cols, const orc_state *s,
                   const int_state *t, const int *na, const cplx *M) {
    const int NWF = t->NWF, n1 = 2 * na[0] + 1, n2 = 2 * na[1] + 1;
    for (int i = 0; i < NWF; i++) {
        char path[4096];
        snprintf(path, sizeof path, "%s/%s.%03d", dir, stem, i + 1);
        FILE *f = fopen(path, "w");
        if (!f) return fail("cannot write %s", path);
        fprintf(f, "%s\n%s\n", title, cols);
        for (int a1 = -na[0]; a1 <= na[0]; a1++)
            for (int a2 = -na[1]; a2 <= na[1]; a2++)
                for (int a3 = -na[2]; a3 <= na[2]; a3++)
                    for (int j = 0; j < NWF; j++) {
                        double rij[3];
                        for (int d = 0; d < 3; d++)
                            rij[d] = (double)a1 * s->a1[d] + (double)a2 * s->a2[d] + (double)a3 * s->a3[d] +
                                     (t->coord[3 * j + d] - t->coord[3 * i + d]);
                        double r = sqrt(rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2]);
                        long R = (a1 + na[0]) + n1 * ((a2 + na[1]) + (long)n2 * (a3 + na[2]));
                        cplx v = M[(R * NWF + j) * NWF + i] * AU;
                        fprintf(f, "%12.5f%12.5f%12.5f\n", r * BOHR, creal(v), cimag(v));
                    }
        fclose(f);
    }
    return 0;
}

static int wr_vs_e(const char *dir, const char *stem, const char *title, const char *cols, const int_state *t,
                   const int *na, const cplx *M /* box x ne */) {
    const int NWF = t->NWF;
    long box = (long)(2 * na[0] + 1) * (2 * na[1] + 1) * (2 * na[2] + 1), R0 = (box - 1) / 2;
    for (int i = 0; i < NWF; i++)
        for (int j = i; j < NWF; j++) {
            char path[4096];
            snprintf(path, sizeof path, "%s/%s.%03d-%03d", dir, stem, i + 1, j + 1);
            FILE *f = fopen(path, "w");
            if (!f) return fail("cannot write %s", path);
            fprintf(f, "%s\n%s\n", title, cols);
            for (int e = 0; e < t->ne; e++) {
                cplx w = t->em[e] * AU, v = M[(((long)e * box + R0) * NWF + j) * NWF + i] * AU;
                fprintf(f, "%12.5f%12.5f%12.5f%12.5f\n", creal(w), cimag(w), creal(v), cimag(v));
            }
            fclose(f);
        }
    return 0;
}

static void rwind(int *tv, int N, int L, int even) {
    if (even) { if (*tv < -N + 1) *tv += L; if (*tv > N) *tv -= L; }
    else { if (*tv < -N) *tv += L; if (*tv > N) *tv -= L; }
}

/* wrt_mvmc (wrt_mvmc_w3d.f90 / wrt_mvmc_j3d.f90): the lattice model on the
 * nkb1 x nkb2 x nkb3 supercell; HR (i,j,R) on the -Na..Na box */
static int wr_mvmc(const char *dir, const orc_state *s, const int_state *t, const int *na, double cut,
                   const cplx *HR, int exchange) {
    const int NWF = t->NWF, L1 = s->nkb[0], L2 = s->nkb[1], L3 = s->nkb[2], Nsite = s->NTK;
    const int n1 = 2 * na[0] + 1, n2 = 2 * na[1] + 1;
    const int even = Nsite % 2 == 0;
    cplx *H = calloc((long)NWF * NWF * Nsite * Nsite, sizeof(cplx));
    const int lo0 = even ? -na[0] + 1 : -na[0], lo1 = even ? -na[1] + 1 : -na[1], lo2 = even ? -na[2] + 1 : -na[2];
    const int off = even ? 1 : 0;
    for (int i1 = lo0; i1 <= na[0]; i1++)
        for (int i2 = lo1; i2 <= na[1]; i2++)
            for (int i3 = lo2; i3 <= na[2]; i3++) {
                long is = (i3 + na[2] - off) + (long)(i2 + na[1] - off) * L3 + (long)(i1 + na[0] - off) * L3 * L2;
                for (int j1 = lo0; j1 <= na[0]; j1++)
                    for (int j2 = lo1; j2 <= na[1]; j2++)
                        for (int j3 = lo2; j3 <= na[2]; j3++) {
                            long js = (j3 + na[2] - off) + (long)(j2 + na[1] - off) * L3 + (long)(j1 + na[0] - off) * L3 * L2;
                            int t1 = j1 - i1, t2 = j2 - i2, t3 = j3 - i3;
                            rwind(&t1, na[0], L1, even); rwind(&t2, na[1], L2, even); rwind(&t3, na[2], L3, even);
                            if (is < 0 || is >= Nsite || js < 0 || js >= Nsite) continue;
                            if (abs(t1) > na[0] || abs(t2) > na[1] || abs(t3) > na[2]) continue;
                            long R = (t1 + na[0]) + n1 * ((t2 + na[1]) + (long)n2 * (t3 + na[2]));
                            for (int b = 0; b < NWF; b++)
                                for (int a = 0; a < NWF; a++)
                                    H[(((long)js * Nsite + is) * NWF + b) * NWF + a] = HR[(R * NWF + b) * NWF + a];
                        }
            }
#define HH(a, b, is, js) H[(((long)(js) * Nsite + (is)) * NWF + (b)) * NWF + (a)]
    const char *eq = "==============================";
    char path[4096];
    if (!exchange) {
        snprintf(path, sizeof path, "%s/zCoulombIntra.def", dir);
        FILE *f = fopen(path, "w");
        if (!f) { free(H); return fail("cannot write %s", path); }
        fprintf(f, "%s\n%-13s%17d\n%s\n%s\n%s\n", eq, "NCoulombIntra", Nsite * NWF, eq, eq, eq);
        for (int is = 0; is < Nsite; is++)
            for (int b = 0; b < NWF; b++)
                fprintf(f, "%5d%15.10f\n", b + is * NWF, creal(HH(b, b, is, is)) * AU);
        fclose(f);
    }
    /* pairs i < j with |H| >= cut (Inter / Hund / Exchange), and i != j (PairHop) */
    const char *names[3] = {"zCoulombInter.def", "zHund.def", "zExchange.def"};
    const char *keys[3] = {"NCoulombInter", "NHund", "NExchange"};
    const int kw[3][2] = {{13, 17}, {5, 25}, {9, 21}};
    int first = exchange ? 1 : 0, last = exchange ? 2 : 0;
    for (int which = first; which <= last + (exchange ? 1 : 0); which++) {
        int pairhop = exchange && which == 3;
        long cnt = 0;
        for (int pass = 0; pass < 2; pass++) {
            FILE *f = NULL;
            if (pass == 1) {
                snprintf(path, sizeof path, "%s/%s", dir, pairhop ? "zPairHop.def" : names[which]);
                f = fopen(path, "w");
                if (!f) { free(H); return fail("cannot write %s", path); }
                if (pairhop) fprintf(f, "%s\n%-8s%22ld\n", eq, "NPairhop", cnt);
                else fprintf(f, "%s\n%-*s%*ld\n", eq, kw[which][0], keys[which], kw[which][1], cnt);
                fprintf(f, "%s\n%s%10.5f%s\n%s\n", eq, exchange ? "=== Jcut >" : "=== Vcut >", cut * AU, "eV =======", eq);
            }
            for (int is = 0; is < Nsite; is++)
                for (int b = 0; b < NWF; b++) {
                    int i = b + is * NWF;
                    for (int js = 0; js < Nsite; js++)
                        for (int c = 0; c < NWF; c++) {
                            int j = c + js * NWF;
                            if (pairhop ? (j == i) : (i >= j)) continue;
                            cplx h = HH(b, c, is, js);
                            if (cabs(h) < cut) continue;
                            if (pass == 0) cnt++;
                            else fprintf(f, "%5d%5d%15.10f\n", i, j, creal(h) * AU);
                        }
                }
            if (f) fclose(f);
        }
    }
#undef HH
    free(H);
    return 0;
}

static int rm_rf_dir(const char *dir) {
    /* the files this program writes; the reference runs `rm -rf` on the folder */
    char cmd[4200];
    snprintf(cmd, sizeof cmd, "rm -rf '%s'", dir);
    return system(cmd) == 0 ? 0 : fail("cannot clear %s", dir);
}

int orc_calc_int(const char *root, const orc_int_params *P, orc_int_dims *dims, double *V, double *W, double *X,
                 double *Jm) {
    double t0 = now_s();
    orc_state s;
    memset(&s, 0, sizeof s);
    int_state t;
    memset(&t, 0, sizeof t);
    orc_params p;
    orc_default_params(&p);
    p.n_calc_band = 1;
    for (int d = 0; d < 3; d++) p.fft_box[d] = P->fft_box[d];
#ifdef _OPENMP
    if (P->nthreads > 0) omp_set_num_threads(P->nthreads);
#endif
    int rc = 1;
    if (setup(&s, root, &p) || int_read(&s, &t, root, P) || int_unfold_q(&s, &t) || int_read_eps(&s, &t, root)) goto done;
    int na[3] = {s.nkb[0] / 2, s.nkb[1] / 2, s.nkb[2] / 2};
    int lo[3] = {P->ix_min, P->iy_min, P->iz_min}, hi[3] = {P->ix_max, P->iy_max, P->iz_max};
    for (int d = 0; d < 3; d++)
        if (lo[d] > hi[d] || lo[d] < -na[d] || hi[d] > na[d]) { fail("intJ range outside -Na..Na"); goto done; }
    if (t.iqgm < 0) { fail("no Gamma point among the q points"); goto done; }
    long box = (long)(2 * na[0] + 1) * (2 * na[1] + 1) * (2 * na[2] + 1);
    if (dims) {
        dims->nwf = t.NWF; dims->ne = t.ne; dims->ntq = t.NTQ;
        for (int d = 0; d < 3; d++) { dims->na[d] = na[d]; dims->nkb[d] = s.nkb[d]; dims->fft_box[d] = s.nw[d]; }
        dims->box = (int)box;
    }
    const int NWF = t.NWF, ne = t.ne, ie = P->calc_ifreq - 1;
    const double qsz = int_qsz(&s, &t), chead = (2.0 / PI_) * qsz;
    double *cheadw = calloc(ne, sizeof(double));
    char dir[4096];
    if (P->do_w) {
        cplx *rho = calloc((long)t.NTQ * NWF * t.NTG2, sizeof(cplx));
        int_rho_w(&s, &t, rho);
        for (int e = 0; e < ne; e++)
            cheadw[e] = creal((2.0 / PI_) * (cplx)t.epsirr[(((long)t.iqgm * ne + e) * t.NTGQ + t.NoG0) * t.NTGQ + t.NoG0] * qsz);
        cplx *func = calloc((long)t.NTQ * NWF * NWF, sizeof(cplx));
        cplx *funcw = calloc((long)ne * t.NTQ * NWF * NWF, sizeof(cplx));
        float complex *epsmk = malloc(sizeof(float complex) * (long)t.NTGQ * t.NTGQ * ne);
        for (int iq = 0; iq < t.NTQ; iq++) {
            int nge = t.NGQ_eps[iq], ngp = t.NGQ_psi[iq];
            for (int i = 0; i < NWF; i++)
                for (int j = 0; j < NWF; j++) {
                    const cplx *a = rho + ((long)iq * NWF + i) * t.NTG2, *b = rho + ((long)iq * NWF + j) * t.NTG2;
                    cplx sum = 0;
                    for (int g = 0; g < ngp; g++) sum = sum + a[g] * conj(b[g]);
                    func[((long)iq * NWF + j) * NWF + i] = sum;
                }
            make_eps(&s, &t, iq, epsmk);
#pragma omp parallel for collapse(2) schedule(static)
            for (int e = 0; e < ne; e++)
                for (int i = 0; i < NWF; i++)
                    for (int j = 0; j < NWF; j++) {
                        const cplx *a = rho + ((long)iq * NWF + i) * t.NTG2, *b = rho + ((long)iq * NWF + j) * t.NTG2;
                        funcw[(((long)e * t.NTQ + iq) * NWF + j) * NWF + i] =
                            int_quad(a, b, epsmk + (long)e * nge * nge, nge, ngp);
                    }
        }
        free(epsmk);
        cplx *Vm = malloc(sizeof(cplx) * box * NWF * NWF), *Wm = malloc(sizeof(cplx) * box * NWF * NWF * ne);
        int_fourier(&t, &s, func, 1, na, chead, NULL, Vm);
        int_fourier(&t, &s, funcw, ne, na, 0.0, cheadw, Wm);
        if (V) memcpy(V, Vm, sizeof(cplx) * box * NWF * NWF);
        if (W) memcpy(W, Wm, sizeof(cplx) * box * NWF * NWF * ne);
        if (P->write_files) {
            snprintf(dir, sizeof dir, "%s/dir-intW", root);
            if (rm_rf_dir(dir) || mkdir_p(dir)) goto w_out;
            char path[4096];
            int full_lo[3] = {-na[0], -na[1], -na[2]};
            snprintf(path, sizeof path, "%s/dat.Vmat", dir);
            if (wr_matrix(path, "#Bare Coulomb: V", "#1:i, 2:j, 3:Re(V_ij) [eV], 4:Im(V_ij) [eV]", &s, &t, na, full_lo, na, Vm)) goto w_out;
            snprintf(path, sizeof path, "%s/dat.Wmat", dir);
            if (wr_matrix(path, "#Screened Coulomb: W at omega=calc_ifreq", "#1:i, 2:j, 3:Re(W_ij) [eV], 4:Im(W_ij) [eV]", &s, &t, na,
                          full_lo, na, Wm + (long)ie * box * NWF * NWF)) goto w_out;
            if (wr_vs_r(dir, "dat.VvsR", "#R dependence of bare Coulomb", "#1:R [AA], 2:Re[V(R)] [eV], 3:Im[V(R)] [eV]", &s, &t, na, Vm)) goto w_out;
            if (wr_vs_r(dir, "dat.WvsR", "#R dependence of screened Coulomb at omega=calc_ifreq", "#1:R [AA], 2:Re[W(R)] [eV], 3:Im[W(R)] [eV]",
                        &s, &t, na, Wm + (long)ie * box * NWF * NWF)) goto w_out;
            if (wr_vs_e(dir, "dat.UvsE", "#Omega dependence of onsite Coulomb", "#1:Re(w) [eV], 2:Im(w) [eV], 3:Re[U(w)] [eV], 4:Im[U(w)] [eV]", &t, na, Wm)) goto w_out;
            snprintf(dir, sizeof dir, "%s/dir-mvmc", root);
            if (mkdir_p(dir)) goto w_out;
            if (wr_mvmc(dir, &s, &t, na, P->wcut_mvmc / AU, Wm + (long)ie * box * NWF * NWF, 0)) goto w_out;
        }
        free(rho); free(func); free(funcw); free(Vm); free(Wm);
        goto w_done;
    w_out:
        free(rho); free(func); free(funcw); free(Vm); free(Wm); free(cheadw);
        goto done;
    w_done:;
    }
    if (P->do_j) {
        cplx *Xm = calloc(box * NWF * NWF, sizeof(cplx)), *Jw = calloc(box * NWF * NWF * ne, sizeof(cplx));
        float complex *epsmk = malloc(sizeof(float complex) * (long)t.NTGQ * t.NTGQ * ne);
        cplx *rho = malloc(sizeof(cplx) * (long)NWF * NWF * t.NTG2);
        cplx *func = calloc((long)t.NTQ * NWF * NWF, sizeof(cplx)), *funcw = calloc((long)ne * t.NTQ * NWF * NWF, sizeof(cplx));
        const int n1 = 2 * na[0] + 1, n2 = 2 * na[1] + 1;
        for (int a1 = lo[0]; a1 <= hi[0]; a1++)
            for (int a2 = lo[1]; a2 <= hi[1]; a2++)
                for (int a3 = lo[2]; a3 <= hi[2]; a3++) {
                    int R[3] = {a1, a2, a3};
                    for (int iq = 0; iq < t.NTQ; iq++) {
                        const double *q = t.SQ + 3 * iq;
                        int gamma = q[0] == 0.0 && q[1] == 0.0 && q[2] == 0.0;
                        int nge = t.NGQ_eps[iq], ngp = t.NGQ_psi[iq];
                        int_rho_ij(&s, &t, iq, R, rho);
                        for (int i = 0; i < NWF; i++)
                            for (int j = 0; j < NWF; j++) {
                                const cplx *r = rho + ((long)j * NWF + i) * ngp;
                                cplx sum = 0;
                                for (int g = 0; g < ngp; g++) sum = sum + r[g] * conj(r[g]);
                                func[((long)iq * NWF + j) * NWF + i] = sum;
                            }
                        /* Gamma reads the irreducible array at the full index (calc_intJ.F:818) */
                        if (gamma) {
                            if (iq >= t.Nq_irr) { fail("Gamma outside the irreducible q list"); goto j_out; }
                            for (int e = 0; e < ne; e++)
                                for (int jg = 0; jg < nge; jg++)
                                    for (int ig = 0; ig < nge; ig++)
                                        epsmk[((long)e * nge + jg) * nge + ig] =
                                            t.epsirr[(((long)iq * ne + e) * t.NTGQ + jg) * t.NTGQ + ig];
                        } else {
                            make_eps(&s, &t, iq, epsmk);
                        }
#pragma omp parallel for collapse(2) schedule(static)
                        for (int e = 0; e < ne; e++)
                            for (int i = 0; i < NWF; i++)
                                for (int j = 0; j < NWF; j++) {
                                    const cplx *r = rho + ((long)j * NWF + i) * ngp;
                                    funcw[(((long)e * t.NTQ + iq) * NWF + j) * NWF + i] =
                                        int_quad(r, r, epsmk + (long)e * nge * nge, nge, ngp);
                                }
                    }
                    long Ri = (a1 + na[0]) + n1 * ((a2 + na[1]) + (long)n2 * (a3 + na[2]));
                    for (int i = 0; i < NWF; i++)
                        for (int j = 0; j < NWF; j++) {
                            cplx sum = 0;
                            for (int iq = 0; iq < t.NTQ; iq++) sum += func[((long)iq * NWF + j) * NWF + i];
                            Xm[(Ri * NWF + j) * NWF + i] = 2.0 * TPI * sum / s.VOLUME / (double)t.NTQ;
                        }
                    for (int e = 0; e < ne; e++)
                        for (int i = 0; i < NWF; i++)
                            for (int j = 0; j < NWF; j++) {
                                cplx sum = 0;
                                for (int iq = 0; iq < t.NTQ; iq++) sum += funcw[(((long)e * t.NTQ + iq) * NWF + j) * NWF + i];
                                Jw[(((long)e * box + Ri) * NWF + j) * NWF + i] = 2.0 * TPI * sum / s.VOLUME / (double)t.NTQ;
                            }
                }
        {
            /* Hybertsen-Louie head on the R = 0 diagonal (calc_intJ.F:876-905) */
            long R0 = (box - 1) / 2;
            for (int e = 0; e < ne; e++)
                cheadw[e] = creal((2.0 / PI_) * (cplx)t.epsirr[(((long)t.iqgm * ne + e) * t.NTGQ + t.NoG0) * t.NTGQ + t.NoG0] * qsz);
            for (int i = 0; i < NWF; i++) {
                Xm[(R0 * NWF + i) * NWF + i] += chead;
                for (int e = 0; e < ne; e++) Jw[(((long)e * box + R0) * NWF + i) * NWF + i] += cheadw[e];
            }
        }
        if (X) memcpy(X, Xm, sizeof(cplx) * box * NWF * NWF);
        if (Jm) memcpy(Jm, Jw, sizeof(cplx) * box * NWF * NWF * ne);
        if (P->write_files) {
            snprintf(dir, sizeof dir, "%s/dir-intJ", root);
            if (rm_rf_dir(dir) || mkdir_p(dir)) goto j_out;
            char path[4096];
            snprintf(path, sizeof path, "%s/dat.Xmat", dir);
            if (wr_matrix(path, "#Bare exchamge: X", "#1:i, 2:j, 3:Re(X_ij) [eV], 4:Im(X_ij) [eV]", &s, &t, na, lo, hi, Xm)) goto j_out;
            snprintf(path, sizeof path, "%s/dat.Jmat", dir);
            if (wr_matrix(path, "#Screened exchamge: J at omega=calc_ifreq", "#1:i, 2:j, 3:Re(J_ij) [eV], 4:Im(J_ij) [eV]", &s, &t, na,
                          lo, hi, Jw + (long)ie * box * NWF * NWF)) goto j_out;
            if (wr_vs_e(dir, "dat.JvsE", "#Omega dependence of screened exchange J", "#Re(w) [eV], Im(w) [eV], Re[J(w)] [eV], Im[J(w)] [eV]", &t, na, Jw)) goto j_out;
            snprintf(dir, sizeof dir, "%s/dir-mvmc", root);
            if (mkdir_p(dir)) goto j_out;
            if (wr_mvmc(dir, &s, &t, na, P->jcut_mvmc / AU, Jw + (long)ie * box * NWF * NWF, 1)) goto j_out;
        }
        free(Xm); free(Jw); free(epsmk); free(rho); free(func); free(funcw);
        goto j_done;
    j_out:
        free(Xm); free(Jw); free(epsmk); free(rho); free(func); free(funcw); free(cheadw);
        goto done;
    j_done:;
    }
    free(cheadw);
    rc = 0;
done:
    if (dims) dims->seconds = now_s() - t0;
    free_int(&t);
    free_state(&s);
    return rc;
}
