/*
 * ram_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; see ram_oracle.h).
 *
 * Restates, loop for loop and with the same double literals and operation
 * order, these reference routines (paths relative to the reference project):
 *   DRIFTPARA  src/ModRamDrift.f90:36-88
 *   DRIFTR     src/ModRamDrift.f90:95-198
 *   DRIFTP     src/ModRamDrift.f90:204-279
 *   DRIFTE     src/ModRamDrift.f90:285-376
 *   DRIFTMU    src/ModRamDrift.f90:382-473
 *   CEPARA     src/ModRamLoss.f90:19-170 (analytic H/He/O branches)
 *   CHAREXCHANGE src/ModRamLoss.f90:457-478
 *   ATMOL      src/ModRamLoss.f90:485-507
 *   SUMRC      src/ModRamRun.f90:231-259
 *   ANISCH     src/ModRamRun.f90:343-415 (moment block only)
 *   ram_run    src/ModRamRun.f90:16-225 (without Coulomb/WPI/EMIC/FLC)
 * Constants are those of src/ModRamConst.f90:13-23.
 *
 * Addition not in the reference: p->closed selects closed outer faces in
 * R, E and MU (FBND at both ends forced to zero) so that the weighted
 * content  sum F2*WE*WMU  is conserved; it is applied identically here and
 * in the CUDA kernels.
 */
#include "ram_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/ModRamConst.f90:13-23 (all double under -fdefault-real-8) */
static const double RE = 6.371E6;
static const double HMIN_UNUSED = 2E5;
static const double Q = 1.602E-19;
static const double CS = 2.998E8;
static const double PI = 3.1415926535897932384626433832795;

/* 1-based Fortran index helpers for one species. */
#define NR (g->nr)
#define NT (g->nt)
#define NE (g->ne)
#define NPA (g->npa)
#define IX4(I, J, K, L) ((size_t)((((L)-1) * NE + (K)-1) * NT + (J)-1) * NR + (I)-1)
#define IXF(I, J, L) ((size_t)(((L)-1) * NT + (J)-1) * (NR + 1) + (I)-1)
#define IX2(I, J) ((size_t)((J)-1) * (NR + 1) + (I)-1)
#define IXM(I, J) ((size_t)((J)-1) * NR + (I)-1)
#define IXG(J, K, L) ((size_t)(((L)-1) * NE + (K)-1) * NT + (J)-1)
#define IXFF(I, K, L) ((size_t)(((L)-1) * NE + (K)-1) * NR + (I)-1)
#define IXRK(I, K) ((size_t)((K)-1) * NR + (I)-1)
#define IXRL(I, L) ((size_t)((L)-1) * NR + (I)-1)

#define F2(I, J, K, L) f2[IX4(I, J, K, L)]
#define FNHS(I, J, L) g->fnhs[IXF(I, J, L)]
#define FNIS(I, J, L) g->fnis[IXF(I, J, L)]
#define BOUNHS(I, J, L) g->bounhs[IXF(I, J, L)]
#define BOUNIS(I, J, L) g->bounis[IXF(I, J, L)]
#define HDNS(I, J, L) g->hdns[IXF(I, J, L)]
#define DIDT(I, J, L) g->didt[IXF(I, J, L)]
#define DIBNDT(I, J, L) g->dibndt[IXF(I, J, L)]
#define BNES(I, J) g->bnes[IX2(I, J)]
#define DBDT(I, J) g->dbdt[IX2(I, J)]
#define EIR(I, J) g->eir[IX2(I, J)]
#define EIP(I, J) g->eip[IX2(I, J)]
#define VT(I, J) vt[IX2(I, J)]
#define OUTSIDE(I, J) g->outside_mgnp[IXM(I, J)]
#define RLZ(I) g->rlz[(I)-1]
#define LZ(I) g->lz[(I)-1]
#define PHI(J) g->phi[(J)-1]
#define EKEV(K) g->ekev[(K)-1]
#define EBND(K) g->ebnd[(K)-1]
#define WE(K) g->we[(K)-1]
#define DE(K) g->de[(K)-1]
#define MU(L) g->mu[(L)-1]
#define DMU(L) g->dmu[(L)-1]
#define WMU(L) g->wmu[(L)-1]
#define UPA(I) g->upa[(I)-1]
#define GREL(K) sp->grel[(K)-1]
#define GRBND(K) sp->grbnd[(K)-1]
#define VV(K) sp->v[(K)-1]
#define FFACTOR(I, K, L) sp->ffactor[IXFF(I, K, L)]
#define EPP(K) sp->epp[(K)-1]
#define ERNH(K) sp->ernh[(K)-1]
#define VR(I) dp->vr[(I)-1]
#define P1(I) dp->p1[(I)-1]
#define P2(I, K) dp->p2[IXRK(I, K)]
#define EDOT(I, K) dp->edot[IXRK(I, K)]
#define MUDOT(I, L) dp->mudot[IXRL(I, L)]

/* Threads for the loops over independent lines inside one routine (the
 * reference runs them serially; the results do not depend on this). */
static int g_inner = 1;
void ro_set_inner_threads(int n) { g_inner = n < 1 ? 1 : n; }

static inline double dmax(double a, double b) { return a > b ? a : b; }
static inline double dmin(double a, double b) { return a < b ? a : b; }
/* Fortran MAX/MIN for the limiter: MAX(MIN(B*R,1.),MIN(R,B)) */
static inline double limiter(double betalim, double r)
{
    return dmax(dmin(betalim * r, 1.), dmin(r, betalim));
}

void ro_vt_vols(const ro_grid *g, double kp, double *vt)
{
    /* AVS=7.05E-6/(1.-0.159*KP+0.0093*KP**2)**3/RE ; PHIOFS = 0 */
    double t = 1. - 0.159 * kp + 0.0093 * (kp * kp);
    double avs = 7.05E-6 / (t * t * t) / RE;
    const double phiofs = 0 * PI / 12.;
    for (int I = 1; I <= NR + 1; ++I)
        for (int J = 1; J <= NT; ++J) {
            double lr = LZ(I) * RE;
            VT(I, J) = avs * (lr * lr) * sin(PHI(J) - phiofs);
        }
}

void ro_driftpara(const ro_grid *g, const ro_species *sp, const ro_params *p, ro_driftpara_t *dp)
{
    const double DTs = p->dts, MDR = g->mdr, DPHI = g->dphi;
    const int QS = sp->qs;
    for (int I = 1; I <= NR; ++I) {
        VR(I) = DTs / MDR / (RLZ(I) + 0.5 * MDR) / 2 / DPHI;
        P1(I) = DTs / DPHI / 2 / MDR / RLZ(I);
        for (int K = 1; K <= NE; ++K)
            P2(I, K) = DTs * EKEV(K) * 1000 * (GREL(K) + 1) / GREL(K) / (RLZ(I) * RLZ(I)) / DPHI / QS;
    }
    for (int I = 1; I <= NR; ++I) {
        for (int L = 1; L <= NPA - 1; ++L) {
            double MUBOUN = MU(L) + 0.5 * WMU(L);
            MUDOT(I, L) = (1. - MUBOUN * MUBOUN) * DTs / 2 / MUBOUN / RLZ(I);
        }
        MUDOT(I, NPA) = 0.;
        for (int K = 1; K <= NE; ++K)
            EDOT(I, K) = EBND(K) * DTs / RLZ(I) * (GRBND(K) + 1) / GRBND(K) / 2.;
    }
}

/* Frozen-limiter branch of one face (for the adjoint): 0 upwind only,
 * 1 LIMITER = BetaLim*R, 2 LIMITER = 1, 3 LIMITER = R, 4 LIMITER = BetaLim,
 * following MAX(MIN(BetaLim*R,1.),MIN(R,BetaLim)) literally. */
static int limiter_case(double betalim, double r)
{
    double a = dmin(betalim * r, 1.), b = dmin(r, betalim);
    if (dmax(a, b) == a && !(b > a)) return (betalim * r < 1.) ? 1 : 2;
    return (r < betalim) ? 3 : 4;
}
#define REC_CLIP 8

/* ------------------------------------------------------------------ DRIFTR */
static double driftr_impl(const ro_grid *g, const ro_species *sp, const ro_params *p,
                          const ro_driftpara_t *dp, const double *vt, const double *fgeos,
                          double *f2, double *cdrift, unsigned char *rec, int *gsrc);

double ro_driftr(const ro_grid *g, const ro_species *sp, const ro_params *p,
                 const ro_driftpara_t *dp, const double *vt, const double *fgeos,
                 double *f2, double *cdrift)
{
    return driftr_impl(g, sp, p, dp, vt, fgeos, f2, cdrift, NULL, NULL);
}

double ro_driftr_rec(const ro_grid *g, const ro_species *sp, const ro_params *p,
                     const ro_driftpara_t *dp, const double *vt, const double *fgeos,
                     double *f2, double *cdrift, unsigned char *rec, int *gsrc)
{
    return driftr_impl(g, sp, p, dp, vt, fgeos, f2, cdrift, rec, gsrc);
}

/* CGR of DRIFTR (src/ModRamDrift.f90:139-144) for face I of line (J,K,L). */
static double driftr_cgr(const ro_grid *g, double P4, double MDR, int I, int J, int J0, int J1, int L)
{
    double CGR1 = FNIS(I + 1, J1, L) + FNIS(I, J1, L) - FNIS(I + 1, J0, L) - FNIS(I, J0, L);
    double CGR2 = BNES(I + 1, J1) + BNES(I, J1) - BNES(I + 1, J0) - BNES(I, J0);
    double CGR3 = CGR1 + (FNIS(I + 1, J, L) + FNIS(I, J, L) - 2 * FNHS(I + 1, J, L)
                          - 2 * FNHS(I, J, L)) * CGR2 / 2. / (BNES(I + 1, J) + BNES(I, J));
    return CGR3 / (FNHS(I, J, L) + FNHS(I + 1, J, L)) * P4 / 2.
           / (BNES(I, J) + BNES(I + 1, J)) / (RLZ(I) + 0.5 * MDR);
}

static double driftr_p4(const ro_grid *g, const ro_species *sp, double DTs, double DPHI, double MDR,
                        int QS, int K)
{
    return DTs * EKEV(K) * 1000.0 * (GREL(K) + 1) / GREL(K) / DPHI / MDR / QS;
}

static double driftr_impl(const ro_grid *g, const ro_species *sp, const ro_params *p,
                          const ro_driftpara_t *dp, const double *vt, const double *fgeos,
                          double *f2, double *cdrift, unsigned char *rec, int *gsrc)
{
    const double DTs = p->dts, MDR = g->mdr, DPHI = g->dphi, BetaLim = p->betalim;
    const int QS = sp->qs;
    double DtDriftR = 100000.0;
    double *CR = (double *)calloc((size_t)NR * NT, sizeof(double));
    /* FGEOS index of the line whose ghost F(NR+1:NR+2) is held when plane
     * (K,L) starts, in the reference's K->L->J line order; -1: none yet, or
     * the last inflow line was outside the magnetopause (ghost 0).  Lines
     * are otherwise independent, so planes may run in parallel. */
    int *plane_src = (int *)malloc(sizeof(int) * (size_t)NE * NPA);

    for (int I = 1; I <= NR; ++I)
        for (int J = 1; J <= NT; ++J) {
            int J0 = J - 1;
            if (J == 1) J0 = NT - 1;
            int J1 = J + 1;
            if (J == NT) J1 = 2;
            double den = BNES(I, J) + BNES(I + 1, J);
            CR[IXM(I, J)] = VR(I) * (VT(I, J0) + VT(I + 1, J0) - VT(I, J1) - VT(I + 1, J1)) / den
                          + (EIP(I, J) + EIP(I + 1, J)) / den * DTs / MDR;
        }
    {
        int src = -1;
        for (int K = 1; K <= NE; ++K) {
            double P4 = driftr_p4(g, sp, DTs, DPHI, MDR, QS, K);
            for (int L = 1; L <= NPA; ++L) {
                plane_src[(size_t)(L - 1) * NE + (K - 1)] = src;
                for (int J = 1; J <= NT; ++J) {
                    int J0 = J - 1;
                    if (J == 1) J0 = NT - 1;
                    int J1 = J + 1;
                    if (J == NT) J1 = 2;
                    double cnr = CR[IXM(NR, J)] + driftr_cgr(g, P4, MDR, NR, J, J0, J1, L);
                    if (cnr < 0) src = (OUTSIDE(NR, J) == 1) ? -1 : (int)IXG(J, K, L);
                }
            }
        }
    }

#ifdef _OPENMP
#pragma omp parallel num_threads(g_inner) reduction(min : DtDriftR)
#endif
    {
        int *sgn = (int *)malloc(sizeof(int) * NR * NT);
        double *F = (double *)calloc((size_t)NR + 2, sizeof(double)); /* F(1:NR+2) -> F[0..NR+1] */
        double *FBND = (double *)calloc((size_t)NR, sizeof(double));
        double *CD = (double *)malloc(sizeof(double) * NR); /* CDriftR(:,J,K,L) of the current line */
#define FF(n) F[(n)-1]
#define FB(n) FBND[(n)-1]
#define SG(i, j) sgn[IXM(i, j)]
        for (int i = 0; i < NR * NT; ++i) sgn[i] = 1;
#ifdef _OPENMP
#pragma omp for collapse(2) schedule(static)
#endif
        for (int K = 1; K <= NE; ++K)
            for (int L = 1; L <= NPA; ++L) {
                double P4 = driftr_p4(g, sp, DTs, DPHI, MDR, QS, K);
                int last_src = plane_src[(size_t)(L - 1) * NE + (K - 1)];
                FF(NR + 1) = 0.;
                FF(NR + 2) = 0.;
                if (last_src >= 0) {
                    int jj = last_src % NT + 1, ll = last_src / (NT * NE) + 1;
                    FF(NR + 1) = fgeos[last_src] * g->conf1 * FNHS(NR, jj, ll);
                    FF(NR + 2) = fgeos[last_src] * g->conf2 * FNHS(NR, jj, ll);
                }
                for (int J = 1; J <= NT; ++J) {
                    for (int I = 1; I <= NR; ++I) FF(I) = F2(I, J, K, L);
                    int J0 = J - 1;
                    if (J == 1) J0 = NT - 1;
                    int J1 = J + 1;
                    if (J == NT) J1 = 2;
                    for (int I = 1; I <= NR; ++I) {
                        CD[I - 1] = CR[IXM(I, J)] + driftr_cgr(g, P4, MDR, I, J, J0, J1, L);
                        if (OUTSIDE(I, J) == 0) {
                            double ctemp = dmax(fabs(CD[I - 1]), 1E-10);
                            DtDriftR = dmin(DtDriftR, p->fraccfl * DTs / ctemp);
                        }
                        SG(I, J) = 1;
                        if (CD[I - 1] < 0) SG(I, J) = -1;
                    }
                    int UR;
                    if (rec)
                        for (int I = 1; I <= NR; ++I) rec[IX4(I, J, K, L)] = 0;
                    if (SG(NR, J) == 1) {
                        FB(1) = 0.;
                        FB(NR) = FF(NR);
                        UR = NR - 1;
                    } else {
                        FB(1) = FF(2);
                        UR = NR;
                        if (OUTSIDE(NR, J) == 1) {
                            FF(NR + 1) = 0.;
                            FF(NR + 2) = 0.;
                            last_src = -1;
                        } else {
                            FF(NR + 1) = fgeos[IXG(J, K, L)] * g->conf1 * FNHS(NR, J, L);
                            FF(NR + 2) = fgeos[IXG(J, K, L)] * g->conf2 * FNHS(NR, J, L);
                            last_src = (int)IXG(J, K, L);
                        }
                    }
                    if (gsrc) gsrc[IXG(J, K, L)] = last_src;
                    for (int I = 2; I <= UR; ++I) {
                        int s = SG(I, J);
                        double X = FF(I + 1) - FF(I);
                        double FUP = 0.5 * (FF(I) + FF(I + 1) - s * X);
                        int cs = 0;
                        if (fabs(X) <= 1.E-27) FB(I) = FUP;
                        if (fabs(X) > 1.E-27) {
                            int N = I + 1 - s;
                            double R = (FF(N) - FF(N - 1)) / X;
                            if (R <= 0) FB(I) = FUP;
                            if (R > 0) {
                                double LIM = limiter(BetaLim, R);
                                double CORR = -0.5 * (CD[I - 1] - s) * X;
                                FB(I) = FUP + LIM * CORR;
                                cs = limiter_case(BetaLim, R);
                            }
                        }
                        if (rec) rec[IX4(I, J, K, L)] = (unsigned char)cs;
                    }
                    if (p->closed) {
                        FB(1) = 0.;
                        FB(NR) = 0.;
                    }
                    for (int I = 2; I <= NR; ++I) {
                        F2(I, J, K, L) = F2(I, J, K, L) - CD[I - 1] * FB(I) + CD[I - 2] * FB(I - 1);
                        if (F2(I, J, K, L) < 0) {
                            F2(I, J, K, L) = 1E-15;
                            if (rec) rec[IX4(I, J, K, L)] |= REC_CLIP;
                        }
                    }
                    if (cdrift)
                        for (int I = 1; I <= NR; ++I) cdrift[IX4(I, J, K, L)] = CD[I - 1];
                }
            }
#undef FF
#undef FB
#undef SG
        free(sgn);
        free(F);
        free(FBND);
        free(CD);
    }
    free(CR);
    free(plane_src);
    return DtDriftR;
}

/* ------------------------------------------------------------------ DRIFTP */
static double driftp_impl(const ro_grid *g, const ro_species *sp, const ro_params *p,
                          const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift,
                          unsigned char *rec);
double ro_driftp(const ro_grid *g, const ro_species *sp, const ro_params *p,
                 const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift)
{
    return driftp_impl(g, sp, p, dp, vt, f2, cdrift, NULL);
}
double ro_driftp_rec(const ro_grid *g, const ro_species *sp, const ro_params *p,
                     const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift,
                     unsigned char *rec)
{
    return driftp_impl(g, sp, p, dp, vt, f2, cdrift, rec);
}
static double driftp_impl(const ro_grid *g, const ro_species *sp, const ro_params *p,
                          const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift,
                          unsigned char *rec)
{
    const double DTs = p->dts, MDR = g->mdr, DPHI = g->dphi, BetaLim = p->betalim;
    double DtDriftP = 100000.0;
    const double OME = 7.3E-5;
#ifdef _OPENMP
#pragma omp parallel num_threads(g_inner) reduction(min : DtDriftP)
#endif
    {
    double *F = (double *)calloc((size_t)NT, sizeof(double));
    double *FBND = (double *)calloc((size_t)NT, sizeof(double));
    double *CD = (double *)calloc((size_t)NT, sizeof(double));
#define FF(n) F[(n)-1]
#define FB(n) FBND[(n)-1]
#define C(n) CD[(n)-1]
#ifdef _OPENMP
#pragma omp for collapse(2) schedule(static)
#endif
    for (int L = 1; L <= NPA; ++L)
        for (int K = 1; K <= NE; ++K)
            for (int I = 2; I <= NR; ++I) {
                for (int J = 1; J <= NT; ++J) FF(J) = F2(I, J, K, L);
                for (int J = 2; J <= NT; ++J) {
                    int J1 = J + 1;
                    if (J == NT) J1 = 2;
                    double GPA1 = FNIS(I, J, L) + FNIS(I, J1, L)
                                  + (FNIS(I + 1, J1, L) + FNIS(I + 1, J, L) - FNIS(I - 1, J, L) - FNIS(I - 1, J1, L))
                                  * RLZ(I) / 2. / MDR;
                    double GPA2 = RLZ(I) / 4. / MDR * (FNIS(I, J, L) + FNIS(I, J1, L) - 2 * FNHS(I, J, L) - 2 * FNHS(I, J1, L))
                                  * (BNES(I + 1, J1) + BNES(I + 1, J) - BNES(I - 1, J) - BNES(I - 1, J1))
                                  / (BNES(I, J) + BNES(I, J1));
                    C(J) = ((VT(I + 1, J) + VT(I + 1, J1) - VT(I - 1, J) - VT(I - 1, J1)) * P1(I)
                            - P2(I, K) * (GPA1 + GPA2) / (FNHS(I, J, L) + FNHS(I, J1, L))
                            - (EIR(I, J1) + EIR(I, J)) / RLZ(I) * DTs / DPHI)
                               / (BNES(I, J) + BNES(I, J1))
                           + OME * DTs / DPHI;
                    if (OUTSIDE(I, J) == 0) {
                        double ctemp = dmax(fabs(C(J)), 1E-10);
                        DtDriftP = dmin(DtDriftP, p->fraccfl * DTs / ctemp);
                    }
                    int s = 1;
                    if (C(J) < 0) s = -1;
                    double X = FF(J1) - FF(J);
                    double FUP = 0.5 * (FF(J) + FF(J1) - s * X);
                    int cs = 0;
                    if (fabs(X) <= 1.E-27) FB(J) = FUP;
                    if (fabs(X) > 1.E-27) {
                        int N = J + 1 - s;
                        if (N > NT) N = N - NT + 1;
                        double R = (FF(N) - FF(N - 1)) / X;
                        if (R <= 0) FB(J) = FUP;
                        if (R > 0) {
                            double LIM = limiter(BetaLim, R);
                            double CORR = -0.5 * (C(J) - s) * X;
                            FB(J) = FUP + LIM * CORR;
                            cs = limiter_case(BetaLim, R);
                        }
                    }
                    if (rec) rec[IX4(I, J, K, L)] = (unsigned char)cs;
                }
                C(1) = C(NT);
                FB(1) = FB(NT);
                if (rec) rec[IX4(I, 1, K, L)] = 0;
                for (int J = 2; J <= NT; ++J) {
                    F2(I, J, K, L) = F2(I, J, K, L) - C(J) * FB(J) + C(J - 1) * FB(J - 1);
                    if (F2(I, J, K, L) < 0) {
                        F2(I, J, K, L) = 1E-15;
                        if (rec) rec[IX4(I, J, K, L)] |= REC_CLIP;
                    }
                }
                F2(I, 1, K, L) = F2(I, NT, K, L);
                if (cdrift)
                    for (int J = 1; J <= NT; ++J) cdrift[IX4(I, J, K, L)] = C(J);
            }
#undef FF
#undef FB
#undef C
    free(F);
    free(FBND);
    free(CD);
    }
    return DtDriftP;
}

/* ------------------------------------------------------------------ DRIFTE */
static double drifte_impl(const ro_grid *g, const ro_species *sp, const ro_params *p,
                          const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift,
                          unsigned char *rec);
double ro_drifte(const ro_grid *g, const ro_species *sp, const ro_params *p,
                 const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift)
{
    return drifte_impl(g, sp, p, dp, vt, f2, cdrift, NULL);
}
double ro_drifte_rec(const ro_grid *g, const ro_species *sp, const ro_params *p,
                     const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift,
                     unsigned char *rec)
{
    return drifte_impl(g, sp, p, dp, vt, f2, cdrift, rec);
}
static double drifte_impl(const ro_grid *g, const ro_species *sp, const ro_params *p,
                          const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift,
                          unsigned char *rec)
{
    const double DTs = p->dts, MDR = g->mdr, DPHI = g->dphi, BetaLim = p->betalim;
    const int QS = sp->qs;
    double DtDriftE = 10000.0;
    const double OME = 7.3E-5;
    /* F(0:NE+2) -> F[0..NE+2] */
    double EZERO = EKEV(1) - WE(1);
    double GRZERO = 1. + EZERO * 1000. * Q / sp->rmas / CS / CS;
#ifdef _OPENMP
#pragma omp parallel num_threads(g_inner) reduction(min : DtDriftE)
#endif
    {
    double *F = (double *)calloc((size_t)NE + 3, sizeof(double));
    double *FBND = (double *)calloc((size_t)NE, sizeof(double));
    double *CD = (double *)calloc((size_t)NE, sizeof(double));
#define FF(n) F[(n)]
#define FB(n) FBND[(n)-1]
#define C(n) CD[(n)-1]
    FF(NE + 1) = 0.;
    FF(NE + 2) = 0.;
#ifdef _OPENMP
#pragma omp for collapse(2) schedule(static)
#endif
    for (int J = 1; J <= NT; ++J) {
        for (int I = 2; I <= NR; ++I) {
            int J0 = J - 1;
            if (J == 1) J0 = NT - 1;
            int J2 = J + 1;
            if (J == NT) J2 = 2;
            double DRD1 = (EIP(I, J) * RLZ(I) - (VT(I, J2) - VT(I, J0)) / 2. / DPHI) / BNES(I, J);
            double DPD1 = OME * RLZ(I) + ((VT(I + 1, J) - VT(I - 1, J)) / 2 / MDR - EIR(I, J)) / BNES(I, J);
            for (int L = 1; L <= NPA; ++L) {
                double GPA = (1. - FNIS(I, J, L) / 2. / FNHS(I, J, L)) / BNES(I, J);
                double GPR1 = GPA * (BNES(I + 1, J) - BNES(I - 1, J)) / 2. / MDR;
                double GPR2 = -FNIS(I, J, L) / FNHS(I, J, L) / RLZ(I);
                double GPR3 = -(FNIS(I + 1, J, L) - FNIS(I - 1, J, L)) / 2. / MDR / FNHS(I, J, L);
                double GPP1 = GPA * (BNES(I, J2) - BNES(I, J0)) / 2. / DPHI;
                double GPP2 = -(FNIS(I, J2, L) - FNIS(I, J0, L)) / 2. / DPHI / FNHS(I, J, L);
                double DRD2 = (FNIS(I, J2, L) - FNIS(I, J0, L)) / 2. / DPHI
                              + (FNIS(I, J, L) - 2 * FNHS(I, J, L)) * (BNES(I, J2) - BNES(I, J0)) / 4 / BNES(I, J) / DPHI;
                double DPD2 = FNIS(I, J, L) + (FNIS(I + 1, J, L) - FNIS(I - 1, J, L)) * RLZ(I) / 2 / MDR
                              + RLZ(I) * (FNIS(I, J, L) - 2 * FNHS(I, J, L)) / 4 / MDR * (BNES(I + 1, J) - BNES(I - 1, J)) / BNES(I, J);
                for (int K = 1; K <= NE; ++K) FF(K) = F2(I, J, K, L);
                FF(1) = FF(2) * GREL(1) / GREL(2) * sqrt((GREL(2) * GREL(2) - 1) / (GREL(1) * GREL(1) - 1));
                FF(0) = FF(1) * GRZERO / GREL(1) * sqrt((GREL(1) * GREL(1) - 1) / (GRZERO * GRZERO - 1));
                for (int K = 1; K <= NE; ++K) {
                    double EDT1 = EBND(K) * 1e3 * (GRBND(K) + 1) / 2 / GRBND(K) / FNHS(I, J, L) / RLZ(I) / BNES(I, J) / QS;
                    double DRDT = DRD1 + EDT1 * DRD2 * RLZ(I);
                    double DPDT = DPD1 - EDT1 * DPD2;
                    double dBdt1 = DBDT(I, J) * (1. - FNIS(I, J, L) / 2. / FNHS(I, J, L)) * RLZ(I) / BNES(I, J);
                    double dIdt1 = -DIDT(I, J, L) * RLZ(I) / FNHS(I, J, L);
                    C(K) = EDOT(I, K) * ((GPR1 + GPR2 + GPR3) * DRDT + (GPP1 + GPP2) * DPDT + dBdt1 + dIdt1);
                    if (OUTSIDE(I, J) == 0) {
                        double ctemp = dmax(fabs(C(K)), 1E-10);
                        DtDriftE = dmin(DtDriftE, p->fraccfl * DTs * DE(K) / ctemp);
                    }
                    int s = 1;
                    if (C(K) < 0) s = -1;
                    double X = FF(K + 1) - FF(K);
                    double FUP = 0.5 * (FF(K) + FF(K + 1) - s * X);
                    int cs = 0;
                    if (fabs(X) <= 1.E-27) FB(K) = FUP;
                    if (fabs(X) > 1.E-27) {
                        int N = K + 1 - s;
                        double R = (FF(N) - FF(N - 1)) / X;
                        if (R <= 0) FB(K) = FUP;
                        if (R > 0) {
                            double LIM = limiter(BetaLim, R);
                            double CORR = -0.5 * (C(K) / DE(K) - s) * X;
                            FB(K) = FUP + LIM * CORR;
                            cs = limiter_case(BetaLim, R);
                        }
                    }
                    if (rec) rec[IX4(I, J, K, L)] = (unsigned char)cs;
                }
                if (p->closed) {
                    FB(1) = 0.;
                    FB(NE) = 0.;
                }
                for (int K = 2; K <= NE; ++K) {
                    F2(I, J, K, L) = F2(I, J, K, L) - C(K) / WE(K) * FB(K) + C(K - 1) / WE(K) * FB(K - 1);
                    if (F2(I, J, K, L) < 0) {
                        F2(I, J, K, L) = 1E-15;
                        if (rec) rec[IX4(I, J, K, L)] |= REC_CLIP;
                    }
                }
                if (cdrift)
                    for (int K = 1; K <= NE; ++K) cdrift[IX4(I, J, K, L)] = C(K);
            }
        }
    }
#undef FF
#undef FB
#undef C
    free(F);
    free(FBND);
    free(CD);
    }
    return DtDriftE;
}

/* ----------------------------------------------------------------- DRIFTMU */
static double driftmu_impl(const ro_grid *g, const ro_species *sp, const ro_params *p,
                           const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift,
                           unsigned char *rec);
double ro_driftmu(const ro_grid *g, const ro_species *sp, const ro_params *p,
                  const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift)
{
    return driftmu_impl(g, sp, p, dp, vt, f2, cdrift, NULL);
}
double ro_driftmu_rec(const ro_grid *g, const ro_species *sp, const ro_params *p,
                      const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift,
                      unsigned char *rec)
{
    return driftmu_impl(g, sp, p, dp, vt, f2, cdrift, rec);
}
static double driftmu_impl(const ro_grid *g, const ro_species *sp, const ro_params *p,
                           const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift,
                           unsigned char *rec)
{
    const double DTs = p->dts, MDR = g->mdr, DPHI = g->dphi, BetaLim = p->betalim;
    const int QS = sp->qs;
    double DtDriftMu = 10000.0;
    const double OME = 7.3E-5;
#ifdef _OPENMP
#pragma omp parallel num_threads(g_inner) reduction(min : DtDriftMu)
#endif
    {
    double *F = (double *)calloc((size_t)NPA, sizeof(double));
    double *FBND = (double *)calloc((size_t)NPA, sizeof(double));
    double *CD = (double *)calloc((size_t)NPA, sizeof(double));
#define FF(n) F[(n)-1]
#define FB(n) FBND[(n)-1]
#define C(n) CD[(n)-1]
#ifdef _OPENMP
#pragma omp for collapse(2) schedule(static)
#endif
    for (int K = 1; K <= NE; ++K)
        for (int J = 1; J <= NT; ++J) {
            for (int I = 2; I <= NR; ++I) {
                int J0 = J - 1;
                if (J == 1) J0 = NT - 1;
                int J1 = J + 1;
                if (J == NT) J1 = 2;
                for (int L = 1; L <= NPA; ++L) FF(L) = F2(I, J, K, L);
                FF(1) = FF(2);
                double DRM1 = (EIP(I, J) * RLZ(I) - (VT(I, J1) - VT(I, J0)) / 2 / DPHI) / BNES(I, J);
                double DPM1 = OME * RLZ(I) + ((VT(I + 1, J) - VT(I - 1, J)) / 2 / MDR - EIR(I, J)) / BNES(I, J);
                for (int L = 2; L <= NPA; ++L) {
                    double CMUDOT = MUDOT(I, L) * BOUNIS(I, J, L) / BOUNHS(I, J, L);
                    double GMR1 = (BNES(I + 1, J) - BNES(I - 1, J)) / 4 / MDR / BNES(I, J);
                    double GMR2 = 1 / RLZ(I);
                    double GMR3 = (BOUNIS(I + 1, J, L) - BOUNIS(I - 1, J, L)) / 2 / MDR / BOUNIS(I, J, L);
                    double GMP1 = (BNES(I, J1) - BNES(I, J0)) / 4 / DPHI / BNES(I, J);
                    double GMP2 = (BOUNIS(I, J1, L) - BOUNIS(I, J0, L)) / 2 / DPHI / BOUNIS(I, J, L);
                    double EDT = EKEV(K) * 1e3 * (GREL(K) + 1) / 2 / GREL(K) / BOUNHS(I, J, L) / RLZ(I) / BNES(I, J) / QS;
                    double DRM2 = (BOUNIS(I, J1, L) - BOUNIS(I, J0, L)) / 2 / DPHI
                                  + (BOUNIS(I, J, L) - 2 * BOUNHS(I, J, L)) * (BNES(I, J1) - BNES(I, J0)) / 4 / BNES(I, J) / DPHI;
                    double DPM2 = BOUNIS(I, J, L) + (BOUNIS(I + 1, J, L) - BOUNIS(I - 1, J, L)) * RLZ(I) / 2 / MDR
                                  + (BOUNIS(I, J, L) - 2 * BOUNHS(I, J, L)) * RLZ(I) / 4 / MDR * (BNES(I + 1, J) - BNES(I - 1, J)) / BNES(I, J);
                    double DRDM = DRM1 + EDT * DRM2 * RLZ(I);
                    double DPDM = DPM1 - EDT * DPM2;
                    double dBdt2 = DBDT(I, J) / 2. / BNES(I, J) * RLZ(I);
                    double dIbndt2 = DIBNDT(I, J, L) * RLZ(I) / BOUNIS(I, J, L);
                    C(L) = -CMUDOT * ((GMR1 + GMR2 + GMR3) * DRDM + (GMP1 + GMP2) * DPDM + dBdt2 + dIbndt2);
                    if (OUTSIDE(I, J) == 0) {
                        double ctemp = dmax(fabs(C(L)), 1E-32);
                        DtDriftMu = dmin(DtDriftMu, p->fraccfl * DTs * DMU(L) / ctemp);
                    }
                    int s = 1;
                    if (C(L) < 0.0) s = -1;
                    if (rec) rec[IX4(I, J, K, L)] = 0;
                    if (L <= NPA - 2) {
                        double X = FF(L + 1) - FF(L);
                        double FUP = 0.5 * (FF(L) + FF(L + 1) - s * X);
                        if (fabs(X) <= 1.E-27) FB(L) = FUP;
                        if (fabs(X) > 1.E-27) {
                            int N = L + 1 - s;
                            double R = (FF(N) - FF(N - 1)) / X;
                            if (R <= 0) FB(L) = FUP;
                            if (R > 0) {
                                double LIM = limiter(BetaLim, R);
                                double CORR = -0.5 * (C(L) / DMU(L) - s) * X;
                                FB(L) = FUP + LIM * CORR;
                                if (rec) rec[IX4(I, J, K, L)] = (unsigned char)limiter_case(BetaLim, R);
                            }
                        }
                    }
                }
                C(1) = 0.;
                FB(1) = 0.;
                FB(NPA - 1) = FF(NPA);
                if (p->closed) FB(NPA - 1) = 0.;
                for (int L = 2; L <= NPA - 1; ++L) {
                    F2(I, J, K, L) = F2(I, J, K, L) - C(L) / WMU(L) * FB(L) + C(L - 1) / WMU(L) * FB(L - 1);
                    if (F2(I, J, K, L) < 0) {
                        F2(I, J, K, L) = 1E-15;
                        if (rec) rec[IX4(I, J, K, L)] |= REC_CLIP;
                    }
                }
                F2(I, J, K, NPA) = F2(I, J, K, NPA - 1) * FNHS(I, J, NPA) * MU(NPA) / FNHS(I, J, NPA - 1) / MU(NPA - 1);
                if (cdrift)
                    for (int L = 1; L <= NPA; ++L) cdrift[IX4(I, J, K, L)] = C(L);
            }
        }
#undef FF
#undef FB
#undef C
    free(F);
    free(FBND);
    free(CD);
    }
    return DtDriftMu;
}

/* ------------------------------------------------------------------ CEPARA */
void ro_cepara(const ro_grid *g, const ro_species *sp, const ro_params *p, double *charge, double *atlos)
{
    const double DTs = p->dts;
    size_t n = (size_t)NR * NT * NE * NPA;
    for (size_t i = 0; i < n; ++i) charge[i] = 1.;
    if (sp->cex_kind >= 1 && sp->cex_kind <= 3) {
#ifdef _OPENMP
#pragma omp parallel for collapse(2) num_threads(g_inner) schedule(static)
#endif
        for (int L = 2; L <= NPA; ++L)
            for (int K = 2; K <= NE; ++K)
                for (int I = 2; I <= NR; ++I)
                    for (int J = 1; J <= NT; ++J) {
                        double X = log10(EKEV(K));
                        if (X < -2.) X = -2.;
                        double X2 = X * X, X3 = X2 * X, X4 = X2 * X2, Y;
                        if (sp->cex_kind == 1)
                            Y = -18.767 - 0.11017 * X - 3.8173e-2 * X2 - 0.1232 * X3 - 5.0488e-2 * X4;
                        else if (sp->cex_kind == 2)
                            Y = -20.789 + 0.92316 * X - 0.68017 * X2 + 0.66153 * X3 - 0.20998 * X4;
                        else
                            Y = -18.987 - 0.10613 * X - 5.4841E-3 * X2 - 1.6262E-2 * X3 - 7.0554E-3 * X4;
                        double ALPHA = pow(10., Y) * VV(K) * HDNS(I, J, L) * DTs;
                        charge[IX4(I, J, K, L)] = exp(-ALPHA);
                    }
    }
    for (int K = 2; K <= NE; ++K)
        for (int I = 2; I <= NR; ++I) {
            double TAUB = 2 * RLZ(I) / VV(K);
            atlos[IXRK(I, K)] = exp(-DTs / TAUB);
        }
}

void ro_charexchange(const ro_grid *g, double *f2, const double *charge)
{
#ifdef _OPENMP
#pragma omp parallel for num_threads(g_inner) schedule(static)
#endif
    for (int K = 2; K <= NE; ++K)
        for (int J = 1; J <= NT; ++J)
            for (int I = 2; I <= NR; ++I)
                for (int L = 2; L <= NPA; ++L) F2(I, J, K, L) = F2(I, J, K, L) * charge[IX4(I, J, K, L)];
}

void ro_atmol(const ro_grid *g, double *f2, const double *atlos)
{
#ifdef _OPENMP
#pragma omp parallel for num_threads(g_inner) schedule(static)
#endif
    for (int K = 2; K <= NE; ++K)
        for (int J = 1; J <= NT; ++J)
            for (int I = 2; I <= NR; ++I) {
                int u = (int)UPA(I);
                for (int L = u; L <= NPA; ++L)
                    F2(I, J, K, L) = F2(I, J, K, L) * pow(atlos[IXRK(I, K)], 1 / FNHS(I, J, L));
            }
}

double ro_sumrc(const ro_grid *g, const double *f2)
{
    double setrc = 0.;
    for (int I = 2; I <= NR; ++I)
        for (int K = 2; K <= NE; ++K)
            for (int L = 2; L <= NPA; ++L)
                for (int J = 1; J <= NT - 1; ++J) {
                    double WEIGHT = F2(I, J, K, L) * WE(K) * WMU(L);
                    setrc = setrc + EKEV(K) * WEIGHT;
                }
    return setrc;
}

void ro_anisch(const ro_grid *g, const ro_species *sp, double *f2, double *ppert, double *ppart)
{
    const double cv = CS * 100;
    const double RFAC = 4 * PI / cv;
    int khi[5] = {6, 10, 25, 30, 35};
    khi[4] = NE;
#ifdef _OPENMP
#pragma omp parallel for collapse(2) num_threads(g_inner) schedule(static)
#endif
    for (int I = 2; I <= NR; ++I)
        for (int J = 1; J <= NT; ++J) {
            int klo = 2;
            double PPERT = 0., PPART = 0.;
            for (int iwa = 0; iwa < 5; ++iwa) {
                double PPER = 0., PPAR = 0., RNHT = 0., EDEN = 0.;
                for (int K = klo; K <= khi[iwa]; ++K) {
                    F2(I, J, K, 1) = F2(I, J, K, 2);
                    double SUME = 0., SUMA = 0., SUMN = 0.;
                    int u = (int)(UPA(I) - 1);
                    for (int L = 1; L <= u; ++L) {
                        double ERNM = WMU(L) / FFACTOR(I, K, L) / FNHS(I, J, L);
                        double EPMA = ERNM * MU(L) * MU(L);
                        double EPME = ERNM - EPMA;
                        SUME = SUME + F2(I, J, K, L) * EPME;
                        SUMA = SUMA + F2(I, J, K, L) * EPMA;
                        SUMN = SUMN + F2(I, J, K, L) * ERNM;
                    }
                    PPER = PPER + EPP(K) * SUME;
                    PPAR = PPAR + EPP(K) * SUMA;
                    RNHT = RNHT + ERNH(K) * SUMN;
                    EDEN = EDEN + ERNH(K) * EKEV(K) * SUMN;
                }
                PPAR = 2 * RFAC * PPAR;
                PPER = RFAC * PPER;
                klo = khi[iwa] + 1;
                PPERT = PPERT + PPER;
                PPART = PPART + PPAR;
            }
            if (ppert) ppert[IXM(I, J)] = PPERT;
            if (ppart) ppart[IXM(I, J)] = PPART;
        }
}

void ro_flux(const ro_grid *g, const ro_species *sp, const double *f2, double *flux)
{
#ifdef _OPENMP
#pragma omp parallel for num_threads(g_inner) schedule(static)
#endif
    for (int I = 2; I <= NR; ++I)
        for (int K = 2; K <= NE; ++K)
            for (int L = 2; L <= NPA; ++L)
                for (int J = 1; J <= NT - 1; ++J)
                    flux[IX4(I, J, K, L)] = F2(I, J, K, L) / FFACTOR(I, K, L) / FNHS(I, J, L);
}

static void alloc_dp(const ro_grid *g, ro_driftpara_t *dp)
{
    dp->vr = (double *)calloc((size_t)NR, sizeof(double));
    dp->p1 = (double *)calloc((size_t)NR, sizeof(double));
    dp->p2 = (double *)calloc((size_t)NR * NE, sizeof(double));
    dp->edot = (double *)calloc((size_t)NR * NE, sizeof(double));
    dp->mudot = (double *)calloc((size_t)NR * NPA, sizeof(double));
}
static void free_dp(ro_driftpara_t *dp)
{
    free(dp->vr);
    free(dp->p1);
    free(dp->p2);
    free(dp->edot);
    free(dp->mudot);
}

void ro_half_step(const ro_grid *g, const ro_species *sp, const ro_params *p,
                  const ro_driftpara_t *dp, const double *vt, const double *fgeos,
                  const double *charge, const double *atlos, double *f2, int order)
{
    if (order == 0) {
        ro_driftr(g, sp, p, dp, vt, fgeos, f2, NULL);
        ro_driftp(g, sp, p, dp, vt, f2, NULL);
        ro_drifte(g, sp, p, dp, vt, f2, NULL);
        ro_driftmu(g, sp, p, dp, vt, f2, NULL);
        if (sp->cex_kind) ro_charexchange(g, f2, charge);
        if (p->do_atmol) ro_atmol(g, f2, atlos);
    } else {
        if (p->do_atmol) ro_atmol(g, f2, atlos);
        if (sp->cex_kind) ro_charexchange(g, f2, charge);
        ro_driftmu(g, sp, p, dp, vt, f2, NULL);
        ro_drifte(g, sp, p, dp, vt, f2, NULL);
        ro_driftp(g, sp, p, dp, vt, f2, NULL);
        ro_driftr(g, sp, p, dp, vt, fgeos, f2, NULL);
    }
}

int ro_ram_run(const ro_grid *g, int ns, const ro_species *sp_all, const ro_params *p,
               double kp, const double *vt_in, double *vt_out,
               const double *const *fgeos, double *const *f2s,
               double *const *ppert, double *const *ppart, double *const *flux,
               ro_losses *losses, double *dts_next, int nthreads)
{
    return ro_ram_run2(g, ns, sp_all, p, kp, vt_in, vt_out, fgeos, f2s, ppert, ppart, flux, losses,
                       dts_next, nthreads, NULL);
}

void ro_padif(const ro_grid *g, const ro_params *p, const double *daa, double *f2);

int ro_ram_run2(const ro_grid *g, int ns, const ro_species *sp_all, const ro_params *p,
                double kp, const double *vt_in, double *vt_out,
                const double *const *fgeos, double *const *f2s,
                double *const *ppert, double *const *ppart, double *const *flux,
                ro_losses *losses, double *dts_next, int nthreads, const double *const *daa)
{
    size_t nvt = (size_t)(NR + 1) * NT;
    double *vt = (double *)malloc(sizeof(double) * nvt);
    if (vt_in)
        memcpy(vt, vt_in, sizeof(double) * nvt);
    else
        ro_vt_vols(g, kp, vt);
    if (vt_out) memcpy(vt_out, vt, sizeof(double) * nvt);

    double *dtr = (double *)malloc(sizeof(double) * ns * 4);
    size_t ncell = (size_t)NR * NT * NE * NPA;
#ifdef _OPENMP
    if (nthreads < 1) nthreads = 1;
    if (g_inner > 1 && nthreads > 1) omp_set_max_active_levels(2);
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1)
#endif
    for (int iS = 0; iS < ns; ++iS) {
        const ro_species *sp = &sp_all[iS];
        double *f2 = f2s[iS];
        double *charge = (double *)malloc(sizeof(double) * ncell);
        double *atlos = (double *)calloc((size_t)NR * NE, sizeof(double));
        ro_driftpara_t dpv;
        ro_driftpara_t *dp = &dpv;
        alloc_dp(g, dp);
        ro_cepara(g, sp, p, charge, atlos);
        ro_driftpara(g, sp, p, dp);
        double setrc = losses ? losses[iS].setrc : 0., s1;
        double lsdr = 0., lscha = 0., lsatm = 0., lswae = 0.;
        /* forward half */
        dtr[iS * 4 + 0] = ro_driftr(g, sp, p, dp, vt, fgeos[iS], f2, NULL);
        dtr[iS * 4 + 1] = ro_driftp(g, sp, p, dp, vt, f2, NULL);
        dtr[iS * 4 + 2] = ro_drifte(g, sp, p, dp, vt, f2, NULL);
        dtr[iS * 4 + 3] = ro_driftmu(g, sp, p, dp, vt, f2, NULL);
        s1 = ro_sumrc(g, f2); lsdr += setrc - s1; setrc = s1;
        const double *dps = daa ? daa[iS] : NULL;
        if (dps) { /* WPADIF after the drifts (src/ModRamRun.f90:91-107) */
            ro_padif(g, p, dps, f2);
            s1 = ro_sumrc(g, f2); lswae += setrc - s1; setrc = s1;
        }
        if (sp->cex_kind) {
            ro_charexchange(g, f2, charge);
            s1 = ro_sumrc(g, f2); lscha += setrc - s1; setrc = s1;
        }
        if (p->do_atmol) {
            ro_atmol(g, f2, atlos);
            s1 = ro_sumrc(g, f2); lsatm += setrc - s1; setrc = s1;
            /* reverse half */
            ro_atmol(g, f2, atlos);
            s1 = ro_sumrc(g, f2); lsatm += setrc - s1; setrc = s1;
        }
        if (sp->cex_kind) {
            ro_charexchange(g, f2, charge);
            s1 = ro_sumrc(g, f2); lscha += setrc - s1; setrc = s1;
        }
        if (dps) { /* and before the reverse drifts (src/ModRamRun.f90:144-158) */
            ro_padif(g, p, dps, f2);
            s1 = ro_sumrc(g, f2); lswae += setrc - s1; setrc = s1;
        }
        ro_driftmu(g, sp, p, dp, vt, f2, NULL);
        ro_drifte(g, sp, p, dp, vt, f2, NULL);
        ro_driftp(g, sp, p, dp, vt, f2, NULL);
        ro_driftr(g, sp, p, dp, vt, fgeos[iS], f2, NULL);
        s1 = ro_sumrc(g, f2); lsdr += setrc - s1; setrc = s1;
        if (losses) {
            losses[iS].setrc = setrc;
            losses[iS].lsdr += lsdr;
            losses[iS].lscha += lscha;
            losses[iS].lsatm += lsatm;
            losses[iS].lswae += lswae;
        }
        free_dp(dp);
        free(charge);
        free(atlos);
    }
    /* periodic copy F2(:,:,NT,:,:) = F2(:,:,1,:,:) and magnetopause mask */
    for (int iS = 0; iS < ns; ++iS) {
        double *f2 = f2s[iS];
        for (int L = 1; L <= NPA; ++L)
            for (int K = 1; K <= NE; ++K)
                for (int I = 1; I <= NR; ++I) F2(I, NT, K, L) = F2(I, 1, K, L);
        for (int I = 1; I <= NR; ++I)
            for (int J = 1; J <= NT; ++J)
                if (OUTSIDE(I, J) == 1)
                    for (int L = 1; L <= NPA; ++L)
                        for (int K = 1; K <= NE; ++K) F2(I, J, K, L) = 1.e-31;
    }
    double dn = 1e300;
    for (int i = 0; i < ns * 4; ++i) dn = dmin(dn, dtr[i]);
    if (ns == 0) dn = p->dtsmin;
    if (dts_next) *dts_next = dmax(dn, p->dtsmin);
    for (int iS = 0; iS < ns; ++iS) {
        ro_anisch(g, &sp_all[iS], f2s[iS], ppert ? ppert[iS] : NULL, ppart ? ppart[iS] : NULL);
        if (flux && flux[iS]) ro_flux(g, &sp_all[iS], f2s[iS], flux[iS]);
    }
    free(dtr);
    free(vt);
    (void)HMIN_UNUSED;
    return 0;
}

/* ==================================================================== adjoint
 * Scalar adjoint of the frozen-limiter scheme.  The forward sweeps are run
 * through the *_rec variants, which record per face the limiter case of
 * MAX(MIN(BetaLim*R,1.),MIN(R,BetaLim)) (0: upwind only, 1: BetaLim*R,
 * 2: 1, 3: R, 4: BetaLim) and REC_CLIP when the updated cell was clipped,
 * and (DRIFTR) per line the FGEOS index that F(NR+1) came from.  With those
 * frozen, each line update is linear in F:
 *   FUP = 0.5*(F(I)+F(I+1)-s*X)     -> weights 0.5*(1+s), 0.5*(1-s)
 *   LIMITER*CORR = a * (LIMITER*X),  a = -0.5*(C[/DE|/DMU] - s),
 *   LIMITER*X = BetaLim*D | X | D | BetaLim*X,  D = F(N)-F(N-1), N = I+1-s,
 * and the functions below apply its transpose to lam (in place). */

static void adj_face(double *Gb, int I, int I1, int N, int s, int cs, double a, double FBb,
                     double beta)
{
    Gb[I] += 0.5 * (1 + s) * FBb;
    Gb[I1] += 0.5 * (1 - s) * FBb;
    if (!cs) return;
    double Lb = a * FBb;
    switch (cs) {
    case 1: Gb[N] += beta * Lb; Gb[N - 1] -= beta * Lb; break;
    case 2: Gb[I1] += Lb; Gb[I] -= Lb; break;
    case 3: Gb[N] += Lb; Gb[N - 1] -= Lb; break;
    default: Gb[I1] += beta * Lb; Gb[I] -= beta * Lb; break;
    }
}

void ro_driftr_adj(const ro_grid *g, const ro_params *p, const double *cd, const unsigned char *rec,
                   const int *gsrc, double *lam, double *gfgeos)
{
    const double beta = p->betalim;
    double *Gb = (double *)malloc(sizeof(double) * (NR + 3));
    double *Pb = (double *)malloc(sizeof(double) * (NR + 1));
    for (int K = 1; K <= NE; ++K)
        for (int L = 1; L <= NPA; ++L)
            for (int J = 1; J <= NT; ++J) {
                for (int i = 0; i <= NR + 2; ++i) Gb[i] = 0.;
                for (int i = 0; i <= NR; ++i) Pb[i] = 0.;
#define CC(I) cd[IX4(I, J, K, L)]
#define RC(I) rec[IX4(I, J, K, L)]
                const int inflow = CC(NR) < 0;
                Gb[1] = lam[IX4(1, J, K, L)];
                for (int I = 2; I <= NR; ++I) {
                    double le = (RC(I) & REC_CLIP) ? 0. : lam[IX4(I, J, K, L)];
                    Gb[I] += le;       /* F2new(I) = F2(I) - C(I)FB(I) + C(I-1)FB(I-1) */
                    Pb[I] -= le;
                    Pb[I - 1] += le;
                }
                if (inflow && !p->closed) Gb[2] += CC(1) * Pb[1]; /* FBND(1) = F(2) */
                int UR = inflow ? NR : NR - 1;
                for (int I = 2; I <= UR; ++I) {
                    if (p->closed && I == NR) continue;
                    int s = CC(I) < 0 ? -1 : 1;
                    adj_face(Gb, I, I + 1, I + 1 - s, s, RC(I) & 7, -0.5 * (CC(I) - s), CC(I) * Pb[I], beta);
                }
                if (!inflow && !p->closed) Gb[NR] += CC(NR) * Pb[NR]; /* FBND(NR) = F(NR) */
                int src = gsrc[IXG(J, K, L)];
                if (src >= 0) {
                    int jj = src % NT + 1, ll = src / (NT * NE) + 1;
                    gfgeos[src] += g->conf1 * FNHS(NR, jj, ll) * Gb[NR + 1];
                    if (inflow) gfgeos[src] += g->conf2 * FNHS(NR, jj, ll) * Gb[NR + 2];
                }
                for (int I = 1; I <= NR; ++I) lam[IX4(I, J, K, L)] = Gb[I];
#undef CC
#undef RC
            }
    free(Gb);
    free(Pb);
}

void ro_driftp_adj(const ro_grid *g, const ro_params *p, const double *cd, const unsigned char *rec,
                   double *lam)
{
    const double beta = p->betalim;
    double *Gb = (double *)malloc(sizeof(double) * (NT + 3));
    double *Pb = (double *)malloc(sizeof(double) * (NT + 1));
    double *lv = (double *)malloc(sizeof(double) * (NT + 1));
    for (int L = 1; L <= NPA; ++L)
        for (int K = 1; K <= NE; ++K)
            for (int I = 2; I <= NR; ++I) {
#define CC(J) cd[IX4(I, J, K, L)]
#define RC(J) rec[IX4(I, J, K, L)]
                for (int J = 0; J <= NT + 2; ++J) Gb[J] = 0.;
                for (int J = 0; J <= NT; ++J) Pb[J] = 0.;
                for (int J = 1; J <= NT; ++J) lv[J] = lam[IX4(I, J, K, L)];
                lv[NT] += lv[1]; /* F2(I,1) = F2new(I,NT) */
                lv[1] = 0.;
                for (int J = 2; J <= NT; ++J) {
                    double le = (RC(J) & REC_CLIP) ? 0. : lv[J];
                    Gb[J] += le;
                    Pb[J] -= le;
                    Pb[J - 1] += le;
                }
                Pb[NT] += Pb[1]; /* FBND(1) = FBND(NT), CDriftP(1) = CDriftP(NT) */
                for (int J = 2; J <= NT; ++J) {
                    int s = CC(J) < 0 ? -1 : 1;
                    int J1 = (J == NT) ? 2 : J + 1;
                    int N = J + 1 - s;
                    if (N > NT) N = N - NT + 1;
                    adj_face(Gb, J, J1, N, s, RC(J) & 7, -0.5 * (CC(J) - s), CC(J) * Pb[J], beta);
                }
                for (int J = 1; J <= NT; ++J) lam[IX4(I, J, K, L)] = Gb[J];
#undef CC
#undef RC
            }
    free(Gb);
    free(Pb);
    free(lv);
}

void ro_drifte_adj(const ro_grid *g, const ro_species *sp, const ro_params *p, const double *cd,
                   const unsigned char *rec, double *lam)
{
    const double beta = p->betalim;
    double *Gb = (double *)malloc(sizeof(double) * (NE + 3)); /* F(0:NE+2) */
    double *FBb = (double *)malloc(sizeof(double) * (NE + 1));
    const double EZERO = EKEV(1) - WE(1);
    const double GRZERO = 1. + EZERO * 1000. * Q / sp->rmas / CS / CS;
    /* F(1) = F(2)*k1, F(0) = F(1)*k0 (src/ModRamDrift.f90:334-335) */
    const double k1 = GREL(1) / GREL(2) * sqrt((GREL(2) * GREL(2) - 1) / (GREL(1) * GREL(1) - 1));
    const double k0 = GRZERO / GREL(1) * sqrt((GREL(1) * GREL(1) - 1) / (GRZERO * GRZERO - 1));
    for (int J = 1; J <= NT; ++J)
        for (int I = 2; I <= NR; ++I)
            for (int L = 1; L <= NPA; ++L) {
#define CC(K) cd[IX4(I, J, K, L)]
#define RC(K) rec[IX4(I, J, K, L)]
                for (int K = 0; K <= NE + 2; ++K) Gb[K] = 0.;
                for (int K = 0; K <= NE; ++K) FBb[K] = 0.;
                double out1 = lam[IX4(I, J, 1, L)];
                for (int K = 2; K <= NE; ++K) {
                    double le = (RC(K) & REC_CLIP) ? 0. : lam[IX4(I, J, K, L)];
                    Gb[K] += le; /* F2 - C(K)/WE(K)*FB(K) + C(K-1)/WE(K)*FB(K-1) */
                    FBb[K] -= CC(K) / WE(K) * le;
                    FBb[K - 1] += CC(K - 1) / WE(K) * le;
                }
                for (int K = 1; K <= NE; ++K) {
                    if (p->closed && (K == 1 || K == NE)) continue;
                    int s = CC(K) < 0 ? -1 : 1;
                    adj_face(Gb, K, K + 1, K + 1 - s, s, RC(K) & 7, -0.5 * (CC(K) / DE(K) - s), FBb[K], beta);
                }
                double g1 = Gb[1] + k0 * Gb[0];
                lam[IX4(I, J, 1, L)] = out1;
                lam[IX4(I, J, 2, L)] = Gb[2] + k1 * g1;
                for (int K = 3; K <= NE; ++K) lam[IX4(I, J, K, L)] = Gb[K];
#undef CC
#undef RC
            }
    free(Gb);
    free(FBb);
}

void ro_driftmu_adj(const ro_grid *g, const ro_params *p, const double *cd, const unsigned char *rec,
                    double *lam)
{
    const double beta = p->betalim;
    double *Gb = (double *)malloc(sizeof(double) * (NPA + 3));
    double *FBb = (double *)malloc(sizeof(double) * (NPA + 1));
    double *lv = (double *)malloc(sizeof(double) * (NPA + 1));
    for (int K = 1; K <= NE; ++K)
        for (int J = 1; J <= NT; ++J)
            for (int I = 2; I <= NR; ++I) {
#define CC(L) cd[IX4(I, J, K, L)]
#define RC(L) rec[IX4(I, J, K, L)]
                for (int L = 0; L <= NPA + 2; ++L) Gb[L] = 0.;
                for (int L = 0; L <= NPA; ++L) FBb[L] = 0.;
                for (int L = 1; L <= NPA; ++L) lv[L] = lam[IX4(I, J, K, L)];
                /* F2(NPA) = F2new(NPA-1)*FNHS(NPA)*MU(NPA)/FNHS(NPA-1)/MU(NPA-1) */
                double rho = 1.0 * FNHS(I, J, NPA) * MU(NPA) / FNHS(I, J, NPA - 1) / MU(NPA - 1);
                lv[NPA - 1] += rho * lv[NPA];
                lv[NPA] = 0.;
                double out1 = lv[1];
                for (int L = 2; L <= NPA - 1; ++L) {
                    double le = (RC(L) & REC_CLIP) ? 0. : lv[L];
                    Gb[L] += le;
                    FBb[L] -= CC(L) / WMU(L) * le;
                    FBb[L - 1] += CC(L - 1) / WMU(L) * le;
                }
                for (int L = 2; L <= NPA - 2; ++L) {
                    int s = CC(L) < 0.0 ? -1 : 1;
                    adj_face(Gb, L, L + 1, L + 1 - s, s, RC(L) & 7, -0.5 * (CC(L) / DMU(L) - s), FBb[L], beta);
                }
                if (!p->closed) Gb[NPA] += FBb[NPA - 1]; /* FBND(NPA-1) = F(NPA) */
                Gb[2] += Gb[1];                           /* F(1) = F(2) */
                lam[IX4(I, J, K, 1)] = out1;
                for (int L = 2; L <= NPA; ++L) lam[IX4(I, J, K, L)] = Gb[L];
#undef CC
#undef RC
            }
    free(Gb);
    free(FBb);
    free(lv);
}

/* ---------------------------------------------------- implicit PA diffusion
 * WPADIF (src/ModRamWPI.f90:643-714) and FLCscatter (src/ModRamLoss.f90:
 * 512-575) share one implicit scheme; daa is their coefficient, D(I,J,K,L):
 * ATAW+ATAC for electrons, ATAW_emic_h+ATAW_emic_he for EMIC, FLC_coef(S,..)
 * for FLC.  The diagnostic file written when a row is not diagonally
 * dominant is left out. */
void ro_padif(const ro_grid *g, const ro_params *p, const double *daa, double *f2)
{
    const double DTs = p->dts;
#ifdef _OPENMP
#pragma omp parallel num_threads(g_inner)
#endif
    {
        double *F = (double *)calloc((size_t)NPA + 1, sizeof(double));
        double *RK = (double *)calloc((size_t)NPA + 1, sizeof(double));
        double *RL = (double *)calloc((size_t)NPA + 1, sizeof(double));
        double *FACMU = (double *)calloc((size_t)NPA + 1, sizeof(double));
#define D(I, J, K, L) daa[IX4(I, J, K, L)]
#ifdef _OPENMP
#pragma omp for collapse(2) schedule(static)
#endif
        for (int J = 1; J <= NT; ++J)
            for (int I = 2; I <= NR; ++I)
                for (int K = 2; K <= NE; ++K) {
                    for (int L = 2; L <= NPA; ++L) {
                        FACMU[L] = FNHS(I, J, L) * MU(L);
                        F[L] = F2(I, J, K, L) / FACMU[L];
                    }
                    FACMU[1] = FNHS(I, J, 1) * MU(1);
                    F[1] = F[2];
                    RK[1] = 0.;
                    RL[1] = -1.;
                    for (int L = 2; L <= NPA - 1; ++L) {
                        double AN = D(I, J, K, L) / DMU(L);
                        double GN = D(I, J, K, L - 1) / DMU(L - 1);
                        AN = AN * DTs / FACMU[L] / WMU(L);
                        GN = GN * DTs / FACMU[L] / WMU(L);
                        double BN = AN + GN;
                        double RP = F[L];
                        double DENOM = BN + GN * RL[L - 1] + 1;
                        RK[L] = (RP + GN * RK[L - 1]) / DENOM;
                        RL[L] = -AN / DENOM;
                    }
                    F2(I, J, K, NPA - 1) = RK[NPA - 1] / (1 + RL[NPA - 1]);
                    for (int L = NPA - 2; L >= 1; --L) F2(I, J, K, L) = RK[L] - RL[L] * F2(I, J, K, L + 1);
                    F2(I, J, K, NPA) = F2(I, J, K, NPA - 1);
                    for (int L = 1; L <= NPA; ++L) F2(I, J, K, L) = F2(I, J, K, L) * FACMU[L];
                }
#undef D
        free(F);
        free(RK);
        free(RL);
        free(FACMU);
    }
}

/* ------------------------------------------------------------ computehI
 * Bounce integrals of computehI (src/ModRamScb.f90:378-406) with
 * integrator_c and bounceaverage_c (src/RamGSL.c:452-606).  The reference
 * integrates, with GSL cquad at 1e-3 tolerance, integrands built on the
 * LINEAR interpolant of B (and of the density) between the field-line
 * nodes (integral_interpolate, src/RamGSL.c:295-322); here those same
 * integrals are evaluated exactly, segment by segment, in closed form:
 * with u = Bm - B linear on a segment, a = sqrt(u0), b = sqrt(u1),
 *   int sqrt(u) = (2/3) dchi (a^2+ab+b^2)/(a+b),  int 1/sqrt(u) = 2 dchi/(a+b),
 *   int (n0 + dn t)/sqrt(u) = dchi (n0 H1 + dn H2), H1 = 2/(a+b),
 *   H2 = 2(b+2a)/(3(a+b)^2),
 * and the part of a segment where B >= Bm (integrand 0) cut off at u = 0. */
static void seg_integrals(double c0, double c1, double B0, double B1, double n0, double n1, double bm,
                          double *yi, double *yh, double *yd)
{
    double u0 = bm - B0, u1 = bm - B1, dchi = c1 - c0;
    if (u0 <= 0 && u1 <= 0) return;
    double a, b, na, nb, w;
    if (u0 > 0 && u1 > 0) {
        a = sqrt(u0); b = sqrt(u1); na = n0; nb = n1; w = dchi;
    } else if (u0 > 0) { /* positive from the segment start to u = 0 */
        double f = u0 / (u0 - u1);
        a = sqrt(u0); b = 0.; na = n0; nb = n0 + (n1 - n0) * f; w = dchi * f;
    } else {             /* positive from u = 0 to the segment end */
        double f = u1 / (u1 - u0);
        a = 0.; b = sqrt(u1); na = n1 + (n0 - n1) * f; nb = n1; w = dchi * f;
    }
    double s = a + b;
    *yi += (2. / 3.) * w * (a * a + a * b + b * b) / s;
    *yh += 2. * w / s;
    if (yd) *yd += w * (na * (2. / s) + (nb - na) * (2. * (b + 2. * a) / (3. * s * s)));
}

static void line_integrals(int nthe, const double *chi, const double *bf, const double *var, double bm,
                           int i0, int i1, double *yi, double *yh, double *yd)
{
    *yi = 0.; *yh = 0.;
    if (yd) *yd = 0.;
    for (int k = i0; k < i1; ++k)
        seg_integrals(chi[k], chi[k + 1], bf[k], bf[k + 1], var ? var[k] : 0., var ? var[k + 1] : 0., bm, yi,
                      yh, yd);
}

/* Mirror-point bracket of integrator_c/bounceaverage_c (src/RamGSL.c:546-563). */
static void mirror_bracket(int nT, const double *chi, const double *bf, double m, int *lh, int *rh, double *a,
                           double *b)
{
    *a = 0; *b = 0; *lh = 0; *rh = 0;
    for (int i = 1; i < nT - 1; i++)
        if (m <= bf[i - 1] && m >= bf[i]) { *a = chi[i - 1]; *lh = i - 1; break; }
    for (int i = nT - 2; i > 0; i--)
        if (m >= bf[i - 1] && m <= bf[i]) { *b = chi[i]; *rh = i; break; }
}

static int index_of(int nT, const double *chi, double v)
{
    for (int i = 0; i < nT; ++i)
        if (chi[i] == v) return i;
    return 0;
}

/* integrator_c (src/RamGSL.c:538-606) with exact segment integrals.
 * var != NULL gives bounceaverage_c (src/RamGSL.c:452-508) instead (yV in yi). */
static void ro_integrator(int nT, int nPa, double *mirror, const double *chi, const double *bf, const double *var,
                          double *yI, double *yH)
{
    int LH[512], RH[512];
    double a[512], b[512], dummy;
    for (int L = 1; L < nPa - 1; L++) mirror_bracket(nT, chi, bf, mirror[L], &LH[L], &RH[L], &a[L], &b[L]);
    if (var) line_integrals(nT, chi, bf, var, mirror[nPa - 1], 0, nT - 1, &dummy, &dummy, &yI[nPa - 1]);
    else line_integrals(nT, chi, bf, NULL, mirror[nPa - 1], 0, nT - 1, &yI[nPa - 1], &yH[nPa - 1], NULL);
    for (int L = nPa - 2; L > 0; L--) {
        if (mirror[L] >= bf[1] || a[L] == 0) a[L] = chi[0];
        if (mirror[L] >= bf[nT - 1] || b[L] == 0) b[L] = chi[nT - 1];
        if (a[L] <= chi[0] || b[L] >= chi[nT - 1]) {
            mirror[L] = mirror[nPa - 1];
            yI[L] = yI[nPa - 1];
            if (!var) yH[L] = yH[nPa - 1];
        } else {
            if ((RH[L] - LH[L]) <= 4) {
                yI[L] = yI[L + 1];
                if (!var) yH[L] = yH[L + 1];
                continue;
            }
            int i0 = index_of(nT, chi, a[L]), i1 = index_of(nT, chi, b[L]);
            if (var) {
                line_integrals(nT, chi, bf, var, mirror[L], i0, i1, &dummy, &dummy, &yI[L]);
                if (yI[L] <= 0) yI[L] = yI[L + 1];
            } else {
                line_integrals(nT, chi, bf, NULL, mirror[L], i0, i1, &yI[L], &yH[L], NULL);
                if (yI[L] <= 0) yI[L] = yI[L + 1];
                if (yH[L] <= 0) yH[L] = yH[L + 1];
            }
        }
    }
    if (var) {
        yI[0] = yI[1];
    } else {
        yI[0] = 0;
        yH[0] = yH[1];
    }
}

void ro_bounce_integrals(const ro_grid *g, int nthe, const double *chi, const double *x, const double *y,
                         const double *z, double *bline, const double *dens, int ieq, double *h, double *fi,
                         double *hd, double *bm)
{
    const double pi_d = 3.141592653589793238462643383279502884197;
    double *mirror = (double *)malloc(sizeof(double) * NPA);
    double *yI = (double *)malloc(sizeof(double) * NPA), *yH = (double *)malloc(sizeof(double) * NPA);
    double *yD = (double *)malloc(sizeof(double) * NPA);
    for (int i = 1; i <= NR; ++i)
        for (int j = 1; j <= NT; ++j) {
            size_t ln = ((size_t)(j - 1) * NR + (i - 1)) * nthe;
            double *bf = bline + ln;
            const double *xl = x + ln, *yl = y + ln, *zl = z + ln;
            for (int L = 1; L <= NPA; ++L) {
                size_t o = ((size_t)(L - 1) * NT + (j - 1)) * NR + (i - 1);
                h[o] = 0.; fi[o] = 0.;
                if (hd) hd[o] = 0.;
                if (bm) bm[o] = 0.;
            }
            if (OUTSIDE(i, j) != 0) continue;
            double length = 0.;
            for (int k = 1; k < nthe; ++k) {
                double dx = xl[k] - xl[k - 1], dy = yl[k] - yl[k - 1], dz = zl[k] - zl[k - 1];
                length = length + sqrt(dx * dx + dy * dy + dz * dz);
            }
            const int e = ieq - 1;
            double r0 = sqrt(xl[e] * xl[e] + yl[e] * yl[e]);
            double bmin = bf[0];
            for (int k = 1; k < nthe; ++k) bmin = dmin(bmin, bf[k]);
            if (fabs(bf[e] - bmin) > 1e-9) {
                if (2. * bmin - bf[e] > 0.) bf[e] = 2. * bmin - bf[e];
                else bf[e] = bmin - 0.01;
            }
            for (int L = 1; L <= NPA - 1; ++L) mirror[L - 1] = bf[e] / (1. - MU(L) * MU(L));
            mirror[NPA - 1] = bf[nthe - 1];
            ro_integrator(nthe, NPA, mirror, chi, bf, NULL, yI, yH);
            if (hd) ro_integrator(nthe, NPA, mirror, chi, bf, dens + ln, yD, NULL);
            for (int L = 1; L <= NPA; ++L) {
                size_t o = ((size_t)(L - 1) * NT + (j - 1)) * NR + (i - 1);
                fi[o] = (length / (pi_d * r0)) * yI[L - 1] / sqrt(mirror[L - 1]);
                h[o] = (length / (pi_d * 2 * r0)) * yH[L - 1] * sqrt(mirror[L - 1]);
                if (hd) hd[o] = yD[L - 1] / yH[L - 1];
                if (bm) bm[o] = mirror[L - 1];
            }
        }
    free(mirror); free(yI); free(yH); free(yD);
}

/* Monotone cubic interpolation of Steffen (1990, A&A 239, 443): interior
 * slopes by his eq. (11) -- the harmonic-limited average of the adjacent
 * secants, zero at local extrema -- and the one-sided secants at the two
 * ends (the simplest boundary choice of his section 2.2); Hermite cubics
 * in between.  Outside [xa[0], xa[n-1]] the value is extrapolated
 * linearly from the first or last two points, and xa is first reduced to
 * its strictly increasing subsequence, as the reference's 1-D wrapper
 * does (src/ModRamGSL.f90:261-311, src/RamGSL.c:111-175). */
static double sgn1(double v) { return v < 0 ? -1.0 : 1.0; }

static void steffen_eval(int n0, const double *xa0, const double *fa0, int nb, const double *xb, double *fb)
{
    double xa[512], fa[512], yp[512];
    int n = 0;
    for (int i = 0; i < n0; ++i)
        if (n == 0 || xa0[i] > xa[n - 1]) { xa[n] = xa0[i]; fa[n] = fa0[i]; ++n; }
    if (n < 2) {
        for (int q = 0; q < nb; ++q) fb[q] = n ? fa[0] : 0.;
        return;
    }
    yp[0] = (fa[1] - fa[0]) / (xa[1] - xa[0]);
    for (int i = 1; i < n - 1; ++i) {
        double hm = xa[i] - xa[i - 1], h = xa[i + 1] - xa[i];
        double sm = (fa[i] - fa[i - 1]) / hm, s = (fa[i + 1] - fa[i]) / h;
        double p = (sm * h + s * hm) / (hm + h);
        double m = fabs(sm);
        if (fabs(s) < m) m = fabs(s);
        if (0.5 * fabs(p) < m) m = 0.5 * fabs(p);
        yp[i] = (sgn1(sm) + sgn1(s)) * m;
    }
    yp[n - 1] = (fa[n - 1] - fa[n - 2]) / (xa[n - 1] - xa[n - 2]);
    for (int q = 0; q < nb; ++q) {
        double x = xb[q];
        if (x <= xa[0]) { fb[q] = fa[0] + (x - xa[0]) / (xa[1] - xa[0]) * (fa[1] - fa[0]); continue; }
        if (x >= xa[n - 1]) {
            fb[q] = fa[n - 1] + (x - xa[n - 1]) / (xa[n - 2] - xa[n - 1]) * (fa[n - 2] - fa[n - 1]);
            continue;
        }
        int i = 0;
        while (i < n - 2 && xa[i + 1] <= x) ++i;
        double h = xa[i + 1] - xa[i], s = (fa[i + 1] - fa[i]) / h;
        double a = (yp[i] + yp[i + 1] - 2 * s) / h / h, b = (3 * s - 2 * yp[i] - yp[i + 1]) / h;
        double t = x - xa[i];
        fb[q] = fa[i] + t * (yp[i] + t * (b + t * a));
    }
}

/* The RAM-variable fill of computehI (src/ModRamScb.f90:520-630) from the
 * bounce integrals of ro_bounce_integrals: h and I interpolated in pitch
 * angle to the bin boundaries PAbn (BOUNHS, BOUNIS, :520-531), lines
 * outside the magnetopause given the previous radial point's values
 * (:458-463), FNHS/FNIS/HDNS/BOUNHS/BOUNIS/BNES for I = 2..NR+1 from line
 * I-1 with the time derivatives over dthi (:566-602), the I = 1 row (:603-
 * 618) and the NaN repair (:620-632).  beq: equatorial B of each line in
 * the units of b, bnormal converts them to nT.  The field arrays (the ones
 * ro_grid points to) are updated in place. */
void ro_install_hI(ro_grid *g, const double *pa, const double *pabn, const double *hc, const double *ic,
                   const double *dc, const double *beq, double bnormal, double dthi, double *fnhs, double *fnis,
                   double *hdns, double *bounhs, double *bounis, double *bnes, double *dbdt, double *didt,
                   double *dibndt, double *eir, double *eip)
{
    size_t na = (size_t)NR * NT * NPA;
    double *h = (double *)malloc(sizeof(double) * na), *fi = (double *)malloc(sizeof(double) * na);
    double *hd = (double *)malloc(sizeof(double) * na), *hb = (double *)malloc(sizeof(double) * na);
    double *ib = (double *)malloc(sizeof(double) * na), *be = (double *)malloc(sizeof(double) * NR * NT);
    memcpy(h, hc, sizeof(double) * na); memcpy(fi, ic, sizeof(double) * na); memcpy(hd, dc, sizeof(double) * na);
    memcpy(be, beq, sizeof(double) * NR * NT);
#define A3(a, i, j, L) a[((size_t)((L)-1) * NT + (j)-1) * NR + (i)-1]
    /* outside the magnetopause: the previous radial point */
    for (int j = 1; j <= NT; ++j)
        for (int i = 2; i <= NR; ++i)
            if (OUTSIDE(i, j) == 1) {
                for (int L = 1; L <= NPA; ++L) {
                    A3(fi, i, j, L) = A3(fi, i - 1, j, L);
                    A3(h, i, j, L) = A3(h, i - 1, j, L);
                    A3(hd, i, j, L) = A3(hd, i - 1, j, L);
                }
                be[(size_t)(j - 1) * NR + i - 1] = be[(size_t)(j - 1) * NR + i - 2];
            }
    /* PA(NPA:1:-1) -> PAbn(NPA-1:2:-1) */
    double xa[512], fa[512], xb[512], fb[512];
    for (int L = 0; L < NPA; ++L) xa[L] = pa[NPA - 1 - L];
    for (int q = 0; q < NPA - 2; ++q) xb[q] = pabn[NPA - 2 - q];
    for (int i = 1; i <= NR; ++i)
        for (int j = 1; j <= NT; ++j) {
            for (int w = 0; w < 2; ++w) {
                const double *src = w ? fi : h;
                double *dst = w ? ib : hb;
                for (int L = 0; L < NPA; ++L) fa[L] = A3(src, i, j, NPA - L);
                steffen_eval(NPA, xa, fa, NPA - 2, xb, fb);
                for (int q = 0; q < NPA - 2; ++q) A3(dst, i, j, NPA - 1 - q) = fb[q];
                A3(dst, i, j, NPA) = A3(dst, i, j, NPA - 1);
                A3(dst, i, j, 1) = A3(dst, i, j, 2);
            }
        }
    const int nf = NR + 1;
#define F3(a, I, J, L) a[((size_t)((L)-1) * NT + (J)-1) * nf + (I)-1]
#define F2D(a, I, J) a[(size_t)((J)-1) * nf + (I)-1]
    const int dt0 = fabs(dthi) <= 1e-9;
    for (int I = 2; I <= NR + 1; ++I)
        for (int J = 1; J <= NT; ++J) {
            double bprev = F2D(bnes, I, J);
            for (int L = 1; L <= NPA; ++L) {
                double fip = F3(fnis, I, J, L), bip = F3(bounis, I, J, L);
                F3(fnhs, I, J, L) = A3(h, I - 1, J, L);
                F3(fnis, I, J, L) = A3(fi, I - 1, J, L);
                F3(hdns, I, J, L) = A3(hd, I - 1, J, L);
                F3(bounhs, I, J, L) = A3(hb, I - 1, J, L);
                F3(bounis, I, J, L) = A3(ib, I - 1, J, L);
                F3(didt, I, J, L) = dt0 ? 0. : (F3(fnis, I, J, L) - fip) / dthi;
                F3(dibndt, I, J, L) = dt0 ? 0. : (F3(bounis, I, J, L) - bip) / dthi;
            }
            F2D(bnes, I, J) = be[(size_t)(J - 1) * NR + I - 2] * bnormal / 1e9;
            F2D(dbdt, I, J) = dt0 ? 0. : (F2D(bnes, I, J) - bprev) / dthi;
        }
    for (int J = 1; J <= NT; ++J) {
        F2D(bnes, 1, J) = 0.32 / (LZ(1) * LZ(1) * LZ(1)) / 1.e4;
        F2D(dbdt, 1, J) = 0.;
        F2D(eir, 1, J) = 0.;
        F2D(eip, 1, J) = 0.;
        for (int L = 1; L <= NPA; ++L) {
            F3(fnhs, 1, J, L) = F3(fnhs, 2, J, L);
            F3(fnis, 1, J, L) = F3(fnis, 2, J, L);
            F3(bounhs, 1, J, L) = F3(bounhs, 2, J, L);
            F3(bounis, 1, J, L) = F3(bounis, 2, J, L);
            F3(hdns, 1, J, L) = F3(hdns, 2, J, L);
            F3(didt, 1, J, L) = 0.;
            F3(dibndt, 1, J, L) = 0.;
        }
    }
    for (int I = 2; I <= NR + 1; ++I)
        for (int J = 1; J <= NT; ++J)
            for (int L = 1; L <= NPA; ++L) {
                if (isnan(F3(fnis, I, J, L))) F3(fnis, I, J, L) = F3(fnis, I - 1, J, L);
                if (isnan(F3(fnhs, I, J, L))) F3(fnhs, I, J, L) = F3(fnhs, I - 1, J, L);
                if (isnan(F3(bounis, I, J, L))) F3(bounis, I, J, L) = F3(bounis, I - 1, J, L);
                if (isnan(F3(bounhs, I, J, L))) F3(bounhs, I, J, L) = F3(bounhs, I - 1, J, L);
                if (isnan(F3(hdns, I, J, L))) F3(hdns, I, J, L) = F3(hdns, I - 1, J, L);
                if (isnan(F3(didt, I, J, L))) F3(didt, I, J, L) = 0.;
                if (isnan(F3(dibndt, I, J, L))) F3(dibndt, I, J, L) = 0.;
            }
#undef A3
#undef F3
#undef F2D
    free(h); free(fi); free(hd); free(hb); free(ib); free(be);
}
