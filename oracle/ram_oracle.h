/*
 * ram_oracle.h -- CPU oracle for the RAM bounce-averaged kinetic step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the
 * reference routines on the advection hot path, used as the checker for
 * the CUDA path and as the timed CPU baseline.  Nothing in the product
 * (the ramgpu library and its host package) links or calls it.
 *
 * Parity status: pinned by the reference itself.  No Fortran compiler
 * exists on either build machine, so oracle/f90c.py translates the
 * reference's own routines (src/ModRamDrift.f90, src/ModRamLoss.f90,
 * src/ModRamRun.f90) to C and oracle/refrun.py runs its ram_run; this
 * restatement equals it bit for bit (F2, moments, FLUX, VT, DtsNext, the
 * SUMRC bookkeeping, every CDrift array and DtDrift minimum, CHARGE and
 * ATLOS: tests/test_ref_translated.py).  Known-answer tests and an
 * independent NumPy restatement (oracle/ram_numpy.py) pin it as well.
 *
 * Layout: every array is Fortran column-major with the reference's
 * dimensions, for ONE species (the reference's leading S index removed):
 *   F2, CDrift*, CHARGE, FLUX : (NR, NT, NE, NPA)
 *   FNHS, FNIS, BOUNHS, BOUNIS, HDNS, dIdt, dIbndt : (NR+1, NT, NPA)
 *   BNES, dBdt, VT, EIR, EIP : (NR+1, NT)
 *   outsideMGNP : int (NR, NT)
 *   FGEOS : (NT, NE, NPA)      FFACTOR : (NR, NE, NPA)
 *   ATLOS : (NR, NE)           PPERT, PPART : (NR, NT)
 * Build: gcc -O2 -ffp-contract=off (the reference is compiled without FMA
 * contraction, and every unsuffixed literal is double because RAM is built
 * with -fdefault-real-8).
 */
#ifndef RAM_ORACLE_H
#define RAM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nr, nt, ne, npa;
    /* radial / azimuthal grid (src/ModRamInit.f90:392-421) */
    const double *lz, *rlz;       /* NR+1 */
    const double *phi;            /* NT */
    double dl1, mdr, dphi, conf1, conf2;
    /* energy grid (src/ModRamInit.f90:429-459) */
    const double *ekev, *ebnd, *we, *de;    /* NE */
    /* pitch-angle cosine grid (src/ModRamInit.f90:477-544) */
    const double *mu, *dmu, *wmu;           /* NPA */
    const double *upa;                      /* NR, real-valued as in the reference */
    /* field tables (src/ModRamVariables.f90:31-37) */
    const double *fnhs, *fnis, *bounhs, *bounis, *hdns, *didt, *dibndt;
    const double *bnes, *dbdt, *eir, *eip;
    const int *outside_mgnp;
} ro_grid;

typedef struct {
    int qs;            /* species(S)%s_charge */
    int cex_kind;      /* 0 none, 1 Hydrogen, 2 HeliumP1, 3 OxygenP1 */
    double rmas;       /* rest mass [kg] */
    const double *grel, *grbnd, *v;          /* NE */
    const double *ffactor;                   /* (NR, NE, NPA) */
    const double *epp, *ernh;                /* NE */
} ro_species;

typedef struct {
    double betalim;    /* BetaLim (src/ModRamParams.f90:86) */
    double fraccfl;    /* FracCFL (src/ModRamVariables.f90:100) */
    double dts;        /* DTs */
    double dtsmin;     /* DTsMin (src/ModRamTiming.f90:28) */
    int closed;        /* 1: closed faces, conservation mode (new; not in the reference) */
    int do_atmol;      /* 1: call ATMOL as ram_run does */
} ro_params;

/* Per-species drift parameters from DRIFTPARA (src/ModRamDrift.f90:36-88). */
typedef struct {
    double *vr, *p1;          /* NR */
    double *p2, *edot;        /* (NR, NE) */
    double *mudot;            /* (NR, NPA) */
} ro_driftpara_t;

/* Loss bookkeeping of one ram_run call (src/ModRamRun.f90:77-175). */
typedef struct {
    double setrc;               /* SETRC after the call */
    double lsdr, lscha, lsatm;  /* ELORC accumulated into LSDR/LSCHA/LSATM */
    double lswae;               /* ELORC of the pitch-angle diffusion (LSWAE) */
} ro_losses;

/* Threads for the loops over independent lines inside each routine
 * (default 1, the reference's serial loops); ro_ram_run nests them inside
 * its per-species threads.  Results are identical for every setting. */
void ro_set_inner_threads(int n);

/* VOLS potential, src/ModRamRun.f90:45-54.  vt: (NR+1, NT). */
void ro_vt_vols(const ro_grid *g, double kp, double *vt);

/* DRIFTPARA.  Arrays in dp are caller-allocated. */
void ro_driftpara(const ro_grid *g, const ro_species *sp, const ro_params *p, ro_driftpara_t *dp);

/* The four sweeps; each updates f2 in place, optionally stores the face
 * coefficients in cdrift (NR,NT,NE,NPA; may be NULL) and returns DtDrift*. */
double ro_driftr(const ro_grid *g, const ro_species *sp, const ro_params *p,
                 const ro_driftpara_t *dp, const double *vt, const double *fgeos,
                 double *f2, double *cdrift);
double ro_driftp(const ro_grid *g, const ro_species *sp, const ro_params *p,
                 const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift);
double ro_drifte(const ro_grid *g, const ro_species *sp, const ro_params *p,
                 const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift);
double ro_driftmu(const ro_grid *g, const ro_species *sp, const ro_params *p,
                  const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift);

/* CEPARA analytic branches: charge (NR,NT,NE,NPA), atlos (NR,NE). */
void ro_cepara(const ro_grid *g, const ro_species *sp, const ro_params *p,
               double *charge, double *atlos);
void ro_charexchange(const ro_grid *g, double *f2, const double *charge);
void ro_atmol(const ro_grid *g, double *f2, const double *atlos);
double ro_sumrc(const ro_grid *g, const double *f2);
/* ANISCH moment block; modifies f2(:,:,K,1) for K=2..NE, I=2..NR. */
void ro_anisch(const ro_grid *g, const ro_species *sp, double *f2, double *ppert, double *ppart);
/* FLUX = F2/FFACTOR/FNHS (src/ModRamRun.f90:208-222); flux must be zeroed by the caller. */
void ro_flux(const ro_grid *g, const ro_species *sp, const double *f2, double *flux);

/* One ram_run call (src/ModRamRun.f90:16-225) for ns species.
 *   kp        : Kp for the VOLS potential (ignored when vt_in != NULL)
 *   vt_in     : optional precomputed potential (NR+1,NT)
 *   vt_out    : optional, receives the potential used
 *   fgeos[s]  : boundary (NT,NE,NPA) per species
 *   f2[s]     : state (NR,NT,NE,NPA) per species, updated in place
 *   ppert/ppart[s] : (NR,NT) per species, may be NULL
 *   flux[s]   : (NR,NT,NE,NPA) per species, may be NULL
 *   losses[s] : per species, may be NULL; setrc must hold the previous SETRC
 *   dts_next  : DtsNext
 *   nthreads  : OpenMP threads over species (the reference's parallel loop)
 * Returns 0. */
int ro_ram_run(const ro_grid *g, int ns, const ro_species *sp, const ro_params *p,
               double kp, const double *vt_in, double *vt_out,
               const double *const *fgeos, double *const *f2,
               double *const *ppert, double *const *ppart, double *const *flux,
               ro_losses *losses, double *dts_next, int nthreads);

/* ro_ram_run with WPADIF (src/ModRamRun.f90:91-107,144-158) for every
 * species s with daa[s] != NULL (daa may be NULL): daa[s] is the
 * pitch-angle diffusion coefficient D(I,J,K,L) of ro_padif. */
int ro_ram_run2(const ro_grid *g, int ns, const ro_species *sp, const ro_params *p,
                double kp, const double *vt_in, double *vt_out,
                const double *const *fgeos, double *const *f2,
                double *const *ppert, double *const *ppart, double *const *flux,
                ro_losses *losses, double *dts_next, int nthreads, const double *const *daa);

/* Implicit pitch-angle diffusion of WPADIF (src/ModRamWPI.f90:643-714) and
 * FLCscatter (src/ModRamLoss.f90:512-575), one species in place, with
 * coefficient daa = D(I,J,K,L) (NR,NT,NE,NPA). */
void ro_padif(const ro_grid *g, const ro_params *p, const double *daa, double *f2);

/* Bounce integrals of computehI (src/ModRamScb.f90:378-406; integrator_c and
 * bounceaverage_c of src/RamGSL.c) on RAM-grid field lines, the integrals of
 * the linearly interpolated integrands evaluated exactly.  Inputs per line
 * (I,J): nthe nodes of chi (shared), x, y, z, B (bline, modified in place by
 * the equator fix of :388-395) and density (dens, may be NULL), all
 * (nthe, NR, NT); ieq = nThetaEquator (1-based).  Outputs (NR,NT,NPA):
 * h = H_cart, fi = I_cart, hd = HDens_cart (may be NULL), bm = the mirror
 * field used (may be NULL); lines with outsideMGNP set are zero. */
void ro_bounce_integrals(const ro_grid *g, int nthe, const double *chi, const double *x, const double *y,
                         const double *z, double *bline, const double *dens, int ieq, double *h, double *fi,
                         double *hd, double *bm);

/* The RAM-variable fill of computehI (src/ModRamScb.f90:458-463,520-632)
 * from the bounce integrals (hc, ic, dc: (NR,NT,NPA); beq: (NR,NT)), with
 * BOUNHS/BOUNIS by Steffen's monotone cubic in pitch angle at PAbn.  The
 * field arrays passed are updated in place ((NR+1,NT,NPA) / (NR+1,NT)). */
void ro_install_hI(ro_grid *g, const double *pa, const double *pabn, const double *hc, const double *ic,
                   const double *dc, const double *beq, double bnormal, double dthi, double *fnhs, double *fnis,
                   double *hdns, double *bounhs, double *bounis, double *bnes, double *dbdt, double *didt,
                   double *dibndt, double *eir, double *eip);

/* One DTs half of ram_run for one species (the measurement "step"):
 * order 0 = R,P,E,MU,[CEX],[ATMOL]; order 1 = [ATMOL],[CEX],MU,E,P,R.
 * charge/atlos from ro_cepara. */
void ro_half_step(const ro_grid *g, const ro_species *sp, const ro_params *p,
                  const ro_driftpara_t *dp, const double *vt, const double *fgeos,
                  const double *charge, const double *atlos, double *f2, int order);

/* ---- frozen-limiter adjoint (new; the reference has no adjoint) ---------
 * *_rec: the sweeps above, also recording per face the limiter case
 * (0 upwind, 1 BetaLim*R, 2 one, 3 R, 4 BetaLim; bit 3: the updated cell was
 * clipped) into rec (NR,NT,NE,NPA) and, for DRIFTR, per line the FGEOS index
 * (NT,NE,NPA layout) that F(NR+1) came from, -1 if none, into gsrc.
 * *_adj: transpose of that frozen line map applied to lam in place, with
 * cd the CDrift* output of the recorded call; DRIFTR adds dJ/dFGEOS. */
double ro_driftr_rec(const ro_grid *g, const ro_species *sp, const ro_params *p,
                     const ro_driftpara_t *dp, const double *vt, const double *fgeos,
                     double *f2, double *cdrift, unsigned char *rec, int *gsrc);
double ro_driftp_rec(const ro_grid *g, const ro_species *sp, const ro_params *p,
                     const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift,
                     unsigned char *rec);
double ro_drifte_rec(const ro_grid *g, const ro_species *sp, const ro_params *p,
                     const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift,
                     unsigned char *rec);
double ro_driftmu_rec(const ro_grid *g, const ro_species *sp, const ro_params *p,
                      const ro_driftpara_t *dp, const double *vt, double *f2, double *cdrift,
                      unsigned char *rec);
void ro_driftr_adj(const ro_grid *g, const ro_params *p, const double *cd, const unsigned char *rec,
                   const int *gsrc, double *lam, double *gfgeos);
void ro_driftp_adj(const ro_grid *g, const ro_params *p, const double *cd, const unsigned char *rec,
                   double *lam);
void ro_drifte_adj(const ro_grid *g, const ro_species *sp, const ro_params *p, const double *cd,
                   const unsigned char *rec, double *lam);
void ro_driftmu_adj(const ro_grid *g, const ro_params *p, const double *cd, const unsigned char *rec,
                    double *lam);

#ifdef __cplusplus
}
#endif
#endif
