/*
 * ramgpu.h -- C ABI of the GB300 (sm_103a) implementation of RAM's
 * bounce-averaged kinetic step.
 *
 * The entry points replace the body of the species loop of the reference's
 * `ram_run` and its tail (src/ModRamRun.f90:64-222), which `run_ramscb`
 * calls once per iteration (src/ModRamScbRun.f90:85).  The reference has no
 * plugin interface: its path is a set of species-indexed Fortran
 * subroutines sharing module globals.  This header turns that state into a
 * context object that owns every device buffer; the distribution function
 * F2 stays resident on the GPU across calls.
 *
 * Conventions
 *  - Every function returns int: RAMGPU_OK (0) or a negative RAMGPU_ERR_*.
 *    ramgpu_last_error() gives the message.  The library never exits or
 *    aborts the caller.
 *  - Host arrays are borrowed for the duration of a call only and use the
 *    reference's Fortran column-major layout and dimensions, so a Fortran
 *    caller passes its module arrays as they are (iso_c_binding).
 *  - Species index s is 0-based here (Fortran S-1); member m is 0-based.
 *  - All arithmetic is IEEE binary64.  Calls are synchronous on the
 *    context's stream unless stated otherwise.
 *  - One context per host thread.
 */
#ifndef RAMGPU_H
#define RAMGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RAMGPU_OK 0
#define RAMGPU_ERR_ARG (-1)      /* bad argument, size or ordering */
#define RAMGPU_ERR_CUDA (-2)     /* CUDA runtime error */
#define RAMGPU_ERR_STATE (-3)    /* call made before its inputs were set */
#define RAMGPU_ERR_NUMERIC (-4)  /* non-finite value detected */
#define RAMGPU_ERR_NOMEM (-5)    /* device allocation failed */
#define RAMGPU_ERR_IO (-6)       /* file cannot be opened, read or written, or fails its checksum */

/* Charge-exchange cross-section branch of CEPARA (src/ModRamLoss.f90:38-87). */
#define RAMGPU_CEX_NONE 0      /* "Electron" (CEX_file 'na'): no loss */
#define RAMGPU_CEX_HYDROGEN 1  /* "Hydrogen"  src/ModRamLoss.f90:39-53 */
#define RAMGPU_CEX_HELIUM1 2   /* "HeliumP1"  src/ModRamLoss.f90:54-68 */
#define RAMGPU_CEX_OXYGEN1 3   /* "OxygenP1"  src/ModRamLoss.f90:69-83 */

/* Flags of ramgpu_config.flags */
#define RAMGPU_FLAG_CLOSED 1u    /* closed outer faces in R, E, MU: conserves sum F2*WE*WMU
                                    (new mode; the reference has no such switch) */
#define RAMGPU_FLAG_NO_ATMOL 2u  /* skip ATMOL (the reference calls it every step,
                                    src/ModRamRun.f90:122,127) */
#define RAMGPU_FLAG_LOSSES 4u    /* SUMRC bookkeeping LSDR/LSCHA/LSATM each ram_run
                                    (src/ModRamRun.f90:77-175,231-259) */

typedef struct ramgpu_ctx ramgpu_ctx;

/* Grid sizes and scheme parameters.  Mirrors #RAMGRID / #RAMLIMITER
 * (src/IM_set_parameters.f90:152-161) and ModRamGrids (src/ModRamGrids.f90:15-19). */
typedef struct {
    int nr, nt, ne, npa;   /* NR, NT, NE, NPA */
    int ns;                /* species kinds (the reference's NS) */
    int n_members;         /* ensemble members; 1 reproduces the reference */
    double betalim;        /* BetaLim, clamped to [1,2] as IM_set_parameters does */
    double fraccfl;        /* FracCFL (0.8 in the reference) */
    double dtsmin;         /* DTsMin (0.1 s in the reference) */
    unsigned flags;        /* RAMGPU_FLAG_* */
} ramgpu_config;

/* Grid and factor tables produced by ARRAYS (src/ModRamInit.f90:364-587).
 * Shapes are the reference's, Fortran order; per-species arrays carry the
 * leading NS index like the reference: GREL(NS,NE), FFACTOR(NS,NR,NE,NPA). */
typedef struct {
    const double *lz, *rlz;          /* (NR+1) */
    const double *phi;               /* (NT) */
    double dl1, mdr, dphi, conf1, conf2;
    const double *ekev, *ebnd, *we, *de;   /* (NE) */
    const double *mu, *dmu, *wmu;          /* (NPA) */
    const double *upa;               /* (NR), real as in the reference */
    const double *rmas;              /* (NS) */
    const double *grel, *grbnd, *v;  /* (NS,NE) */
    const double *epp, *ernh;        /* (NS,NE) */
    const double *ffactor;           /* (NS,NR,NE,NPA) */
} ramgpu_grid;

/* ---- lifetime ------------------------------------------------------------ */

/* Replaces ram_allocate's RAM arrays (src/ModRamInit.f90:68-120).
 * n_members x ns is at most 65535 (one launch-grid row per work item). */
int ramgpu_create(const ramgpu_config *cfg, ramgpu_ctx **out);
int ramgpu_destroy(ramgpu_ctx *ctx);
/* Copies the last error message of ctx (or of the last failed create when
 * ctx is NULL) into buf. */
int ramgpu_last_error(const ramgpu_ctx *ctx, char *buf, size_t len);
/* Use this CUDA stream (cudaStream_t) for all work; NULL = the context's own. */
int ramgpu_set_stream(ramgpu_ctx *ctx, void *stream);

/* ---- inputs -------------------------------------------------------------- */

/* species(S)%s_charge and the CEPARA branch (src/ModRamSpecies.f90:37-138). */
int ramgpu_set_species(ramgpu_ctx *ctx, int s, int charge, int cex_kind);
/* ARRAYS output (src/ModRamInit.f90:364-587). */
int ramgpu_set_grid(ramgpu_ctx *ctx, const ramgpu_grid *grid);
/* computehI / dipole field tables (src/ModRamScb.f90:567-619):
 * FNHS, FNIS, BOUNHS, BOUNIS, HDNS, dIdt, dIbndt : (NR+1,NT,NPA)
 * BNES, dBdt, EIR, EIP : (NR+1,NT);  outsideMGNP : int (NR,NT) */
int ramgpu_set_fields(ramgpu_ctx *ctx, const double *fnhs, const double *fnis,
                      const double *bounhs, const double *bounis, const double *hdns,
                      const double *didt, const double *dibndt, const double *bnes,
                      const double *dbdt, const double *eir, const double *eip,
                      const int *outside_mgnp);
/* Implicit pitch-angle diffusion of species s, the scheme WPADIF
 * (src/ModRamWPI.f90:643-714) and FLCscatter (src/ModRamLoss.f90:512-575)
 * share, with coefficient daa = D(I,J,K,L) (NR,NT,NE,NPA), host or device
 * memory: ATAW+ATAC for electrons (chorus and hiss), ATAW_emic_h +
 * ATAW_emic_he for EMIC, FLC_coef(S,:,:,:,:) for FLC.  While a coefficient
 * is set, ramgpu_ram_run applies the diffusion to species s after the
 * forward drifts and again before the reverse ones, where ram_run calls
 * WPADIF (src/ModRamRun.f90:91-107,144-158); RAMGPU_OP_PADIF applies it
 * once.  daa = NULL removes it.  The adjoint does not cover it. */
int ramgpu_set_pa_diffusion(ramgpu_ctx *ctx, int s, const double *daa);

/* The field tables as the context holds them (for example after
 * ramgpu_compute_hI), same shapes as ramgpu_set_fields; any output may be
 * NULL. */
int ramgpu_get_fields(ramgpu_ctx *ctx, double *fnhs, double *fnis, double *bounhs, double *bounis,
                      double *hdns, double *didt, double *dibndt, double *bnes, double *dbdt,
                      double *eir, double *eip);

/* GEOSB output FGEOS(S,:,:,:) of one species (src/ModRamBoundary.f90:241-319):
 * (NT,NE,NPA), host or device memory.  member < 0 sets it for every member. */
int ramgpu_set_boundary(ramgpu_ctx *ctx, int member, int s, const double *fgeos_s);
/* Potential VT(NR+1,NT) for a member (the non-VOLS branch, src/ModRamRun.f90:49). */
int ramgpu_set_potential(ramgpu_ctx *ctx, int member, const double *vt);
/* Kp for the Volland-Stern potential computed on the device
 * (src/ModRamRun.f90:45-54).  member < 0 sets every member. */
int ramgpu_set_kp(ramgpu_ctx *ctx, int member, double kp);
/* Kp of every member at once (n_members values), VOLS mode for all. */
int ramgpu_set_kp_all(ramgpu_ctx *ctx, const double *kp);
/* Species a member advances (default: all ns).  list holds 0-based species. */
int ramgpu_set_member_species(ramgpu_ctx *ctx, int member, int n, const int *list);
/* Retire (0) or re-activate (1) a member; retired members are not advanced. */
int ramgpu_set_member_active(ramgpu_ctx *ctx, int member, int active);

/* ---- state --------------------------------------------------------------- */

/* F2(S,:,:,:,:) of one species as a contiguous (NR,NT,NE,NPA) array in host
 * or device memory (unified addressing decides the copy direction). */
int ramgpu_upload_f2(ramgpu_ctx *ctx, int member, int s, const double *f2_s);
int ramgpu_download_f2(ramgpu_ctx *ctx, int member, int s, double *f2_s);
/* Stream-ordered forms: the copies (and the moment read-back) are queued on
 * the context's stream behind or ahead of ramgpu_ram_run_async and do not
 * wait; the caller keeps the buffers alive and unchanged until
 * ramgpu_synchronize returns.  With page-locked host buffers they overlap
 * nothing but run at full link speed and cost the host no round trips. */
int ramgpu_upload_f2_async(ramgpu_ctx *ctx, int member, int s, const double *f2_s);
int ramgpu_download_f2_async(ramgpu_ctx *ctx, int member, int s, double *f2_s);
int ramgpu_moments_async(ramgpu_ctx *ctx, int member, int s, double *ppert, double *ppart);
int ramgpu_synchronize(ramgpu_ctx *ctx);
/* The whole reference array F2(NS,NR,NT,NE,NPA) of one member
 * (src/ModRamVariables.f90:31), transposed on the device (synchronous). */
int ramgpu_upload_f2_all(ramgpu_ctx *ctx, int member, const double *f2);
int ramgpu_download_f2_all(ramgpu_ctx *ctx, int member, double *f2);
/* Device pointer to F2 of (member, s), (NR,NT,NE,NPA) contiguous; for
 * zero-copy interop.  Valid until ramgpu_destroy. */
int ramgpu_f2_device_ptr(ramgpu_ctx *ctx, int member, int s, double **dptr);

/* ---- the step ------------------------------------------------------------ */

/* One ram_run call (src/ModRamRun.f90:16-225, without the optional
 * Coulomb/WPI/EMIC/FLC processes): for every active member and species the
 * Strang pair R,P,E,MU,[CEX],ATMOL | ATMOL,[CEX],MU,E,P,R of length dts each,
 * then F2(:,:,NT,:,:)=F2(:,:,1,:,:), the magnetopause mask, DtsNext, and
 * the ANISCH moments (with their F2(:,:,:,:,1) side effect). */
int ramgpu_ram_run(ramgpu_ctx *ctx, double dts);
/* One DTs half of ram_run without the tail: order 0 = R,P,E,MU,[CEX],ATMOL;
 * order 1 = ATMOL,[CEX],MU,E,P,R. */
int ramgpu_half_step(ramgpu_ctx *ctx, double dts, int order);
/* Same as ramgpu_ram_run but enqueued only (no synchronisation, no host
 * reads), for CUDA-graph capture and overlap.  Inputs set by the calls
 * above are read at execution time. */
int ramgpu_ram_run_async(ramgpu_ctx *ctx, double dts);
/* One ram_run call with F2 crossing the host boundary, as the reference's
 * host array does every call: f2[slot] (slot = member*NS + species, host
 * pointers: page-locked buffers go through the copy engines, ordinary
 * pageable ones through an SM copy where the device reaches pageable memory
 * (a coherent host link such as Grace's), else blocking copies) holds that
 * item's F2(S,:,:,:,:) as in
 * ramgpu_upload_f2; it is uploaded, advanced and written back in place.
 * The active items are split into groups (ramgpu_set_pipeline_groups,
 * default 4) that run on their own streams as their uploads land, so the
 * copies of one group overlap the sweeps of the others.  ppert/ppart,
 * when not NULL, receive each item's (NR,NT) moments (NULL entries are
 * skipped), and so does f2 (a NULL entry leaves that item's F2 resident
 * and unchanged on the host side).  Returns when every copy is back.
 * Every pointer is classified (page-locked or pageable) on every call; with
 * graphs on, the call is captured on first use and replayed while the same
 * pointers with the same classification come back (memory freed and
 * reallocated, registered or unregistered at the same address is
 * classified anew and the graph rebuilt). */
int ramgpu_ram_run_host(ramgpu_ctx *ctx, double dts, double *const *f2, double *const *ppert,
                        double *const *ppart);
/* One ram_run call on the arrays exactly as RAM holds them: replaces the
 * body of ram_run's species loop and tail (src/ModRamRun.f90:64-222) for a
 * caller whose state is the module array F2(NS,NR,NT,NE,NPA)
 * (src/ModRamVariables.f90:31, species index fastest) and whose moments are
 * PPERT(NS,NR,NT), PPART(NS,NR,NT).  f2[m], ppert[m], ppart[m]: member m's
 * arrays (NULL skips the transfer; ppert/ppart tables may be NULL).  The
 * device reads F2 in place and transposes it into its per-species blocks
 * (and back) with no host-side pass: arrays the device reaches (device,
 * mapped page-locked, or pageable memory over a coherent host link) are read
 * and written by the transposing kernels directly, others go through a
 * device staging buffer and the copy engines.  Every species of a member is
 * transferred; F2's L >= 2 planes go back while the moments are computed.
 * Results equal ramgpu_ram_run_host's bit for bit.  With ramgpu_set_graph on
 * (and every array reachable) the call is one CUDA graph per array set,
 * rebuilt when an address or how the device reaches it changes. */
int ramgpu_ram_run_ref(ramgpu_ctx *ctx, double dts, double *const *f2, double *const *ppert,
                       double *const *ppart);
/* How ramgpu_ram_run_ref and ramgpu_upload/download_f2_all move arrays the
 * device could reach in place (no reference counterpart): force = 0 (the
 * default) in place, read and written by the transposing kernels; 1 every
 * array through the device staging buffer and the copy engines,
 * unpipelined; 2 page-locked F2 arrays of ramgpu_ram_run_ref through the
 * copy engines plane chunk by plane chunk into a device staging area
 * inside the pipeline, the others in place.  On GB300's coherent Grace
 * link in place is fastest (0.88 ms per four-species call, against
 * 0.95-1.08 ms for 2 and 1.00 ms for 1); 1 and 2 are for hosts whose link
 * favours the copy engines. */
int ramgpu_set_ref_staging(ramgpu_ctx *ctx, int force);
/* Chunks of L planes the host calls (ramgpu_ram_run_host, ramgpu_ram_run_ref)
 * pipeline F2 over: 1..8, or 0 for the item-group pipeline of
 * ramgpu_set_pipeline_groups (also taken with RAMGPU_FLAG_LOSSES, the
 * pitch-angle diffusion or the pipeline trace; the reference-layout call
 * then runs unpipelined), or -1 (default): item groups for
 * ramgpu_ram_run_host, 4 chunks for ramgpu_ram_run_ref, the faster choice
 * of each on the four-species step.  L is F2's slowest index,
 * so a chunk is one contiguous range of every array, and the R, P, E sweeps
 * and the closing copy/mask work plane by plane: chunk c's forward R, P, E
 * run while chunk c+1 lands, the pitch-angle sweeps once all are in, and
 * chunk c goes back right after its reverse R while the next computes.
 * Results are the same for every count. */
int ramgpu_set_pipeline_chunks(ramgpu_ctx *ctx, int chunks);
/* Number of item groups ramgpu_ram_run_host pipelines its copies over
 * (1..8, default 4, at most one per item; 1 with RAMGPU_FLAG_LOSSES). */
int ramgpu_set_pipeline_groups(ramgpu_ctx *ctx, int groups);
/* The configured pipeline group count (0 for a bad context). */
int ramgpu_pipeline_groups(const ramgpu_ctx *ctx);
/* Diagnostics (no reference counterpart): with the trace on, each
 * ramgpu_ram_run_host call runs without its graph and records, per group g,
 * the times (ms after the call's first enqueued work) at which its uploads
 * had landed, its sweeps were done and its read-back was done;
 * ramgpu_pipeline_trace returns them for the last call as ms[3*g + 0..2]
 * (ms holds at least 24 values) and the group count in *groups. */
int ramgpu_set_pipeline_trace(ramgpu_ctx *ctx, int enable);
int ramgpu_pipeline_trace(ramgpu_ctx *ctx, int *groups, float *ms);
/* Number of item groups whose sweeps ramgpu_ram_run (and _async) runs on
 * concurrent streams (1..8, default 4, at most one per item): one group's
 * launch tails and the gaps between its dependent launches fill with the
 * others' CTAs.  Results are the same for every count; the loss
 * bookkeeping (RAMGPU_FLAG_LOSSES) and per-kernel timing passes run as one
 * group.  The autotuner picks the count. */
int ramgpu_set_step_groups(ramgpu_ctx *ctx, int groups);
/* The configured step group count (0 for a bad context). */
int ramgpu_step_groups(const ramgpu_ctx *ctx);

/* Diagnostic: one operator of the step on every active item, as the
 * reference routine of the same name (the coefficient tables for dts are
 * rebuilt first).  op: 0 DRIFTR, 1 DRIFTP, 2 DRIFTE, 3 DRIFTMU,
 * 4 CHAREXCHANGE (src/ModRamLoss.f90:457), 5 ATMOL (src/ModRamLoss.f90:485),
 * 6 ANISCH moments.  cfl != 0 also records the DtDrift* of that sweep. */
#define RAMGPU_OP_DRIFTR 0
#define RAMGPU_OP_DRIFTP 1
#define RAMGPU_OP_DRIFTE 2
#define RAMGPU_OP_DRIFTMU 3
#define RAMGPU_OP_CHAREXCHANGE 4
#define RAMGPU_OP_ATMOL 5
#define RAMGPU_OP_ANISCH 6
#define RAMGPU_OP_PADIF 7   /* one implicit pitch-angle diffusion (WPADIF / FLCscatter) */
int ramgpu_apply_op(ramgpu_ctx *ctx, double dts, int op, int cfl);

/* ---- outputs ------------------------------------------------------------- */

/* PPERT(S,:,:), PPART(S,:,:) of the last ram_run: (NR,NT) each. */
int ramgpu_moments(ramgpu_ctx *ctx, int member, int s, double *ppert, double *ppart);
/* FLUX(S,:,:,:,:) = F2/FFACTOR/FNHS of the current state (src/ModRamRun.f90:208-222):
 * (NR,NT,NE,NPA); entries the reference leaves unset are 0. */
int ramgpu_flux(ramgpu_ctx *ctx, int member, int s, double *flux_s);
/* DtDriftR/P/E/Mu of the last ram_run for (member,s), and DtsNext over all
 * species of the member (src/ModRamRun.f90:204-205).  out: 5 doubles. */
int ramgpu_cfl(ramgpu_ctx *ctx, int member, int s, double *out5);
/* SUMRC bookkeeping (needs RAMGPU_FLAG_LOSSES): SETRC, LSDR, LSCHA, LSATM
 * accumulated since the last ramgpu_reset_losses, which zeroes the losses
 * and takes SETRC of the current state as the starting ENOLD.  out: 4 doubles. */
int ramgpu_losses(ramgpu_ctx *ctx, int member, int s, double *out4);
/* LSWAE (src/ModRamRun.f90:99,106,150,157): the ELORC of the pitch-angle
 * diffusion accumulated since the last ramgpu_reset_losses. */
int ramgpu_loss_wae(ramgpu_ctx *ctx, int member, int s, double *lswae);
int ramgpu_reset_losses(ramgpu_ctx *ctx);

/* Virtual spacecraft on the equatorial plane.  FLUX of the current state
 * (src/ModRamRun.f90:208-222) sampled at (L-shell [RE], MLT [h]) for every
 * species, energy and pitch-angle bin, the RAM-grid counterpart of the flux
 * part of fly_sats (src/ModRamSats.f90:640-666):
 *   SatFlux(S,E,PA): bilinear in (R, MLT) over the four FLUX cells around
 *     the point (J = NT folded onto J = 1); BadDataFlag (-1e10,
 *     src/ModRamSats.f90:35) unless all four are > 0, which also makes the
 *     E = 1 and PA = 1 bins and species outside the member BadDataFlag;
 *   OmnFlux(S,E) = sum over PA of SatFlux*4*pi*WMU(PA) for SatFlux > 0, and
 *     BadDataFlag when that sum is not > 0.
 * The reference interpolates flux3DEQ on the SCB mesh with GSL
 * natural-neighbour weights; without SCB the sampling mesh is RAM's own
 * equatorial grid.  Trajectory interpolation in time is the caller's.
 * sat_flux: nsat*NS*NE*NPA, per satellite SatFlux(NS,NE,NPA) in Fortran
 * order; omni_flux: nsat*NS*NE, per satellite OmnFlux(NS,NE).  Either
 * output may be NULL (not both). */
typedef struct {
    int member;
    double lshell;   /* [RE] */
    double mlt;      /* [h] */
} ramgpu_sat;
int ramgpu_fly_sats(ramgpu_ctx *ctx, const ramgpu_sat *sats, int nsat, double *sat_flux,
                    double *omni_flux);

/* Bounce integrals of computehI (src/ModRamScb.f90:378-406, with
 * integrator_c and bounceaverage_c of src/RamGSL.c:452-606) on field lines
 * through the RAM grid: line (I,J), I = 1..NR, is the one through LZ(I+1).
 * Inputs (host or device memory): chi (nthe), the field-line coordinate;
 * x, y, z, b, dens (nthe, NR, NT), positions [RE], |B| and the density to
 * bounce-average (dens may be NULL); ieq = nThetaEquator (1-based).  The
 * equator fix of :388-395 is applied to a copy of b.  The integrals of the
 * reference's linearly interpolated integrands are evaluated exactly
 * (the reference's GSL cquad runs at 1e-3 tolerance).  Outputs (NR,NT,NPA):
 * h = H_cart, fi = I_cart, hdens = HDens_cart (needs dens; may be NULL),
 * bmirror = the mirror field of each pitch angle as the integrals used it
 * (may be NULL).  Lines with outsideMGNP (ramgpu_set_fields) set give 0. */
int ramgpu_bounce_integrals(ramgpu_ctx *ctx, int nthe, const double *chi, const double *x,
                            const double *y, const double *z, const double *b, const double *dens,
                            int ieq, double *h, double *fi, double *hdens, double *bmirror);

/* computehI's producer on the device: the bounce integrals above, then the
 * RAM-variable fill of src/ModRamScb.f90:458-463,520-632 written straight
 * into the context's field tables -- lines outside the magnetopause take
 * the previous radial point; FNHS, FNIS, HDNS for I = 2..NR+1 from line
 * I-1; BOUNHS, BOUNIS from h and I interpolated in pitch angle at the bin
 * boundaries PAbn (Steffen's monotone cubic, as the reference's default
 * 1-D interpolation); BNES = equatorial B * bnormal / 1e9; dIdt, dIbndt,
 * dBdt over dthi seconds (0 when |dthi| <= 1e-9); the I = 1 row (dipole
 * BNES, EIR = EIP = 0) and the NaN repair.  pa, pabn: PA and PAbn of
 * ARRAYS (NPA).  The SCB-to-RAM line conversion, the outside-SCB scaling
 * and the optional Gaussian smoothing are the caller's.  The next step
 * rebuilds every derived table. */
int ramgpu_compute_hI(ramgpu_ctx *ctx, int nthe, const double *chi, const double *x, const double *y,
                      const double *z, const double *b, const double *dens, int ieq, const double *pa,
                      const double *pabn, double bnormal, double dthi);

/* SCB hand-off, ram_sum_pressure (src/ModRamFunctions.f90:272-297):
 * PAllSum(I,J) = sum_S (2/3 PPERT(S,I,J) + 1/3 PPART(S,I,J)) and
 * PParSum(I,J) = sum_S PPART(S,I,J) over the member's species, in species
 * order, from the moments of the last ram_run.  Outputs (NR,NT) each. */
int ramgpu_sum_pressure(ramgpu_ctx *ctx, int member, double *pallsum, double *pparsum);

/* ---- execution tuning (no reference counterpart) ------------------------ */

/* Sweeps whose face coefficient C and CORR factor the forward half of a
 * ram_run call keeps for its reverse half, which then reads them instead of
 * recomputing them: bit 0 R, 1 P, 2 E, 3 MU.  Each set bit costs 16 bytes
 * per cell and (member, species) of device memory, taken only while it fits
 * in a quarter of the free memory.  Default 4 (DRIFTE only, whose C costs
 * two FP64 operations; for the other sweeps the stores cost more time than
 * the FP64 work they save).  Results are identical for every mask. */
int ramgpu_set_coef_store(ramgpu_ctx *ctx, int mask);

/* Replay ram_run / ram_run_async from a CUDA graph captured on first use and
 * re-captured when dts, the active (member, species) list, the flags or the
 * launch shapes change.  Inputs (F2, Kp/VT, FGEOS, fields) are read when the
 * graph runs, so set_* calls between steps take effect.  Timing mode
 * (ramgpu_set_timing) bypasses the graph. */
int ramgpu_set_graph(ramgpu_ctx *ctx, int enable);
/* Launch shape of sweep w (0 DRIFTR, 1 DRIFTP, 2 DRIFTE, 3 DRIFTMU):
 * threads per CTA (32..256, multiple of 32) and, when persistent_ctas > 0,
 * a persistent grid of that many CTAs looping over (item, line-block) units. */
int ramgpu_set_launch_shape(ramgpu_ctx *ctx, int sweep, int threads, int persistent_ctas);
int ramgpu_get_launch_shape(ramgpu_ctx *ctx, int *threads4, int *persistent4);
/* Lanes per DRIFTMU line: 4 (NPA >= 24), 2 (adjacent lanes share a line,
 * the default for NPA >= 12) or 1.  Results are the same bit for bit; the
 * autotuner tries each. */
int ramgpu_set_mu_lanes(ramgpu_ctx *ctx, int lanes);
/* Autotuner: for each sweep in turn, tries 32/64/128/256 threads per CTA,
 * each with a one-unit-per-CTA grid and a persistent grid (resident CTAs x
 * SMs), timing whole ram_run steps on the context's active items (best of
 * reps), keeps the fastest, then times 1, 2, 4 and 8 item groups
 * (ramgpu_set_step_groups) on those shapes and keeps the fastest, and
 * restores F2 afterwards (it allocates a temporary snapshot).  best_ms4
 * (may be NULL) receives the best step time of each sweep's round. */
int ramgpu_autotune(ramgpu_ctx *ctx, double dts, int reps, double *best_ms4);
/* The best whole-step trial time of the last ramgpu_autotune for each sweep
 * (R, P, E, MU) with a plain grid and with a persistent grid [ms]; 0 where
 * that kind was not tried (diagnostics: why the tuner chose what it chose). */
int ramgpu_autotune_trials(ramgpu_ctx *ctx, double *plain_ms4, double *persistent_ms4);

/* ---- status word ---------------------------------------------------------
 * The reference stops when a moment is no longer finite (ANISCH,
 * src/ModRamRun.f90:410-413); the library reports instead.  One device pass
 * over the active items counts non-finite F2 cells and moments, the
 * sweeps of the last call whose largest Courant number exceeded 1 (the
 * DtDrift* of that sweep is then below FracCFL*DTs) and, with the check
 * on, the clip events of the last call. */
typedef struct {
    long long f2_nonfinite;       /* NaN or infinite F2 cells of the active items */
    long long moments_nonfinite;  /* NaN or infinite PPERT/PPART values */
    long long cfl_over;           /* (item, sweep) pairs of the last call with a Courant number > 1 */
    long long clips;              /* cells the last call's sweeps clipped to 1e-15 (F2 < 0 after an
                                     update, src/ModRamDrift.f90:187-190); counted only while
                                     ramgpu_set_check is on, else 0 */
    int first_member;             /* first item (list order) holding a non-finite value: member, */
    int first_species;            /* species; -1, -1 if none */
} ramgpu_status;
/* Runs the pass now (synchronises) and fills *st (may be NULL); returns
 * RAMGPU_ERR_NUMERIC when a non-finite value was found, else RAMGPU_OK. */
int ramgpu_check(ramgpu_ctx *ctx, ramgpu_status *st);
/* F2 diagnostics of (member, s) in one device pass (no reference
 * counterpart: the reductions the reference's logs would need, done where
 * F2 lives): the smallest and largest F2 over all cells (exact), and the
 * number content, the sum of F2*WE(K)*WMU(L) over the cells the sweeps
 * update (I >= 2, J <= NT-1, K >= 2, 2 <= L <= NPA-1), which closed
 * boundaries conserve.  The sum runs in a fixed order: the same bits on
 * every call.  Any output may be NULL; synchronises the context's stream. */
int ramgpu_f2_stats(ramgpu_ctx *ctx, int member, int s, double *f2_min, double *f2_max, double *content);
/* With enable != 0 every ramgpu_ram_run / _async / ramgpu_ram_run_host
 * appends the pass to the call (inside its graph); ramgpu_ram_run and
 * ramgpu_ram_run_host then return RAMGPU_ERR_NUMERIC after a call that
 * left a non-finite value, and ramgpu_last_status gives the word of the
 * last call that ran the pass (for _async: after the stream was
 * synchronised).  Off by default. */
int ramgpu_set_check(ramgpu_ctx *ctx, int enable);
int ramgpu_last_status(ramgpu_ctx *ctx, ramgpu_status *st);

/* Number of kernel launches this context has issued (diagnostics). */
long long ramgpu_launch_count(const ramgpu_ctx *ctx);
/* Bounds-checked builds (no reference counterpart): libramgpu_bounds.so is
 * the same library compiled with RAMGPU_BOUNDS_CHECK, whose sweep and
 * transposed-sweep kernels test every line's index ranges (work item,
 * slot, first and last cell, table rows, coefficient-store item) before
 * touching it, count a failed test in the context's log and skip that line.
 * *checked: 1 in such a build, 0 otherwise (the log is then empty);
 * *failures: failed tests since ramgpu_create; *check, *value: the id of the
 * first failed test (1-4 the R, P, E, MU sweeps, 11-14 their transposes; 0
 * when none failed) and the line it was testing.  Any pointer may be NULL.
 * Synchronises the context's stream. */
int ramgpu_bounds_report(ramgpu_ctx *ctx, int *checked, long long *failures, int *check, long long *value);

/* Per-kernel timing with CUDA events recorded on the context's stream
 * around every launch group (diagnostics; no reference counterpart).
 * Kernel classes: 0 member tables, 1 DRIFTR ghost planes, 2 DRIFTR, 3 DRIFTP,
 * 4 DRIFTE, 5 DRIFTMU (+fused loss), 6 periodic copy/mask, 7 ANISCH,
 * 8 DTs tables, 9 SUMRC/loss bookkeeping, 10 pitch-angle diffusion.
 * ramgpu_kernel_times synchronises,
 * adds the elapsed times of completed launches into ms[16] and counts[16]
 * (caller-zeroed) and forgets them. */
#define RAMGPU_NKCLASS 16
/* Measured FP64 fma throughput of the current device in lane-operations
 * per second (a dependent-free fma loop over 8 x SMs x 256 threads); the
 * denominator of the FP64 roofline this path is bound by on GB300. */
int ramgpu_probe_fp64(double *lane_ops_per_s);
/* Measured L2 read bandwidth of the current device in bytes per second
 * (16-byte loads that bypass L1, 200 passes over a 32 MB buffer held in
 * L2); the denominator of the sweeps' L2 view (no reference counterpart). */
int ramgpu_probe_l2(double *bytes_per_s);
/* Device self-test of the integer-pipe FP64 multiply the sweeps use, bit
 * for bit against the FP64 unit on n random operand pairs (normal, short
 * significands and ties, zeros, subnormals, infinities, NaN, extreme
 * exponents); *mismatches receives the count of differing results. */
int ramgpu_selftest_arith(long long n, unsigned long long seed, long long *mismatches);
int ramgpu_set_timing(ramgpu_ctx *ctx, int enable);
int ramgpu_kernel_times(ramgpu_ctx *ctx, double *ms, long long *counts);

/* ---- frozen-limiter adjoint (no reference counterpart) ------------------- */

/* One log-flux observation: FLUX = F2/FFACTOR/FNHS of (member, s) at
 * energy bin k and pitch-angle bin l (0-based, both >= 1 as FLUX is defined
 * for K, L >= 2), bilinear in L-shell (between LZ(I), I >= 2) and in MLT
 * (periodic), taken after ram_run call `call` (0-based) of the window.
 * The misfit is J = sum over observations of (log flux_model - log_obs)^2. */
typedef struct {
    int member, s, call, k, l;
    double lshell;   /* [RE] */
    double mlt;      /* [h] */
    double log_obs;
} ramgpu_obs;

/* Forward pass of a window of ncalls ram_run calls of length dts from the
 * current F2, with Kp of call c and member m in kp[c*n_members + m] (VOLS).
 * Saves a checkpoint of F2 every k_ckpt calls, evaluates J per member into
 * J[n_members] and leaves F2 at the end of the window (the moments are
 * those of the window's last call).  The calls of the last nkeep checkpoint
 * segments record every limiter branch and clip into a ring of branch
 * records (4 bits per face and sweep: 4 bytes per cell, item and call) that
 * holds as many segments as the record budget allows
 * (ramgpu_set_adj_record_budget; at least one, two when the window has
 * several segments and the overlapped recomputation is on); the earlier calls, which ramgpu_adj_backward recomputes from their
 * checkpoints, run the plain step (the same F2 bits).  ramgpu_adj_digest
 * returns a digest of the recorded pattern.  The checkpoint buffer and the
 * ring are allocated by the first window and reused by later windows of the
 * same shape. */
int ramgpu_adj_forward(ramgpu_ctx *ctx, int ncalls, double dts, const double *kp, int k_ckpt,
                       const ramgpu_obs *obs, int nobs, double *J);
/* Backward pass: gradients of J with respect to the window's initial F2
 * (grad_f2: n_members*ns*NR*NT*NE*NPA, per (member, s) the Fortran-order
 * F2(S,:,:,:,:)) and to FGEOS (grad_fgeos: n_members*ns*NT*NE*NPA), with the
 * limiter branches frozen as recorded.  Each checkpoint segment before the
 * kept ones is recomputed from its checkpoint with recording, then every
 * call is transposed in reverse order; when the ring keeps every segment
 * (or k_ckpt >= ncalls) nothing is recomputed.  With the overlapped
 * recomputation on (ramgpu_set_adj_overlap) segment s-1 is recomputed on a
 * second stream, with its own per-member tables, while segment s is
 * transposed; the results are the same bits.  Either
 * output may be NULL; both may be host or device memory.  On return F2 is
 * the window's initial state again. */
int ramgpu_adj_backward(ramgpu_ctx *ctx, double *grad_f2, double *grad_fgeos);
/* Device bytes the adjoint's branch-record ring may take: bytes < 0 (the
 * default) means half of the free device memory when ramgpu_adj_forward
 * starts; a budget below one segment keeps one segment (two with the
 * overlapped recomputation), so every earlier segment is recomputed from
 * its checkpoint. */
int ramgpu_set_adj_record_budget(ramgpu_ctx *ctx, long long bytes);
/* Overlapped recomputation in ramgpu_adj_backward (on = 1, the default):
 * needs a ring of two segments (ramgpu_adj_forward then keeps at least
 * two) and device memory for a copy of the per-member tables and ghost
 * planes, allocated by the first backward pass that recomputes. */
int ramgpu_set_adj_overlap(ramgpu_ctx *ctx, int on);
/* Checkpoint segments of the last ramgpu_adj_forward and how many of them
 * (the last ones) the record ring keeps. */
int ramgpu_adj_segments(ramgpu_ctx *ctx, int *nseg, int *nkeep);
/* Digest of every branch recorded by the last ramgpu_adj_forward (the
 * calls of the kept segments): equal digests mean the same frozen-limiter
 * pattern. */
int ramgpu_adj_digest(ramgpu_ctx *ctx, unsigned long long *digest);
/* Copy of the branch record of one call of a kept checkpoint segment of
 * the last ramgpu_adj_forward: 8 sweeps (R,P,E,MU,MU,E,P,R) x active items x
 * NR*NT*NE*NPA bytes, per face the limiter case (bits 0-2: 0 upwind only,
 * 1 beta*D, 2 X, 3 D, 4 beta*X) and bit 3 set when the updated cell was
 * clipped (diagnostics; the device keeps four bits per face, the forward
 * and reverse sweeps of one direction sharing a byte).  Available until a
 * ramgpu_adj_backward that had to recompute earlier segments replaces it. */
int ramgpu_adj_record(ramgpu_ctx *ctx, int call, unsigned char *out);
/* The last window run again from the current F2 with every limiter branch
 * and clip taken from the record (the frozen-limiter scheme that
 * ramgpu_adj_backward differentiates, which is affine in F2 and FGEOS):
 * J[n_members] of that run; F2 ends at the window's end.  Needs every call's
 * record: k_ckpt >= ncalls, or a ring that keeps every segment.  With the recorded
 * F2 it reproduces the recorded run bit for bit; it exists to check the
 * adjoint by finite differences on long windows, where unfrozen
 * perturbations cross limiter kinks. */
int ramgpu_adj_replay(ramgpu_ctx *ctx, double *J);

/* ---- snapshots ----------------------------------------------------------- */

/* The evolving state of a context in one file, the counterpart of RAM's
 * write_restart / read_restart (src/ModRamRestart.f90:12,386) for the state
 * this library owns: per member its species set, active flag, Kp or
 * explicit potential and VT, per (member, species) F2, FGEOS and the last
 * moments.  Grid and field tables are inputs and are set again by the
 * caller.  Layout (little-endian): a 128-byte header "RAMGPUS1", version 1,
 * header size, NR, NT, NE, NPA, NS, members (int32), flags, 0 (uint32), the
 * caller's time (double), payload bytes, checksum (uint64: FNV-1a over the
 * payload's 64-bit words), zero padding; then per member {species mask,
 * active, VT mode, 0 (int32), Kp, VT(NR+1,NT)} and per slot {F2, FGEOS,
 * PPERT, PPART} in the ABI's layouts.  ramgpu_load_state checks the whole
 * file (RAMGPU_ERR_IO: unreadable or checksum mismatch; RAMGPU_ERR_ARG:
 * other dimensions) before it changes anything, and returns the saved time
 * in *time (may be NULL).  Both synchronise the context's stream. */
typedef struct {
    int nr, nt, ne, npa, ns, n_members;
    unsigned flags;
    double time;
} ramgpu_snapshot_info_t;
int ramgpu_save_state(ramgpu_ctx *ctx, const char *path, double time);
int ramgpu_load_state(ramgpu_ctx *ctx, const char *path, double *time);
/* Header of a snapshot file after checking its checksum; needs no context
 * (and no GPU).  Errors go to ramgpu_last_error(NULL, ...). */
int ramgpu_snapshot_info(const char *path, ramgpu_snapshot_info_t *info);

/* ---- no-allocation variant --------------------------------------------- */

/* SETRC = sum EKEV*F2*WE*WMU (the energy-content sum of SUMRC) of one
 * species' F2 already on the device, for callers that cannot allocate
 * device memory: a host model that gives every device byte to its own pool
 * and forbids libraries to call cudaMalloc, or code that must not call
 * allocation APIs (cudaMalloc may synchronise the device) while work is in
 * flight.  It allocates nothing: its only scratch is a fixed 36 KiB array in
 * this library's device image, so NE and NPA are limited to 1024 and larger
 * sizes are rejected with RAMGPU_ERR_ARG.
 *   f2_dev : device pointer, (NR,NT,NE,NPA) Fortran order (e.g. from
 *            ramgpu_f2_device_ptr);  we, wmu, ekev : host arrays (NE)/(NPA)/(NE)
 *   stream : cudaStream_t or NULL;  setrc : host, receives the sum.
 * The first call on a device looks up the scratch address on that device
 * (make it before any stream capture) and keeps it for the life of the
 * process, so do not call this after a cudaDeviceReset of that device.
 * Every call reuses the same scratch, which keeps the last call's contents;
 * calls that overlap on the GPU race.  The call is synchronous (it waits for
 * its stream): made on a stream under capture it returns RAMGPU_ERR_STATE
 * and leaves the capture intact.
 * Errors are reported by ramgpu_last_error(NULL, ...).  No counterpart in the
 * reference: it exists only for callers that cannot allocate. */
int ramgpu_sumrc_noalloc(const double *f2_dev, int nr, int nt, int ne, int npa,
                         const double *we, const double *wmu, const double *ekev,
                         void *stream, double *setrc);

#ifdef __cplusplus
}
#endif
#endif
