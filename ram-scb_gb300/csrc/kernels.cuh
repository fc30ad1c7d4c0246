// kernels.cuh -- launchers shared between the kernel files and the C ABI.
#pragma once
#include <string>

#include "ramgpu_internal.cuh"

namespace ramgpu {

// DRIFTR boundary ghost F(NR+n) = FGEOS(S,J,K,L)*CONFn*FNHS(NR,J,L), or 0 outside
// the magnetopause (src/ModRamDrift.f90:161-167).  0-based j,k,l.
__device__ __forceinline__ double ghost_value(const Dev& d, int slot, int j, int k, int l,
                                              double conf) {
  const int nr = d.nr;
  if (d.outside[(long long)j * nr + nr - 1] == 1) return 0.0;
  const double fg = d.fgeos[(long long)slot * d.nt * d.ne * d.npa + ((long long)l * d.ne + k) * d.nt + j];
  return fg * conf * d.fnhs[((long long)l * d.nt + j) * d.nf + nr - 1];
}

// Sign test of CDriftR(NR,J,K,L) exactly as the sweep computes it.
__device__ __forceinline__ bool inflow_line(const Dev& d, int m, int j, int l, double p4) {
  const int nr = d.nr;
  const double c = fma(d.grt[((long long)l * d.nt + j) * nr + nr - 1], p4,
                       d.cr[((long long)m * d.nt + j) * nr + nr - 1]);
  return is_neg(c);
}

// Stale F(NR+1) seen by outflow line (J,K,L): the value written by the most
// recent inflow line before it in the K->L->J order of DRIFTR, 0 if none.
__device__ __forceinline__ double stale_ghost(const Dev& d, int m, int slot, int j, int k, int l,
                                              double p4) {
  for (int jj = j - 1; jj >= 0; --jj)
    if (inflow_line(d, m, jj, l, p4)) return ghost_value(d, slot, jj, k, l, d.conf1);
  return d.plane_carry[(long long)slot * d.ne * d.npa + (long long)k * d.npa + l];
}

// Thread-local error text returned by ramgpu_last_error(NULL, ...).
void set_thread_error(const std::string& msg);

// rec (may be null): per-face branch record of the frozen-limiter adjoint,
// (items, ncell) bytes for this sweep instance.
// FGEOS index (L*NE+K)*NT+J of the inflow line whose F(NR+1) outflow line
// (J,K,L) reads as its stale ghost, or -1 (value 0) -- the source that
// stale_ghost() takes its value from.
__device__ __forceinline__ int stale_ghost_src(const Dev& d, int m, int slot, int j, int k, int l,
                                               double p4) {
  for (int jj = j - 1; jj >= 0; --jj)
    if (inflow_line(d, m, jj, l, p4)) return (l * d.ne + k) * d.nt + jj;
  return d.plane_carry_src[(long long)slot * d.ne * d.npa + (long long)k * d.npa + l];
}

// rec: branch record of the sweep, written (replay false) or, with replay
// true, read back to run the sweep with those branches and clips frozen;
// rsh: its nibble of the record bytes (4: high, forward half, written
// first; 0: low, reverse half, ORed in).
void launch_sweep_r(const Dev& d, double dts, bool cfl, cudaStream_t st, unsigned char* rec = nullptr,
                    bool replay = false, int co = 0, int rsh = 0);
void launch_sweep_p(const Dev& d, double dts, bool cfl, cudaStream_t st, unsigned char* rec = nullptr,
                    bool replay = false, int co = 0, int rsh = 0);
void launch_sweep_e(const Dev& d, double dts, bool cfl, cudaStream_t st, unsigned char* rec = nullptr,
                    bool replay = false, int co = 0, int rsh = 0);
void launch_sweep_mu(const Dev& d, double dts, bool cfl, int loss_mode, const double* loss,
                     cudaStream_t st, unsigned char* rec = nullptr, bool replay = false, int co = 0, int rsh = 0);

int sweep_max_blocks_per_sm(int w, int blk);

void launch_field_tables(const Dev& d, cudaStream_t st);
void launch_species_static(const Dev& d, unsigned long long* sep_dev, cudaStream_t st);
void launch_dts_tables(const Dev& d, double dts, cudaStream_t st);
void launch_member_coef(const Dev& d, double dts, cudaStream_t st);
void launch_ghost(const Dev& d, cudaStream_t st);
void launch_loss_apply(const Dev& d, const double* table, cudaStream_t st);
void launch_finish(const Dev& d, cudaStream_t st);
void launch_moments(const Dev& d, cudaStream_t st);
void launch_anisch_state(const Dev& d, cudaStream_t st);
void launch_sumrc(const Dev& d, double* part, int nblk, cudaStream_t st);
void launch_flux(const Dev& d, int slot, int s, double* out, cudaStream_t st);

// ---- frozen-limiter adjoint (adjoint.cu)
struct ObsDev {
  int member, slot, call, k, l;
  int item;            // place of (member, s) in the work list
  int i0, j0, j1;      // 0-based corner indices: I = i0, i0+1; J = j0, j1
  double wi, wj;       // bilinear weights of the upper corners
  double log_obs;
};
// co (DRIFTE only): 0 compute C, 1 compute and store it, 2 load it (needs
// the DRIFTE coefficient store).
void launch_adj_sweep(const Dev& d, int w, const unsigned char* rec, int rsh, cudaStream_t st, int co = 0,
                      const double* loss = nullptr);
void launch_adj_tail(const Dev& d, cudaStream_t st);
void launch_obs_fwd(const Dev& d, const ObsDev* obs, int nobs, int call, double* fm, double* J,
                    cudaStream_t st);
void launch_obs_adj(const Dev& d, const ObsDev* obs, int nobs, int call, const double* fm,
                    cudaStream_t st);
void launch_digest(const unsigned char* rec, long long n, unsigned long long* out, cudaStream_t st);

// implicit pitch-angle diffusion (padif.cu)
void launch_padif_tables(const Dev& d, double dts, cudaStream_t st);
void launch_padif(const Dev& d, const double* loss, cudaStream_t st);

// bounce integrals of computehI (bounce.cu); line arrays (nthe, NR, NT),
// per-angle arrays (NR*NT lines, NPA), outputs (NR, NT, NPA)
struct BounceDev {
  int nr, nt, npa, nthe, ieq;
  const double *chi, *x, *y, *z, *dens, *mu;
  double* b;                     // copied in, equator-fixed in place
  const int* outside;            // (NR, NT)
  int* line_ok;
  double *length, *r0;           // per line
  double *mirror, *mirror2, *yi, *yh, *yd;
  unsigned char *st, *sd;
  double *h_out, *i_out, *d_out, *m_out;
};
void launch_bounce(const BounceDev& q, cudaStream_t st);
// computehI's field-table fill: inputs h, fi, hd (NR,NT,NPA) and beq (NR,NT)
// (modified: the outside-magnetopause copy), outputs the context's tables
struct HiDev {
  int nr, nt, npa;
  double dthi, bnormal, lz0;
  const int* outside;
  const double *pa, *pabn_rev;   // PA (NPA); PAbn(NPA-1:2:-1) (NPA-2)
  double *h, *fi, *hd, *beq, *hb, *ib, *scratch;
  double *fnhs, *fnis, *hdns, *bounhs, *bounis, *didt, *dibndt, *bnes, *dbdt, *eir, *eip;
};
void launch_hi_fill(const HiDev& q, cudaStream_t st);

// virtual spacecraft and SCB hand-off (outputs.cu)
struct SatDev {
  int member;
  unsigned active_mask;  // bit s: (member, s) is active
  int i0, j0, j1;        // bilinear stencil, as ObsDev
  double wi, wj;
};
void launch_fly_sats(const Dev& d, const SatDev* sats, int nsat, double* sat_flux, double* omni,
                     cudaStream_t st);
void launch_sum_pressure(const Dev& d, int member, unsigned mask, double* pall, double* ppar,
                         cudaStream_t st);

// F2 / moments in the reference's layout (layout.cu): slots[s*stride + c]
// <-> ref[c*ns + s] for cells c in [c0, c1); ref may be host memory the
// device reaches (mapped page-locked, or pageable over a coherent link).
void launch_ref_gather(const double* ref, double* slots, int ns, long long stride, long long c0, long long c1,
                       int nsm, cudaStream_t st);
void launch_ref_scatter(const double* slots, double* ref, int ns, long long stride, long long c0, long long c1,
                        int nsm, cudaStream_t st);

void launch_selftest_mul(long long n, unsigned long long seed, unsigned long long* bad, cudaStream_t st);
// Status word of the active items (status.cu): st[5] device words.
void launch_status(const Dev& d, unsigned long long* st, cudaStream_t s);

}  // namespace ramgpu
