// tables.cu -- coefficient tables, losses, moments and bookkeeping kernels.
//
// The drift coefficients of the reference are recomputed per cell and per
// call; here they are split into factors that change at different rates:
//   fields only (set_fields)      : grt, gpt, gre, gpe, ze, wet, gmr, gmp, zm, hm, cmu0, rho
//   species only (set_grid)       : eb, ek, kap, ANISCH weights mw_a (mw_be, mw_ba: fields)
//   DTs (when DTs changes)        : p4, p2, edot, cmudot, wm, CHARGE/ATMOL factors
//   DTs and fields                : mij (E x B factors per I, J)
//   potential VT (every ram_run)  : cr, ca, ue, um
// so that a sweep face needs one or two FP64 operations for its coefficient.
// Formulas restate src/ModRamDrift.f90:36-88 (DRIFTPARA), :118-146 (DRIFTR),
// :232-239 (DRIFTP), :310-342 (DRIFTE), :415-433 (DRIFTMU),
// src/ModRamLoss.f90:19-170 (CEPARA), :485-507 (ATMOL),
// src/ModRamRun.f90:45-54 (VOLS), :186-201 (periodic copy, mask),
// :231-259 (SUMRC), :343-404 (ANISCH moments), :208-222 (FLUX).
#include <math.h>
#include "kernels.cuh"

namespace ramgpu {

// 1-based accessors in the reference's index order (I, J, L) / (I, J).
#define NRr (d.nr)
#define NTt (d.nt)
#define FIX(I, J, L) ((((long long)(L)-1) * d.nt + ((J)-1)) * d.nf + ((I)-1))
#define BIX(I, J) (((long long)(J)-1) * d.nf + ((I)-1))
#define TIX(I, J, L) ((((long long)(L)-1) * d.nt + ((J)-1)) * d.nr + ((I)-1))
#define FNHS(I, J, L) d.fnhs[FIX(I, J, L)]
#define FNIS(I, J, L) d.fnis[FIX(I, J, L)]
#define BOUNHS(I, J, L) d.bounhs[FIX(I, J, L)]
#define BOUNIS(I, J, L) d.bounis[FIX(I, J, L)]
#define HDNS(I, J, L) d.hdns[FIX(I, J, L)]
#define DIDT(I, J, L) d.didt[FIX(I, J, L)]
#define DIBNDT(I, J, L) d.dibndt[FIX(I, J, L)]
#define BNES(I, J) d.bnes[BIX(I, J)]
#define DBDT(I, J) d.dbdt[BIX(I, J)]
#define EIR(I, J) d.eir[BIX(I, J)]
#define EIP(I, J) d.eip[BIX(I, J)]
#define RLZ(I) d.rlz[(I)-1]
#define LZ(I) d.lz[(I)-1]
#define EKEV(K) d.ekev[(K)-1]
#define EBND(K) d.ebnd[(K)-1]
#define WE(K) d.we[(K)-1]
#define MU(L) d.mu[(L)-1]
#define WMU(L) d.wmu[(L)-1]

__device__ __forceinline__ void wrapj(int J, int nt, int& J0, int& J1) {
  J0 = J - 1;
  if (J == 1) J0 = nt - 1;
  J1 = J + 1;
  if (J == nt) J1 = 2;
}

// ------------------------------------------------------------ field tables
__global__ void k_field_tables(Dev d) {
  const long long n = (long long)d.nr * d.nt * d.npa;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int I = 1 + (int)(t % d.nr);
  const int J = 1 + (int)((t / d.nr) % d.nt);
  const int L = 1 + (int)(t / ((long long)d.nr * d.nt));
  const double MDR = d.mdr, DPHI = d.dphi;
  int J0, J1;
  wrapj(J, d.nt, J0, J1);
  // DRIFTR gradient-curvature factor (src/ModRamDrift.f90:140-144)
  {
    double CGR1 = FNIS(I + 1, J1, L) + FNIS(I, J1, L) - FNIS(I + 1, J0, L) - FNIS(I, J0, L);
    double CGR2 = BNES(I + 1, J1) + BNES(I, J1) - BNES(I + 1, J0) - BNES(I, J0);
    double CGR3 = CGR1 + (FNIS(I + 1, J, L) + FNIS(I, J, L) - 2 * FNHS(I + 1, J, L) - 2 * FNHS(I, J, L))
                             * CGR2 / 2. / (BNES(I + 1, J) + BNES(I, J));
    d.grt[t] = CGR3 / (FNHS(I, J, L) + FNHS(I + 1, J, L)) / 2. / (BNES(I, J) + BNES(I + 1, J))
               / (RLZ(I) + 0.5 * MDR);
  }
  double gpt = 0, gre = 0, gpe = 0, ze = 0, wet = 0, gmr = 0, gmp = 0, zm = 0, hm = 0, cmu0 = 0;
  if (I >= 2) {
    const double R = RLZ(I);
    // DRIFTP (src/ModRamDrift.f90:232-237), J = 2..NT only
    if (J >= 2) {
      int Jp = J + 1;
      if (J == d.nt) Jp = 2;
      double GPA1 = FNIS(I, J, L) + FNIS(I, Jp, L)
                    + (FNIS(I + 1, Jp, L) + FNIS(I + 1, J, L) - FNIS(I - 1, J, L) - FNIS(I - 1, Jp, L)) * R / 2. / MDR;
      double GPA2 = R / 4. / MDR * (FNIS(I, J, L) + FNIS(I, Jp, L) - 2 * FNHS(I, J, L) - 2 * FNHS(I, Jp, L))
                    * (BNES(I + 1, Jp) + BNES(I + 1, J) - BNES(I - 1, J) - BNES(I - 1, Jp)) / (BNES(I, J) + BNES(I, Jp));
      gpt = -(GPA1 + GPA2) / (FNHS(I, J, L) + FNHS(I, Jp, L)) / (BNES(I, J) + BNES(I, Jp));
    }
    // DRIFTE (src/ModRamDrift.f90:323-341), J2 = J1
    {
      const double fis = FNIS(I, J, L), fhs = FNHS(I, J, L), b = BNES(I, J);
      double GPA = (1. - fis / 2. / fhs) / b;
      double GPR1 = GPA * (BNES(I + 1, J) - BNES(I - 1, J)) / 2. / MDR;
      double GPR2 = -fis / fhs / R;
      double GPR3 = -(FNIS(I + 1, J, L) - FNIS(I - 1, J, L)) / 2. / MDR / fhs;
      double GPP1 = GPA * (BNES(I, J1) - BNES(I, J0)) / 2. / DPHI;
      double GPP2 = -(FNIS(I, J1, L) - FNIS(I, J0, L)) / 2. / DPHI / fhs;
      double DRD2 = (FNIS(I, J1, L) - FNIS(I, J0, L)) / 2. / DPHI
                    + (fis - 2 * fhs) * (BNES(I, J1) - BNES(I, J0)) / 4 / b / DPHI;
      double DPD2 = fis + (FNIS(I + 1, J, L) - FNIS(I - 1, J, L)) * R / 2 / MDR
                    + R * (fis - 2 * fhs) / 4 / MDR * (BNES(I + 1, J) - BNES(I - 1, J)) / b;
      double dBdt1 = DBDT(I, J) * (1. - fis / 2. / fhs) * R / b;
      double dIdt1 = -DIDT(I, J, L) * R / fhs;
      gre = GPR1 + GPR2 + GPR3;
      gpe = GPP1 + GPP2;
      ze = dBdt1 + dIdt1;
      // EDT1 = eb(K)/(FNHS*RLZ*BNES); inner = UE + eb(K)*wet
      wet = (gre * DRD2 * R - gpe * DPD2) / fhs / R / b;
    }
    // DRIFTMU (src/ModRamDrift.f90:418-433)
    {
      const double bis = BOUNIS(I, J, L), bhs = BOUNHS(I, J, L), b = BNES(I, J);
      cmu0 = bis / bhs;
      double GMR1 = (BNES(I + 1, J) - BNES(I - 1, J)) / 4 / MDR / b;
      double GMR2 = 1 / R;
      double GMR3 = (BOUNIS(I + 1, J, L) - BOUNIS(I - 1, J, L)) / 2 / MDR / bis;
      double GMP1 = (BNES(I, J1) - BNES(I, J0)) / 4 / DPHI / b;
      double GMP2 = (BOUNIS(I, J1, L) - BOUNIS(I, J0, L)) / 2 / DPHI / bis;
      double DRM2 = (BOUNIS(I, J1, L) - BOUNIS(I, J0, L)) / 2 / DPHI
                    + (bis - 2 * bhs) * (BNES(I, J1) - BNES(I, J0)) / 4 / b / DPHI;
      double DPM2 = bis + (BOUNIS(I + 1, J, L) - BOUNIS(I - 1, J, L)) * R / 2 / MDR
                    + (bis - 2 * bhs) * R / 4 / MDR * (BNES(I + 1, J) - BNES(I - 1, J)) / b;
      double dBdt2 = DBDT(I, J) / 2. / b * R;
      double dIbndt2 = DIBNDT(I, J, L) * R / bis;
      gmr = GMR1 + GMR2 + GMR3;
      gmp = GMP1 + GMP2;
      zm = dBdt2 + dIbndt2;
      hm = (gmr * DRM2 * R - gmp * DPM2) / bhs / R / b;
    }
    if (L == 1) d.rho[(long long)(J - 1) * d.nr + (I - 1)] =
        FNHS(I, J, d.npa) * MU(d.npa) / FNHS(I, J, d.npa - 1) / MU(d.npa - 1);
  } else if (L == 1) {
    d.rho[(long long)(J - 1) * d.nr] = 0.0;
  }
  d.gpt[t] = gpt;
  d.gre[t] = gre; d.gpe[t] = gpe; d.ze[t] = ze; d.wet[t] = wet;
  d.gmr[t] = gmr; d.gmp[t] = gmp; d.zm[t] = zm; d.hm[t] = hm; d.cmu0[t] = cmu0;
}

void launch_field_tables(const Dev& d, cudaStream_t st) {
  long long n = (long long)d.nr * d.nt * d.npa;
  k_field_tables<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d);
}

// ------------------------------------------------------- species constants
__global__ void k_species_static(Dev d) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.ns * d.ne) return;
  const int s = t / d.ne, K = 1 + t % d.ne;
  const double* grel = d.grel + s * d.ne;
  const double* grbnd = d.grbnd + s * d.ne;
  const double QS = (double)d.qs[s];
  d.eb[t] = EBND(K) * 1e3 * (grbnd[K - 1] + 1) / 2 / grbnd[K - 1] / QS;
  d.ek[t] = EKEV(K) * 1e3 * (grel[K - 1] + 1) / 2 / grel[K - 1] / QS;
  if (K == 1) {
    const double G1 = grel[0], G2 = grel[1];
    d.kap[2 * s + 1] = G1 / G2 * sqrt((G2 * G2 - 1) / (G1 * G1 - 1));
    const double EZERO = EKEV(1) - WE(1);
    const double GRZERO = 1. + EZERO * 1000. * kQ / d.rmas[s] / kCS / kCS;
    d.kap[2 * s + 0] = GRZERO / G1 * sqrt((G1 * G1 - 1) / (GRZERO * GRZERO - 1));
  }
}

// ANISCH weights (src/ModRamRun.f90:372-374 and :380-389).  The reference's
// ERNM = WMU(L)/FFACTOR(S,I,K,L)/FNHS(I,J,L), EPMA = ERNM*MU^2,
// EPME = ERNM-EPMA, with the energy weight EPP(S,K) and the band factors
// RFAC folded in, is the product of a species factor and a field factor:
//   mw_a (S,L,K,I)  = RFAC*EPP(S,K)/FFACTOR(S,I,K,L)
//   mw_be(L,J,I)    = WMU(L)/FNHS(I,J,L)*(1-MU(L)^2)   (as B - B*MU*MU)
//   mw_ba(L,J,I)    = 2*WMU(L)/FNHS(I,J,L)*MU(L)^2
// so PPERT = sum over K>=2, L<=u of (F2*mw_a)*mw_be and PPART likewise.
// ARRAYS builds FFACTOR(S,I,K,L) = LZ^2*GREL/SQRT(GREL^2-1)*MU(L) with
// FFACTOR(S,I,K,1) = FFACTOR(S,I,K,2) (src/ModRamInit.f90:565-568): then the
// species factor leaves the L-sum,
//   mws_a(S,K,I)    = RFAC*EPP(S,K)*MU(2)/FFACTOR(S,I,K,2)
//   mws_be(L,J,I)   = mw_be/MU'(L),  mws_ba = mw_ba/MU'(L),  MU'(1) = MU(2),
// PPERT = sum over K of mws_a * sum over L of F2*mws_be: two fma per cell.
// k_mom_sep_check measures how far the given FFACTOR is from that form.
// The reference sums the same products band by band (khi = 6,10,25,30,NE)
// and scales each band by RFAC; the orders differ by rounding only.  All
// tables stay in L2.
__global__ void k_moment_weights(Dev d) {
  const long long na = (long long)d.ns * d.npa * d.ne * d.nr;
  const long long nb = (long long)d.npa * d.nt * d.nr;
  const long long nsa = (long long)d.ns * d.ne * d.nr;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const double RFAC = 4 * kPI / (kCS * 100);
  if (t < na) {
    const int I = 1 + (int)(t % d.nr);
    const int K = 1 + (int)((t / d.nr) % d.ne);
    const int L = 1 + (int)((t / ((long long)d.nr * d.ne)) % d.npa);
    const int s = (int)(t / ((long long)d.nr * d.ne * d.npa));
    const double ff = d.ffactor[(long long)s * d.nr * d.ne * d.npa + (((long long)L - 1) * d.ne + (K - 1)) * d.nr + (I - 1)];
    d.mw_a[t] = RFAC * d.epp[s * d.ne + K - 1] / ff;
  } else if (t < na + nb) {
    const long long c = t - na;
    const int I = 1 + (int)(c % d.nr);
    const int J = 1 + (int)((c / d.nr) % d.nt);
    const int L = 1 + (int)(c / ((long long)d.nr * d.nt));
    const double B = WMU(L) / FNHS(I, J, L);
    const double BA = B * MU(L) * MU(L);
    d.mw_be[c] = B - BA;
    d.mw_ba[c] = 2 * BA;
    const double mup = L == 1 ? MU(2) : MU(L);
    d.mws_be[c] = (B - BA) / mup;
    d.mws_ba[c] = (2 * BA) / mup;
  } else if (t < na + nb + nsa) {
    const long long c = t - na - nb;
    const int I = 1 + (int)(c % d.nr);
    const int K = 1 + (int)((c / d.nr) % d.ne);
    const int s = (int)(c / ((long long)d.nr * d.ne));
    const double ff2 = d.ffactor[(long long)s * d.nr * d.ne * d.npa + ((long long)1 * d.ne + (K - 1)) * d.nr + (I - 1)];
    d.mws_a[c] = RFAC * d.epp[s * d.ne + K - 1] * MU(2) / ff2;
  }
}

// Largest relative distance, over the summed cells, between the general
// species weight and its separable form mws_a/MU'(L): the maximum of
// |mw_a*MU'(L) - mws_a| / mws_a as bits into *out (atomic max).
__global__ void k_mom_sep_check(Dev d, unsigned long long* out) {
  const long long na = (long long)d.ns * d.npa * d.ne * d.nr;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double dev = 0.0;
  if (t < na) {
    const int I = 1 + (int)(t % d.nr);
    const int K = 1 + (int)((t / d.nr) % d.ne);
    const int L = 1 + (int)((t / ((long long)d.nr * d.ne)) % d.npa);
    const int s = (int)(t / ((long long)d.nr * d.ne * d.npa));
    if (I >= 2 && K >= 2 && L <= d.upa_mom[I - 1]) {
      const double ws = d.mws_a[((long long)s * d.ne + (K - 1)) * d.nr + (I - 1)];
      const double mup = L == 1 ? MU(2) : MU(L);
      dev = fabs(d.mw_a[t] * mup - ws) / ws;
      if (!(dev == dev)) dev = 1.0;  // NaN: not separable
    }
  }
  warp_atomic_max(out, dbits(dev));
}

void launch_species_static(const Dev& d, unsigned long long* sep_dev, cudaStream_t st) {
  int n = d.ns * d.ne;
  k_species_static<<<(n + 127) / 128, 128, 0, st>>>(d);
  const long long na = (long long)d.ns * d.npa * d.ne * d.nr;
  const long long nw = na + (long long)d.npa * d.nt * d.nr + (long long)d.ns * d.ne * d.nr;
  k_moment_weights<<<(unsigned)((nw + 255) / 256), 256, 0, st>>>(d);
  cudaMemsetAsync(sep_dev, 0, sizeof(unsigned long long), st);
  k_mom_sep_check<<<(unsigned)((na + 255) / 256), 256, 0, st>>>(d, sep_dev);
}

// ------------------------------------------------------------- DTs tables
__global__ void k_dts_small(Dev d, double DTs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.ns * d.ne * d.nr) return;
  const int i = t % d.nr, k = (t / d.nr) % d.ne, s = t / (d.nr * d.ne);
  const int I = i + 1, K = k + 1;
  const double g = d.grel[s * d.ne + k], gb = d.grbnd[s * d.ne + k];
  const double QS = (double)d.qs[s];
  const double MDR = d.mdr, DPHI = d.dphi;
  if (i == 0) d.p4[s * d.ne + k] = DTs * EKEV(K) * 1000.0 * (g + 1) / g / DPHI / MDR / QS;
  d.p2[t] = DTs * EKEV(K) * 1000 * (g + 1) / g / (RLZ(I) * RLZ(I)) / DPHI / QS;
  d.edot[t] = EBND(K) * DTs / RLZ(I) * (gb + 1) / gb / 2.;
}

__global__ void k_dts_cells(Dev d, double DTs) {
  const long long n = (long long)d.nr * d.nt * d.npa;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int I = 1 + (int)(t % d.nr);
  const int L = 1 + (int)(t / ((long long)d.nr * d.nt));
  double mudot = 0.0;
  if (L < d.npa) {
    const double MUBOUN = MU(L) + 0.5 * WMU(L);
    mudot = (1. - MUBOUN * MUBOUN) * DTs / 2 / MUBOUN / RLZ(I);
  }
  const double cm = mudot * d.cmu0[t];
  d.cmudot[t] = cm;
  d.wm[t] = -cm * d.hm[t];
}

// CEPARA analytic cross sections and ATMOL factor, per species and cell.
__global__ void k_dts_loss(Dev d, double DTs) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)d.ns * d.ncell) return;
  const int s = (int)(t / d.ncell);
  const long long c = t % d.ncell;
  const int I = 1 + (int)(c % d.nr);
  const int J = 1 + (int)((c / d.nr) % d.nt);
  const int K = 1 + (int)((c / ((long long)d.nr * d.nt)) % d.ne);
  const int L = 1 + (int)(c / ((long long)d.nr * d.nt * d.ne));
  const double V = d.vel[s * d.ne + K - 1];
  double ch = 1.0, at = 1.0;
  const int kind = d.cex_kind[s];
  if (kind >= 1 && kind <= 3 && L >= 2 && K >= 2 && I >= 2) {
    double X = log10(EKEV(K));
    if (X < -2.) X = -2.;
    const double X2 = X * X, X3 = X2 * X, X4 = X2 * X2;
    double Y;
    if (kind == 1) Y = -18.767 - 0.11017 * X - 3.8173e-2 * X2 - 0.1232 * X3 - 5.0488e-2 * X4;
    else if (kind == 2) Y = -20.789 + 0.92316 * X - 0.68017 * X2 + 0.66153 * X3 - 0.20998 * X4;
    else Y = -18.987 - 0.10613 * X - 5.4841E-3 * X2 - 1.6262E-2 * X3 - 7.0554E-3 * X4;
    const double ALPHA = pow(10., Y) * V * HDNS(I, J, L) * DTs;
    ch = exp(-ALPHA);
  }
  if (!(d.flags & 2u) && K >= 2 && I >= 2 && L >= d.upa_atm[I - 1]) {
    const double TAUB = 2 * RLZ(I) / V;
    const double ATLOS = exp(-DTs / TAUB);
    at = pow(ATLOS, 1 / FNHS(I, J, L));
  }
  d.charge[t] = ch;
  d.atm[t] = at;
  d.loss1[t] = ch * at;
  d.loss2[t] = ((ch * at) * at) * ch;
}

// VT-independent parts of the per-call E x B terms, per (I, J) (src/ModRamDrift.f90:118-127,
// :232-239 and DRIFTPARA :60-75), so that each per-call term is one fma on
// the VT combination:
//   CR   = crk*(VT(I,J0)+VT(I+1,J0)-VT(I,J1)-VT(I+1,J1)) + cr0
//   CA   = cak*(VT(I+1,J)+VT(I+1,J1)-VT(I-1,J)-VT(I-1,J1)) + ca0   (I, J >= 2)
//   DRD1 = d1k*(VT(I,J1)-VT(I,J0)) + d10,  DPD1 = p1k*(VT(I+1,J)-VT(I-1,J)) + p10
// (the reference's quotients regrouped; they agree to rounding).  mij is
// (8, NT, NR) in that order: crk, cr0, cak, ca0, d1k, d10, p1k, p10.
__global__ void k_dts_ij(Dev d, double DTs) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = d.nr * d.nt;
  if (t >= n) return;
  const int I = 1 + t % d.nr, J = 1 + t / d.nr;
  int J0, J1;
  wrapj(J, d.nt, J0, J1);
  const double MDR = d.mdr, DPHI = d.dphi;
  const double VR = DTs / MDR / (RLZ(I) + 0.5 * MDR) / 2 / DPHI;
  const double den = BNES(I, J) + BNES(I + 1, J);
  double v[8] = {VR / den, (EIP(I, J) + EIP(I + 1, J)) / den * DTs / MDR, 0., 0., 0., 0., 0., 0.};
  if (I >= 2) {
    const double R = RLZ(I);
    if (J >= 2) {
      const double denp = BNES(I, J) + BNES(I, J1);
      v[2] = DTs / DPHI / 2 / MDR / R / denp;
      v[3] = kOME * DTs / DPHI - (EIR(I, J1) + EIR(I, J)) / R * DTs / DPHI / denp;
    }
    v[4] = -0.5 / DPHI / BNES(I, J);
    v[5] = EIP(I, J) * R / BNES(I, J);
    v[6] = 0.5 / MDR / BNES(I, J);
    v[7] = kOME * R - EIR(I, J) / BNES(I, J);
  }
  for (int q = 0; q < 8; ++q) d.mij[(long long)q * n + t] = v[q];
}

void launch_dts_tables(const Dev& d, double dts, cudaStream_t st) {
  int n = d.ns * d.ne * d.nr;
  k_dts_small<<<(n + 127) / 128, 128, 0, st>>>(d, dts);
  const int nij = d.nr * d.nt;
  k_dts_ij<<<(nij + 127) / 128, 128, 0, st>>>(d, dts);
  long long nc = (long long)d.nr * d.nt * d.npa;
  k_dts_cells<<<(unsigned)((nc + 255) / 256), 256, 0, st>>>(d, dts);
  long long nl = (long long)d.ns * d.ncell;
  k_dts_loss<<<(unsigned)((nl + 255) / 256), 256, 0, st>>>(d, dts);
}

// ------------------------------------------------ per-member (VT) tables
// VT(I,J) of member m: the VOLS formula (src/ModRamRun.f90:45-54)
// AVS*(LZ*RE)**2*SIN(PHI-PHIOFS) with (LZ*RE)**2 and the sine tabulated, or
// the explicit potential of ramgpu_set_potential.
struct VtSource {
  const double* vt;
  double avs;
  bool vols;
  __device__ VtSource(const Dev& d, int m) : vt(d.vt + (long long)m * d.nf * d.nt), avs(0.0), vols(d.vt_mode[m] == 1) {
    if (vols) {
      const double KP = d.kp[m];
      const double tt = 1. - 0.159 * KP + 0.0093 * (KP * KP);
      avs = 7.05E-6 / (tt * tt * tt) / kRE;
    }
  }
  __device__ double operator()(const Dev& d, int I, int J) const {
    return vols ? avs * d.lr2[I - 1] * d.sinphi[J - 1] : vt[BIX(I, J)];
  }
};

// Per (member, I, J): the E x B terms of DRIFTR and DRIFTP and the
// DRD1/DPD1 (= DRM1/DPM1) factors of DRIFTE/DRIFTMU, one fma each on the
// VT combination (k_dts_ij holds the rest).
__global__ void k_member_ij(Dev d) {
  const int per = d.nr * d.nt;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)d.nm * per) return;
  const int m = (int)(t / per);
  const int ij = (int)(t % per);
  const int I = 1 + ij % d.nr;
  const int J = 1 + ij / d.nr;
  const VtSource VT(d, m);
  const double* __restrict__ q = d.mij + ij;
  int J0, J1;
  wrapj(J, d.nt, J0, J1);
  d.cr[t] = fma(q[0], VT(d, I, J0) + VT(d, I + 1, J0) - VT(d, I, J1) - VT(d, I + 1, J1), q[per]);
  double ca = 0.0, drd1 = 0.0, dpd1 = 0.0;
  if (I >= 2) {
    if (J >= 2) ca = fma(q[2 * per], VT(d, I + 1, J) + VT(d, I + 1, J1) - VT(d, I - 1, J) - VT(d, I - 1, J1), q[3 * per]);
    drd1 = fma(q[4 * per], VT(d, I, J1) - VT(d, I, J0), q[5 * per]);
    dpd1 = fma(q[6 * per], VT(d, I + 1, J) - VT(d, I - 1, J), q[7 * per]);
  }
  d.ca[t] = ca;
  d.drd1[t] = drd1;
  d.dpd1[t] = dpd1;
}

// DRIFTR ghost planes.  Plane p = (K-1)*NPA + (L-1) in the reference's
// K->L loop order.  One warp per plane: lanes test 32 lines J at a time
// from the top, a ballot finds the highest inflow J.
__device__ __forceinline__ void ghost_plane(const Dev& d, int it, int p) {
  const int np = d.ne * d.npa;
  const int lane = threadIdx.x & 31;
  const int2 item = d.items[it];
  const int m = item.x, s = item.y, slot = m * d.ns + s;
  if (p >= np) return;  // uniform per warp
  const int k = p / d.npa, l = p % d.npa;
  const double p4 = d.p4[s * d.ne + k];
  int has = 0, src = -1;
  double v = 0.0;
  for (int top = d.nt - 1; top >= 0; top -= 32) {
    const int jj = top - lane;
    const bool inf = jj >= 0 && inflow_line(d, m, jj, l, p4);
    const unsigned b = __ballot_sync(0xffffffffu, inf);
    if (b) {
      has = 1;
      const int jsel = top - (__ffs(b) - 1);
      v = ghost_value(d, slot, jsel, k, l, d.conf1);
      src = (l * d.ne + k) * d.nt + jsel;
      break;
    }
  }
  if (lane == 0) {
    d.plane_has[(long long)slot * np + p] = has;
    d.plane_last[(long long)slot * np + p] = v;
    d.plane_last_src[(long long)slot * np + p] = src;
  }
}

// Per (member, I, J, L): UE and UM from the (I,J) factors; the blocks past
// nb_ijl find the ghost planes of every work item (4 planes per block).
__global__ void __launch_bounds__(128) k_member_ijl(Dev d, int nb_ijl) {
  if ((int)blockIdx.x >= nb_ijl) {
    const int np = d.ne * d.npa, bpi = (np + 3) / 4;
    const int b = (int)blockIdx.x - nb_ijl;
    ghost_plane(d, b / bpi, (b % bpi) * 4 + (threadIdx.x >> 5));
    return;
  }
  const long long per = (long long)d.nr * d.nt * d.npa;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)d.nm * per) return;
  const int m = (int)(t / per);
  const long long c = t % per;
  const int i = (int)(c % d.nr);
  const long long ij = (long long)m * d.nr * d.nt + (c % ((long long)d.nr * d.nt));
  double ue = 0.0, um = 0.0;
  if (i >= 1) {
    const double drd1 = d.drd1[ij], dpd1 = d.dpd1[ij];
    ue = d.gre[c] * drd1 + d.gpe[c] * dpd1 + d.ze[c];
    um = -d.cmudot[c] * (d.gmr[c] * drd1 + d.gmp[c] * dpd1 + d.zm[c]);
  }
  d.ue[t] = ue;
  d.um[t] = um;
}

// Two launches: the (I,J) terms, then the (I,J,L) terms with the ghost
// planes alongside (launch_ghost then scans the planes).
void launch_member_coef(const Dev& d, double dts, cudaStream_t st) {
  (void)dts;  // DTs enters through k_dts_ij
  const int nij = d.nm * d.nr * d.nt;
  k_member_ij<<<(nij + 127) / 128, 128, 0, st>>>(d);
  const long long n = (long long)d.nm * d.nr * d.nt * d.npa;
  const int nb_ijl = (int)((n + 127) / 128);
  const int nb_ghost = ((d.ne * d.npa + 3) / 4) * d.nitems;
  k_member_ijl<<<(unsigned)(nb_ijl + nb_ghost), 128, 0, st>>>(d, nb_ijl);
}

// Exclusive "last defined" scan over planes: one block per work item.
// combine(left, right) = right if right has a value else left (associative),
// scanned with warp shuffles, then across the 32 warp totals.
__device__ __forceinline__ void last_scan_warp(int& h, double& v, int& src) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int lh = __shfl_up_sync(0xffffffffu, h, o);
    const double lv = __shfl_up_sync(0xffffffffu, v, o);
    const int ls = __shfl_up_sync(0xffffffffu, src, o);
    if (lane >= o && !h) { h = lh; v = lv; src = ls; }
  }
}

__global__ void __launch_bounds__(1024) k_ghost_scan(Dev d) {
  __shared__ int s_h[32];
  __shared__ double s_v[32];
  __shared__ int s_s[32];
  const int np = d.ne * d.npa;
  const int2 item = d.items[blockIdx.x];
  const int slot = item.x * d.ns + item.y;
  const int* has = d.plane_has + (long long)slot * np;
  const double* last = d.plane_last + (long long)slot * np;
  double* carry = d.plane_carry + (long long)slot * np;
  const int* lsrc = d.plane_last_src + (long long)slot * np;
  int* csrc = d.plane_carry_src + (long long)slot * np;
  const int nth = blockDim.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int cs = (np + nth - 1) / nth;
  const int p0 = min(np, threadIdx.x * cs), p1 = min(np, p0 + cs);
  int h = 0, sc = -1;
  double v = 0.0;
  for (int p = p0; p < p1; ++p)
    if (has[p]) { h = 1; v = last[p]; sc = lsrc[p]; }
  // inclusive scan within the warp
  int ih = h, is = sc;
  double iv = v;
  last_scan_warp(ih, iv, is);
  if (lane == 31) { s_h[warp] = ih; s_v[warp] = iv; s_s[warp] = is; }
  __syncthreads();
  if (warp == 0) {
    int wh = lane < (nth >> 5) ? s_h[lane] : 0;
    double wv = lane < (nth >> 5) ? s_v[lane] : 0.0;
    int ws = lane < (nth >> 5) ? s_s[lane] : -1;
    last_scan_warp(wh, wv, ws);  // inclusive over warps
    s_h[lane] = wh;
    s_v[lane] = wv;
    s_s[lane] = ws;
  }
  __syncthreads();
  // exclusive value for this thread: inclusive of the previous thread
  int eh = __shfl_up_sync(0xffffffffu, ih, 1);
  double ev = __shfl_up_sync(0xffffffffu, iv, 1);
  int es = __shfl_up_sync(0xffffffffu, is, 1);
  if (lane == 0) { eh = 0; ev = 0.0; es = -1; }
  if (!eh && warp > 0) { eh = s_h[warp - 1]; ev = s_v[warp - 1]; es = s_s[warp - 1]; }
  double run = eh ? ev : 0.0;
  int rsrc = eh ? es : -1;
  for (int p = p0; p < p1; ++p) {
    carry[p] = run;
    csrc[p] = rsrc;
    if (has[p]) { run = last[p]; rsrc = lsrc[p]; }
  }
}

// The planes themselves are found in launch_member_coef's second kernel.
void launch_ghost(const Dev& d, cudaStream_t st) { k_ghost_scan<<<d.nitems, 1024, 0, st>>>(d); }

// -------------------------------------------------- loss factor (bookkeeping path)
__global__ void k_loss_apply(Dev d, const double* __restrict__ table) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= d.ncell) return;
  const int2 item = d.items[blockIdx.y];
  const int slot = item.x * d.ns + item.y;
  double* f = d.f2 + (long long)slot * d.ncell + c;
  *f = *f * table[(long long)item.y * d.ncell + c];
}

void launch_loss_apply(const Dev& d, const double* table, cudaStream_t st) {
  k_loss_apply<<<dim3((unsigned)((d.ncell + 255) / 256), d.nitems), 256, 0, st>>>(d, table);
}

// ------------------------------------ periodic copy + magnetopause mask
__global__ void k_finish(Dev d, int any_outside) {
  // the (I, K, L) of the L window [lw0, lw1)
  const long long n = (long long)d.nr * d.ne * (d.lw1 - d.lw0);
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x + (long long)d.lw0 * d.nr * d.ne;
  if (t >= n + (long long)d.lw0 * d.nr * d.ne) return;
  const int2 item = d.items[blockIdx.y];
  const int slot = item.x * d.ns + item.y;
  const int i = (int)(t % d.nr);
  const long long kl = t / d.nr;  // K + NE*L
  double* f = d.f2 + (long long)slot * d.ncell + kl * d.nt * d.nr + i;
  f[(long long)(d.nt - 1) * d.nr] = f[0];  // F2(:,:,NT,:,:) = F2(:,:,1,:,:)
  if (any_outside)
    for (int j = 0; j < d.nt; ++j)
      if (d.outside[(long long)j * d.nr + i] == 1) f[(long long)j * d.nr] = 1.e-31;
}

void launch_finish(const Dev& d, cudaStream_t st) {
  // any_outside is folded into the flags word bit 31 by the host
  long long n = (long long)d.nr * d.ne * (d.lw1 - d.lw0);
  k_finish<<<dim3((unsigned)((n + 255) / 256), d.nitems), 256, 0, st>>>(d, (d.flags >> 31) & 1u);
}

// ---------------------------------------------------------- ANISCH moments
// Stage 1: one thread per (I>=2, J, K>=2, L-chunk): the L=1 side effect
// F2(S,I,J,K,1) = F2(S,I,J,K,2) (chunk 0; src/ModRamRun.f90:366) and the
// chunk's share of both weighted pitch-angle sums, L = 1..int(UPA(I)-1)
// split into kMomChunks equal runs.  Partials: (slot, J, I, Q) pairs of
// doubles, Q = (K-2)*kMomChunks + chunk, so each (I,J) owns one contiguous
// run for stage 2.
constexpr int kMomChunks = 4;
template <bool kSep>
__global__ void __launch_bounds__(128) k_moments_part(Dev d) {
  const int nr1 = d.nr - 1, ne1 = d.ne - 1;
  const long long n = (long long)nr1 * d.nt * ne1 * kMomChunks;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int2 item = d.items[blockIdx.y];
  const int s = item.y, slot = item.x * d.ns + s;
  const int i = 1 + (int)(t % nr1);
  const int j = (int)((t / nr1) % d.nt);
  const int k = 1 + (int)((t / ((long long)nr1 * d.nt)) % ne1);
  const int ch = (int)(t / ((long long)nr1 * d.nt * ne1));
  const long long st = (long long)d.ne * d.nt * d.nr;
  const long long off = ((long long)k * d.nt + j) * d.nr + i;
  double* f = d.f2 + (long long)slot * d.ncell + off;
  const long long sa = (long long)d.ne * d.nr, sb = (long long)d.nt * d.nr;  // L strides
  const double* __restrict__ wa = d.mw_a + (long long)s * d.npa * sa + (long long)k * d.nr + i;
  const double* __restrict__ be = (kSep ? d.mws_be : d.mw_be) + (long long)j * d.nr + i;
  const double* __restrict__ ba = (kSep ? d.mws_ba : d.mw_ba) + (long long)j * d.nr + i;
  const double f2 = f[st];
  if (ch == 0) f[0] = f2;
  const int u = d.upa_mom[i];
  const int cl = (u + kMomChunks - 1) / kMomChunks;
  const int l0 = 1 + ch * cl, l1 = min(u, (ch + 1) * cl);
  double sume = 0.0, suma = 0.0;
#pragma unroll 4
  for (int L = l0; L <= l1; ++L) {
    const double v = (L == 1) ? f2 : f[(long long)(L - 1) * st];
    const double g = kSep ? v : v * wa[(long long)(L - 1) * sa];
    sume = fma(g, be[(long long)(L - 1) * sb], sume);
    suma = fma(g, ba[(long long)(L - 1) * sb], suma);
  }
  if (kSep) {  // the species factor of (S, I, K), once per partial
    const double ws = d.mws_a[((long long)s * d.ne + k) * d.nr + i];
    sume *= ws;
    suma *= ws;
  }
  const int nq = ne1 * kMomChunks;
  double2* part = reinterpret_cast<double2*>(d.mom_part) +
                  (((long long)slot * d.nt + j) * d.nr + i) * nq + (k - 1) * kMomChunks + ch;
  *part = make_double2(sume, suma);
}

// Stage 2: one warp per (I>=2, J): lanes sum strided runs of the (I,J)'s
// partials, then an xor butterfly (every lane ends with the same sums).
__global__ void __launch_bounds__(128) k_moments_reduce(Dev d) {
  const int nr1 = d.nr - 1;
  const int lane = threadIdx.x & 31;
  const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (w >= nr1 * d.nt) return;  // uniform per warp
  const int2 item = d.items[blockIdx.y];
  const int slot = item.x * d.ns + item.y;
  const int i = 1 + w % nr1, j = w / nr1;
  const int nq = (d.ne - 1) * kMomChunks;
  const double2* __restrict__ p =
      reinterpret_cast<const double2*>(d.mom_part) + (((long long)slot * d.nt + j) * d.nr + i) * nq;
  double e = 0.0, a = 0.0;
  for (int q = lane; q < nq; q += 32) {
    const double2 v = p[q];
    e += v.x;
    a += v.y;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    e += __shfl_xor_sync(0xffffffffu, e, o);
    a += __shfl_xor_sync(0xffffffffu, a, o);
  }
  if (lane == 0) {
    const long long o = (long long)slot * d.nr * d.nt + (long long)j * d.nr + i;
    d.ppert[o] = e;
    d.ppart[o] = a;
  }
}

void launch_moments(const Dev& d, cudaStream_t st) {
  long long n = (long long)(d.nr - 1) * d.nt * (d.ne - 1) * kMomChunks;
  if (d.mom_sep) k_moments_part<true><<<dim3((unsigned)((n + 127) / 128), d.nitems), 128, 0, st>>>(d);
  else k_moments_part<false><<<dim3((unsigned)((n + 127) / 128), d.nitems), 128, 0, st>>>(d);
  int n2 = (d.nr - 1) * d.nt;
  k_moments_reduce<<<dim3((n2 + 3) / 4, d.nitems), 128, 0, st>>>(d);
}

// ANISCH's only effect on F2, F2(I,J,K,1) = F2(I,J,K,2) for I, K >= 2
// (src/ModRamRun.f90:366), for runs that need the state but not the
// moments (the adjoint's forward and recomputation passes).
__global__ void k_anisch_state(Dev d) {
  const int nr1 = d.nr - 1, ne1 = d.ne - 1;
  const long long n = (long long)nr1 * d.nt * ne1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int2 item = d.items[blockIdx.y];
  const int slot = item.x * d.ns + item.y;
  const int i = 1 + (int)(t % nr1);
  const int j = (int)((t / nr1) % d.nt);
  const int k = 1 + (int)(t / ((long long)nr1 * d.nt));
  double* f = d.f2 + (long long)slot * d.ncell + ((long long)k * d.nt + j) * d.nr + i;
  f[0] = f[(long long)d.ne * d.nt * d.nr];
}

void launch_anisch_state(const Dev& d, cudaStream_t st) {
  const long long n = (long long)(d.nr - 1) * d.nt * (d.ne - 1);
  k_anisch_state<<<dim3((unsigned)((n + 255) / 256), d.nitems), 256, 0, st>>>(d);
}

// ------------------------------------------------------------------ SUMRC
// Per-block partial sums of EKEV*F2*WE*WMU over I=2..NR, J=1..NT-1,
// K=2..NE, L=2..NPA (src/ModRamRun.f90:246-255).  part: (nitems, nblk).
__global__ void __launch_bounds__(256) k_sumrc(Dev d, double* part, int nblk) {
  __shared__ double sh[256];
  const int2 item = d.items[blockIdx.y];
  const int slot = item.x * d.ns + item.y;
  const double* f = d.f2 + (long long)slot * d.ncell;
  double acc = 0.0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < d.ncell;
       c += (long long)gridDim.x * blockDim.x) {
    const int I = 1 + (int)(c % d.nr);
    const int J = 1 + (int)((c / d.nr) % d.nt);
    const int K = 1 + (int)((c / ((long long)d.nr * d.nt)) % d.ne);
    const int L = 1 + (int)(c / ((long long)d.nr * d.nt * d.ne));
    if (I >= 2 && J <= d.nt - 1 && K >= 2 && L >= 2) {
      const double WEIGHT = f[c] * WE(K) * WMU(L);
      acc = acc + EKEV(K) * WEIGHT;
    }
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[(long long)blockIdx.y * nblk + blockIdx.x] = sh[0];
}

void launch_sumrc(const Dev& d, double* part, int nblk, cudaStream_t st) {
  k_sumrc<<<dim3(nblk, d.nitems), 256, 0, st>>>(d, part, nblk);
}

// ------------------------------------------------------------------- FLUX
__global__ void k_flux(Dev d, int slot, int s, double* out) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= d.ncell) return;
  const int I = 1 + (int)(c % d.nr);
  const int J = 1 + (int)((c / d.nr) % d.nt);
  const int K = 1 + (int)((c / ((long long)d.nr * d.nt)) % d.ne);
  const int L = 1 + (int)(c / ((long long)d.nr * d.nt * d.ne));
  double v = 0.0;
  if (I >= 2 && K >= 2 && L >= 2 && J <= d.nt - 1) {
    const double ff = d.ffactor[(long long)s * d.nr * d.ne * d.npa + (((long long)L - 1) * d.ne + (K - 1)) * d.nr + (I - 1)];
    v = d.f2[(long long)slot * d.ncell + c] / ff / FNHS(I, J, L);
  }
  out[c] = v;
}

void launch_flux(const Dev& d, int slot, int s, double* out, cudaStream_t st) {
  k_flux<<<(unsigned)((d.ncell + 255) / 256), 256, 0, st>>>(d, slot, s, out);
}

}  // namespace ramgpu
