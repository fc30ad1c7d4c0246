// adjoint.cu -- frozen-limiter adjoint of the RAM kinetic step.
//
// With the limiter branch of every face and the clip state of every cell
// frozen (recorded by the forward sweeps, four bits per face: 0 upwind
// only, 1 beta*D, 2 X, 3 D, 4 beta*X, plus kClipBit; a call's forward and
// reverse sweeps of one direction share a byte, the forward one in the high
// nibble, read here with the shift rsh), each sweep of
// src/ModRamDrift.f90 is a linear map of its line
//   Fnew(i) = G(i) + w(i) (Phi(i-1) - Phi(i)),  Phi(f) = C(f) FBND(f),
//   FBND(f) = FUP(f) + a(f) LX(f),  LX in {beta D, X, D, beta X},
// so its adjoint is the transposed map, applied here line by line with the
// coefficients recomputed from the same tables as the forward pass.  The
// tail of ram_run (periodic copy, magnetopause mask, ANISCH's F2(:,:,:,:,1)
// side effect), the CEX/ATMOL factors and the log-flux observation operator
// are transposed too.  dJ/dFGEOS collects the ghost cells of DRIFTR,
// including the stale ghosts an outflow line inherits from an earlier
// inflow line.
#include <math.h>

#include <type_traits>

#include "kernels.cuh"

namespace ramgpu {

// Transposed sweeps.  With the record frozen, one face f contributes
//   FBb(f) = dJ/dFBND(f) = C(f) * (w(f+1) le(f+1) - w(f) le(f))
// (le = lambda of an updated, unclipped cell, w the update weight: 1 for R
// and P, 1/WE, 1/WMU for E and MU) and scatters it to the cells of
// FBND(f) = FUP + a LX:  the upwind cell, and for LX = beta D | X | D |
// beta X the two cells of D (f-1,f for s=+1; f+1,f+2 for s=-1) or of X
// (f,f+1).  Every face touches cells f-1..f+2 only, so each line is
// streamed once with a rolling window of four cell accumulators in
// registers: after face f, cell f-1 is final and is written out.

// Scatter of one face into the window (cm1, c0, c1, c2) = cells f-1..f+2.
// FBND(f) = FUP + a LX depends on adjacent cells only: with C >= 0 (FUP =
// F(f)) on (f-1, f) for LX = D, (f, f+1) for LX = X; with C < 0 (FUP =
// F(f+1)) on (f, f+1) for LX = X, (f+1, f+2) for LX = D; its derivatives on
// that pair are (-ak, 1+ak) when the pair ends at the upwind cell and
// (1-ak, ak) when it starts there (upwind only: (1, 0)), with ak = a
// (cases 2, 3) or beta*a (cases 1, 4).  The pair and the signed
// coefficients are picked by integer selects, so a face costs one add and
// two fma on the FP64 pipe whatever its case.
__device__ __forceinline__ void face_acc(double FBb, bool neg, int cs, double ak, double& cm1,
                                         double& c0, double& c1, double& c2) {
  const bool xt = (cs == 2) | (cs == 4);  // LX = X (f, f+1)
  const bool dt = (cs == 1) | (cs == 3);  // LX = D (f-1, f) or (f+1, f+2)
  const bool ends = (dt & !neg) | (xt & neg);  // pair ends at the upwind cell
  const bool starts = (xt & !neg) | (dt & neg);
  const double sak = ends ? bitsd(dbits(ak) ^ kSignMask) : (starts ? ak : 0.0);
  const double m = 1.0 - sak;
  const double b0 = ends ? sak : m, b1 = ends ? m : sak;
  // first cell of the pair in the window: 0 = f-1, 1 = f, 2 = f+1
  const int p = neg ? (ends ? 1 : 2) : (ends ? 0 : 1);
  const double p0 = p == 0 ? cm1 : (p == 1 ? c0 : c1);
  const double p1 = p == 0 ? c0 : (p == 1 ? c1 : c2);
  const double t0 = fma(b0, FBb, p0);
  const double t1 = fma(b1, FBb, p1);
  cm1 = p == 0 ? t0 : cm1;
  c0 = p == 0 ? t1 : (p == 1 ? t0 : c0);
  c1 = p == 1 ? t1 : (p == 2 ? t0 : c1);
  c2 = p == 2 ? t1 : c2;
}

// ---- the face weights on the integer pipe
// The transposed sweeps are bound by the FP64 unit with three quarters of
// their issue slots free (one FP64 warp instruction holds its pipe about as
// long as 65 issue slots), so the two FP64 operations per face that form
// the weights of face_acc, ak = k*a and m = 1 - sak, can move to integer
// instructions where the sweep has the latency to spare (kAdjIntMask).
// The fixed point is a signed 64-bit integer with 2^52 as 1: it keeps every
// bit of its input down to 2^-52, so a and m differ from the FP64 fma and
// add they replace by at most 2^-53 and 2^-52 absolute; they scale FBb in
// the two accumulations, whose own rounding is of that size.  Courant
// numbers of 1024 and more, inf and NaN give NaN weights.

// Sweeps (bit w: R, P, E, MU) whose transposes form ak and m on the
// integer pipe.
constexpr unsigned kAdjIntMask = 0xBu;
// Sweeps whose transposes form the face product FBb = C*DL (and, in E, the
// coefficient's EDOT product) with mul_rn_int, the FP64 product bit for bit
// on the integer pipe.  Measured on GB300: the DRIFTE transposes that form
// C gain, the one that loads C (fewer FP64 operations left) loses and keeps
// the FP64 product (the bits are the same either way); R (shared-memory
// tiles, integer weights) loses over the whole adjoint window; P (bit 2) is
// neutral and MU (bit 8) loses (backward 0.720-0.731 s with E alone, 0.725
// with E and P, 0.736 with E and MU, 0.755 with all three, on one box).
constexpr unsigned kAdjMulIntMask = 0x4u;
__device__ __forceinline__ double adj_mul(unsigned bit, double a, double b) {
  return (kAdjMulIntMask & bit) ? mul_rn_int(a, b) : a * b;
}
constexpr bits64 kNaNBits = 0x7FF8000000000000ULL;

// |v| 2^-52 (v < 2^63) as the bits of a double with the given sign.
__device__ __forceinline__ bits64 fix52_to_bits(bits64 v, bool neg) {
  const int lz = __clzll((long long)(v | 1ULL));
  const bits64 r = ((bits64)(1034 - lz) << 52) | (((v << lz) >> 11) & kMantMask);
  return (neg ? kSignMask : 0ULL) | (v ? r : 0ULL);
}
// |x| 2^52 for the bits of a double with |x| < 1024 (lower bits cut).
__device__ __forceinline__ bits64 bits_to_fix52(bits64 x) {
  const int e = (int)((x >> 52) & 0x7FF);
  const bits64 mant = (x & kMantMask) | (e ? kImplicit : 0ULL);
  const int sh = e - 1023;
  return sh >= 0 ? (mant << (sh < 10 ? sh : 10)) : (mant >> (-sh < 63 ? -sh : 63));
}
// The CORR factor a = s*0.5*(1 - u) (s = -1 for neg) as bits, from the bits
// ub of the Courant number u >= 0.
__device__ __forceinline__ bits64 corr_a_fix(bits64 ub, bool neg) {
  const long long D = (long long)(1ULL << 52) - (long long)bits_to_fix52(ub);  // (1 - u) 2^52
  const bits64 r = fix52_to_bits((bits64)(D < 0 ? -D : D), neg != (D < 0));
  const bits64 half = (r << 1) ? r - (1ULL << 52) : r;  // r / 2
  return (ub >> 52) >= 1033 ? kNaNBits : half;
}
// 1 - x for the bits of x (|x| < 1024) as bits.
__device__ __forceinline__ bits64 one_minus_bits(bits64 x) {
  const bits64 X = bits_to_fix52(x);
  const long long M = (x >> 63) ? (long long)((1ULL << 52) + X) : (long long)(1ULL << 52) - (long long)X;
  const bits64 r = fix52_to_bits((bits64)(M < 0 ? -M : M), M < 0);
  return ((x >> 52) & 0x7FF) >= 1033 ? kNaNBits : r;
}
// face_acc with ak = k*a from the CORR factor a (bits; k = beta for cases
// 1, 4 by babs_bits) and m = 1 - sak, both on the integer pipe.
__device__ __forceinline__ void face_acc_a(double FBb, bool neg, int cs, bits64 a, const BetaBits& beta,
                                           double& cm1, double& c0, double& c1, double& c2) {
  const bool xt = (cs == 2) | (cs == 4);
  const bool dt = (cs == 1) | (cs == 3);
  const bool ends = (dt & !neg) | (xt & neg);
  const bool starts = (xt & !neg) | (dt & neg);
  const bool kb = (cs == 1) | (cs == 4);
  const bits64 ak = kb ? ((a & kSignMask) | babs_bits(beta, bitsd(a))) : a;
  const bits64 sak = ends ? (ak ^ kSignMask) : (starts ? ak : 0ULL);
  const bits64 m = one_minus_bits(sak);
  const double b0 = bitsd(ends ? sak : m), b1 = bitsd(ends ? m : sak);
  const int p = neg ? (ends ? 1 : 2) : (ends ? 0 : 1);
  const double p0 = p == 0 ? cm1 : (p == 1 ? c0 : c1);
  const double p1 = p == 0 ? c0 : (p == 1 ? c1 : c2);
  const double t0 = fma(b0, FBb, p0);
  const double t1 = fma(b1, FBb, p1);
  cm1 = p == 0 ? t0 : cm1;
  c0 = p == 0 ? t1 : (p == 1 ? t0 : c0);
  c1 = p == 1 ? t1 : (p == 2 ? t0 : c1);
  c2 = p == 2 ? t1 : c2;
}
// Bits of the Courant number |c|*y (y = 1/DE or 1/DMU, positive normal):
// the significands' product cut to 53 bits (as mul_pos_bits), 0 for zero,
// subnormal or underflowing |c|*y, inf when it overflows or c is not finite.
__device__ __forceinline__ bits64 courant_u(double c, double y) {
  const bits64 ax = dbits(c) & kAbsMask, uy = dbits(y);
  const int ex = (int)(ax >> 52);
  const bits64 p = __umul64hi(((ax & kMantMask) | kImplicit) << 11, ((uy & kMantMask) | kImplicit) << 11);
  const int hi = (int)(p >> 63);
  const int e = ex + (int)(uy >> 52) - 1023 + hi;
  const bits64 r = ((bits64)e << 52) | ((p >> (10 + hi)) & kMantMask);
  return (ex == 0x7FF || e >= 0x7FF) ? 0x7FF0000000000000ULL : ((ax < kImplicit || e <= 0) ? 0ULL : r);
}

// ak = LIMITER weight times the CORR factor a = -0.5*(C*q - s) of a face:
// fma(C, -0.5*k*q, 0.5*k*s) with k = beta for cases 1, 4 and 1 otherwise
// (q = 1 for R and P; -0.5*q comes from the -0.5/DE, -0.5/DMU tables).
// 0.5*k*s is formed either as a select of four constants or by flipping
// the sign bit of 0.5*k; the two give the same value, and the compiler's
// schedule is measurably faster with the first in the R and P transposes
// and with the second in E and MU (hb = 0.5*beta).
template <bool kXorSign>
__device__ __forceinline__ double face_ak(double C, bool neg, int cs, double mh, double bmh, double hb) {
  const bool kb = (cs == 1) | (cs == 4);
  double shk;
  if (kXorSign) {
    const double hk = kb ? hb : 0.5;
    shk = bitsd(dbits(hk) ^ (neg ? kSignMask : 0ULL));
  } else {
    shk = neg ? (kb ? -hb : -0.5) : (kb ? hb : 0.5);
  }
  return fma(C, kb ? bmh : mh, shk);
}

// lambda of cell c of a line (stride st) masked by the clip bit.  Both
// loads are issued unconditionally (the record through the read-only path)
// so that the next cells' loads can run ahead of the window's arithmetic.
__device__ __forceinline__ double masked(const double* __restrict__ lam, const unsigned char* __restrict__ rl,
                                         long long off, int rsh) {
  const double v = lam[off];
  return ((__ldg(rl + off) >> rsh) & kClipBit) ? 0.0 : v;
}

#define WORK_LOOP(NLINES)                                                          \
  const int bpi = (NLINES + blockDim.x - 1) / blockDim.x;                          \
  const long long nunits = (long long)bpi * d.nitems;                              \
  for (long long u = blockIdx.x + (long long)blockIdx.y * gridDim.x; u < nunits;   \
       u += (long long)gridDim.x * gridDim.y)

// The loops below are peeled so that no floating-point operation in the
// main loop depends on the position along the line (the FP64 pipe is the
// bottleneck and predicated-off branches would still cost issue slots).

// ------------------------------------------------------------------ DRIFTR^T
// Cells 1..NR, ghosts NR+1, NR+2.  new(1) = F(1); faces 2..NR-1 (and NR on
// inflow lines); FBND(1) = F(2) on inflow lines, FBND(NR) = F(NR) on outflow
// lines (both 0 when closed).  The ghosts' adjoints go to dJ/dFGEOS, for an
// outflow line to the FGEOS cell its stale ghost came from.
// A CTA takes blockDim.x consecutive lines of one item.  They are contiguous
// in memory (blockDim.x*NR doubles of lambda and as many record bytes), so
// the CTA loads them into shared memory with coalesced loads, each thread
// transposes its line there, and the CTA stores the tile back coalesced.
// Read in place, the lanes' lines lie 8*NR bytes apart: every warp load
// touches 32 sectors and leans on L1, and at seven CTAs per SM L1 no longer
// held them (four times slower).  Rows of the lambda tile are NR|1 doubles
// apart, so the 8-byte accesses of a half-warp fall in distinct banks.
#ifdef RAMGPU_BOUNDS_CHECK
constexpr bool kBoundsChecked = true;
#else
constexpr bool kBoundsChecked = false;
#endif
size_t adj_r_smem(const Dev& d, int threads) {
  return (size_t)threads * (size_t)(d.nr | 1) * sizeof(double) + (size_t)threads * (size_t)d.nr;
}
template <int rsh>
__global__ void __launch_bounds__(128) k_adj_r(Dev d, const unsigned char* __restrict__ rec) {
  extern __shared__ double tile[];
  const int nr = d.nr, nt = d.nt, ne = d.ne;
  const int ts = nr | 1;
  unsigned char* rtile = (unsigned char*)(tile + (size_t)blockDim.x * ts);
  const int nlines = nt * ne * d.npa;
  const int bpi = (nlines + blockDim.x - 1) / blockDim.x;
  const long long nunits = (long long)bpi * d.nitems;
  for (long long u = blockIdx.x + (long long)blockIdx.y * gridDim.x; u < nunits;
       u += (long long)gridDim.x * gridDim.y) {  // uniform across the CTA
    const int2 item = d.items[u / bpi];
    const int m = item.x, s = item.y, slot = m * d.ns + s;
    const int lfirst = (int)(u % bpi) * blockDim.x;
    const int nl = min((int)blockDim.x, nlines - lfirst);
    // bounds-checked builds: the tile's cells (the whole CTA skips it)
    if (kBoundsChecked) {
      const bool ok = rg_item(d, item) && rg_span((long long)lfirst * nr, (long long)nl * nr, 1, d.ncell);
      if (threadIdx.x == 0) rg_ok(d, ok, kRgAdjR, lfirst);
      if (!ok) continue;
    }
    double* __restrict__ gl = d.lam + (long long)slot * d.ncell + (long long)lfirst * nr;
    const unsigned char* __restrict__ gr = rec + (u / bpi) * d.ncell + (long long)lfirst * nr;
    for (int e = threadIdx.x; e < nl * nr; e += blockDim.x) {
      const int ln = e / nr;
      tile[ln * ts + (e - ln * nr)] = gl[e];
      rtile[e] = __ldg(gr + e);
    }
    __syncthreads();
    const int line = lfirst + threadIdx.x;
    const int j = line % nt, k = (line / nt) % ne, l = line / (nt * ne);
    // bounds-checked builds: the line's GRT and CR rows
    const bool lok = threadIdx.x < nl &&
        (!kBoundsChecked ||
         rg_ok(d, rg_span(((long long)l * nt + j) * nr, nr, 1, (long long)nr * nt * d.npa) &&
                      rg_span(((long long)m * nt + j) * nr, nr, 1, (long long)d.nm * nr * nt),
               kRgAdjR, line));
    if (lok) {
      double* lam = tile + threadIdx.x * ts;
      const unsigned char* rl = rtile + threadIdx.x * nr;
      const double* __restrict__ grt = d.grt + ((long long)l * nt + j) * nr;
      const double* __restrict__ cr = d.cr + ((long long)m * nt + j) * nr;
      const double p4 = d.p4[s * ne + k];
      const double hb = 0.5 * d.betalim, bmh = -hb;
      const BetaBits beta(d.betalim);
      const bool closed = d.flags & 1u;
      const int n = nr;  // >= 4
      auto mk = [&](int c) { return ((rl[c] >> rsh) & kClipBit) ? 0.0 : lam[c]; };  // masked lambda
      const double cN = fma(grt[n - 1], p4, cr[n - 1]);
      const bool inflow = is_neg(cN);
      // le(i) = lambda of updated, unclipped cell i (i = 2..NR); window = cells f-1..f+2
      double le0 = mk(1), le1 = mk(2), le2 = mk(3);
      double cm1 = lam[0], c0 = le0, c1 = le1, c2 = le2;
      if (inflow && !closed) c0 += fma(grt[0], p4, cr[0]) * le0;  // FBND(1) = F(2)
      auto face = [&](int f, double C) {
        const bool neg = is_neg(C);
        const int cs = (rl[f - 1] >> rsh) & 7;
        if (kAdjIntMask & 1u)
          face_acc_a(adj_mul(1u, C, le1 - le0), neg, cs, corr_a_fix(dbits(C) & kAbsMask, neg), beta, cm1, c0, c1,
                     c2);
        else
          face_acc(adj_mul(1u, C, le1 - le0), neg, cs, face_ak<false>(C, neg, cs, -0.5, bmh, hb), cm1, c0, c1, c2);
      };
      auto advance = [&](int f, double le3) {  // cell f-1 is final; cell f+3 enters
        lam[f - 2] = cm1;
        cm1 = c0; c0 = c1; c1 = c2; c2 = le3;
        le0 = le1; le1 = le2; le2 = le3;
      };
      int f = 2;
      for (; f <= n - 3; ++f) {
        face(f, fma(grt[f - 1], p4, cr[f - 1]));
        advance(f, mk(f + 2));
      }
      for (; f <= n - 1; ++f) {
        face(f, fma(grt[f - 1], p4, cr[f - 1]));
        advance(f, 0.0);
      }
      // face NR: transposed on inflow lines, FBND(NR) = F(NR) on outflow lines
      if (!closed) {
        if (inflow) face(n, cN);
        else c0 -= cN * le0;
      }
      lam[n - 2] = cm1;
      lam[n - 1] = c0;
      const double gN1 = c1, gN2 = c2;  // ghosts F(NR+1), F(NR+2)
      const long long nfg = (long long)nt * ne * d.npa;
      if (inflow) {
        if (d.outside[(long long)j * nr + n - 1] != 1) {
          const double fh = d.fnhs[((long long)l * nt + j) * d.nf + n - 1];
          atomicAdd(&d.gfg[slot * nfg + line], d.conf1 * fh * gN1 + d.conf2 * fh * gN2);
        }
      } else if (gN1 != 0.0) {
        const int src = stale_ghost_src(d, m, slot, j, k, l, p4);
        if (src >= 0) {
          const int jj = src % nt, ll = src / (nt * ne);
          if (d.outside[(long long)jj * nr + n - 1] != 1) {
            const double fh = d.fnhs[((long long)ll * nt + jj) * d.nf + n - 1];
            atomicAdd(&d.gfg[slot * nfg + src], d.conf1 * fh * gN1);
          }
        }
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nl * nr; e += blockDim.x) {
      const int ln = e / nr;
      gl[e] = tile[ln * ts + (e - ln * nr)];
    }
    __syncthreads();  // the next unit reuses the tile
  }
}

// ------------------------------------------------------------------ DRIFTP^T
// Cells 1..NT with J = 1 == J = NT: new(1) is overwritten by new(NT), faces
// J = 2..NT with FBND(1) = FBND(NT).  Faces NT-1 and NT wrap onto cells
// 1..3; they are transposed first, their contributions held in registers
// and added when the window reaches those cells (NT >= 7).
template <int rsh>
__global__ void __launch_bounds__(128) k_adj_p(Dev d, const unsigned char* __restrict__ rec) {
  const int nr = d.nr, nt = d.nt, ne = d.ne;
  const int nlines = (nr - 1) * ne * d.npa;
  WORK_LOOP(nlines) {
    const int2 item = d.items[u / bpi];
    const int m = item.x, s = item.y, slot = m * d.ns + s;
    const int line = (int)(u % bpi) * blockDim.x + threadIdx.x;
    if (line >= nlines) continue;
    const int i = 1 + line % (nr - 1);
    const int kl = line / (nr - 1);
    const int k = kl % ne, l = kl / ne;
    const long long st = nr;
    const long long base = ((long long)kl * nt) * nr + i;
    // bounds-checked builds: the line's cells, its GPT and CA columns
    if (!rg_ok(d, rg_item(d, item) && rg_span(base, nt, nr, d.ncell) &&
                      rg_span((long long)l * nt * nr + i, nt, nr, (long long)nr * nt * d.npa) &&
                      rg_span((long long)m * nt * nr + i, nt, nr, (long long)d.nm * nr * nt),
               kRgAdjP, line))
      continue;
    double* __restrict__ lam = d.lam + (long long)slot * d.ncell + base;
    const unsigned char* __restrict__ rl = rec + (u / bpi) * d.ncell + base;
    const double* __restrict__ gpt = d.gpt + ((long long)l * nt) * nr + i;
    const double* __restrict__ ca = d.ca + ((long long)m * nt) * nr + i;
    const double p2 = d.p2[((long long)s * ne + k) * nr + i];
    const double hb = 0.5 * d.betalim, bmh = -hb;
    const BetaBits beta(d.betalim);
    const int n = nt;
#define PC(J) fma(gpt[(long long)((J)-1) * nr], p2, ca[(long long)((J)-1) * nr])
#define PLE(J) masked(lam, rl, (long long)((J)-1) * st, rsh)
    // le(NT) takes lambda of cell 1 too (F2(1) = F2new(NT))
    const double leN = ((rl[(long long)(n - 1) * st] >> rsh) & kClipBit) ? 0.0 : lam[(long long)(n - 1) * st] + lam[0];
    const double leNm = PLE(n - 1), le2 = PLE(2);
    // w1..w3: contributions to cells 1..3, tNm2..tN: to cells NT-2..NT
    double w1 = 0.0, w2 = 0.0, w3 = 0.0, tNm2 = 0.0, tNm1 = 0.0, tN = 0.0;
    {  // face NT-1: X = F(NT)-F(NT-1); D = F(NT-1)-F(NT-2) (s=+1) or F(2)-F(1) (s=-1)
      const double C = PC(n - 1);
      const bool neg = is_neg(C);
      const int cs = (rl[(long long)(n - 2) * st] >> rsh) & 7;
      const double FBb = adj_mul(2u, C, leN - leNm);
      const double V = face_ak<false>(C, neg, cs, -0.5, bmh, hb) * FBb;
      if (neg) tN += FBb; else tNm1 += FBb;
      if (cs == 2 || cs == 4) { tN += V; tNm1 -= V; }
      else if (cs && !neg) { tNm1 += V; tNm2 -= V; }
      else if (cs) { w2 += V; w1 -= V; }
    }
    {  // face NT: X = F(2)-F(NT); D = F(NT)-F(NT-1) (s=+1) or F(3)-F(2) (s=-1)
      const double C = PC(n);
      const bool neg = is_neg(C);
      const int cs = (rl[(long long)(n - 1) * st] >> rsh) & 7;
      const double FBb = adj_mul(2u, C, le2 - leN);  // Pb(NT) = -le(NT) + Pb(1), Pb(1) = le(2)
      const double V = face_ak<false>(C, neg, cs, -0.5, bmh, hb) * FBb;
      if (neg) w2 += FBb; else tN += FBb;
      if (cs == 2 || cs == 4) { w2 += V; tN -= V; }
      else if (cs && !neg) { tN += V; tNm1 -= V; }
      else if (cs) { w3 += V; w2 -= V; }
    }
    // faces 2..NT-2 streamed; window cells 1..4 (cell 1 has no own term)
    double le0 = le2, le1 = PLE(3), lnext = PLE(4);
    double cm1 = w1, c0 = le2 + w2, c1 = le1 + w3, c2 = lnext;
    auto step = [&](int J, double add, double lec) {  // face J, then cell J+3 enters
      const double C = PC(J);
      const bool neg = is_neg(C);
      const int cs = (rl[(long long)(J - 1) * st] >> rsh) & 7;
      if (kAdjIntMask & 2u)
        face_acc_a(adj_mul(2u, C, le1 - le0), neg, cs, corr_a_fix(dbits(C) & kAbsMask, neg), beta, cm1, c0, c1, c2);
      else
        face_acc(adj_mul(2u, C, le1 - le0), neg, cs, face_ak<false>(C, neg, cs, -0.5, bmh, hb), cm1, c0, c1, c2);
      lam[(long long)(J - 2) * st] = cm1;
      cm1 = c0; c0 = c1; c1 = c2; c2 = add;
      le0 = le1; le1 = lnext; lnext = lec;
    };
    for (int J = 2; J <= n - 6; ++J) {
      const double lec = PLE(J + 3);
      step(J, lec, lec);
    }
    { const double lec = PLE(n - 2); step(n - 5, lec + tNm2, lec); }
    step(n - 4, leNm + tNm1, leNm);
    step(n - 3, leN + tN, leN);
    step(n - 2, 0.0, 0.0);
    lam[(long long)(n - 3) * st] = cm1;
    lam[(long long)(n - 2) * st] = c0;
    lam[(long long)(n - 1) * st] = c1;
#undef PC
#undef PLE
  }
}

// ------------------------------------------------------------------ DRIFTE^T
// Cells 0..NE+2: G(1) = kap1 F(2) and G(0) = kap0 G(1) are extrapolated,
// G(NE+1) = G(NE+2) = 0; faces 1..NE (not 1 and NE when closed); cell 1
// is never updated (NE >= 6).
// kCo: 0 compute the face coefficients C, 1 compute and keep them in the
// DRIFTE coefficient store, 2 read them from it.  A call's two DRIFTE
// transposes (of the reverse and the forward half) share C (same DTs and
// potential), so the first keeps it for the second, as the forward sweeps
// do; the stored value is the recomputed one, so the results do not change.
template <int kCo, int rsh>
__global__ void __launch_bounds__(128) k_adj_e(Dev d, const unsigned char* __restrict__ rec) {
  const int nr = d.nr, nt = d.nt, ne = d.ne;
  const int nlines = (nr - 1) * nt * d.npa;
  WORK_LOOP(nlines) {
    const int2 item = d.items[u / bpi];
    const int m = item.x, s = item.y, slot = m * d.ns + s;
    const int line = (int)(u % bpi) * blockDim.x + threadIdx.x;
    if (line >= nlines) continue;
    const int i = 1 + line % (nr - 1);
    const int jl = line / (nr - 1);
    const int j = jl % nt, l = jl / nt;
    const long long st = (long long)nt * nr;
    const long long base = ((long long)l * ne * nt + j) * nr + i;
    // bounds-checked builds: the line's cells, its (I,J,L) entry and UE, its
    // EDOT column, the coefficient store's item
    if (!rg_ok(d, rg_item(d, item) && rg_span(base, ne, st, d.ncell) &&
                      rg_span((long long)m * nr * nt * d.npa + ((long long)l * nt + j) * nr + i, 1, 1,
                              (long long)d.nm * nr * nt * d.npa) &&
                      rg_span((long long)s * ne * nr + i, ne, nr, (long long)d.ns * ne * nr) &&
                      (!kCo || d.item0 + u / bpi < d.coef_items),
               kRgAdjE, line))
      continue;
    double* __restrict__ lam = d.lam + (long long)slot * d.ncell + base;
    const unsigned char* __restrict__ rl = rec + (u / bpi) * d.ncell + base;
    double* __restrict__ cst = kCo ? coef_ptr(d, 2, 0, u / bpi) + base : nullptr;
    double* __restrict__ csa = kCo ? coef_ptr(d, 2, 1, u / bpi) + base : nullptr;
    const long long fij = ((long long)l * nt + j) * nr + i;
    const double wet = d.wet[fij];
    const double ue = d.ue[(long long)m * nr * nt * d.npa + fij];
    const double* __restrict__ edot = d.edot + (long long)s * ne * nr + i;
    const double* __restrict__ eb = d.eb + s * ne;
    const double hb = 0.5 * d.betalim;
    const BetaBits beta(d.betalim);
    const bool closed = d.flags & 1u;
    const int n = ne;
#define EC(K) adj_mul(4u, edot[(long long)((K)-1) * nr], fma(eb[(K)-1], wet, ue))
#define ELE(K) masked(lam, rl, (long long)((K)-1) * st, rsh)
    const double out1 = lam[0];
    // wl(K) = le(K)/WE(K) for K = 2..NE, 0 elsewhere; window = cells K-1..K+2
    const double le2 = ELE(2), le3 = ELE(3);
    double wl0 = 0.0, wl1 = le2 * d.iwe[1], wl2 = le3 * d.iwe[2];
    double cm1 = 0.0, c0 = 0.0, c1 = le2, c2 = le3;
    auto face = [&](int K) {
      const double C = (kCo == 2) ? cst[(long long)(K - 1) * st] : EC(K);
      if (kCo == 1) cst[(long long)(K - 1) * st] = C;
      const bool neg = is_neg(C);
      const int cs = (rl[(long long)(K - 1) * st] >> rsh) & 7;
      if (kAdjIntMask & 4u) {
        // the CORR factor a too goes to the store (case-free: each transpose
        // applies its own record's k)
        const bits64 a = (kCo == 2) ? dbits(csa[(long long)(K - 1) * st]) : corr_a_fix(courant_u(C, d.ide[K - 1]), neg);
        if (kCo == 1) csa[(long long)(K - 1) * st] = bitsd(a);
        face_acc_a(C * (wl1 - wl0), neg, cs, a, beta, cm1, c0, c1, c2);
      } else {
        face_acc(adj_mul(kCo == 2 ? 0u : 4u, C, wl1 - wl0), neg, cs,
                 face_ak<true>(C, neg, cs, d.mhde[K - 1], d.bmhde[K - 1], hb), cm1, c0, c1, c2);
      }
    };
    auto shift = [&](double lec, double wl) {
      cm1 = c0; c0 = c1; c1 = c2; c2 = lec;
      wl0 = wl1; wl1 = wl2; wl2 = wl;
    };
    if (!closed) face(1);
    const double g0 = cm1;  // cell 0
    { const double lec = ELE(4); shift(lec, lec * d.iwe[3]); }
    face(2);
    const double g1 = fma(d.kap[2 * s + 0], g0, cm1);  // cell 1 (+ kap0 * cell 0)
    { const double lec = ELE(5); shift(lec, lec * d.iwe[4]); }
    face(3);
    lam[st] = fma(d.kap[2 * s + 1], g1, cm1);  // cell 2 (+ kap1 * cell 1)
    { const double lec = ELE(6); shift(lec, lec * d.iwe[5]); }
    int K = 4;
    for (; K <= n - 3; ++K) {
      face(K);
      lam[(long long)(K - 2) * st] = cm1;
      const double lec = ELE(K + 3);
      shift(lec, lec * d.iwe[K + 2]);
    }
    for (; K <= n - 1; ++K) {
      face(K);
      lam[(long long)(K - 2) * st] = cm1;
      shift(0.0, 0.0);
    }
    if (!closed) face(n);
    lam[(long long)(n - 2) * st] = cm1;
    lam[(long long)(n - 1) * st] = c0;
    lam[0] = out1;
#undef EC
#undef ELE
  }
}

// ----------------------------------------------------------------- DRIFTMU^T
// Cells 1..NPA: G(1) = F(2); faces 2..NPA-2; FBND(NPA-1) = F(NPA) (0 when
// closed); cells 2..NPA-1 updated; then F2(NPA) = F2new(NPA-1)*rho
// (NPA >= 9).
// loss (may be null): the CEX/ATMOL factor table the forward sweep applied
// to its result (cells L >= 2 of its lines; the table is 1 elsewhere), so
// lambda is scaled by it as it is read, the transposed loss fused in.
template <bool kLoss, int rsh>
__global__ void __launch_bounds__(128) k_adj_mu(Dev d, const unsigned char* __restrict__ rec,
                                                const double* __restrict__ loss) {
  const int nr = d.nr, nt = d.nt, ne = d.ne, npa = d.npa;
  const int nlines = (nr - 1) * nt * ne;
  WORK_LOOP(nlines) {
    const int2 item = d.items[u / bpi];
    const int m = item.x, s = item.y, slot = m * d.ns + s;
    const int line = (int)(u % bpi) * blockDim.x + threadIdx.x;
    if (line >= nlines) continue;
    const int i = 1 + line % (nr - 1);
    const int jk = line / (nr - 1);
    const int j = jk % nt;
    const long long st = (long long)ne * nt * nr;
    const long long off = (long long)jk * nr + i;
    // bounds-checked builds: the line's cells, its WM and UM columns
    if (!rg_ok(d, rg_item(d, item) && rg_span(off, npa, st, d.ncell) &&
                      rg_span((long long)j * nr + i, npa, (long long)nt * nr, (long long)nr * nt * npa) &&
                      rg_span((long long)m * nt * nr * npa + (long long)j * nr + i, npa, (long long)nt * nr,
                              (long long)d.nm * nr * nt * npa),
               kRgAdjMu, line))
      continue;
    double* __restrict__ lam = d.lam + (long long)slot * d.ncell + off;
    const unsigned char* __restrict__ rl = rec + (u / bpi) * d.ncell + off;
    const long long sij = (long long)nt * nr;
    const long long fij = (long long)j * nr + i;
    const double* __restrict__ wm = d.wm + fij;
    const double* __restrict__ um = d.um + (long long)m * nt * nr * npa + fij;
    const double ekv = d.ek[s * ne + jk / nt];
    const double hb = 0.5 * d.betalim;
    const BetaBits beta(d.betalim);
    const bool closed = d.flags & 1u;
    const int n = npa;
#define MC(L) fma(ekv, wm[(long long)((L)-1) * sij], um[(long long)((L)-1) * sij])
    const double* __restrict__ ls = kLoss ? loss + (long long)s * d.ncell + off : nullptr;
    auto lv = [&](int L) {  // lambda of cell L (>= 2), scaled by the loss factor
      const double v = lam[(long long)(L - 1) * st];
      return kLoss ? v * ls[(long long)(L - 1) * st] : v;
    };
    auto mle = [&](int L) {  // masked as in masked(): both loads issued unconditionally
      const double v = lv(L);
      return ((__ldg(rl + (long long)(L - 1) * st) >> rsh) & kClipBit) ? 0.0 : v;
    };
#define MLE(L) mle(L)
    const double out1 = lam[0];
    // le(NPA-1) takes rho * lambda(NPA) (F2(NPA) = F2new(NPA-1)*rho)
    const double leNm = ((rl[(long long)(n - 2) * st] >> rsh) & kClipBit) ? 0.0 : fma(d.rho[fij], lv(n), lv(n - 1));
    const double le2 = MLE(2), le3 = MLE(3), le4 = MLE(4);
    double wl0 = le2 * d.iwmu[1], wl1 = le3 * d.iwmu[2], wl2 = le4 * d.iwmu[3];
    double cm1 = 0.0, c0 = le2, c1 = le3, c2 = le4;
    auto face = [&](int L) {
      const double C = MC(L);
      const bool neg = is_neg(C);
      const int cs = (rl[(long long)(L - 1) * st] >> rsh) & 7;
      if (kAdjIntMask & 8u)
        face_acc_a(adj_mul(8u, C, wl1 - wl0), neg, cs, corr_a_fix(courant_u(C, d.idmu[L - 1]), neg), beta, cm1, c0, c1,
                   c2);
      else
        face_acc(adj_mul(8u, C, wl1 - wl0), neg, cs, face_ak<true>(C, neg, cs, d.mhdmu[L - 1], d.bmhdmu[L - 1], hb),
                 cm1, c0, c1, c2);
    };
    auto shift = [&](double lec, double wl) {
      cm1 = c0; c0 = c1; c1 = c2; c2 = lec;
      wl0 = wl1; wl1 = wl2; wl2 = wl;
    };
    face(2);
    const double gb1 = cm1;  // cell 1 -> cell 2 (G(1) = F(2))
    { const double lec = MLE(5); shift(lec, lec * d.iwmu[4]); }
    face(3);
    lam[st] = cm1 + gb1;
    { const double lec = MLE(6); shift(lec, lec * d.iwmu[5]); }
    int L = 4;
    for (; L <= n - 5; ++L) {
      face(L);
      lam[(long long)(L - 2) * st] = cm1;
      const double lec = MLE(L + 3);
      shift(lec, lec * d.iwmu[L + 2]);
    }
    face(n - 4);  // cell NPA-1 enters
    lam[(long long)(n - 6) * st] = cm1;
    shift(leNm, leNm * d.iwmu[n - 2]);
    for (L = n - 3; L <= n - 2; ++L) {
      face(L);
      lam[(long long)(L - 2) * st] = cm1;
      shift(0.0, 0.0);
    }
    // window: cells NPA-2, NPA-1, NPA; FBND(NPA-1) = F(NPA): Pb(NPA-1) = -le(NPA-1)/WMU
    if (!closed) c1 -= MC(n - 1) * wl0;
    lam[(long long)(n - 3) * st] = cm1;
    lam[(long long)(n - 2) * st] = c0;
    lam[(long long)(n - 1) * st] = c1;
    lam[0] = out1;
#undef MC
#undef MLE
  }
}

void launch_adj_sweep(const Dev& d, int w, const unsigned char* rec, int rsh, cudaStream_t st, int co,
                      const double* loss) {
  const int blk = 128;
  int nl;
  switch (w) {
    case 0: nl = d.nt * d.ne * d.npa; break;
    case 1: nl = (d.nr - 1) * d.ne * d.npa; break;
    case 2: nl = (d.nr - 1) * d.nt * d.npa; break;
    default: nl = (d.nr - 1) * d.nt * d.ne; break;
  }
  dim3 g((nl + blk - 1) / blk, d.nitems, 1);
  // the record nibble is a template parameter: 0 low (reverse half), 4 high
  auto go = [&](auto sh) {
    constexpr int R = decltype(sh)::value;
    switch (w) {
      case 0: k_adj_r<R><<<g, blk, adj_r_smem(d, blk), st>>>(d, rec); break;
      case 1: k_adj_p<R><<<g, blk, 0, st>>>(d, rec); break;
      case 2:
        if (co == 1) k_adj_e<1, R><<<g, blk, 0, st>>>(d, rec);
        else if (co == 2) k_adj_e<2, R><<<g, blk, 0, st>>>(d, rec);
        else k_adj_e<0, R><<<g, blk, 0, st>>>(d, rec);
        break;
      default:
        if (loss) k_adj_mu<true, R><<<g, blk, 0, st>>>(d, rec, loss);
        else k_adj_mu<false, R><<<g, blk, 0, st>>>(d, rec, nullptr);
        break;
    }
  };
  if (rsh) go(std::integral_constant<int, 4>());
  else go(std::integral_constant<int, 0>());
}

// ---------------------------------------------------------- ram_run tail^T
// Forward order: F2(:,:,NT,:,:) = F2(:,:,1,:,:); mask; ANISCH's
// F2(I,J,K,1) = F2(I,J,K,2) (I, K >= 2).  Adjoint in reverse.
__global__ void k_adj_anisch(Dev d) {
  const long long n = (long long)(d.nr - 1) * d.nt * (d.ne - 1);
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int2 item = d.items[blockIdx.y];
  const int slot = item.x * d.ns + item.y;
  const int i = 1 + (int)(t % (d.nr - 1));
  const int j = (int)((t / (d.nr - 1)) % d.nt);
  const int k = 1 + (int)(t / ((long long)(d.nr - 1) * d.nt));
  double* lam = d.lam + (long long)slot * d.ncell + ((long long)k * d.nt + j) * d.nr + i;
  const long long st = (long long)d.ne * d.nt * d.nr;
  lam[st] += lam[0];
  lam[0] = 0.0;
}

__global__ void k_adj_copy_mask(Dev d, int any_outside) {
  const long long n = (long long)d.nr * d.ne * d.npa;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int2 item = d.items[blockIdx.y];
  const int slot = item.x * d.ns + item.y;
  const int i = (int)(t % d.nr);
  const long long kl = t / d.nr;
  double* lam = d.lam + (long long)slot * d.ncell + kl * d.nt * d.nr + i;
  if (any_outside)
    for (int j = 0; j < d.nt; ++j)
      if (d.outside[(long long)j * d.nr + i] == 1) lam[(long long)j * d.nr] = 0.0;
  lam[0] += lam[(long long)(d.nt - 1) * d.nr];
  lam[(long long)(d.nt - 1) * d.nr] = 0.0;
}

void launch_adj_tail(const Dev& d, cudaStream_t st) {
  long long n1 = (long long)(d.nr - 1) * d.nt * (d.ne - 1);
  k_adj_anisch<<<dim3((unsigned)((n1 + 255) / 256), d.nitems), 256, 0, st>>>(d);
  long long n2 = (long long)d.nr * d.ne * d.npa;
  k_adj_copy_mask<<<dim3((unsigned)((n2 + 255) / 256), d.nitems), 256, 0, st>>>(d, (d.flags >> 31) & 1u);
}

// ------------------------------------------------------------- observations
// flux = F2/FFACTOR/FNHS (src/ModRamRun.f90:214) at bin (K, L), bilinear in
// (L-shell, MLT) over the four cells (i0|i0+1, j0|j1).
__device__ __forceinline__ double obs_cell_factor(const Dev& d, int s, int i, int j, int k, int l) {
  const double ff = d.ffactor[(long long)s * d.nr * d.ne * d.npa + ((long long)l * d.ne + k) * d.nr + i];
  const double fh = d.fnhs[((long long)l * d.nt + j) * d.nf + i];
  return ff * fh;
}

__global__ void k_obs_fwd(Dev d, const ObsDev* __restrict__ obs, int nobs, int call, double* fm,
                          double* J) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nobs) return;
  const ObsDev o = obs[t];
  if (o.call != call) return;
  const int s = o.slot % d.ns;
  const double* f2 = d.f2 + (long long)o.slot * d.ncell;
  double v = 0.0;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      const int i = o.i0 + a, j = b ? o.j1 : o.j0;
      const double w = (a ? o.wi : 1.0 - o.wi) * (b ? o.wj : 1.0 - o.wj);
      const long long c = (((long long)o.l * d.ne + o.k) * d.nt + j) * d.nr + i;
      const double ff = d.ffactor[(long long)s * d.nr * d.ne * d.npa + ((long long)o.l * d.ne + o.k) * d.nr + i];
      const double fh = d.fnhs[((long long)o.l * d.nt + j) * d.nf + i];
      v += w * (f2[c] / ff / fh);
    }
  fm[t] = v;
  const double r = log(v) - o.log_obs;
  atomicAdd(&J[o.member], r * r);
}

__global__ void k_obs_adj(Dev d, const ObsDev* __restrict__ obs, int nobs, int call,
                          const double* __restrict__ fm) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nobs) return;
  const ObsDev o = obs[t];
  if (o.call != call || o.item < d.item0 || o.item >= d.item0 + d.nitems) return;  // call c, this group
  const int s = o.slot % d.ns;
  const double v = fm[t];
  const double g = 2.0 * (log(v) - o.log_obs) / v;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      const int i = o.i0 + a, j = b ? o.j1 : o.j0;
      const double w = (a ? o.wi : 1.0 - o.wi) * (b ? o.wj : 1.0 - o.wj);
      const long long c = (((long long)o.l * d.ne + o.k) * d.nt + j) * d.nr + i;
      atomicAdd(&d.lam[(long long)o.slot * d.ncell + c], g * w / obs_cell_factor(d, s, i, j, o.k, o.l));
    }
}

void launch_obs_fwd(const Dev& d, const ObsDev* obs, int nobs, int call, double* fm, double* J,
                    cudaStream_t st) {
  if (nobs > 0) k_obs_fwd<<<(nobs + 127) / 128, 128, 0, st>>>(d, obs, nobs, call, fm, J);
}
void launch_obs_adj(const Dev& d, const ObsDev* obs, int nobs, int call, const double* fm,
                    cudaStream_t st) {
  if (nobs > 0) k_obs_adj<<<(nobs + 127) / 128, 128, 0, st>>>(d, obs, nobs, call, fm);
}

// Order-independent digest of a branch record: two sums (mod 2^32) of
// position-mixed 32-bit hashes of its 32-bit words, read 16 bytes at a time
// (a ragged tail byte by byte).  Equal digests of two runs mean an
// unchanged pattern with overwhelming probability.
__device__ __forceinline__ unsigned mix32(unsigned w, unsigned long long i, unsigned c1, unsigned c2) {
  unsigned h = (w + (unsigned)i * 0x9E3779B9u + (unsigned)(i >> 32)) * c1;
  h ^= h >> 15;
  h *= c2;
  return h ^ (h >> 13);
}

__global__ void k_digest(const unsigned char* __restrict__ rec, long long n, unsigned long long* out) {
  unsigned lo = 0u, hi = 0u;
  const bool al = ((unsigned long long)rec & 15ULL) == 0ULL;
  const long long n16 = al ? n / 16 : 0;
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long nth = (long long)gridDim.x * blockDim.x;
  const uint4* r4 = reinterpret_cast<const uint4*>(rec);
  for (long long c = tid; c < n16; c += nth) {
    const uint4 v = r4[c];
    const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const unsigned long long i = 4ULL * c + q;
      lo += mix32(w[q], i, 0x85EBCA6Bu, 0xC2B2AE35u);
      hi += mix32(w[q], i, 0x27D4EB2Fu, 0x165667B1u);
    }
  }
  for (long long b = 16 * n16 + tid; b < n; b += nth) {
    const unsigned long long i = 0x100000000ULL + (unsigned long long)b;
    lo += mix32(rec[b], i, 0x85EBCA6Bu, 0xC2B2AE35u);
    hi += mix32(rec[b], i, 0x27D4EB2Fu, 0x165667B1u);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo += __shfl_xor_sync(0xffffffffu, lo, o);
    hi += __shfl_xor_sync(0xffffffffu, hi, o);
  }
  if ((threadIdx.x & 31) == 0) atomicAdd(out, ((unsigned long long)hi << 32) + lo);
}

void launch_digest(const unsigned char* rec, long long n, unsigned long long* out, cudaStream_t st) {
  k_digest<<<1024, 256, 0, st>>>(rec, n, out);
}

}  // namespace ramgpu
