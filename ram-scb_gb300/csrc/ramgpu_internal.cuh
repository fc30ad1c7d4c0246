// ramgpu_internal.cuh -- device-side state and shared helpers of the GB300
// RAM kinetic step.
//
// Data layout in HBM (all FP64, Fortran order inside one species):
//   f2      [member][species][L][K][J][I]   (= F2(S,I,J,K,L) of the reference
//                                            with S hoisted out; I fastest)
//   fields  [L][J][I'] with I' = 1..NR+1     (FNHS etc., src/ModRamVariables.f90:31-37)
//   per-member tables (VT-dependent) [member][L][J][I]
//   per-species tables (DTs-dependent) [species][...]
// One thread advances one line of a sweep; the line is streamed through a
// rolling register window, so no line buffer is kept.
//
// Cost model: on GB300 the FP64 pipe (add/mul/fma, and also FP64 min/max and
// compares) issues ~0.53 T lane-ops/s while the integer and FP32 pipes are
// ~35-70x faster, so every sign test, threshold test, min/max and select is
// done on the integer bit pattern, leaving 8-9 FP64 add/mul/fma per face.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ramgpu {

constexpr double kOME = 7.3E-5;        // Earth's angular velocity, src/ModRamDrift.f90:224
constexpr double kRE = 6.371E6;        // src/ModRamConst.f90:14
constexpr double kQ = 1.602E-19;       // src/ModRamConst.f90:19
constexpr double kCS = 2.998E8;        // src/ModRamConst.f90:20
constexpr double kPI = 3.1415926535897932384626433832795;

struct Dev {
  // sizes
  int nr, nt, ne, npa, ns, nm;
  long long ncell;  // NR*NT*NE*NPA
  int nf;           // NR+1
  // scalars
  double mdr, dphi, dl1, conf1, conf2, betalim;
  unsigned flags;
  // grid vectors
  const double *lz, *rlz, *phi, *ekev, *ebnd, *we, *de, *mu, *dmu, *wmu;
  const double *lr2, *sinphi;  // (LZ(I)*RE)**2 (NR+1) and SIN(PHI(J)-PHIOFS) (NT) of the VOLS formula
  const int *upa_atm;   // int(UPA(I)): first loss-cone L (1-based), NR
  const int *upa_mom;   // int(UPA(I)-1): last L of the ANISCH sum, NR
  // reciprocal grid tables: -0.5/DE, 1/WE, 1/DE (NE); -0.5/DMU, 1/WMU, 1/DMU (NPA)
  const double *mhde, *iwe, *ide, *mhdmu, *iwmu, *idmu;
  const double *bmhde, *bmhdmu;  // BetaLim times -0.5/DE and -0.5/DMU (adjoint)
  // per-species grid (ns x NE)
  const double *grel, *grbnd, *vel;
  const double *epp;
  const double *rmas;     // (ns)
  const double *ffactor;  // (ns, NR, NE, NPA)
  const int *qs;        // species charge
  const int *cex_kind;
  // fields, (NR+1,NT,NPA) / (NR+1,NT) / int (NR,NT)
  const double *fnhs, *fnis, *bounhs, *bounis, *hdns, *didt, *dibndt;
  const double *bnes, *dbdt, *eir, *eip;
  const int *outside;
  // field-only derived tables, (NR,NT,NPA) unless noted
  double *grt;            // R: gradient-curvature factor, CGR = grt*P4(K)
  double *gpt;            // P: CDriftP = A(I,J) + P2(I,K)*gpt
  double *gre, *gpe, *ze, *wet;   // E: GPR1+2+3, GPP1+2, dBdt1+dIdt1, EDT1 factor
  double *gmr, *gmp, *zm, *hm, *cmu0;  // MU
  double *rho;            // (NR,NT): FNHS(NPA)*MU(NPA)/FNHS(NPA-1)/MU(NPA-1)
  double *mw_a;           // (ns, NPA, NE, NR): ANISCH weight RFAC*EPP(K)/FFACTOR
  double *mw_be, *mw_ba;  // (NPA, NT, NR): ANISCH weights WMU/FNHS*(1-MU^2), 2*WMU/FNHS*MU^2
  double *mws_a;          // (ns, NE, NR): RFAC*EPP(K)*MU(2)/FFACTOR(L=2), the separable species factor
  double *mws_be, *mws_ba;  // (NPA, NT, NR): mw_be, mw_ba over MU'(L) (MU'(1) = MU(2))
  int mom_sep;            // FFACTOR has the separable ARRAYS form: two-fma moment sums
  // DTs-dependent per-species small tables
  double *p4;             // (ns, NE)
  double *p2;             // (ns, NR, NE)
  double *edot;           // (ns, NR, NE)
  double *eb, *ek;        // (ns, NE)
  double *kap;            // (ns, 2): extrapolation factors of F(1), F(0) in DRIFTE
  double *wm;             // (NR,NT,NPA): -CMUDOT*HM, DTs-dependent, species-free
  double *cmudot;         // (NR,NT,NPA): MUDOT(I,L)*BOUNIS/BOUNHS, DTs-dependent
  double *loss1;          // (ns, ncell): CHARGE*ATLOS^(1/FNHS) (one half step)
  double *loss2;          // (ns, ncell): ((CHARGE*ATM)*ATM)*CHARGE (both halves)
  double *charge, *atm;   // (ns, ncell): separate factors for the bookkeeping path
  // implicit pitch-angle diffusion (WPADIF / FLCscatter): per species the
  // coefficient D and the elimination tables; FACMU and 1/FACMU (NR,NT,NPA)
  const int *pd_on;       // (ns): species has a coefficient
  const double *pd_d;     // (ns, ncell)
  double *pd_gn, *pd_inv, *pd_rl;  // (ns, ncell)
  double *pd_fac, *pd_ifac;        // (NR, NT, NPA)
  // per-member VT-dependent tables
  double *kp;             // (nm)
  int *vt_mode;           // (nm): 1 = VOLS from kp, 0 = explicit VT
  double *vt;             // (nm, NR+1, NT)
  double *cr;             // (nm, NR, NT)
  double *ca;             // (nm, NR, NT)
  double *ue, *um;        // (nm, NR, NT, NPA)
  double *drd1, *dpd1;    // (nm, NR, NT): DRD1 = DRM1, DPD1 = DPM1 of DRIFTE/DRIFTMU
  double *mij;            // (8, NT, NR): VT-independent factors of cr, ca, drd1, dpd1 (DTs, fields)
  // per (member, species) slot
  double *f2;             // (nm*ns, ncell)
  double *fgeos;          // (nm*ns, NT*NE*NPA)
  double *plane_last;     // (nm*ns, NE*NPA): DRIFTR F(NR+1) of the last inflow line of plane (K,L)
  int *plane_has;         // (nm*ns, NE*NPA): plane (K,L) has an inflow line
  double *plane_carry;    // (nm*ns, NE*NPA): F(NR+1) left by planes before (K,L) in K->L order
  int *plane_last_src;    // (nm*ns, NE*NPA): FGEOS index (L*NE+K)*NT+J of that last inflow line
  int *plane_carry_src;   // (nm*ns, NE*NPA): FGEOS index behind plane_carry, -1 if none
  // frozen-limiter adjoint: lambda (same layout as f2) and dJ/dFGEOS per slot
  double *lam;            // (nm*ns, ncell)
  double *gfg;            // (nm*ns, NT*NE*NPA)
  unsigned long long *cflq;  // (nm*ns, 4): max over cells of the CFL quotient, as bits
  unsigned long long *clipq;  // (nm*ns): clip events of the last call (follows cflq)
  int count_clips;            // the sweeps count clip events (status pass on)
  double *mom_part;       // (nm*ns, NT, NR, (NE-1)*4 chunks, 2) moment partials
  double *ppert, *ppart;  // (nm*ns, NR, NT)
  double *sumrc_part;     // (nm*ns, nblk) SUMRC partial sums
  // face coefficients C and a of the forward sweeps, read back by the
  // reverse ones: (stored sweeps, 2, coef_items, ncell); coef_slot[w] is
  // sweep w's place or -1; null when not allocated
  double *coef;
  long long coef_items;
  int coef_slot[4];
  // work list
  const int2 *items;      // (member, species)
  int nitems;
  int item0;              // position of items[0] in the full list (a group's view of it)
  // launch shape of the sweeps R, P, E, MU: threads per CTA and, when > 0,
  // a persistent grid of that many CTAs looping over (item, line-block) units
  int blk[4];
  int pers[4];
  int mu_lanes;  // lanes per DRIFTMU line: 2 (lane pairs, NPA >= 12) or 1
  // L window of the R, P and E sweeps and the closing copy/mask: planes
  // [lw0, lw1) (0 and NPA: all); a host pipeline runs them chunk by chunk
  int lw0, lw1;
  // bounds-checked builds: {failed tests, first check id + 1, its value};
  // null otherwise
  unsigned long long* bounds;
};

// ---------------------------------------------------- bounds-checked builds
// Compiled with RAMGPU_BOUNDS_CHECK (libramgpu_bounds.so), the streaming
// kernels test, per line, the index ranges they are about to use (work
// item, slot, the line's first and last cell, the table rows it reads).  A
// failed test is counted in the context's log with the id of the first one
// and its value, and the line is skipped, so nothing is read or written out
// of range; the line's lanes still take part in every warp-wide operation.
// Without the macro the tests compile away (rg_ok is true).
#ifdef RAMGPU_BOUNDS_CHECK
__device__ __forceinline__ bool rg_ok(const Dev& d, bool ok, int check, long long value) {
  if (!ok && d.bounds) {
    if (atomicAdd(d.bounds, 1ULL) == 0ULL) {
      d.bounds[1] = (unsigned long long)(check + 1);
      d.bounds[2] = (unsigned long long)value;
    }
  }
  return ok;
}
#else
__device__ __forceinline__ bool rg_ok(const Dev&, bool, int, long long) { return true; }
#endif
// [first, first + (n - 1) * stride] inside [0, size)
__device__ __forceinline__ bool rg_span(long long first, long long n, long long stride, long long size) {
  return first >= 0 && n >= 1 && first + (n - 1) * stride < size;
}
// The work item's (member, species) and slot inside the context's arrays.
__device__ __forceinline__ bool rg_item(const Dev& d, int2 item) {
  return item.x >= 0 && item.x < d.nm && item.y >= 0 && item.y < d.ns;
}
// check ids
enum RgCheck { kRgSweepR = 1, kRgSweepP, kRgSweepE, kRgSweepMu, kRgAdjR = 11, kRgAdjP, kRgAdjE, kRgAdjMu,
               kRgGather = 21, kRgScatter };

// ---------------------------------------------------------------- bit tests
// The bit pattern moves through an opaque PTX mov: with a plain bit cast
// the compiler may fold the integer sign-bit masks and tests below back
// into FP64 abs/negate/compare instructions, which issue on the FP64 pipe.
using bits64 = unsigned long long;
constexpr bits64 kAbsMask = 0x7FFFFFFFFFFFFFFFULL;
constexpr bits64 kSignMask = 0x8000000000000000ULL;
__device__ __forceinline__ bits64 dbits(double x) {
  bits64 u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  return u;
}
__device__ __forceinline__ double bitsd(bits64 u) {
  double x;
  asm("mov.b64 %0, %1;" : "=d"(x) : "l"(u));
  return x;
}
constexpr bits64 kMantMask = 0x000FFFFFFFFFFFFFULL;
constexpr bits64 kImplicit = 0x0010000000000000ULL;
// The limiter's beta (1 <= beta <= 2, as the ABI clamps it): its 53-bit
// significand shifted left by 11, and its unbiased exponent (0, or 1 for 2).
struct BetaBits {
  double beta;
  bits64 m11;
  int e;
  __device__ __forceinline__ explicit BetaBits(double b) : beta(b) {
    const bits64 u = dbits(b);
    m11 = ((u & kMantMask) | kImplicit) << 11;
    e = (int)(u >> 52) - 1023;
  }
};
// beta*|x| as bits, formed on the integer pipe: the product of the two
// significands by a 64x64-bit high multiply, truncated to 53 bits (at most
// one unit in the last place below the rounded FP64 product; the limiter
// compares these bits and, in its beta branches, uses them as the value).
// Subnormal and zero |x| give the subnormal-range product the same way;
// inf and NaN pass through.  Replaces one FP64 multiply per face.
__device__ __forceinline__ bits64 babs_bits(const BetaBits& b, double x) {
  const bits64 ax = dbits(x) & kAbsMask;
  const int ex = (int)(ax >> 52);
  const bits64 mant = ax & kMantMask;
  const bits64 mx = ex ? (mant | kImplicit) : mant;
  const bits64 p = __umul64hi(mx << 11, b.m11);  // floor(mx*mb / 2^42)
  const int hi = (int)(p >> 63);                  // normal |x|: p in [2^62, 2^64)
  const bits64 normal = ((bits64)(ex + b.e + hi) << 52) | ((p >> (10 + hi)) & kMantMask);
  const bits64 sub = (p >> 10) << b.e;            // floor(mant*beta) < 2^53: its own encoding
  return ex == 0x7FF ? ax : (ex ? normal : sub);
}
// ax*y as bits for a non-negative normal ax (bits) and a positive normal y,
// formed on the integer pipe as in babs_bits (truncated: at most one unit in
// the last place below the rounded FP64 product); inf and NaN pass through.
// The CFL quotients |C|/DE and |C|/DMU are only compared and maximised, so
// this replaces one FP64 multiply per face in DRIFTE and DRIFTMU.
__device__ __forceinline__ bits64 mul_pos_bits(bits64 ax, double y) {
  const bits64 uy = dbits(y);
  const int ex = (int)(ax >> 52);
  const bits64 p = __umul64hi(((ax & kMantMask) | kImplicit) << 11, ((uy & kMantMask) | kImplicit) << 11);
  const int hi = (int)(p >> 63);
  const bits64 r = ((bits64)(ex + (int)(uy >> 52) - 1023 + hi) << 52) | ((p >> (10 + hi)) & kMantMask);
  return ex == 0x7FF ? ax : r;
}
// The CORR factor a = 0.5*(s - u) of a face, s = +-1 the upwind sign and
// u >= 0 its Courant number (|C| in R and P, |C|/DE and |C|/DMU in E and
// MU), i.e. a = s*0.5*(1 - u), formed on the integer pipe for u < 1:
// 1 - u in 64-bit fixed point (2^63 is 1; exact for u >= 2^-11, below that
// u loses bits past 2^-63), normalised by a count of leading zeros and cut
// to 53 bits.  The result is at most one unit in the last place below the
// rounded 0.5*(s - u) (the FP64 fma it replaces) in magnitude; it only
// scales the limited correction a*LX, so the flux it feeds stays within the
// 1e-12 parity bar and conservation is untouched (the flux leaving one cell
// is the flux entering the next).  ub: bits of u (non-negative); u >= 1,
// inf and NaN take the FP64 fma fma(c, mh, s*0.5) behind a warp-uniform
// branch.  Replaces one FP64 operation per face.
static __device__ __noinline__ double corr_a_fallback(double c, double mh, bool neg) {
  return fma(c, mh, neg ? -0.5 : 0.5);
}
__device__ __forceinline__ double corr_a_int(bits64 ub, bool neg, double c, double mh) {
  const int eu = (int)(ub >> 52);
  const bits64 mu = (ub & kMantMask) | (eu ? kImplicit : 0ULL);
  const int sl = eu - 1012;  // E + 11: U = u * 2^63
  const bits64 U = sl >= 0 ? (mu << (sl < 63 ? sl : 63)) : (mu >> (-sl < 63 ? -sl : 63));
  const bits64 D = 0x8000000000000000ULL - U;  // (1 - u) * 2^63 > 0 for u < 1
  const int lz = __clzll((long long)D);
  const bits64 N = D << lz;
  double out = bitsd((neg ? kSignMask : 0ULL) | ((bits64)(1022 - lz) << 52) | ((N >> 11) & kMantMask));
  if (eu >= 1023) out = corr_a_fallback(c, mh, neg);
  return out;
}

// a*b rounded to nearest even, computed on the integer pipe: the 53-bit
// significands' 106-bit product from a 64x64 multiply (high and low
// halves), the dropped bits and a sticky bit decide the rounding (IEEE-754
// round-half-even), the exponents add.  Zero operands give the signed zero;
// subnormal, infinite and NaN operands and results outside the normal range
// take the FP64 multiply, behind a warp-uniform branch so that warps without
// such a lane do not issue it.  Bit-identical to the FP64 multiply; it
// moves work off the FP64 unit, which is the limit of the sweeps.
// The fallback lives out of line: a one-instruction body would be turned
// into a predicated FP64 multiply, which the FP64 unit still issues.
static __device__ __noinline__ double mul_rn_fallback(double a, double b) { return a * b; }
__device__ __forceinline__ double mul_rn_int(double a, double b) {
  const bits64 ua = dbits(a), ub = dbits(b);
  const bits64 sign = (ua ^ ub) & kSignMask;
  const int ea = (int)((ua >> 52) & 0x7FF), eb = (int)((ub >> 52) & 0x7FF);
  const bits64 x = ((ua & kMantMask) | kImplicit) << 11, y = ((ub & kMantMask) | kImplicit) << 11;
  const bits64 hi = __umul64hi(x, y);  // product / 2^64, in [2^62, 2^64)
  const bits64 lo = x * y;
  const int top = (int)(hi >> 63);
  const int sh = 10 + top;
  bits64 sig = hi >> sh;                       // 53 bits
  const bits64 rem = hi & ((1ULL << sh) - 1);  // dropped bits of the high half
  const bits64 half = 1ULL << (sh - 1);
  const bool up = rem > half || (rem == half && (lo != 0 || (sig & 1)));
  sig += up ? 1 : 0;
  const int carry = (int)(sig >> 53);          // rounded up to 2^53
  sig >>= carry;
  const int E = ea + eb - 1023 + top + carry;
  bits64 r = sign | ((bits64)E << 52) | (sig & kMantMask);
  const bool zero = ((ua << 1) == 0) | ((ub << 1) == 0);
  r = zero ? sign : r;
  const bool special = (ea == 0x7FF) | (eb == 0x7FF) | (!zero & ((ea == 0) | (eb == 0) | (E <= 0) | (E >= 0x7FF)));
  double out = bitsd(r);
  if (special) out = mul_rn_fallback(a, b);
  return out;
}
// x < 0.0 exactly as the Fortran test `C.lt.0` (false for -0.0 and NaN with
// the sign bit clear).
__device__ __forceinline__ bool is_neg(double x) { return dbits(x) > 0x8000000000000000ULL; }
// |x| > 1e-27
__device__ __forceinline__ bool abs_gt_1em27(double x) {
  const unsigned long long t = 0x3A53CE9A36F23C10ULL;  // bits of 1.0E-27
  return (dbits(x) & 0x7FFFFFFFFFFFFFFFULL) > t;
}
// d*x > 0 (both nonzero, same sign)
__device__ __forceinline__ bool same_sign_nonzero(double d, double x) {
  unsigned long long bd = dbits(d), bx = dbits(x);
  return ((long long)(bd ^ bx) >= 0) && ((bd << 1) != 0) && ((bx << 1) != 0);
}

// min / max of non-negative doubles on their bit patterns (integer pipe).
// For x, y >= +0 the IEEE-754 encodings order like the values; FP64
// fmin/fmax would issue on the slow FP64 pipe.
__device__ __forceinline__ unsigned long long umin64(unsigned long long a, unsigned long long b) {
  return a < b ? a : b;
}
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}

// Flux-limited face value of the reference sweeps (src/ModRamDrift.f90:169-183):
//   FUP = upwind value; if |X|<=1e-27 or R<=0: FBND=FUP
//   else FBND = FUP + LIMITER(R)*CORR, LIMITER = max(min(beta R,1),min(R,beta)),
//        CORR = -0.5*(Cd - s)*X = a*X,  R = D/X.
// Division-free: for D*X>0, LIMITER*X = sign(X)*max(min(beta|D|,|X|),min(|D|,beta|X|)).
// bx = beta*|x|, bd = beta*|d| as bits (bd is the neighbour face's bx).
// The min/max run on bit patterns of the non-negative magnitudes, so a face
// costs one FP64 fma here.  cs reports which limiter candidate was taken,
// for the frozen-limiter adjoint: 0 upwind only, 1 beta*D, 2 X, 3 D, 4 beta*X.
__device__ __forceinline__ double face_value_case(double x, bits64 bx, double d, bits64 bd,
                                                  double fup, double a, int& cs) {
  const bits64 ux = dbits(x), ud = dbits(d);
  const bits64 m1 = umin64(bd, ux & kAbsMask);
  const bits64 m2 = umin64(ud & kAbsMask, bx);
  const bits64 m = umax64(m1, m2);
  const double lx = bitsd(m | (ux & kSignMask));
  const double fb = fma(a, lx, fup);
  const bool act = abs_gt_1em27(x) && same_sign_nonzero(d, x);
  cs = !act ? 0 : (m == m1 ? (m1 == bd ? 1 : 2) : (m2 == (ud & kAbsMask) ? 3 : 4));
  return act ? fb : fup;
}
constexpr int kClipBit = 8;  // recorded with the case: the updated cell was clipped
// kRec modes of the sweeps: 0 plain, 1 record branches, 2 replay them,
// 3 plain and count clip events into Dev::clipq
constexpr int kRecCount = 3;

// Stored face coefficient array q (0: C, 1: a) of sweep w for work item `it`.
__device__ __forceinline__ double* coef_ptr(const Dev& d, int w, int q, long long it) {
  return d.coef + (((long long)(d.coef_slot[w] * 2 + q) * d.coef_items) + d.item0 + it) * d.ncell;
}

// Face value with the branch taken from a record (frozen-limiter replay):
// LIMITER*X = beta*D | X | D | beta*X for cases 1..4, FUP for case 0, the
// beta products formed as in face_value_case.  For the recorded branch this
// equals face_value_case bit for bit.
__device__ __forceinline__ double face_value_frozen(double x, double d, double fup, double a, const BetaBits& beta,
                                                    int cs) {
  const double bd = bitsd(babs_bits(beta, d) | (dbits(d) & kSignMask));
  const double bx = bitsd(babs_bits(beta, x) | (dbits(x) & kSignMask));
  const double lx = cs == 1 ? bd : cs == 2 ? x : cs == 3 ? d : bx;
  return cs ? fma(a, lx, fup) : fup;
}
// F2 < 0 -> 1e-15 applied as recorded
__device__ __forceinline__ double clip_frozen(double v, unsigned char r) { return (r & kClipBit) ? 1E-15 : v; }

// Running CFL quotient max(|C|, floor) as bits (integer max).
__device__ __forceinline__ unsigned long long cfl_bits(double c, unsigned long long floor_bits) {
  return umax64(dbits(c) & kAbsMask, floor_bits);
}
constexpr unsigned long long kBits1em10 = 0x3DDB7CDFD9D7BDBBULL;  // 1.0E-10
constexpr unsigned long long kBits1em32 = 0x3949F623D5A8A733ULL;  // 1.0E-32

// F2 < 0 -> 1e-15 (src/ModRamDrift.f90:187-190)
__device__ __forceinline__ double clip(double v) { return is_neg(v) ? 1E-15 : v; }

// 64-bit max-reduction of a non-negative double across a warp, then one
// atomicMax on the bit pattern (order-independent, hence deterministic).
// Warp sum of a per-lane count added to *slot (every lane of the warp calls it).
__device__ __forceinline__ void warp_atomic_add(unsigned long long *slot, unsigned v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v != 0u) atomicAdd(slot, (unsigned long long)v);
}

__device__ __forceinline__ void warp_atomic_max(unsigned long long *slot, unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  if ((threadIdx.x & 31) == 0 && v != 0ULL) atomicMax(slot, v);
}

__host__ __device__ inline long long idx4(int i, int j, int k, int l, int nr, int nt, int ne) {
  return (((long long)l * ne + k) * nt + j) * nr + i;
}

}  // namespace ramgpu
