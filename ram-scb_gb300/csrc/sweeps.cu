// sweeps.cu -- the four operator-split flux-limited upwind sweeps of RAM.
//
// Each kernel advances whole lines in place: thread (blockIdx.x*blockDim.x +
// threadIdx.x) owns one line of the swept axis, blockIdx.y indexes the
// (member, species) work item.  The line is streamed once through a rolling
// window G(f-1..f+2) kept in registers, so every F2 value is read once and
// written once per sweep.  The face arithmetic follows the reference:
//   DRIFTR  src/ModRamDrift.f90:95-198
//   DRIFTP  src/ModRamDrift.f90:204-279
//   DRIFTE  src/ModRamDrift.f90:285-376
//   DRIFTMU src/ModRamDrift.f90:382-473
// with the face coefficients taken from separable tables built in tables.cu
// (C = A(I,J) + G(I,J,L)*k(K) etc.).  The FP64 unit is the limit: sign,
// abs and limiter tests run on bit patterns, and the products that are only
// compared (beta*|X|, the CFL quotients) and the flux C*FBND (mul_rn_int,
// rounded exactly like the FP64 multiply) run on the integer pipe, leaving
// 6 FP64 add/mul/fma per face.  More integer work than that made the
// forward DRIFTE and DRIFTMU issue-bound (measured).
#include "ramgpu_internal.cuh"
#include "kernels.cuh"

namespace ramgpu {

// Branch records hold two sweeps per byte, four bits each (three case bits
// and the clip bit): a call's forward-half sweep in the high nibble
// (rsh = 4), written first, and the reverse-half sweep of the same
// direction in the low one, which ORs its code into that byte.  (The
// reverse half is transposed first; its nibble is the cheaper one to read.)
__device__ __forceinline__ unsigned rget(const unsigned char* p, int rsh) { return (unsigned)*p >> rsh; }
__device__ __forceinline__ void rput(unsigned char* p, int rsh, unsigned v) {
  *p = (unsigned char)(rsh ? (v << 4) : (*p | v));
}

// ----------------------------------------------------------------- DRIFTR
// Line (J,K,L) along I = 1..NR.  Faces 2..NR-1 (and NR on inflow lines).
template <bool kCfl, int kRec, int kCo>
__global__ void __launch_bounds__(256) k_sweep_r(Dev d, double dts, unsigned char* __restrict__ rec, int rsh) {
  const int nr = d.nr, nt = d.nt, ne = d.ne;
  // the lines of the L window [lw0, lw1) (all of them unless a pipeline
  // runs the step plane chunk by plane chunk): L is the slowest index
  const int line0 = d.lw0 * nt * ne;
  const int nlines = nt * ne * (d.lw1 - d.lw0);
  // Work units are (item, block of lines).  A grid of (blocks per item,
  // items) gives one unit per CTA; a persistent grid loops over them.
  const int bpi = (nlines + blockDim.x - 1) / blockDim.x;
  const long long nunits = (long long)bpi * d.nitems;
  for (long long u = blockIdx.x + (long long)blockIdx.y * gridDim.x; u < nunits;
       u += (long long)gridDim.x * gridDim.y) {
    const int2 item = d.items[u / bpi];
    const int m = item.x, s = item.y, slot = m * d.ns + s;
    const int line = line0 + (int)(u % bpi) * blockDim.x + threadIdx.x;
    unsigned long long q = 0ULL;  // CFL quotient bits
    unsigned nclip = 0;  // clip events (kRec == kRecCount)
    // bounds-checked builds: the line's cells, its GRT and CR rows, the
    // coefficient store's item
    const bool lok = line >= line0 + nlines ||
        rg_ok(d, rg_item(d, item) && rg_span((long long)line * nr, nr, 1, d.ncell) &&
                     rg_span(((long long)(line / (nt * ne)) * nt + line % nt) * nr, nr, 1, (long long)nr * nt * d.npa) &&
                     rg_span(((long long)item.x * nt + line % nt) * nr, nr, 1, (long long)d.nm * nr * nt) &&
                     (!kCo || d.item0 + u / bpi < d.coef_items),
              kRgSweepR, line);
    if (line < line0 + nlines && lok) {
      const int j = line % nt;
      const int l = line / (nt * ne);
      double* __restrict__ fl = d.f2 + (long long)slot * d.ncell + (long long)line * nr;
      // branch record of the frozen-limiter adjoint: one byte per face/cell
      unsigned char* __restrict__ rl = (kRec == 1 || kRec == 2) ? rec + (u / bpi) * d.ncell + (long long)line * nr : nullptr;
      // face coefficients C and CORR factor a: stored by the forward sweep,
      // read back by the reverse one (same DTs, same potential)
      double* __restrict__ cst = kCo ? coef_ptr(d, 0, 0, u / bpi) + (long long)line * nr : nullptr;
      double* __restrict__ ast = kCo ? coef_ptr(d, 0, 1, u / bpi) + (long long)line * nr : nullptr;
      const double* __restrict__ grt = d.grt + ((long long)l * nt + j) * nr;
      const double* __restrict__ cr = d.cr + ((long long)m * nt + j) * nr;
      const int* __restrict__ outside = d.outside + (long long)j * nr;
      const double p4 = d.p4[s * ne + (line / nt) % ne];
      const BetaBits beta(d.betalim);
      const bool closed = d.flags & 1u;

      const int k = (line / nt) % ne;
      const double cN = (kCo == 2) ? cst[nr - 1] : fma(grt[nr - 1], p4, cr[nr - 1]);
      const double cNm = (kCo == 2) ? cst[nr - 2] : fma(grt[nr - 2], p4, cr[nr - 2]);
      if (kCo == 1) { cst[nr - 1] = cN; cst[nr - 2] = cNm; }
      const bool inflow = is_neg(cN);
      // F(NR+1), F(NR+2): boundary ghosts on inflow lines.  On an outflow line
      // F(NR+1) is read only by face NR-1 when it is upwinded from the right,
      // and then it is the stale value of the most recent inflow line in the
      // reference's K->L->J loop order (F persists across lines in DRIFTR).
      double g1 = 0.0, g2 = 0.0;
      if (inflow) {  // line index = (L*NE+K)*NT+J, the layout of FGEOS(J,K,L)
        g1 = ghost_value(d, slot, j, k, l, d.conf1);
        g2 = ghost_value(d, slot, j, k, l, d.conf2);
      } else if (is_neg(cNm)) {
        g1 = stale_ghost(d, m, slot, j, k, l, p4);
      }
      double gm = fl[0], g0 = fl[1], gp = fl[2];
      double c = (kCo == 2) ? cst[0] : fma(grt[0], p4, cr[0]);
      if (kCo == 1) cst[0] = c;
      if (kCfl && outside[0] == 0) q = umax64(q, cfl_bits(c, kBits1em10));
      // face 1: FBND(1) = 0 (outflow) or F(2) (inflow)
      double phi_prev = c * ((inflow && !closed) ? g0 : 0.0);
      double xm = g0 - gm; bits64 bxm = babs_bits(beta, xm);
      double x = gp - g0; bits64 bx = babs_bits(beta, x);
      for (int f = 2; f <= nr - 1; ++f) {  // 1-based face f, updates cell f
        const double gpp = (f + 2 <= nr) ? fl[f + 1] : g1;
        const double xp = gpp - gp; const bits64 bxp = babs_bits(beta, xp);
        c = (kCo == 2) ? cst[f - 1] : ((f == nr - 1) ? cNm : fma(grt[f - 1], p4, cr[f - 1]));
        if (kCfl && outside[f - 1] == 0) q = umax64(q, cfl_bits(c, kBits1em10));
        const bool neg = is_neg(c);
        const double a = (kCo == 2) ? ast[f - 1] : corr_a_int(dbits(c) & kAbsMask, neg, c, -0.5);
        if (kCo == 1) { cst[f - 1] = c; ast[f - 1] = a; }
        int cs;
        const double fb = (kRec == 2)
            ? face_value_frozen(x, neg ? xp : xm, neg ? gp : g0, a, beta, cs = rget(rl + (f - 1), rsh) & 7)
            : face_value_case(x, bx, neg ? xp : xm, neg ? bxp : bxm, neg ? gp : g0, a, cs);
        const double phi = mul_rn_int(c, fb);
        const double raw = (g0 - phi) + phi_prev;
        fl[f - 1] = (kRec == 2) ? clip_frozen(raw, rget(rl + (f - 1), rsh)) : clip(raw);
        if (kRec == kRecCount) nclip += is_neg(raw);
        if (kRec == 1) rput(rl + (f - 1), rsh, cs | (is_neg(raw) ? kClipBit : 0));
        phi_prev = phi;
        gm = g0; g0 = gp; gp = gpp;
        xm = x; bxm = bx; x = xp; bx = bxp;
      }
      // face NR (g0 = F(NR), gp = F(NR+1), x = X(NR))
      if (kCfl && outside[nr - 1] == 0) q = umax64(q, cfl_bits(cN, kBits1em10));
      double fbn;
      int csn = 0;
      if (!inflow) {
        fbn = g0;
      } else {
        const double xp = g2 - g1; const bits64 bxp = babs_bits(beta, xp);
        const double an = corr_a_int(dbits(cN) & kAbsMask, true, cN, -0.5);
        fbn = (kRec == 2) ? face_value_frozen(x, xp, g1, an, beta, csn = rget(rl + (nr - 1), rsh) & 7)
                          : face_value_case(x, bx, xp, bxp, g1, an, csn);
      }
      if (closed) fbn = 0.0;
      const double phin = cN * fbn;
      const double rawn = (g0 - phin) + phi_prev;
      fl[nr - 1] = (kRec == 2) ? clip_frozen(rawn, rget(rl + (nr - 1), rsh)) : clip(rawn);
      if (kRec == kRecCount) nclip += is_neg(rawn);
      if (kRec == 1) rput(rl + (nr - 1), rsh, csn | (is_neg(rawn) ? kClipBit : 0));
    }
    if (kRec == kRecCount) warp_atomic_add(&d.clipq[slot], nclip);
    if (kCfl) warp_atomic_max(&d.cflq[slot * 4 + 0], q);
  }
}

// ----------------------------------------------------------------- DRIFTP
// Line (I,K,L), I = 2..NR, along J = 1..NT, periodic with J=1 == J=NT.
template <bool kCfl, int kRec, int kCo>
__global__ void __launch_bounds__(256) k_sweep_p(Dev d, double dts, unsigned char* __restrict__ rec, int rsh) {
  const int nr = d.nr, nt = d.nt, ne = d.ne;
  const int line0 = d.lw0 * (nr - 1) * ne;  // the L window, as in DRIFTR
  const int nlines = (nr - 1) * ne * (d.lw1 - d.lw0);
  // Work units are (item, block of lines).  A grid of (blocks per item,
  // items) gives one unit per CTA; a persistent grid loops over them.
  const int bpi = (nlines + blockDim.x - 1) / blockDim.x;
  const long long nunits = (long long)bpi * d.nitems;
  for (long long u = blockIdx.x + (long long)blockIdx.y * gridDim.x; u < nunits;
       u += (long long)gridDim.x * gridDim.y) {
    const int2 item = d.items[u / bpi];
    const int m = item.x, s = item.y, slot = m * d.ns + s;
    const int line = line0 + (int)(u % bpi) * blockDim.x + threadIdx.x;
    unsigned long long q = 0ULL;  // CFL quotient bits
    unsigned nclip = 0;  // clip events (kRec == kRecCount)
    // bounds-checked builds: the line's cells, its GPT and CA columns, the
    // coefficient store's item
    const bool lok = line >= line0 + nlines ||
        rg_ok(d, rg_item(d, item) &&
                     rg_span((long long)(line / (nr - 1)) * nt * nr + 1 + line % (nr - 1), nt, nr, d.ncell) &&
                     rg_span((long long)(line / (nr - 1) / ne) * nt * nr + 1 + line % (nr - 1), nt, nr,
                             (long long)nr * nt * d.npa) &&
                     rg_span((long long)item.x * nt * nr + 1 + line % (nr - 1), nt, nr, (long long)d.nm * nr * nt) &&
                     (!kCo || d.item0 + u / bpi < d.coef_items),
              kRgSweepP, line);
    if (line < line0 + nlines && lok) {
      const int i = 1 + line % (nr - 1);
      const int kl = line / (nr - 1);
      const int k = kl % ne, l = kl / ne;
      const long long st = nr;  // stride between consecutive J
      double* __restrict__ fl = d.f2 + (long long)slot * d.ncell + ((long long)kl * nt) * nr + i;
      unsigned char* __restrict__ rl =
          (kRec == 1 || kRec == 2) ? rec + (u / bpi) * d.ncell + ((long long)kl * nt) * nr + i : nullptr;
      double* __restrict__ cst = kCo ? coef_ptr(d, 1, 0, u / bpi) + ((long long)kl * nt) * nr + i : nullptr;
      double* __restrict__ ast = kCo ? coef_ptr(d, 1, 1, u / bpi) + ((long long)kl * nt) * nr + i : nullptr;
      const double* __restrict__ gpt = d.gpt + ((long long)l * nt) * nr + i;
      const double* __restrict__ ca = d.ca + ((long long)m * nt) * nr + i;
      const int* __restrict__ outside = d.outside + i;
      const double p2 = d.p2[((long long)s * ne + k) * nr + i];
      const BetaBits beta(d.betalim);
  #define GJ(J) fl[(long long)((J)-1) * st]
  #define CJ(J) fma(gpt[(long long)((J)-1) * nr], p2, ca[(long long)((J)-1) * nr])
      const double G1 = GJ(1), G2 = GJ(2), G3 = GJ(3), GNm = GJ(nt - 1), GN = GJ(nt);
      const double X1 = G2 - G1; const bits64 bX1 = babs_bits(beta, X1);
      const double X2 = G3 - G2; const bits64 bX2 = babs_bits(beta, X2);
      const double XNm = GN - GNm; const bits64 bXNm = babs_bits(beta, XNm);
      const double XN = G2 - GN; const bits64 bXN = babs_bits(beta, XN);
      // face NT first: its flux enters cell 2 through FBND(1)=FBND(NT)
      const double cN = (kCo == 2) ? cst[(long long)(nt - 1) * st] : CJ(nt);
      if (kCfl && outside[(long long)(nt - 1) * nr] == 0) q = umax64(q, cfl_bits(cN, kBits1em10));
      double phiN;
      int csN;
      {
        const bool neg = is_neg(cN);
        const double a = (kCo == 2) ? ast[(long long)(nt - 1) * st] : corr_a_int(dbits(cN) & kAbsMask, neg, cN, -0.5);
        if (kCo == 1) { cst[(long long)(nt - 1) * st] = cN; ast[(long long)(nt - 1) * st] = a; }
        phiN = cN * ((kRec == 2)
            ? face_value_frozen(XN, neg ? X2 : XNm, neg ? G2 : GN, a, beta, csN = rget(rl + (long long)(nt - 1) * st, rsh) & 7)
            : face_value_case(XN, bXN, neg ? X2 : XNm, neg ? bX2 : bXNm, neg ? G2 : GN, a, csN));
      }
      double phi_prev = phiN;
      double g0 = G2, gp = G3, xm = X1, x = X2;
      bits64 bxm = bX1, bx = bX2;
      // the cell two faces ahead is loaded one iteration early, before this
      // face's store: the compiler cannot move a load past a store to the
      // line at a run-time stride (DRIFTR's contiguous lines come from L1)
      double nxt = GJ(4);
      for (int J = 2; J <= nt - 1; ++J) {
        double gpp = 0.0, xp;
        bits64 bxp;
        const double nn = GJ(min(J + 3, nt));
        if (J <= nt - 3) {
          gpp = nxt;
          xp = gpp - gp;
          bxp = babs_bits(beta, xp);
        } else if (J == nt - 2) {
          gpp = GN;
          xp = XNm;
          bxp = bXNm;
        } else {  // J = NT-1: N = NT+1 wraps to 2, D = F(2)-F(1)
          xp = X1;
          bxp = bX1;
        }
        const double c = (kCo == 2) ? cst[(long long)(J - 1) * st] : CJ(J);
        if (kCfl && outside[(long long)(J - 1) * nr] == 0) q = umax64(q, cfl_bits(c, kBits1em10));
        const bool neg = is_neg(c);
        const double a = (kCo == 2) ? ast[(long long)(J - 1) * st] : corr_a_int(dbits(c) & kAbsMask, neg, c, -0.5);
        if (kCo == 1) { cst[(long long)(J - 1) * st] = c; ast[(long long)(J - 1) * st] = a; }
        int cs;
        const unsigned char* rj = (kRec == 1 || kRec == 2) ? rl + (long long)(J - 1) * st : nullptr;
        const double fb = (kRec == 2)
            ? face_value_frozen(x, neg ? xp : xm, neg ? gp : g0, a, beta, cs = rget(rj, rsh) & 7)
            : face_value_case(x, bx, neg ? xp : xm, neg ? bxp : bxm, neg ? gp : g0, a, cs);
        const double phi = mul_rn_int(c, fb);
        const double raw = (g0 - phi) + phi_prev;
        GJ(J) = (kRec == 2) ? clip_frozen(raw, rget(rj, rsh)) : clip(raw);
        if (kRec == kRecCount) nclip += is_neg(raw);
        if (kRec == 1) rput(rl + ((long long)(J - 1) * st), rsh, cs | (is_neg(raw) ? kClipBit : 0));
        phi_prev = phi;
        g0 = gp; gp = gpp;
        nxt = nn;
        xm = x; bxm = bx; x = xp; bx = bxp;
      }
      const double rawN = (GN - phiN) + phi_prev;
      const double vN = (kRec == 2) ? clip_frozen(rawN, rget(rl + (long long)(nt - 1) * st, rsh)) : clip(rawN);
      if (kRec == kRecCount) nclip += is_neg(rawN);
      GJ(nt) = vN;
      GJ(1) = vN;
      if (kRec == 1) rput(rl + ((long long)(nt - 1) * st), rsh, csN | (is_neg(rawN) ? kClipBit : 0));
  #undef GJ
  #undef CJ
    }
    if (kRec == kRecCount) warp_atomic_add(&d.clipq[slot], nclip);
    if (kCfl) warp_atomic_max(&d.cflq[slot * 4 + 1], q);
  }
}

// ----------------------------------------------------------------- DRIFTE
// Line (I,J,L), I = 2..NR, along K = 1..NE with extrapolated F(0), F(1)
// and F(NE+1) = F(NE+2) = 0.  Cell K = 1 is never written.
template <bool kCfl, int kRec, int kCo>
__global__ void __launch_bounds__(256) k_sweep_e(Dev d, double dts, unsigned char* __restrict__ rec, int rsh) {
  const int nr = d.nr, nt = d.nt, ne = d.ne;
  const int line0 = d.lw0 * (nr - 1) * nt;  // the L window, as in DRIFTR
  const int nlines = (nr - 1) * nt * (d.lw1 - d.lw0);
  // Work units are (item, block of lines).  A grid of (blocks per item,
  // items) gives one unit per CTA; a persistent grid loops over them.
  const int bpi = (nlines + blockDim.x - 1) / blockDim.x;
  const long long nunits = (long long)bpi * d.nitems;
  for (long long u = blockIdx.x + (long long)blockIdx.y * gridDim.x; u < nunits;
       u += (long long)gridDim.x * gridDim.y) {
    const int2 item = d.items[u / bpi];
    const int m = item.x, s = item.y, slot = m * d.ns + s;
    const int line = line0 + (int)(u % bpi) * blockDim.x + threadIdx.x;
    unsigned long long q = 0ULL;  // CFL quotient bits
    unsigned nclip = 0;  // clip events (kRec == kRecCount)
    // bounds-checked builds: the line's cells, its (I,J,L) table entry and
    // UE, its EDOT column, the coefficient store's item
    const bool lok = line >= line0 + nlines ||
        rg_ok(d, rg_item(d, item) &&
                     rg_span(((long long)(line / (nr - 1) / nt) * ne * nt + (line / (nr - 1)) % nt) * nr + 1 +
                                 line % (nr - 1), ne, (long long)nt * nr, d.ncell) &&
                     rg_span((long long)item.x * nr * nt * d.npa + (long long)(line / (nr - 1)) * nr + 1 +
                                 line % (nr - 1), 1, 1, (long long)d.nm * nr * nt * d.npa) &&
                     rg_span((long long)item.y * ne * nr + 1 + line % (nr - 1), ne, nr, (long long)d.ns * ne * nr) &&
                     (!kCo || d.item0 + u / bpi < d.coef_items),
              kRgSweepE, line);
    if (line < line0 + nlines && lok) {
      const int i = 1 + line % (nr - 1);
      const int jl = line / (nr - 1);
      const int j = jl % nt, l = jl / nt;
      const long long st = (long long)nt * nr;  // stride between consecutive K
      double* __restrict__ fl = d.f2 + (long long)slot * d.ncell + ((long long)l * ne * nt + j) * nr + i;
      unsigned char* __restrict__ rl =
          (kRec == 1 || kRec == 2) ? rec + (u / bpi) * d.ncell + ((long long)l * ne * nt + j) * nr + i : nullptr;
      double* __restrict__ cst =
          kCo ? coef_ptr(d, 2, 0, u / bpi) + ((long long)l * ne * nt + j) * nr + i : nullptr;
      double* __restrict__ ast =
          kCo ? coef_ptr(d, 2, 1, u / bpi) + ((long long)l * ne * nt + j) * nr + i : nullptr;
      const long long fij = ((long long)l * nt + j) * nr + i;
      const double wet = d.wet[fij];
      const double ue = d.ue[(long long)m * nr * nt * d.npa + fij];
      const double* __restrict__ edot = d.edot + (long long)s * ne * nr + i;
      const double* __restrict__ eb = d.eb + s * ne;
      const double* __restrict__ mhde = d.mhde;
      const double* __restrict__ iwe = d.iwe;
      const bool inside = d.outside[(long long)j * nr + i] == 0;
      const BetaBits beta(d.betalim);
      const bool closed = d.flags & 1u;
  #define GK(K) fl[(long long)((K)-1) * st]
  #define CK(K) (edot[(long long)((K)-1) * nr] * fma(eb[(K)-1], wet, ue))
      const double F2v = GK(2);
      const double G1 = d.kap[2 * s + 1] * F2v;
      const double G0 = d.kap[2 * s + 0] * G1;
      const double G2 = F2v, G3 = GK(3);
      const double X0 = G1 - G0; const bits64 bX0 = babs_bits(beta, X0);
      const double X1 = G2 - G1; const bits64 bX1 = babs_bits(beta, X1);
      const double X2 = G3 - G2; const bits64 bX2 = babs_bits(beta, X2);
      double phi_prev;
      {
        const double c = (kCo == 2) ? cst[0] : CK(1);
        if (kCfl && inside) q = umax64(q, mul_pos_bits(cfl_bits(c, kBits1em10), d.ide[0]));
        const bool neg = is_neg(c);
        const double a = (kCo == 2) ? ast[0] : fma(c, mhde[0], neg ? -0.5 : 0.5);
        if (kCo == 1) { cst[0] = c; ast[0] = a; }
        int cs;
        double fb = (kRec == 2) ? face_value_frozen(X1, neg ? X2 : X0, neg ? G2 : G1, a, beta, cs = rget(rl, rsh) & 7)
                                : face_value_case(X1, bX1, neg ? X2 : X0, neg ? bX2 : bX0, neg ? G2 : G1, a, cs);
        if (closed) fb = 0.0;
        if (kRec == 1) rput(rl, rsh, cs);
        phi_prev = c * fb;
      }
      double g0 = G2, gp = G3, xm = X1, x = X2;
      bits64 bxm = bX1, bx = bX2;
      double nxt = GK(4);  // loaded one iteration ahead, as in DRIFTP
      for (int K = 2; K <= ne; ++K) {
        const double gpp = (K + 2 <= ne) ? nxt : 0.0;
        nxt = GK(min(K + 3, ne));
        const double xp = gpp - gp; const bits64 bxp = babs_bits(beta, xp);
        const double c = (kCo == 2) ? cst[(long long)(K - 1) * st] : CK(K);
        if (kCfl && inside) q = umax64(q, mul_pos_bits(cfl_bits(c, kBits1em10), d.ide[K - 1]));
        const bool neg = is_neg(c);
        const double a = (kCo == 2) ? ast[(long long)(K - 1) * st] : fma(c, mhde[K - 1], neg ? -0.5 : 0.5);
        if (kCo == 1) { cst[(long long)(K - 1) * st] = c; ast[(long long)(K - 1) * st] = a; }
        int cs;
        const unsigned char* rk = (kRec == 1 || kRec == 2) ? rl + (long long)(K - 1) * st : nullptr;
        double fb = (kRec == 2) ? face_value_frozen(x, neg ? xp : xm, neg ? gp : g0, a, beta, cs = rget(rk, rsh) & 7)
                                : face_value_case(x, bx, neg ? xp : xm, neg ? bxp : bxm, neg ? gp : g0, a, cs);
        if (closed && K == ne) fb = 0.0;
        // loaded coefficients leave this sweep few FP64 operations to hide its
        // loads behind: the FP64 multiply (uncontracted, bit-equal to mul_rn_int)
        const double phi = (kCo == 2) ? __dmul_rn(c, fb) : mul_rn_int(c, fb);
        const double raw = fma(phi_prev - phi, iwe[K - 1], g0);
        GK(K) = (kRec == 2) ? clip_frozen(raw, rget(rk, rsh)) : clip(raw);
        if (kRec == kRecCount) nclip += is_neg(raw);
        if (kRec == 1) rput(rl + ((long long)(K - 1) * st), rsh, cs | (is_neg(raw) ? kClipBit : 0));
        phi_prev = phi;
        g0 = gp; gp = gpp;
        xm = x; bxm = bx; x = xp; bx = bxp;
      }
  #undef GK
  #undef CK
    }
    if (kRec == kRecCount) warp_atomic_add(&d.clipq[slot], nclip);
    if (kCfl) warp_atomic_max(&d.cflq[slot * 4 + 2], q);
  }
}

// ---------------------------------------------------------------- DRIFTMU
// Line (I,J,K), I = 2..NR, along L = 1..NPA with F(1) = F(2); limiter on
// faces 2..NPA-2, FBND(NPA-1) = F(NPA), then the F2(NPA) extrapolation.
// kLoss: 0 none, 1 multiply the result by table lossA (loss after the sweep),
//        2 multiply the input by lossA (loss before the sweep).
// kSplit 2 or 4: there are few pitch-angle lines (NR-1)*NT*NE, so kSplit
// adjacent lanes share one, lane q updating cells b+1..lim of segment q
// (b = q*S, lim = (q+1)*S with S = NPA/kSplit; lane 0 from cell 2, the last
// lane to NPA).  All run the same instructions: a "pre-face" (face 1,
// whose flux is zero, for lane 0; face b, recomputed bit for bit from the
// old values, for the others), then their faces.  Every old value a lane
// needs from its neighbours' cells (its entering window and the two cells
// past lim) is loaded before a __syncwarp, and no lane writes before it.
// Segments keep at least 4 cells (2 lanes: NPA >= 12; 4 lanes: NPA >= 24),
// so no lane but lane 0 sees the F(1) = F(2) rule.
template <bool kCfl, int kLoss, int kRec, int kCo, int kSplit>
__global__ void __launch_bounds__(256) k_sweep_mu(Dev d, double dts, const double* __restrict__ lossA,
                                                   unsigned char* __restrict__ rec, int rsh) {
  const int nr = d.nr, nt = d.nt, ne = d.ne, npa = d.npa;
  const int nlines = (nr - 1) * nt * ne;
  // Work units are (item, block of lines).  A grid of (blocks per item,
  // items) gives one unit per CTA; a persistent grid loops over them.
  const int lpb = blockDim.x / kSplit;  // lines per CTA
  const int bpi = (nlines + lpb - 1) / lpb;
  const long long nunits = (long long)bpi * d.nitems;
  // lane pairs: the even lane ends at Lm, the odd one takes the rest
  const int half = kSplit == 2 ? (int)(threadIdx.x & 1) : 0;
  const int Lm = kSplit == 2 ? npa / 2 : npa;  // last cell of the even lane
  // four lanes: segment q4 of seg4 cells (the last one to NPA)
  const int q4 = kSplit == 4 ? (int)(threadIdx.x & 3) : 0;
  const int seg4 = npa / 4;
  const int pre = kSplit == 4 ? q4 : half;  // nonzero: the pre-face is recomputed
  const bool last = kSplit == 4 ? q4 == 3 : (half || kSplit == 1);
  for (long long u = blockIdx.x + (long long)blockIdx.y * gridDim.x; u < nunits;
       u += (long long)gridDim.x * gridDim.y) {
    const int2 item = d.items[u / bpi];
    const int m = item.x, s = item.y, slot = m * d.ns + s;
    const int line = (int)(u % bpi) * lpb + (int)threadIdx.x / kSplit;
    // bounds-checked builds: the line's cells, its WM and UM columns, the
    // coefficient store's item (the lanes sharing a line test the same)
    const bool active = line < nlines &&
        rg_ok(d, rg_item(d, item) &&
                     rg_span((long long)(line / (nr - 1)) * nr + 1 + line % (nr - 1), npa, (long long)ne * nt * nr,
                             d.ncell) &&
                     rg_span((long long)((line / (nr - 1)) % nt) * nr + 1 + line % (nr - 1), npa, (long long)nt * nr,
                             (long long)nr * nt * npa) &&
                     rg_span((long long)item.x * nt * nr * npa + ((line / (nr - 1)) % nt) * nr + 1 + line % (nr - 1),
                             npa, (long long)nt * nr, (long long)d.nm * nr * nt * npa) &&
                     (!kCo || d.item0 + u / bpi < d.coef_items),
              kRgSweepMu, line);
    unsigned long long q = 0ULL;  // CFL quotient bits
    unsigned nclip = 0;  // clip events (kRec == kRecCount)
    const int lc = active ? line : 0;
    const int i = 1 + lc % (nr - 1);
    const int jk = lc / (nr - 1);
    const int j = jk % nt;
    const long long st = (long long)ne * nt * nr;  // stride between consecutive L
    const long long off = (long long)jk * nr + i;  // (K*NT + J)*NR + I
    double* __restrict__ fl = d.f2 + (long long)slot * d.ncell + off;
    unsigned char* __restrict__ rl = (kRec == 1 || kRec == 2) ? rec + (u / bpi) * d.ncell + off : nullptr;
    double* __restrict__ cst = kCo ? coef_ptr(d, 3, 0, u / bpi) + off : nullptr;
    double* __restrict__ ast = kCo ? coef_ptr(d, 3, 1, u / bpi) + off : nullptr;
    const double* __restrict__ la = lossA ? lossA + (long long)s * d.ncell + off : nullptr;
    const long long sij = (long long)nt * nr;     // stride of (I,J,L) tables in L
    const long long fij = (long long)j * nr + i;
    const double* __restrict__ wm = d.wm + fij;
    const double* __restrict__ um = d.um + (long long)m * nt * nr * npa + fij;
    const double ekv = d.ek[s * ne + jk / nt];
    const double* __restrict__ mhdmu = d.mhdmu;
    const double* __restrict__ iwmu = d.iwmu;
    const bool inside = d.outside[fij] == 0;
    const BetaBits beta(d.betalim);
    const bool closed = d.flags & 1u;
  #define GL(L) fl[(long long)((L)-1) * st]
  #define LA(L) la[(long long)((L)-1) * st]
  #define GLS(L) (kLoss == 2 ? GL(L) * LA(L) : GL(L))
  #define CL(L) fma(ekv, wm[(long long)((L)-1) * sij], um[(long long)((L)-1) * sij])
    // pre-face b (1, Lm or q4*seg4) and its window G(b-1..b+2); the first
    // lane's F(1) is F(2); lim: last cell of this lane's range (its
    // look-ahead beyond lim comes from the halo hA = G(lim+1), hB = G(lim+2))
    const int b = kSplit == 4 ? (q4 ? q4 * seg4 : 1) : (half ? Lm : 1);
    const int lim = kSplit == 4 ? (q4 == 3 ? npa : (q4 + 1) * seg4) : (half ? npa : Lm);
    double w0 = 0.0, w1 = 0.0, w2 = 0.0, w3 = 0.0, nxt = 0.0, hA = 0.0, hB = 0.0;
    if (active) {
      w0 = GLS(pre ? b - 1 : 2);
      w1 = GLS(pre ? b : 2);
      w2 = GLS(b + 1 > 2 ? b + 1 : 2);
      w3 = GLS(b + 2);
      nxt = GL(b + 3);
      if (kSplit > 1) {
        hA = GLS(min(lim + 1, npa));
        hB = GLS(min(lim + 2, npa));
      }
    }
    if (kSplit > 1) __syncwarp();
    if (active) {
      // pre-face: the flux entering this lane's first cell
      double phi_prev;
      {
        const double c = pre ? ((kCo == 2) ? cst[(long long)(b - 1) * st] : CL(b)) : 0.0;
        const bool neg = is_neg(c);
        const double a = (kCo == 2 && pre) ? ast[(long long)(b - 1) * st] : fma(c, mhdmu[b - 1], neg ? -0.5 : 0.5);
        const double xm = w1 - w0, x = w2 - w1, xp = w3 - w2;
        int cs;
        const double fb = (kRec == 2)
            ? face_value_frozen(x, neg ? xp : xm, neg ? w2 : w1, a, beta, cs = rget(rl + (long long)(b - 1) * st, rsh) & 7)
            : face_value_case(x, babs_bits(beta, x), neg ? xp : xm, babs_bits(beta, neg ? xp : xm),
                              neg ? w2 : w1, a, cs);
        phi_prev = c * fb;
      }
      double g0 = w2, gp = w3;
      double xm = w2 - w1;
      bits64 bxm = babs_bits(beta, xm);
      double x = w3 - w2;
      bits64 bx = babs_bits(beta, x);
      const int Lend = last ? npa - 2 : (kSplit == 4 ? lim : Lm);
      for (int L = b + 1; L <= Lend; ++L) {
        double gpp;
        if (kSplit > 1) {
          gpp = (L + 2 <= lim) ? nxt : (L + 2 == lim + 1 ? hA : hB);
          if (kLoss == 2 && L + 2 <= lim) gpp *= LA(L + 2);
          nxt = GL(min(L + 3, lim));
        } else {
          gpp = nxt;
          nxt = GL(min(L + 3, npa));
          if (kLoss == 2) gpp *= LA(L + 2);
        }
        const double xp = gpp - gp; const bits64 bxp = babs_bits(beta, xp);
        const double c = (kCo == 2) ? cst[(long long)(L - 1) * st] : CL(L);
        if (kCfl && inside) q = umax64(q, mul_pos_bits(cfl_bits(c, kBits1em32), d.idmu[L - 1]));
        const bool neg = is_neg(c);
        const double a = (kCo == 2) ? ast[(long long)(L - 1) * st] : fma(c, mhdmu[L - 1], neg ? -0.5 : 0.5);
        if (kCo == 1) { cst[(long long)(L - 1) * st] = c; ast[(long long)(L - 1) * st] = a; }
        int cs;
        const unsigned char* rq = (kRec == 1 || kRec == 2) ? rl + (long long)(L - 1) * st : nullptr;
        const double fb = (kRec == 2) ? face_value_frozen(x, neg ? xp : xm, neg ? gp : g0, a, beta, cs = rget(rq, rsh) & 7)
                                      : face_value_case(x, bx, neg ? xp : xm, neg ? bxp : bxm, neg ? gp : g0, a, cs);
        const double phi = mul_rn_int(c, fb);
        const double raw = fma(phi_prev - phi, iwmu[L - 1], g0);
        if (kRec == 1) rput(rl + ((long long)(L - 1) * st), rsh, cs | (is_neg(raw) ? kClipBit : 0));
        double v = (kRec == 2) ? clip_frozen(raw, rget(rq, rsh)) : clip(raw);
        if (kRec == kRecCount) nclip += is_neg(raw);
        if (kLoss == 1) v *= LA(L);
        GL(L) = v;
        phi_prev = phi;
        g0 = gp; gp = gpp;
        xm = x; bxm = bx; x = xp; bx = bxp;
      }
      // face NPA-1: FBND = F(NPA); cell NPA-1; then the F2(NPA) ghost
      if (last) {
        const int L = npa - 1;
        const double c = (kCo == 2) ? cst[(long long)(L - 1) * st] : CL(L);
        if (kCo == 1) cst[(long long)(L - 1) * st] = c;
        if (kCfl && inside) q = umax64(q, mul_pos_bits(cfl_bits(c, kBits1em32), d.idmu[L - 1]));
        const double phi = c * (closed ? 0.0 : gp);
        const double raw = fma(phi_prev - phi, iwmu[L - 1], g0);
        if (kRec == 1) rput(rl + ((long long)(L - 1) * st), rsh, is_neg(raw) ? kClipBit : 0);
        const double v = (kRec == 2) ? clip_frozen(raw, rget(rl + (long long)(L - 1) * st, rsh)) : clip(raw);
        if (kRec == kRecCount) nclip += is_neg(raw);
        const double vN = v * d.rho[fij];
        if (kLoss == 1) {
          GL(L) = v * LA(L);
          GL(npa) = vN * LA(npa);
        } else {
          GL(L) = v;
          GL(npa) = vN;
        }
      }
    }
  #undef GL
  #undef LA
  #undef GLS
  #undef CL
    if (kRec == kRecCount) warp_atomic_add(&d.clipq[slot], nclip);
    if (kCfl) warp_atomic_max(&d.cflq[slot * 4 + 3], q);
  }
}

// ---------------------------------------------------------------- launchers
// Grid: (blocks per item, items), or a persistent grid of d.pers[w] CTAs.
static inline dim3 grid_for(const Dev& d, int w, int nlines) {
  const int blk = d.blk[w];
  if (d.pers[w] > 0) return dim3(d.pers[w], 1, 1);
  return dim3((nlines + blk - 1) / blk, d.nitems, 1);
}
// Lines of sweep w: R, P and E within the L window [lw0, lw1); every
// pitch-angle line spans all L, so DRIFTMU always takes them all.
static inline int nlines_of(const Dev& d, int w) {
  switch (w) {
    case 0: return d.nt * d.ne * (d.lw1 - d.lw0);
    case 1: return (d.nr - 1) * d.ne * (d.lw1 - d.lw0);
    case 2: return (d.nr - 1) * d.nt * (d.lw1 - d.lw0);
    default: return (d.nr - 1) * d.nt * d.ne;
  }
}

// co: 0 compute the face coefficients, 1 compute and store them, 2 load
// the stored ones (needs d.coef; the plain, store and load forms give
// identical results).
void launch_sweep_r(const Dev& d, double dts, bool cfl, cudaStream_t st, unsigned char* rec, bool replay, int co,
                    int rsh) {
  dim3 g = grid_for(d, 0, nlines_of(d, 0));
  const int b = d.blk[0];
  const bool n = d.count_clips;
  if (rec && replay) k_sweep_r<false, 2, 0><<<g, b, 0, st>>>(d, dts, rec, rsh);
  else if (rec) k_sweep_r<false, 1, 0><<<g, b, 0, st>>>(d, dts, rec, rsh);
  else if (co == 1) (n ? k_sweep_r<true, 3, 1> : k_sweep_r<true, 0, 1>)<<<g, b, 0, st>>>(d, dts, nullptr, 0);
  else if (co == 2) (n ? k_sweep_r<false, 3, 2> : k_sweep_r<false, 0, 2>)<<<g, b, 0, st>>>(d, dts, nullptr, 0);
  else if (cfl) (n ? k_sweep_r<true, 3, 0> : k_sweep_r<true, 0, 0>)<<<g, b, 0, st>>>(d, dts, nullptr, 0);
  else (n ? k_sweep_r<false, 3, 0> : k_sweep_r<false, 0, 0>)<<<g, b, 0, st>>>(d, dts, nullptr, 0);
}
void launch_sweep_p(const Dev& d, double dts, bool cfl, cudaStream_t st, unsigned char* rec, bool replay, int co,
                    int rsh) {
  dim3 g = grid_for(d, 1, nlines_of(d, 1));
  const int b = d.blk[1];
  const bool n = d.count_clips;
  if (rec && replay) k_sweep_p<false, 2, 0><<<g, b, 0, st>>>(d, dts, rec, rsh);
  else if (rec) k_sweep_p<false, 1, 0><<<g, b, 0, st>>>(d, dts, rec, rsh);
  else if (co == 1) (n ? k_sweep_p<true, 3, 1> : k_sweep_p<true, 0, 1>)<<<g, b, 0, st>>>(d, dts, nullptr, 0);
  else if (co == 2) (n ? k_sweep_p<false, 3, 2> : k_sweep_p<false, 0, 2>)<<<g, b, 0, st>>>(d, dts, nullptr, 0);
  else if (cfl) (n ? k_sweep_p<true, 3, 0> : k_sweep_p<true, 0, 0>)<<<g, b, 0, st>>>(d, dts, nullptr, 0);
  else (n ? k_sweep_p<false, 3, 0> : k_sweep_p<false, 0, 0>)<<<g, b, 0, st>>>(d, dts, nullptr, 0);
}
void launch_sweep_e(const Dev& d, double dts, bool cfl, cudaStream_t st, unsigned char* rec, bool replay, int co,
                    int rsh) {
  dim3 g = grid_for(d, 2, nlines_of(d, 2));
  const int b = d.blk[2];
  const bool n = d.count_clips;
  if (rec && replay) k_sweep_e<false, 2, 0><<<g, b, 0, st>>>(d, dts, rec, rsh);
  else if (rec && co == 1) k_sweep_e<false, 1, 1><<<g, b, 0, st>>>(d, dts, rec, rsh);
  else if (rec && co == 2) k_sweep_e<false, 1, 2><<<g, b, 0, st>>>(d, dts, rec, rsh);
  else if (rec) k_sweep_e<false, 1, 0><<<g, b, 0, st>>>(d, dts, rec, rsh);
  else if (co == 1) (n ? k_sweep_e<true, 3, 1> : k_sweep_e<true, 0, 1>)<<<g, b, 0, st>>>(d, dts, nullptr, 0);
  else if (co == 2) (n ? k_sweep_e<false, 3, 2> : k_sweep_e<false, 0, 2>)<<<g, b, 0, st>>>(d, dts, nullptr, 0);
  else if (cfl) (n ? k_sweep_e<true, 3, 0> : k_sweep_e<true, 0, 0>)<<<g, b, 0, st>>>(d, dts, nullptr, 0);
  else (n ? k_sweep_e<false, 3, 0> : k_sweep_e<false, 0, 0>)<<<g, b, 0, st>>>(d, dts, nullptr, 0);
}
// The clip-counting forms of the plain (unrecorded) pitch-angle sweeps.
template <int kLoss, int kS>
static void mu_count(const Dev& d, dim3 g, int b, double dts, const double* loss, cudaStream_t st, bool cfl,
                     int co) {
  if (co == 1) k_sweep_mu<true, kLoss, 3, 1, kS><<<g, b, 0, st>>>(d, dts, loss, nullptr, 0);
  else if (co == 2) k_sweep_mu<false, kLoss, 3, 2, kS><<<g, b, 0, st>>>(d, dts, loss, nullptr, 0);
  else if (cfl) k_sweep_mu<true, kLoss, 3, 0, kS><<<g, b, 0, st>>>(d, dts, loss, nullptr, 0);
  else k_sweep_mu<false, kLoss, 3, 0, kS><<<g, b, 0, st>>>(d, dts, loss, nullptr, 0);
}

template <int kLoss, int kS>
static void mu_launch(const Dev& d, dim3 g, int b, double dts, const double* loss, cudaStream_t st,
                      unsigned char* rec, bool replay, bool cfl, int co, int rsh) {
  const bool n = d.count_clips;
  if (rec && replay) k_sweep_mu<false, kLoss, 2, 0, kS><<<g, b, 0, st>>>(d, dts, loss, rec, rsh);
  else if (rec) k_sweep_mu<false, kLoss, 1, 0, kS><<<g, b, 0, st>>>(d, dts, loss, rec, rsh);
  else if (n) mu_count<kLoss, kS>(d, g, b, dts, loss, st, cfl, co);
  else if (co == 1) k_sweep_mu<true, kLoss, 0, 1, kS><<<g, b, 0, st>>>(d, dts, loss, nullptr, 0);
  else if (co == 2) k_sweep_mu<false, kLoss, 0, 2, kS><<<g, b, 0, st>>>(d, dts, loss, nullptr, 0);
  else if (cfl) k_sweep_mu<true, kLoss, 0, 0, kS><<<g, b, 0, st>>>(d, dts, loss, nullptr, 0);
  else k_sweep_mu<false, kLoss, 0, 0, kS><<<g, b, 0, st>>>(d, dts, loss, nullptr, 0);
}
// Lines are split between d.mu_lanes adjacent lanes (2 for NPA >= 12, 4
// for NPA >= 24: every segment keeps at least four cells, so no lane but
// the first reads the F(1) rule).
void launch_sweep_mu(const Dev& d, double dts, bool cfl, int loss_mode, const double* loss,
                     cudaStream_t st, unsigned char* rec, bool replay, int co, int rsh) {
  const int lanes = (d.mu_lanes == 4 && d.npa >= 24) ? 4 : ((d.mu_lanes >= 2 && d.npa >= 12) ? 2 : 1);
  dim3 g = grid_for(d, 3, lanes * nlines_of(d, 3));
  const int b = d.blk[3];
  if (lanes == 4) {
    if (loss_mode == 1) mu_launch<1, 4>(d, g, b, dts, loss, st, rec, replay, cfl, co, rsh);
    else if (loss_mode == 2) mu_launch<2, 4>(d, g, b, dts, loss, st, rec, replay, cfl, co, rsh);
    else mu_launch<0, 4>(d, g, b, dts, nullptr, st, rec, replay, cfl, co, rsh);
  } else if (lanes == 2) {
    if (loss_mode == 1) mu_launch<1, 2>(d, g, b, dts, loss, st, rec, replay, cfl, co, rsh);
    else if (loss_mode == 2) mu_launch<2, 2>(d, g, b, dts, loss, st, rec, replay, cfl, co, rsh);
    else mu_launch<0, 2>(d, g, b, dts, nullptr, st, rec, replay, cfl, co, rsh);
  } else {
    if (loss_mode == 1) mu_launch<1, 1>(d, g, b, dts, loss, st, rec, replay, cfl, co, rsh);
    else if (loss_mode == 2) mu_launch<2, 1>(d, g, b, dts, loss, st, rec, replay, cfl, co, rsh);
    else mu_launch<0, 1>(d, g, b, dts, nullptr, st, rec, replay, cfl, co, rsh);
  }
}

// Resident CTAs per SM of sweep w at block size blk (for persistent grids).
int sweep_max_blocks_per_sm(int w, int blk) {
  int n = 0;
  cudaError_t e = cudaSuccess;
  switch (w) {
    case 0: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_r<false, 0, 0>, blk, 0); break;
    case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_p<false, 0, 0>, blk, 0); break;
    case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_e<false, 0, 0>, blk, 0); break;
    default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_sweep_mu<false, 0, 0, 0, 2>, blk, 0); break;
  }
  return e == cudaSuccess ? n : 0;
}

}  // namespace ramgpu
