// adjoint.cu -- frozen-limiter adjoint of the RAM kinetic step.
//
// With the limiter branch of every face and the clip state of every cell
// frozen (recorded by the forward sweeps, one byte per face: 0 upwind only,
// 1 beta*D, 2 X, 3 D, 4 beta*X, plus kClipBit), each sweep of
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

#include "kernels.cuh"

namespace ramgpu {

constexpr int kMaxLine = 160;  // longest line of the adjoint (NR, NT, NE, NPA <= 160)

// Scatter of one face: FBb = dJ/dFBND(f).  up is the upwind cell, cs the
// recorded case, a the CORR factor, (f, f+1) the face's cells and
// (dm, dp) the cells of D = G(dp) - G(dm).
__device__ __forceinline__ void scatter_face(double* Gb, double FBb, int up, int cs, double a,
                                             double beta, int f, int f1, int dm, int dp) {
  Gb[up] += FBb;
  if (cs) {
    const double Lb = a * FBb;
    const double Vb = (cs == 1 || cs == 4) ? beta * Lb : Lb;
    if (cs == 2 || cs == 4) {  // V = X = G(f1) - G(f)
      Gb[f1] += Vb;
      Gb[f] -= Vb;
    } else {                   // V = D
      Gb[dp] += Vb;
      Gb[dm] -= Vb;
    }
  }
}

#define WORK_LOOP(NLINES)                                                          \
  const int bpi = (NLINES + blockDim.x - 1) / blockDim.x;                          \
  const long long nunits = (long long)bpi * d.nitems;                              \
  for (long long u = blockIdx.x + (long long)blockIdx.y * gridDim.x; u < nunits;   \
       u += (long long)gridDim.x * gridDim.y)

// ------------------------------------------------------------------ DRIFTR^T
__global__ void __launch_bounds__(64) k_adj_r(Dev d, const unsigned char* __restrict__ rec) {
  const int nr = d.nr, nt = d.nt, ne = d.ne;
  const int nlines = nt * ne * d.npa;
  WORK_LOOP(nlines) {
    const int2 item = d.items[u / bpi];
    const int m = item.x, s = item.y, slot = m * d.ns + s;
    const int line = (int)(u % bpi) * blockDim.x + threadIdx.x;
    if (line >= nlines) continue;
    const int j = line % nt, k = (line / nt) % ne, l = line / (nt * ne);
    double* lam = d.lam + (long long)slot * d.ncell + (long long)line * nr;
    const unsigned char* rl = rec + (u / bpi) * d.ncell + (long long)line * nr;
    const double* grt = d.grt + ((long long)l * nt + j) * nr;
    const double* cr = d.cr + ((long long)m * nt + j) * nr;
    const double p4 = d.p4[s * ne + k];
    const double beta = d.betalim;
    const bool closed = d.flags & 1u;
    const int n = nr;
    double C[kMaxLine + 1], Gb[kMaxLine + 3], Pb[kMaxLine + 1];
    for (int i = 1; i <= n; ++i) {
      C[i] = fma(grt[i - 1], p4, cr[i - 1]);
      Gb[i] = 0.0;
      Pb[i] = 0.0;
    }
    Gb[0] = Gb[n + 1] = Gb[n + 2] = 0.0;
    const bool inflow = is_neg(C[n]);
    Gb[1] = lam[0];  // cell 1 is not updated
    for (int i = 2; i <= n; ++i) {
      const double le = (rl[i - 1] & kClipBit) ? 0.0 : lam[i - 1];
      Gb[i] += le;
      Pb[i] -= le;
      Pb[i - 1] += le;
    }
    if (inflow && !closed) Gb[2] += C[1] * Pb[1];  // FBND(1) = F(2)
    const int UR = inflow ? n : n - 1;
    for (int f = 2; f <= UR; ++f) {
      if (closed && f == n) continue;
      const double FBb = C[f] * Pb[f];
      const bool neg = is_neg(C[f]);
      const double a = fma(C[f], -0.5, neg ? -0.5 : 0.5);
      scatter_face(Gb, FBb, neg ? f + 1 : f, rl[f - 1] & 7, a, beta, f, f + 1, neg ? f + 1 : f - 1,
                   neg ? f + 2 : f);
    }
    if (!inflow && !closed) Gb[n] += C[n] * Pb[n];  // FBND(NR) = F(NR)
    // ghost cells -> dJ/dFGEOS
    const long long nfg = (long long)nt * ne * d.npa;
    if (inflow) {
      if (d.outside[(long long)j * nr + n - 1] != 1) {
        const double fh = d.fnhs[((long long)l * nt + j) * d.nf + n - 1];
        atomicAdd(&d.gfg[slot * nfg + line], d.conf1 * fh * Gb[n + 1] + d.conf2 * fh * Gb[n + 2]);
      }
    } else if (Gb[n + 1] != 0.0) {
      const int src = stale_ghost_src(d, m, slot, j, k, l, p4);
      if (src >= 0) {
        const int jj = src % nt, ll = src / (nt * ne);
        if (d.outside[(long long)jj * nr + n - 1] != 1) {
          const double fh = d.fnhs[((long long)ll * nt + jj) * d.nf + n - 1];
          atomicAdd(&d.gfg[slot * nfg + src], d.conf1 * fh * Gb[n + 1]);
        }
      }
    }
    for (int i = 1; i <= n; ++i) lam[i - 1] = Gb[i];
  }
}

// ------------------------------------------------------------------ DRIFTP^T
__global__ void __launch_bounds__(64) k_adj_p(Dev d, const unsigned char* __restrict__ rec) {
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
    const long long base = ((long long)kl * nt) * nr + i;
    double* lam = d.lam + (long long)slot * d.ncell + base;
    const unsigned char* rl = rec + (u / bpi) * d.ncell + base;
    const double* gpt = d.gpt + ((long long)l * nt) * nr + i;
    const double* ca = d.ca + ((long long)m * nt) * nr + i;
    const double p2 = d.p2[((long long)s * ne + k) * nr + i];
    const double beta = d.betalim;
    const int n = nt;
    double C[kMaxLine + 1], Gb[kMaxLine + 3], Pb[kMaxLine + 1], lv[kMaxLine + 1];
    for (int J = 1; J <= n; ++J) {
      C[J] = (J >= 2) ? fma(gpt[(long long)(J - 1) * nr], p2, ca[(long long)(J - 1) * nr]) : 0.0;
      lv[J] = lam[(long long)(J - 1) * nr];
      Gb[J] = 0.0;
      Pb[J] = 0.0;
    }
    lv[n] += lv[1];  // F2(1) = F2new(NT)
    lv[1] = 0.0;
    for (int J = 2; J <= n; ++J) {
      const double le = (rl[(long long)(J - 1) * nr] & kClipBit) ? 0.0 : lv[J];
      Gb[J] += le;
      Pb[J] -= le;
      Pb[J - 1] += le;
    }
    Pb[n] += Pb[1];  // FBND(1) = FBND(NT), CDriftP(1) = CDriftP(NT)
    for (int J = 2; J <= n; ++J) {
      const double FBb = C[J] * Pb[J];
      const bool neg = is_neg(C[J]);
      const double a = fma(C[J], -0.5, neg ? -0.5 : 0.5);
      const int J1 = (J == n) ? 2 : J + 1;
      int dm, dp;
      if (!neg) { dm = J - 1; dp = J; }
      else if (J <= n - 2) { dm = J + 1; dp = J + 2; }
      else if (J == n - 1) { dm = 1; dp = 2; }
      else { dm = 2; dp = 3; }
      scatter_face(Gb, FBb, neg ? J1 : J, rl[(long long)(J - 1) * nr] & 7, a, beta, J, J1, dm, dp);
    }
    for (int J = 1; J <= n; ++J) lam[(long long)(J - 1) * nr] = Gb[J];
  }
}

// ------------------------------------------------------------------ DRIFTE^T
__global__ void __launch_bounds__(64) k_adj_e(Dev d, const unsigned char* __restrict__ rec) {
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
    double* lam = d.lam + (long long)slot * d.ncell + base;
    const unsigned char* rl = rec + (u / bpi) * d.ncell + base;
    const long long fij = ((long long)l * nt + j) * nr + i;
    const double wet = d.wet[fij];
    const double ue = d.ue[(long long)m * nr * nt * d.npa + fij];
    const double* edot = d.edot + (long long)s * ne * nr + i;
    const double* eb = d.eb + s * ne;
    const double beta = d.betalim;
    const bool closed = d.flags & 1u;
    const int n = ne;
    double C[kMaxLine + 1], Gb[kMaxLine + 3], Pb[kMaxLine + 1];
    for (int K = 1; K <= n; ++K) {
      C[K] = edot[(long long)(K - 1) * nr] * fma(eb[K - 1], wet, ue);
      Gb[K] = 0.0;
      Pb[K] = 0.0;
    }
    Gb[0] = Gb[n + 1] = Gb[n + 2] = 0.0;
    const double out1 = lam[0];  // cell K = 1 is not updated
    for (int K = 2; K <= n; ++K) {
      const double le = (rl[(long long)(K - 1) * st] & kClipBit) ? 0.0 : lam[(long long)(K - 1) * st];
      const double w = d.iwe[K - 1];
      Gb[K] += le;
      Pb[K] -= w * le;
      Pb[K - 1] += w * le;
    }
    for (int K = 1; K <= n; ++K) {
      if (closed && (K == 1 || K == n)) continue;
      const double FBb = C[K] * Pb[K];
      const bool neg = is_neg(C[K]);
      const double a = fma(C[K], d.mhde[K - 1], neg ? -0.5 : 0.5);
      scatter_face(Gb, FBb, neg ? K + 1 : K, rl[(long long)(K - 1) * st] & 7, a, beta, K, K + 1,
                   neg ? K + 1 : K - 1, neg ? K + 2 : K);
    }
    // G(1) = kap1 F(2), G(0) = kap0 G(1); G(NE+1) = G(NE+2) = 0
    const double g1 = Gb[1] + d.kap[2 * s + 0] * Gb[0];
    lam[0] = out1;
    lam[st] = Gb[2] + d.kap[2 * s + 1] * g1;
    for (int K = 3; K <= n; ++K) lam[(long long)(K - 1) * st] = Gb[K];
  }
}

// ----------------------------------------------------------------- DRIFTMU^T
__global__ void __launch_bounds__(64) k_adj_mu(Dev d, const unsigned char* __restrict__ rec) {
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
    double* lam = d.lam + (long long)slot * d.ncell + off;
    const unsigned char* rl = rec + (u / bpi) * d.ncell + off;
    const long long sij = (long long)nt * nr;
    const long long fij = (long long)j * nr + i;
    const double* wm = d.wm + fij;
    const double* um = d.um + (long long)m * nt * nr * npa + fij;
    const double ekv = d.ek[s * ne + jk / nt];
    const double beta = d.betalim;
    const bool closed = d.flags & 1u;
    const int n = npa;
    double C[kMaxLine + 1], Gb[kMaxLine + 3], Pb[kMaxLine + 1], lv[kMaxLine + 1];
    for (int L = 1; L <= n; ++L) {
      C[L] = (L >= 2 && L <= n - 1) ? fma(ekv, wm[(long long)(L - 1) * sij], um[(long long)(L - 1) * sij]) : 0.0;
      lv[L] = lam[(long long)(L - 1) * st];
      Gb[L] = 0.0;
      Pb[L] = 0.0;
    }
    Gb[n + 1] = Gb[n + 2] = 0.0;
    lv[n - 1] += d.rho[fij] * lv[n];  // F2(NPA) = F2new(NPA-1) * rho
    lv[n] = 0.0;
    const double out1 = lv[1];       // cell L = 1 is not updated
    for (int L = 2; L <= n - 1; ++L) {
      const double le = (rl[(long long)(L - 1) * st] & kClipBit) ? 0.0 : lv[L];
      const double w = d.iwmu[L - 1];
      Gb[L] += le;
      Pb[L] -= w * le;
      Pb[L - 1] += w * le;
    }
    for (int L = 2; L <= n - 2; ++L) {
      const double FBb = C[L] * Pb[L];
      const bool neg = is_neg(C[L]);
      const double a = fma(C[L], d.mhdmu[L - 1], neg ? -0.5 : 0.5);
      scatter_face(Gb, FBb, neg ? L + 1 : L, rl[(long long)(L - 1) * st] & 7, a, beta, L, L + 1,
                   neg ? L + 1 : L - 1, neg ? L + 2 : L);
    }
    if (!closed) Gb[n] += C[n - 1] * Pb[n - 1];  // FBND(NPA-1) = F(NPA)
    Gb[2] += Gb[1];                               // F(1) = F(2)
    lam[0] = out1;
    for (int L = 2; L <= n; ++L) lam[(long long)(L - 1) * st] = Gb[L];
  }
}

void launch_adj_sweep(const Dev& d, int w, const unsigned char* rec, cudaStream_t st) {
  const int blk = 64;
  int nl;
  switch (w) {
    case 0: nl = d.nt * d.ne * d.npa; break;
    case 1: nl = (d.nr - 1) * d.ne * d.npa; break;
    case 2: nl = (d.nr - 1) * d.nt * d.npa; break;
    default: nl = (d.nr - 1) * d.nt * d.ne; break;
  }
  dim3 g((nl + blk - 1) / blk, d.nitems, 1);
  switch (w) {
    case 0: k_adj_r<<<g, blk, 0, st>>>(d, rec); break;
    case 1: k_adj_p<<<g, blk, 0, st>>>(d, rec); break;
    case 2: k_adj_e<<<g, blk, 0, st>>>(d, rec); break;
    default: k_adj_mu<<<g, blk, 0, st>>>(d, rec); break;
  }
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

__global__ void k_scale_lam(Dev d, const double* __restrict__ table) {
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= d.ncell) return;
  const int2 item = d.items[blockIdx.y];
  const int slot = item.x * d.ns + item.y;
  d.lam[(long long)slot * d.ncell + c] *= table[(long long)item.y * d.ncell + c];
}

void launch_scale_lam(const Dev& d, const double* table, cudaStream_t st) {
  k_scale_lam<<<dim3((unsigned)((d.ncell + 255) / 256), d.nitems), 256, 0, st>>>(d, table);
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
  if (o.call != call) return;
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

// Order-independent digest of a branch record (sum of mixed position*code
// terms modulo 2^64): equal digests of two runs mean an unchanged pattern
// with overwhelming probability.
__global__ void k_digest(const unsigned char* __restrict__ rec, long long n, unsigned long long* out) {
  unsigned long long acc = 0ULL;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
       c += (long long)gridDim.x * blockDim.x) {
    unsigned long long x = (unsigned long long)c * 0x9E3779B97F4A7C15ULL + rec[c];
    x ^= x >> 29;
    x *= 0xBF58476D1CE4E5B9ULL;
    x ^= x >> 32;
    acc += x * (rec[c] + 1ULL);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

void launch_digest(const unsigned char* rec, long long n, unsigned long long* out, cudaStream_t st) {
  k_digest<<<1024, 256, 0, st>>>(rec, n, out);
}

}  // namespace ramgpu
