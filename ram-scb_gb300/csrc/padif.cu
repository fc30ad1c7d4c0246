// padif.cu -- implicit pitch-angle diffusion: WPADIF (src/ModRamWPI.f90:
// 643-714) and FLCscatter (src/ModRamLoss.f90:512-575) share one scheme,
//   (1 + AN + GN) F(L) - AN F(L+1) - GN F(L-1) = F_old(L),  F = F2/(FNHS*MU),
// with AN = D(L)/DMU(L)*DTs/(FNHS(L)*MU(L))/WMU(L), GN = D(L-1)/DMU(L-1)*DTs/
// (FNHS(L)*MU(L))/WMU(L), F(1) = F(2) below and F(NPA) = F(NPA-1) above,
// solved by the reference's forward elimination (RK, RL) and back
// substitution.  RL and the pivots depend only on D, the fields and DTs,
// so they are tabulated once (k_padif_tables, with the reference's
// divisions); a call then costs per cell one fma and two multiplies in the
// forward sweep and one fma and one multiply in the backward sweep, and
// reads F2 once (the forward sweep parks RK in F2's own line, which stays
// in L2 until the backward sweep reads it back).  Every line pointer is
// __restrict__: the table loads of the next cells do not depend on the
// elimination, and only the compiler's aliasing doubt would hold them
// behind each store to the line.
#include "kernels.cuh"

namespace ramgpu {

// FACMU = FNHS*MU and its reciprocal, (NR, NT, NPA) with I fastest.
__global__ void k_padif_fac(Dev d) {
  const long long n = (long long)d.nr * d.nt * d.npa;
  const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int i = (int)(c % d.nr), j = (int)((c / d.nr) % d.nt), l = (int)(c / ((long long)d.nr * d.nt));
  const double fac = d.fnhs[((long long)l * d.nt + j) * d.nf + i] * d.mu[l];
  d.pd_fac[c] = fac;
  d.pd_ifac[c] = 1.0 / fac;
}

// Per line (I>=2, J, K>=2) of each species with a coefficient: GN(L), the
// reciprocal pivot 1/DENOM(L) and RL(L) for L = 2..NPA-1, and at L = NPA
// the reciprocal 1/(1+RL(NPA-1)) of the upper boundary.
__global__ void k_padif_tables(Dev d, double dts) {
  const int nr1 = d.nr - 1, ne1 = d.ne - 1;
  const long long nl = (long long)nr1 * d.nt * ne1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int s = blockIdx.y;
  if (t >= nl || !d.pd_on[s]) return;
  const int i = 1 + (int)(t % nr1);
  const int j = (int)((t / nr1) % d.nt);
  const int k = 1 + (int)(t / ((long long)nr1 * d.nt));
  const long long st = (long long)d.ne * d.nt * d.nr;
  const long long off = ((long long)k * d.nt + j) * d.nr + i;
  const double* __restrict__ D = d.pd_d + (long long)s * d.ncell + off;
  double* __restrict__ gn = d.pd_gn + (long long)s * d.ncell + off;
  double* __restrict__ inv = d.pd_inv + (long long)s * d.ncell + off;
  double* __restrict__ rl = d.pd_rl + (long long)s * d.ncell + off;
  const int npa = d.npa;
  double rlp = -1.0;  // RL(1)
  for (int L = 2; L <= npa - 1; ++L) {
    const double facmu = d.fnhs[((long long)(L - 1) * d.nt + j) * d.nf + i] * d.mu[L - 1];
    double AN = D[(long long)(L - 1) * st] / d.dmu[L - 1];
    double GN = D[(long long)(L - 2) * st] / d.dmu[L - 2];
    AN = AN * dts / facmu / d.wmu[L - 1];
    GN = GN * dts / facmu / d.wmu[L - 1];
    const double BN = AN + GN;
    const double DENOM = BN + GN * rlp + 1;
    const double RL = -AN / DENOM;
    gn[(long long)(L - 1) * st] = GN;
    inv[(long long)(L - 1) * st] = 1.0 / DENOM;
    rl[(long long)(L - 1) * st] = RL;
    rlp = RL;
  }
  inv[(long long)(npa - 1) * st] = 1.0 / (1 + rlp);
}

// One application on every active item.  Items whose species has no
// coefficient only get the optional diagonal factor `loss` (the fused
// CEX/ATMOL product of the middle of ram_run), applied here to the result.
__global__ void __launch_bounds__(128) k_padif(Dev d, const double* __restrict__ loss) {
  const int nr1 = d.nr - 1, ne1 = d.ne - 1;
  const long long nl = (long long)nr1 * d.nt * ne1;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= nl) return;
  const int2 item = d.items[blockIdx.y];
  const int s = item.y, slot = item.x * d.ns + s;
  const bool on = d.pd_on[s];
  if (!on && !loss) return;
  const int i = 1 + (int)(t % nr1);
  const int j = (int)((t / nr1) % d.nt);
  const int k = 1 + (int)(t / ((long long)nr1 * d.nt));
  const int npa = d.npa;
  const long long st = (long long)d.ne * d.nt * d.nr;
  const long long off = ((long long)k * d.nt + j) * d.nr + i;
  double* __restrict__ fl = d.f2 + (long long)slot * d.ncell + off;
  const double* __restrict__ la = loss ? loss + (long long)s * d.ncell + off : nullptr;
  if (!on) {
#pragma unroll 8
    for (int L = 1; L <= npa; ++L) fl[(long long)(L - 1) * st] *= la[(long long)(L - 1) * st];
    return;
  }
  const long long so = (long long)s * d.ncell + off;
  const double* __restrict__ gn = d.pd_gn + so;
  const double* __restrict__ inv = d.pd_inv + so;
  const double* __restrict__ rl = d.pd_rl + so;
  const long long sij = (long long)d.nt * d.nr, fij = (long long)j * d.nr + i;
  const double* __restrict__ fac = d.pd_fac + fij;
  const double* __restrict__ ifac = d.pd_ifac + fij;
  // forward elimination: RK(L) = (F(L) + GN(L) RK(L-1)) / DENOM(L), RK(1) = 0.
  // A species' lines are few (3-4 warps per SM), so the loads of a block of
  // kB cells are issued together into registers before the block's
  // dependent chain: the memory latency is paid once per block, not per cell.
  constexpr int kB = 16;
  double rk = 0.0;
  int L = 2;
  for (; L + kB - 1 <= npa - 1; L += kB) {
    double F[kB], g[kB], iv[kB];
#pragma unroll
    for (int u = 0; u < kB; ++u) {
      const long long q = (long long)(L + u - 1) * st;
      F[u] = fl[q] * ifac[(long long)(L + u - 1) * sij];
      g[u] = gn[q];
      iv[u] = inv[q];
    }
#pragma unroll
    for (int u = 0; u < kB; ++u) {
      rk = fma(g[u], rk, F[u]) * iv[u];
      fl[(long long)(L + u - 1) * st] = rk;
    }
  }
  for (; L <= npa - 1; ++L) {
    const long long q = (long long)(L - 1) * st;
    const double F = fl[q] * ifac[(long long)(L - 1) * sij];
    rk = fma(gn[q], rk, F) * inv[q];
    fl[q] = rk;
  }
  // upper boundary F(NPA-1) = RK/(1+RL), F(NPA) = F(NPA-1); back substitution
  double x = rk * inv[(long long)(npa - 1) * st];
  auto put = [&](int Lq, double v) {
    const long long q = (long long)(Lq - 1) * st;
    double o = v * fac[(long long)(Lq - 1) * sij];
    if (loss) o *= la[q];
    fl[q] = o;
  };
  put(npa, x);
  put(npa - 1, x);
  L = npa - 2;
  for (; L - kB + 1 >= 2; L -= kB) {
    double r[kB], rk2[kB], fc[kB], lf[kB];
#pragma unroll
    for (int u = 0; u < kB; ++u) {
      const long long q = (long long)(L - u - 1) * st;
      r[u] = rl[q];
      rk2[u] = fl[q];
      fc[u] = fac[(long long)(L - u - 1) * sij];
      lf[u] = loss ? la[q] : 1.0;
    }
#pragma unroll
    for (int u = 0; u < kB; ++u) {
      x = fma(-r[u], x, rk2[u]);
      double o = x * fc[u];
      if (loss) o *= lf[u];
      fl[(long long)(L - u - 1) * st] = o;
    }
  }
  for (; L >= 2; --L) {
    const long long q = (long long)(L - 1) * st;
    x = fma(-rl[q], x, fl[q]);
    put(L, x);
  }
  put(1, x);  // F(1) = RK(1) - RL(1) F(2) = F(2)
}

void launch_padif_tables(const Dev& d, double dts, cudaStream_t st) {
  const long long n = (long long)d.nr * d.nt * d.npa;
  k_padif_fac<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d);
  const long long nl = (long long)(d.nr - 1) * d.nt * (d.ne - 1);
  k_padif_tables<<<dim3((unsigned)((nl + 127) / 128), d.ns), 128, 0, st>>>(d, dts);
}

void launch_padif(const Dev& d, const double* loss, cudaStream_t st) {
  const long long nl = (long long)(d.nr - 1) * d.nt * (d.ne - 1);
  if (d.nitems > 0) k_padif<<<dim3((unsigned)((nl + 127) / 128), d.nitems), 128, 0, st>>>(d, loss);
}

}  // namespace ramgpu
