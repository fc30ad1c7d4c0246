// bounce.cu -- the bounce integrals of computehI (src/ModRamScb.f90:378-406
// with integrator_c and bounceaverage_c, src/RamGSL.c:452-606): h, I and the
// bounce-averaged density of every RAM-grid field line and pitch angle.
//
// The reference integrates, with GSL cquad at 1e-3 tolerance, integrands
// built on the linear interpolant of B (and density) between the line's
// nodes.  Here the same integrals are evaluated exactly in closed form,
// segment by segment (u = Bm - B is linear on a segment):
//   int sqrt(u) = 2/3 w (a^2+ab+b^2)/(a+b),   int 1/sqrt(u) = 2 w/(a+b),
//   int (n0 + dn t)/sqrt(u) = w (n0 H1 + dn H2),
//   H1 = 2/(a+b), H2 = 2(b+2a)/(3(a+b)^2),   a = sqrt(u0), b = sqrt(u1),
// cut at u = 0 where B >= Bm; no cancellation occurs in these forms.
//
// Three kernels: per line the geometry, the equator fix and the full-line
// baseline; per (line, pitch angle) the reference's bracket logic and the
// integrals; per line the reference's descending copy rules and the
// normalisation into H_cart, I_cart and HDens_cart.
#include <math.h>

#include "kernels.cuh"

namespace ramgpu {

namespace {

__device__ void seg_int(double c0, double c1, double B0, double B1, double n0, double n1, double bm, bool dens,
                        double& yi, double& yh, double& yd) {
  const double u0 = bm - B0, u1 = bm - B1, dchi = c1 - c0;
  if (u0 <= 0 && u1 <= 0) return;
  double a, b, na, nb, w;
  if (u0 > 0 && u1 > 0) {
    a = sqrt(u0); b = sqrt(u1); na = n0; nb = n1; w = dchi;
  } else if (u0 > 0) {
    const double f = u0 / (u0 - u1);
    a = sqrt(u0); b = 0.0; na = n0; nb = n0 + (n1 - n0) * f; w = dchi * f;
  } else {
    const double f = u1 / (u1 - u0);
    a = 0.0; b = sqrt(u1); na = n1 + (n0 - n1) * f; nb = n1; w = dchi * f;
  }
  const double s = a + b;
  if (dens) {
    yd += w * (na * (2. / s) + (nb - na) * (2. * (b + 2. * a) / (3. * s * s)));
  } else {
    yi += (2. / 3.) * w * (a * a + a * b + b * b) / s;
    yh += 2. * w / s;
  }
}

__device__ void line_int(int nthe, const double* chi, const double* bf, const double* var, double bm, int i0,
                         int i1, double& yi, double& yh, double& yd) {
  yi = 0.0; yh = 0.0; yd = 0.0;
  for (int k = i0; k < i1; ++k)
    seg_int(chi[k], chi[k + 1], bf[k], bf[k + 1], var ? var[k] : 0.0, var ? var[k + 1] : 0.0, bm, var != nullptr,
            yi, yh, yd);
}

// Bracket of the mirror points and the reference's fallback, as indices:
// returns 0 (integrate over [lh, rh]), 1 (mirror outside the line: take the
// full-line value), 2 (bracket of at most 4 segments: copy L+1).
__device__ int bracket(int nT, const double* chi, const double* bf, double m, int& lh, int& rh) {
  double a = 0, b = 0;
  lh = 0; rh = 0;
  for (int i = 1; i < nT - 1; i++)
    if (m <= bf[i - 1] && m >= bf[i]) { a = chi[i - 1]; lh = i - 1; break; }
  for (int i = nT - 2; i > 0; i--)
    if (m >= bf[i - 1] && m <= bf[i]) { b = chi[i]; rh = i; break; }
  if (m >= bf[1] || a == 0) a = chi[0];
  if (m >= bf[nT - 1] || b == 0) b = chi[nT - 1];
  if (a <= chi[0] || b >= chi[nT - 1]) return 1;
  if (rh - lh <= 4) return 2;
  return 0;
}

}  // namespace

// per line: length, r0, equator fix, mirror fields, full-line baselines
__global__ void k_bounce_lines(BounceDev q) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= q.nr * q.nt) return;
  const int nthe = q.nthe, npa = q.npa;
  double* bf = q.b + (long long)t * nthe;
  q.line_ok[t] = q.outside[t] == 0;
  if (!q.line_ok[t]) return;
  const double* x = q.x + (long long)t * nthe;
  const double* y = q.y + (long long)t * nthe;
  const double* z = q.z + (long long)t * nthe;
  double length = 0.0;
  for (int k = 1; k < nthe; ++k) {
    const double dx = x[k] - x[k - 1], dy = y[k] - y[k - 1], dz = z[k] - z[k - 1];
    length = length + sqrt(dx * dx + dy * dy + dz * dz);
  }
  const int e = q.ieq - 1;
  const double r0 = sqrt(x[e] * x[e] + y[e] * y[e]);
  double bmin = bf[0];
  for (int k = 1; k < nthe; ++k) bmin = bf[k] < bmin ? bf[k] : bmin;
  if (fabs(bf[e] - bmin) > 1e-9) bf[e] = (2. * bmin - bf[e] > 0.) ? 2. * bmin - bf[e] : bmin - 0.01;
  q.length[t] = length;
  q.r0[t] = r0;
  const long long lo = (long long)t * npa;
  for (int L = 0; L < npa - 1; ++L) q.mirror[lo + L] = bf[e] / (1. - q.mu[L] * q.mu[L]);
  q.mirror[lo + npa - 1] = bf[nthe - 1];
  double yi, yh, yd;
  line_int(nthe, q.chi, bf, nullptr, bf[nthe - 1], 0, nthe - 1, yi, yh, yd);
  q.yi[lo + npa - 1] = yi;
  q.yh[lo + npa - 1] = yh;
  if (q.dens) {
    line_int(nthe, q.chi, bf, q.dens + (long long)t * nthe, bf[nthe - 1], 0, nthe - 1, yi, yh, yd);
    q.yd[lo + npa - 1] = yd;
  }
}

// per (line, L) for L = 2..NPA-1 (1-based): the integrator's and the bounce
// average's decisions and integrals (the latter with the mirror the
// integrator leaves: the full-line one when the mirror lies outside)
__global__ void k_bounce_angles(BounceDev q) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int npa = q.npa, nm = npa - 2;
  if (t >= (long long)q.nr * q.nt * nm) return;
  const int line = (int)(t / nm), L = 1 + (int)(t % nm);
  if (!q.line_ok[line]) return;
  const int nthe = q.nthe;
  const double* bf = q.b + (long long)line * nthe;
  const long long o = (long long)line * npa + L;
  double m = q.mirror[o];
  int lh, rh;
  const int st = bracket(nthe, q.chi, bf, m, lh, rh);
  double yi = 0, yh = 0, yd = 0;
  if (st == 0) line_int(nthe, q.chi, bf, nullptr, m, lh, rh, yi, yh, yd);
  if (st == 1) m = q.mirror[(long long)line * npa + npa - 1];
  q.st[o] = (unsigned char)st;
  q.yi[o] = yi;
  q.yh[o] = yh;
  q.mirror2[o] = m;
  if (q.dens) {
    const int sd = bracket(nthe, q.chi, bf, m, lh, rh);
    double d = 0;
    if (sd == 0) line_int(nthe, q.chi, bf, q.dens + (long long)line * nthe, m, lh, rh, yi, yh, d);
    q.sd[o] = (unsigned char)sd;
    q.yd[o] = d;
  }
}

// per line: the descending copy rules, then H_cart, I_cart, HDens_cart
__global__ void k_bounce_finish(BounceDev q) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= q.nr * q.nt) return;
  const int npa = q.npa;
  const int i = t % q.nr, j = t / q.nr;
  auto out = [&](double* a, int L, double v) {
    if (a) a[((long long)L * q.nt + j) * q.nr + i] = v;
  };
  if (!q.line_ok[t]) {
    for (int L = 0; L < npa; ++L) {
      out(q.h_out, L, 0.0); out(q.i_out, L, 0.0); out(q.d_out, L, 0.0); out(q.m_out, L, 0.0);
    }
    return;
  }
  const long long lo = (long long)t * npa;
  double* yi = q.yi + lo;
  double* yh = q.yh + lo;
  double* yd = q.yd ? q.yd + lo : nullptr;
  double* m2 = q.mirror2 + lo;
  m2[0] = q.mirror[lo];
  m2[npa - 1] = q.mirror[lo + npa - 1];
  for (int L = npa - 2; L > 0; --L) {
    const int st = q.st[lo + L];
    if (st == 1) { yi[L] = yi[npa - 1]; yh[L] = yh[npa - 1]; }
    else if (st == 2) { yi[L] = yi[L + 1]; yh[L] = yh[L + 1]; }
    else {
      if (yi[L] <= 0) yi[L] = yi[L + 1];
      if (yh[L] <= 0) yh[L] = yh[L + 1];
    }
    if (yd) {
      const int sd = q.sd[lo + L];
      if (sd == 1) yd[L] = yd[npa - 1];
      else if (sd == 2 || yd[L] <= 0) yd[L] = yd[L + 1];
    }
  }
  yi[0] = 0;
  yh[0] = yh[1];
  if (yd) yd[0] = yd[1];
  const double pi_d = kPI, len = q.length[t], r0 = q.r0[t];
  for (int L = 0; L < npa; ++L) {
    out(q.i_out, L, (len / (pi_d * r0)) * yi[L] / sqrt(m2[L]));
    out(q.h_out, L, (len / (pi_d * 2 * r0)) * yh[L] * sqrt(m2[L]));
    if (yd) out(q.d_out, L, yd[L] / yh[L]);
    out(q.m_out, L, m2[L]);
  }
}

void launch_bounce(const BounceDev& q, cudaStream_t st) {
  const int nl = q.nr * q.nt;
  k_bounce_lines<<<(nl + 127) / 128, 128, 0, st>>>(q);
  const long long na = (long long)nl * (q.npa - 2);
  k_bounce_angles<<<(unsigned)((na + 127) / 128), 128, 0, st>>>(q);
  k_bounce_finish<<<(nl + 127) / 128, 128, 0, st>>>(q);
}

}  // namespace ramgpu

namespace ramgpu {

// ------------------------------------------------------- the field-table fill
// computehI's RAM-variable fill (src/ModRamScb.f90:458-463,520-632) on the
// device, from the bounce integrals: BOUNHS/BOUNIS by Steffen's (1990)
// monotone cubic in pitch angle at the bin boundaries PAbn (interior slopes
// by his eq. (11), one-sided secants at the ends, linear extrapolation
// outside the data, as the reference's 1-D interpolation wrapper), then
// FNHS..BOUNIS, BNES and the time derivatives written into the context's
// field tables, the I = 1 row and the NaN repair.

namespace {
__device__ double sgn1(double v) { return v < 0 ? -1.0 : 1.0; }

// Steffen slopes and values at xb of data (xa ascending, distinct)
__device__ void steffen_line(int n, const double* xa, const double* fa, double* yp, int nb, const double* xb,
                             double* fb, long long fbs) {
  yp[0] = (fa[1] - fa[0]) / (xa[1] - xa[0]);
  for (int i = 1; i < n - 1; ++i) {
    const double hm = xa[i] - xa[i - 1], h = xa[i + 1] - xa[i];
    const double sm = (fa[i] - fa[i - 1]) / hm, s = (fa[i + 1] - fa[i]) / h;
    const double p = (sm * h + s * hm) / (hm + h);
    double m = fabs(sm);
    if (fabs(s) < m) m = fabs(s);
    if (0.5 * fabs(p) < m) m = 0.5 * fabs(p);
    yp[i] = (sgn1(sm) + sgn1(s)) * m;
  }
  yp[n - 1] = (fa[n - 1] - fa[n - 2]) / (xa[n - 1] - xa[n - 2]);
  for (int q = 0; q < nb; ++q) {
    const double x = xb[q];
    double v;
    if (x <= xa[0]) {
      v = fa[0] + (x - xa[0]) / (xa[1] - xa[0]) * (fa[1] - fa[0]);
    } else if (x >= xa[n - 1]) {
      v = fa[n - 1] + (x - xa[n - 1]) / (xa[n - 2] - xa[n - 1]) * (fa[n - 2] - fa[n - 1]);
    } else {
      int i = 0;
      while (i < n - 2 && xa[i + 1] <= x) ++i;
      const double h = xa[i + 1] - xa[i], s = (fa[i + 1] - fa[i]) / h;
      const double a = (yp[i] + yp[i + 1] - 2 * s) / h / h, b = (3 * s - 2 * yp[i] - yp[i + 1]) / h;
      const double t = x - xa[i];
      v = fa[i] + t * (yp[i] + t * (b + t * a));
    }
    fb[(long long)q * fbs] = v;
  }
}
}  // namespace

// per J: lines outside the magnetopause take the previous radial point
__global__ void k_hi_outside(HiDev q) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= q.nt) return;
  const long long sl = (long long)q.nr * q.nt;
  for (int i = 1; i < q.nr; ++i) {
    if (q.outside[(long long)j * q.nr + i] != 1) continue;
    for (int L = 0; L < q.npa; ++L) {
      const long long o = (long long)L * sl + (long long)j * q.nr + i;
      q.h[o] = q.h[o - 1];
      q.fi[o] = q.fi[o - 1];
      q.hd[o] = q.hd[o - 1];
    }
    q.beq[(long long)j * q.nr + i] = q.beq[(long long)j * q.nr + i - 1];
  }
}

// per line: h and I interpolated to PAbn (x ascending: PA(NPA:1:-1))
__global__ void k_hi_interp(HiDev q) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nl = q.nr * q.nt;
  if (t >= 2 * nl) return;
  const int w = t / nl, line = t % nl;
  const int npa = q.npa;
  const long long sl = nl;
  const double* src = (w ? q.fi : q.h) + line;
  double* dst = (w ? q.ib : q.hb) + line;
  double* sc = q.scratch + (long long)t * 3 * npa;
  double *fa = sc, *yp = sc + npa;
  // data in ascending PA, reduced to strictly increasing x
  int n = 0;
  double* xa = sc + 2 * npa;
  for (int L = 0; L < npa; ++L) {
    const double x = q.pa[npa - 1 - L];
    if (n == 0 || x > xa[n - 1]) { xa[n] = x; fa[n] = src[(long long)(npa - 1 - L) * sl]; ++n; }
  }
  // targets PAbn(NPA-1:2:-1) -> BOUN*(NPA-1 .. 2)
  steffen_line(n, xa, fa, yp, npa - 2, q.pabn_rev, dst + (long long)(npa - 2) * sl, -sl);
  dst[(long long)(npa - 1) * sl] = dst[(long long)(npa - 2) * sl];
  dst[0] = dst[sl];
}

// per (I >= 2, J, L): the fields of row I from line I-1, with time derivatives
__global__ void k_hi_fill(HiDev q) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long n = (long long)q.nr * q.nt * q.npa;
  if (t >= n) return;
  const int i = (int)(t % q.nr);                     // line index, row I = i+2 (1-based)
  const int j = (int)((t / q.nr) % q.nt);
  const int L = (int)(t / ((long long)q.nr * q.nt));
  const int nf = q.nr + 1;
  const long long f = ((long long)L * q.nt + j) * nf + (i + 1);
  const double fip = q.fnis[f], bip = q.bounis[f];
  const bool dt0 = fabs(q.dthi) <= 1e-9;
  q.fnhs[f] = q.h[t];
  q.fnis[f] = q.fi[t];
  q.hdns[f] = q.hd[t];
  q.bounhs[f] = q.hb[t];
  q.bounis[f] = q.ib[t];
  q.didt[f] = dt0 ? 0.0 : (q.fi[t] - fip) / q.dthi;
  q.dibndt[f] = dt0 ? 0.0 : (q.ib[t] - bip) / q.dthi;
  if (L == 0) {
    const long long f2 = (long long)j * nf + (i + 1);
    const double bprev = q.bnes[f2];
    q.bnes[f2] = q.beq[(long long)j * q.nr + i] * q.bnormal / 1e9;
    q.dbdt[f2] = dt0 ? 0.0 : (q.bnes[f2] - bprev) / q.dthi;
  }
}

// per (J, L): the I = 1 row, then the NaN repair in increasing I
__global__ void k_hi_rows(HiDev q) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= q.nt * q.npa) return;
  const int j = t % q.nt, L = t / q.nt;
  const int nf = q.nr + 1;
  const long long b = ((long long)L * q.nt + j) * nf;
  if (L == 0) {
    const long long b2 = (long long)j * nf;
    q.bnes[b2] = 0.32 / (q.lz0 * q.lz0 * q.lz0) / 1.e4;
    q.dbdt[b2] = 0.0;
    q.eir[b2] = 0.0;
    q.eip[b2] = 0.0;
  }
  q.fnhs[b] = q.fnhs[b + 1];
  q.fnis[b] = q.fnis[b + 1];
  q.bounhs[b] = q.bounhs[b + 1];
  q.bounis[b] = q.bounis[b + 1];
  q.hdns[b] = q.hdns[b + 1];
  q.didt[b] = 0.0;
  q.dibndt[b] = 0.0;
  for (int I = 1; I < nf; ++I) {
    const long long c = b + I;
    if (isnan(q.fnis[c])) q.fnis[c] = q.fnis[c - 1];
    if (isnan(q.fnhs[c])) q.fnhs[c] = q.fnhs[c - 1];
    if (isnan(q.bounis[c])) q.bounis[c] = q.bounis[c - 1];
    if (isnan(q.bounhs[c])) q.bounhs[c] = q.bounhs[c - 1];
    if (isnan(q.hdns[c])) q.hdns[c] = q.hdns[c - 1];
    if (isnan(q.didt[c])) q.didt[c] = 0.0;
    if (isnan(q.dibndt[c])) q.dibndt[c] = 0.0;
  }
}

void launch_hi_fill(const HiDev& q, cudaStream_t st) {
  k_hi_outside<<<(q.nt + 63) / 64, 64, 0, st>>>(q);
  const int nl2 = 2 * q.nr * q.nt;
  k_hi_interp<<<(nl2 + 63) / 64, 64, 0, st>>>(q);
  const long long n = (long long)q.nr * q.nt * q.npa;
  k_hi_fill<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(q);
  const int nr2 = q.nt * q.npa;
  k_hi_rows<<<(nr2 + 127) / 128, 128, 0, st>>>(q);
}

}  // namespace ramgpu
