// outputs.cu -- products of the state handed to callers: virtual-spacecraft
// flux samples and the species-summed pressures SCB reads.
//
//   k_fly_sats       FLUX (src/ModRamRun.f90:208-222) at equatorial points,
//                    SatFlux(S,E,PA) and OmnFlux(S,E) as fly_sats forms them
//                    (src/ModRamSats.f90:640-666)
//   k_sum_pressure   PAllSum = sum_S 2/3 PPERT + 1/3 PPART, PParSum = sum_S PPART
//                    (ram_sum_pressure, src/ModRamFunctions.f90:272-297)
#include <math.h>

#include "kernels.cuh"

namespace ramgpu {

constexpr double kBadData = -1.0E10;  // BadDataFlag, src/ModRamSats.f90:35

// One CTA per (satellite, species); thread k handles energy bin K = k+1 and
// walks the pitch-angle bins in order, so OmnFlux sums in the reference's
// order.  FLUX is defined for I, K, L >= 2 and J <= NT-1 (zero elsewhere),
// so a corner outside that range makes the sample BadDataFlag.
__global__ void k_fly_sats(Dev d, const SatDev* __restrict__ sats, double* __restrict__ sat_flux,
                           double* __restrict__ omni) {
  const SatDev q = sats[blockIdx.x];
  const int s = blockIdx.y;
  const int ns = d.ns, ne = d.ne, npa = d.npa;
  const bool active = (q.active_mask >> s) & 1u;
  const double* f2 = d.f2 + (long long)(q.member * ns + s) * d.ncell;
  const double* ff = d.ffactor + (long long)s * d.nr * ne * npa;
  for (int k = threadIdx.x; k < ne; k += blockDim.x) {
    double om = 0.0;
    for (int l = 0; l < npa; ++l) {
      double v = kBadData;
      if (active && k >= 1 && l >= 1) {
        double acc = 0.0;
        bool pos = true;
        for (int a = 0; a < 2; ++a)
          for (int b = 0; b < 2; ++b) {
            const int i = q.i0 + a, j = b ? q.j1 : q.j0;
            const double w = __dmul_rn(a ? q.wi : 1.0 - q.wi, b ? q.wj : 1.0 - q.wj);
            const long long c = (((long long)l * ne + k) * d.nt + j) * d.nr + i;
            const double fl = f2[c] / ff[((long long)l * ne + k) * d.nr + i] / d.fnhs[((long long)l * d.nt + j) * d.nf + i];
            pos = pos && fl > 0.0;
            acc = __dadd_rn(acc, __dmul_rn(w, fl));
          }
        if (pos) v = acc;
      }
      if (sat_flux) sat_flux[(long long)blockIdx.x * ns * ne * npa + s + (long long)ns * (k + (long long)ne * l)] = v;
      if (v > 0.0) om = __dadd_rn(om, __dmul_rn(__dmul_rn(__dmul_rn(v, 4.0), kPI), d.wmu[l]));
    }
    if (omni) omni[(long long)blockIdx.x * ns * ne + s + (long long)ns * k] = om > 0.0 ? om : kBadData;
  }
}

void launch_fly_sats(const Dev& d, const SatDev* sats, int nsat, double* sat_flux, double* omni,
                     cudaStream_t st) {
  if (nsat > 0) k_fly_sats<<<dim3((unsigned)nsat, (unsigned)d.ns), 64, 0, st>>>(d, sats, sat_flux, omni);
}

__global__ void k_sum_pressure(Dev d, int member, unsigned mask, double* __restrict__ pall,
                               double* __restrict__ ppar) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = d.nr * d.nt;
  if (c >= n) return;
  const double onethird = 1.0 / 3.0, twothird = 2.0 / 3.0;
  double a = 0.0, p = 0.0;
  for (int s = 0; s < d.ns; ++s) {
    if (!((mask >> s) & 1u)) continue;
    const long long o = (long long)(member * d.ns + s) * n + c;
    const double pe = d.ppert[o], pa = d.ppart[o];
    a = __dadd_rn(__dadd_rn(a, __dmul_rn(twothird, pe)), __dmul_rn(onethird, pa));
    p = __dadd_rn(p, pa);
  }
  pall[c] = a;
  ppar[c] = p;
}

void launch_sum_pressure(const Dev& d, int member, unsigned mask, double* pall, double* ppar,
                         cudaStream_t st) {
  const int n = d.nr * d.nt;
  k_sum_pressure<<<(n + 127) / 128, 128, 0, st>>>(d, member, mask, pall, ppar);
}

}  // namespace ramgpu
