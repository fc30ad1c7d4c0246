// status.cu -- the device status word of a context.
//
// The reference stops the run when a moment is no longer finite (ANISCH,
// src/ModRamRun.f90:410-413) and lets the caller shorten DTs from the
// DtDrift* of the sweeps (src/ModRamRun.f90:204-205).  The library never
// stops; one pass over the active items' F2 and moments instead counts
// what the caller needs to decide:
//   st[0]  F2 cells that are NaN or infinite,
//   st[1]  PPERT / PPART values that are NaN or infinite,
//   st[2]  (item, sweep) pairs of the last call whose largest Courant
//          number (|C| for R and P, |C|/DE and |C|/DMU for E and MU, the
//          quantity DtDrift* divides FracCFL*DTs by) exceeded 1,
//   st[3]  the smallest list position of an item holding a non-finite
//          value (all bits set if none),
//   st[4]  updated cells the sweeps of the last call clipped to 1e-15
//          because they came out negative (src/ModRamDrift.f90:187-190 and
//          the same lines of DRIFTP/E/MU), counted while the status pass is
//          appended to each call.
// Integer tests on the exponent bits: no FP64 work, one read of F2.
#include <string.h>

#include "kernels.cuh"
#include "diag.cuh"

namespace ramgpu {

namespace {
constexpr bits64 kExpBits = 0x7ff0000000000000ULL;
__device__ __forceinline__ unsigned nonfinite(double v) { return (dbits(v) & kExpBits) == kExpBits; }
}  // namespace

__global__ void __launch_bounds__(256) k_status(Dev d, unsigned long long* __restrict__ st) {
  const int it = blockIdx.y;
  const int2 item = d.items[it];
  const long long slot = (long long)item.x * d.ns + item.y;
  const double* __restrict__ f = d.f2 + slot * d.ncell;
  const long long nm2 = (long long)d.nr * d.nt;
  const double* __restrict__ pe = d.ppert + slot * nm2;
  const double* __restrict__ pa = d.ppart + slot * nm2;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  unsigned long long nf = 0, nmom = 0;
  for (long long c = t0; c < d.ncell; c += stride) nf += nonfinite(__ldg(f + c));
  for (long long c = t0; c < nm2; c += stride) nmom += nonfinite(__ldg(pe + c)) + nonfinite(__ldg(pa + c));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    nf += __shfl_xor_sync(0xffffffffu, nf, o);
    nmom += __shfl_xor_sync(0xffffffffu, nmom, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (nf) atomicAdd(&st[0], nf);
    if (nmom) atomicAdd(&st[1], nmom);
    if (nf | nmom) atomicMin(&st[3], (unsigned long long)it);
  }
  if (blockIdx.x == 0 && threadIdx.x < 4) {
    // the CFL accumulators hold the bits of the largest quotient of the
    // last call (0: the sweep recorded none); DRIFTMU's floor term as in
    // DtDriftMu (src/ModRamDrift.f90:435)
    const unsigned long long q = d.cflq[slot * 4 + threadIdx.x];
    double qq = bitsd(q);
    if (threadIdx.x == 3) qq = fmax(qq, 1E-32 / d.dmu[d.npa - 1]);
    if (q != 0ULL && qq > 1.0) atomicAdd(&st[2], 1ULL);
    if (threadIdx.x == 0) {
      const unsigned long long nc = d.clipq[slot];
      if (nc) atomicAdd(&st[4], nc);
    }
  }
}

void launch_status(const Dev& d, unsigned long long* st, cudaStream_t s) {
  cudaMemsetAsync(st, 0, 5 * sizeof(unsigned long long), s);
  cudaMemsetAsync(st + 3, 0xff, sizeof(unsigned long long), s);
  if (d.nitems == 0) return;
  long long gx = (d.ncell + 256LL * 16 - 1) / (256LL * 16);  // 16 cells per thread
  gx = gx < 1 ? 1 : (gx > 4096 ? 4096 : gx);
  k_status<<<dim3((unsigned)gx, (unsigned)d.nitems), 256, 0, s>>>(d, st);
}

// ------------------------------------------------------------ F2 statistics
// One (member, species) slot: the smallest and largest F2 over all cells
// and the number content, the sum of F2*WE(K)*WMU(L) over the cells the
// sweeps update (I >= 2, J <= NT-1 with J = NT the periodic copy of J = 1,
// K >= 2, 2 <= L <= NPA-1), the quantity closed boundaries conserve.  Each
// block sums a fixed set of cells in a fixed order and reduces through
// shared memory in a fixed tree, so the partials, and the host's ordered sum
// of them, are the same bits on every call.  Min and max go through an
// order-preserving integer key (sign-magnitude to two's-complement order).
namespace {
__device__ __forceinline__ bits64 order_key(double v) {
  const bits64 b = dbits(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}
}  // namespace

__global__ void __launch_bounds__(256) k_f2_stats(Dev d, long long slot, double* __restrict__ part,
                                                  unsigned long long* __restrict__ mm) {
  __shared__ double sh[256];
  __shared__ unsigned long long smin[8], smax[8];
  const double* __restrict__ f = d.f2 + slot * d.ncell;
  const long long nrt = (long long)d.nr * d.nt, nrte = nrt * d.ne;
  double acc = 0.0;
  bits64 kmin = ~0ULL, kmax = 0ULL;
  for (long long c = blockIdx.x * 256LL + threadIdx.x; c < d.ncell; c += 256LL * gridDim.x) {
    const double v = __ldg(f + c);
    const bits64 k = order_key(v);
    kmin = k < kmin ? k : kmin;
    kmax = k > kmax ? k : kmax;
    const int i = (int)(c % d.nr), j = (int)((c / d.nr) % d.nt);
    const int k3 = (int)((c / nrt) % d.ne), l = (int)(c / nrte);
    if (i >= 1 && j <= d.nt - 2 && k3 >= 1 && l >= 1 && l <= d.npa - 2) acc = fma(v, d.we[k3] * d.wmu[l], acc);
  }
  sh[threadIdx.x] = acc;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const bits64 a = __shfl_xor_sync(0xffffffffu, kmin, o), b = __shfl_xor_sync(0xffffffffu, kmax, o);
    kmin = a < kmin ? a : kmin;
    kmax = b > kmax ? b : kmax;
  }
  if ((threadIdx.x & 31) == 0) {
    smin[threadIdx.x >> 5] = kmin;
    smax[threadIdx.x >> 5] = kmax;
  }
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[blockIdx.x] = sh[0];
    for (int w = 1; w < 8; ++w) {
      kmin = smin[w] < kmin ? smin[w] : kmin;
      kmax = smax[w] > kmax ? smax[w] : kmax;
    }
    atomicMin(&mm[0], smin[0] < kmin ? smin[0] : kmin);
    atomicMax(&mm[1], smax[0] > kmax ? smax[0] : kmax);
  }
}

double f2_stats_key_value(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFULL) : ~k;
  double v;
  memcpy(&v, &b, sizeof v);
  return v;
}

void launch_f2_stats(const Dev& d, long long slot, double* part, unsigned long long* mm, cudaStream_t s) {
  cudaMemsetAsync(mm, 0xff, sizeof(unsigned long long), s);                          // min key
  cudaMemsetAsync(mm + 1, 0, sizeof(unsigned long long), s);                         // max key
  k_f2_stats<<<kF2StatBlocks, 256, 0, s>>>(d, slot, part, mm);
}

}  // namespace ramgpu
