// layout.cu -- F2 in the reference's own layout.
//
// RAM holds the distribution as one array F2(NS,NR,NT,NE,NPA)
// (src/ModRamVariables.f90:31), the species index fastest; the moments
// PPERT/PPART as (NS,NR,NT).  The device keeps one contiguous block per
// (member, species) slot, so a transfer in the reference's layout is a
// transpose between "cell-major, species-minor" and "species-major".  Each
// CTA takes a tile of consecutive cells: the interleaved side (host or
// device memory) is read or written as one contiguous run, the slot side as
// NS contiguous runs, through shared memory.  When the host array is
// reachable from the device (page-locked and mapped, or pageable memory over
// a coherent host link) the kernels read or write it in place, so the
// transpose costs no pass of its own.
#include "ramgpu_internal.cuh"
#include "kernels.cuh"

namespace ramgpu {

constexpr int kLayoutTile = 256;  // cells per CTA tile (= threads per CTA)

// slots[s*stride + c] = ref[c*ns + s] for cells c in [c0, c1)
__global__ void __launch_bounds__(kLayoutTile) k_ref_gather(const double* __restrict__ ref, double* __restrict__ slots,
                                                            int ns, long long stride, long long c0, long long c1) {
  extern __shared__ double tile[];
  for (long long b = c0 + (long long)blockIdx.x * kLayoutTile; b < c1; b += (long long)gridDim.x * kLayoutTile) {
    const int nc = (int)min((long long)kLayoutTile, c1 - b);
    const double* src = ref + b * ns;
    for (int e = threadIdx.x; e < nc * ns; e += kLayoutTile) tile[e] = src[e];
    __syncthreads();
    if (threadIdx.x < nc)
      for (int s = 0; s < ns; ++s) slots[s * stride + b + threadIdx.x] = tile[threadIdx.x * ns + s];
    __syncthreads();
  }
}

// ref[c*ns + s] = slots[s*stride + c] for cells c in [c0, c1)
__global__ void __launch_bounds__(kLayoutTile) k_ref_scatter(const double* __restrict__ slots, double* __restrict__ ref,
                                                             int ns, long long stride, long long c0, long long c1) {
  extern __shared__ double tile[];
  for (long long b = c0 + (long long)blockIdx.x * kLayoutTile; b < c1; b += (long long)gridDim.x * kLayoutTile) {
    const int nc = (int)min((long long)kLayoutTile, c1 - b);
    if (threadIdx.x < nc)
      for (int s = 0; s < ns; ++s) tile[threadIdx.x * ns + s] = slots[s * stride + b + threadIdx.x];
    __syncthreads();
    double* dst = ref + b * ns;
    for (int e = threadIdx.x; e < nc * ns; e += kLayoutTile) dst[e] = tile[e];
    __syncthreads();
  }
}

// The host link, not the SMs, limits these copies when one side is host
// memory; a grid of one CTA per SM keeps enough loads in flight.
static int layout_grid(long long ncells, int nsm) {
  const long long tiles = (ncells + kLayoutTile - 1) / kLayoutTile;
  return (int)std::max(1LL, std::min(tiles, (long long)nsm * 2));
}

void launch_ref_gather(const double* ref, double* slots, int ns, long long stride, long long c0, long long c1,
                       int nsm, cudaStream_t st) {
  if (c1 <= c0) return;
  k_ref_gather<<<layout_grid(c1 - c0, nsm), kLayoutTile, kLayoutTile * ns * sizeof(double), st>>>(ref, slots, ns,
                                                                                                  stride, c0, c1);
}

void launch_ref_scatter(const double* slots, double* ref, int ns, long long stride, long long c0, long long c1,
                        int nsm, cudaStream_t st) {
  if (c1 <= c0) return;
  k_ref_scatter<<<layout_grid(c1 - c0, nsm), kLayoutTile, kLayoutTile * ns * sizeof(double), st>>>(slots, ref, ns,
                                                                                                   stride, c0, c1);
}

}  // namespace ramgpu
