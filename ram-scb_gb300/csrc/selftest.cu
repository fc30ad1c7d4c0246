// selftest.cu -- device self-test of the integer-pipe arithmetic helpers
// against the FP64 unit, on random operands: full random significands,
// significands with only their top bits set (exact products and ties to
// even), zeros, subnormals, infinities and extreme exponents.
#include "kernels.cuh"

namespace ramgpu {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// A random double whose class depends on the hash: mostly normal numbers
// around 1e-40..1e40, some with short significands, a few specials.
__device__ __forceinline__ double test_operand(unsigned long long h, unsigned long long h2) {
  const int kind = (int)(h2 % 64);
  unsigned long long sign = (h2 >> 8) & 1ULL;
  unsigned long long mant = h & kMantMask;
  int e = 1023 + (int)((h2 >> 16) % 260) - 130;
  if (kind < 16) mant &= ~((1ULL << (52 - (int)((h2 >> 32) % 30))) - 1);  // short significand
  if (kind == 60) e = 0, mant = 0;                                        // zero
  if (kind == 61) e = 0;                                                  // subnormal
  if (kind == 62) e = 0x7FF, mant = (h2 >> 40) & 1 ? mant : 0;           // inf or NaN
  if (kind == 63) e = (h2 >> 40) & 1 ? 1 : 2046;                          // extreme exponents
  return bitsd((sign << 63) | ((unsigned long long)e << 52) | mant);
}

__global__ void k_selftest_mul(long long n, unsigned long long seed, unsigned long long* bad) {
  unsigned long long nbad = 0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const double a = test_operand(mix64(seed ^ (2 * t)), mix64(seed + 3 * t));
    const double b = test_operand(mix64(seed ^ (2 * t + 1)), mix64(seed + 3 * t + 1));
    const double r = mul_rn_int(a, b), h = a * b;
    const bool same = dbits(r) == dbits(h) || (r != r && h != h);
    nbad += same ? 0 : 1;
  }
  if (nbad) atomicAdd(bad, nbad);
}

void launch_selftest_mul(long long n, unsigned long long seed, unsigned long long* bad, cudaStream_t st) {
  k_selftest_mul<<<608, 256, 0, st>>>(n, seed, bad);
}

}  // namespace ramgpu
