// diag.cuh -- diagnostic reductions over F2 (status.cu).
#pragma once

#include "ramgpu_internal.cuh"

namespace ramgpu {

// F2 statistics of one slot: kF2StatBlocks partial content sums into part,
// the order keys of the smallest and largest F2 into mm[0] and mm[1]
// (f2_stats_key_value turns a key back into the value).
constexpr int kF2StatBlocks = 256;
void launch_f2_stats(const Dev& d, long long slot, double* part, unsigned long long* mm, cudaStream_t s);
double f2_stats_key_value(unsigned long long key);

}  // namespace ramgpu
