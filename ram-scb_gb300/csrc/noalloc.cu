// noalloc.cu -- SUMRC energy content without any device allocation.
//
// Some callers of this library cannot allocate device memory: a host model
// that hands every device byte to its own pool and forbids libraries to call
// cudaMalloc (which can also synchronise the device and stall work already in
// flight), or code that must not call allocation APIs while another thread
// has a stream under capture.  ramgpu_sumrc_noalloc serves them: it computes
// SETRC = sum EKEV*F2*WE*WMU over I=2..NR, J=1..NT-1, K=2..NE, L=2..NPA
// (the sum of src/ModRamRun.f90:246-255) of one species' F2 that is already
// on the device, using as scratch only the fixed array below.
//
// The scratch is a file-scope __device__ array, so every GPU that loads this
// library holds it (kScratchDoubles doubles = 36 KiB) until the process exits.
// In host code the array's name is only a host-side stand-in for the symbol,
// not a device address; its device address is looked up once per device with
// cudaGetSymbolAddress, with that device current, by the first call of
// ramgpu_sumrc_noalloc on that device.  Make that first call before any
// stream capture.  The address is kept for the life of the process: after a
// cudaDeviceReset of that device the module is loaded again and the kept
// address is stale, so do not call this entry point after resetting the
// device.  All calls share the one array and it keeps the contents of the
// last call; calls that overlap on the GPU (from two host threads or two
// streams) race on it.  Every call is synchronous (it copies the grid
// vectors from host memory and waits for its stream), so it cannot be made
// while its stream is being captured: such a call returns RAMGPU_ERR_STATE
// and leaves the capture intact.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/ramgpu.h"
#include "kernels.cuh"

namespace {

constexpr int kMaxBlocks = 1024;            // partial sums (one per block)
constexpr int kMaxVec = 1024;               // maximum NE and NPA
// layout: [0, kMaxBlocks) partials | WE | WMU | EKEV | result (+ padding)
constexpr int kOffWe = kMaxBlocks;
constexpr int kOffWmu = kOffWe + kMaxVec;
constexpr int kOffEkev = kOffWmu + kMaxVec;
constexpr int kOffResult = kOffEkev + kMaxVec;
constexpr int kScratchDoubles = kOffResult + 512;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_dev[kMaxDevices] = {nullptr};  // device address per device

__global__ void k_sumrc_partials(const double* __restrict__ f2, int nr, int nt, int ne, int npa,
                                 double* __restrict__ scratch) {
  __shared__ double sh[256];
  const double* we = scratch + kOffWe;
  const double* wmu = scratch + kOffWmu;
  const double* ekev = scratch + kOffEkev;
  const long long ncell = (long long)nr * nt * ne * npa;
  double acc = 0.0;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < ncell;
       c += (long long)gridDim.x * blockDim.x) {
    const int I = 1 + (int)(c % nr);
    const int J = 1 + (int)((c / nr) % nt);
    const int K = 1 + (int)((c / ((long long)nr * nt)) % ne);
    const int L = 1 + (int)(c / ((long long)nr * nt * ne));
    if (I >= 2 && J <= nt - 1 && K >= 2 && L >= 2) {
      const double weight = f2[c] * we[K - 1] * wmu[L - 1];
      acc = acc + ekev[K - 1] * weight;
    }
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) scratch[blockIdx.x] = sh[0];  // every slot < gridDim.x is rewritten
}

// One thread adds the partials in block order (deterministic).
__global__ void k_sumrc_final(double* scratch, int nblk) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nblk; ++b) s += scratch[b];
  scratch[kOffResult] = s;
}

int scratch_for_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    ramgpu::set_thread_error("ramgpu_sumrc_noalloc: no current CUDA device");
    return RAMGPU_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    ramgpu::set_thread_error("ramgpu_sumrc_noalloc: device index " + std::to_string(dev) +
                             " beyond the 64 devices the address table holds");
    return RAMGPU_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_dev[dev]) {
    double* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      ramgpu::set_thread_error(std::string("ramgpu_sumrc_noalloc: cudaGetSymbolAddress of the scratch failed: ") +
                               cudaGetErrorString(e));
      return RAMGPU_ERR_CUDA;
    }
    g_scratch_dev[dev] = p;
  }
  *out = g_scratch_dev[dev];
  return RAMGPU_OK;
}

}  // namespace

extern "C" int ramgpu_sumrc_noalloc(const double* f2_dev, int nr, int nt, int ne, int npa,
                                    const double* we, const double* wmu, const double* ekev,
                                    void* stream, double* setrc) {
  if (!f2_dev || !we || !wmu || !ekev || !setrc) {
    ramgpu::set_thread_error("ramgpu_sumrc_noalloc: null argument");
    return RAMGPU_ERR_ARG;
  }
  if (nr < 2 || nt < 2 || ne < 2 || npa < 2) {
    ramgpu::set_thread_error("ramgpu_sumrc_noalloc: grid dimensions must be >= 2");
    return RAMGPU_ERR_ARG;
  }
  if (ne > kMaxVec || npa > kMaxVec) {
    ramgpu::set_thread_error("ramgpu_sumrc_noalloc: NE and NPA must be <= 1024 "
                             "(fixed scratch of the no-allocation path)");
    return RAMGPU_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    ramgpu::set_thread_error("ramgpu_sumrc_noalloc: the stream is being captured; this call synchronises its "
                             "stream and cannot be captured");
    return RAMGPU_ERR_STATE;
  }
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != RAMGPU_OK) return rc;
  cudaError_t e = cudaMemcpyAsync(scratch + kOffWe, we, sizeof(double) * ne, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(scratch + kOffWmu, wmu, sizeof(double) * npa, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(scratch + kOffEkev, ekev, sizeof(double) * ne, cudaMemcpyHostToDevice, st);
  const long long ncell = (long long)nr * nt * ne * npa;
  int nblk = (int)((ncell + 255) / 256);
  if (nblk > kMaxBlocks) nblk = kMaxBlocks;
  if (e == cudaSuccess) {
    k_sumrc_partials<<<nblk, 256, 0, st>>>(f2_dev, nr, nt, ne, npa, scratch);
    k_sumrc_final<<<1, 32, 0, st>>>(scratch, nblk);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(setrc, scratch + kOffResult, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    ramgpu::set_thread_error(std::string("ramgpu_sumrc_noalloc: ") + cudaGetErrorString(e));
    return RAMGPU_ERR_CUDA;
  }
  return RAMGPU_OK;
}
