// mge_noalloc.cu -- residual norm of euler.f90:431-447 for callers that
// cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: a Fortran or C host
// that runs inside a CUDA stream capture it does not own, or one whose device
// memory is handed out by its own pool and may not grow behind its back.  For
// them mge_residual_norm_noalloc computes rtrms from device arrays the caller
// already holds and allocates nothing.  Its partial sums live in the
// file-scope array below, which every GPU that loads the library holds until
// the process exits (32 KiB).  The kernels are the same two-pass,
// fixed-order reduction the cycle uses, so the result equals the one
// mge_get_rtrms reports for the same fields.
#include <mutex>

#include "../../include/mge_gpu.h"

namespace {

constexpr int kThreads = 256;
constexpr int kCellsPerPartial = kThreads * 8;
constexpr int kMaxPartials = 4096;  // capacity of the static scratch
constexpr long long kMaxCells = (long long)kMaxPartials * kCellsPerPartial;

// Partial sums of the last call.  Every call overwrites the entries it uses
// before reading them, so nothing needs clearing; calls that overlap on the
// GPU (two streams, or two host threads) race on it.
static __device__ __align__(256) double g_rtrms_partials[kMaxPartials];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// Device address of g_rtrms_partials per device, as last looked up outside a
// stream capture.  A call inside a capture cannot look it up and reuses this.
double* g_scratch[kMaxDevices] = {nullptr};

// The device address of the static scratch on the current device.  Outside a
// capture it is looked up on every call: after cudaDeviceReset, or after the
// primary context is destroyed and made again, the module loads anew and the
// array may sit elsewhere.  Inside a capture the address of the last call
// made outside one is used (none yet: an error).
int scratch_address(int dev, cudaStream_t s, double** out) {
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) return MGE_ECUDA;
  std::lock_guard<std::mutex> lk(g_mu);
  if (cap == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_rtrms_partials) != cudaSuccess) return MGE_ECUDA;
    g_scratch[dev] = (double*)p;
  } else if (!g_scratch[dev]) {
    return MGE_EBADCFG;  // first call on this device made inside a capture
  }
  *out = g_scratch[dev];
  return MGE_OK;
}

__global__ void k_noalloc_partial(const double* __restrict__ dw, const double* __restrict__ vdtim,
                                  const int32_t* __restrict__ blank, int nx, int ny, int nz, double cfl, int vt,
                                  double dtim, double* partial, int npart) {
  __shared__ double sh[kThreads];
  const long long Pi = nx + 4, Pj = ny + 4;
  const long long tot = (long long)nx * ny * nz;
  const long long per = (tot + npart - 1) / npart;
  const long long lo = (long long)blockIdx.x * per, hi = min(tot, lo + per);
  double acc = 0.0;
  for (long long t = lo + threadIdx.x; t < hi; t += blockDim.x) {
    long long i = 2 + t % nx, j = 2 + (t / nx) % ny, k = 2 + t / ((long long)nx * ny);
    long long c = i + Pi * (j + Pj * k);
    double de = cfl * (vt ? dtim : vdtim[c]);
    double rt = 0.0;
    if (blank[c] != 0) rt = dw[c] / de;
    acc = acc + rt * rt;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] = sh[threadIdx.x] + sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// one warp: lane l adds partials l, l+32, ... in turn, then a fixed halving
// tree over the lanes (the order the cycle's own norm uses)
__global__ void k_noalloc_final(const double* partial, int npart, double ncell, double* out) {
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  double a = 0.0;
  for (int q = lane; q < npart; q += 32) a = a + partial[q];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a = a + __shfl_down_sync(0xffffffffu, a, o);
  if (lane == 0) *out = sqrt(a / ncell);
}

}  // namespace

extern "C" int mge_residual_norm_noalloc(const double* dw_rho, const double* vdtim, const int32_t* blank, int nx,
                                         int ny, int nz, double cfl, int vt, double dtim, double* norm_out,
                                         void* stream) {
  if (!dw_rho || !vdtim || !blank || !norm_out || nx < 1 || ny < 1 || nz < 1) return MGE_EBADCFG;
  const long long ncell = (long long)nx * ny * nz;
  if (ncell > kMaxCells) return MGE_EBADCFG;  // more partial sums than the static scratch holds
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MGE_ECUDA;
  // an error left pending by earlier work is not this call's: report it
  // without clearing it, and launch nothing
  if (cudaPeekAtLastError() != cudaSuccess) return MGE_ECUDA;
  cudaStream_t s = (cudaStream_t)stream;
  double* scratch = nullptr;
  const int rc = scratch_address(dev, s, &scratch);
  if (rc != MGE_OK) return rc;
  int npart = (int)((ncell + kCellsPerPartial - 1) / kCellsPerPartial);
  if (npart < 1) npart = 1;
  k_noalloc_partial<<<npart, kThreads, 0, s>>>(dw_rho, vdtim, blank, nx, ny, nz, cfl, vt, dtim, scratch, npart);
  if (cudaGetLastError() != cudaSuccess) return MGE_ECUDA;
  k_noalloc_final<<<1, 32, 0, s>>>(scratch, npart, (double)ncell, norm_out);
  if (cudaGetLastError() != cudaSuccess) return MGE_ECUDA;
  return MGE_OK;
}
