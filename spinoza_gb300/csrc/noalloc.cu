// spz_xyz_expectation_value_noalloc: <X>, <Y> or <Z> per target without any
// device allocation, for callers that cannot call cudaMalloc — code running
// inside another framework's memory pool or arena, whose accounting a stray
// cudaMalloc would bypass, or in a process whose memory budget is fixed up
// front.
//
// The reduction's scratch (block partials and one result slot per target)
// lives in the file-scope array below, 10 KiB per GPU that loads the library,
// held until the process exits.  Its device address is looked up once per
// device (cudaGetSymbolAddress, with that device current) on the first call
// made on that device, and kept for the life of the process: make that first
// call before any stream capture, and make no call on a device after
// cudaDeviceReset, which would leave the kept address stale.  Every call
// shares the one array, so calls that overlap on the GPU (on different
// streams or host threads) race with each other and must be serialised by the
// caller.  The block partials are fully rewritten by each call and each slot
// is written before it is read, so nothing needs clearing.  The call ends by
// copying the results to `out` and synchronising the stream.
#include <algorithm>
#include <mutex>

#include "common.cuh"

namespace spz {
namespace {

constexpr int kNaThreads = 256;
constexpr int kNaMaxBlocks = kNumSMs * 8;  // 1216 partials
constexpr int kNaDoubles = kNaMaxBlocks + SPZ_NOALLOC_MAX_TARGETS;
constexpr int kNaMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNaDoubles];

std::mutex g_na_mutex;
double* g_na_ptr[kNaMaxDevices] = {};

__device__ __forceinline__ double na_block_sum(double v, double* smem) {
  for (int off = 16; off > 0; off >>= 1) v = dadd(v, __shfl_down_sync(0xffffffffu, v, off));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) smem[warp] = v;
  __syncthreads();
  double r = 0.0;
  if (warp == 0) {
    r = lane < (int)(blockDim.x >> 5) ? smem[lane] : 0.0;
    for (int off = 16; off > 0; off >>= 1) r = dadd(r, __shfl_down_sync(0xffffffffu, r, off));
  }
  __syncthreads();
  return r;
}

// Per-pair Re<psi|P_t|psi>: X 2(ac+bd), Y 2(ad-bc), Z |s0|^2-|s1|^2.
template <char OBS>
__global__ void __launch_bounds__(kNaThreads) na_pauli_kernel(const double* __restrict__ re,
                                                              const double* __restrict__ im, uint64_t nwork,
                                                              int t, double* __restrict__ partials) {
  __shared__ double smem[32];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t tbit = 1ull << t, lowmask = tbit - 1;
  double acc = 0.0;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwork; w += stride) {
    const uint64_t s0 = ((w & ~lowmask) << 1) | (w & lowmask);
    const uint64_t s1 = s0 | tbit;
    const double a = re[s0], b = im[s0], c = re[s1], d = im[s1];
    if (OBS == 'x') acc = dadd(acc, dmul(2.0, dfma(a, c, dmul(b, d))));
    else if (OBS == 'y') acc = dadd(acc, dmul(2.0, dfma(a, d, dmul(dneg(b), c))));
    else acc = dadd(acc, dsub(dfma(a, a, dmul(b, b)), dfma(c, c, dmul(d, d))));
  }
  const double s = na_block_sum(acc, smem);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void na_finalize_kernel(const double* __restrict__ partials, int nblocks, double* __restrict__ slot) {
  __shared__ double smem[32];
  double v = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) v = dadd(v, partials[b]);
  v = na_block_sum(v, smem);
  if (threadIdx.x == 0) *slot = v;
}

// Device address of g_noalloc_scratch on the current device (set up once).
int scratch_address(double** out) {
  int dev = 0;
  SPZ_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNaMaxDevices) return fail(SPZ_ERR_UNSUPPORTED, "device index beyond 63");
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_ptr[dev]) {
    double* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_na_ptr[dev] = p;
  }
  *out = g_na_ptr[dev];
  return SPZ_OK;
}

}  // namespace
}  // namespace spz

using namespace spz;

extern "C" int spz_xyz_expectation_value_noalloc(const double* d_reals, const double* d_imags, uint32_t n,
                                                 char observable, const uint32_t* targets, uint32_t ntargets,
                                                 double* out, void* stream) {
  if (!d_reals || !d_imags || (ntargets && (!targets || !out))) return fail(SPZ_ERR_NULL, "NULL argument");
  if (n == 0 || n > kMaxQubits) return fail(SPZ_ERR_INVALID_ARGUMENT, "n must be in 1..SPZ_MAX_QUBITS");
  if (ntargets > SPZ_NOALLOC_MAX_TARGETS)
    return fail(SPZ_ERR_INVALID_ARGUMENT,
                "ntargets exceeds SPZ_NOALLOC_MAX_TARGETS (64): the static scratch holds 64 result slots");
  if (observable != 'x' && observable != 'y' && observable != 'z')
    return fail(SPZ_ERR_INVALID_ARGUMENT, "observable must be 'x', 'y' or 'z'");
  for (uint32_t i = 0; i < ntargets; ++i)
    if (targets[i] >= n) return fail(SPZ_ERR_INVALID_ARGUMENT, "target qubit out of range");
  if (ntargets == 0) return SPZ_OK;
  double* scratch;
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  double* partials = scratch;
  double* slots = scratch + kNaMaxBlocks;
  cudaStream_t s = (cudaStream_t)stream;
  const uint64_t nwork = (1ull << n) / 2;
  const int blocks = std::min<int>(grid_for(nwork, kNaThreads, 8), kNaMaxBlocks);
  for (uint32_t i = 0; i < ntargets; ++i) {
    const int t = (int)targets[i];
    switch (observable) {
      case 'x': na_pauli_kernel<'x'><<<blocks, kNaThreads, 0, s>>>(d_reals, d_imags, nwork, t, partials); break;
      case 'y': na_pauli_kernel<'y'><<<blocks, kNaThreads, 0, s>>>(d_reals, d_imags, nwork, t, partials); break;
      default: na_pauli_kernel<'z'><<<blocks, kNaThreads, 0, s>>>(d_reals, d_imags, nwork, t, partials); break;
    }
    na_finalize_kernel<<<1, 1024, 0, s>>>(partials, blocks, slots + i);
    SPZ_CHECK_LAUNCH("na_pauli_kernel");
  }
  SPZ_CUDA(cudaMemcpyAsync(out, slots, ntargets * sizeof(double), cudaMemcpyDefault, s));
  SPZ_CUDA(cudaStreamSynchronize(s));
  return SPZ_OK;
}
