// State handles: allocation, wrapping of caller memory, host<->device copies,
// reset, clone and seeded synthetic fills.  Replaces State::new / Clone and the
// public reals/imags fields of spinoza/src/core.rs:18-51.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "common.cuh"

namespace spz {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  set_error(msg);
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  set_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? SPZ_ERR_OUT_OF_MEMORY : SPZ_ERR_CUDA;
}

namespace {
bool alloc_failure_injected() {
  const char* v = std::getenv("SPZ_INJECT_ALLOC_FAILURE");
  return v && v[0] == '1' && v[1] == 0;
}
}  // namespace

cudaError_t dev_alloc(void** p, size_t bytes) {
  if (alloc_failure_injected()) return cudaErrorMemoryAllocation;
  return cudaMalloc(p, bytes);
}

cudaError_t host_alloc(void** p, size_t bytes) {
  if (alloc_failure_injected()) return cudaErrorMemoryAllocation;
  return cudaMallocHost(p, bytes);
}

// The copy direction for a caller's buffer `p` moving into (to_device) or out
// of the state: explicit host<->device kinds for host memory, pinned or not.
// On systems where the GPU also reads host page tables, cudaMemcpyDefault on a
// host pointer was measured at 47 GB/s for a 16 GiB pinned buffer that the
// explicit kind moves at 211 GB/s (GB300).
cudaMemcpyKind copy_kind(const void* p, bool to_device) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the sticky error of an unknown pointer: treat it as host memory
    return to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
  }
  if (a.type == cudaMemoryTypeDevice) return cudaMemcpyDeviceToDevice;
  if (a.type == cudaMemoryTypeManaged) return cudaMemcpyDefault;
  return to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost;
}

int grid_for(uint64_t work, int threads, int per_sm) {
  uint64_t blocks = (work + threads - 1) / threads;
  uint64_t cap = (uint64_t)kNumSMs * per_sm;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

int ensure_dev_scratch(spz_state_t h, size_t bytes, void** out) {
  if (h->dev_scratch.bytes < bytes) {
    if (h->dev_scratch.ptr) {
      SPZ_CUDA(cudaStreamSynchronize(h->stream));
      SPZ_CUDA(cudaFree(h->dev_scratch.ptr));
      h->dev_scratch.ptr = nullptr;
      h->dev_scratch.bytes = 0;
    }
    size_t sz = bytes < 4096 ? 4096 : bytes;
    SPZ_CUDA(dev_alloc(&h->dev_scratch.ptr, sz));
    h->dev_scratch.bytes = sz;
  }
  *out = h->dev_scratch.ptr;
  return SPZ_OK;
}

int ensure_host_scratch(spz_state_t h, size_t bytes, void** out) {
  if (h->host_scratch.bytes < bytes) {
    if (h->host_scratch.ptr) {
      SPZ_CUDA(cudaStreamSynchronize(h->stream));
      SPZ_CUDA(cudaFreeHost(h->host_scratch.ptr));
      h->host_scratch.ptr = nullptr;
      h->host_scratch.bytes = 0;
    }
    size_t sz = bytes < 4096 ? 4096 : bytes;
    SPZ_CUDA(host_alloc(&h->host_scratch.ptr, sz));
    h->host_scratch.bytes = sz;
  }
  *out = h->host_scratch.ptr;
  return SPZ_OK;
}

// ------------------------------------------------------------ kernels
__global__ void zero_state_kernel(double* __restrict__ re, double* __restrict__ im, uint64_t N) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N; i += stride) {
    re[i] = i == 0 ? 1.0 : 0.0;
    im[i] = 0.0;
  }
}

// Counter-based splitmix64 stream: u64(seed, i) = mix(mix(seed + G) + (i+1) G).
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;

__device__ __forceinline__ double stream_uniform(uint64_t key, uint64_t i) {
  return (double)(mix64(key + (i + 1) * kGolden) >> 11) * 0x1.0p-53;
}

// dist 0: uniform [-1,1) (exact, bit-reproducible on the host);
// dist 1: N(0,1) via Box-Muller on the pair (u(2i), u(2i+1)).
__global__ void fill_kernel(double* __restrict__ re, double* __restrict__ im, uint64_t N, uint64_t key,
                            int dist) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N; i += stride) {
    double u1 = stream_uniform(key, 2 * i), u2 = stream_uniform(key, 2 * i + 1);
    if (dist == 0) {
      re[i] = dadd(dmul(2.0, u1), -1.0);
      im[i] = dadd(dmul(2.0, u2), -1.0);
    } else {
      double r = sqrt(-2.0 * log(1.0 - u1));
      double s, c;
      sincospi(2.0 * u2, &s, &c);
      re[i] = r * c;
      im[i] = r * s;
    }
  }
}

__global__ void scale_kernel(double* __restrict__ re, double* __restrict__ im, uint64_t N,
                             const double* __restrict__ scale_ptr) {
  const double s = *scale_ptr;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < N; i += stride) {
    re[i] = dmul(re[i], s);
    im[i] = dmul(im[i], s);
  }
}

__global__ void rsqrt_kernel(double* p) { p[1] = 1.0 / sqrt(p[0]); }

// Multiply every amplitude by the complex factor (fr, fi); a real factor
// (fi == 0) costs one multiply per number.  Two amplitudes per thread
// (double2 loads), so the pass is bound by HBM.
__global__ void __launch_bounds__(kThreads) factor_kernel(double* __restrict__ re, double* __restrict__ im,
                                                          uint64_t npairs, double fr, double fi) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < npairs; w += stride) {
    double2 r = reinterpret_cast<const double2*>(re)[w];
    double2 i = reinterpret_cast<const double2*>(im)[w];
    if (fi == 0.0) {
      r.x = dmul(r.x, fr); r.y = dmul(r.y, fr);
      i.x = dmul(i.x, fr); i.y = dmul(i.y, fr);
    } else {
      const double ax = r.x, bx = i.x, ay = r.y, by = i.y;
      r.x = dfma(ax, fr, dmul(dneg(bx), fi)); i.x = dfma(ax, fi, dmul(bx, fr));
      r.y = dfma(ay, fr, dmul(dneg(by), fi)); i.y = dfma(ay, fi, dmul(by, fr));
    }
    reinterpret_cast<double2*>(re)[w] = r;
    reinterpret_cast<double2*>(im)[w] = i;
  }
}

void clear_factor(spz_state_t h) {
  h->factor_re = 1.0;
  h->factor_im = 0.0;
  h->factor_exp = 0;
}

int settle(spz_state_t h) {
  if (h->factor_re == 1.0 && h->factor_im == 0.0 && h->factor_exp == 0) return SPZ_OK;
  const double fr = std::ldexp(h->factor_re, h->factor_exp), fi = std::ldexp(h->factor_im, h->factor_exp);
  clear_factor(h);
  if (h->N >= 2) {
    factor_kernel<<<grid_for(h->N / 2), kThreads, 0, h->stream>>>(h->re, h->im, h->N / 2, fr, fi);
  } else {
    return fail(SPZ_ERR_INVALID_ARGUMENT, "state too small");
  }
  SPZ_CHECK_LAUNCH("factor_kernel");
  return SPZ_OK;
}

// The arrays hold the state divided by the factor; a lazy gate that applies
// (its matrix / f) multiplies the factor by f.  The factor is kept as
// mantissa x 2^exp; once the arrays have grown by 2^400 (each lazy gate grows
// them by at most sqrt 2) the factor is folded in, so they never overflow.
int scale_factor(spz_state_t h, double f_re, double f_im) {
  const double r = h->factor_re * f_re - h->factor_im * f_im;
  const double i = h->factor_re * f_im + h->factor_im * f_re;
  int e = 0;
  const double mag = std::max(std::fabs(r), std::fabs(i));
  if (mag == 0.0) return fail(SPZ_ERR_INVALID_ARGUMENT, "zero lazy factor");
  std::frexp(mag, &e);
  h->factor_re = std::ldexp(r, -e);
  h->factor_im = std::ldexp(i, -e);
  h->factor_exp += e;
  if (h->factor_exp < -400 || h->factor_exp > 400) return settle(h);
  return SPZ_OK;
}

int norm_sqr_to_device(spz_state_t h, double* d_out);  // reduce.cu

}  // namespace spz

using namespace spz;

// ================================================================== C ABI
extern "C" {

const char* spz_last_error(void) { return g_last_error.c_str(); }

const char* spz_version(void) { return "spinoza_gb300 0.1.0 sm_103a"; }

static int alloc_handle(uint32_t n, spz_state_t* out) {
  if (!out) return fail(SPZ_ERR_NULL, "out is NULL");
  if (n == 0) return fail(SPZ_ERR_INVALID_ARGUMENT, "n must be > 0 (core.rs:33 asserts n > 0)");
  if (n > kMaxQubits) return fail(SPZ_ERR_INVALID_ARGUMENT, "n exceeds SPZ_MAX_QUBITS");
  spz_state_t h = new (std::nothrow) spz_state_s();
  if (!h) return fail(SPZ_ERR_OUT_OF_MEMORY, "host allocation of handle failed");
  h->n = n;
  h->N = 1ull << n;
  cudaError_t e = cudaGetDevice(&h->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(e, "stream creation");
  }
  h->stream = h->own_stream;
  *out = h;
  return SPZ_OK;
}

int spz_state_create(uint32_t n, spz_state_t* out) {
  int rc = alloc_handle(n, out);
  if (rc) return rc;
  spz_state_t h = *out;
  cudaError_t e = dev_alloc(&h->re, h->N * sizeof(double));
  if (e == cudaSuccess) e = dev_alloc(&h->im, h->N * sizeof(double));
  if (e != cudaSuccess) {
    if (h->re) cudaFree(h->re);
    cudaStreamDestroy(h->own_stream);
    delete h;
    *out = nullptr;
    return cuda_fail(e, "cudaMalloc of the state");
  }
  h->owns = true;
  rc = spz_state_reset_zero(h);
  if (rc) {
    spz_state_destroy(h);
    *out = nullptr;
  }
  return rc;
}

int spz_state_wrap(uint32_t n, double* d_reals, double* d_imags, spz_state_t* out) {
  if (!d_reals || !d_imags) return fail(SPZ_ERR_NULL, "device arrays are NULL");
  if (((uintptr_t)d_reals & 15) || ((uintptr_t)d_imags & 15))
    return fail(SPZ_ERR_INVALID_ARGUMENT, "device arrays must be 16-byte aligned");
  int rc = alloc_handle(n, out);
  if (rc) return rc;
  (*out)->re = d_reals;
  (*out)->im = d_imags;
  (*out)->owns = false;
  return SPZ_OK;
}

int spz_state_destroy(spz_state_t h) {
  if (!h) return SPZ_OK;
  cudaStreamSynchronize(h->stream);
  if (h->owns) {
    cudaFree(h->re);
    cudaFree(h->im);
  }
  for (int j = 0; j < 2; ++j) {
    if (h->aux_re[j]) cudaFree(h->aux_re[j]);
    if (h->aux_im[j]) cudaFree(h->aux_im[j]);
  }
  if (h->dev_scratch.ptr) cudaFree(h->dev_scratch.ptr);
  if (h->host_scratch.ptr) cudaFreeHost(h->host_scratch.ptr);
  if (h->copy_stream) {
    cudaStreamSynchronize(h->copy_stream);
    cudaStreamDestroy(h->copy_stream);
  }
  if (h->meas) cudaFree(h->meas);
  if (h->tma_err) cudaFree(h->tma_err);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
  return SPZ_OK;
}

int spz_state_set_stream(spz_state_t h, void* stream) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return SPZ_OK;
}

int spz_state_synchronize(spz_state_t h) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  SPZ_CUDA(cudaStreamSynchronize(h->stream));
  return SPZ_OK;
}

int spz_state_num_qubits(spz_state_t h, uint32_t* n) {
  if (!h || !n) return fail(SPZ_ERR_NULL, "NULL argument");
  *n = h->n;
  return SPZ_OK;
}

int spz_state_device_arrays(spz_state_t h, double** d_reals, double** d_imags) {
  if (!h || !d_reals || !d_imags) return fail(SPZ_ERR_NULL, "NULL argument");
  int rc = settle(h);  // the caller reads the arrays directly
  if (rc) return rc;
  *d_reals = h->re;
  *d_imags = h->im;
  return SPZ_OK;
}

int spz_state_upload(spz_state_t h, const double* reals, const double* imags) {
  if (!h || !reals || !imags) return fail(SPZ_ERR_NULL, "NULL argument");
  clear_factor(h);
  const cudaMemcpyKind kind = copy_kind(reals, true);
  SPZ_CUDA(cudaMemcpyAsync(h->re, reals, h->N * sizeof(double), kind, h->stream));
  SPZ_CUDA(cudaMemcpyAsync(h->im, imags, h->N * sizeof(double), kind, h->stream));
  SPZ_CUDA(cudaStreamSynchronize(h->stream));
  return SPZ_OK;
}

int spz_state_download(spz_state_t h, double* reals, double* imags) {
  if (!h || !reals || !imags) return fail(SPZ_ERR_NULL, "NULL argument");
  int rc = settle(h);
  if (rc) return rc;
  const cudaMemcpyKind kind = copy_kind(reals, false);
  SPZ_CUDA(cudaMemcpyAsync(reals, h->re, h->N * sizeof(double), kind, h->stream));
  SPZ_CUDA(cudaMemcpyAsync(imags, h->im, h->N * sizeof(double), kind, h->stream));
  SPZ_CUDA(cudaStreamSynchronize(h->stream));
  return SPZ_OK;
}

int spz_state_reset_zero(spz_state_t h) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  clear_factor(h);
  zero_state_kernel<<<grid_for(h->N), kThreads, 0, h->stream>>>(h->re, h->im, h->N);
  SPZ_CHECK_LAUNCH("zero_state_kernel");
  return SPZ_OK;
}

int spz_state_copy(spz_state_t dst, spz_state_t src) {
  if (!dst || !src) return fail(SPZ_ERR_NULL, "handle is NULL");
  if (dst->n != src->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "qubit counts differ");
  if (dst == src) return SPZ_OK;
  int rc = settle(src);
  if (rc) return rc;
  clear_factor(dst);
  // Order after src's pending work, then run on dst's stream.
  cudaEvent_t ev;
  SPZ_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  SPZ_CUDA(cudaEventRecord(ev, src->stream));
  SPZ_CUDA(cudaStreamWaitEvent(dst->stream, ev, 0));
  SPZ_CUDA(cudaEventDestroy(ev));
  SPZ_CUDA(cudaMemcpyAsync(dst->re, src->re, dst->N * sizeof(double), cudaMemcpyDeviceToDevice, dst->stream));
  SPZ_CUDA(cudaMemcpyAsync(dst->im, src->im, dst->N * sizeof(double), cudaMemcpyDeviceToDevice, dst->stream));
  return SPZ_OK;
}

int spz_state_fill_random(spz_state_t h, uint64_t seed, int dist, int normalise) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  if (dist != 0 && dist != 1) return fail(SPZ_ERR_INVALID_ARGUMENT, "dist must be 0 or 1");
  clear_factor(h);
  const uint64_t key = mix64(seed + kGolden);
  fill_kernel<<<grid_for(h->N), kThreads, 0, h->stream>>>(h->re, h->im, h->N, key, dist);
  SPZ_CHECK_LAUNCH("fill_kernel");
  if (normalise) {
    void* scratch;
    int rc = ensure_dev_scratch(h, 64 * 1024 * sizeof(double), &scratch);
    if (rc) return rc;
    // norm_sqr_to_device writes the sum to the last two slots of scratch
    double* slot = (double*)scratch + 64 * 1024 - 2;
    rc = norm_sqr_to_device(h, slot);
    if (rc) return rc;
    rsqrt_kernel<<<1, 1, 0, h->stream>>>(slot);
    scale_kernel<<<grid_for(h->N), kThreads, 0, h->stream>>>(h->re, h->im, h->N, slot + 1);
    SPZ_CHECK_LAUNCH("scale_kernel");
  }
  return SPZ_OK;
}

int spz_state_set_lazy(spz_state_t h, int enable) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  h->lazy = enable != 0;
  return h->lazy ? SPZ_OK : settle(h);
}

int spz_state_set_tile(spz_state_t h, int tile_qubits, int threads) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  if (tile_qubits != 0 && (tile_qubits < 4 || tile_qubits > 10))
    return fail(SPZ_ERR_INVALID_ARGUMENT, "tile_qubits must be 0 or in 4..10");
  if (threads != 0 && threads != 32 && threads != 64)
    return fail(SPZ_ERR_INVALID_ARGUMENT, "threads must be 0, 32 or 64");
  h->tile_k = tile_qubits;
  h->tile_threads = threads;
  return SPZ_OK;
}

int spz_state_settle(spz_state_t h) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  return settle(h);
}

}  // extern "C"
