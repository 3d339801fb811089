// Dense k-qubit unitaries: transform_u / c_transform_u (spinoza/src/gates.rs:1388-1487)
// and apply_unitary (spinoza/src/unitaries.rs).
//
// A 2^m x 2^m complex matrix U (row-major, separate real and imaginary arrays,
// as `Unitary { reals, imags, height, width }`) acts on qubits t .. t+m-1: for
// every assignment of the other bits (and, with a control, only where the
// control reads 1) the 2^m amplitudes with index prefix | (j << t) | suffix
// form a vector v and become U v.  Each output is accumulated in the
// reference's order (unitary_col_vec_mul, gates.rs:1388-1425):
//   re += a*v_re - b*v_im;  im += a*v_im + b*v_re   for j = 0 .. 2^m - 1.
// The reference's transform_u takes the state size from the matrix width
// (gates.rs:1430), so only a full-state matrix at t = 0 works there; here n is
// the state's, and any block fits.  A control inside the block is rejected
// (the reference would mix stale vector entries, gates.rs:1455-1487).
//
// One thread per output amplitude, reading its group's inputs from a copy of
// the state (the work vector of the handle); this is the reference's "last
// resort" path and is not fused.
#include "common.cuh"

namespace spz {

__global__ void unitary_kernel(const double* __restrict__ in_re, const double* __restrict__ in_im,
                               double* __restrict__ out_re, double* __restrict__ out_im,
                               const double* __restrict__ ur, const double* __restrict__ ui, int m, int t,
                               uint64_t nwork, uint8_t npos, const uint8_t* __restrict__ pos_g, uint64_t ones) {
  __shared__ uint8_t pos[kMaxQubits + 2];
  for (int j = threadIdx.x; j < npos; j += blockDim.x) pos[j] = pos_g[j];
  __syncthreads();
  const uint64_t M = 1ull << m, stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwork; w += stride) {
    const uint64_t g = w >> m, i = w & (M - 1);
    const uint64_t base = deposit(g, pos, npos) | ones;
    double re = 0.0, im = 0.0;
    for (uint64_t j = 0; j < M; ++j) {
      const double a = ur[i * M + j], b = ui[i * M + j];
      const uint64_t k = base | (j << t);
      const double sr = in_re[k], si = in_im[k];
      re = dadd(re, dsub(dmul(a, sr), dmul(b, si)));
      im = dadd(im, dadd(dmul(a, si), dmul(b, sr)));
    }
    const uint64_t k = base | (i << t);
    out_re[k] = re;
    out_im[k] = im;
  }
}

int apply_unitary(spz_state_t h, const double* u_re, const double* u_im, uint32_t m, uint32_t t, int32_t control) {
  if (!u_re || !u_im) return fail(SPZ_ERR_NULL, "matrix is NULL");
  if (m == 0 || m > 12) return fail(SPZ_ERR_INVALID_ARGUMENT, "unitary must act on 1..12 qubits");
  if (t + m > h->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "unitary block exceeds the state");
  if (control >= 0 && ((uint32_t)control >= h->n || ((uint32_t)control >= t && (uint32_t)control < t + m)))
    return fail(SPZ_ERR_INVALID_ARGUMENT, "control must be a qubit outside the unitary's block");
  if (!h->aux_re[0]) {
    SPZ_CUDA(dev_alloc(&h->aux_re[0], h->N * sizeof(double)));
    cudaError_t e = dev_alloc(&h->aux_im[0], h->N * sizeof(double));
    if (e != cudaSuccess) {
      cudaFree(h->aux_re[0]);
      h->aux_re[0] = nullptr;
      return cuda_fail(e, "cudaMalloc of the unitary work vector");
    }
  }
  const uint64_t M = 1ull << m;
  uint64_t special = ((M - 1) << t);
  uint64_t ones = 0;
  if (control >= 0) {
    special |= 1ull << control;
    ones = 1ull << control;
  }
  std::vector<uint8_t> pos;
  for (int q = 0; q < 64; ++q)
    if ((special >> q) & 1) pos.push_back((uint8_t)q);
  const uint64_t groups = h->N >> pos.size();
  const uint64_t nwork = groups * M;
  void* scratch;
  const size_t mat = M * M * sizeof(double);
  int rc = ensure_dev_scratch(h, 2 * mat + 256, &scratch);
  if (rc) return rc;
  double* dur = (double*)scratch;
  double* dui = dur + M * M;
  uint8_t* dpos = (uint8_t*)(dui + M * M);
  SPZ_CUDA(cudaMemcpyAsync(dur, u_re, mat, cudaMemcpyDefault, h->stream));
  SPZ_CUDA(cudaMemcpyAsync(dui, u_im, mat, cudaMemcpyDefault, h->stream));
  SPZ_CUDA(cudaMemcpyAsync(dpos, pos.data(), pos.size(), cudaMemcpyHostToDevice, h->stream));
  SPZ_CUDA(cudaMemcpyAsync(h->aux_re[0], h->re, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  SPZ_CUDA(cudaMemcpyAsync(h->aux_im[0], h->im, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  unitary_kernel<<<grid_for(nwork), kThreads, 0, h->stream>>>(h->aux_re[0], h->aux_im[0], h->re, h->im, dur, dui,
                                                                (int)m, (int)t, nwork, (uint8_t)pos.size(), dpos,
                                                                ones);
  SPZ_CHECK_LAUNCH("unitary_kernel");
  // The matrix copies above are from caller memory; keep it valid until done.
  SPZ_CUDA(cudaStreamSynchronize(h->stream));
  return SPZ_OK;
}

}  // namespace spz

extern "C" int spz_apply_unitary(spz_state_t h, const double* u_reals, const double* u_imags, uint32_t m,
                                 uint32_t target, int32_t control) {
  if (!h) return spz::fail(SPZ_ERR_NULL, "handle is NULL");
  return spz::apply_unitary(h, u_reals, u_imags, m, target, control);
}
