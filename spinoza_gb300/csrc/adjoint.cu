// Adjoint differentiation (Jones & Gacon, arXiv:2009.02823) of
// E(theta) = <psi(theta)| H |psi(theta)>, H a sum of Pauli strings.
// No reference counterpart: a new form built on the gate path.
//
//   forward   psi = G_L ... G_1 |psi_0>          (fused executor)
//             lam = H psi, E = Re<psi|lam>
//   backward  for j = L .. 1:
//               if G_j = G(theta_j):  dE/dtheta_j = 2 Re<lam| K_j |psi>,
//                 where dG/dtheta = K G (K = -(i/2) Pi_c (x) sigma for
//                 RX/RY/RZ, K = i Pi_c (x) |1><1| for P; Pi_c projects on the
//                 controls), i.e. Im<lam|Pi sigma|psi> or -2 Im<lam|Pi |1><1||psi>
//               psi <- G_j^dagger psi,  lam <- G_j^dagger lam
//
// Device memory: psi stays in the handle (it holds psi(theta) on return); the
// sweep runs on two extra state vectors (a working copy of psi, and lam).
#include <algorithm>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace spz {

int run_gates(spz_state_t h, const std::vector<GateApp>& gates, uint32_t flags, spz_exec_stats* st);

constexpr int kAdjThreads = 256;
constexpr int kAdjMaxBlocks = kNumSMs * 8;

__device__ __forceinline__ double adj_block_sum(double v, double* smem) {
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

__global__ void adj_finalize_kernel(const double* __restrict__ partials, int nblocks, double* __restrict__ out) {
  __shared__ double smem[32];
  double v = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) v = dadd(v, partials[b]);
  v = adj_block_sum(v, smem);
  if (threadIdx.x == 0) *out = v;
}

enum GradMode { GM_X = 0, GM_Y = 1, GM_Z = 2, GM_P1 = 3 };

struct GradArgs {
  const double* pr;  // psi
  const double* pi;
  const double* lr;  // lambda
  const double* li;
  uint64_t nwork;
  uint64_t ones;
  uint64_t tbit;
  int32_t npos;
  uint8_t pos[kMaxQubits + 2];
};

// Im of the per-pair contribution to <lam| Pi sigma |psi> (see file comment).
template <int MODE>
__global__ void __launch_bounds__(kAdjThreads) grad_pair_kernel(GradArgs A, double* __restrict__ partials) {
  __shared__ double smem[32];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  double acc = 0.0;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < A.nwork; w += stride) {
    const uint64_t s0 = deposit(w, A.pos, A.npos) | A.ones;
    const uint64_t s1 = s0 | A.tbit;
    const double a = A.pr[s0], b = A.pi[s0], c = A.pr[s1], d = A.pi[s1];
    const double p = A.lr[s0], q = A.li[s0], r = A.lr[s1], s = A.li[s1];
    double v;
    if constexpr (MODE == GM_X) {  // Im(conj(l0) psi1 + conj(l1) psi0)
      v = dadd(dfma(p, d, dmul(dneg(q), c)), dfma(r, b, dmul(dneg(s), a)));
    } else if constexpr (MODE == GM_Y) {  // Im(-i conj(l0) psi1 + i conj(l1) psi0)
      v = dsub(dfma(r, a, dmul(s, b)), dfma(p, c, dmul(q, d)));
    } else if constexpr (MODE == GM_Z) {  // Im(conj(l0) psi0 - conj(l1) psi1)
      v = dsub(dfma(p, b, dmul(dneg(q), a)), dfma(r, d, dmul(dneg(s), c)));
    } else {  // Im(conj(l1) psi1)
      v = dfma(r, d, dmul(dneg(s), c));
    }
    acc = dadd(acc, v);
  }
  const double t = adj_block_sum(acc, smem);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

// lam = D psi for the diagonal terms (or 0 when there are none).
struct DiagSum {
  int nterms;
  double coeff[64];
  uint64_t zmask[64];
};

__global__ void hamiltonian_diag_kernel(const double* __restrict__ pr, const double* __restrict__ pi,
                                        double* __restrict__ lr, double* __restrict__ li, uint64_t N, DiagSum T) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < N; x += stride) {
    double dsum = 0.0;
    for (int k = 0; k < T.nterms; ++k)
      dsum = dadd(dsum, (__popcll(x & T.zmask[k]) & 1) ? dneg(T.coeff[k]) : T.coeff[k]);
    lr[x] = dmul(dsum, pr[x]);
    li[x] = dmul(dsum, pi[x]);
  }
}

// lam_x += sum_k c_k i^ny_k (-1)^popc(y & z_k) psi_y,  y = x ^ xmask.
struct XSum {
  int nterms;
  uint64_t xmask;
  double coeff[64];
  uint64_t zmask[64];
  int ny[64];
};

__global__ void hamiltonian_x_kernel(const double* __restrict__ pr, const double* __restrict__ pi,
                                     double* __restrict__ lr, double* __restrict__ li, uint64_t N, XSum T) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < N; x += stride) {
    const uint64_t y = x ^ T.xmask;
    double cr = 0.0, ci = 0.0;
    for (int k = 0; k < T.nterms; ++k) {
      double v = (__popcll(y & T.zmask[k]) & 1) ? dneg(T.coeff[k]) : T.coeff[k];
      const int ny = T.ny[k] & 3;
      if (ny >= 2) v = dneg(v);
      if (ny & 1) ci = dadd(ci, v); else cr = dadd(cr, v);
    }
    const double yr = pr[y], yi = pi[y];
    lr[x] = dadd(lr[x], dfma(cr, yr, dmul(dneg(ci), yi)));
    li[x] = dadd(li[x], dfma(cr, yi, dmul(ci, yr)));
  }
}

__global__ void inner_re_kernel(const double* __restrict__ pr, const double* __restrict__ pi,
                                const double* __restrict__ lr, const double* __restrict__ li, uint64_t N,
                                double* __restrict__ partials) {
  __shared__ double smem[32];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  double acc = 0.0;
  for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < N; x += stride)
    acc = dadd(acc, dfma(pr[x], lr[x], dmul(pi[x], li[x])));
  const double t = adj_block_sum(acc, smem);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

namespace {

int ensure_aux(spz_state_t h, int j) {
  if (!h->aux_re[j]) {
    SPZ_CUDA(cudaMalloc(&h->aux_re[j], h->N * sizeof(double)));
    cudaError_t e = cudaMalloc(&h->aux_im[j], h->N * sizeof(double));
    if (e != cudaSuccess) {
      cudaFree(h->aux_re[j]);
      h->aux_re[j] = nullptr;
      return cuda_fail(e, "cudaMalloc of an adjoint work vector");
    }
  }
  return SPZ_OK;
}

// Inverse of a gate (gates.rs:80-92: angle negation; U(t,p,l)^-1 = U(-t,-l,-p)).
spz_gate inverse_gate(const spz_gate& g) {
  spz_gate r = g;
  switch (g.kind) {
    case SPZ_GATE_P:
    case SPZ_GATE_RX:
    case SPZ_GATE_RY:
    case SPZ_GATE_RZ:
      r.p[0] = -g.p[0];
      break;
    case SPZ_GATE_U:
      r.p[0] = -g.p[0];
      r.p[1] = -g.p[2];
      r.p[2] = -g.p[1];
      break;
    default:
      break;
  }
  return r;
}

// The same handle, viewing other device arrays (no ownership).
spz_state_s view_of(spz_state_t h, double* re, double* im) {
  spz_state_s v;
  v.n = h->n;
  v.N = h->N;
  v.re = re;
  v.im = im;
  v.owns = false;
  v.own_stream = nullptr;
  v.stream = h->stream;
  v.device = h->device;
  return v;
}

}  // namespace

int adjoint_gradient(spz_state_t h, const spz_op* ops, size_t nops, const uint32_t* param_index, size_t nparams,
                     const spz_pauli_term* terms, size_t nterms, double* energy, double* grad) {
  if (nops && !ops) return fail(SPZ_ERR_NULL, "ops is NULL");
  if (nparams && (!param_index || !grad)) return fail(SPZ_ERR_NULL, "param_index/grad is NULL");
  if (nterms && !terms) return fail(SPZ_ERR_NULL, "terms is NULL");
  if (!energy) return fail(SPZ_ERR_NULL, "energy is NULL");
  const uint32_t n = h->n;
  // Forward gate list, with each op's inverse.
  std::vector<GateApp> fwd(nops), inv(nops);
  std::vector<int> skip(nops, 0);
  for (size_t i = 0; i < nops; ++i) {
    const spz_op& op = ops[i];
    if (op.gate.kind == SPZ_GATE_M) return fail(SPZ_ERR_UNSUPPORTED, "measurement inside a differentiated circuit");
    spz_gate g = op.gate;
    if (g.kind == SPZ_GATE_BITFLIP) {
      if (!(g.p[1] <= g.p[0])) { skip[i] = 1; continue; }
      g = spz_gate{};
      g.kind = SPZ_GATE_X;
    }
    uint64_t ones = op.controls, zeros = 0;
    if (op.controls_kind == SPZ_CONTROLS_NONE) ones = 0;
    if (op.controls_kind == SPZ_CONTROLS_MIXED) {
      ones = op.controls & ~op.zeros;
      zeros = op.zeros;
    }
    int rc = make_gate_app(n, g, op.target, ones, zeros, &fwd[i]);
    if (rc) return rc;
    rc = make_gate_app(n, inverse_gate(g), op.target, ones, zeros, &inv[i]);
    if (rc) return rc;
  }
  // Which ops are differentiated, and by which mode.
  std::vector<int> mode_of(nops, -1);
  for (size_t j = 0; j < nparams; ++j) {
    const uint32_t k = param_index[j];
    if (k >= nops) return fail(SPZ_ERR_INVALID_ARGUMENT, "param_index out of range");
    if (skip[k]) return fail(SPZ_ERR_INVALID_ARGUMENT, "parameter of a gate that is not applied");
    switch (ops[k].gate.kind) {
      case SPZ_GATE_RX: mode_of[k] = GM_X; break;
      case SPZ_GATE_RY: mode_of[k] = GM_Y; break;
      case SPZ_GATE_RZ: mode_of[k] = GM_Z; break;
      case SPZ_GATE_P: mode_of[k] = GM_P1; break;
      default: return fail(SPZ_ERR_UNSUPPORTED, "only P, RX, RY and RZ angles can be differentiated");
    }
  }
  for (size_t k = 0; k < nterms; ++k)
    if (n < 64 && ((terms[k].x_mask | terms[k].z_mask) >> n) != 0)
      return fail(SPZ_ERR_INVALID_ARGUMENT, "Pauli term acts on a qubit out of range");
  // Forward.
  std::vector<GateApp> applied;
  for (size_t i = 0; i < nops; ++i)
    if (!skip[i]) applied.push_back(fwd[i]);
  int rc = run_gates(h, applied, SPZ_EXEC_DEFAULT, nullptr);
  if (rc) return rc;
  rc = ensure_aux(h, 0);
  if (rc) return rc;
  rc = ensure_aux(h, 1);
  if (rc) return rc;
  double *lr = h->aux_re[0], *li = h->aux_im[0], *wr = h->aux_re[1], *wi = h->aux_im[1];
  // lam = H psi.
  std::vector<std::vector<size_t>> groups;
  std::vector<uint64_t> gx;
  for (size_t k = 0; k < nterms; ++k) {
    size_t g = 0;
    for (; g < groups.size(); ++g)
      if (gx[g] == terms[k].x_mask && groups[g].size() < 64) break;
    if (g == groups.size()) { groups.emplace_back(); gx.push_back(terms[k].x_mask); }
    groups[g].push_back(k);
  }
  DiagSum D{};
  for (size_t g = 0; g < groups.size(); ++g)
    if (gx[g] == 0)
      for (size_t k : groups[g]) {
        if (D.nterms == 64) return fail(SPZ_ERR_UNSUPPORTED, "more than 64 diagonal terms");
        D.coeff[D.nterms] = terms[k].coeff;
        D.zmask[D.nterms++] = terms[k].z_mask;
      }
  hamiltonian_diag_kernel<<<grid_for(h->N), kThreads, 0, h->stream>>>(h->re, h->im, lr, li, h->N, D);
  for (size_t g = 0; g < groups.size(); ++g) {
    if (gx[g] == 0) continue;
    XSum X{};
    X.xmask = gx[g];
    for (size_t k : groups[g]) {
      X.coeff[X.nterms] = terms[k].coeff;
      X.zmask[X.nterms] = terms[k].z_mask;
      X.ny[X.nterms++] = __builtin_popcountll(terms[k].x_mask & terms[k].z_mask);
    }
    hamiltonian_x_kernel<<<grid_for(h->N), kThreads, 0, h->stream>>>(h->re, h->im, lr, li, h->N, X);
  }
  SPZ_CHECK_LAUNCH("hamiltonian kernels");
  // Scratch: partials + one slot per op + the energy slot.
  void* scratch;
  rc = ensure_dev_scratch(h, (kAdjMaxBlocks + nops + 8) * sizeof(double), &scratch);
  if (rc) return rc;
  double* partials = (double*)scratch;
  double* slots = partials + kAdjMaxBlocks;  // slots[0] = energy, slots[1 + i] = op i
  {
    const int blocks = std::min<int>(grid_for(h->N, kAdjThreads, 8), kAdjMaxBlocks);
    inner_re_kernel<<<blocks, kAdjThreads, 0, h->stream>>>(h->re, h->im, lr, li, h->N, partials);
    adj_finalize_kernel<<<1, 1024, 0, h->stream>>>(partials, blocks, slots);
  }
  // Working copy of psi.
  SPZ_CUDA(cudaMemcpyAsync(wr, h->re, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  SPZ_CUDA(cudaMemcpyAsync(wi, h->im, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  spz_state_s psi_v = view_of(h, wr, wi), lam_v = view_of(h, lr, li);
  for (size_t ii = nops; ii-- > 0;) {
    if (skip[ii]) continue;
    if (mode_of[ii] >= 0) {
      const GateApp& g = fwd[ii];
      GradArgs A{};
      A.pr = wr; A.pi = wi; A.lr = lr; A.li = li;
      A.ones = g.ones;
      A.tbit = 1ull << g.target;
      const uint64_t special = g.ones | g.zeros | A.tbit;
      for (int q = 0; q < 64; ++q)
        if ((special >> q) & 1) A.pos[A.npos++] = (uint8_t)q;
      A.nwork = h->N >> A.npos;
      const int blocks = std::min<int>(grid_for(A.nwork, kAdjThreads, 8), kAdjMaxBlocks);
      switch (mode_of[ii]) {
        case GM_X: grad_pair_kernel<GM_X><<<blocks, kAdjThreads, 0, h->stream>>>(A, partials); break;
        case GM_Y: grad_pair_kernel<GM_Y><<<blocks, kAdjThreads, 0, h->stream>>>(A, partials); break;
        case GM_Z: grad_pair_kernel<GM_Z><<<blocks, kAdjThreads, 0, h->stream>>>(A, partials); break;
        default: grad_pair_kernel<GM_P1><<<blocks, kAdjThreads, 0, h->stream>>>(A, partials); break;
      }
      adj_finalize_kernel<<<1, 1024, 0, h->stream>>>(partials, blocks, slots + 1 + ii);
      SPZ_CHECK_LAUNCH("grad_pair_kernel");
    }
    rc = launch_gate(&psi_v, inv[ii]);
    if (rc) return rc;
    rc = launch_gate(&lam_v, inv[ii]);
    if (rc) return rc;
  }
  std::vector<double> host(nops + 1);
  SPZ_CUDA(cudaMemcpyAsync(host.data(), slots, (nops + 1) * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  SPZ_CUDA(cudaStreamSynchronize(h->stream));
  *energy = host[0];
  for (size_t j = 0; j < nparams; ++j) {
    const uint32_t k = param_index[j];
    const double im = host[1 + k];
    grad[j] = mode_of[k] == GM_P1 ? -2.0 * im : im;
  }
  return SPZ_OK;
}

}  // namespace spz

using namespace spz;

extern "C" int spz_adjoint_gradient(spz_state_t h, const spz_op* ops, size_t nops, const uint32_t* param_index,
                                    size_t nparams, const spz_pauli_term* terms, size_t nterms, double* energy,
                                    double* grad) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  return adjoint_gradient(h, ops, nops, param_index, nparams, terms, nterms, energy, grad);
}
