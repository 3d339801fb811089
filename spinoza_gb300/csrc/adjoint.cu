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
//
// The backward sweep is fused like the forward executor: the inverse gates,
// in reverse order, are planned into passes over tiles of 2^k amplitudes that
// hold psi and lam together in shared memory; per gate and tile each warp adds
// its share of the gradient to its own accumulator (fixed order: the results
// are identical from run to run), then the inverse gate is applied to both.
// Reordering by the planner only exchanges gates that commute, and a gate that
// commutes with G_j also commutes with its generator K_j (same qubits, same
// diagonal / non-diagonal roles), so each gradient still sees the states it
// would see in program order.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "executor.cuh"
#include "gate_math.cuh"
#include "tile_ops.cuh"

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

// ------------------------------------------------------------ fused sweep
#ifndef SPZ_ADJ_TILE_K
#define SPZ_ADJ_TILE_K 10
#endif
#ifndef SPZ_ADJ_THREADS
#define SPZ_ADJ_THREADS 64
#endif
constexpr int kAdjTileK = SPZ_ADJ_TILE_K;  // psi and lam tiles: 4 x 2^10 doubles = 32 KiB
constexpr int kAdjTileThreads = SPZ_ADJ_THREADS;
constexpr int kAdjWarps = kAdjTileThreads / 32;
constexpr int kAdjMaxSlots = 256;   // differentiated gates per backward pass

struct AdjOp {
  int32_t mode;  // GradMode, or -1: no gradient at this gate
  int32_t slot;  // its accumulator within the pass
};

struct AdjPassArgs {
  double* pr;  // psi (working copy)
  double* pi;
  double* lr;  // lam
  double* li;
  uint64_t ntiles;
  const TileGate* gates;  // inverse gates, backward order
  const AdjOp* aops;
  double* partials;       // [nslots][gridDim.x]
  int ngates;
  int nslots;
  int k;
  int c;
  int nhigh;
  uint8_t lpos[16];
};

// Gradient term of one pair / element, as in grad_pair_kernel.
__device__ __forceinline__ double adj_pair_term(int mode, double a, double b, double c, double d, double p, double q,
                                                double r, double s) {
  switch (mode) {
    case GM_X: return dadd(dfma(p, d, dmul(dneg(q), c)), dfma(r, b, dmul(dneg(s), a)));
    case GM_Y: return dsub(dfma(r, a, dmul(s, b)), dfma(p, c, dmul(q, d)));
    case GM_Z: return dsub(dfma(p, b, dmul(dneg(q), a)), dfma(r, d, dmul(dneg(s), c)));
    default: return dfma(r, d, dmul(dneg(s), c));
  }
}

// This thread's gradient share over the gate's pairs, then G^-1 on psi and lam.
template <int KIND, int NPOS>
__device__ __forceinline__ double adj_pair(const TileGate& g, int mode, double* pr, double* pi, double* lr, double* li,
                                           uint32_t nw) {
  const Enumerator<NPOS, TileGate> E(g);
  const uint32_t tbit = g.tbit;
  const Coef cf = g.c;
  double acc = 0.0;
  for (uint32_t m = threadIdx.x; m < nw; m += blockDim.x) {
    const uint32_t s0 = E(m), s1 = s0 | tbit;
    double a = pr[s0], b = pi[s0], c = pr[s1], d = pi[s1];
    double p = lr[s0], q = li[s0], r = lr[s1], s = li[s1];
    if (mode >= 0) acc = dadd(acc, adj_pair_term(mode, a, b, c, d, p, q, r, s));
    if constexpr (KIND >= FK_LAZY_H) {
      fast_pair<KIND>(cf, a, b, c, d);
      fast_pair<KIND>(cf, p, q, r, s);
    } else {
      gate_pair<KIND>(cf, a, b, c, d);
      gate_pair<KIND>(cf, p, q, r, s);
    }
    pr[s0] = a; pi[s0] = b; pr[s1] = c; pi[s1] = d;
    lr[s0] = p; li[s0] = q; lr[s1] = r; li[s1] = s;
  }
  return acc;
}

// Diagonal gates (Z, P, RZ): elementwise; the target bit comes from the
// element or, for a non-local target, from the tile (global_one).  Gradient:
// Z mode +-Im(conj(lam) psi) by the target bit; P1 mode over the 1 half, which
// is all the enumeration visits for P.
template <int KIND, int NPOS>
__device__ __forceinline__ double adj_diag(const TileGate& g, int mode, int global_one, double* pr, double* pi,
                                           double* lr, double* li, uint32_t nw) {
  const Enumerator<NPOS, TileGate> E(g);
  const uint32_t tbit = g.tbit;
  const Coef cf = g.c;
  double acc = 0.0;
  for (uint32_t m = threadIdx.x; m < nw; m += blockDim.x) {
    const uint32_t e = E(m);
    const bool one = global_one >= 0 ? global_one != 0 : (e & tbit) != 0;
    double a = pr[e], b = pi[e], p = lr[e], q = li[e];
    if (mode >= 0) {
      const double v = dfma(p, b, dmul(dneg(q), a));  // Im(conj(lam) psi)
      acc = (mode == GM_Z && one) ? dsub(acc, v) : dadd(acc, v);
    }
    gate_diag<KIND>(cf, one, a, b);
    gate_diag<KIND>(cf, one, p, q);
    pr[e] = a; pi[e] = b; lr[e] = p; li[e] = q;
  }
  return acc;
}

template <int KIND>
__device__ __forceinline__ double adj_pair_any(const TileGate& g, int mode, double* pr, double* pi, double* lr,
                                               double* li, uint32_t nw) {
  double r = 0.0;
#define SPZ_CALL(N) r = adj_pair<KIND, N>(g, mode, pr, pi, lr, li, nw)
  SPZ_BY_NPOS(g.npos, SPZ_CALL)
#undef SPZ_CALL
  return r;
}

template <int KIND>
__device__ __forceinline__ double adj_diag_any(const TileGate& g, int mode, int global_one, double* pr, double* pi,
                                               double* lr, double* li, uint32_t nw) {
  double r = 0.0;
#define SPZ_CALL(N) r = adj_diag<KIND, N>(g, mode, global_one, pr, pi, lr, li, nw)
  SPZ_BY_NPOS(g.npos, SPZ_CALL)
#undef SPZ_CALL
  return r;
}

__global__ void __launch_bounds__(kAdjTileThreads) adj_tile_kernel(const __grid_constant__ AdjPassArgs A) {
  extern __shared__ double sm[];
  const int K = A.k;
  const uint32_t T = 1u << K;
  double* pr = sm;
  double* pi = sm + T;
  double* lr = sm + 2 * T;
  double* li = sm + 3 * T;
  uint64_t* rowoff = reinterpret_cast<uint64_t*>(sm + 4 * T);
  double* wacc = reinterpret_cast<double*>(rowoff + (1u << A.nhigh));  // [kAdjWarps][kAdjMaxSlots]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t cmask = (1u << A.c) - 1;
  for (uint32_t r = threadIdx.x; r < (1u << A.nhigh); r += blockDim.x)
    rowoff[r] = row_offset_param<kAdjTileK>(r, A.lpos, A.c, K);
  for (int j = threadIdx.x; j < kAdjWarps * kAdjMaxSlots; j += blockDim.x) wacc[j] = 0.0;
  __syncthreads();
  for (uint64_t tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
    const uint64_t base = deposit_param<kAdjTileK>(tile, A.lpos, K);
    for (uint32_t e2 = threadIdx.x; e2 < T / 2; e2 += blockDim.x) {
      const uint32_t e = 2 * e2;
      const uint64_t gi = base | rowoff[e >> A.c] | (e & cmask);
      *reinterpret_cast<double2*>(pr + e) = *reinterpret_cast<const double2*>(A.pr + gi);
      *reinterpret_cast<double2*>(pi + e) = *reinterpret_cast<const double2*>(A.pi + gi);
      *reinterpret_cast<double2*>(lr + e) = *reinterpret_cast<const double2*>(A.lr + gi);
      *reinterpret_cast<double2*>(li + e) = *reinterpret_cast<const double2*>(A.li + gi);
    }
    __syncthreads();
    for (int gi = 0; gi < A.ngates; ++gi) {
      const TileGate& g = A.gates[gi];
      if ((base & g.g_ones) != g.g_ones || (base & g.g_zeros) != 0) continue;  // uniform per tile
      const int mode = A.aops[gi].mode;
      const uint32_t nw = T >> g.npos;
      double v = 0.0;
      switch (g.mode) {
        case TM_PAIR:
          switch (g.kind) {
            case SPZ_GATE_H: v = adj_pair_any<SPZ_GATE_H>(g, mode, pr, pi, lr, li, nw); break;
            case SPZ_GATE_X: v = adj_pair_any<SPZ_GATE_X>(g, mode, pr, pi, lr, li, nw); break;
            case SPZ_GATE_Y: v = adj_pair_any<SPZ_GATE_Y>(g, mode, pr, pi, lr, li, nw); break;
            case SPZ_GATE_RX: v = adj_pair_any<SPZ_GATE_RX>(g, mode, pr, pi, lr, li, nw); break;
            case SPZ_GATE_RY: v = adj_pair_any<SPZ_GATE_RY>(g, mode, pr, pi, lr, li, nw); break;
            case FK_LAZY_H: v = adj_pair_any<FK_LAZY_H>(g, mode, pr, pi, lr, li, nw); break;
            case FK_LAZY_RX_A: v = adj_pair_any<FK_LAZY_RX_A>(g, mode, pr, pi, lr, li, nw); break;
            case FK_LAZY_RX_B: v = adj_pair_any<FK_LAZY_RX_B>(g, mode, pr, pi, lr, li, nw); break;
            case FK_LAZY_RY_A: v = adj_pair_any<FK_LAZY_RY_A>(g, mode, pr, pi, lr, li, nw); break;
            case FK_LAZY_RY_B: v = adj_pair_any<FK_LAZY_RY_B>(g, mode, pr, pi, lr, li, nw); break;
            default: v = adj_pair_any<SPZ_GATE_U>(g, mode, pr, pi, lr, li, nw); break;
          }
          break;
        case TM_DIAG_LOCAL:
        case TM_DIAG_GLOBAL: {
          int gone = -1;
          if (g.mode == TM_DIAG_GLOBAL) {
            gone = (base & g.g_tbit) ? 1 : 0;
            if (!gone && g.kind != SPZ_GATE_RZ) break;  // Z / P (and the P1 gradient) live on the 1 half
          }
          switch (g.kind) {
            case SPZ_GATE_Z: v = adj_diag_any<SPZ_GATE_Z>(g, mode, gone, pr, pi, lr, li, nw); break;
            case SPZ_GATE_P: v = adj_diag_any<SPZ_GATE_P>(g, mode, gone, pr, pi, lr, li, nw); break;
            default: v = adj_diag_any<SPZ_GATE_RZ>(g, mode, gone, pr, pi, lr, li, nw); break;
          }
          break;
        }
        default:  // TM_SWAP: no gradient
          tile_swap_any(g, pr, pi, nw);
          tile_swap_any(g, lr, li, nw);
      }
      if (mode >= 0) {  // uniform: the whole block takes this branch
        for (int off = 16; off > 0; off >>= 1) v = dadd(v, __shfl_down_sync(0xffffffffu, v, off));
        if (lane == 0) wacc[warp * kAdjMaxSlots + A.aops[gi].slot] += v;
      }
      __syncthreads();
    }
    for (uint32_t e2 = threadIdx.x; e2 < T / 2; e2 += blockDim.x) {
      const uint32_t e = 2 * e2;
      const uint64_t gi = base | rowoff[e >> A.c] | (e & cmask);
      *reinterpret_cast<double2*>(A.pr + gi) = *reinterpret_cast<const double2*>(pr + e);
      *reinterpret_cast<double2*>(A.pi + gi) = *reinterpret_cast<const double2*>(pi + e);
      *reinterpret_cast<double2*>(A.lr + gi) = *reinterpret_cast<const double2*>(lr + e);
      *reinterpret_cast<double2*>(A.li + gi) = *reinterpret_cast<const double2*>(li + e);
    }
    __syncthreads();
  }
  for (int sl = threadIdx.x; sl < A.nslots; sl += blockDim.x) {
    double t = 0.0;
    for (int w = 0; w < kAdjWarps; ++w) t = dadd(t, wacc[w * kAdjMaxSlots + sl]);
    A.partials[(uint64_t)sl * gridDim.x + blockIdx.x] = t;
  }
}

// Device outputs: grad[j] = mul[j] * slots[sel[j]], energy = slots[0].
__global__ void adj_gather_kernel(const double* __restrict__ slots, const int32_t* __restrict__ sel,
                                  const double* __restrict__ mul, uint32_t nparams, double* __restrict__ grad,
                                  double* __restrict__ energy) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nparams) grad[j] = dmul(mul[j], slots[sel[j]]);
  if (j == 0) *energy = slots[0];
}

// out[slot_op[s]] = sum over blocks of partials[s][.], one block per slot.
__global__ void adj_slots_kernel(const double* __restrict__ partials, int nblocks, const int32_t* __restrict__ slot_op,
                                 double* __restrict__ out) {
  __shared__ double smem[32];
  const double* row = partials + (uint64_t)blockIdx.x * nblocks;
  double v = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) v = dadd(v, row[b]);
  v = adj_block_sum(v, smem);
  if (threadIdx.x == 0) out[slot_op[blockIdx.x]] = v;
}

namespace {

int ensure_aux(spz_state_t h, int j) {
  if (!h->aux_re[j]) {
    SPZ_CUDA(dev_alloc(&h->aux_re[j], h->N * sizeof(double)));
    cudaError_t e = dev_alloc(&h->aux_im[j], h->N * sizeof(double));
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

}  // namespace

// With d_energy / d_grad (device pointers) the results are written there and
// nothing waits for the device; otherwise they come back to energy / grad.
int adjoint_gradient(spz_state_t h, const spz_op* ops, size_t nops, const uint32_t* param_index, size_t nparams,
                     const spz_pauli_term* terms, size_t nterms, uint32_t flags, double* energy, double* grad,
                     double* d_energy, double* d_grad) {
  const bool on_device = d_energy != nullptr;
  const bool fast = (flags & SPZ_EXEC_FAST) != 0;
  if (nops && !ops) return fail(SPZ_ERR_NULL, "ops is NULL");
  if (nparams && (!param_index || (on_device ? !d_grad : !grad))) return fail(SPZ_ERR_NULL, "param_index/grad is NULL");
  if (nterms && !terms) return fail(SPZ_ERR_NULL, "terms is NULL");
  if (!on_device && !energy) return fail(SPZ_ERR_NULL, "energy is NULL");
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
  int rc = run_gates(h, applied, fast ? SPZ_EXEC_FAST : SPZ_EXEC_DEFAULT, nullptr);
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
  // Backward: the inverse gates in reverse order, fused into tile passes
  // (passes with more than kAdjMaxSlots differentiated gates are cut).
  std::vector<GateApp> bwd;
  for (size_t ii = nops; ii-- > 0;) {
    if (skip[ii]) continue;
    GateApp g = inv[ii];
    g.src = (int64_t)ii;
    bwd.push_back(g);
  }
  // Fast mode: uncontrolled H / RX / RY inverses become lazy ops (the gate
  // divided by a real scalar: 4 FMAs per pair) and uncontrolled RZ inverses
  // become P (the 1 half only) times a unit phase.  psi and lam pass through
  // the same ops, so the phases cancel in <lam|K|psi> and the real scalars S
  // (product so far) enter as S^2 on each gradient.  Above 800 lazy ops S could
  // leave the exponent range; the sweep then stays exact.
  std::vector<double> lazy_scale(nops, 1.0);
  if (fast) {
    size_t lazy = 0;
    for (const GateApp& g : bwd)
      lazy += (g.ones | g.zeros) == 0 &&
              (g.kind == SPZ_GATE_H || g.kind == SPZ_GATE_RX || g.kind == SPZ_GATE_RY);
    if (lazy <= 800)
      for (GateApp& g : bwd) {
        if ((g.ones | g.zeros) != 0) continue;
        const int64_t src = g.src;
        if (g.kind == SPZ_GATE_H) {
          GateApp l = g;
          l.kind = FK_LAZY_H;
          lazy_scale[src] = std::sqrt(0.5);
          g = l;
        } else if (g.kind == SPZ_GATE_RX || g.kind == SPZ_GATE_RY) {
          const bool is_x = g.kind == SPZ_GATE_RX;
          const double cs = g.c.cs, sn = g.c.sn;  // cos, sin of theta/2
          GateApp l = g;
          if (std::fabs(cs) >= std::fabs(sn)) {
            l.kind = is_x ? FK_LAZY_RX_A : FK_LAZY_RY_A;
            l.c.cs = sn / cs;
            lazy_scale[src] = cs;
          } else {
            l.kind = is_x ? FK_LAZY_RX_B : FK_LAZY_RY_B;
            l.c.cs = cs / sn;
            lazy_scale[src] = sn;
          }
          g = l;
        } else if (g.kind == SPZ_GATE_RZ) {  // RZ = e^{-i theta/2} P(theta): d1 / d0 = e^{i theta}
          const std::complex<double> d0(g.c.d0re, g.c.d0im), d1(g.c.d1re, g.c.d1im);
          spz_gate pg{};
          pg.kind = SPZ_GATE_P;
          pg.p[0] = std::arg(d1 / d0);
          GateApp l;
          rc = make_gate_app(n, pg, g.target, 0, 0, &l);
          if (rc) return rc;
          l.src = src;
          g = l;
          // P visits only the target's 1 half, so RZ's gradient is taken in
          // P's form: Im<lam|psi> is 0 (H is Hermitian, and psi, lam pass
          // through the same unitaries), so sum over the 0 half minus sum over
          // the 1 half of Im(conj(lam) psi) equals -2 x the 1-half sum.
          if (mode_of[src] == GM_Z) mode_of[src] = GM_P1;
        }
      }
  }
  const int k = std::min<int>((int)n, kAdjTileK);
  const int c = std::min<int>(kTileLowBits, k);
  std::vector<PlannedPass> passes;
  for (PlannedPass& P : plan_passes(bwd, n, k, c, /*exact=*/false)) {
    PlannedPass cur;
    cur.local = P.local;
    int slots = 0;
    for (const GateApp& g : P.gates) {
      const bool grad = mode_of[g.src] >= 0;
      if (grad && slots == kAdjMaxSlots) {
        passes.push_back(cur);
        cur.gates.clear();
        slots = 0;
      }
      cur.gates.push_back(g);
      slots += grad;
    }
    if (!cur.gates.empty()) passes.push_back(std::move(cur));
  }
  // S^2 for each differentiated op: S = product of the lazy scalars applied
  // before its gradient, in the order the passes run.
  std::vector<double> grad_scale(nops, 1.0);
  {
    double S = 1.0;
    for (const PlannedPass& P : passes)
      for (const GateApp& g : P.gates) {
        if (mode_of[g.src] >= 0) grad_scale[g.src] = S * S;
        S *= lazy_scale[g.src];
      }
  }
  std::vector<TileGate> tg;
  std::vector<AdjOp> ao;
  std::vector<int32_t> slot_op;
  std::vector<size_t> gate_off, slot_off;
  size_t max_slots = 0;
  for (const PlannedPass& P : passes) {
    gate_off.push_back(tg.size());
    slot_off.push_back(slot_op.size());
    int slots = 0;
    for (const GateApp& g : P.gates) {
      tg.push_back(make_tile_gate(g, P.local));
      AdjOp a{mode_of[g.src], -1};
      if (a.mode >= 0) {
        a.slot = slots++;
        slot_op.push_back((int32_t)(1 + g.src));
      }
      ao.push_back(a);
    }
    max_slots = std::max<size_t>(max_slots, (size_t)slots);
  }
  gate_off.push_back(tg.size());
  slot_off.push_back(slot_op.size());
  // Launch shape: one wave of resident blocks.
  const uint32_t T = 1u << k;
  const size_t smem = (4 * (size_t)T + (size_t)(1u << (k - c)) + (size_t)kAdjWarps * kAdjMaxSlots) * sizeof(double);
  // Resident blocks per SM and the SM count, set up once per device (kernel
  // attributes are per device; first calls may come from several threads).
  static std::mutex shape_mu;
  static int shape_resident[kMaxDevices] = {}, shape_sms[kMaxDevices] = {};
  if (h->device < 0 || h->device >= kMaxDevices) return fail(SPZ_ERR_INVALID_ARGUMENT, "device index out of range");
  int resident = 0, sms = 0;
  {
    std::lock_guard<std::mutex> lock(shape_mu);
    if (!shape_resident[h->device]) {
      int count = 0;
      SPZ_CUDA(cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, h->device));
      const size_t max_smem = (4 * ((size_t)1 << kAdjTileK) + ((size_t)1 << (kAdjTileK - kTileLowBits)) +
                               (size_t)kAdjWarps * kAdjMaxSlots) * sizeof(double);
      SPZ_CUDA(cudaFuncSetAttribute(adj_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem));
      int per_sm = 0;
      SPZ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, adj_tile_kernel, kAdjTileThreads, max_smem));
      shape_sms[h->device] = count;
      shape_resident[h->device] = std::max(1, per_sm);
    }
    resident = shape_resident[h->device];
    sms = shape_sms[h->device];
  }
  const uint64_t ntiles = 1ull << (n - k);
  const int blocks = (int)std::min<uint64_t>(ntiles, (uint64_t)sms * resident);
  // Scratch: slots (energy + one per op), partials, then the pass descriptors.
  const size_t nslot_words = (nops + 8 + 31) / 32 * 32;
  const size_t npart = std::max<size_t>((size_t)kAdjMaxBlocks, max_slots * (size_t)blocks);
  const size_t desc_off = (nslot_words + npart) * sizeof(double);
  const size_t tg_bytes = (tg.size() * sizeof(TileGate) + 255) / 256 * 256;
  const size_t ao_bytes = (ao.size() * sizeof(AdjOp) + 255) / 256 * 256;
  const size_t so_bytes = (slot_op.size() * sizeof(int32_t) + 255) / 256 * 256;
  // device outputs: per parameter, its slot and factor (-2 for P, else 1)
  std::vector<int32_t> gsel(nparams);
  std::vector<double> gmul(nparams);
  for (size_t j = 0; j < nparams; ++j) {
    gsel[j] = (int32_t)(1 + param_index[j]);
    gmul[j] = (mode_of[param_index[j]] == GM_P1 ? -2.0 : 1.0) * grad_scale[param_index[j]];
  }
  const size_t gs_bytes = (nparams * sizeof(int32_t) + 255) / 256 * 256;
  const size_t gm_bytes = nparams * sizeof(double);
  void* scratch;
  rc = ensure_dev_scratch(h, desc_off + tg_bytes + ao_bytes + so_bytes + gs_bytes + gm_bytes + 256, &scratch);
  if (rc) return rc;
  double* slots = (double*)scratch;  // slots[0] = energy, slots[1 + i] = op i
  double* partials = slots + nslot_words;
  TileGate* d_tg = (TileGate*)((char*)scratch + desc_off);
  AdjOp* d_ao = (AdjOp*)((char*)d_tg + tg_bytes);
  int32_t* d_so = (int32_t*)((char*)d_ao + ao_bytes);
  int32_t* d_gs = (int32_t*)((char*)d_so + so_bytes);
  double* d_gm = (double*)((char*)d_gs + gs_bytes);
  // From pageable memory: the runtime stages the bytes before returning.
  if (!tg.empty()) {
    SPZ_CUDA(cudaMemcpyAsync(d_tg, tg.data(), tg.size() * sizeof(TileGate), cudaMemcpyHostToDevice, h->stream));
    SPZ_CUDA(cudaMemcpyAsync(d_ao, ao.data(), ao.size() * sizeof(AdjOp), cudaMemcpyHostToDevice, h->stream));
  }
  if (!slot_op.empty())
    SPZ_CUDA(cudaMemcpyAsync(d_so, slot_op.data(), slot_op.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                             h->stream));
  if (on_device && nparams) {
    SPZ_CUDA(cudaMemcpyAsync(d_gs, gsel.data(), nparams * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    SPZ_CUDA(cudaMemcpyAsync(d_gm, gmul.data(), nparams * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  }
  SPZ_CUDA(cudaMemsetAsync(slots, 0, (nops + 1) * sizeof(double), h->stream));
  {
    const int rb = std::min<int>(grid_for(h->N, kAdjThreads, 8), kAdjMaxBlocks);
    inner_re_kernel<<<rb, kAdjThreads, 0, h->stream>>>(h->re, h->im, lr, li, h->N, partials);
    adj_finalize_kernel<<<1, 1024, 0, h->stream>>>(partials, rb, slots);
  }
  // Working copy of psi.
  SPZ_CUDA(cudaMemcpyAsync(wr, h->re, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  SPZ_CUDA(cudaMemcpyAsync(wi, h->im, h->N * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  for (size_t p = 0; p < passes.size(); ++p) {
    const PlannedPass& P = passes[p];
    AdjPassArgs A{};
    A.pr = wr;
    A.pi = wi;
    A.lr = lr;
    A.li = li;
    A.ntiles = ntiles;
    A.gates = d_tg + gate_off[p];
    A.aops = d_ao + gate_off[p];
    A.partials = partials;
    A.ngates = (int)(gate_off[p + 1] - gate_off[p]);
    A.nslots = (int)(slot_off[p + 1] - slot_off[p]);
    A.k = (int)P.local.size();
    A.c = c;
    A.nhigh = A.k - c;
    for (int j = 0; j < A.k; ++j) A.lpos[j] = (uint8_t)P.local[j];
    adj_tile_kernel<<<blocks, kAdjTileThreads, smem, h->stream>>>(A);
    SPZ_CHECK_LAUNCH("adj_tile_kernel");
    if (A.nslots) {
      adj_slots_kernel<<<A.nslots, 256, 0, h->stream>>>(partials, blocks, d_so + slot_off[p], slots);
      SPZ_CHECK_LAUNCH("adj_slots_kernel");
    }
  }
  if (on_device) {
    adj_gather_kernel<<<(unsigned)std::max<size_t>(1, (nparams + 255) / 256), 256, 0, h->stream>>>(
        slots, d_gs, d_gm, (uint32_t)nparams, d_grad, d_energy);
    SPZ_CHECK_LAUNCH("adj_gather_kernel");
    return SPZ_OK;
  }
  std::vector<double> host(nops + 1);
  SPZ_CUDA(cudaMemcpyAsync(host.data(), slots, (nops + 1) * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  SPZ_CUDA(cudaStreamSynchronize(h->stream));
  *energy = host[0];
  for (size_t j = 0; j < nparams; ++j) {
    const uint32_t k = param_index[j];
    const double im = host[1 + k];
    grad[j] = (mode_of[k] == GM_P1 ? -2.0 * im : im) * grad_scale[k];
  }
  return SPZ_OK;
}

}  // namespace spz

using namespace spz;

extern "C" int spz_adjoint_gradient(spz_state_t h, const spz_op* ops, size_t nops, const uint32_t* param_index,
                                    size_t nparams, const spz_pauli_term* terms, size_t nterms, uint32_t flags,
                                    double* energy, double* grad) {
  NvtxRange range("spz_adjoint_gradient");
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  if (int rc = settle(h)) return rc;
  return adjoint_gradient(h, ops, nops, param_index, nparams, terms, nterms, flags, energy, grad, nullptr, nullptr);
}
