// Batched variational workload: forward <H> and adjoint gradients of many
// independent parameterised circuits of uneven qubit counts in ONE persistent
// launch, replayed as a CUDA graph.  No reference counterpart (a new form built
// on the gate path).
//
// Work split.  CTAs take work items from a global counter.  An item is either
// a whole instance (smaller instances), run by one CTA:
//   forward passes   psi = G_L ... G_1 |0>          (tiles of 2^k amplitudes)
//   Hamiltonian      lam = H psi, E = Re<psi|lam>    (Pauli terms, tile passes)
//   backward passes  per gate in reverse: the tile's part of <lam|K|psi>,
//                    then G^dagger on both psi and lam (fused: one load of each)
// or, for a wide instance (at least `wide_qubits` qubits), one pass of it over
// a range of its tiles, so that one instance is spread over many CTAs.  A
// wide instance's items of pass p wait until every item of its earlier passes
// is complete (a per-instance completion counter), and the queue holds them
// after all of those, so a waiting item only ever waits on items already
// taken by running CTAs.  Each wait is bounded: past its limit the CTA sets
// the batch's error flag and stops, every other CTA stops at its next item or
// wait, and the run returns SPZ_ERR_TIMEOUT.  Wide items write their energy
// and gradient partial sums to slots that a second kernel folds in a fixed
// order.
//
// An instance of n <= k qubits lives entirely in shared memory (no HBM traffic
// beyond parameters in and energy / gradients out).  Larger instances stream
// tiles through HBM workspace (psi and lam, 2 x 16 B x 2^n): per CTA for the
// whole-instance items, per instance for the wide ones.
//
// Determinism: fixed items, tiles in a fixed order within an item, fixed
// reduction trees and partial-slot order: results are identical from run to
// run.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "gate_math.cuh"
#include "tile_ops.cuh"

namespace spz {

bool exactly_commuting_kinds(int a, int b);

namespace {

constexpr int kBatchMaxK = 12;
constexpr int kBatchLowBits = 3;
// Gradient accumulators per backward pass (passes with more parameters are
// split); each warp keeps its own set in shared memory.  48 keeps a 2^9-tile,
// 64-thread CTA under 18 KiB of shared memory, so that 12 fit on an SM.
constexpr int kMaxPassParams = 48;
constexpr uint64_t kWorkspaceBudget = 128ull << 30;  // HBM for streamed instances' psi and lam
// From about 2^18 amplitudes one instance (with two more running beside it on
// other streams) keeps the GPU's block slots busy; below, one CTA per instance
// does better.  4096 instances of 10-22 qubits measured 32.5 s with
// the persistent kernel alone and 26.1-26.7 s with the threshold at 17-20.
constexpr int kDefaultWideQubits = 18;
constexpr int kWideStreams = 4;         // at most this many wide instances in flight (whole-GPU path)
constexpr int kDefaultWideStreams = 3;  // SPZ_BATCH_WIDE_STREAMS in the environment overrides it (1..4)
// Tiles per work item of a wide instance (2^9-amplitude tiles: 64 tiles of a
// 22-qubit pass make 128 items).  The 4096-instance batch of 10-22 qubits
// measured 25.65 s with 64, 25.71 s
// with 16, 25.83 s with 4.
constexpr int kDefaultTilesPerItem = 64;
// Polls (about 0.3 us each) before a dependency wait gives up: far longer
// than any item takes, short enough that a lost dependency ends the launch.
constexpr unsigned long long kDefaultWaitPolls = 1ull << 24;
// HBM for the wide instances' own psi and lam: at most this share of the free
// memory (the rest take the separate whole-GPU path).
constexpr double kWideWorkspaceShare = 0.6;

enum BPassKind { BP_FWD = 0, BP_HAM = 1, BP_BWD = 2 };
enum BMode { BM_PAIR = 0, BM_DIAG_LOCAL = 1, BM_DIAG_GLOBAL = 2, BM_SWAP = 3 };
enum BGrad { BG_NONE = -1, BG_X = 0, BG_Y = 1, BG_Z = 2, BG_P1 = 3 };

struct BGate {
  int32_t kind;
  int32_t mode;
  uint32_t tbit, tbit2, l_ones;
  int32_t npos;
  uint8_t pos[16];
  uint64_t g_ones, g_zeros, g_tbit;
  int32_t param;      // instance-relative parameter whose angle this gate uses (-1: fixed)
  int32_t sign;       // +1: angle, -1: inverse gate (negated angle)
  int32_t grad;       // backward: BGrad mode of the gradient taken before un-applying
  int32_t gacc;       // backward: accumulator slot within the pass
  Coef c;
};

struct HTerm {
  double coeff;
  uint64_t x_local;   // X-part as a mask of local bits
  uint64_t x_global;  // X-part as a mask of qubits
  uint64_t z_mask;    // Z-part as a mask of qubits
  int32_t ny;         // number of Y factors (phase i^ny)
  int32_t pad;
};

struct BPass {
  uint32_t gate_begin, gate_count;
  uint32_t term_begin, term_count;
  int32_t kind, k, c, nhigh;
  int32_t first;      // FWD: synthesise |0..0>; HAM: lambda starts at 0
  int32_t nparams;    // BWD: accumulator slots used
  uint8_t lpos[16];
};

struct BInst {
  uint32_t n;
  uint32_t pass_begin, npass;
  int32_t resident;   // n <= k: the whole instance stays in shared memory
  int64_t param_offset;
  int32_t nparams;
  int32_t wide;       // >= 0: index of this wide instance (its completion counter); -1: whole-instance item
  uint64_t ws_offset; // wide: psi_re, psi_im, lam_re, lam_im (2^n doubles each) from here in wide_ws
};

constexpr uint32_t kWholeInstance = 0xFFFFFFFFu;

// One entry of the persistent kernel's queue.
struct BItem {
  uint32_t inst;
  uint32_t pass;        // kWholeInstance, or the instance-relative pass this item runs
  uint32_t need;        // wide: items of this instance that must be complete before this one starts
  uint32_t slot;        // wide HAM / BWD: first partial-sum slot this item writes
  uint64_t tile_begin, tile_end;
};

// Fold of partial-sum slots: out = factor * sum_{r < count} partials[base + r * stride].
struct BSum {
  uint64_t out;         // energies[out] (energy) or grads[out]
  uint64_t base;
  uint32_t stride, count;
  double factor;
  int32_t energy;
  int32_t pad;
};

struct BatchArgs {
  const BInst* inst;
  const BItem* items;
  uint32_t nitems;
  const BPass* passes;
  const BGate* gates;
  const HTerm* terms;
  double* energies;
  double* grads;
  double* workspace;      // per CTA: psi_re, psi_im, lam_re, lam_im of 2^ws_qubits each
  uint32_t ws_qubits;
  double* wide_ws;        // per wide instance (BInst::ws_offset)
  unsigned int* done;     // per wide instance: completed items
  double* partials;
  int* error;             // 0, or 1 after a wait ran out
  unsigned long long wait_limit;
  unsigned int* counter;
  int kmax;
};

__device__ __forceinline__ double bsum(double v, double* red) {
  for (int off = 16; off > 0; off >>= 1) v = dadd(v, __shfl_down_sync(0xffffffffu, v, off));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double r = 0.0;
  if (warp == 0) {
    r = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
    for (int off = 16; off > 0; off >>= 1) r = dadd(r, __shfl_down_sync(0xffffffffu, r, off));
  }
  __syncthreads();
  return r;  // thread 0
}

// Apply one gate to a tile (caller checked the non-local control predicate).
__device__ void b_apply(const BGate& g, uint64_t base, double* re, double* im, uint32_t T) {
  const uint32_t nw = T >> g.npos;
  switch (g.mode) {
    case BM_PAIR:
      switch (g.kind) {
        case SPZ_GATE_H: tile_pair_any<SPZ_GATE_H>(g, re, im, nw); break;
        case SPZ_GATE_X: tile_pair_any<SPZ_GATE_X>(g, re, im, nw); break;
        case SPZ_GATE_Y: tile_pair_any<SPZ_GATE_Y>(g, re, im, nw); break;
        case SPZ_GATE_RX: tile_pair_any<SPZ_GATE_RX>(g, re, im, nw); break;
        case SPZ_GATE_RY: tile_pair_any<SPZ_GATE_RY>(g, re, im, nw); break;
        default: tile_pair_any<SPZ_GATE_U>(g, re, im, nw); break;
      }
      break;
    case BM_DIAG_LOCAL:
    case BM_DIAG_GLOBAL: {
      int gone = -1;
      if (g.mode == BM_DIAG_GLOBAL) {
        gone = (base & g.g_tbit) ? 1 : 0;
        if (!gone && g.kind != SPZ_GATE_RZ) break;
      }
      switch (g.kind) {
        case SPZ_GATE_Z: tile_diag_any<SPZ_GATE_Z>(g, re, im, nw, gone); break;
        case SPZ_GATE_P: tile_diag_any<SPZ_GATE_P>(g, re, im, nw, gone); break;
        default: tile_diag_any<SPZ_GATE_RZ>(g, re, im, nw, gone); break;
      }
      break;
    }
    default:
      tile_swap_any(g, re, im, nw);
  }
}

// Backward step of one gate on a tile, in one loop over the gate's pairs (or
// elements): this thread's share of the gradient term Im<lam| Pi sigma |psi>
// when the gate carries a parameter, taken from psi and lam as they are before
// the step, then the inverse gate (the descriptor already holds it) on both.
// X and Y generators pair s0 with s1 (the target is local); the diagonal
// generators (Z for RZ, |1><1| for P) are elementwise, sum over x of
// +-Im(conj(lam_x) psi_x), with the target bit read from the element or, for a
// non-local target, from the tile base (gone).
template <int KIND, int NPOS>
__device__ __forceinline__ double b_bwd_pair(const BGate& g, double* pr, double* pi, double* lr, double* li,
                                             uint32_t nw) {
  const Enumerator<NPOS, BGate> E(g);
  const uint32_t tbit = g.tbit;
  const Coef cf = g.c;
  const int grad = g.grad;
  double acc = 0.0;
  for (uint32_t m = threadIdx.x; m < nw; m += blockDim.x) {
    const uint32_t s0 = E(m), s1 = s0 | tbit;
    double a = pr[s0], b = pi[s0], c = pr[s1], d = pi[s1];
    double p = lr[s0], q = li[s0], r = lr[s1], s = li[s1];
    if (grad != BG_NONE) {
      double v;
      switch (grad) {
        case BG_X: v = dadd(dfma(p, d, dmul(dneg(q), c)), dfma(r, b, dmul(dneg(s), a))); break;
        case BG_Y: v = dsub(dfma(r, a, dmul(s, b)), dfma(p, c, dmul(q, d))); break;
        case BG_Z: v = dsub(dfma(p, b, dmul(dneg(q), a)), dfma(r, d, dmul(dneg(s), c))); break;
        default: v = dfma(r, d, dmul(dneg(s), c)); break;
      }
      acc = dadd(acc, v);
    }
    gate_pair<KIND>(cf, a, b, c, d);
    gate_pair<KIND>(cf, p, q, r, s);
    pr[s0] = a; pi[s0] = b; pr[s1] = c; pi[s1] = d;
    lr[s0] = p; li[s0] = q; lr[s1] = r; li[s1] = s;
  }
  return acc;
}

template <int KIND, int NPOS>
__device__ __forceinline__ double b_bwd_diag(const BGate& g, int gone, double* pr, double* pi, double* lr, double* li,
                                             uint32_t nw) {
  const Enumerator<NPOS, BGate> E(g);
  const uint32_t tbit = g.tbit;
  const Coef cf = g.c;
  const int grad = g.grad;
  double acc = 0.0;
  for (uint32_t m = threadIdx.x; m < nw; m += blockDim.x) {
    const uint32_t e = E(m);
    const bool one = gone >= 0 ? gone != 0 : (e & tbit) != 0;
    double a = pr[e], b = pi[e], p = lr[e], q = li[e];
    if (grad != BG_NONE && !(grad == BG_P1 && !one)) {
      const double v = dfma(p, b, dmul(dneg(q), a));  // Im(conj(lam) psi)
      acc = (grad == BG_Z && one) ? dsub(acc, v) : dadd(acc, v);
    }
    gate_diag<KIND>(cf, one, a, b);
    gate_diag<KIND>(cf, one, p, q);
    pr[e] = a; pi[e] = b; lr[e] = p; li[e] = q;
  }
  return acc;
}

template <int KIND>
__device__ __forceinline__ double b_bwd_pair_any(const BGate& g, double* pr, double* pi, double* lr, double* li,
                                                 uint32_t nw) {
  double r = 0.0;
#define SPZ_CALL(N) r = b_bwd_pair<KIND, N>(g, pr, pi, lr, li, nw)
  SPZ_BY_NPOS(g.npos, SPZ_CALL)
#undef SPZ_CALL
  return r;
}

template <int KIND>
__device__ __forceinline__ double b_bwd_diag_any(const BGate& g, int gone, double* pr, double* pi, double* lr,
                                                 double* li, uint32_t nw) {
  double r = 0.0;
#define SPZ_CALL(N) r = b_bwd_diag<KIND, N>(g, gone, pr, pi, lr, li, nw)
  SPZ_BY_NPOS(g.npos, SPZ_CALL)
#undef SPZ_CALL
  return r;
}

// This thread's gradient share of gate g on the tile, with g applied to psi and lam.
__device__ double b_bwd_gate(const BGate& g, uint64_t base, double* pr, double* pi, double* lr, double* li,
                             uint32_t T) {
  const uint32_t nw = T >> g.npos;
  double v = 0.0;
  switch (g.mode) {
    case BM_PAIR:
      switch (g.kind) {
        case SPZ_GATE_H: v = b_bwd_pair_any<SPZ_GATE_H>(g, pr, pi, lr, li, nw); break;
        case SPZ_GATE_X: v = b_bwd_pair_any<SPZ_GATE_X>(g, pr, pi, lr, li, nw); break;
        case SPZ_GATE_Y: v = b_bwd_pair_any<SPZ_GATE_Y>(g, pr, pi, lr, li, nw); break;
        case SPZ_GATE_RX: v = b_bwd_pair_any<SPZ_GATE_RX>(g, pr, pi, lr, li, nw); break;
        case SPZ_GATE_RY: v = b_bwd_pair_any<SPZ_GATE_RY>(g, pr, pi, lr, li, nw); break;
        default: v = b_bwd_pair_any<SPZ_GATE_U>(g, pr, pi, lr, li, nw); break;
      }
      break;
    case BM_DIAG_LOCAL:
    case BM_DIAG_GLOBAL: {
      int gone = -1;
      if (g.mode == BM_DIAG_GLOBAL) {
        gone = (base & g.g_tbit) ? 1 : 0;
        if (!gone && g.kind != SPZ_GATE_RZ) break;  // Z / P (and the P1 gradient) live on the 1 half
      }
      switch (g.kind) {
        case SPZ_GATE_Z: v = b_bwd_diag_any<SPZ_GATE_Z>(g, gone, pr, pi, lr, li, nw); break;
        case SPZ_GATE_P: v = b_bwd_diag_any<SPZ_GATE_P>(g, gone, pr, pi, lr, li, nw); break;
        default: v = b_bwd_diag_any<SPZ_GATE_RZ>(g, gone, pr, pi, lr, li, nw); break;
      }
      break;
    }
    default:
      tile_swap_any(g, pr, pi, nw);
      tile_swap_any(g, lr, li, nw);
  }
  return v;
}

__device__ __forceinline__ uint64_t b_global(uint64_t base, const uint64_t* rowoff, uint32_t e, int c) {
  return base | rowoff[e >> c] | (e & ((1u << c) - 1));
}

struct BSmem {
  double *pr, *pi, *lr, *li;
  uint64_t* rowoff;
  double* red;
  double* gacc;
};

// One pass of instance I over tiles [t0, t1): load each tile (or synthesise
// |0...0>), apply the pass's work, store it back.  wpr .. wli: the instance's
// psi and lam in HBM (unused when resident).  Energy terms add into *s_energy
// (thread 0), gradient parts into S.gacc (zeroed here).  Workspace loads
// bypass L1 (ld.global.cg): a wide instance's tiles are written by other CTAs.
__device__ void run_pass(const BatchArgs& A, const BInst& I, const BPass& P, uint64_t t0, uint64_t t1, double* wpr,
                         double* wpi, double* wlr, double* wli, const BSmem& S, double* s_energy) {
  const int K = P.k, C = P.c;
  const uint32_t T = 1u << K;
  double* pr = S.pr;
  // A forward pass (psi only) may use a tile twice the shared-memory layout's:
  // its imaginary parts then take the space of lam's real parts.
  double* pi = K > A.kmax ? pr + T : S.pi;
  double* lr = S.lr;
  double* li = S.li;
  uint64_t* rowoff = S.rowoff;
  if (!I.resident) {
    for (uint32_t r = threadIdx.x; r < (1u << P.nhigh); r += blockDim.x) {
      uint64_t off = 0;
      for (int j = 0; j < P.nhigh; ++j)
        if ((r >> j) & 1) off |= 1ull << P.lpos[C + j];
      rowoff[r] = off;
    }
  }
  const int nwarps = (int)(blockDim.x >> 5), warp = (int)(threadIdx.x >> 5), lane = (int)(threadIdx.x & 31);
  if (P.kind == BP_BWD)
    for (int j = threadIdx.x; j < nwarps * kMaxPassParams; j += blockDim.x) S.gacc[j] = 0.0;
  __syncthreads();
  for (uint64_t tile = t0; tile < t1; ++tile) {
    const uint64_t base = I.resident ? 0 : deposit(tile, P.lpos, K);
    // ---- load
    if (P.kind == BP_FWD && P.first) {
      for (uint32_t e = threadIdx.x; e < T; e += blockDim.x) {
        const uint64_t gi = I.resident ? e : b_global(base, rowoff, e, C);
        pr[e] = gi == 0 ? 1.0 : 0.0;
        pi[e] = 0.0;
      }
    } else if (!I.resident) {
      for (uint32_t e2 = threadIdx.x; e2 < T / 2; e2 += blockDim.x) {
        const uint32_t e = 2 * e2;
        const uint64_t gi = b_global(base, rowoff, e, C);
        *reinterpret_cast<double2*>(pr + e) = __ldcg(reinterpret_cast<const double2*>(wpr + gi));
        *reinterpret_cast<double2*>(pi + e) = __ldcg(reinterpret_cast<const double2*>(wpi + gi));
        if (P.kind == BP_BWD || (P.kind == BP_HAM && !P.first)) {
          *reinterpret_cast<double2*>(lr + e) = __ldcg(reinterpret_cast<const double2*>(wlr + gi));
          *reinterpret_cast<double2*>(li + e) = __ldcg(reinterpret_cast<const double2*>(wli + gi));
        }
      }
    }
    __syncthreads();
    // ---- work
    if (P.kind == BP_FWD) {
      for (uint32_t gi = 0; gi < P.gate_count; ++gi) {
        const BGate& g = A.gates[P.gate_begin + gi];
        if ((base & g.g_ones) != g.g_ones || (base & g.g_zeros) != 0) continue;
        b_apply(g, base, pr, pi, T);
        __syncthreads();
      }
    } else if (P.kind == BP_HAM) {
      double eacc = 0.0;
      for (uint32_t e = threadIdx.x; e < T; e += blockDim.x) {
        const uint64_t gx = I.resident ? e : b_global(base, rowoff, e, C);
        double dr = 0.0, di = 0.0;
        for (uint32_t k = 0; k < P.term_count; ++k) {
          const HTerm& h = A.terms[P.term_begin + k];
          const uint32_t ye = e ^ (uint32_t)h.x_local;
          const uint64_t gy = gx ^ h.x_global;
          double cf = (__popcll(gy & h.z_mask) & 1) ? dneg(h.coeff) : h.coeff;
          const int ny = h.ny & 3;
          if (ny >= 2) cf = dneg(cf);
          const double yr = pr[ye], yi = pi[ye];
          if (ny & 1) {  // i * cf * psi_y
            dr = dfma(dneg(cf), yi, dr);
            di = dfma(cf, yr, di);
          } else {
            dr = dfma(cf, yr, dr);
            di = dfma(cf, yi, di);
          }
        }
        eacc = dadd(eacc, dfma(pr[e], dr, dmul(pi[e], di)));
        if (P.first) {
          lr[e] = dr;
          li[e] = di;
        } else {
          lr[e] = dadd(lr[e], dr);
          li[e] = dadd(li[e], di);
        }
      }
      const double es = bsum(eacc, S.red);
      if (threadIdx.x == 0) *s_energy = dadd(*s_energy, es);
    } else {  // BP_BWD
      for (uint32_t gi = 0; gi < P.gate_count; ++gi) {
        const BGate& g = A.gates[P.gate_begin + gi];
        if ((base & g.g_ones) != g.g_ones || (base & g.g_zeros) != 0) continue;
        double part = b_bwd_gate(g, base, pr, pi, lr, li, T);
        if (g.grad != BG_NONE) {  // uniform: this warp's share, into its own accumulator
          for (int off = 16; off > 0; off >>= 1) part = dadd(part, __shfl_down_sync(0xffffffffu, part, off));
          if (lane == 0) S.gacc[warp * kMaxPassParams + g.gacc] = dadd(S.gacc[warp * kMaxPassParams + g.gacc], part);
        }
        __syncthreads();
      }
    }
    __syncthreads();
    // ---- store
    if (!I.resident) {
      const bool store_psi = P.kind != BP_HAM;
      const bool store_lam = P.kind != BP_FWD;
      for (uint32_t e2 = threadIdx.x; e2 < T / 2; e2 += blockDim.x) {
        const uint32_t e = 2 * e2;
        const uint64_t gi = b_global(base, rowoff, e, C);
        if (store_psi) {
          *reinterpret_cast<double2*>(wpr + gi) = *reinterpret_cast<const double2*>(pr + e);
          *reinterpret_cast<double2*>(wpi + gi) = *reinterpret_cast<const double2*>(pi + e);
        }
        if (store_lam) {
          *reinterpret_cast<double2*>(wlr + gi) = *reinterpret_cast<const double2*>(lr + e);
          *reinterpret_cast<double2*>(wli + gi) = *reinterpret_cast<const double2*>(li + e);
        }
      }
    }
    __syncthreads();
  }
  if (P.kind == BP_BWD) {  // the warps' accumulators, summed in warp order, into row 0
    for (int j = threadIdx.x; j < P.nparams; j += blockDim.x) {
      double v = S.gacc[j];
      for (int w = 1; w < nwarps; ++w) v = dadd(v, S.gacc[w * kMaxPassParams + j]);
      S.gacc[j] = v;
    }
    __syncthreads();
  }
}

__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_volatile_int(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

// Thread 0 waits until *ctr >= need, at most A.wait_limit polls; returns false
// (in every thread) on timeout, after setting the error flag, or when another
// CTA already set it.
__device__ bool wait_until(const BatchArgs& A, const unsigned int* ctr, unsigned int need, int* s_flag) {
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned long long polls = 0;
    while (ld_acquire_gpu(ctr) < need) {
      if (ld_volatile_int(A.error)) {
        ok = 0;
        break;
      }
      if (++polls > A.wait_limit) {
        atomicCAS(A.error, 0, 1);
        ok = 0;
        break;
      }
      __nanosleep(256);
    }
    *s_flag = ok;
  }
  __syncthreads();
  const bool ok = *s_flag != 0;
  __syncthreads();
  return ok;
}

// Copy a pass descriptor to shared memory, so that the pass reads it without
// global loads after every block barrier.  Barriers on both sides: the previous
// pass's readers are done before it is overwritten.
__device__ __forceinline__ const BPass& stage_pass(const BPass* src, BPass* dst) {
  static_assert(sizeof(BPass) % 4 == 0, "BPass is copied as 32-bit words");
  __syncthreads();
  if (threadIdx.x < sizeof(BPass) / 4)
    reinterpret_cast<uint32_t*>(dst)[threadIdx.x] = reinterpret_cast<const uint32_t*>(src)[threadIdx.x];
  __syncthreads();
  return *dst;
}

// Instantiated for the default 64-thread CTAs (12 per SM: up to 85 registers
// a thread) and for CTAs of up to 1024 threads (64 registers a thread).
template <int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) batch_kernel(BatchArgs A) {
  extern __shared__ double sm[];
  const uint32_t TMAX = 1u << A.kmax;
  BSmem S;
  S.pr = sm;
  S.pi = sm + TMAX;
  S.lr = sm + 2 * TMAX;
  S.li = sm + 3 * TMAX;
  S.rowoff = reinterpret_cast<uint64_t*>(sm + 4 * TMAX);
  S.red = sm + 4 * TMAX + ((2 * TMAX) >> kBatchLowBits);  // after the row table (sized for forward tiles)
  S.gacc = S.red + (blockDim.x >> 5);  // the block reduction needs one slot per warp
  __shared__ unsigned int s_next;
  __shared__ int s_flag;
  __shared__ double s_energy;
  __shared__ BPass s_pass;
  const uint64_t wsN = 1ull << A.ws_qubits;
  double* wpr = A.workspace ? A.workspace + (uint64_t)blockIdx.x * 4 * wsN : nullptr;
  double* wpi = wpr ? wpr + wsN : nullptr;
  double* wlr = wpr ? wpr + 2 * wsN : nullptr;
  double* wli = wpr ? wpr + 3 * wsN : nullptr;

  for (;;) {
    if (threadIdx.x == 0) s_next = ld_volatile_int(A.error) ? A.nitems : atomicAdd(A.counter, 1u);
    __syncthreads();
    const unsigned int q = s_next;
    __syncthreads();
    if (q >= A.nitems) break;
    const BItem W = A.items[q];
    const BInst I = A.inst[W.inst];
    if (threadIdx.x == 0) s_energy = 0.0;
    __syncthreads();
    if (W.pass == kWholeInstance) {
      for (uint32_t pidx = 0; pidx < I.npass; ++pidx) {
        const BPass& P = stage_pass(A.passes + I.pass_begin + pidx, &s_pass);
        run_pass(A, I, P, 0, 1ull << (I.n - P.k), wpr, wpi, wlr, wli, S, &s_energy);
        if (P.kind == BP_BWD) {
          for (uint32_t gi = threadIdx.x; gi < P.gate_count; gi += blockDim.x) {
            const BGate& g = A.gates[P.gate_begin + gi];
            if (g.grad != BG_NONE) {
              const double v = S.gacc[g.gacc];
              A.grads[I.param_offset + g.param] = g.grad == BG_P1 ? dmul(-2.0, v) : v;
            }
          }
          __syncthreads();
        }
      }
      if (threadIdx.x == 0) A.energies[W.inst] = s_energy;
      __syncthreads();
      continue;
    }
    // one pass of a wide instance over a tile range
    if (!wait_until(A, A.done + I.wide, W.need, &s_flag)) break;
    const BPass& P = stage_pass(A.passes + I.pass_begin + W.pass, &s_pass);
    const uint64_t N = 1ull << I.n;
    double* ipr = A.wide_ws + I.ws_offset;
    run_pass(A, I, P, W.tile_begin, W.tile_end, ipr, ipr + N, ipr + 2 * N, ipr + 3 * N, S, &s_energy);
    if (P.kind == BP_HAM) {
      if (threadIdx.x == 0) A.partials[W.slot] = s_energy;
    } else if (P.kind == BP_BWD) {
      for (int j = threadIdx.x; j < P.nparams; j += blockDim.x) A.partials[W.slot + j] = S.gacc[j];
    }
    __syncthreads();  // every thread's tile stores and partials are issued
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(A.done + I.wide, 1u);
    }
  }
}

// The wide instances' energies and gradients from their items' partial sums,
// each a sequential sum in item order.
__global__ void batch_fold_kernel(const BSum* __restrict__ sums, uint32_t nsums, const double* __restrict__ partials,
                                  double* __restrict__ energies, double* __restrict__ grads) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsums) return;
  const BSum f = sums[i];
  double v = 0.0;
  for (uint32_t r = 0; r < f.count; ++r) v = dadd(v, partials[f.base + (uint64_t)r * f.stride]);
  v = dmul(f.factor, v);
  if (f.energy) energies[f.out] = v;
  else grads[f.out] = v;
}

const void* batch_kernel_fn(int threads) {
  return threads <= 64 ? (const void*)batch_kernel<64, 12> : (const void*)batch_kernel<1024, 1>;
}

// Coefficients of every parameterised gate from the current angles.
struct CoefJob {
  uint32_t gate;
  int32_t kind;
  int64_t theta_index;
  int32_t sign;
  int32_t pad;
};

__global__ void batch_coef_kernel(BGate* gates, const CoefJob* jobs, uint32_t njobs, const double* theta) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= njobs) return;
  const CoefJob j = jobs[i];
  const double th = j.sign > 0 ? theta[j.theta_index] : -theta[j.theta_index];
  Coef& c = gates[j.gate].c;
  double s, co;
  switch (j.kind) {
    case SPZ_GATE_P:
      sincos(th, &s, &co);
      c.sn = s; c.cs = co; c.nsn = -s;
      break;
    case SPZ_GATE_RX:
      sincos(th * 0.5, &s, &co);
      c.cs = co; c.nsn = -s; c.sn = s;
      break;
    case SPZ_GATE_RY:
      sincos(th * 0.5, &s, &co);
      c.sn = s; c.cs = co; c.nsn = -s;
      break;
    default:  // RZ
      sincos(th * 0.5, &s, &co);
      c.d0re = co; c.d0im = -s; c.d1re = co; c.d1im = s;
      break;
  }
}

BGate to_bgate(const GateApp& g, const std::vector<int>& local) {
  int where[64];
  for (int q = 0; q < 64; ++q) where[q] = -1;
  for (size_t j = 0; j < local.size(); ++j) where[local[j]] = (int)j;
  BGate t{};
  t.kind = g.kind;
  t.c = g.c;
  t.param = -1;
  t.sign = 1;
  t.grad = BG_NONE;
  uint32_t l_ones = 0, l_zeros = 0;
  for (int q = 0; q < 64; ++q) {
    const uint64_t b = 1ull << q;
    if (g.ones & b) {
      if (where[q] >= 0) l_ones |= 1u << where[q]; else t.g_ones |= b;
    }
    if (g.zeros & b) {
      if (where[q] >= 0) l_zeros |= 1u << where[q]; else t.g_zeros |= b;
    }
  }
  uint32_t special = l_ones | l_zeros;
  if (g.kind == SPZ_GATE_SWAP) {
    t.mode = BM_SWAP;
    t.tbit = 1u << where[g.target];
    t.tbit2 = 1u << where[g.target2];
    special |= t.tbit | t.tbit2;
  } else if (is_diagonal(g.kind)) {
    if (where[g.target] >= 0) {
      t.mode = BM_DIAG_LOCAL;
      t.tbit = 1u << where[g.target];
      if (g.kind != SPZ_GATE_RZ) {
        special |= t.tbit;
        l_ones |= t.tbit;
      }
    } else {
      t.mode = BM_DIAG_GLOBAL;
      t.g_tbit = 1ull << g.target;
    }
  } else {
    t.mode = BM_PAIR;
    t.tbit = 1u << where[g.target];
    special |= t.tbit;
  }
  t.l_ones = l_ones;
  for (int j = 0; j < 32; ++j)
    if ((special >> j) & 1) t.pos[t.npos++] = (uint8_t)j;
  return t;
}

spz_gate inverse_of(const spz_gate& g) {
  spz_gate r = g;
  switch (g.kind) {
    case SPZ_GATE_P: case SPZ_GATE_RX: case SPZ_GATE_RY: case SPZ_GATE_RZ: r.p[0] = -g.p[0]; break;
    case SPZ_GATE_U: r.p[0] = -g.p[0]; r.p[1] = -g.p[2]; r.p[2] = -g.p[1]; break;
    default: break;
  }
  return r;
}

}  // namespace

// An instance run across the whole GPU (fused executor + fused adjoint sweep).
struct WideInst {
  uint32_t idx = 0, n = 0;
  std::vector<spz_op> ops;            // angles of parameter ops are set per run
  std::vector<uint32_t> pidx;         // instance-relative op of each parameter
  std::vector<spz_pauli_term> terms;
  uint64_t param_offset = 0;
  double cost = 0.0;
};

struct BatchImpl {
  int device = 0;
  // 2^9 tiles x 64 threads (12 CTAs per SM): the batch of 4096 instances of 10-22
  // qubits, the wide ones as work items) in 25.7 s, against 26.7 s with 2^10 x
  // 128, 28.2 s with 2^11 x 128, 26.9 s with 2^9 x 128 and with 2^8 x 64.
  int kmax = 9, threads = 64;
  int wide_qubits = kDefaultWideQubits;
  uint32_t wide_flags = 0;            // SPZ_EXEC_FAST: wide instances use the fast adjoint
  uint32_t nnarrow = 0;               // instances in the persistent kernel
  std::vector<WideInst> wide;         // the others, largest first
  // Wide instances run on kWideStreams streams at once (a pass of one 20-22
  // qubit instance leaves block slots empty; another instance fills them),
  // each stream with its own state per size (lazily created).
  int wide_streams = kDefaultWideStreams;
  cudaStream_t wide_stream[kWideStreams] = {};
  cudaEvent_t wide_done[kWideStreams] = {};
  spz_state_t wide_h[kWideStreams][31] = {};
  uint32_t ninst = 0;
  uint64_t nparams_total = 0;
  uint32_t ws_qubits = 0;
  int grid = 0;
  size_t smem = 0;
  cudaStream_t stream = nullptr;
  // wide instances inside the persistent kernel (work items)
  int tiles_per_item = kDefaultTilesPerItem;
  uint32_t nitems = 0, nwide_items = 0, nwide_in_kernel = 0, nsums = 0;
  uint64_t npartials = 0, wide_ws_doubles = 0;
  unsigned long long wait_limit = kDefaultWaitPolls;
  bool stall_for_test = false;
  // device
  BInst* d_inst = nullptr;
  BItem* d_items = nullptr;
  BSum* d_sums = nullptr;
  double* d_partials = nullptr;
  double* d_wide_ws = nullptr;
  unsigned int* d_done = nullptr;
  int* d_error = nullptr;
  int* h_error = nullptr;
  BPass* d_pass = nullptr;
  BGate* d_gates = nullptr;
  HTerm* d_terms = nullptr;
  CoefJob* d_jobs = nullptr;
  uint32_t njobs = 0;
  double* d_theta = nullptr;
  double* d_energy = nullptr;
  double* d_grad = nullptr;
  double* d_ws = nullptr;
  unsigned int* d_counter = nullptr;
  // pinned staging
  double* h_theta = nullptr;
  double* h_energy = nullptr;
  double* h_grad = nullptr;
  cudaGraphExec_t graph = nullptr;
  // plan statistics
  uint64_t fwd_passes = 0, ham_passes = 0, bwd_passes = 0, resident = 0;
};

}  // namespace spz

struct spz_batch_s : spz::BatchImpl {};

namespace spz {
namespace {

void free_batch(spz_batch_t b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (int si = 0; si < kWideStreams; ++si) {
    for (spz_state_t w : b->wide_h[si])
      if (w) spz_state_destroy(w);
    if (b->wide_done[si]) cudaEventDestroy(b->wide_done[si]);
    if (b->wide_stream[si]) cudaStreamDestroy(b->wide_stream[si]);
  }
  cudaFree(b->d_inst); cudaFree(b->d_items); cudaFree(b->d_sums); cudaFree(b->d_partials); cudaFree(b->d_wide_ws);
  cudaFree(b->d_done); cudaFree(b->d_error); cudaFreeHost(b->h_error);
  cudaFree(b->d_pass); cudaFree(b->d_gates); cudaFree(b->d_terms);
  cudaFree(b->d_jobs); cudaFree(b->d_theta); cudaFree(b->d_energy); cudaFree(b->d_grad); cudaFree(b->d_ws);
  cudaFree(b->d_counter);
  cudaFreeHost(b->h_theta); cudaFreeHost(b->h_energy); cudaFreeHost(b->h_grad);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

template <typename T>
int upload(T** dst, const std::vector<T>& src) {
  const size_t bytes = std::max<size_t>(1, src.size()) * sizeof(T);
  SPZ_CUDA(dev_alloc((void**)dst, bytes));
  if (!src.empty()) SPZ_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return SPZ_OK;
}

int build_batch(spz_batch_t b, const spz_batch_instance* inst, size_t ninst, const spz_op* ops,
                const uint32_t* param_index, const spz_pauli_term* terms) {
  std::vector<BInst> vinst(ninst);
  std::vector<BPass> vpass;
  std::vector<BGate> vgates;
  std::vector<HTerm> vterms;
  std::vector<CoefJob> jobs;
  std::vector<double> cost(ninst);
  uint64_t ptotal = 0;
  uint32_t ws_qubits = 0;
  std::vector<uint32_t> narrow, wide_in;
  std::vector<int32_t> wide_index(ninst, -1);
  size_t free_b = 0, total_b = 0;
  SPZ_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const uint64_t wide_budget = (uint64_t)(kWideWorkspaceShare * (double)free_b);
  uint64_t wide_ws = 0;
  for (size_t ii = 0; ii < ninst; ++ii) {
    const spz_batch_instance& in = inst[ii];
    const uint32_t n = in.n;
    if (n == 0 || n > 30) return fail(SPZ_ERR_INVALID_ARGUMENT, "batch instance qubits must be in 1..30");
    // Wide instances run as work items inside the persistent kernel, with
    // their own psi and lam in HBM, when the workspace fits; the fast adjoint
    // (SPZ_EXEC_FAST) and anything beyond the budget take the whole-GPU path.
    const bool wide = (int)n >= b->wide_qubits && (int)n > b->kmax;
    const uint64_t ws_need = 4ull * (1ull << n);
    const bool in_kernel = wide && !(b->wide_flags & (SPZ_EXEC_FAST | SPZ_BATCH_WIDE_APART)) &&
                           (wide_ws + ws_need) * 8 <= wide_budget;
    if (wide && in_kernel) {
      wide_index[ii] = (int32_t)wide_in.size();
      wide_in.push_back((uint32_t)ii);
      wide_ws += ws_need;
    }
    if (wide && !in_kernel) {  // whole-GPU path: keep the instance's own lists
      WideInst w;
      w.idx = (uint32_t)ii;
      w.n = n;
      w.ops.assign(ops + in.op_offset, ops + in.op_offset + in.nops);
      w.pidx.assign(param_index + in.param_offset, param_index + in.param_offset + in.nparams);
      w.terms.assign(terms + in.term_offset, terms + in.term_offset + in.nterms);
      w.param_offset = in.param_offset;
      w.cost = (double)(in.nops + 8) * (double)(1ull << n);
      for (uint32_t j = 0; j < in.nparams; ++j) {
        if (w.pidx[j] >= in.nops) return fail(SPZ_ERR_INVALID_ARGUMENT, "batch param_index out of range");
        const int kind = w.ops[w.pidx[j]].gate.kind;
        if (kind != SPZ_GATE_RX && kind != SPZ_GATE_RY && kind != SPZ_GATE_RZ && kind != SPZ_GATE_P)
          return fail(SPZ_ERR_UNSUPPORTED, "only P, RX, RY and RZ angles can be batch parameters");
      }
      for (const spz_op& op : w.ops)
        if (op.gate.kind == SPZ_GATE_M || op.gate.kind == SPZ_GATE_BITFLIP)
          return fail(SPZ_ERR_UNSUPPORTED, "measurements and noise cannot be batched");
      ptotal = std::max<uint64_t>(ptotal, in.param_offset + in.nparams);
      b->wide.push_back(std::move(w));
      continue;
    }
    if (!wide) narrow.push_back((uint32_t)ii);
    const int k = std::min<int>((int)n, b->kmax);
    const int c = std::min<int>(kBatchLowBits, k);
    // forward gate list (+ which op carries which parameter)
    std::vector<int> param_of_op(in.nops, -1);
    for (uint32_t j = 0; j < in.nparams; ++j) {
      const uint32_t op = param_index[in.param_offset + j];
      if (op >= in.nops) return fail(SPZ_ERR_INVALID_ARGUMENT, "batch param_index out of range");
      if (param_of_op[op] >= 0) return fail(SPZ_ERR_INVALID_ARGUMENT, "an op carries two parameters");
      const int kind = ops[in.op_offset + op].gate.kind;
      if (kind != SPZ_GATE_RX && kind != SPZ_GATE_RY && kind != SPZ_GATE_RZ && kind != SPZ_GATE_P)
        return fail(SPZ_ERR_UNSUPPORTED, "only P, RX, RY and RZ angles can be batch parameters");
      param_of_op[op] = (int)j;
    }
    std::vector<GateApp> fwd;
    std::vector<spz_gate> fwd_gate;
    for (uint32_t o = 0; o < in.nops; ++o) {
      const spz_op& op = ops[in.op_offset + o];
      if (op.gate.kind == SPZ_GATE_M || op.gate.kind == SPZ_GATE_BITFLIP)
        return fail(SPZ_ERR_UNSUPPORTED, "measurements and noise cannot be batched");
      uint64_t ones = 0, zeros = 0;
      if (op.controls_kind == SPZ_CONTROLS_MIXED) {
        ones = op.controls & ~op.zeros;
        zeros = op.zeros;
      } else if (op.controls_kind != SPZ_CONTROLS_NONE) {
        ones = op.controls;
      }
      GateApp a;
      int rc = make_gate_app(n, op.gate, op.target, ones, zeros, &a);
      if (rc) return rc;
      a.src = o;
      fwd.push_back(a);
      fwd_gate.push_back(op.gate);
    }
    BInst& I = vinst[ii];
    I.n = n;
    I.pass_begin = (uint32_t)vpass.size();
    I.resident = (int)n <= b->kmax;
    I.param_offset = (int64_t)in.param_offset;
    I.nparams = (int)in.nparams;
    I.wide = wide_index[ii];
    ptotal = std::max<uint64_t>(ptotal, in.param_offset + in.nparams);
    if (!I.resident && I.wide < 0) ws_qubits = std::max<uint32_t>(ws_qubits, n);
    // forward passes (a resident instance is one pass over all n qubits, in program order)
    std::vector<int> all_local(n);
    std::iota(all_local.begin(), all_local.end(), 0);
    std::vector<PlannedPass> fp;
    if (I.resident) {
      if (!fwd.empty()) fp.push_back(PlannedPass{all_local, fwd});
    } else {
      // forward passes hold psi only, so their tiles may be twice as large
      fp = plan_passes(fwd, n, std::min<int>((int)n, b->kmax + 1), c);
    }
    std::vector<GateApp> applied;  // in the order the passes apply them
    bool first = true;
    for (const PlannedPass& P : fp) {
      BPass bp{};
      bp.kind = BP_FWD;
      bp.k = (int)P.local.size();
      bp.c = c;
      bp.nhigh = bp.k - c;
      bp.first = first;
      first = false;
      for (int j = 0; j < bp.k; ++j) bp.lpos[j] = (uint8_t)P.local[j];
      bp.gate_begin = (uint32_t)vgates.size();
      for (const GateApp& g : P.gates) {
        BGate t = to_bgate(g, P.local);
        const int pj = param_of_op[g.src];
        if (pj >= 0) {
          t.param = pj;
          jobs.push_back(CoefJob{(uint32_t)vgates.size(), g.kind, (int64_t)in.param_offset + pj, 1, 0});
        }
        vgates.push_back(t);
        applied.push_back(g);
      }
      bp.gate_count = (uint32_t)(vgates.size() - bp.gate_begin);
      vpass.push_back(bp);
      b->fwd_passes++;
    }
    if (fp.empty()) {  // no gates: one empty first pass to set |0...0>
      BPass bp{};
      bp.kind = BP_FWD; bp.k = k; bp.c = c; bp.nhigh = k - c; bp.first = 1;
      for (int j = 0; j < k; ++j) bp.lpos[j] = (uint8_t)j;
      bp.gate_begin = (uint32_t)vgates.size();
      vpass.push_back(bp);
    }
    // Hamiltonian passes: diagonal terms in the first; X-type terms in passes
    // whose local set covers their X bits.
    std::vector<int> done(in.nterms, 0);
    size_t remaining = in.nterms;
    bool hfirst = true;
    while (remaining > 0 || hfirst) {
      uint64_t L = (c >= 64) ? ~0ull : ((1ull << c) - 1);
      int nl = c;
      std::vector<uint32_t> take;
      for (uint32_t t = 0; t < in.nterms; ++t) {
        if (done[t]) continue;
        const spz_pauli_term& tm = terms[in.term_offset + t];
        if (n < 64 && ((tm.x_mask | tm.z_mask) >> n) != 0)
          return fail(SPZ_ERR_INVALID_ARGUMENT, "Pauli term acts on a qubit out of range");
        const uint64_t need = tm.x_mask & ~L;
        const int add = __builtin_popcountll(need);
        if (nl + add <= k) {
          L |= need;
          nl += add;
          take.push_back(t);
        } else if (__builtin_popcountll(tm.x_mask) > k) {
          return fail(SPZ_ERR_UNSUPPORTED, "Pauli term with more X/Y qubits than a tile holds");
        }
      }
      for (int q = 0; q < (int)n && nl < k; ++q)
        if (!((L >> q) & 1)) { L |= 1ull << q; nl++; }
      std::vector<int> local;
      for (int q = 0; q < (int)n; ++q)
        if ((L >> q) & 1) local.push_back(q);
      int where[64];
      for (int q = 0; q < 64; ++q) where[q] = -1;
      for (size_t j = 0; j < local.size(); ++j) where[local[j]] = (int)j;
      BPass bp{};
      bp.kind = BP_HAM;
      bp.k = (int)local.size();
      bp.c = c;
      bp.nhigh = bp.k - c;
      bp.first = hfirst;
      hfirst = false;
      for (int j = 0; j < bp.k; ++j) bp.lpos[j] = (uint8_t)local[j];
      bp.term_begin = (uint32_t)vterms.size();
      for (uint32_t t : take) {
        const spz_pauli_term& tm = terms[in.term_offset + t];
        HTerm h{};
        h.coeff = tm.coeff;
        h.x_global = tm.x_mask;
        h.z_mask = tm.z_mask;
        h.ny = __builtin_popcountll(tm.x_mask & tm.z_mask);
        for (int q = 0; q < 64; ++q)
          if ((tm.x_mask >> q) & 1) h.x_local |= 1ull << where[q];
        vterms.push_back(h);
        done[t] = 1;
        remaining--;
      }
      bp.term_count = (uint32_t)(vterms.size() - bp.term_begin);
      vpass.push_back(bp);
      b->ham_passes++;
    }
    // backward: the applied order reversed, as inverse gates with gradients
    std::vector<GateApp> bwd;
    for (size_t j = applied.size(); j-- > 0;) {
      GateApp inv;
      int rc = make_gate_app(n, inverse_of(fwd_gate[applied[j].src]), applied[j].target, applied[j].ones,
                             applied[j].zeros, &inv);
      if (rc) return rc;
      inv.src = applied[j].src;
      bwd.push_back(inv);
    }
    std::vector<PlannedPass> bp_list;
    if (I.resident) {
      if (!bwd.empty()) bp_list.push_back(PlannedPass{all_local, bwd});
    } else {
      bp_list = plan_passes(bwd, n, k, c);
    }
    for (const PlannedPass& P : bp_list) {
      // split passes with more gradient slots than the accumulators hold
      size_t g0 = 0;
      while (g0 < P.gates.size()) {
        BPass bp{};
        bp.kind = BP_BWD;
        bp.k = (int)P.local.size();
        bp.c = c;
        bp.nhigh = bp.k - c;
        for (int j = 0; j < bp.k; ++j) bp.lpos[j] = (uint8_t)P.local[j];
        bp.gate_begin = (uint32_t)vgates.size();
        int slots = 0;
        size_t g1 = g0;
        for (; g1 < P.gates.size(); ++g1) {
          const GateApp& g = P.gates[g1];
          const int pj = param_of_op[g.src];
          if (pj >= 0 && slots == kMaxPassParams) break;
          BGate t = to_bgate(g, P.local);
          if (pj >= 0) {
            t.param = pj;
            t.sign = -1;
            t.gacc = slots++;
            switch (g.kind) {
              case SPZ_GATE_RX: t.grad = BG_X; break;
              case SPZ_GATE_RY: t.grad = BG_Y; break;
              case SPZ_GATE_RZ: t.grad = BG_Z; break;
              default: t.grad = BG_P1; break;
            }
            jobs.push_back(CoefJob{(uint32_t)vgates.size(), g.kind, (int64_t)in.param_offset + pj, -1, 0});
          }
          vgates.push_back(t);
        }
        bp.gate_count = (uint32_t)(vgates.size() - bp.gate_begin);
        bp.nparams = slots;
        vpass.push_back(bp);
        b->bwd_passes++;
        g0 = g1;
      }
    }
    I.npass = (uint32_t)(vpass.size() - I.pass_begin);
    b->resident += I.resident;
    cost[ii] = (double)(applied.size() + 8) * (double)(1ull << n);
  }
  std::vector<uint32_t> order = narrow;
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t c2) { return cost[a] > cost[c2]; });
  std::stable_sort(b->wide.begin(), b->wide.end(), [](const WideInst& a, const WideInst& c2) { return a.cost > c2.cost; });
  // Queue: whole instances first, largest first (the longest single-CTA jobs
  // start at once), then the wide instances' items pass by pass (pass p of
  // every wide instance, largest instance first, before pass p + 1 of any),
  // so that an item's dependencies sit far ahead of it in the queue.
  std::vector<BItem> items;
  for (uint32_t ii : order) items.push_back(BItem{ii, kWholeInstance, 0, 0, 0, 0});
  std::vector<uint32_t> worder = wide_in;
  std::stable_sort(worder.begin(), worder.end(), [&](uint32_t a, uint32_t c2) { return cost[a] > cost[c2]; });
  // per wide instance: items per pass, partial-slot bases (contiguous per instance)
  std::vector<BSum> sums;
  std::vector<std::vector<uint32_t>> pass_items(ninst);
  std::vector<std::vector<uint64_t>> pass_slot(ninst);
  uint64_t nslots = 0;
  uint32_t max_pass = 0;
  const uint64_t tpi = (uint64_t)std::max(1, b->tiles_per_item);
  uint64_t ws_off = 0;
  for (uint32_t ii : worder) {
    BInst& I = vinst[ii];
    I.ws_offset = ws_off;
    ws_off += 4ull * (1ull << I.n);
    max_pass = std::max(max_pass, I.npass);
    uint64_t ham_base = nslots, ham_count = 0;
    for (uint32_t p = 0; p < I.npass; ++p) {  // HAM slots of the instance first, contiguous
      const BPass& P = vpass[I.pass_begin + p];
      const uint64_t ntiles = 1ull << (I.n - P.k);
      const uint32_t m = (uint32_t)((ntiles + tpi - 1) / tpi);
      pass_items[ii].push_back(m);
      pass_slot[ii].push_back(0);
      if (P.kind == BP_HAM) {
        pass_slot[ii][p] = nslots;
        nslots += m;
        ham_count += m;
      }
    }
    sums.push_back(BSum{ii, ham_base, 1, (uint32_t)ham_count, 1.0, 1, 0});
    for (uint32_t p = 0; p < I.npass; ++p) {
      const BPass& P = vpass[I.pass_begin + p];
      if (P.kind != BP_BWD) continue;
      pass_slot[ii][p] = nslots;
      const uint32_t m = pass_items[ii][p];
      for (uint32_t gi = 0; gi < P.gate_count; ++gi) {
        const BGate& g = vgates[P.gate_begin + gi];
        if (g.grad == BG_NONE) continue;
        sums.push_back(BSum{(uint64_t)(I.param_offset + g.param), nslots + (uint64_t)g.gacc, (uint32_t)P.nparams, m,
                            g.grad == BG_P1 ? -2.0 : 1.0, 0, 0});
      }
      nslots += (uint64_t)m * (uint64_t)P.nparams;
    }
  }
  const uint32_t poison = 0xFFFFFFFFu;  // SPZ_BATCH_TEST_STALL: a count no item ever reaches
  for (uint32_t p = 0; p < max_pass; ++p) {
    for (uint32_t ii : worder) {
      const BInst& I = vinst[ii];
      if (p >= I.npass) continue;
      const BPass& P = vpass[I.pass_begin + p];
      const uint64_t ntiles = 1ull << (I.n - P.k);
      uint32_t need = 0;
      for (uint32_t q = 0; q < p; ++q) need += pass_items[ii][q];
      if (b->stall_for_test && p > 0) need = poison;
      const uint32_t m = pass_items[ii][p];
      const uint32_t per_item = P.kind == BP_BWD ? (uint32_t)P.nparams : (P.kind == BP_HAM ? 1u : 0u);
      for (uint32_t r = 0; r < m; ++r) {
        const uint64_t t0 = (uint64_t)r * tpi, t1 = std::min<uint64_t>(ntiles, t0 + tpi);
        items.push_back(BItem{ii, p, need, (uint32_t)(pass_slot[ii][p] + (uint64_t)r * per_item), t0, t1});
      }
    }
  }
  if (nslots >= 0xFFFFFFFFull) return fail(SPZ_ERR_UNSUPPORTED, "batch: too many partial-sum slots");
  b->ninst = (uint32_t)ninst;
  b->nnarrow = (uint32_t)narrow.size();
  b->nitems = (uint32_t)items.size();
  b->nwide_items = (uint32_t)(items.size() - order.size());
  b->nwide_in_kernel = (uint32_t)wide_in.size();
  b->nsums = (uint32_t)sums.size();
  b->npartials = nslots;
  b->wide_ws_doubles = ws_off;
  b->nparams_total = ptotal;
  b->ws_qubits = ws_qubits;
  b->njobs = (uint32_t)jobs.size();
  int rc;
  if ((rc = upload(&b->d_inst, vinst)) || (rc = upload(&b->d_items, items)) || (rc = upload(&b->d_sums, sums)) ||
      (rc = upload(&b->d_pass, vpass)) || (rc = upload(&b->d_gates, vgates)) || (rc = upload(&b->d_terms, vterms)) ||
      (rc = upload(&b->d_jobs, jobs)))
    return rc;
  SPZ_CUDA(dev_alloc(&b->d_partials, std::max<uint64_t>(1, nslots) * sizeof(double)));
  SPZ_CUDA(dev_alloc(&b->d_done, std::max<size_t>(1, wide_in.size()) * sizeof(unsigned int)));
  SPZ_CUDA(dev_alloc(&b->d_error, sizeof(int)));
  SPZ_CUDA(host_alloc(&b->h_error, sizeof(int)));
  if (ws_off) SPZ_CUDA(dev_alloc(&b->d_wide_ws, ws_off * sizeof(double)));
  SPZ_CUDA(dev_alloc(&b->d_theta, std::max<uint64_t>(1, ptotal) * sizeof(double)));
  SPZ_CUDA(dev_alloc(&b->d_grad, std::max<uint64_t>(1, ptotal) * sizeof(double)));
  SPZ_CUDA(dev_alloc(&b->d_energy, std::max<size_t>(1, ninst) * sizeof(double)));
  SPZ_CUDA(dev_alloc(&b->d_counter, sizeof(unsigned int)));
  SPZ_CUDA(cudaMemset(b->d_grad, 0, std::max<uint64_t>(1, ptotal) * sizeof(double)));
  SPZ_CUDA(host_alloc(&b->h_theta, std::max<uint64_t>(1, ptotal) * sizeof(double)));
  SPZ_CUDA(host_alloc(&b->h_grad, std::max<uint64_t>(1, ptotal) * sizeof(double)));
  SPZ_CUDA(host_alloc(&b->h_energy, std::max<size_t>(1, ninst) * sizeof(double)));
  // launch shape: persistent CTAs, as many per SM as shared memory allows
  const uint32_t TMAX = 1u << b->kmax;
  b->smem = (4 * TMAX + ((2 * TMAX) >> kBatchLowBits) + (size_t)(b->threads / 32) * (1 + kMaxPassParams)) *
            sizeof(double);
  const void* kfn = batch_kernel_fn(b->threads);
  SPZ_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem));
  int per_sm = 0;
  SPZ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, b->threads, b->smem));
  if (per_sm < 1) return fail(SPZ_ERR_UNSUPPORTED, "batch kernel does not fit on an SM with this configuration");
  int sms = 0;
  SPZ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device));
  b->grid = std::max(1, std::min<int>(sms * per_sm, (int)b->nitems));
  if (ws_qubits) {
    // Each CTA owns psi and lam of the largest streamed instance; keep the
    // workspace within half of the free device memory, at most
    // kWorkspaceBudget (and at least one CTA per SM).
    SPZ_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const uint64_t budget = std::min<uint64_t>(kWorkspaceBudget, free_b / 2);
    const uint64_t per_cta = 4ull * (1ull << ws_qubits) * sizeof(double);
    const uint64_t cap = std::max<uint64_t>((uint64_t)sms, budget / per_cta);
    b->grid = (int)std::min<uint64_t>((uint64_t)b->grid, cap);
    const size_t bytes = (size_t)b->grid * 4 * (1ull << ws_qubits) * sizeof(double);
    SPZ_CUDA(dev_alloc(&b->d_ws, bytes));
  }
  return SPZ_OK;
}

int capture_graph(spz_batch_t b) {
  cudaGraph_t g;
  SPZ_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  cudaMemcpyAsync(b->d_theta, b->h_theta, std::max<uint64_t>(1, b->nparams_total) * sizeof(double),
                  cudaMemcpyHostToDevice, b->stream);
  cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned int), b->stream);
  cudaMemsetAsync(b->d_done, 0, std::max<size_t>(1, b->nwide_in_kernel) * sizeof(unsigned int), b->stream);
  cudaMemsetAsync(b->d_error, 0, sizeof(int), b->stream);
  if (b->njobs) batch_coef_kernel<<<(b->njobs + 255) / 256, 256, 0, b->stream>>>(b->d_gates, b->d_jobs, b->njobs, b->d_theta);
  BatchArgs A{};
  A.inst = b->d_inst;
  A.items = b->d_items;
  A.nitems = b->nitems;
  A.wide_ws = b->d_wide_ws;
  A.done = b->d_done;
  A.partials = b->d_partials;
  A.error = b->d_error;
  A.wait_limit = b->wait_limit;
  A.passes = b->d_pass;
  A.gates = b->d_gates;
  A.terms = b->d_terms;
  A.energies = b->d_energy;
  A.grads = b->d_grad;
  A.workspace = b->d_ws;
  A.ws_qubits = b->ws_qubits;
  A.counter = b->d_counter;
  A.kmax = b->kmax;
  if (b->nitems) {
    if (b->threads <= 64) batch_kernel<64, 12><<<b->grid, b->threads, b->smem, b->stream>>>(A);
    else batch_kernel<1024, 1><<<b->grid, b->threads, b->smem, b->stream>>>(A);
  }
  if (b->nsums)
    batch_fold_kernel<<<(b->nsums + 255) / 256, 256, 0, b->stream>>>(b->d_sums, b->nsums, b->d_partials, b->d_energy,
                                                                     b->d_grad);
  cudaMemcpyAsync(b->h_error, b->d_error, sizeof(int), cudaMemcpyDeviceToHost, b->stream);
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (e != cudaSuccess) return cuda_fail(e, "batch graph capture");
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "batch graph instantiation");
  return SPZ_OK;
}

}  // namespace
}  // namespace spz

using namespace spz;

extern "C" {

int spz_batch_create(const spz_batch_instance* instances, size_t ninstances, const spz_op* ops,
                     const uint32_t* param_index, const spz_pauli_term* terms, const spz_batch_config* config,
                     spz_batch_t* out) {
  if (!out || (ninstances && !instances)) return fail(SPZ_ERR_NULL, "NULL argument");
  spz_batch_t b = new (std::nothrow) spz_batch_s();
  if (!b) return fail(SPZ_ERR_OUT_OF_MEMORY, "host allocation failed");
  if (config) {
    if (config->tile_qubits) b->kmax = config->tile_qubits;
    if (config->threads) b->threads = config->threads;
    if (config->wide_qubits) b->wide_qubits = config->wide_qubits;
    b->wide_flags = (uint32_t)config->flags & (SPZ_EXEC_FAST | SPZ_BATCH_WIDE_APART);
    if (config->tiles_per_item) b->tiles_per_item = config->tiles_per_item;
  }
  {
    const char* v = std::getenv("SPZ_BATCH_WIDE_STREAMS");
    if (v && v[0] >= '1' && v[0] <= '0' + kWideStreams && v[1] == 0) b->wide_streams = v[0] - '0';
  }
  {  // host-side fault injection for tests: wide items wait on counts never reached
    const char* v = std::getenv("SPZ_BATCH_TEST_STALL");
    if (v && v[0] == '1' && v[1] == 0) {
      b->stall_for_test = true;
      b->wait_limit = 4096;
    }
  }
  if (b->tiles_per_item < 1) {
    delete b;
    return fail(SPZ_ERR_INVALID_ARGUMENT, "batch config: tiles_per_item must be >= 1");
  }
  if (b->kmax < 4 || b->kmax > kBatchMaxK || b->threads < 64 || b->threads > 1024 || (b->threads & 31)) {
    delete b;
    return fail(SPZ_ERR_INVALID_ARGUMENT, "batch config: tile_qubits in 4..12, threads a multiple of 32 in 64..1024");
  }
  cudaError_t e = cudaGetDevice(&b->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete b;
    return cuda_fail(e, "batch stream");
  }
  int rc = build_batch(b, instances, ninstances, ops, param_index, terms);
  if (rc) {
    free_batch(b);
    return rc;
  }
  *out = b;
  return SPZ_OK;
}

int spz_batch_run(spz_batch_t b, const double* theta, double* energies, double* grads) {
  NvtxRange range("spz_batch_run");
  if (!b || !theta || !energies || (b->nparams_total && !grads)) return fail(SPZ_ERR_NULL, "NULL argument");
  std::memcpy(b->h_theta, theta, b->nparams_total * sizeof(double));
  if (!b->graph) {
    int rc = capture_graph(b);
    if (rc) return rc;
  }
  SPZ_CUDA(cudaGraphLaunch(b->graph, b->stream));
  // Wide instances, largest first, one at a time across the GPU; results
  // straight into the device output arrays (no wait in between).
  auto wait_all = [&]() {
    for (int si = 0; si < kWideStreams; ++si)
      if (b->wide_stream[si]) cudaStreamSynchronize(b->wide_stream[si]);
    cudaStreamSynchronize(b->stream);
  };
  for (size_t wi = 0; wi < b->wide.size(); ++wi) {
    WideInst& w = b->wide[wi];
    const int si = (int)(wi % (size_t)b->wide_streams);
    if (!b->wide_stream[si]) {
      SPZ_CUDA(cudaStreamCreateWithFlags(&b->wide_stream[si], cudaStreamNonBlocking));
      SPZ_CUDA(cudaEventCreateWithFlags(&b->wide_done[si], cudaEventDisableTiming));
    }
    spz_state_t& h = b->wide_h[si][w.n];
    if (!h) {
      int rc = spz_state_create(w.n, &h);
      if (rc) {
        wait_all();
        return rc;
      }
      SPZ_CUDA(cudaStreamSynchronize(h->stream));  // its |0...0> fill ran on its own stream
      h->stream = b->wide_stream[si];
    }
    for (size_t j = 0; j < w.pidx.size(); ++j) w.ops[w.pidx[j]].gate.p[0] = theta[w.param_offset + j];
    int rc = spz_state_reset_zero(h);
    if (!rc)
      rc = adjoint_gradient(h, w.ops.data(), w.ops.size(), w.pidx.data(), w.pidx.size(), w.terms.data(),
                            w.terms.size(), b->wide_flags & SPZ_EXEC_FAST, nullptr, nullptr, b->d_energy + w.idx,
                            b->d_grad + w.param_offset);
    if (rc) {
      wait_all();
      return rc;
    }
  }
  for (int si = 0; si < kWideStreams; ++si)  // the read-back waits for every wide stream
    if (b->wide_stream[si]) {
      SPZ_CUDA(cudaEventRecord(b->wide_done[si], b->wide_stream[si]));
      SPZ_CUDA(cudaStreamWaitEvent(b->stream, b->wide_done[si], 0));
    }
  SPZ_CUDA(cudaMemcpyAsync(b->h_energy, b->d_energy, std::max<size_t>(1, b->ninst) * sizeof(double),
                           cudaMemcpyDeviceToHost, b->stream));
  SPZ_CUDA(cudaMemcpyAsync(b->h_grad, b->d_grad, std::max<uint64_t>(1, b->nparams_total) * sizeof(double),
                           cudaMemcpyDeviceToHost, b->stream));
  SPZ_CUDA(cudaStreamSynchronize(b->stream));
  if (*b->h_error)
    return fail(SPZ_ERR_TIMEOUT, "batch: a work item's dependency wait ran out; the launch stopped early and its "
                                 "outputs are incomplete");
  std::memcpy(energies, b->h_energy, b->ninst * sizeof(double));
  if (b->nparams_total) std::memcpy(grads, b->h_grad, b->nparams_total * sizeof(double));
  return SPZ_OK;
}

int spz_batch_info(spz_batch_t b, spz_batch_stats* st) {
  if (!b || !st) return fail(SPZ_ERR_NULL, "NULL argument");
  st->instances = b->ninst;
  st->resident_instances = b->resident;
  st->forward_passes = b->fwd_passes;
  st->hamiltonian_passes = b->ham_passes;
  st->backward_passes = b->bwd_passes;
  st->ctas = (uint64_t)b->grid;
  st->workspace_bytes = b->ws_qubits ? (uint64_t)b->grid * 4 * (1ull << b->ws_qubits) * sizeof(double) : 0;
  st->tile_qubits = b->kmax;
  st->threads = b->threads;
  st->wide_in_kernel = b->nwide_in_kernel;
  st->work_items = b->nitems;
  st->wide_separate = b->wide.size();
  st->wide_workspace_bytes = b->wide_ws_doubles * sizeof(double);
  st->tiles_per_item = b->tiles_per_item;
  return SPZ_OK;
}

int spz_batch_destroy(spz_batch_t b) {
  if (b) cudaStreamSynchronize(b->stream);
  free_batch(b);
  return SPZ_OK;
}

}  // extern "C"
