// Shared definitions of the spinoza_gb300 CUDA library (sm_103a).
//
// State layout in HBM: two FP64 arrays reals[2^n], imags[2^n] (SoA), as
// `State { reals, imags, n }` in spinoza/src/core.rs:20-27.  Amplitude index i
// has bit q equal to the value of qubit q.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/spinoza_gb300.h"

// NVTX ranges (header-only NVTX 3): executor calls and fused passes show as
// named host ranges under a profiler; without one the calls return at once.
#if defined(__has_include)
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define SPZ_HAVE_NVTX 1
#endif
#endif

namespace spz {

struct NvtxRange {
  explicit NvtxRange(const char* name) {
#ifdef SPZ_HAVE_NVTX
    nvtxRangePushA(name);
#else
    (void)name;
#endif
  }
  ~NvtxRange() {
#ifdef SPZ_HAVE_NVTX
    nvtxRangePop();
#endif
  }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

constexpr int kMaxQubits = SPZ_MAX_QUBITS;
constexpr int kNumSMs = 152;          // GB300: 2 dies x 76 SMs
constexpr int kThreads = 256;
// Per-device caches (kernel attributes, launch shapes) hold this many devices.
constexpr int kMaxDevices = 64;

// ------------------------------------------------------------ error state
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define SPZ_CUDA(call)                                   \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return ::spz::cuda_fail(e_, #call); \
  } while (0)

#define SPZ_CHECK_LAUNCH(what)                           \
  do {                                                   \
    cudaError_t e_ = cudaGetLastError();                 \
    if (e_ != cudaSuccess) return ::spz::cuda_fail(e_, what); \
  } while (0)

// ------------------------------------------------------------ allocation
// Every device and page-locked host allocation of the library goes through
// these two.  While the environment variable SPZ_INJECT_ALLOC_FAILURE is set
// to 1 they return cudaErrorMemoryAllocation without allocating: a host-side
// fault injection that exercises the out-of-memory paths (the call returns
// SPZ_ERR_OUT_OF_MEMORY and leaves its handle usable) with no GPU fault.
cudaError_t dev_alloc(void** p, size_t bytes);
cudaError_t host_alloc(void** p, size_t bytes);
template <class T>
inline cudaError_t dev_alloc(T** p, size_t bytes) { return dev_alloc(reinterpret_cast<void**>(p), bytes); }
template <class T>
inline cudaError_t host_alloc(T** p, size_t bytes) { return host_alloc(reinterpret_cast<void**>(p), bytes); }

// ------------------------------------------------------------ the handle
struct Scratch {
  void* ptr = nullptr;
  size_t bytes = 0;
};

}  // namespace spz

struct spz_state_s {
  uint32_t n = 0;
  uint64_t N = 0;
  double* re = nullptr;
  double* im = nullptr;
  bool owns = false;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  int device = 0;
  // Reduction / planning scratch, grown on demand and reused.
  spz::Scratch dev_scratch;
  spz::Scratch host_scratch;  // pinned
  // Two extra state vectors for adjoint differentiation (lazily allocated).
  double* aux_re[2] = {nullptr, nullptr};
  double* aux_im[2] = {nullptr, nullptr};
  // Second stream for host <-> device copies that overlap tile passes
  // (spz_circuit_execute_host; lazily created).
  cudaStream_t copy_stream = nullptr;
  // Measurements made inside the executor, kept on the device (lazily
  // allocated): prob0[64], scale[64] (doubles), then outcome[64] (int32).
  double* meas = nullptr;
  // Lazy per-gate mode (spz_state_set_lazy): the state is
  // (factor_re + i factor_im) * 2^factor_exp * (re, im); the factor is folded
  // into the arrays (settle) before anything reads them.
  bool lazy = false;
  double factor_re = 1.0, factor_im = 0.0;
  int factor_exp = 0;
  // TMA-staged tile passes (SPZ_EXEC_TMA*): tensor maps of re and im viewed as
  // 2^(n-3) rows of 8 doubles (CUtensorMap, opaque 128 bytes each), built on
  // first use, and a device word in which a timed-out wait is reported.
  alignas(64) unsigned char tma_map[2][128] = {};
  bool tma_ready = false;
  int* tma_err = nullptr;
  // Tile geometry of this handle's fused passes (spz_state_set_tile): log2 of
  // the tile's amplitudes and threads per block; 0 = the library default.
  int tile_k = 0, tile_threads = 0;
};

namespace spz {

int ensure_dev_scratch(spz_state_t h, size_t bytes, void** out);
// Lazy per-gate mode (state.cu): fold a pending factor into the arrays (one
// scaling pass, nothing when the factor is 1); forget it (the arrays were
// overwritten); multiply it by f.
int settle(spz_state_t h);
void clear_factor(spz_state_t h);
int scale_factor(spz_state_t h, double f_re, double f_im);
int ensure_host_scratch(spz_state_t h, size_t bytes, void** out);
// Copy kind for a caller's buffer moving into (to_device) or out of device memory.
cudaMemcpyKind copy_kind(const void* p, bool to_device);
int grid_for(uint64_t work, int threads = kThreads, int per_sm = 16);

// ------------------------------------------------------ FP64 primitives
// Adds and multiplies are issued as fused multiply-adds that round exactly
// like the plain operation:  a*b == fma(a, b, -0.0),  a+b == fma(1, a, b),
// a-b == fma(-1, b, a).  On GB300 the DFMA pipe issues ~18% faster than
// DADD/DMUL, and the results are bit-identical.  Inline PTX keeps the
// compiler from folding them back.  Negation flips the sign bit on the
// integer pipe.
__device__ __forceinline__ double dfma(double a, double b, double c) {
  double d;
  asm("fma.rn.f64 %0, %1, %2, %3;" : "=d"(d) : "d"(a), "d"(b), "d"(c));
  return d;
}
__device__ __forceinline__ double dmul(double a, double b) { return dfma(a, b, -0.0); }
__device__ __forceinline__ double dadd(double a, double b) { return dfma(1.0, a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return dfma(-1.0, b, a); }
__device__ __forceinline__ double dneg(double a) {
  return __longlong_as_double(__double_as_longlong(a) ^ (long long)0x8000000000000000ull);
}

// Insert a zero bit at each of the sorted positions pos[0] < pos[1] < ...
// (so that the result has those bits clear and the other bits are k's bits in
// order).  This enumerates the "s0" amplitudes of controlled gates.
__device__ __forceinline__ uint64_t deposit(uint64_t k, const uint8_t* pos, int npos) {
  for (int j = 0; j < npos; ++j) {
    const uint64_t p = pos[j];
    const uint64_t low = k & ((1ull << p) - 1);
    k = ((k >> p) << (p + 1)) | low;
  }
  return k;
}

// deposit() for positions held in a kernel parameter: pos[] is read at
// constant indices only (j < MAXK, unrolled).  A run-time index into a
// by-value kernel parameter makes the compiler copy the whole parameter block
// to local memory, after which every read of it is a local load.
template <int MAXK>
__device__ __forceinline__ uint64_t deposit_param(uint64_t k, const uint8_t* pos, int npos) {
#pragma unroll
  for (int j = 0; j < MAXK; ++j) {
    if (j < npos) {
      const uint64_t p = pos[j];
      k = ((k >> p) << (p + 1)) | (k & ((1ull << p) - 1));
    }
  }
  return k;
}

// Offset of row r of a tile: bit j of r scattered to position pos[c + j].
template <int MAXK>
__device__ __forceinline__ uint64_t row_offset_param(uint32_t r, const uint8_t* pos, int c, int k) {
  uint64_t off = 0;
#pragma unroll
  for (int j = 0; j < MAXK; ++j)
    if (j >= c && j < k && ((r >> (j - c)) & 1)) off |= 1ull << pos[j];
  return off;
}

// ------------------------------------------------------ gate coefficients
// Host-computed coefficients, exactly as the reference computes them
// (glibc sin/cos, the same sub-expressions); see coef_for() in gates.cu.
struct Coef {
  double a, k, l, q, r, s, t;    // U: g = [(a,0), (k,l), (q,r), (s,t)]  (gates.rs:1285-1304)
  double cs, sn, nsn;            // P: cos, sin; RX: cos, -, neg_sin; RY: cos, sin
  double d0re, d0im, d1re, d1im; // RZ diagonal (gates.rs:930-937)
};

int coef_for(const spz_gate& g, Coef* out);

// Ops produced by the fast-mode lowering (fast.cu); they exist only inside the
// fused executor.  Lazy ops are a gate divided by a scalar that is carried in
// the executor's global factor; phase ops multiply amplitudes by table entries
// selected by parities of index bits.
enum FastKind {
  FK_LAZY_H = 100,     // [[1, 1], [1, -1]]                (H = 2^-1/2 x this)
  FK_LAZY_RX_A = 101,  // [[1, -i t], [-i t, 1]], t = tan  (RX = cos x this)
  FK_LAZY_RX_B = 102,  // [[u, -i], [-i, u]],     u = cot  (RX = sin x this)
  FK_LAZY_RY_A = 103,  // [[1, -t], [t, 1]]                (RY = cos x this)
  FK_LAZY_RY_B = 104,  // [[u, -1], [1, u]]                (RY = sin x this)
  FK_PHASE = 105       // x -> table[parities of x & mask_j] x (only where x & half_bit, if set)
};

constexpr int kPhaseMaxTerms = 8;

// One phase op: 2^m complex entries indexed by the parities of the index under
// m masks; applied to every amplitude, or only to those with half_bit set.
struct PhaseTable {
  int m = 0;
  uint64_t mask[kPhaseMaxTerms] = {};
  uint64_t half_bit = 0;
  std::vector<double> re, im;  // 2^m entries
};

// Validated, normalised description of one gate application.
struct GateApp {
  int kind;          // enum spz_gate_kind (H,X,Y,Z,P,RX,RY,RZ,U,SWAP)
  uint32_t target;   // target (SWAP: q0)
  uint32_t target2;  // SWAP: q1
  uint64_t ones;     // controls that must read 1
  uint64_t zeros;    // controls that must read 0
  Coef c;
  int64_t src = -1;  // index of the circuit op it came from (planning reports)
  int32_t table = -1;  // FK_PHASE: index of its PhaseTable
  uint64_t touch = 0;  // FK_PHASE: qubits its phases depend on (diagonal action)
  int32_t cond = -1;   // applies only if the qubit `cond`, measured on the device, read 1
};

// Fast-mode lowering (fast.cu): rewrite `in` into lazy ops, phase ops and
// exact gates with the same overall action (up to rounding).
void lower_fast(const std::vector<GateApp>& in, uint32_t n, std::vector<GateApp>* out,
                std::vector<PhaseTable>* tables);

// Validate and build a GateApp (returns a status).
int make_gate_app(uint32_t n, const spz_gate& g, uint32_t target, uint64_t ones, uint64_t zeros,
                  GateApp* out);

// True for gates whose matrix is diagonal (they need no amplitude pairing).
inline bool is_diagonal(int kind) { return kind == SPZ_GATE_Z || kind == SPZ_GATE_P || kind == SPZ_GATE_RZ; }

// Launch one gate over the whole state (the plain per-gate path).
int launch_gate(spz_state_t h, const GateApp& g);

// Algorithmic HBM bytes of one unfused gate application on 2^n amplitudes.
uint64_t gate_algorithmic_bytes(uint32_t n, const GateApp& g);

// FP64-pipe instructions (DFMA-issued adds, multiplies and FMAs) one gate
// application needs on 2^n amplitudes.
uint64_t gate_fp64_ops(uint32_t n, const GateApp& g);

// Fusion planner (circuit.cu): passes of gates over tiles of k local qubits,
// the low c qubits always local.
struct PlannedPass {
  std::vector<int> local;  // sorted local qubits
  std::vector<GateApp> gates;
};
// exact: reorder only gates whose exchange is bit-identical (else any that commute).
std::vector<PlannedPass> plan_passes(const std::vector<GateApp>& gates, uint32_t n, int k, int c, bool exact = true);

// Adjoint gradient of <psi|H|psi> on h (adjoint.cu); with d_energy / d_grad
// (device) the results stay on the device and nothing waits for it.
int adjoint_gradient(spz_state_t h, const spz_op* ops, size_t nops, const uint32_t* param_index, size_t nparams,
                     const spz_pauli_term* terms, size_t nterms, uint32_t flags, double* energy, double* grad,
                     double* d_energy, double* d_grad);

// Reductions used by measurement and the executor.
int prob0_device(spz_state_t h, uint32_t target, double* out);
// Measure `target` without leaving the device: prob0 -> outcome (1 iff
// u < 1 - prob0) -> collapse (and reset to 0 when `reset`), the outcome kept in
// h->meas for gates conditioned on it and for the tracker.
int measure_on_device(spz_state_t h, uint32_t target, int reset, double u);
constexpr int kMeasOutcomeOffset = 128;  // doubles before the outcome array in h->meas
int collapse_device(spz_state_t h, uint32_t target, int outcome, double scale);

}  // namespace spz
