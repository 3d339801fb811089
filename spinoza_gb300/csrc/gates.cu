// Per-gate amplitude kernels: the plain drop-in for gates::apply, c_apply,
// cc_apply and mc_apply (spinoza/src/gates.rs:215-320).
//
// Every gate runs as one pass over the amplitudes it touches:
//   * pair gates (H, X, Y, RX, RY, U): one thread per two consecutive pairs,
//     double2 (16-byte) coalesced loads of reals and imags at s0 and s1;
//   * diagonal gates (Z, P, RZ): elementwise over the amplitudes whose fixed
//     bits match, double2 loads;
//   * SWAP: the (01 <-> 10) exchange over the remaining bits.
// Controls are bits inserted into the enumeration (value 1 for `ones`, 0 for
// `zeros`), so a k-control gate reads only 2^-k of the state.
//
// Arithmetic is the reference's own, operation by operation (cited per gate),
// so a single gate is bit-identical to the reference's CPU result.
#include <algorithm>
#include <cmath>
#include <string>

#include "common.cuh"
#include "gate_math.cuh"

namespace spz {

// ------------------------------------------------------------ coefficients
int coef_for(const spz_gate& g, Coef* out) {
  Coef c{};
  switch (g.kind) {
    case SPZ_GATE_P: {  // gates.rs:862 sin_cos(angle)
      c.sn = std::sin(g.p[0]);
      c.cs = std::cos(g.p[0]);
      c.nsn = -c.sn;
      break;
    }
    case SPZ_GATE_RX: {  // gates.rs:749-751
      const double theta = g.p[0] * 0.5;
      c.cs = std::cos(theta);
      c.nsn = -std::sin(theta);
      c.sn = -c.nsn;
      break;
    }
    case SPZ_GATE_RY: {  // gates.rs:1123-1124
      const double theta = g.p[0] * 0.5;
      c.sn = std::sin(theta);
      c.cs = std::cos(theta);
      c.nsn = -c.sn;
      break;
    }
    case SPZ_GATE_RZ: {  // gates.rs:932-936
      const double theta = g.p[0] * 0.5;
      const double s = std::sin(theta), co = std::cos(theta);
      c.d0re = co;
      c.d0im = -s;
      c.d1re = co;
      c.d1im = s;
      break;
    }
    case SPZ_GATE_U: {  // gates.rs:1285-1304
      const double theta = g.p[0], phi = g.p[1], lambda = g.p[2];
      const double st = std::sin(theta * 0.5), ct = std::cos(theta * 0.5);
      const double sl = std::sin(lambda), cl = std::cos(lambda);
      const double spl = std::sin(phi + lambda), cpl = std::cos(phi + lambda);
      const double sp = std::sin(phi), cp = std::cos(phi);
      c.a = ct;
      c.k = -cl * st;
      c.l = -sl * st;
      c.q = cp * st;
      c.r = sp * st;
      c.s = cpl * ct;
      c.t = spl * ct;
      break;
    }
    case SPZ_GATE_H:
    case SPZ_GATE_X:
    case SPZ_GATE_Y:
    case SPZ_GATE_Z:
    case SPZ_GATE_SWAP:
      break;
    default:
      return fail(SPZ_ERR_UNSUPPORTED, "gate kind has no 2x2 coefficients");
  }
  *out = c;
  return SPZ_OK;
}

int make_gate_app(uint32_t n, const spz_gate& g, uint32_t target, uint64_t ones, uint64_t zeros,
                  GateApp* out) {
  const uint64_t cm = ones | zeros;
  if (ones & zeros) return fail(SPZ_ERR_INVALID_ARGUMENT, "a control cannot be both 1 and 0");
  if (n < 64 && (cm >> n) != 0) return fail(SPZ_ERR_INVALID_ARGUMENT, "control qubit out of range");
  GateApp a{};
  a.kind = g.kind;
  a.ones = ones;
  a.zeros = zeros;
  switch (g.kind) {
    case SPZ_GATE_SWAP:
      if (g.q0 >= n || g.q1 >= n) return fail(SPZ_ERR_INVALID_ARGUMENT, "SWAP qubit out of range");
      if ((cm >> g.q0) & 1 || (cm >> g.q1) & 1)
        return fail(SPZ_ERR_INVALID_ARGUMENT, "SWAP qubit is also a control");
      a.target = g.q0;
      a.target2 = g.q1;
      break;
    case SPZ_GATE_H:
    case SPZ_GATE_X:
    case SPZ_GATE_Y:
    case SPZ_GATE_Z:
    case SPZ_GATE_P:
    case SPZ_GATE_RX:
    case SPZ_GATE_RY:
    case SPZ_GATE_RZ:
    case SPZ_GATE_U:
      if (target >= n) return fail(SPZ_ERR_INVALID_ARGUMENT, "target qubit out of range");
      if ((cm >> target) & 1) return fail(SPZ_ERR_INVALID_ARGUMENT, "target qubit is also a control");
      a.target = target;
      a.target2 = target;
      break;
    case SPZ_GATE_M:
      return fail(SPZ_ERR_UNSUPPORTED, "M is only valid inside a circuit (spz_circuit_execute)");
    case SPZ_GATE_UNITARY:
      return fail(SPZ_ERR_UNSUPPORTED, "dense Unitary application is not on this path");
    default:
      return fail(SPZ_ERR_INVALID_ARGUMENT, "unknown gate kind");
  }
  int rc = coef_for(g, &a.c);
  if (rc) return rc;
  *out = a;
  return SPZ_OK;
}

uint64_t gate_algorithmic_bytes(uint32_t n, const GateApp& g) {
  const uint64_t N = 1ull << n;
  const int nc = __builtin_popcountll(g.ones | g.zeros);
  uint64_t full;
  switch (g.kind) {
    case SPZ_GATE_Z:
    case SPZ_GATE_P:
    case SPZ_GATE_SWAP:
      full = 16 * N;  // half of the amplitudes read and written
      break;
    default:
      full = 32 * N;  // every amplitude read and written
  }
  return full >> nc;
}

uint64_t gate_fp64_ops(uint32_t n, const GateApp& g) {
  const int nc = __builtin_popcountll(g.ones | g.zeros);
  const uint64_t pairs = (1ull << (n - 1)) >> nc;
  switch (g.kind) {
    case SPZ_GATE_H: return 8 * pairs;     // 4 mul + 4 add
    case SPZ_GATE_RX:
    case SPZ_GATE_RY: return 12 * pairs;   // 8 mul + 4 add
    case SPZ_GATE_U: return 14 * pairs;    // 4 mul + 10 fma
    case SPZ_GATE_P: return 4 * pairs;     // s1 only: 2 mul + 2 fma
    case SPZ_GATE_RZ: return 8 * pairs;    // both: 4 mul + 4 fma
    default: return 0;                     // X, Y, Z, SWAP move or negate only
  }
}

// ------------------------------------------------------------ kernels
struct PairArgs {
  double* re;
  double* im;
  uint64_t nwork;
  uint64_t ones;
  uint64_t tbit;
  Coef c;
  int32_t npos;
  uint8_t pos[kMaxQubits + 2];
};

// Exact gates use the reference's arithmetic; the lazy kinds (FK_LAZY_*, the
// gate divided by a scalar) use the 4-instruction forms.
template <int KIND>
__device__ __forceinline__ void pair_op(const Coef& c, double& a, double& b, double& x, double& d) {
  if constexpr (KIND >= FK_LAZY_H) fast_pair<KIND>(c, a, b, x, d);
  else gate_pair<KIND>(c, a, b, x, d);
}

// Two consecutive pairs per thread; requires every special position >= 1.
template <int KIND>
__global__ void __launch_bounds__(kThreads) pair_kernel_v2(PairArgs A) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < A.nwork; w += stride) {
    const uint64_t s0 = deposit(2 * w, A.pos, A.npos) | A.ones;
    const uint64_t s1 = s0 | A.tbit;
    double2 r0 = *reinterpret_cast<const double2*>(A.re + s0);
    double2 i0 = *reinterpret_cast<const double2*>(A.im + s0);
    double2 r1 = *reinterpret_cast<const double2*>(A.re + s1);
    double2 i1 = *reinterpret_cast<const double2*>(A.im + s1);
    pair_op<KIND>(A.c, r0.x, i0.x, r1.x, i1.x);
    pair_op<KIND>(A.c, r0.y, i0.y, r1.y, i1.y);
    *reinterpret_cast<double2*>(A.re + s0) = r0;
    *reinterpret_cast<double2*>(A.im + s0) = i0;
    *reinterpret_cast<double2*>(A.re + s1) = r1;
    *reinterpret_cast<double2*>(A.im + s1) = i1;
  }
}

// Target 0 (no control on bit 0): the pair (s0, s0 + 1) is one double2.
template <int KIND>
__global__ void __launch_bounds__(kThreads) pair_kernel_t0(PairArgs A) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < A.nwork; w += stride) {
    const uint64_t s0 = deposit(w, A.pos, A.npos) | A.ones;
    double2 r = *reinterpret_cast<const double2*>(A.re + s0);
    double2 i = *reinterpret_cast<const double2*>(A.im + s0);
    pair_op<KIND>(A.c, r.x, i.x, r.y, i.y);
    *reinterpret_cast<double2*>(A.re + s0) = r;
    *reinterpret_cast<double2*>(A.im + s0) = i;
  }
}

// Scalar form (a control on bit 0).
template <int KIND>
__global__ void __launch_bounds__(kThreads) pair_kernel_s(PairArgs A) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < A.nwork; w += stride) {
    const uint64_t s0 = deposit(w, A.pos, A.npos) | A.ones;
    const uint64_t s1 = s0 | A.tbit;
    double a = A.re[s0], b = A.im[s0], c = A.re[s1], d = A.im[s1];
    pair_op<KIND>(A.c, a, b, c, d);
    A.re[s0] = a;
    A.im[s0] = b;
    A.re[s1] = c;
    A.im[s1] = d;
  }
}

// Diagonal gates: every amplitude with the fixed bits (ones) set; the element's
// own target bit picks the diagonal entry.
template <int KIND>
__global__ void __launch_bounds__(kThreads) diag_kernel_v2(PairArgs A) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < A.nwork; w += stride) {
    const uint64_t e = deposit(2 * w, A.pos, A.npos) | A.ones;
    double2 r = *reinterpret_cast<const double2*>(A.re + e);
    double2 i = *reinterpret_cast<const double2*>(A.im + e);
    gate_diag<KIND>(A.c, (e & A.tbit) != 0, r.x, i.x);
    gate_diag<KIND>(A.c, ((e + 1) & A.tbit) != 0, r.y, i.y);
    *reinterpret_cast<double2*>(A.re + e) = r;
    *reinterpret_cast<double2*>(A.im + e) = i;
  }
}

template <int KIND>
__global__ void __launch_bounds__(kThreads) diag_kernel_s(PairArgs A) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < A.nwork; w += stride) {
    const uint64_t e = deposit(w, A.pos, A.npos) | A.ones;
    double r = A.re[e], i = A.im[e];
    gate_diag<KIND>(A.c, (e & A.tbit) != 0, r, i);
    A.re[e] = r;
    A.im[e] = i;
  }
}

// SWAP(q0, q1): exchange amplitude (q0=0, q1=1) with (q0=1, q1=0).
// tbit = 1 << q0 (added to the first), ones carries 1 << q1 for the second.
__global__ void __launch_bounds__(kThreads) swap_kernel_v2(PairArgs A, uint64_t bit_a, uint64_t bit_b) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < A.nwork; w += stride) {
    const uint64_t base = deposit(2 * w, A.pos, A.npos) | A.ones;
    const uint64_t i = base | bit_b, j = base | bit_a;
    double2 ri = *reinterpret_cast<const double2*>(A.re + i);
    double2 ii = *reinterpret_cast<const double2*>(A.im + i);
    double2 rj = *reinterpret_cast<const double2*>(A.re + j);
    double2 ij = *reinterpret_cast<const double2*>(A.im + j);
    *reinterpret_cast<double2*>(A.re + i) = rj;
    *reinterpret_cast<double2*>(A.im + i) = ij;
    *reinterpret_cast<double2*>(A.re + j) = ri;
    *reinterpret_cast<double2*>(A.im + j) = ii;
  }
}

__global__ void __launch_bounds__(kThreads) swap_kernel_s(PairArgs A, uint64_t bit_a, uint64_t bit_b) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < A.nwork; w += stride) {
    const uint64_t base = deposit(w, A.pos, A.npos) | A.ones;
    const uint64_t i = base | bit_b, j = base | bit_a;
    double r = A.re[i], m = A.im[i];
    A.re[i] = A.re[j];
    A.im[i] = A.im[j];
    A.re[j] = r;
    A.im[j] = m;
  }
}

// ------------------------------------------------------------ launching
namespace {

void fill_positions(PairArgs& A, uint64_t special) {
  A.npos = 0;
  for (int q = 0; q < 64; ++q)
    if ((special >> q) & 1) A.pos[A.npos++] = (uint8_t)q;
}

template <int KIND>
int launch_pair(spz_state_t h, PairArgs& A, uint64_t special) {
  const int lowest = __builtin_ctzll(special);
  const uint64_t pairs = h->N >> __builtin_popcountll(special);
  if (lowest >= 1) {
    A.nwork = pairs / 2;
    if (A.nwork == 0) {  // a single pair (every qubit is special): scalar form
      A.nwork = pairs;
      pair_kernel_s<KIND><<<1, kThreads, 0, h->stream>>>(A);
    } else {
      pair_kernel_v2<KIND><<<grid_for(A.nwork), kThreads, 0, h->stream>>>(A);
    }
  } else if (A.tbit == 1) {
    A.nwork = pairs;
    pair_kernel_t0<KIND><<<grid_for(A.nwork), kThreads, 0, h->stream>>>(A);
  } else {
    A.nwork = pairs;
    pair_kernel_s<KIND><<<grid_for(A.nwork), kThreads, 0, h->stream>>>(A);
  }
  SPZ_CHECK_LAUNCH("pair kernel");
  return SPZ_OK;
}

template <int KIND>
int launch_diag(spz_state_t h, PairArgs& A, uint64_t fixed) {
  const uint64_t elems = h->N >> __builtin_popcountll(fixed);
  const int lowest = fixed ? __builtin_ctzll(fixed) : 64;
  if (lowest >= 1 && elems >= 2) {
    A.nwork = elems / 2;
    diag_kernel_v2<KIND><<<grid_for(A.nwork), kThreads, 0, h->stream>>>(A);
  } else {
    A.nwork = elems;
    diag_kernel_s<KIND><<<grid_for(A.nwork), kThreads, 0, h->stream>>>(A);
  }
  SPZ_CHECK_LAUNCH("diagonal kernel");
  return SPZ_OK;
}

}  // namespace

int launch_gate(spz_state_t h, const GateApp& g) {
  PairArgs A{};
  A.re = h->re;
  A.im = h->im;
  A.c = g.c;
  const uint64_t controls = g.ones | g.zeros;
  if (g.kind == SPZ_GATE_SWAP) {
    if (g.target == g.target2) return SPZ_OK;  // swap_apply with t0 == t1 is the identity
    const uint64_t special = controls | (1ull << g.target) | (1ull << g.target2);
    fill_positions(A, special);
    A.ones = g.ones;
    const uint64_t work = h->N >> __builtin_popcountll(special);
    const uint64_t bit_a = 1ull << g.target, bit_b = 1ull << g.target2;
    if (__builtin_ctzll(special) >= 1 && work >= 2) {
      A.nwork = work / 2;
      swap_kernel_v2<<<grid_for(A.nwork), kThreads, 0, h->stream>>>(A, bit_a, bit_b);
    } else {
      A.nwork = work;
      swap_kernel_s<<<grid_for(A.nwork), kThreads, 0, h->stream>>>(A, bit_a, bit_b);
    }
    SPZ_CHECK_LAUNCH("swap kernel");
    return SPZ_OK;
  }
  const uint64_t tbit = 1ull << g.target;
  A.tbit = tbit;
  if (is_diagonal(g.kind)) {
    // Z and P touch only amplitudes with the target bit set; RZ touches both halves.
    const uint64_t fixed = g.kind == SPZ_GATE_RZ ? controls : (controls | tbit);
    A.ones = g.kind == SPZ_GATE_RZ ? g.ones : (g.ones | tbit);
    fill_positions(A, fixed);
    switch (g.kind) {
      case SPZ_GATE_Z: return launch_diag<SPZ_GATE_Z>(h, A, fixed);
      case SPZ_GATE_P: return launch_diag<SPZ_GATE_P>(h, A, fixed);
      default: return launch_diag<SPZ_GATE_RZ>(h, A, fixed);
    }
  }
  const uint64_t special = controls | tbit;
  A.ones = g.ones;
  fill_positions(A, special);
  switch (g.kind) {
    case SPZ_GATE_H: return launch_pair<SPZ_GATE_H>(h, A, special);
    case SPZ_GATE_X: return launch_pair<SPZ_GATE_X>(h, A, special);
    case SPZ_GATE_Y: return launch_pair<SPZ_GATE_Y>(h, A, special);
    case SPZ_GATE_RX: return launch_pair<SPZ_GATE_RX>(h, A, special);
    case SPZ_GATE_RY: return launch_pair<SPZ_GATE_RY>(h, A, special);
    case SPZ_GATE_U: return launch_pair<SPZ_GATE_U>(h, A, special);
    default: return fail(SPZ_ERR_UNSUPPORTED, "gate kind not supported by the pair kernels");
  }
}

// Lazy per-gate mode (opt-in, spz_state_set_lazy): uncontrolled H, RX and RY
// are applied as the gate divided by a real scalar (1/sqrt 2, or the larger
// in magnitude of cos and sin of theta/2, so the remaining coefficient is at
// most 1): 4 FP64 instructions per pair instead of 8-12, which makes them
// bound by HBM.  RZ(theta) = e^{-i theta/2} P(theta): P touches only the 1
// half.  The scalars and phases multiply the handle's pending factor.  Sets
// *done when the gate was applied here.
int apply_lazy(spz_state_t h, const spz_gate& gate, uint32_t target, bool* done) {
  *done = false;
  const int k = gate.kind;
  if (k != SPZ_GATE_H && k != SPZ_GATE_RX && k != SPZ_GATE_RY && k != SPZ_GATE_RZ) return SPZ_OK;
  GateApp a;
  int rc = make_gate_app(h->n, gate, target, 0, 0, &a);
  if (rc) return rc;
  PairArgs A{};
  A.re = h->re;
  A.im = h->im;
  const uint64_t tbit = 1ull << target;
  A.tbit = tbit;
  if (k == SPZ_GATE_RZ) {
    spz_gate p{};
    p.kind = SPZ_GATE_P;
    p.p[0] = gate.p[0];
    rc = coef_for(p, &A.c);
    if (rc) return rc;
    A.ones = tbit;
    fill_positions(A, tbit);
    rc = launch_diag<SPZ_GATE_P>(h, A, tbit);
    if (rc) return rc;
    *done = true;
    return scale_factor(h, a.c.d0re, a.c.d0im);
  }
  fill_positions(A, tbit);
  double f;
  if (k == SPZ_GATE_H) {
    rc = launch_pair<FK_LAZY_H>(h, A, tbit);
    f = std::sqrt(0.5);
  } else {
    const double c = a.c.cs, sn = a.c.sn;
    const bool x = k == SPZ_GATE_RX;
    if (std::fabs(c) >= std::fabs(sn)) {
      A.c.cs = sn / c;
      rc = x ? launch_pair<FK_LAZY_RX_A>(h, A, tbit) : launch_pair<FK_LAZY_RY_A>(h, A, tbit);
      f = c;
    } else {
      A.c.cs = c / sn;
      rc = x ? launch_pair<FK_LAZY_RX_B>(h, A, tbit) : launch_pair<FK_LAZY_RY_B>(h, A, tbit);
      f = sn;
    }
  }
  if (rc) return rc;
  *done = true;
  return scale_factor(h, f, 0.0);
}

// Apply one gate under controls, with BitFlipNoise resolved on the host.
int apply_controlled(spz_state_t h, const spz_gate* gate, uint32_t target, uint64_t ones, uint64_t zeros) {
  if (!h || !gate) return fail(SPZ_ERR_NULL, "NULL argument");
  if (h->lazy && ones == 0 && zeros == 0) {
    bool done = false;
    int rc = apply_lazy(h, *gate, target, &done);
    if (rc || done) return rc;
  }
  if (gate->kind == SPZ_GATE_BITFLIP) {
    if (target >= h->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "target qubit out of range");
    if (!(gate->p[1] <= gate->p[0])) return SPZ_OK;  // gates.rs:1369: X iff epsilon <= prob
    spz_gate x{};
    x.kind = SPZ_GATE_X;
    GateApp a;
    int rc = make_gate_app(h->n, x, target, ones, zeros, &a);
    return rc ? rc : launch_gate(h, a);
  }
  GateApp a;
  int rc = make_gate_app(h->n, *gate, target, ones, zeros, &a);
  if (rc) return rc;
  return launch_gate(h, a);
}

}  // namespace spz

using namespace spz;

extern "C" {

int spz_apply(spz_state_t h, const spz_gate* gate, uint32_t target) {
  return apply_controlled(h, gate, target, 0, 0);
}

int spz_c_apply(spz_state_t h, const spz_gate* gate, uint32_t control, uint32_t target) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  if (control >= h->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "control qubit out of range");
  return apply_controlled(h, gate, target, 1ull << control, 0);
}

int spz_cc_apply(spz_state_t h, const spz_gate* gate, uint32_t control0, uint32_t control1, uint32_t target) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  if (control0 >= h->n || control1 >= h->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "control qubit out of range");
  if (control0 == control1) return fail(SPZ_ERR_INVALID_ARGUMENT, "duplicate control qubit");
  return apply_controlled(h, gate, target, (1ull << control0) | (1ull << control1), 0);
}

int spz_mc_apply(spz_state_t h, const spz_gate* gate, const uint32_t* controls, uint32_t ncontrols,
                 const uint32_t* zeros, uint32_t nzeros, uint32_t target) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  if (ncontrols && !controls) return fail(SPZ_ERR_NULL, "controls is NULL");
  if (nzeros && !zeros) return fail(SPZ_ERR_NULL, "zeros is NULL");
  uint64_t cm = 0, zm = 0;
  for (uint32_t i = 0; i < ncontrols; ++i) {
    if (controls[i] >= h->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "control qubit out of range");
    if ((cm >> controls[i]) & 1) return fail(SPZ_ERR_INVALID_ARGUMENT, "duplicate control qubit");
    cm |= 1ull << controls[i];
  }
  for (uint32_t i = 0; i < nzeros; ++i) {
    if (zeros[i] >= h->n || !((cm >> zeros[i]) & 1))
      return fail(SPZ_ERR_INVALID_ARGUMENT, "every zero must also be a control");
    zm |= 1ull << zeros[i];
  }
  return apply_controlled(h, gate, target, cm & ~zm, zm);
}

}  // extern "C"
