// ORACLE — test infrastructure only.
//
// CPU restatement of the reference's (QuState/spinoza v0.5.1) gate-application
// path, used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
// reference arm as the checker and as the timed CPU baseline.  Nothing in the
// product (spinoza_gb300/) links, loads or calls this file.
//
// The reference is Rust and cannot be built here (no cargo/rustc, crates not
// vendored), so this is a restatement, pinned against the golden vectors of
// the reference's own tests (tests/golden/reference_goldens.json).
//
// Arithmetic rules, so that results are bit-identical to the reference's:
//   * compile with -ffp-contract=off: Rust never contracts a*b+c into an FMA;
//   * std::fma exactly where the reference calls mul_add;
//   * gate coefficients from glibc sin/cos, as Rust's f64::sin_cos does;
//   * per-pair arithmetic copied operation by operation from the reference's
//     target functions (cited below).
// Where the reference is wrong, this file implements the intended math and
// says so (multi-control pairing, parallel H, RY under mc_apply, Mixed zeros).
//
// Parallelism: OpenMP over pairs/chunks from 15 qubits up, mirroring the
// reference's LOW_QUBIT_THRESHOLD (spinoza/src/gates.rs:14).  Gate results do
// not depend on the thread count; reductions use a fixed sequential order.

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>

#if defined(_OPENMP)
#include <omp.h>
#endif

namespace {

constexpr int kLowQubitThreshold = 15;              // gates.rs:14
constexpr double kSqrtOneHalf = 0.70710678118654752440;  // math.rs:5 (FRAC_1_SQRT_2)
constexpr double kPi = 3.14159265358979323846;           // math.rs:8

enum Kind { H = 0, M = 1, X = 2, Y = 3, Z = 4, P = 5, RX = 6, RY = 7, RZ = 8, SWAP = 9, U = 10,
            UNITARY = 11, BITFLIP = 12 };

enum Err { OK = 0, EINVAL_ = 1, EUNSUP = 2 };

struct Gate {
  int32_t kind;
  uint32_t q0, q1, pad;
  double p[3];
};

struct Op {  // same layout as spz_op in include/spinoza_gb300.h
  Gate gate;
  uint32_t target;
  int32_t controls_kind;
  uint64_t controls;
  uint64_t zeros;
};

// ------------------------------------------------------------ coefficients
// All 2x2 coefficients are computed exactly as the reference computes them.
struct Coef {
  double a, k, l, q, r, s, t;   // u_apply_target naming (gates.rs:1243-1254)
  double c, sn;                 // cos / sin (P, RY) or cos / neg_sin (RX)
  double d0re, d0im, d1re, d1im;  // RZ diagonal (gates.rs:930-937)
};

Coef coef_for(const Gate& g) {
  Coef c{};
  switch (g.kind) {
    case P: {  // gates.rs:862: let (sin, cos) = Float::sin_cos(angle)
      c.sn = std::sin(g.p[0]);
      c.c = std::cos(g.p[0]);
      break;
    }
    case RX: {  // gates.rs:749-751
      double theta = g.p[0] * 0.5;
      c.c = std::cos(theta);
      c.sn = -std::sin(theta);  // neg_sin
      break;
    }
    case RY: {  // gates.rs:1123-1124
      double theta = g.p[0] * 0.5;
      c.sn = std::sin(theta);
      c.c = std::cos(theta);
      break;
    }
    case RZ: {  // gates.rs:932-936
      double theta = g.p[0] * 0.5;
      double s = std::sin(theta), co = std::cos(theta);
      c.d0re = co; c.d0im = -s; c.d1re = co; c.d1im = s;
      break;
    }
    case U: {  // gates.rs:1285-1304
      double theta = g.p[0], phi = g.p[1], lambda = g.p[2];
      double st = std::sin(theta * 0.5), ct = std::cos(theta * 0.5);
      double sl = std::sin(lambda), cl = std::cos(lambda);
      double spl = std::sin(phi + lambda), cpl = std::cos(phi + lambda);
      double sp = std::sin(phi), cp = std::cos(phi);
      c.a = ct;                 // g[0] = (ct, 0)
      c.k = -cl * st;           // g[1] = (-cl*st, -sl*st)
      c.l = -sl * st;
      c.q = cp * st;            // g[2] = (cp*st, sp*st)
      c.r = sp * st;
      c.s = cpl * ct;           // g[3] = (cpl*ct, spl*ct)
      c.t = spl * ct;
      break;
    }
    default: break;
  }
  return c;
}

// ------------------------------------------------------------- pair updates
// (a, b) = (re, im) of s0; (c, d) = (re, im) of s1.
inline void h_pair(double& a, double& b, double& c, double& d) {  // gates.rs:547-562
  double a1 = kSqrtOneHalf * a, b1 = kSqrtOneHalf * b, c1 = kSqrtOneHalf * c, d1 = kSqrtOneHalf * d;
  a = a1 + c1; b = b1 + d1; c = a1 - c1; d = b1 - d1;
}
inline void x_pair(double& a, double& b, double& c, double& d) {  // gates.rs:329-334
  std::swap(a, c); std::swap(b, d);
}
inline void y_pair(double& a, double& b, double& c, double& d) {  // gates.rs:455-463
  std::swap(a, c); std::swap(b, d);   // swap s0 <-> s1
  std::swap(a, b); std::swap(c, d);   // swap re <-> im at s0 and at s1
  b = -b; c = -c;                     // im[s0] = -im[s0]; re[s1] = -re[s1]
}
inline void rx_pair(double& a, double& b, double& c, double& d, double cs, double nsn) {  // gates.rs:703-726
  double na = a * cs - d * nsn;
  double nb = b * cs + c * nsn;
  double nc = b * -nsn + c * cs;
  double nd = d * cs + a * nsn;
  a = na; b = nb; c = nc; d = nd;
}
inline void ry_pair(double& a, double& b, double& c, double& d, double sn, double cs) {  // gates.rs:1116-1119
  double na = a * cs - c * sn;
  double nb = b * cs - d * sn;
  double nc = a * sn + c * cs;
  double nd = b * sn + d * cs;
  a = na; b = nb; c = nc; d = nd;
}
inline void u_pair(double& c0, double& d0, double& m0, double& n0, const Coef& g) {  // gates.rs:1231-1267
  double c = c0, d = d0, m = m0, n = n0;
  double t0 = std::fma(g.a, c, std::fma(g.k, m, -g.l * n));
  double t1 = std::fma(g.a, d, std::fma(g.k, n, g.l * m));
  double t2 = std::fma(g.q, c, std::fma(-g.r, d, std::fma(g.s, m, -g.t * n)));
  double t3 = std::fma(g.q, d, std::fma(g.r, c, std::fma(g.s, n, g.t * m)));
  c0 = t0; d0 = t1; m0 = t2; n0 = t3;
}
inline void phase_elem(double& re, double& im, double cs, double sn) {  // gates.rs:837-838 (P)
  double z_re = re, z_im = im;
  re = std::fma(z_re, cs, -z_im * sn);
  im = std::fma(z_im, cs, z_re * sn);
}
inline void diag_elem(double& re, double& im, double mre, double mim) {  // gates.rs:939-946 (RZ)
  double c = re, d = im;
  re = std::fma(c, mre, -d * mim);
  im = std::fma(c, mim, d * mre);
}

// Apply the gate's action to one pair (s0, s1) — shared by the plain,
// controlled and multi-controlled forms, as in the reference, where the
// controlled functions call the same *_apply_target arithmetic.
inline void pair_update(int kind, const Coef& g, double* re, double* im, uint64_t s0, uint64_t s1) {
  double a = re[s0], b = im[s0], c = re[s1], d = im[s1];
  switch (kind) {
    case H: h_pair(a, b, c, d); break;
    case X: x_pair(a, b, c, d); break;
    case Y: y_pair(a, b, c, d); break;
    case Z: c = -c; d = -d; break;                                  // gates.rs:1054-1056
    case P: phase_elem(c, d, g.c, g.sn); break;                      // s1 only
    case RX: rx_pair(a, b, c, d, g.c, g.sn); break;
    case RY: ry_pair(a, b, c, d, g.sn, g.c); break;
    case RZ: diag_elem(a, b, g.d0re, g.d0im); diag_elem(c, d, g.d1re, g.d1im); break;
    case U: u_pair(a, b, c, d, g); break;
    default: break;
  }
  re[s0] = a; im[s0] = b; re[s1] = c; im[s1] = d;
}

bool is_one_qubit_kind(int k) { return k == H || k == X || k == Y || k == Z || k == P || k == RX || k == RY || k == RZ || k == U; }

inline bool par(int n) { return n >= kLowQubitThreshold; }

// ----------------------------------------------------------- gate kernels
// apply (gates.rs:215-232): chunked pair loop of every *_apply: chunk c of size
// 2^(t+1), pairs (base + i, base + i + 2^t) for i < 2^t.
void apply_1q(int n, double* re, double* im, int kind, const Coef& g, int t) {
  const uint64_t N = 1ull << n, dist = 1ull << t, chunks = N >> (t + 1);
#pragma omp parallel for schedule(static) if (par(n))
  for (int64_t ch = 0; ch < (int64_t)chunks; ++ch) {
    uint64_t base = (2 * (uint64_t)ch) << t;
    for (uint64_t i = 0; i < dist; ++i) pair_update(kind, g, re, im, base + i, base + i + dist);
  }
}

// c_apply family (gates.rs:376-399 and siblings): N/4 indices, insert a 1 at
// the higher then the lower of (control, target) (gates.rs:386-388), s0 = s1 - 2^t.
void c_apply_1q(int n, double* re, double* im, int kind, const Coef& g, int control, int t) {
  const uint64_t N = 1ull << n, end = N >> 2, dist = 1ull << t;
  const int lo = std::min(control, t), hi = std::max(control, t);
#pragma omp parallel for schedule(static) if (par(n))
  for (int64_t ii = 0; ii < (int64_t)end; ++ii) {
    uint64_t i = (uint64_t)ii;
    uint64_t x = i + (1ull << (hi - 1)) + ((i >> (hi - 1)) << (hi - 1));
    uint64_t s1 = x + (1ull << lo) + ((x >> lo) << lo);
    uint64_t s0 = s1 - dist;
    pair_update(kind, g, re, im, s0, s1);
  }
}

// Multi-control (gates.rs:290-320 and x_mc_apply :425, p_mc_apply :912,
// rx_mc_apply :807, ry_mc_apply :1209), with the intended semantics: the pair
// (s0, s0 + 2^t) is updated for every s0 whose target bit is 0, whose `ones`
// bits are all 1 and whose `zeros` bits are all 0.  The reference's scan
// (`if i & mask == mask { ...; i += dist }; i += 1`) never checks the target
// bit and mis-pairs for target >= 1; its mc_apply drops `zeros` from the mask
// instead of requiring 0; and ry_mc_apply applies RX.  None of these defects is
// reproduced here.
void mc_apply_1q(int n, double* re, double* im, int kind, const Coef& g, uint64_t ones,
                 uint64_t zeros, int t) {
  const uint64_t N = 1ull << n, dist = 1ull << t, cm = ones | zeros;
#pragma omp parallel for schedule(static) if (par(n))
  for (int64_t ii = 0; ii < (int64_t)N; ++ii) {
    uint64_t i = (uint64_t)ii;
    if ((i & dist) != 0) continue;
    if ((i & cm) != ones) continue;
    pair_update(kind, g, re, im, i, i + dist);
  }
}

// swap_apply (gates.rs:1376-1386) generalised to optional controls: swap
// amplitudes where bit t0 = 0 and bit t1 = 1 with the partner (t0 = 1, t1 = 0).
void swap_apply(int n, double* re, double* im, int t0, int t1, uint64_t ones, uint64_t zeros) {
  const uint64_t N = 1ull << n, cm = ones | zeros;
  for (uint64_t i = 0; i < N; ++i) {
    if (((i >> t0) & 1) == 0 && ((i >> t1) & 1) == 1 && (i & cm) == ones) {
      uint64_t j = i + (1ull << t0) - (1ull << t1);
      std::swap(re[i], re[j]);
      std::swap(im[i], im[j]);
    }
  }
}

bool valid_qubit(int n, int64_t q) { return q >= 0 && q < n; }

int do_apply(int n, double* re, double* im, const Gate& gate, int t) {
  if (gate.kind == SWAP) {
    if (!valid_qubit(n, gate.q0) || !valid_qubit(n, gate.q1)) return EINVAL_;
    if (gate.q0 == gate.q1) return OK;
    swap_apply(n, re, im, (int)gate.q0, (int)gate.q1, 0, 0);
    return OK;
  }
  if (gate.kind == BITFLIP) {  // gates.rs:1365-1374: X iff epsilon <= prob
    if (!valid_qubit(n, t)) return EINVAL_;
    if (gate.p[1] <= gate.p[0]) apply_1q(n, re, im, X, Coef{}, t);
    return OK;
  }
  if (!is_one_qubit_kind(gate.kind)) return EUNSUP;
  if (!valid_qubit(n, t)) return EINVAL_;
  apply_1q(n, re, im, gate.kind, coef_for(gate), t);
  return OK;
}

// Dispatch for a gate under a control set (ones must be 1, zeros must be 0).
int do_controlled(int n, double* re, double* im, const Gate& gate, uint64_t ones, uint64_t zeros, int t) {
  const uint64_t cm = ones | zeros;
  if ((cm >> n) != 0) return EINVAL_;
  if (gate.kind == SWAP) {
    if (!valid_qubit(n, gate.q0) || !valid_qubit(n, gate.q1)) return EINVAL_;
    if (((cm >> gate.q0) & 1) || ((cm >> gate.q1) & 1)) return EINVAL_;
    if (gate.q0 == gate.q1) return OK;
    swap_apply(n, re, im, (int)gate.q0, (int)gate.q1, ones, zeros);
    return OK;
  }
  if (!is_one_qubit_kind(gate.kind)) return EUNSUP;
  if (!valid_qubit(n, t) || ((cm >> t) & 1)) return EINVAL_;
  const Coef g = coef_for(gate);
  if (cm == 0) {
    apply_1q(n, re, im, gate.kind, g, t);
  } else if (zeros == 0 && __builtin_popcountll(ones) == 1) {
    c_apply_1q(n, re, im, gate.kind, g, __builtin_ctzll(ones), t);
  } else {
    mc_apply_1q(n, re, im, gate.kind, g, ones, zeros, t);
  }
  return OK;
}

// ----------------------------------------------------------- measurement
// measurement.rs:16-29: prob0 = sum over s0 of re^2 + im^2 (fixed sequential order here).
double prob0_of(int n, const double* re, const double* im, int t) {
  const uint64_t N = 1ull << n, dist = 1ull << t;
  double sum = 0.0;
  for (uint64_t base = 0; base < N; base += 2 * dist)
    for (uint64_t i = 0; i < dist; ++i) {
      double r = re[base + i], m = im[base + i];
      sum += r * r + m * m;
    }
  return sum;
}

// measurement.rs:12-92 with the outcome drawn from an explicit uniform u
// (outcome 1 iff u < 1 - prob0, i.e. Binomial(1, 1 - prob0)).
int measure(int n, double* re, double* im, int t, int reset, int forced, double u, uint8_t* out,
            double* p0out) {
  if (!valid_qubit(n, t)) return EINVAL_;
  if (forced != -1 && forced != 0 && forced != 1) return EINVAL_;
  const uint64_t N = 1ull << n, dist = 1ull << t;
  double prob0 = prob0_of(n, re, im, t);
  if (p0out) *p0out = prob0;
  uint8_t val = forced >= 0 ? (uint8_t)forced : (uint8_t)(u < 1.0 - prob0 ? 1 : 0);
  if (val == 0) {
    double scale = 1.0 / std::sqrt(prob0);
    for (uint64_t base = 0; base < N; base += 2 * dist)
      for (uint64_t i = 0; i < dist; ++i) {
        re[base + i] *= scale; im[base + i] *= scale;
        re[base + i + dist] = 0.0; im[base + i + dist] = 0.0;
      }
  } else {
    double prob1 = 1.0 - prob0;
    double scale = 1.0 / std::sqrt(prob1);
    for (uint64_t base = 0; base < N; base += 2 * dist)
      for (uint64_t i = 0; i < dist; ++i) {
        re[base + i + dist] *= scale; im[base + i + dist] *= scale;
        re[base + i] = 0.0; im[base + i] = 0.0;
      }
    if (reset) apply_1q(n, re, im, X, Coef{}, t);  // measurement.rs:87-89
  }
  *out = val;
  return OK;
}

// -------------------------------------------------------------- sampling
// The library's fixed blocked cumulative order (the reference's reservoir
// sampler is unseeded, so parity there is defined by this shared rule):
//   p_i = re*re + im*im; sub-chunks of 32 amplitudes, chunks of 8 sub-chunks
//   (256 amplitudes), super-chunks of 1024 chunks (all clipped to the state);
//   sub_total = sequential sum of its p; chunk_total = sequential sum of its
//   sub_totals; super_total = sequential sum of its chunk totals; super_base =
//   exclusive sequential scan; chunk_base = super_base + exclusive sequential
//   scan of chunk totals inside the super-chunk; target = u * total (clamped
//   below total); chunk = first c with chunk_end[c] > target; inside it the
//   running sum r = chunk_base + sub_total_k (sequential) picks the first
//   sub-chunk k with r > target, and from that sub-chunk's base the running
//   sum r + p_j (sequential) picks the first j with r > target.  When no
//   sub-chunk (or no j) qualifies, the outcome is the last index with p > 0 in
//   the chunk (or in the sub-chunk), or the chunk's first index.
constexpr uint64_t kSub = 32, kChunk = 256, kSuper = 1024;

int sample(int n, const double* re, const double* im, const double* u, uint64_t nshots, uint64_t* out) {
  const uint64_t N = 1ull << n;
  const uint64_t cs = std::min<uint64_t>(N, kChunk);
  const uint64_t ss = std::min<uint64_t>(cs, kSub);
  const uint64_t ns = cs / ss;  // sub-chunks per chunk
  const uint64_t nchunks = N / cs;
  const uint64_t nsuper = (nchunks + kSuper - 1) / kSuper;
  std::vector<double> sub(N / ss), ct(nchunks), st(nsuper), sb(nsuper), cb(nchunks), ce(nchunks);
  auto prob = [&](uint64_t i) { double r = re[i], m = im[i]; return r * r + m * m; };
  for (uint64_t b = 0; b < N / ss; ++b) {
    double t = 0.0;
    for (uint64_t j = 0; j < ss; ++j) t = t + prob(b * ss + j);
    sub[b] = t;
  }
  for (uint64_t c = 0; c < nchunks; ++c) {
    double t = 0.0;
    for (uint64_t k = 0; k < ns; ++k) t = t + sub[c * ns + k];
    ct[c] = t;
  }
  for (uint64_t s = 0; s < nsuper; ++s) {
    double t = 0.0;
    for (uint64_t c = s * kSuper; c < std::min(nchunks, (s + 1) * kSuper); ++c) t = t + ct[c];
    st[s] = t;
  }
  double total = 0.0;
  for (uint64_t s = 0; s < nsuper; ++s) { sb[s] = total; total = total + st[s]; }
  for (uint64_t s = 0; s < nsuper; ++s) {
    double pre = 0.0;
    for (uint64_t c = s * kSuper; c < std::min(nchunks, (s + 1) * kSuper); ++c) {
      cb[c] = sb[s] + pre;
      pre = pre + ct[c];
    }
  }
  for (uint64_t c = 0; c + 1 < nchunks; ++c) ce[c] = cb[c + 1];
  ce[nchunks - 1] = total;
  if (!(total > 0.0)) return EINVAL_;
  for (uint64_t k = 0; k < nshots; ++k) {
    double target = u[k] * total;
    if (target >= total) target = std::nextafter(total, 0.0);
    // first c with ce[c] > target
    uint64_t lo = 0, hi = nchunks - 1;
    while (lo < hi) {
      uint64_t mid = lo + (hi - lo) / 2;
      if (ce[mid] > target) hi = mid; else lo = mid + 1;
    }
    const uint64_t c = lo;
    double r = cb[c];
    uint64_t kk = ns;  // the sub-chunk, ns = none
    for (uint64_t q = 0; q < ns; ++q) {
      const double rn = r + sub[c * ns + q];
      if (rn > target) { kk = q; break; }
      r = rn;
    }
    uint64_t outcome = UINT64_MAX;
    if (kk < ns) {
      uint64_t last_pos = UINT64_MAX;
      for (uint64_t j = 0; j < ss; ++j) {
        const uint64_t i = c * cs + kk * ss + j;
        const double pj = prob(i);
        if (pj > 0.0) last_pos = i;
        r = r + pj;
        if (r > target) { outcome = i; break; }
      }
      if (outcome == UINT64_MAX) outcome = last_pos;
    }
    if (outcome == UINT64_MAX) {  // the last index of the chunk with p > 0, or its first
      outcome = c * cs;
      for (uint64_t j = cs; j-- > 0;)
        if (prob(c * cs + j) > 0.0) { outcome = c * cs + j; break; }
    }
    out[k] = outcome;
  }
  return OK;
}

// ------------------------------------------------------------------ rng
inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;
inline uint64_t stream_u64(uint64_t seed, uint64_t i) { return mix64(mix64(seed + kGolden) + (i + 1) * kGolden); }
inline double stream_uniform(uint64_t seed, uint64_t i) { return (double)(stream_u64(seed, i) >> 11) * 0x1.0p-53; }

}  // namespace

// =================================================================== C API
extern "C" {

int orc_apply(int n, double* re, double* im, const Gate* gate, int target) {
  return do_apply(n, re, im, *gate, target);
}

// c_apply (gates.rs:257-269), extended with Z (controlled-Z).
int orc_c_apply(int n, double* re, double* im, const Gate* gate, int control, int target) {
  if (!valid_qubit(n, control)) return EINVAL_;
  return do_controlled(n, re, im, *gate, 1ull << control, 0, target);
}

// cc_apply (gates.rs:272-277 -> x_cc_apply :401-423, correct pairing).
int orc_cc_apply(int n, double* re, double* im, const Gate* gate, int c0, int c1, int target) {
  if (!valid_qubit(n, c0) || !valid_qubit(n, c1) || c0 == c1) return EINVAL_;
  return do_controlled(n, re, im, *gate, (1ull << c0) | (1ull << c1), 0, target);
}

// mc_apply (gates.rs:290-320) with masks: `controls` all controls, `zeros` the
// subset that must read 0.
int orc_mc_apply(int n, double* re, double* im, const Gate* gate, uint64_t controls, uint64_t zeros,
                 int target) {
  if ((zeros & ~controls) != 0) return EINVAL_;
  return do_controlled(n, re, im, *gate, controls & ~zeros, zeros, target);
}

// QuantumCircuit::execute (circuit.rs:552-600), with QubitTracker state in
// (measured, values).  Ones with any number of controls applies the gate under
// all of them (the reference's cc_apply path reads only controls[0..2]).
int orc_execute(int n, double* re, double* im, const Op* ops, uint64_t nops, uint64_t* measured,
                uint64_t* values) {
  uint64_t meas = measured ? *measured : 0, vals = values ? *values : 0;
  for (uint64_t i = 0; i < nops; ++i) {
    const Op& op = ops[i];
    int rc = OK;
    const int t = (int)op.target;
    if (op.gate.kind == M) {
      if (op.controls_kind != 0) return EUNSUP;
      if (!valid_qubit(n, t)) return EINVAL_;
      if (!((meas >> t) & 1)) {
        uint8_t v = 0;
        rc = measure(n, re, im, t, 1, -1, op.gate.p[0], &v, nullptr);
        meas |= 1ull << t;
        vals = (vals & ~(1ull << t)) | ((uint64_t)v << t);
      }
    } else if (op.controls_kind == 0) {
      rc = do_apply(n, re, im, op.gate, t);
    } else if (op.controls_kind == 1) {
      if (op.controls == 0 || (op.controls & (op.controls - 1)) != 0) return EINVAL_;
      int c = __builtin_ctzll(op.controls);
      if ((meas >> c) & 1) {
        if ((vals >> c) & 1) rc = do_apply(n, re, im, op.gate, t);
      } else {
        rc = do_controlled(n, re, im, op.gate, op.controls, 0, t);
      }
    } else if (op.controls_kind == 2) {
      rc = do_controlled(n, re, im, op.gate, op.controls, 0, t);
    } else if (op.controls_kind == 3) {
      if ((op.zeros & ~op.controls) != 0) return EINVAL_;
      rc = do_controlled(n, re, im, op.gate, op.controls & ~op.zeros, op.zeros, t);
    } else {
      return EINVAL_;
    }
    if (rc != OK) return rc;
  }
  if (measured) *measured = meas;
  if (values) *values = vals;
  return OK;
}

int orc_measure_qubit(int n, double* re, double* im, int target, int reset, int forced, double u,
                      uint8_t* out, double* prob0) {
  return measure(n, re, im, target, reset, forced, u, out, prob0);
}

double orc_prob0(int n, const double* re, const double* im, int target) { return prob0_of(n, re, im, target); }

// core.rs:198-219
double orc_qubit_expectation_value(int n, const double* re, const double* im, int target) {
  return 2.0 * prob0_of(n, re, im, target) - 1.0;
}

// core.rs:222-264: clone, apply the Pauli, Re<psi|O psi> = sum a*c + b*d.
int orc_xyz_expectation_value(int n, const double* re, const double* im, char obs, const uint32_t* targets,
                              uint32_t nt, double* out) {
  if (obs != 'x' && obs != 'y' && obs != 'z') return EINVAL_;
  const uint64_t N = 1ull << n;
  std::vector<double> wr(re, re + N), wi(im, im + N);
  for (uint32_t k = 0; k < nt; ++k) {
    if (!valid_qubit(n, targets[k])) return EINVAL_;
    int kind = obs == 'z' ? Z : (obs == 'y' ? Y : X);
    apply_1q(n, wr.data(), wi.data(), kind, Coef{}, (int)targets[k]);
    double s = 0.0;
    for (uint64_t i = 0; i < N; ++i) s += re[i] * wr[i] + im[i] * wi[i];
    out[k] = s;
    std::memcpy(wr.data(), re, N * 8);
    std::memcpy(wi.data(), im, N * 8);
  }
  return OK;
}

struct Term { double coeff; uint64_t x_mask; uint64_t z_mask; };

// Sum of Pauli strings, by the reference's mechanism (core.rs:222-264): for
// each term clone the state, apply the string qubit by qubit (X, Y = both
// masks, Z), and add coeff * Re<psi|P psi>.
int orc_pauli_expectation(int n, const double* re, const double* im, const Term* terms, uint64_t nterms,
                          double* out) {
  const uint64_t N = 1ull << n;
  std::vector<double> wr(N), wi(N);
  double total = 0.0;
  for (uint64_t k = 0; k < nterms; ++k) {
    if (((terms[k].x_mask | terms[k].z_mask) >> n) != 0) return EINVAL_;
    std::memcpy(wr.data(), re, N * 8);
    std::memcpy(wi.data(), im, N * 8);
    for (int q = 0; q < n; ++q) {
      bool x = (terms[k].x_mask >> q) & 1, z = (terms[k].z_mask >> q) & 1;
      if (x && z) apply_1q(n, wr.data(), wi.data(), Y, Coef{}, q);
      else if (x) apply_1q(n, wr.data(), wi.data(), X, Coef{}, q);
      else if (z) apply_1q(n, wr.data(), wi.data(), Z, Coef{}, q);
    }
    double s = 0.0;
    for (uint64_t i = 0; i < N; ++i) s += re[i] * wr[i] + im[i] * wi[i];
    total += terms[k].coeff * s;
  }
  *out = total;
  return OK;
}

// core.rs:184-191
int orc_iqft(int n, double* re, double* im, const uint32_t* targets, uint32_t nt) {
  for (int64_t j = (int64_t)nt - 1; j >= 0; --j) {
    Gate h{H, 0, 0, 0, {0, 0, 0}};
    int rc = do_apply(n, re, im, h, (int)targets[j]);
    if (rc) return rc;
    for (int64_t k = j - 1; k >= 0; --k) {
      Gate p{P, 0, 0, 0, {-kPi / std::ldexp(1.0, (int)(j - k)), 0, 0}};
      if (!valid_qubit(n, targets[k])) return EINVAL_;
      rc = do_controlled(n, re, im, p, 1ull << targets[j], 0, (int)targets[k]);
      if (rc) return rc;
    }
  }
  return OK;
}

// transform_u / c_transform_u (gates.rs:1427-1487) with the state's own n
// (the reference takes n from the matrix width, gates.rs:1430) and the
// row accumulation of unitary_col_vec_mul (gates.rs:1388-1425):
// re += a*v_re - b*v_im; im += a*v_im + b*v_re, j ascending.
int orc_apply_unitary(int n, double* re, double* im, const double* ur, const double* ui, int m, int t, int control) {
  if (m < 1 || t < 0 || t + m > n) return EINVAL_;
  if (control >= 0 && (control >= n || (control >= t && control < t + m))) return EINVAL_;
  const uint64_t N = 1ull << n, M = 1ull << m;
  std::vector<double> vr(M), vi(M);
  for (uint64_t suffix = 0; suffix < (1ull << t); ++suffix)
    for (uint64_t prefix = 0; prefix < (N >> (t + m)); ++prefix) {
      const uint64_t base = prefix * (1ull << (t + m)) + suffix;
      if (control >= 0 && !((base >> control) & 1)) continue;
      for (uint64_t j = 0; j < M; ++j) {
        vr[j] = re[base + j * (1ull << t)];
        vi[j] = im[base + j * (1ull << t)];
      }
      for (uint64_t i = 0; i < M; ++i) {
        double dr = 0.0, di = 0.0;
        for (uint64_t j = 0; j < M; ++j) {
          const double a = ur[i * M + j], b = ui[i * M + j];
          dr += a * vr[j] - b * vi[j];
          di += a * vi[j] + b * vr[j];
        }
        re[base + i * (1ull << t)] = dr;
        im[base + i * (1ull << t)] = di;
      }
    }
  return OK;
}

int orc_sample(int n, const double* re, const double* im, const double* u, uint64_t nshots, uint64_t* out) {
  return sample(n, re, im, u, nshots, out);
}

uint64_t orc_stream_u64(uint64_t seed, uint64_t i) { return stream_u64(seed, i); }
double orc_stream_uniform(uint64_t seed, uint64_t i) { return stream_uniform(seed, i); }

// Uniform [-1,1) state from the counter stream: re[i] = 2 u(2i) - 1, im[i] = 2 u(2i+1) - 1.
void orc_fill_uniform(int n, double* re, double* im, uint64_t seed) {
  const uint64_t N = 1ull << n;
#pragma omp parallel for schedule(static) if (par(n))
  for (int64_t i = 0; i < (int64_t)N; ++i) {
    re[i] = 2.0 * stream_uniform(seed, 2 * (uint64_t)i) - 1.0;
    im[i] = 2.0 * stream_uniform(seed, 2 * (uint64_t)i + 1) - 1.0;
  }
}

int orc_num_threads(void) {
#if defined(_OPENMP)
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
