// Per-pair and per-element gate arithmetic, shared by the plain per-gate
// kernels and the fused tile executor.  Each function performs the reference's
// floating-point operations in the reference's order (no contraction, FMA only
// where the reference calls mul_add), so results are bit-identical to
// spinoza's CPU path; the cited lines are in spinoza/src/gates.rs.
//
// (a, b) = (re, im) of s0 (target bit 0); (c, d) = (re, im) of s1.
#pragma once

#include "common.cuh"

namespace spz {

constexpr double kSqrtOneHalf = 0.70710678118654752440;  // math.rs:5

template <int KIND>
__device__ __forceinline__ void gate_pair(const Coef& g, double& a, double& b, double& c, double& d) {
  if constexpr (KIND == SPZ_GATE_H) {  // h_apply_strat2, gates.rs:547-562
    const double a1 = dmul(kSqrtOneHalf, a), b1 = dmul(kSqrtOneHalf, b);
    const double c1 = dmul(kSqrtOneHalf, c), d1 = dmul(kSqrtOneHalf, d);
    a = dadd(a1, c1);
    b = dadd(b1, d1);
    c = dsub(a1, c1);
    d = dsub(b1, d1);
  } else if constexpr (KIND == SPZ_GATE_X) {  // x_apply_target, gates.rs:329-334
    double t = a; a = c; c = t;
    t = b; b = d; d = t;
  } else if constexpr (KIND == SPZ_GATE_Y) {  // y_proc_chunk, gates.rs:455-463
    const double na = d, nb = dneg(c), nc = dneg(b), nd = a;
    a = na; b = nb; c = nc; d = nd;
  } else if constexpr (KIND == SPZ_GATE_Z) {  // z_proc_chunk, gates.rs:1054-1056
    c = dneg(c);
    d = dneg(d);
  } else if constexpr (KIND == SPZ_GATE_P) {  // p_proc_chunk, gates.rs:837-838 (s1 only)
    const double zr = c, zi = d;
    c = dfma(zr, g.cs, dmul(zi, g.nsn));
    d = dfma(zi, g.cs, dmul(zr, g.sn));
  } else if constexpr (KIND == SPZ_GATE_RX) {  // rx_apply_target, gates.rs:713-725
    const double na = dsub(dmul(a, g.cs), dmul(d, g.nsn));
    const double nb = dadd(dmul(b, g.cs), dmul(c, g.nsn));
    const double nc = dadd(dmul(b, g.sn), dmul(c, g.cs));  // b * -neg_sin + c * cos
    const double nd = dadd(dmul(d, g.cs), dmul(a, g.nsn));
    a = na; b = nb; c = nc; d = nd;
  } else if constexpr (KIND == SPZ_GATE_RY) {  // ry_apply_strategy2, gates.rs:1116-1119
    const double na = dsub(dmul(a, g.cs), dmul(c, g.sn));
    const double nb = dsub(dmul(b, g.cs), dmul(d, g.sn));
    const double nc = dadd(dmul(a, g.sn), dmul(c, g.cs));
    const double nd = dadd(dmul(b, g.sn), dmul(d, g.cs));
    a = na; b = nb; c = nc; d = nd;
  } else if constexpr (KIND == SPZ_GATE_RZ) {  // rz_apply_strategy1, gates.rs:939-946
    const double ar = a, ai = b, cr = c, ci = d;
    a = dfma(ar, g.d0re, dmul(dneg(ai), g.d0im));
    b = dfma(ar, g.d0im, dmul(ai, g.d0re));
    c = dfma(cr, g.d1re, dmul(dneg(ci), g.d1im));
    d = dfma(cr, g.d1im, dmul(ci, g.d1re));
  } else if constexpr (KIND == SPZ_GATE_U) {  // u_apply_target, gates.rs:1256-1259
    const double cc = a, dd = b, m = c, n = d;
    const double t0 = dfma(g.a, cc, dfma(g.k, m, dmul(dneg(g.l), n)));
    const double t1 = dfma(g.a, dd, dfma(g.k, n, dmul(g.l, m)));
    const double t2 = dfma(g.q, cc, dfma(dneg(g.r), dd, dfma(g.s, m, dmul(dneg(g.t), n))));
    const double t3 = dfma(g.q, dd, dfma(g.r, cc, dfma(g.s, n, dmul(g.t, m))));
    a = t0; b = t1; c = t2; d = t3;
  }
}

// Fast-mode lazy ops (the gate divided by a scalar carried elsewhere): four
// FP64 instructions per pair.  Coefficient in g.cs (t or u).
template <int FK>
__device__ __forceinline__ void fast_pair_t(const double t, double& a, double& b, double& c, double& d) {
  double na, nb, nc, nd;
  if constexpr (FK == FK_LAZY_H) {
    na = dadd(a, c); nb = dadd(b, d); nc = dsub(a, c); nd = dsub(b, d);
  } else if constexpr (FK == FK_LAZY_RX_A) {  // s0 - i t s1, -i t s0 + s1
    na = dfma(t, d, a); nb = dfma(dneg(t), c, b); nc = dfma(t, b, c); nd = dfma(dneg(t), a, d);
  } else if constexpr (FK == FK_LAZY_RX_B) {  // u s0 - i s1, -i s0 + u s1
    na = dfma(t, a, d); nb = dfma(t, b, dneg(c)); nc = dfma(t, c, b); nd = dfma(t, d, dneg(a));
  } else if constexpr (FK == FK_LAZY_RY_A) {  // s0 - t s1, t s0 + s1
    na = dfma(dneg(t), c, a); nb = dfma(dneg(t), d, b); nc = dfma(t, a, c); nd = dfma(t, b, d);
  } else {  // FK_LAZY_RY_B: u s0 - s1, s0 + u s1
    na = dfma(t, a, dneg(c)); nb = dfma(t, b, dneg(d)); nc = dfma(t, c, a); nd = dfma(t, d, b);
  }
  a = na; b = nb; c = nc; d = nd;
}

template <int FK>
__device__ __forceinline__ void fast_pair(const Coef& g, double& a, double& b, double& c, double& d) {
  fast_pair_t<FK>(g.cs, a, b, c, d);
}

// A lazy op whose kind is known only at run time (uniform over the block).
__device__ __forceinline__ void fast_pair_kind(int kind, double t, double& a, double& b, double& c, double& d) {
  switch (kind) {
    case FK_LAZY_H: fast_pair_t<FK_LAZY_H>(t, a, b, c, d); break;
    case FK_LAZY_RX_A: fast_pair_t<FK_LAZY_RX_A>(t, a, b, c, d); break;
    case FK_LAZY_RX_B: fast_pair_t<FK_LAZY_RX_B>(t, a, b, c, d); break;
    case FK_LAZY_RY_A: fast_pair_t<FK_LAZY_RY_A>(t, a, b, c, d); break;
    default: fast_pair_t<FK_LAZY_RY_B>(t, a, b, c, d); break;
  }
}

// Diagonal gates on one amplitude; `one` is the amplitude's target bit.
template <int KIND>
__device__ __forceinline__ void gate_diag(const Coef& g, bool one, double& re, double& im) {
  if constexpr (KIND == SPZ_GATE_Z) {
    if (one) { re = dneg(re); im = dneg(im); }
  } else if constexpr (KIND == SPZ_GATE_P) {
    if (one) {
      const double zr = re, zi = im;
      re = dfma(zr, g.cs, dmul(zi, g.nsn));
      im = dfma(zi, g.cs, dmul(zr, g.sn));
    }
  } else if constexpr (KIND == SPZ_GATE_RZ) {
    const double mre = one ? g.d1re : g.d0re, mim = one ? g.d1im : g.d0im;
    const double cr = re, ci = im;
    re = dfma(cr, mre, dmul(dneg(ci), mim));
    im = dfma(cr, mim, dmul(ci, mre));
  }
}

}  // namespace spz
