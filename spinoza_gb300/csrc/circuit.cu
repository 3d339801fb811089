// Circuit executor: QuantumCircuit::execute (spinoza/src/circuit.rs:552-600)
// and iqft (spinoza/src/core.rs:184-191).
//
// The reference makes one full pass over the state per gate.  Here a host-side
// planner groups gates into passes over shared-memory tiles: a pass fixes a set
// L of k "local" qubits (always including the lowest qubits, so every tile row is
// a contiguous, coalesced run of amplitudes); each thread block loads a tile of
// 2^k amplitudes (all values of the local bits, for one value of the other
// bits) into shared memory, applies every gate of the pass whose target(s) lie
// in L — controls and diagonal gates may sit on any qubit — and writes the tile
// back.  A run of gates costs one HBM read and one write of the state.
//
// Exactness: each gate's per-pair arithmetic is the plain kernel's (the
// reference's own operations).  The planner keeps program order except where a
// swap of two gates is bit-exact (see ExactClass below).  So a fused run is
// bit-identical to the sequential one.
#include <cuda.h>  // CUtensorMap (the encoder is reached through the runtime's driver entry point)
#include <cudaTypedefs.h>

#include <algorithm>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "gate_math.cuh"
#include "tile_ops.cuh"
#include "executor.cuh"

namespace spz {

int measure_qubit(spz_state_t h, uint32_t target, int reset, int forced, double u, uint8_t* outcome,
                  double* prob0_out);
int apply_controlled(spz_state_t h, const spz_gate* gate, uint32_t target, uint64_t ones, uint64_t zeros);

struct PassArgs {
  double* re;
  double* im;
  uint64_t tile_begin;  // tiles tile_begin .. ntiles - 1 of the pass
  uint64_t ntiles;
  const TileGate* gates;
  const double2* tables;  // fast-mode phase tables (re, im)
  const int32_t* outcomes;  // device-side measurement outcomes (conditioned gates)
  int ngates;
  int k;            // local qubits
  int c;            // low contiguous local qubits (0..c-1)
  int nhigh;        // k - c
  uint8_t lpos[kTileMaxK];  // sorted local qubits
  // slab_on != 0: the launch covers only the tiles whose three tile-index bits
  // at slab_pos (the non-local qubits of one host-copy slab) read `slab`; the
  // loop index t then runs over the other tile-index bits.
  uint32_t slab_on;
  uint32_t slab_pos;
  uint32_t slab;
};

// The tile index of loop index t (see PassArgs::slab_on).
__device__ __forceinline__ uint64_t slab_tile(const PassArgs& A, uint64_t t) {
  if (!A.slab_on) return t;
  const uint32_t sp = A.slab_pos;
  return ((t >> sp) << (sp + 3)) | ((uint64_t)A.slab << sp) | (t & ((1ull << sp) - 1));
}

// ------------------------------------------------------------ device side
// Nibble-swizzled tile layout: removes the 2-way bank conflicts of pair ops on
// tile bits 0-3, but measured no faster on the 30-qubit brickwork (the passes
// are DFMA-bound, not shared-memory bound), so off by default.
#ifndef SPZ_TILE_SWIZZLE
#define SPZ_TILE_SWIZZLE 0
#endif
#if SPZ_TILE_SWIZZLE
using TileSwizzle = NibbleSwizzle;  // tile layout in shared memory (tile_ops.cuh)
#else
using TileSwizzle = NoSwizzle;
#endif

// Lazy op with its phase: s1 *= table[parities], then the lazy rotation.  Lazy
// ops are uncontrolled, so the target is the only inserted position.  The
// masks exclude the target, so both members of a pair share the entry.  (The
// tables, 2-8 entries in a brickwork, are read through L1; holding them one
// entry per lane and reading them with warp shuffles measured 1.2% slower.)
template <int FK, int PM>
__device__ __forceinline__ void tile_fast_phase(const TileGate& g, const double2* __restrict__ tab, uint64_t base,
                                                double* sre, double* sim, uint32_t npairs) {
  const Enumerator<1, TileGate> E(g);
  const uint32_t tbit = g.tbit;
  const Coef c = g.c;
  uint32_t em[PM];
  uint32_t bidx = 0;
#pragma unroll
  for (int j = 0; j < PM; ++j) {
    bidx |= (uint32_t)(__popcll(base & g.pmask[j]) & 1) << j;
    em[j] = g.pemask[j];
  }
  if constexpr (kTileBatch > 1) {  // see tile_pair
    const uint32_t step = blockDim.x;
    for (uint32_t m0 = threadIdx.x; m0 < npairs; m0 += kTileBatch * step) {
      uint32_t s0[kTileBatch], s1[kTileBatch];
      double a[kTileBatch], b[kTileBatch], x[kTileBatch], d[kTileBatch];
      double2 w[kTileBatch];
#pragma unroll
      for (int u = 0; u < kTileBatch; ++u) {
        const uint32_t m = m0 + u * step;
        const uint32_t e0 = E(m < npairs ? m : m0);
        s0[u] = TileSwizzle::at(e0);
        s1[u] = TileSwizzle::at(e0 | tbit);
        uint32_t idx = bidx;
#pragma unroll
        for (int j = 0; j < PM; ++j) idx ^= (uint32_t)(__popc(e0 & em[j]) & 1) << j;
        w[u] = __ldg(tab + idx);
        a[u] = sre[s0[u]]; b[u] = sim[s0[u]]; x[u] = sre[s1[u]]; d[u] = sim[s1[u]];
      }
#pragma unroll
      for (int u = 0; u < kTileBatch; ++u) {
        const double r = x[u], i = d[u];
        x[u] = dfma(r, w[u].x, dmul(dneg(i), w[u].y));
        d[u] = dfma(r, w[u].y, dmul(i, w[u].x));
        fast_pair<FK>(c, a[u], b[u], x[u], d[u]);
      }
#pragma unroll
      for (int u = 0; u < kTileBatch; ++u) {
        if (m0 + u * step < npairs) {
          sre[s0[u]] = a[u]; sim[s0[u]] = b[u]; sre[s1[u]] = x[u]; sim[s1[u]] = d[u];
        }
      }
    }
  } else {
#pragma unroll kTileUnroll
    for (uint32_t m = threadIdx.x; m < npairs; m += blockDim.x) {
      const uint32_t e0 = E(m);
      const uint32_t s0 = TileSwizzle::at(e0), s1 = TileSwizzle::at(e0 | tbit);
      uint32_t idx = bidx;
#pragma unroll
      for (int j = 0; j < PM; ++j) idx ^= (uint32_t)(__popc(e0 & em[j]) & 1) << j;
      const double2 w = __ldg(tab + idx);
      double a = sre[s0], b = sim[s0];
      const double r = sre[s1], i = sim[s1];
      double x = dfma(r, w.x, dmul(dneg(i), w.y));
      double d = dfma(r, w.y, dmul(i, w.x));
      fast_pair<FK>(c, a, b, x, d);
      sre[s0] = a; sim[s0] = b; sre[s1] = x; sim[s1] = d;
    }
  }
}

template <int FK>
__device__ __forceinline__ void tile_fast_phase_pm(const TileGate& g, const double2* tab, uint64_t base, double* sre,
                                                   double* sim, uint32_t npairs) {
  switch (g.pm) {
    case 1: tile_fast_phase<FK, 1>(g, tab, base, sre, sim, npairs); break;
    case 2: tile_fast_phase<FK, 2>(g, tab, base, sre, sim, npairs); break;
    case 3: tile_fast_phase<FK, 3>(g, tab, base, sre, sim, npairs); break;
    case 4: tile_fast_phase<FK, 4>(g, tab, base, sre, sim, npairs); break;
    case 5: tile_fast_phase<FK, 5>(g, tab, base, sre, sim, npairs); break;
    case 6: tile_fast_phase<FK, 6>(g, tab, base, sre, sim, npairs); break;
    case 7: tile_fast_phase<FK, 7>(g, tab, base, sre, sim, npairs); break;
    default: tile_fast_phase<FK, kPhaseMaxTerms>(g, tab, base, sre, sim, npairs); break;
  }
}

// Fast-mode phase op: per amplitude, a table entry chosen by index parities.
// The amplitudes visited are the tile's (npos = 0) or, for a local half bit,
// those with that bit set (inserted by the enumeration).
// parity(x & mask) = parity(base & mask) ^ parity(e & local part of mask); the
// first is uniform over the tile.
template <int NPOS, int PM>
__device__ __forceinline__ void tile_phase(const TileGate& g, const double2* __restrict__ tab, uint64_t base,
                                           double* sre, double* sim, uint32_t nelem) {
  const Enumerator<NPOS, TileGate> E(g);
  uint32_t em[PM > 0 ? PM : 1];
  uint32_t bidx = 0;
#pragma unroll
  for (int j = 0; j < PM; ++j) {
    bidx |= (uint32_t)(__popcll(base & g.pmask[j]) & 1) << j;
    em[j] = g.pemask[j];
  }
#pragma unroll kTileUnroll
  for (uint32_t m = threadIdx.x; m < nelem; m += blockDim.x) {
    const uint32_t e0 = E(m);
    uint32_t idx = bidx;
#pragma unroll
    for (int j = 0; j < PM; ++j) idx ^= (uint32_t)(__popc(e0 & em[j]) & 1) << j;
    const uint32_t e = TileSwizzle::at(e0);
    const double2 w = __ldg(tab + idx);
    const double r = sre[e], i = sim[e];
    sre[e] = dfma(r, w.x, dmul(dneg(i), w.y));
    sim[e] = dfma(r, w.y, dmul(i, w.x));
  }
}

template <int NPOS>
__device__ __forceinline__ void tile_phase_pm(const TileGate& g, const double2* tab, uint64_t base, double* sre,
                                              double* sim, uint32_t nelem) {
  switch (g.pm) {
    case 0: tile_phase<NPOS, 0>(g, tab, base, sre, sim, nelem); break;
    case 1: tile_phase<NPOS, 1>(g, tab, base, sre, sim, nelem); break;
    case 2: tile_phase<NPOS, 2>(g, tab, base, sre, sim, nelem); break;
    case 3: tile_phase<NPOS, 3>(g, tab, base, sre, sim, nelem); break;
    case 4: tile_phase<NPOS, 4>(g, tab, base, sre, sim, nelem); break;
    case 5: tile_phase<NPOS, 5>(g, tab, base, sre, sim, nelem); break;
    case 6: tile_phase<NPOS, 6>(g, tab, base, sre, sim, nelem); break;
    case 7: tile_phase<NPOS, 7>(g, tab, base, sre, sim, nelem); break;
    default: tile_phase<NPOS, kPhaseMaxTerms>(g, tab, base, sre, sim, nelem); break;
  }
}

// Fast mode, two lazy rotations fused (TM_LAZY2): on each block of four
// amplitudes (tile bits b1 = tbit, b2 = tbit2), the first op's phase on the
// b1 = 1 half and the second op's phase on the b2 = 1 half are applied
// together (the second op's phase masks never contain the first op's qubit,
// so it commutes with the first rotation): three complex multiplies by one
// table row instead of four, then the first rotation on the two pairs along
// b1 and the second on the two pairs along b2.  28 FP64 instructions per
// block instead of 32, one shared-memory round trip and one barrier for both.
template <int PM>
__device__ __forceinline__ void tile_lazy2(const TileGate& g, const double2* __restrict__ tab, uint64_t base,
                                           double* sre, double* sim, uint32_t nblocks) {
  const Enumerator<2, TileGate> E(g);
  const uint32_t b1 = g.tbit, b2 = g.tbit2;
  const double t1 = g.c.cs, t2 = g.c.sn;
  const int k1 = g.kind, k2 = g.kind2;
  uint32_t em[PM > 0 ? PM : 1];
  uint32_t bidx = 0;
#pragma unroll
  for (int j = 0; j < PM; ++j) {
    if (j < g.pm) {
      bidx |= (uint32_t)(__popcll(base & g.pmask[j]) & 1) << j;
      em[j] = g.pemask[j];
    } else {
      em[j] = 0;
    }
  }
  for (uint32_t m = threadIdx.x; m < nblocks; m += blockDim.x) {
    const uint32_t e = E(m);
    uint32_t idx = bidx;
#pragma unroll
    for (int j = 0; j < PM; ++j) idx ^= (uint32_t)(__popc(e & em[j]) & 1) << j;
    const double2* row = tab + 3 * idx;
    const uint32_t e1 = TileSwizzle::at(e | b1), e2 = TileSwizzle::at(e | b2), e3 = TileSwizzle::at(e | b1 | b2);
    const uint32_t e0 = TileSwizzle::at(e);
    double r0 = sre[e0], i0 = sim[e0];
    double r1 = sre[e1], i1 = sim[e1];
    double r2 = sre[e2], i2 = sim[e2];
    double r3 = sre[e3], i3 = sim[e3];
    {
      const double2 w1 = __ldg(row), w2 = __ldg(row + 1), w3 = __ldg(row + 2);
      double x = r1, y = i1;
      r1 = dfma(x, w1.x, dmul(dneg(y), w1.y));
      i1 = dfma(x, w1.y, dmul(y, w1.x));
      x = r2; y = i2;
      r2 = dfma(x, w2.x, dmul(dneg(y), w2.y));
      i2 = dfma(x, w2.y, dmul(y, w2.x));
      x = r3; y = i3;
      r3 = dfma(x, w3.x, dmul(dneg(y), w3.y));
      i3 = dfma(x, w3.y, dmul(y, w3.x));
    }
    fast_pair_kind(k1, t1, r0, i0, r1, i1);  // along b1
    fast_pair_kind(k1, t1, r2, i2, r3, i3);
    fast_pair_kind(k2, t2, r0, i0, r2, i2);  // along b2
    fast_pair_kind(k2, t2, r1, i1, r3, i3);
    sre[e0] = r0; sim[e0] = i0;
    sre[e1] = r1; sim[e1] = i1;
    sre[e2] = r2; sim[e2] = i2;
    sre[e3] = r3; sim[e3] = i3;
  }
}

__device__ __forceinline__ void tile_lazy2_pm(const TileGate& g, const double2* tab, uint64_t base, double* sre,
                                              double* sim, uint32_t nblocks) {
  switch (g.pm) {
    case 2: tile_lazy2<2>(g, tab, base, sre, sim, nblocks); break;
    case 3: tile_lazy2<3>(g, tab, base, sre, sim, nblocks); break;
    case 4: tile_lazy2<4>(g, tab, base, sre, sim, nblocks); break;
    case 5: tile_lazy2<5>(g, tab, base, sre, sim, nblocks); break;
    case 6: tile_lazy2<6>(g, tab, base, sre, sim, nblocks); break;
    default: tile_lazy2<kPhaseMaxTerms>(g, tab, base, sre, sim, nblocks); break;
  }
}

// ------------------------------------------------ warp-shuffle runs
// SPZ_EXEC_SHUFFLE: a run of consecutive gates whose pairs lie inside 32
// consecutive amplitudes of the tile (target on tile bits 0-4) is applied
// with the amplitudes in registers: lane l of a warp holds amplitude 32 r + l
// of rows r, the partner of a pair is fetched with __shfl_xor_sync, and no
// block barrier separates the gates of the run (each warp owns its rows).
// Each lane computes only its own member's outputs; every product that the
// other member's output needs is computed by the lane that owns its operand
// and passed across, so a pair costs the same FP64 instructions as in shared
// memory and each result is formed by the same operations in the same order
// (bit-identical to the shared-memory ops).  Eligible (chosen on the host):
// X and Y with any controls, uncontrolled H / RX / RY and the fast-mode lazy
// ops (with their phase entry), phase ops over the whole tile, and diagonal
// gates whose every amplitude is touched (Z with any controls).
__device__ __forceinline__ double shfl_x(double v, uint32_t m) { return __shfl_xor_sync(0xffffffffu, v, m); }

__device__ __forceinline__ uint32_t phase_index(const TileGate& g, uint64_t base, uint32_t e) {
  uint32_t idx = 0;
  for (int j = 0; j < g.pm; ++j)
    idx |= (uint32_t)((__popcll(base & g.pmask[j]) ^ __popc(e & g.pemask[j])) & 1) << j;
  return idx;
}

// Lazy op of a run: the descriptor's phase masks are read once per row group
// into registers (PM of them; the table index of an amplitude is the tile's
// parities xor the local ones).
template <int R, int PM>
__device__ __forceinline__ void run_lazy(const TileGate& g, const double2* __restrict__ tables, uint64_t base,
                                         uint32_t lane, const uint32_t* e, double* xr, double* xi) {
  const uint32_t tb = g.tbit;
  const bool hi = (lane & tb) != 0;
  const int kind = g.kind;
  const double t = g.c.cs;
  const double2* tab = tables + g.ptab;
  uint32_t em[PM > 0 ? PM : 1];
  uint32_t bidx = 0;
#pragma unroll
  for (int j = 0; j < PM; ++j) {
    if (j < g.pm) {
      bidx |= (uint32_t)(__popcll(base & g.pmask[j]) & 1) << j;
      em[j] = g.pemask[j];
    } else {
      em[j] = 0;
    }
  }
#pragma unroll
  for (int u = 0; u < R; ++u) {
    double pr = shfl_x(xr[u], tb), pi = shfl_x(xi[u], tb);
    if constexpr (PM > 0) {  // s1 x w: the s1 lane forms the real part, the s0 lane the imaginary part
      uint32_t idx = bidx;
#pragma unroll
      for (int j = 0; j < PM; ++j) idx ^= (uint32_t)(__popc(e[u] & em[j]) & 1) << j;
      const double2 w = __ldg(tab + idx);
      const double r = hi ? xr[u] : pr, i = hi ? xi[u] : pi;
      const double v = dfma(r, hi ? w.x : w.y, dmul(hi ? dneg(i) : i, hi ? w.y : w.x));
      const double vp = shfl_x(v, tb);
      if (hi) {
        xr[u] = v; xi[u] = vp;
      } else {
        pr = vp; pi = v;
      }
    }
    const double a = xr[u], b = xi[u];
    switch (kind) {
      case FK_LAZY_H: {  // s0 + s1, s0 - s1
        const double sg = hi ? -1.0 : 1.0;
        xr[u] = dfma(sg, a, pr); xi[u] = dfma(sg, b, pi);
        break;
      }
      case FK_LAZY_RX_A:  // s0 - i t s1, -i t s0 + s1
        xr[u] = dfma(t, pi, a); xi[u] = dfma(dneg(t), pr, b);
        break;
      case FK_LAZY_RX_B:  // u s0 - i s1, -i s0 + u s1
        xr[u] = dfma(t, a, pi); xi[u] = dfma(t, b, dneg(pr));
        break;
      case FK_LAZY_RY_A: {  // s0 - t s1, t s0 + s1
        const double ts = hi ? t : dneg(t);
        xr[u] = dfma(ts, pr, a); xi[u] = dfma(ts, pi, b);
        break;
      }
      default:  // FK_LAZY_RY_B: u s0 - s1, s0 + u s1
        xr[u] = dfma(t, a, hi ? pr : dneg(pr)); xi[u] = dfma(t, b, hi ? pi : dneg(pi));
    }
  }
}

template <int R>
__device__ __forceinline__ void run_pair(const TileGate& g, const double2* __restrict__ tables, uint64_t base,
                                         uint32_t lane, const uint32_t* e, double* xr, double* xi) {
  const uint32_t tb = g.tbit;
  const bool hi = (lane & tb) != 0;
  const int kind = g.kind;
  if (kind == SPZ_GATE_X || kind == SPZ_GATE_Y) {
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const double pr = shfl_x(xr[u], tb), pi = shfl_x(xi[u], tb);
      if (((e[u] & ~tb) & g.e_mask) == g.l_ones) {
        if (kind == SPZ_GATE_X) {
          xr[u] = pr; xi[u] = pi;
        } else {  // (a, b, c, d) -> (d, -c, -b, a)
          xr[u] = hi ? dneg(pi) : pi;
          xi[u] = hi ? pr : dneg(pr);
        }
      }
    }
  } else if (kind == SPZ_GATE_H) {  // a' = a1 + c1, c' = a1 - c1 with x1 = x / sqrt 2
    const double sg = hi ? -1.0 : 1.0;
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const double orr = dmul(kSqrtOneHalf, xr[u]), oi = dmul(kSqrtOneHalf, xi[u]);
      const double qr = shfl_x(orr, tb), qi = shfl_x(oi, tb);
      xr[u] = dfma(sg, orr, qr);
      xi[u] = dfma(sg, oi, qi);
    }
  } else if (kind == SPZ_GATE_RY) {  // a' = a cos - c sin, c' = a sin + c cos
    const double sg = hi ? 1.0 : -1.0, cs = g.c.cs, sn = g.c.sn;
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const double pr = dmul(xr[u], cs), pi = dmul(xi[u], cs);
      const double qr = shfl_x(dmul(xr[u], sn), tb), qi = shfl_x(dmul(xi[u], sn), tb);
      xr[u] = dfma(sg, qr, pr);
      xi[u] = dfma(sg, qi, pi);
    }
  } else if (kind == SPZ_GATE_RX) {
    // a' = a cos - d nsn, b' = b cos + c nsn, c' = b sn + c cos, d' = d cos + a nsn
    const double sg = hi ? 1.0 : -1.0, cs = g.c.cs, nsn = g.c.nsn, sx = hi ? g.c.nsn : g.c.sn;
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const double pr = dmul(xr[u], cs), pi = dmul(xi[u], cs);
      const double sp = shfl_x(dmul(xi[u], sx), tb), tp = shfl_x(dmul(xr[u], nsn), tb);
      xr[u] = dfma(sg, sp, pr);
      xi[u] = dfma(1.0, pi, tp);
    }
  } else {  // fast-mode lazy ops, s1 first multiplied by its phase entry when the op carries one
    switch (g.pm) {
      case 0: run_lazy<R, 0>(g, tables, base, lane, e, xr, xi); break;
      case 1: run_lazy<R, 1>(g, tables, base, lane, e, xr, xi); break;
      case 2: run_lazy<R, 2>(g, tables, base, lane, e, xr, xi); break;
      case 3: run_lazy<R, 3>(g, tables, base, lane, e, xr, xi); break;
      case 4: run_lazy<R, 4>(g, tables, base, lane, e, xr, xi); break;
      default: run_lazy<R, kPhaseMaxTerms>(g, tables, base, lane, e, xr, xi); break;
    }
  }
}

template <int R>
__device__ __forceinline__ void run_elementwise(const TileGate& g, const double2* __restrict__ tables, uint64_t base,
                                                const uint32_t* e, double* xr, double* xi) {
  if (g.mode == TM_PHASE) {  // the whole tile (a local half bit is never in a run)
    const double2* tab = tables + g.ptab;
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const double2 w = __ldg(tab + phase_index(g, base, e[u]));
      const double r = xr[u], i = xi[u];
      xr[u] = dfma(r, w.x, dmul(dneg(i), w.y));
      xi[u] = dfma(r, w.y, dmul(i, w.x));
    }
    return;
  }
  int gone = -1;
  if (g.mode == TM_DIAG_GLOBAL) {
    gone = (base & g.g_tbit) ? 1 : 0;
    if (!gone && g.kind != SPZ_GATE_RZ) return;  // Z / P act on the 1 half only
  }
#pragma unroll
  for (int u = 0; u < R; ++u) {
    if ((e[u] & g.e_mask) != g.l_ones) continue;
    const bool one = gone >= 0 ? gone != 0 : (e[u] & g.tbit) != 0;
    switch (g.kind) {
      case SPZ_GATE_Z: gate_diag<SPZ_GATE_Z>(g.c, one, xr[u], xi[u]); break;
      case SPZ_GATE_P: gate_diag<SPZ_GATE_P>(g.c, one, xr[u], xi[u]); break;
      default: gate_diag<SPZ_GATE_RZ>(g.c, one, xr[u], xi[u]); break;
    }
  }
}

// Gates g0 .. g1 - 1 of the pass as one run; rows of 32 amplitudes, R per
// warp at a time.  Requires 2^k >= 32 R and whole warps.
constexpr int kRunRows = 4;

__device__ void tile_run_shfl(const PassArgs& A, uint64_t base, double* sre, double* sim, uint32_t T, int g0,
                              int g1) {
  constexpr int R = kRunRows;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const uint32_t rows = T >> 5;
  for (uint32_t r0 = warp * R; r0 < rows; r0 += nwarps * R) {
    uint32_t e[R];
    double xr[R], xi[R];
#pragma unroll
    for (int u = 0; u < R; ++u) {
      e[u] = ((r0 + u) << 5) | lane;
      xr[u] = sre[TileSwizzle::at(e[u])];
      xi[u] = sim[TileSwizzle::at(e[u])];
    }
    for (int gi = g0; gi < g1; ++gi) {
      const TileGate& g = A.gates[gi];
      if ((base & g.g_ones) != g.g_ones || (base & g.g_zeros) != 0) continue;
      if (g.cond >= 0 && A.outcomes[g.cond] == 0) continue;
      if (g.mode == TM_PAIR) run_pair<R>(g, A.tables, base, lane, e, xr, xi);
      else run_elementwise<R>(g, A.tables, base, e, xr, xi);
    }
#pragma unroll
    for (int u = 0; u < R; ++u) {
      sre[TileSwizzle::at(e[u])] = xr[u];
      sim[TileSwizzle::at(e[u])] = xi[u];
    }
  }
}

// Every gate of the pass on one tile held in shared memory (sre, sim), in
// pass order, with a block barrier after each (with SHFL, after each run of
// warp-shuffle gates; without, runs are ignored and every gate is applied in
// shared memory).
template <bool SHFL>
__device__ __forceinline__ void tile_pass_gates(const PassArgs& A, uint64_t base, double* sre, double* sim,
                                                uint32_t T) {
  for (int gi = 0; gi < A.ngates; ++gi) {
    const TileGate& g = A.gates[gi];
    if constexpr (SHFL) {
      if (g.run_end > gi) {
        tile_run_shfl(A, base, sre, sim, T, gi, g.run_end);
        gi = g.run_end - 1;
        __syncthreads();
        continue;
      }
    }
    if ((base & g.g_ones) != g.g_ones || (base & g.g_zeros) != 0) continue;  // uniform per tile
    if (g.cond >= 0 && A.outcomes[g.cond] == 0) continue;                   // classical condition
    const uint32_t nw = T >> g.npos;
    switch (g.mode) {
      case TM_PAIR:
        switch (g.kind) {
          case SPZ_GATE_H: tile_pair_any<SPZ_GATE_H, TileGate, TileSwizzle>(g, sre, sim, nw); break;
          case SPZ_GATE_X: tile_pair_any<SPZ_GATE_X, TileGate, TileSwizzle>(g, sre, sim, nw); break;
          case SPZ_GATE_Y: tile_pair_any<SPZ_GATE_Y, TileGate, TileSwizzle>(g, sre, sim, nw); break;
          case SPZ_GATE_RX: tile_pair_any<SPZ_GATE_RX, TileGate, TileSwizzle>(g, sre, sim, nw); break;
          case SPZ_GATE_RY: tile_pair_any<SPZ_GATE_RY, TileGate, TileSwizzle>(g, sre, sim, nw); break;
#define SPZ_LAZY(FK)                                                            \
  case FK:                                                                      \
    if (g.pm) tile_fast_phase_pm<FK>(g, A.tables + g.ptab, base, sre, sim, nw); \
    else tile_pair<FK, 1, TileGate, TileSwizzle>(g, sre, sim, nw);              \
    break;
          SPZ_LAZY(FK_LAZY_H)
          SPZ_LAZY(FK_LAZY_RX_A)
          SPZ_LAZY(FK_LAZY_RX_B)
          SPZ_LAZY(FK_LAZY_RY_A)
          SPZ_LAZY(FK_LAZY_RY_B)
#undef SPZ_LAZY
          default: tile_pair_any<SPZ_GATE_U, TileGate, TileSwizzle>(g, sre, sim, nw); break;
        }
        break;
      case TM_PHASE:
        if (g.npos) tile_phase_pm<1>(g, A.tables + g.ptab, base, sre, sim, nw);
        else tile_phase_pm<0>(g, A.tables + g.ptab, base, sre, sim, nw);
        break;
      case TM_LAZY2:
        tile_lazy2_pm(g, A.tables + g.ptab, base, sre, sim, nw);
        break;
      case TM_DIAG_LOCAL:
      case TM_DIAG_GLOBAL: {
        int gone = -1;
        if (g.mode == TM_DIAG_GLOBAL) {
          gone = (base & g.g_tbit) ? 1 : 0;
          if (!gone && g.kind != SPZ_GATE_RZ) break;  // Z / P act on the 1 half only
        }
        switch (g.kind) {
          case SPZ_GATE_Z: tile_diag_any<SPZ_GATE_Z, TileGate, TileSwizzle>(g, sre, sim, nw, gone); break;
          case SPZ_GATE_P: tile_diag_any<SPZ_GATE_P, TileGate, TileSwizzle>(g, sre, sim, nw, gone); break;
          default: tile_diag_any<SPZ_GATE_RZ, TileGate, TileSwizzle>(g, sre, sim, nw, gone); break;
        }
        break;
      }
      default:  // TM_SWAP
        tile_swap_any<TileGate, TileSwizzle>(g, sre, sim, nw);
    }
    __syncthreads();
  }
}

template <bool SHFL>
__global__ void __launch_bounds__(kTileThreads, SHFL ? 12 : SPZ_TILE_MIN_BLOCKS) tile_kernel(PassArgs A) {
  extern __shared__ double smem[];
  const int K = A.k;
  const uint32_t T = 1u << K;
  double* sre = smem;
  double* sim = smem + T;
  // Row offsets >> c (their bits are local qubits >= c, so 32 bits hold them
  // for up to 34 qubits): half the shared memory of 64-bit entries, which
  // lets a 13th block of 2^10-amplitude tiles onto an SM.
  uint32_t* rowoff = reinterpret_cast<uint32_t*>(smem + 2 * T);
  const uint32_t nrows = 1u << A.nhigh;
  const uint32_t cmask = (1u << A.c) - 1;
  // Row offsets: scatter of the high local bits, the same for every tile.
  // (The run-time index into A.lpos here and in deposit() keeps the parameter
  // block in local memory.  Reading lpos at constant indices instead
  // (deposit_param) removes it but measured 1.9% slower on the 30-qubit
  // brickwork, in fast mode, and no faster in the exact mode; the adjoint
  // kernel, where it measured 1.3% faster, uses that form.)
  for (uint32_t r = threadIdx.x; r < nrows; r += blockDim.x) {
    uint64_t off = 0;
    for (int j = 0; j < A.nhigh; ++j)
      if ((r >> j) & 1) off |= 1ull << A.lpos[A.c + j];
    rowoff[r] = (uint32_t)(off >> A.c);
  }
  __syncthreads();
  for (uint64_t t = A.tile_begin + blockIdx.x; t < A.ntiles; t += gridDim.x) {
    const uint64_t base = deposit(slab_tile(A, t), A.lpos, K);
    // load (pairs of consecutive amplitudes: c >= 1)
    for (uint32_t e2 = threadIdx.x; e2 < T / 2; e2 += blockDim.x) {
      const uint32_t e = 2 * e2;
      const uint64_t gi = base | ((uint64_t)rowoff[e >> A.c] << A.c) | (e & cmask);
      double2 r = *reinterpret_cast<const double2*>(A.re + gi);
      double2 m = *reinterpret_cast<const double2*>(A.im + gi);
      // e even: e and e + 1 share a 16-byte slot, in reverse order when the
      // swizzle flips the low bits.
      const uint32_t p = TileSwizzle::at(e) & ~1u;
      if (p != e) {
        r = make_double2(r.y, r.x);
        m = make_double2(m.y, m.x);
      }
      *reinterpret_cast<double2*>(sre + p) = r;
      *reinterpret_cast<double2*>(sim + p) = m;
    }
    __syncthreads();
    tile_pass_gates<SHFL>(A, base, sre, sim, T);
    // store
    for (uint32_t e2 = threadIdx.x; e2 < T / 2; e2 += blockDim.x) {
      const uint32_t e = 2 * e2;
      const uint64_t gi = base | ((uint64_t)rowoff[e >> A.c] << A.c) | (e & cmask);
      const uint32_t p = TileSwizzle::at(e) & ~1u;
      double2 r = *reinterpret_cast<const double2*>(sre + p);
      double2 m = *reinterpret_cast<const double2*>(sim + p);
      if (p != e) {
        r = make_double2(r.y, r.x);
        m = make_double2(m.y, m.x);
      }
      *reinterpret_cast<double2*>(A.re + gi) = r;
      *reinterpret_cast<double2*>(A.im + gi) = m;
    }
    __syncthreads();
  }
}


// ------------------------------------------------------------ TMA staging
// The same pass with each tile fetched by the Tensor Memory Accelerator: the
// state is viewed as 2^(n-3) rows of 8 doubles (one 64-byte row per value of
// the three low qubits, which every pass keeps local), and a tile's 2^(k-3)
// rows, at scattered row indices, arrive by cp.async.bulk.tensor gathers of
// four rows each (tile::gather4), issued by the first warp and counted on an
// mbarrier.  PREFETCH keeps two tile buffers and fetches the next tile while
// the current one computes.  Compute and store are the thread-load kernel's,
// so the results are identical.  Waits are bounded: past the limit the block
// records the timeout in *err, waits (bounded) for its copies in flight and
// returns; the call then reports SPZ_ERR_TIMEOUT.
#ifndef SPZ_TMA_WAIT_POLLS
#define SPZ_TMA_WAIT_POLLS (1u << 24)
#endif

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n"
      "  .reg .pred p;\n"
      "  mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n"
      "  selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < SPZ_TMA_WAIT_POLLS; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Four 64-byte rows (row indices r0..r3 of the 8-column view) into 256
// contiguous bytes of shared memory; completion counted on `bar`.
__device__ __forceinline__ void tma_gather4(double* dst, const CUtensorMap* map, int r0, int r1, int r2, int r3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(smem_u32(bar))
      : "memory");
}

template <bool PREFETCH>
__global__ void __launch_bounds__(kTileThreads) tile_kernel_tma(PassArgs A, const __grid_constant__ CUtensorMap map_re,
                                                                const __grid_constant__ CUtensorMap map_im, int* err) {
  extern __shared__ double smem_raw[];
  __shared__ __align__(8) uint64_t bars[2];
  const int K = A.k;
  const uint32_t T = 1u << K;
  const uint32_t nrows = T >> kTileLowBits;
  // tile buffers at a 128-byte boundary (the gathers' destinations)
  double* bufs = reinterpret_cast<double*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
  constexpr int kBufs = PREFETCH ? 2 : 1;
  uint64_t* rowoff = reinterpret_cast<uint64_t*>(bufs + 2 * kBufs * T);
  for (uint32_t r = threadIdx.x; r < nrows; r += blockDim.x) {
    uint64_t off = 0;
    for (int j = 0; j < A.nhigh; ++j)
      if ((r >> j) & 1) off |= 1ull << A.lpos[kTileLowBits + j];
    rowoff[r] = off;
  }
  if (threadIdx.x == 0) {
    for (int b = 0; b < kBufs; ++b) mbar_init(&bars[b], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u;
  const bool issuer = threadIdx.x < 32;
  auto issue = [&](uint64_t tile, int b) {  // the first warp; after the buffer's last generic access
    if (!issuer) return;
    const uint64_t base = deposit(tile, A.lpos, K);
    if (lane == 0) mbar_arrive_expect_tx(&bars[b], 2u * T * (uint32_t)sizeof(double));
    __syncwarp();
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    double* dre = bufs + (size_t)b * 2 * T;
    double* dim = dre + T;
    for (uint32_t j = lane; j < nrows / 4; j += 32) {
      const int r0 = (int)((base | rowoff[4 * j + 0]) >> kTileLowBits);
      const int r1 = (int)((base | rowoff[4 * j + 1]) >> kTileLowBits);
      const int r2 = (int)((base | rowoff[4 * j + 2]) >> kTileLowBits);
      const int r3 = (int)((base | rowoff[4 * j + 3]) >> kTileLowBits);
      tma_gather4(dre + 32 * j, &map_re, r0, r1, r2, r3, &bars[b]);
      tma_gather4(dim + 32 * j, &map_im, r0, r1, r2, r3, &bars[b]);
    }
  };
  uint32_t parity[2] = {0u, 0u};
  uint64_t tile = A.tile_begin + blockIdx.x;
  if (tile < A.ntiles) issue(tile, 0);
  int b = 0;
  for (; tile < A.ntiles; tile += gridDim.x) {
    const uint64_t next = tile + gridDim.x;
    bool pending_next = false;
    if (PREFETCH && next < A.ntiles) {
      issue(next, b ^ 1);
      pending_next = true;
    }
    const bool ok = mbar_wait_bounded(&bars[b], parity[b]);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicExch(err, 1);
        mbar_wait_bounded(&bars[b], parity[b]);
        if (pending_next) mbar_wait_bounded(&bars[b ^ 1], parity[b ^ 1]);
      }
      __syncthreads();
      return;
    }
    parity[b] ^= 1u;
    double* sre = bufs + (size_t)b * 2 * T;
    double* sim = sre + T;
    const uint64_t base = deposit(tile, A.lpos, K);
    tile_pass_gates<false>(A, base, sre, sim, T);
    for (uint32_t e2 = threadIdx.x; e2 < T / 2; e2 += blockDim.x) {  // store, as the thread-load kernel
      const uint32_t e = 2 * e2;
      const uint64_t gi = base | rowoff[e >> kTileLowBits] | (e & ((1u << kTileLowBits) - 1));
      *reinterpret_cast<double2*>(A.re + gi) = *reinterpret_cast<const double2*>(sre + e);
      *reinterpret_cast<double2*>(A.im + gi) = *reinterpret_cast<const double2*>(sim + e);
    }
    __syncthreads();
    if (!PREFETCH && next < A.ntiles) issue(next, 0);
    if (PREFETCH) b ^= 1;
  }
}

// ------------------------------------------------------------ planner
namespace {

// Exact-commutation classes.  Two gates that commute mathematically (disjoint
// non-diagonal qubits) also commute bit for bit when one of them only moves or
// negates amplitudes (X, Z, SWAP: rounding is sign-symmetric), or when one is
// Y (moves and multiplies by +-i) and the other's arithmetic treats real and
// imaginary parts alike (H, RX, RY, and the moves).  P, RZ and U use FMAs whose
// rounding differs between the real and imaginary parts, so G(i z) != i G(z)
// in the last bit; two arithmetic gates never swap.
enum ExactClass { EC_PERM = 0, EC_Y = 1, EC_ICOV = 2, EC_FMA = 3 };

inline int exact_class(int kind) {
  switch (kind) {
    case SPZ_GATE_X:
    case SPZ_GATE_Z:
    case SPZ_GATE_SWAP: return EC_PERM;
    case SPZ_GATE_Y: return EC_Y;
    case SPZ_GATE_H:
    case SPZ_GATE_RX:
    case SPZ_GATE_RY: return EC_ICOV;
    default: return EC_FMA;  // P, RZ, U
  }
}

// Qubits a gate acts on non-diagonally (targets of pair gates, SWAP qubits)
// and diagonally only (controls, and all qubits of diagonal gates).
inline uint64_t nd_mask(const GateApp& g) {
  if (g.kind == SPZ_GATE_SWAP) return (1ull << g.target) | (1ull << g.target2);
  if (is_diagonal(g.kind) || g.kind == FK_PHASE) return 0;
  return 1ull << g.target;
}
inline uint64_t d_mask(const GateApp& g) {
  uint64_t m = g.ones | g.zeros | g.touch;
  if (is_diagonal(g.kind)) m |= 1ull << g.target;
  return m;
}

// Greedy planner: see the file comment.  `k` local qubits per pass, the low
// `c` qubits always local.  With exact = false (fast mode) any two gates that
// commute mathematically may be swapped.
std::vector<PlannedPass> plan(const std::vector<GateApp>& gates, uint32_t n, int k, int c, bool exact = true) {
  std::vector<PlannedPass> passes;
  std::vector<GateApp> remaining = gates;
  const uint64_t low = c >= 64 ? ~0ull : ((1ull << c) - 1);
  while (!remaining.empty()) {
    PlannedPass P;
    uint64_t L = low;
    int nl = __builtin_popcountll(L);
    std::vector<GateApp> deferred;
    uint64_t def_nd = 0, def_d = 0;
    bool def_y = false, def_icov = false, def_fma = false;  // classes present among deferred gates
    const size_t lookahead = 4096;
    size_t i = 0;
    for (; i < remaining.size(); ++i) {
      const GateApp& g = remaining[i];
      if (deferred.size() > lookahead) break;
      const uint64_t nd = nd_mask(g), d = d_mask(g);
      const bool commutes = (nd & (def_nd | def_d)) == 0 && (d & def_nd) == 0;
      const int ec = exact_class(g.kind);
      const bool exact_ok = !exact || ec == EC_PERM || (ec == EC_Y && !def_fma) ||
                            (ec == EC_ICOV && !def_icov && !def_fma) ||
                            (ec == EC_FMA && !def_icov && !def_fma && !def_y);
      bool take = false;
      if (deferred.empty() || (commutes && exact_ok)) {
        const uint64_t need = nd & ~L;
        const int add = __builtin_popcountll(need);
        if (nl + add <= k) {
          L |= need;
          nl += add;
          take = true;
        }
      }
      if (take) {
        P.gates.push_back(g);
      } else {
        deferred.push_back(g);
        def_nd |= nd;
        def_d |= d;
        def_y |= ec == EC_Y;
        def_icov |= ec == EC_ICOV;
        def_fma |= ec == EC_FMA;
      }
    }
    for (; i < remaining.size(); ++i) deferred.push_back(remaining[i]);
    if (P.gates.empty()) {  // cannot happen for k >= c + 2; keep progress regardless
      P.gates.push_back(deferred.front());
      deferred.erase(deferred.begin());
      L |= nd_mask(P.gates[0]);
    }
    for (int q = 0; q < (int)n; ++q)
      if ((L >> q) & 1) P.local.push_back(q);
    passes.push_back(std::move(P));
    remaining.swap(deferred);
  }
  return passes;
}

// Build the device description of a gate inside a pass with local qubits `L`.
TileGate tile_gate(const GateApp& g, const std::vector<int>& local, const std::vector<PhaseTable>* tables = nullptr,
                   const std::vector<uint32_t>* table_offsets = nullptr) {
  int where[64];
  for (int q = 0; q < 64; ++q) where[q] = -1;
  for (size_t j = 0; j < local.size(); ++j) where[local[j]] = (int)j;
  TileGate t{};
  t.kind = g.kind;
  t.c = g.c;
  t.cond = g.cond;
  if (g.kind == FK_PHASE) {  // elementwise; any qubits (the global index is formed per amplitude)
    const PhaseTable& tab = (*tables)[g.table];
    t.mode = TM_PHASE;
    t.half_bit = tab.half_bit;
    t.pm = tab.m;
    for (int j = 0; j < tab.m; ++j) {
      t.pmask[j] = tab.mask[j];
      for (int q = 0; q < 64; ++q)
        if (((tab.mask[j] >> q) & 1) && where[q] >= 0) t.pemask[j] |= 1u << where[q];
    }
    t.ptab = (*table_offsets)[g.table];
    if (tab.half_bit) {
      // Only the half with the bit set is touched: a local bit is inserted into
      // the enumeration (every lane busy); a non-local one is a tile predicate.
      const int q = __builtin_ctzll(tab.half_bit);
      if (where[q] >= 0) {
        t.tbit = 1u << where[q];
        t.l_ones = t.tbit;
        t.pos[0] = (uint8_t)where[q];
        t.npos = 1;
      } else {
        t.g_ones = tab.half_bit;
      }
    }
    t.e_mask = t.l_ones;
    return t;
  }
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
    t.mode = TM_SWAP;
    t.tbit = 1u << where[g.target];
    t.tbit2 = 1u << where[g.target2];
    special |= t.tbit | t.tbit2;
    t.l_ones = l_ones;
  } else if (is_diagonal(g.kind)) {
    if (where[g.target] >= 0) {
      t.mode = TM_DIAG_LOCAL;
      t.tbit = 1u << where[g.target];
      if (g.kind != SPZ_GATE_RZ) {  // Z and P touch the target-1 half only
        special |= t.tbit;
        l_ones |= t.tbit;
      }
    } else {
      t.mode = TM_DIAG_GLOBAL;
      t.g_tbit = 1ull << g.target;
    }
    t.l_ones = l_ones;
  } else {
    t.mode = TM_PAIR;
    t.tbit = 1u << where[g.target];
    special |= t.tbit;
    t.l_ones = l_ones;
    if (g.kind >= FK_LAZY_H && g.table >= 0) {  // lazy op that first multiplies s1 by a phase entry
      const PhaseTable& tab = (*tables)[g.table];
      t.pm = tab.m;
      for (int j = 0; j < tab.m; ++j) {
        t.pmask[j] = tab.mask[j];
        for (int q = 0; q < 64; ++q)
          if (((tab.mask[j] >> q) & 1) && where[q] >= 0) t.pemask[j] |= 1u << where[q];
      }
      t.ptab = (*table_offsets)[g.table];
    }
  }
  t.npos = 0;
  for (int j = 0; j < 32; ++j)
    if ((special >> j) & 1) t.pos[t.npos++] = (uint8_t)j;
  t.e_mask = special;
  return t;
}


}  // namespace

TileGate make_tile_gate(const GateApp& g, const std::vector<int>& local) { return tile_gate(g, local); }

namespace {

// Gates that tile_run_shfl applies: pairs inside a row of 32 amplitudes whose
// per-lane split costs no extra FP64 work, and elementwise ops that touch
// every amplitude of the tile (Z, with no FP64 work, under any controls).
bool shfl_eligible(const TileGate& t) {
  switch (t.mode) {
    case TM_PAIR:
      if (t.tbit >= 32u) return false;
      if (t.kind == SPZ_GATE_X || t.kind == SPZ_GATE_Y) return true;
      if (t.kind == SPZ_GATE_H || t.kind == SPZ_GATE_RX || t.kind == SPZ_GATE_RY ||
          (t.kind >= FK_LAZY_H && t.kind <= FK_LAZY_RY_B))
        return t.e_mask == t.tbit;  // uncontrolled within the tile
      return false;
    case TM_PHASE:
      return t.npos == 0;
    case TM_DIAG_LOCAL:
    case TM_DIAG_GLOBAL:
      return t.kind == SPZ_GATE_Z || t.e_mask == 0;
    default:
      return false;
  }
}

// A run shorter than this gains nothing over the shared-memory ops (its rows
// are loaded and stored once either way).
constexpr int kMinShuffleRun = 2;

// SPZ_EXEC_SHUFFLE: mark the runs in one tile pass's descriptors g[0 .. count)
// (a pass of k local qubits: rows of 32 amplitudes, kRunRows per warp).
// Returns the number of gates in runs.
size_t mark_shuffle_runs(TileGate* g, size_t count, int k) {
  if ((1u << k) < 32u * kRunRows) return 0;
  size_t in_runs = 0;
  for (size_t i = 0; i < count;) {
    if (!shfl_eligible(g[i])) {
      ++i;
      continue;
    }
    size_t j = i + 1;
    while (j < count && shfl_eligible(g[j])) ++j;
    if (j - i >= (size_t)kMinShuffleRun) {
      g[i].run_end = (int32_t)j;
      in_runs += j - i;
    }
    i = j;
  }
  return in_runs;
}

// Fast mode: fuse consecutive lazy rotations on two distinct tile qubits,
// both carrying a phase entry, into one TM_LAZY2 op, when the second op's
// phase masks do not contain the first op's qubit (its phase then commutes
// with the first rotation) and the two tables have at most kPhaseMaxTerms
// masks between them.  pg[i] is the descriptor of gates[i]; the joint tables
// are appended to `flat` (re, im pairs).  Returns the FP64 instructions
// saved: 4 per block of four amplitudes, 2^n per fused pair.  SPZ_FAST_PAIRS=0
// in the environment turns the fusion off (for A/B measurements).
bool fast_pairs_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("SPZ_FAST_PAIRS");
    return !(v && v[0] == '0');
  }();
  return on;
}

bool lazy_with_table(const GateApp& g) {
  return g.kind >= FK_LAZY_H && g.kind <= FK_LAZY_RY_B && g.table >= 0 && g.cond < 0 && g.ones == 0 &&
         g.zeros == 0;
}

uint64_t fuse_lazy_pairs(std::vector<TileGate>& pg, const std::vector<GateApp>& gates,
                         const std::vector<PhaseTable>& tables, std::vector<double>* flat, uint32_t n) {
  if (!fast_pairs_enabled()) return 0;
  std::vector<TileGate> out;
  uint64_t saved = 0;
  size_t i = 0;
  while (i < pg.size()) {
    if (i + 1 < pg.size() && lazy_with_table(gates[i]) && lazy_with_table(gates[i + 1]) &&
        gates[i].target != gates[i + 1].target && pg[i].mode == TM_PAIR && pg[i + 1].mode == TM_PAIR) {
      const PhaseTable& T1 = tables[gates[i].table];
      const PhaseTable& T2 = tables[gates[i + 1].table];
      const uint64_t q1b = 1ull << gates[i].target, q2b = 1ull << gates[i + 1].target;
      bool ok = T1.m + T2.m <= kPhaseMaxTerms;
      for (int j = 0; ok && j < T2.m; ++j) ok = (T2.mask[j] & q1b) == 0;
      if (ok) {
        TileGate t = pg[i];
        const TileGate& u = pg[i + 1];
        t.mode = TM_LAZY2;
        t.kind2 = u.kind;
        t.tbit2 = u.tbit;
        t.c.sn = u.c.cs;
        const int p1 = __builtin_ctz(t.tbit), p2 = __builtin_ctz(u.tbit);
        t.npos = 2;
        t.pos[0] = (uint8_t)std::min(p1, p2);
        t.pos[1] = (uint8_t)std::max(p1, p2);
        t.l_ones = 0;
        t.e_mask = t.tbit | u.tbit;
        t.pm1 = T1.m;
        t.pm = T1.m + T2.m;
        for (int j = 0; j < T2.m; ++j) {
          t.pmask[T1.m + j] = u.pmask[j];
          t.pemask[T1.m + j] = u.pemask[j];
        }
        uint32_t flip = 0;
        for (int j = 0; j < T1.m; ++j)
          if (T1.mask[j] & q2b) flip |= 1u << j;
        t.ptab = (uint32_t)(flat->size() / 2);
        const uint32_t E = 1u << t.pm;
        for (uint32_t idx = 0; idx < E; ++idx) {
          const uint32_t i1 = idx & ((1u << T1.m) - 1), i2 = idx >> T1.m;
          const std::complex<double> w1(T1.re[i1], T1.im[i1]), w2(T2.re[i2], T2.im[i2]);
          const std::complex<double> w3 = std::complex<double>(T1.re[i1 ^ flip], T1.im[i1 ^ flip]) * w2;
          for (const std::complex<double>& w : {w1, w2, w3}) {
            flat->push_back(w.real());
            flat->push_back(w.imag());
          }
        }
        out.push_back(t);
        saved += 1ull << n;
        i += 2;
        continue;
      }
    }
    out.push_back(pg[i]);
    ++i;
  }
  pg.swap(out);
  return saved;
}

}  // namespace

namespace {

// Optional per-pass device timing (SPZ_EXEC_TIME_PASSES): an event pair around
// every launch on the handle's stream, summed after one synchronisation.
struct PassTimer {
  bool on = false;
  cudaStream_t stream = nullptr;
  std::vector<cudaEvent_t> ev;
  std::vector<bool> tile;
  int begin() {
    if (!on) return SPZ_OK;
    cudaEvent_t a, b;
    SPZ_CUDA(cudaEventCreate(&a));
    SPZ_CUDA(cudaEventCreate(&b));
    ev.push_back(a);
    ev.push_back(b);
    SPZ_CUDA(cudaEventRecord(a, stream));
    return SPZ_OK;
  }
  int end(bool is_tile) {
    if (!on) return SPZ_OK;
    SPZ_CUDA(cudaEventRecord(ev.back(), stream));
    tile.push_back(is_tile);
    return SPZ_OK;
  }
  int collect(spz_exec_stats* st) {
    if (!on) return SPZ_OK;
    int rc = SPZ_OK;
    cudaError_t e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "pass timing synchronisation");
    for (size_t i = 0; i + 1 < ev.size(); i += 2) {
      float ms = 0.f;
      if (rc == SPZ_OK && i / 2 < tile.size() && cudaEventElapsedTime(&ms, ev[i], ev[i + 1]) == cudaSuccess && st)
        (tile[i / 2] ? st->tile_ms : st->plain_ms) += ms;
      cudaEventDestroy(ev[i]);
      cudaEventDestroy(ev[i + 1]);
    }
    ev.clear();
    tile.clear();
    return rc;
  }
};

}  // namespace

// A tile pass whose gates touch fewer than k qubits gets the lowest untouched
// qubits as extra local qubits: its tiles then hold 2^k amplitudes, so every
// thread of a block has pairs to work on (a pass on 5 qubits would otherwise
// run 32-amplitude tiles with half of each warp idle in every pair op).  The
// tiling is only a partition of the amplitudes: results are unchanged.
static void pad_tile_passes(std::vector<PlannedPass>& passes, uint32_t n, int k) {
  for (PlannedPass& P : passes) {
    const bool tiled = P.gates.size() > 1 || P.gates[0].kind >= FK_LAZY_H || P.gates[0].cond >= 0;
    if (!tiled || (int)P.local.size() >= k) continue;
    uint64_t L = 0;
    for (int q : P.local) L |= 1ull << q;
    for (int q = 0; q < (int)n && __builtin_popcountll(L) < k; ++q) L |= 1ull << q;
    P.local.clear();
    for (int q = 0; q < (int)n; ++q)
      if ((L >> q) & 1) P.local.push_back(q);
  }
}

std::vector<PlannedPass> plan_passes(const std::vector<GateApp>& gates, uint32_t n, int k, int c, bool exact) {
  return plan(gates, n, k, c, exact);
}

bool exactly_commuting_kinds(int a, int b) {
  const int ea = exact_class(a), eb = exact_class(b);
  return ea == EC_PERM || eb == EC_PERM || (ea == EC_Y && eb != EC_FMA) || (eb == EC_Y && ea != EC_FMA);
}

// Run a list of already validated gate applications on h.
// FP64-pipe instructions of one executed op (lowered fast ops included).
uint64_t op_fp64_ops(uint32_t n, const GateApp& g, const std::vector<PhaseTable>& tables) {
  const uint64_t N = 1ull << n;
  if (g.kind >= FK_LAZY_H && g.kind <= FK_LAZY_RY_B) return (g.table >= 0 ? 8 : 4) * (N / 2);
  if (g.kind == FK_PHASE) return tables[g.table].half_bit ? 4 * (N / 2) : 4 * N;
  return gate_fp64_ops(n, g);
}

// Resident blocks per SM for a tile pass of `threads` x `smem` and the SM
// count; the grid of a tile pass is one wave of them (each block loops over
// tiles), so no block waits for a second wave.  Cached per device and tile
// size (kernel attributes are per device); callers may be on several threads.
int tile_launch_shape(int device, int threads, size_t smem, int* resident_out, int* sms_out, bool shfl) {
  static std::mutex mu;
  static int sms[kMaxDevices] = {};
  // by log2 of the tile, 32 / 64 threads, and the instantiation
  static int resident[kMaxDevices][kTileMaxK + 2][2][2] = {};
  if (device < 0 || device >= kMaxDevices) return fail(SPZ_ERR_INVALID_ARGUMENT, "device index out of range");
  std::lock_guard<std::mutex> lock(mu);
  if (!sms[device]) {
    int count = 0;
    SPZ_CUDA(cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, device));
    const int max_smem = (2 << kTileMaxK) * 8 + (1 << (kTileMaxK - kTileLowBits)) * 8;
    for (const void* fn : {(const void*)tile_kernel<false>, (const void*)tile_kernel<true>}) {
      SPZ_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
      SPZ_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                    cudaSharedmemCarveoutMaxShared));
    }
    sms[device] = count;
  }
  int lg = 0;  // the largest lg with 2 x 8 B x 2^lg <= smem (the tile's re and im)
  while (lg <= kTileMaxK && (16ull << (lg + 1)) <= smem) ++lg;
  int& r = resident[device][lg][threads > 32 ? 1 : 0][shfl ? 1 : 0];
  if (!r) {
    int per_sm = 0;
    const void* fn = shfl ? (const void*)tile_kernel<true> : (const void*)tile_kernel<false>;
    SPZ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
    r = std::max(1, per_sm);
  }
  *resident_out = r;
  *sms_out = sms[device];
  return SPZ_OK;
}

// TMA staging: tensor maps of the handle's arrays, 2^(n-3) rows of 8 doubles
// (64-byte rows, boxes one row high as tile::gather4 requires), built once.
int ensure_tma_maps(spz_state_t h) {
  if (h->tma_ready) return SPZ_OK;
  if (h->n < 5) return fail(SPZ_ERR_UNSUPPORTED, "TMA staging needs at least 5 qubits");
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  static std::mutex mu;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!encode) {
      void* fn = nullptr;
      cudaDriverEntryPointQueryResult q{};
      SPZ_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
      if (q != cudaDriverEntryPointSuccess || !fn) return fail(SPZ_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
  }
  double* arrays[2] = {h->re, h->im};
  for (int a = 0; a < 2; ++a) {
    if (reinterpret_cast<uintptr_t>(arrays[a]) & 15) return fail(SPZ_ERR_UNSUPPORTED, "TMA needs 16-byte aligned arrays");
    alignas(64) CUtensorMap m;
    const cuuint64_t dims[2] = {8, h->N >> 3};
    const cuuint64_t strides[1] = {8 * sizeof(double)};
    const cuuint32_t box[2] = {8, 1};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = encode(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, arrays[a], dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(SPZ_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    static_assert(sizeof(CUtensorMap) == sizeof(h->tma_map[0]), "tensor map size");
    std::memcpy(h->tma_map[a], &m, sizeof(m));
  }
  if (!h->tma_err) SPZ_CUDA(dev_alloc(&h->tma_err, sizeof(int)));
  h->tma_ready = true;
  return SPZ_OK;
}

// Blocks per SM of the TMA-staged kernel (per device and variant).
int tma_launch_shape(int device, bool prefetch, int threads, size_t smem, int* resident_out) {
  static std::mutex mu;
  static int resident[kMaxDevices][2] = {};
  if (device < 0 || device >= kMaxDevices) return fail(SPZ_ERR_INVALID_ARGUMENT, "device index out of range");
  std::lock_guard<std::mutex> lock(mu);
  int& r = resident[device][prefetch];
  if (!r) {
    const void* fn = prefetch ? (const void*)tile_kernel_tma<true> : (const void*)tile_kernel_tma<false>;
    const int max_smem = (prefetch ? 4 : 2) * (8 << kTileMaxK) + (1 << (kTileMaxK - kTileLowBits)) * 8 + 128;
    SPZ_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, max_smem));
    SPZ_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared));
    int per_sm = 0;
    SPZ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
    r = std::max(1, per_sm);
  }
  *resident_out = r;
  return SPZ_OK;
}

// Host arrays that one run of gates uploads from before it and downloads to
// after it, with the copies overlapping the leading and the last tile passes
// where a pass can be cut into kIoChunks slabs: slab j holds the amplitudes whose
// three slab qubits q, q+1, q+2 read j, where those are the pass's three
// highest non-local qubits; the pass's tiles then fall into slabs by
// contiguous ranges of tile index.  In memory a slab is 2^(n-q-3) runs of 2^q
// amplitudes (one run when q = n-3).
constexpr int kIoChunks = 8;
constexpr int kIoMaxRuns = 64;  // copies per slab and array, at most
struct HostIo {
  const double* in_re = nullptr;  // upload before the first pass (nullptr: none)
  const double* in_im = nullptr;
  double* out_re = nullptr;       // download after the last pass (nullptr: none)
  double* out_im = nullptr;
  cudaEvent_t up[kIoChunks] = {};
  cudaEvent_t down[kIoChunks] = {};
};

// The lowest slab qubit q for a pass with these local qubits, or -1 when its
// three highest non-local qubits are not consecutive or a slab would take more
// than kIoMaxRuns copies.
int slab_qubit(uint64_t local_mask, uint32_t n) {
  int top[3], found = 0;
  for (int q = (int)n - 1; q >= 0 && found < 3; --q)
    if (!((local_mask >> q) & 1)) top[found++] = q;
  if (found < 3 || top[1] != top[0] - 1 || top[2] != top[1] - 1) return -1;
  const int q = top[2];
  if ((int)n - q - 3 > 6) return -1;
  return (1 << ((int)n - q - 3)) <= kIoMaxRuns ? q : -1;
}

// Copy slab j (slab qubits q..q+2) of both arrays on the copy stream.  A state
// of fewer than 3 qubits (q < 0) is one slab: slab 0 copies it whole.
int io_copy_slab(spz_state_t h, double* dre, double* dim, const double* sre, const double* sim, int j, int q,
                 cudaMemcpyKind kind) {
  if (q < 0) {
    if (j == 0) {
      SPZ_CUDA(cudaMemcpyAsync(dre, sre, h->N * sizeof(double), kind, h->copy_stream));
      SPZ_CUDA(cudaMemcpyAsync(dim, sim, h->N * sizeof(double), kind, h->copy_stream));
    }
    return SPZ_OK;
  }
  const uint64_t runs = 1ull << (h->n - q - 3), len = 1ull << q;
  if (runs > (uint64_t)kIoMaxRuns) {  // one strided copy per array: rows of 2^q amplitudes, pitch 2^(q+3)
    const size_t width = len * sizeof(double), pitch = width << 3, off = (size_t)j << q;
    SPZ_CUDA(cudaMemcpy2DAsync(dre + off, pitch, sre + off, pitch, width, runs, kind, h->copy_stream));
    SPZ_CUDA(cudaMemcpy2DAsync(dim + off, pitch, sim + off, pitch, width, runs, kind, h->copy_stream));
    return SPZ_OK;
  }
  for (uint64_t r = 0; r < runs; ++r) {
    const uint64_t off = (r << (q + 3)) | ((uint64_t)j << q);
    SPZ_CUDA(cudaMemcpyAsync(dre + off, sre + off, len * sizeof(double), kind, h->copy_stream));
    SPZ_CUDA(cudaMemcpyAsync(dim + off, sim + off, len * sizeof(double), kind, h->copy_stream));
  }
  return SPZ_OK;
}

// Upload slab j on the copy stream; event up[j] marks it done.
int io_upload(spz_state_t h, HostIo* io, int j, int q) {
  int rc = io_copy_slab(h, h->re, h->im, io->in_re, io->in_im, j, q, cudaMemcpyHostToDevice);
  if (rc) return rc;
  SPZ_CUDA(cudaEventRecord(io->up[j], h->copy_stream));
  return SPZ_OK;
}

// Download slab j on the copy stream once event down[j] (compute) has passed.
int io_download(spz_state_t h, HostIo* io, int j, int q) {
  SPZ_CUDA(cudaStreamWaitEvent(h->copy_stream, io->down[j], 0));
  return io_copy_slab(h, io->out_re, io->out_im, h->re, h->im, j, q, cudaMemcpyDeviceToHost);
}

// Run a list of already validated gate applications on h (with io: host
// copies before and after, overlapped where the leading / last passes allow).
int run_gates_io(spz_state_t h, const std::vector<GateApp>& gates_in, uint32_t flags, spz_exec_stats* st,
                 HostIo* io) {
  if (gates_in.empty()) return SPZ_OK;
  const uint32_t n = h->n;
  const bool fast = (flags & SPZ_EXEC_FAST) != 0;
  std::vector<GateApp> lowered;
  std::vector<PhaseTable> tables;
  if (fast) lower_fast(gates_in, n, &lowered, &tables);
  const std::vector<GateApp>& gates = fast ? lowered : gates_in;
  if (st)
    for (const GateApp& g : gates) st->fp64_ops += op_fp64_ops(n, g, tables);
  PassTimer timer;
  timer.on = (flags & SPZ_EXEC_TIME_PASSES) != 0;
  timer.stream = h->stream;
  // Upload slabs in the first tile pass's geometry (or contiguous ones); each
  // pass waits for what it reads.
  int up_q = -1;
  auto queue_uploads = [&](int q) -> int {
    if (!(io && io->in_re)) return SPZ_OK;
    up_q = q >= 0 ? q : (int)n - 3;
    for (int j = 0; j < kIoChunks; ++j) {
      int rc = io_upload(h, io, j, up_q);
      if (rc) return rc;
    }
    return SPZ_OK;
  };
  bool uploaded_wait = false;  // the compute stream already waits for every slab
  auto wait_all_uploads = [&]() -> int {
    if (io && io->in_re && !uploaded_wait) {
      SPZ_CUDA(cudaStreamWaitEvent(h->stream, io->up[kIoChunks - 1], 0));  // slabs upload in order
      uploaded_wait = true;
    }
    return SPZ_OK;
  };
  auto download_all = [&]() -> int {
    if (io && io->out_re) {
      for (int j = 0; j < kIoChunks; ++j) {
        SPZ_CUDA(cudaEventRecord(io->down[j], h->stream));
        int rc = io_download(h, io, j, (int)n - 3);
        if (rc) return rc;
      }
    }
    return SPZ_OK;
  };
  if ((flags & SPZ_EXEC_UNFUSED) && !fast) {
    {
      int rc = queue_uploads(-1);
      if (!rc) rc = wait_all_uploads();
      if (rc) return rc;
    }
    for (const GateApp& g : gates) {
      int rc = timer.begin();
      if (!rc) rc = launch_gate(h, g);
      if (!rc) rc = timer.end(false);
      if (rc) {
        timer.collect(nullptr);
        return rc;
      }
      if (st) {
        st->passes++;
        st->bytes_moved += gate_algorithmic_bytes(n, g);
      }
    }
    int rc = download_all();
    if (rc) {
      timer.collect(nullptr);
      return rc;
    }
    return timer.collect(st);
  }
  const int k = std::min<int>((int)n, h->tile_k ? h->tile_k : kTileMaxK);
  const int c = std::min<int>(kTileLowBits, k);
  std::vector<PlannedPass> passes = plan(gates, n, k, c, !fast);
  pad_tile_passes(passes, n, k);
  // Phase tables, flattened (re, im) after the gate list.
  std::vector<uint32_t> table_offsets;
  std::vector<double> flat;
  for (const PhaseTable& t : tables) {
    table_offsets.push_back((uint32_t)(flat.size() / 2));
    for (size_t i = 0; i < t.re.size(); ++i) {
      flat.push_back(t.re[i]);
      flat.push_back(t.im[i]);
    }
  }
  // A pass runs as a tile pass unless it is one exact gate (the plain kernel
  // touches only what that gate needs); lowered fast ops exist only in tiles.
  auto tiled = [&](const PlannedPass& P) {
    return P.gates.size() > 1 || P.gates[0].kind >= FK_LAZY_H || P.gates[0].cond >= 0;
  };
  std::vector<TileGate> all;
  std::vector<size_t> offs, counts;
  for (const PlannedPass& P : passes) {
    offs.push_back(all.size());
    std::vector<TileGate> pg;
    if (tiled(P)) {
      for (const GateApp& g : P.gates) pg.push_back(tile_gate(g, P.local, &tables, &table_offsets));
      if (fast) {
        const uint64_t saved = fuse_lazy_pairs(pg, P.gates, tables, &flat, n);
        if (st) st->fp64_ops -= saved;
      }
      if (flags & SPZ_EXEC_SHUFFLE) {
        const size_t r = mark_shuffle_runs(pg.data(), pg.size(), (int)P.local.size());
        if (st) st->shuffle_gates += r;
      }
      all.insert(all.end(), pg.begin(), pg.end());
    }
    counts.push_back(pg.size());
  }
  TileGate* dgates = nullptr;
  const double2* dtables = nullptr;
  if (!all.empty()) {
    void* dscr;
    const size_t gbytes = (all.size() * sizeof(TileGate) + 255) / 256 * 256;
    const size_t tbytes = flat.size() * sizeof(double);
    int rc = ensure_dev_scratch(h, gbytes + tbytes, &dscr);
    if (rc) return rc;
    // From pageable memory: the runtime stages the bytes before returning, so
    // `all` and `flat` may go out of scope while the copies are still queued.
    SPZ_CUDA(cudaMemcpyAsync(dscr, all.data(), all.size() * sizeof(TileGate), cudaMemcpyHostToDevice, h->stream));
    if (tbytes)
      SPZ_CUDA(cudaMemcpyAsync((char*)dscr + gbytes, flat.data(), tbytes, cudaMemcpyHostToDevice, h->stream));
    dgates = (TileGate*)dscr;
    dtables = (const double2*)((char*)dscr + gbytes);
  }

  // TMA staging (SPZ_EXEC_TMA*): tensor maps once per handle; the timeout word
  // is cleared here and read back at the end of the run.
  const bool shfl = (flags & SPZ_EXEC_SHUFFLE) != 0;
  bool use_tma = false;
#if !SPZ_TILE_SWIZZLE
  if ((flags & (SPZ_EXEC_TMA | SPZ_EXEC_TMA_PREFETCH)) && n >= 5) {
    int rc = ensure_tma_maps(h);
    if (rc) return rc;
    SPZ_CUDA(cudaMemsetAsync(h->tma_err, 0, sizeof(int), h->stream));
    use_tma = true;
  }
#endif
  auto pass_slab_q = [&](const PlannedPass& P) -> int {
    if (!io || n < 3 || !tiled(P) || (n - P.local.size()) < 3) return -1;
    uint64_t local_mask = 0;
    for (int q : P.local) local_mask |= 1ull << q;
    return slab_qubit(local_mask, n);
  };
  {
    int rc = queue_uploads(passes.empty() ? -1 : pass_slab_q(passes[0]));
    if (rc) return rc;
  }
  // Tiles [part * ntiles / parts, (part + 1) * ntiles / parts) of tile pass p.
  // slab_q >= 0: slab `part` of kIoChunks whose slab qubits slab_q .. slab_q + 2
  // are non-local in pass p (the tiles are selected by their index bits).
  auto launch_tiles = [&](size_t p, int part, int parts, int slab_q = -1) -> int {
    const PlannedPass& P = passes[p];
    char label[96];
    std::snprintf(label, sizeof label, "tile pass %zu: %zu ops, %zu local qubits, part %d of %d", p, counts[p],
                  P.local.size(), part, parts);
    NvtxRange range(label);
    PassArgs A{};
    A.re = h->re;
    A.im = h->im;
    A.k = (int)P.local.size();
    A.c = c;
    A.nhigh = A.k - c;
    for (int j = 0; j < A.k; ++j) A.lpos[j] = (uint8_t)P.local[j];
    const uint64_t ntiles = 1ull << (n - A.k);
    uint64_t per = ntiles / parts;
    if (slab_q >= 0) {
      uint64_t L = 0;
      for (int q : P.local) L |= 1ull << q;
      A.slab_on = 1;
      A.slab_pos = (uint32_t)(slab_q - __builtin_popcountll(L & ((1ull << slab_q) - 1)));
      A.slab = (uint32_t)part;
      per = ntiles / kIoChunks;
      A.tile_begin = 0;
      A.ntiles = per;
    } else {
      A.tile_begin = per * part;
      A.ntiles = per * (part + 1);
    }
    A.gates = dgates + offs[p];
    A.tables = dtables;
    A.outcomes = h->meas ? reinterpret_cast<const int32_t*>(h->meas + kMeasOutcomeOffset) : nullptr;
    A.ngates = (int)counts[p];
    const uint32_t T = 1u << A.k;
    const size_t smem = 2 * T * sizeof(double) + (size_t)(1u << A.nhigh) * sizeof(uint32_t);
    const int threads = h->tile_threads ? h->tile_threads
                                        : (int)std::min<uint32_t>(kTileThreads, std::max<uint32_t>(32, T / 2));
    int resident = 0, sms = 0;
    int rc = tile_launch_shape(h->device, threads, smem, &resident, &sms, shfl);
    if (rc) return rc;
    if (use_tma && !A.slab_on && A.c == kTileLowBits && A.k >= kTileLowBits + 2) {
      const bool pre = (flags & SPZ_EXEC_TMA_PREFETCH) != 0;
      const size_t tsmem = (pre ? 4 : 2) * T * sizeof(double) + (size_t)(1u << A.nhigh) * sizeof(uint64_t) + 128;
      int tres = 0;
      rc = tma_launch_shape(h->device, pre, threads, tsmem, &tres);
      if (rc) return rc;
      CUtensorMap mre, mim;
      std::memcpy(&mre, h->tma_map[0], sizeof(mre));
      std::memcpy(&mim, h->tma_map[1], sizeof(mim));
      const uint64_t tblocks = std::min<uint64_t>(per, (uint64_t)sms * tres);
      if (pre) tile_kernel_tma<true><<<(unsigned)tblocks, threads, tsmem, h->stream>>>(A, mre, mim, h->tma_err);
      else tile_kernel_tma<false><<<(unsigned)tblocks, threads, tsmem, h->stream>>>(A, mre, mim, h->tma_err);
      SPZ_CHECK_LAUNCH("tile_kernel_tma");
      return SPZ_OK;
    }
    const uint64_t blocks = std::min<uint64_t>(per, (uint64_t)sms * resident);
    if (shfl) tile_kernel<true><<<(unsigned)blocks, threads, smem, h->stream>>>(A);
    else tile_kernel<false><<<(unsigned)blocks, threads, smem, h->stream>>>(A);
    SPZ_CHECK_LAUNCH("tile_kernel");
    return SPZ_OK;
  };
  // Slab-major prefix: the leading tile passes whose three highest non-local
  // qubits are the upload's slab qubits all read and write slab j within slab
  // j's tile range, so they run slab by slab (upload j, passes 0 .. m-1 on slab
  // j, then slab j + 1), hiding m passes of compute behind the upload instead
  // of one.  When that covers every pass, each slab's download follows its
  // last launch.
  size_t first = 0;
  if (io && io->in_re && up_q >= 0) {
    size_t m = 0;
    while (m < passes.size() && pass_slab_q(passes[m]) == up_q) ++m;
    if (m >= 2) {
      const bool all = m == passes.size();
      const bool down = all && io->out_re;
      int rc = timer.begin();
      for (int j = 0; j < kIoChunks && !rc; ++j) {
        cudaError_t we = cudaStreamWaitEvent(h->stream, io->up[j], 0);
        if (we != cudaSuccess) rc = cuda_fail(we, "cudaStreamWaitEvent");
        for (size_t p = 0; p < m && !rc; ++p) rc = launch_tiles(p, j, kIoChunks);
        if (!rc && down) {
          cudaError_t re = cudaEventRecord(io->down[j], h->stream);
          rc = re == cudaSuccess ? io_download(h, io, j, up_q) : cuda_fail(re, "cudaEventRecord");
        }
      }
      uploaded_wait = true;
      if (!rc) rc = timer.end(true);
      if (!rc && all && !down) rc = download_all();
      if (rc) {
        timer.collect(nullptr);
        return rc;
      }
      if (st) {
        st->passes += m;
        st->tile_passes += m;
        st->bytes_moved += m * (32ull << n);
        st->io_slab_passes += m;
      }
      first = m;
    }
  }
  // Slab-major suffix: the trailing tile passes that all keep three
  // consecutive qubits q .. q + 2 non-local run slab by slab (passes s .. last
  // on slab j, then slab j's download), so the download hides behind several
  // passes instead of the last one.  q is the one that gives the longest
  // suffix (the highest among equals); its slabs are copied as up to 64 runs
  // (q >= n - 9) or as one strided copy of rows of 2^q amplitudes
  // (15 <= q <= 24).  Rows of 2^11 amplitudes (16 KiB) measured about half
  // the contiguous copy rate (2 GiB slabs in 20 ms against 10 ms); rows of at
  // least 256 KiB keep the per-row cost negligible.
  size_t suf = passes.size();
  int suf_q = -1;
  if (io && io->out_re && !use_tma && passes.size() > first) {
    const size_t room = passes.size() - first - (io->in_re && !uploaded_wait ? 1 : 0);
    size_t best = 1;
    for (int q = (int)n - 3; q >= 3; --q) {
      if ((int)n - q - 3 > 6 && (q < 15 || q > 24)) continue;
      const uint64_t slab_bits = 7ull << q;
      size_t m = 0;
      while (m < room) {
        const PlannedPass& P = passes[passes.size() - 1 - m];
        if (!tiled(P)) break;
        uint64_t L = 0;
        for (int x : P.local) L |= 1ull << x;
        if (L & slab_bits) break;
        ++m;
      }
      if (m > best) {
        best = m;
        suf_q = q;
      }
    }
    if (suf_q >= 0) suf = passes.size() - best;
  }
  for (size_t p = first; p < suf; ++p) {
    const PlannedPass& P = passes[p];
    const bool last = p + 1 == passes.size();
    if (!tiled(P)) {
      int rc = wait_all_uploads();
      if (!rc) rc = timer.begin();
      if (!rc) rc = launch_gate(h, P.gates[0]);
      if (!rc) rc = timer.end(false);
      if (!rc && last) rc = download_all();
      if (rc) {
        timer.collect(nullptr);
        return rc;
      }
      if (st) {
        st->passes++;
        st->bytes_moved += gate_algorithmic_bytes(n, P.gates[0]);
      }
      continue;
    }
    // With host copies to overlap, the first / last pass runs slab by slab
    // (the first pass only in the geometry its uploads were queued in).
    const int sq = pass_slab_q(P);
    const bool split_in = sq >= 0 && io->in_re && !uploaded_wait && sq == up_q;
    const bool split_out = sq >= 0 && io->out_re && last;
    int rc = SPZ_OK;
    if (!split_in) rc = wait_all_uploads();
    if (!rc) rc = timer.begin();
    if (rc) {
      timer.collect(nullptr);
      return rc;
    }
    const int launches = (split_in || split_out) ? kIoChunks : 1;
    for (int j = 0; j < launches; ++j) {
      if (split_in) {
        cudaError_t we = cudaStreamWaitEvent(h->stream, io->up[j], 0);
        if (we != cudaSuccess) {
          timer.collect(nullptr);
          return cuda_fail(we, "cudaStreamWaitEvent");
        }
      }
      rc = launch_tiles(p, j, launches);
      if (rc) {
        timer.collect(nullptr);
        return rc;
      }
      if (split_out) {
        cudaError_t re = cudaEventRecord(io->down[j], h->stream);
        if (re == cudaSuccess) rc = io_download(h, io, j, sq);
        else rc = cuda_fail(re, "cudaEventRecord");
        if (rc) {
          timer.collect(nullptr);
          return rc;
        }
      }
    }
    if (split_in) uploaded_wait = true;
    if (st && launches > 1) st->io_slab_passes++;
    rc = timer.end(true);
    if (!rc && last && !split_out) rc = download_all();
    if (rc) {
      timer.collect(nullptr);
      return rc;
    }
    if (st) {
      st->passes++;
      st->tile_passes++;
      st->bytes_moved += 32ull << n;
    }
  }
  if (suf < passes.size()) {
    const size_t m = passes.size() - suf;
    int rc = wait_all_uploads();
    if (!rc) rc = timer.begin();
    for (int j = 0; j < kIoChunks && !rc; ++j) {
      for (size_t p = suf; p < passes.size() && !rc; ++p) rc = launch_tiles(p, j, kIoChunks, suf_q);
      if (!rc) {
        cudaError_t re = cudaEventRecord(io->down[j], h->stream);
        rc = re == cudaSuccess ? io_download(h, io, j, suf_q) : cuda_fail(re, "cudaEventRecord");
      }
    }
    if (!rc) rc = timer.end(true);
    if (rc) {
      timer.collect(nullptr);
      return rc;
    }
    if (st) {
      st->passes += m;
      st->tile_passes += m;
      st->bytes_moved += m * (32ull << n);
      st->io_slab_passes += m;
    }
  }
  int rc = timer.collect(st);
  if (!rc && use_tma) {
    int bad = 0;
    SPZ_CUDA(cudaMemcpyAsync(&bad, h->tma_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    SPZ_CUDA(cudaStreamSynchronize(h->stream));
    if (bad) return fail(SPZ_ERR_TIMEOUT, "a TMA tile load did not complete within its wait limit");
  }
  return rc;
}

// Run a list of already validated gate applications on h.
int run_gates(spz_state_t h, const std::vector<GateApp>& gates, uint32_t flags, spz_exec_stats* st) {
  return run_gates_io(h, gates, flags, st, nullptr);
}

namespace {

// Resolve one op of a circuit into zero or one GateApp (no M).
// `on_device`: measured qubits whose outcome is only on the device; a Single
// control on one of them becomes a device-side condition of the gate.
int op_to_app(spz_state_t h, const spz_op& op, const spz_tracker& tr, uint64_t on_device, bool* skip,
              GateApp* out) {
  *skip = false;
  spz_gate gate = op.gate;
  uint64_t ones = 0, zeros = 0;
  int cond = -1;
  switch (op.controls_kind) {
    case SPZ_CONTROLS_NONE:
      break;
    case SPZ_CONTROLS_SINGLE: {
      if (op.controls == 0 || (op.controls & (op.controls - 1)) != 0)
        return fail(SPZ_ERR_INVALID_ARGUMENT, "Single controls need exactly one control qubit");
      const int c = __builtin_ctzll(op.controls);
      if ((on_device >> c) & 1) {  // classical control on a device-side outcome
        cond = c;
      } else if ((tr.measured >> c) & 1) {  // classical control (circuit.rs:570-578)
        if (!((tr.values >> c) & 1)) {
          *skip = true;
          return SPZ_OK;
        }
      } else {
        ones = op.controls;
      }
      break;
    }
    case SPZ_CONTROLS_ONES:
      ones = op.controls;
      break;
    case SPZ_CONTROLS_MIXED:
      if (op.zeros & ~op.controls) return fail(SPZ_ERR_INVALID_ARGUMENT, "zeros must be a subset of controls");
      ones = op.controls & ~op.zeros;
      zeros = op.zeros;
      break;
    default:
      return fail(SPZ_ERR_INVALID_ARGUMENT, "unknown controls kind");
  }
  if (gate.kind == SPZ_GATE_BITFLIP) {  // gates.rs:1365-1374 with the draw in p[1]
    if (!(gate.p[1] <= gate.p[0])) {
      if (op.target >= h->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "target qubit out of range");
      *skip = true;
      return SPZ_OK;
    }
    gate = spz_gate{};
    gate.kind = SPZ_GATE_X;
  }
  int rc = make_gate_app(h->n, gate, op.target, ones, zeros, out);
  if (!rc) out->cond = cond;
  return rc;
}

}  // namespace

// With io: the state is first uploaded from io's host arrays and finally
// downloaded to them (the copies overlap the first and last run of gates).
int execute(spz_state_t h, const spz_op* ops, size_t nops, spz_tracker* tracker, uint32_t flags,
            spz_exec_stats* st, HostIo* io = nullptr) {
  spz_tracker tr{};
  if (tracker) tr = *tracker;
  std::vector<GateApp> seg;
  bool in_pending = io && io->in_re;
  // Measurements stay on the device unless every gate runs as a plain kernel
  // (which cannot test a device-side condition).
  const bool device_meas = !(flags & SPZ_EXEC_UNFUSED) || (flags & SPZ_EXEC_FAST);
  uint64_t on_device = 0;  // qubits measured in this call, outcome on the device
  auto run_seg = [&](bool final_seg) -> int {
    HostIo sub;
    HostIo* use = nullptr;
    if (io) {
      sub = *io;
      if (!in_pending) sub.in_re = sub.in_im = nullptr;
      if (!final_seg) sub.out_re = sub.out_im = nullptr;
      if (sub.in_re || sub.out_re) use = &sub;
    }
    in_pending = false;
    if (!seg.empty()) return run_gates_io(h, seg, flags, st, use);
    const size_t bytes = h->N * sizeof(double);
    if (use && use->in_re) {
      SPZ_CUDA(cudaMemcpyAsync(h->re, use->in_re, bytes, cudaMemcpyHostToDevice, h->stream));
      SPZ_CUDA(cudaMemcpyAsync(h->im, use->in_im, bytes, cudaMemcpyHostToDevice, h->stream));
    }
    if (use && use->out_re) {
      SPZ_CUDA(cudaMemcpyAsync(use->out_re, h->re, bytes, cudaMemcpyDeviceToHost, h->stream));
      SPZ_CUDA(cudaMemcpyAsync(use->out_im, h->im, bytes, cudaMemcpyDeviceToHost, h->stream));
    }
    return SPZ_OK;
  };
  for (size_t i = 0; i < nops; ++i) {
    const spz_op& op = ops[i];
    if (op.gate.kind == SPZ_GATE_M) {  // circuit.rs:559-566: a barrier
      if (op.controls_kind != SPZ_CONTROLS_NONE)
        return fail(SPZ_ERR_UNSUPPORTED, "a measurement cannot be controlled");
      if (op.target >= h->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "target qubit out of range");
      if (!((tr.measured >> op.target) & 1)) {
        int rc = run_seg(false);
        if (rc) return rc;
        seg.clear();
        if (device_meas) {  // outcome stays on the device; later gates test it there
          rc = measure_on_device(h, op.target, 1, op.gate.p[0]);
          if (rc) return rc;
          on_device |= 1ull << op.target;
        } else {
          uint8_t v = 0;
          rc = measure_qubit(h, op.target, 1, -1, op.gate.p[0], &v, nullptr);
          if (rc) return rc;
          tr.values = (tr.values & ~(1ull << op.target)) | ((uint64_t)v << op.target);
        }
        tr.measured |= 1ull << op.target;
        if (st) st->passes += 2;
      }
      continue;
    }
    bool skip;
    GateApp a;
    int rc = op_to_app(h, op, tr, on_device, &skip, &a);
    if (rc) return rc;
    if (skip) continue;
    seg.push_back(a);
    if (st) {
      st->gates++;
      st->algorithmic_bytes += gate_algorithmic_bytes(h->n, a);
    }
  }
  int rc = run_seg(true);
  if (rc) return rc;
  if (on_device && tracker) {  // the outcomes measured on the device, into the tracker
    void* pinned;
    rc = ensure_host_scratch(h, 64 * sizeof(int32_t), &pinned);
    if (rc) return rc;
    SPZ_CUDA(cudaMemcpyAsync(pinned, h->meas + kMeasOutcomeOffset, 64 * sizeof(int32_t), cudaMemcpyDeviceToHost,
                             h->stream));
    SPZ_CUDA(cudaStreamSynchronize(h->stream));
    const int32_t* out = (const int32_t*)pinned;
    for (int q = 0; q < 64; ++q)
      if ((on_device >> q) & 1) tr.values = (tr.values & ~(1ull << q)) | ((uint64_t)(out[q] != 0) << q);
  }
  if (tracker) *tracker = tr;
  return SPZ_OK;
}

// Plan without executing (host only): fills the counters run_gates would.
int plan_stats(uint32_t n, const spz_op* ops, size_t nops, uint32_t flags, spz_exec_stats* st,
               std::vector<uint32_t>* order = nullptr, std::vector<uint32_t>* pass_of = nullptr,
               std::vector<uint64_t>* masks = nullptr, std::vector<uint32_t>* pass_ops = nullptr) {
  // masks / pass_ops: per pass (as counted in st->passes), the tile pass's
  // local qubits (0: not a tile pass) and its device ops
  auto record = [&](uint64_t mask, uint32_t count) {
    if (masks) {
      masks->push_back(mask);
      pass_ops->push_back(count);
    }
  };
  spz_state_s fake;
  fake.n = n;
  fake.N = 1ull << n;
  const bool device_meas = !(flags & SPZ_EXEC_UNFUSED) || (flags & SPZ_EXEC_FAST);
  uint64_t on_device = 0;
  spz_tracker tr{};
  std::vector<GateApp> seg;
  auto flush = [&]() {
    if (seg.empty()) return;
    const bool fast = (flags & SPZ_EXEC_FAST) != 0;
    std::vector<GateApp> lowered;
    std::vector<PhaseTable> tables;
    if (fast) lower_fast(seg, n, &lowered, &tables);
    const std::vector<GateApp>& run = fast ? lowered : seg;
    for (const GateApp& g : run) st->fp64_ops += op_fp64_ops(n, g, tables);
    if ((flags & SPZ_EXEC_UNFUSED) && !fast) {
      for (const GateApp& g : seg) {
        if (order) {
          order->push_back((uint32_t)g.src);
          pass_of->push_back((uint32_t)st->passes);
        }
        st->passes++;
        st->bytes_moved += gate_algorithmic_bytes(n, g);
        record(0, 1);
      }
    } else {
      const int k = std::min<int>((int)n, kTileMaxK);
      const int c = std::min<int>(kTileLowBits, k);
      const std::vector<uint32_t> no_offsets(tables.size(), 0);
      std::vector<PlannedPass> planned = plan(run, n, k, c, !fast);
      pad_tile_passes(planned, n, k);
      std::vector<double> no_flat;
      for (const PlannedPass& P : planned) {
        const bool tiled = P.gates.size() > 1 || P.gates[0].kind >= FK_LAZY_H || P.gates[0].cond >= 0;
        size_t device_ops = P.gates.size();
        if ((fast || (flags & SPZ_EXEC_SHUFFLE) || masks) && tiled) {
          std::vector<TileGate> tg;
          for (const GateApp& g : P.gates) tg.push_back(tile_gate(g, P.local, &tables, &no_offsets));
          if (fast) st->fp64_ops -= fuse_lazy_pairs(tg, P.gates, tables, &no_flat, n);
          if (flags & SPZ_EXEC_SHUFFLE) st->shuffle_gates += mark_shuffle_runs(tg.data(), tg.size(), (int)P.local.size());
          no_flat.clear();
          device_ops = tg.size();
        }
        uint64_t L = 0;
        if (tiled)
          for (int q : P.local) L |= 1ull << q;
        record(L, (uint32_t)device_ops);
        if (order && !fast)
          for (const GateApp& g : P.gates) {
            order->push_back((uint32_t)g.src);
            pass_of->push_back((uint32_t)st->passes);
          }
        st->passes++;
        if (P.gates.size() > 1 || P.gates[0].kind >= FK_LAZY_H || P.gates[0].cond >= 0) {
          st->tile_passes++;
          st->bytes_moved += 32ull << n;
        } else {
          st->bytes_moved += gate_algorithmic_bytes(n, P.gates[0]);
        }
      }
    }
    seg.clear();
  };
  for (size_t i = 0; i < nops; ++i) {
    const spz_op& op = ops[i];
    if (op.gate.kind == SPZ_GATE_M) {
      if (op.controls_kind != SPZ_CONTROLS_NONE) return fail(SPZ_ERR_UNSUPPORTED, "a measurement cannot be controlled");
      if (op.target >= n) return fail(SPZ_ERR_INVALID_ARGUMENT, "target qubit out of range");
      if (!((tr.measured >> op.target) & 1)) {
        flush();
        tr.measured |= 1ull << op.target;
        if (device_meas) on_device |= 1ull << op.target;  // later gates: device-side condition
        // (else the outcome is unknown while planning: assume 0)
        if (order) {
          order->push_back((uint32_t)i);
          pass_of->push_back((uint32_t)st->passes);
        }
        st->passes += 2;
        record(0, 0);
        record(0, 0);
      }
      continue;
    }
    bool skip;
    GateApp a;
    int rc = op_to_app(&fake, op, tr, on_device, &skip, &a);
    if (rc) return rc;
    if (skip) continue;
    a.src = (int64_t)i;
    seg.push_back(a);
    st->gates++;
    st->algorithmic_bytes += gate_algorithmic_bytes(n, a);
  }
  flush();
  return SPZ_OK;
}

// ------------------------------------------------------------ programs
// A circuit planned once: lowered (fast mode), fused into passes, its tile
// descriptors and phase tables uploaded to device memory it owns.  A run
// replays the launches as a CUDA graph captured per target state (the graph
// holds the state's device pointers), so a repeated run costs no planning,
// no uploads and one graph launch.
struct ProgramPass {
  bool tiled = false;
  GateApp plain{};     // !tiled: the one exact gate, through the plain kernel
  PassArgs args{};     // tiled: everything but the state pointers
  int threads = 0;
  size_t smem = 0;
  uint64_t blocks = 0;
  bool shfl = false;   // tiled: launched as tile_kernel<true> (SPZ_EXEC_SHUFFLE)
};

}  // namespace spz

struct spz_program_s {
  uint32_t n = 0;
  int device = 0;
  std::vector<spz::ProgramPass> passes;
  void* dbuf = nullptr;            // tile descriptors + phase tables
  cudaStream_t capture = nullptr;  // private stream the graph is captured on
  cudaGraphExec_t exec = nullptr;  // the captured launches ...
  double* exec_re = nullptr;       // ... for this state
  double* exec_im = nullptr;
  spz_exec_stats stats{};
};

namespace spz {
namespace {

void free_program(spz_program_t p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->capture) cudaStreamDestroy(p->capture);
  if (p->dbuf) cudaFree(p->dbuf);
  delete p;
}

int build_program(spz_program_t p, const spz_op* ops, size_t nops, uint32_t flags) {
  const uint32_t n = p->n;
  spz_state_s fake;  // op validation needs only n
  fake.n = n;
  fake.N = 1ull << n;
  spz_tracker tr{};
  std::vector<GateApp> gates_in;
  for (size_t i = 0; i < nops; ++i) {
    const spz_op& op = ops[i];
    if (op.gate.kind == SPZ_GATE_M) return fail(SPZ_ERR_UNSUPPORTED, "a program cannot hold measurements");
    bool skip;
    GateApp a;
    int rc = op_to_app(&fake, op, tr, 0, &skip, &a);
    if (rc) return rc;
    if (skip) continue;
    a.src = (int64_t)i;
    gates_in.push_back(a);
    p->stats.gates++;
    p->stats.algorithmic_bytes += gate_algorithmic_bytes(n, a);
  }
  const bool fast = (flags & SPZ_EXEC_FAST) != 0;
  std::vector<GateApp> lowered;
  std::vector<PhaseTable> tables;
  if (fast) lower_fast(gates_in, n, &lowered, &tables);
  const std::vector<GateApp>& gates = fast ? lowered : gates_in;
  for (const GateApp& g : gates) p->stats.fp64_ops += op_fp64_ops(n, g, tables);
  if ((flags & SPZ_EXEC_UNFUSED) && !fast) {
    for (const GateApp& g : gates) {
      ProgramPass pp;
      pp.plain = g;
      p->passes.push_back(pp);
      p->stats.passes++;
      p->stats.bytes_moved += gate_algorithmic_bytes(n, g);
    }
    return SPZ_OK;
  }
  const int k = std::min<int>((int)n, kTileMaxK);
  const int c = std::min<int>(kTileLowBits, k);
  std::vector<PlannedPass> planned = plan(gates, n, k, c, !fast);
  pad_tile_passes(planned, n, k);
  std::vector<uint32_t> table_offsets;
  std::vector<double> flat;
  for (const PhaseTable& t : tables) {
    table_offsets.push_back((uint32_t)(flat.size() / 2));
    for (size_t i = 0; i < t.re.size(); ++i) {
      flat.push_back(t.re[i]);
      flat.push_back(t.im[i]);
    }
  }
  std::vector<TileGate> all;
  std::vector<size_t> offs, counts;
  for (const PlannedPass& P : planned) {
    offs.push_back(all.size());
    const bool tiled = P.gates.size() > 1 || P.gates[0].kind >= FK_LAZY_H || P.gates[0].cond >= 0;
    std::vector<TileGate> pg;
    if (tiled) {
      for (const GateApp& g : P.gates) pg.push_back(tile_gate(g, P.local, &tables, &table_offsets));
      if (fast) p->stats.fp64_ops -= fuse_lazy_pairs(pg, P.gates, tables, &flat, n);
      if (flags & SPZ_EXEC_SHUFFLE)
        p->stats.shuffle_gates += mark_shuffle_runs(pg.data(), pg.size(), (int)P.local.size());
      all.insert(all.end(), pg.begin(), pg.end());
    }
    counts.push_back(pg.size());
  }
  const size_t gbytes = (all.size() * sizeof(TileGate) + 255) / 256 * 256;
  const size_t tbytes = flat.size() * sizeof(double);
  if (gbytes + tbytes) {
    SPZ_CUDA(dev_alloc(&p->dbuf, gbytes + tbytes));
    if (!all.empty())
      SPZ_CUDA(cudaMemcpy(p->dbuf, all.data(), all.size() * sizeof(TileGate), cudaMemcpyHostToDevice));
    if (tbytes) SPZ_CUDA(cudaMemcpy((char*)p->dbuf + gbytes, flat.data(), tbytes, cudaMemcpyHostToDevice));
  }

  for (size_t q = 0; q < planned.size(); ++q) {
    const PlannedPass& P = planned[q];
    ProgramPass pp;
    pp.tiled = P.gates.size() > 1 || P.gates[0].kind >= FK_LAZY_H || P.gates[0].cond >= 0;
    p->stats.passes++;
    if (!pp.tiled) {
      pp.plain = P.gates[0];
      p->stats.bytes_moved += gate_algorithmic_bytes(n, P.gates[0]);
      p->passes.push_back(pp);
      continue;
    }
    PassArgs& A = pp.args;
    A.k = (int)P.local.size();
    A.c = c;
    A.nhigh = A.k - c;
    for (int j = 0; j < A.k; ++j) A.lpos[j] = (uint8_t)P.local[j];
    A.ntiles = 1ull << (n - A.k);
    A.gates = (const TileGate*)p->dbuf + offs[q];
    A.tables = (const double2*)((char*)p->dbuf + gbytes);
    A.ngates = (int)counts[q];
    const uint32_t T = 1u << A.k;
    pp.smem = 2 * T * sizeof(double) + (size_t)(1u << A.nhigh) * sizeof(uint32_t);
    pp.threads = (int)std::min<uint32_t>(kTileThreads, std::max<uint32_t>(32, T / 2));
    pp.shfl = (flags & SPZ_EXEC_SHUFFLE) != 0;
    int resident = 0, sms = 0;
    int rc = tile_launch_shape(p->device, pp.threads, pp.smem, &resident, &sms, pp.shfl);
    if (rc) return rc;
    pp.blocks = std::min<uint64_t>(A.ntiles, (uint64_t)sms * resident);
    p->stats.tile_passes++;
    p->stats.bytes_moved += 32ull << n;
    p->passes.push_back(pp);
  }
  return SPZ_OK;
}

// Capture the program's launches for state h (on the private stream).
int capture_program(spz_program_t p, spz_state_t h) {
  if (!p->capture) SPZ_CUDA(cudaStreamCreateWithFlags(&p->capture, cudaStreamNonBlocking));
  spz_state_s v;  // h's arrays, launched on the capture stream
  v.n = h->n;
  v.N = h->N;
  v.re = h->re;
  v.im = h->im;
  v.owns = false;
  v.stream = p->capture;
  v.device = h->device;
  SPZ_CUDA(cudaStreamBeginCapture(p->capture, cudaStreamCaptureModeThreadLocal));
  int rc = SPZ_OK;
  for (const ProgramPass& pp : p->passes) {
    if (!pp.tiled) {
      rc = launch_gate(&v, pp.plain);
    } else {
      PassArgs A = pp.args;
      A.re = h->re;
      A.im = h->im;
      A.outcomes = nullptr;
      if (pp.shfl) tile_kernel<true><<<(unsigned)pp.blocks, pp.threads, pp.smem, p->capture>>>(A);
      else tile_kernel<false><<<(unsigned)pp.blocks, pp.threads, pp.smem, p->capture>>>(A);
      cudaError_t le = cudaGetLastError();
      if (le != cudaSuccess) rc = cuda_fail(le, "tile_kernel");
    }
    if (rc) break;
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(p->capture, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "program graph capture");
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
  }
  e = cudaGraphInstantiate(&p->exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "program graph instantiation");
  p->exec_re = h->re;
  p->exec_im = h->im;
  return SPZ_OK;
}

}  // namespace

}  // namespace spz

using namespace spz;

extern "C" {

int spz_circuit_execute(spz_state_t h, const spz_op* ops, size_t nops, spz_tracker* tracker, uint32_t flags,
                        spz_exec_stats* stats) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  if (nops && !ops) return fail(SPZ_ERR_NULL, "ops is NULL");
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (int rc = settle(h)) return rc;  // measurements read the state
  NvtxRange range("spz_circuit_execute");
  return execute(h, ops, nops, tracker, flags, stats);
}

int spz_circuit_execute_host(spz_state_t h, const double* in_reals, const double* in_imags, double* out_reals,
                             double* out_imags, const spz_op* ops, size_t nops, spz_tracker* tracker, uint32_t flags,
                             spz_exec_stats* stats) {
  if (!h || !in_reals || !in_imags || !out_reals || !out_imags) return fail(SPZ_ERR_NULL, "NULL argument");
  if (nops && !ops) return fail(SPZ_ERR_NULL, "ops is NULL");
  if (stats) std::memset(stats, 0, sizeof(*stats));
  clear_factor(h);  // the handle's contents are replaced by the input arrays
  NvtxRange range("spz_circuit_execute_host");
  auto pinned = [](const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return a.type == cudaMemoryTypeHost;
  };
  if (!pinned(in_reals) || !pinned(in_imags) || !pinned(out_reals) || !pinned(out_imags)) {
    // pageable: staged copies, nothing to overlap
    int rc = spz_state_upload(h, in_reals, in_imags);
    if (!rc) rc = execute(h, ops, nops, tracker, flags, stats);
    if (!rc) rc = spz_state_download(h, out_reals, out_imags);
    return rc;
  }
  if (!h->copy_stream) SPZ_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
  // The copy stream runs every upload slab before any download slab, so the
  // output may alias the input.
  HostIo io;
  io.in_re = in_reals;
  io.in_im = in_imags;
  io.out_re = out_reals;
  io.out_im = out_imags;
  int rc = SPZ_OK;
  int made = 0;
  for (; made < kIoChunks && !rc; ++made) {
    cudaError_t e1 = cudaEventCreateWithFlags(&io.up[made], cudaEventDisableTiming);
    cudaError_t e2 = e1 == cudaSuccess ? cudaEventCreateWithFlags(&io.down[made], cudaEventDisableTiming) : e1;
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
      if (e1 == cudaSuccess) cudaEventDestroy(io.up[made]);
      rc = cuda_fail(e1 != cudaSuccess ? e1 : e2, "cudaEventCreateWithFlags");
      break;
    }
  }
  if (!rc) rc = execute(h, ops, nops, tracker, flags, stats, &io);
  // Copies may be in flight on either stream (also after an error): they read
  // and write the caller's arrays, so wait for both before returning.
  cudaError_t s1 = cudaStreamSynchronize(h->copy_stream);
  cudaError_t s2 = cudaStreamSynchronize(h->stream);
  for (int j = 0; j < made; ++j) {
    cudaEventDestroy(io.up[j]);
    cudaEventDestroy(io.down[j]);
  }
  if (rc) return rc;
  if (s1 != cudaSuccess) return cuda_fail(s1, "cudaStreamSynchronize");
  if (s2 != cudaSuccess) return cuda_fail(s2, "cudaStreamSynchronize");
  return SPZ_OK;
}

int spz_plan_stats(uint32_t n, const spz_op* ops, size_t nops, uint32_t flags, spz_exec_stats* stats) {
  if (!stats) return fail(SPZ_ERR_NULL, "stats is NULL");
  if (nops && !ops) return fail(SPZ_ERR_NULL, "ops is NULL");
  if (n == 0 || n > kMaxQubits) return fail(SPZ_ERR_INVALID_ARGUMENT, "n out of range");
  std::memset(stats, 0, sizeof(*stats));
  return plan_stats(n, ops, nops, flags, stats);
}

int spz_plan_passes(uint32_t n, const spz_op* ops, size_t nops, uint32_t flags, uint64_t* local_mask,
                    uint32_t* pass_ops, size_t capacity, size_t* count) {
  if (!count || (capacity && (!local_mask || !pass_ops))) return fail(SPZ_ERR_NULL, "NULL argument");
  if (nops && !ops) return fail(SPZ_ERR_NULL, "ops is NULL");
  if (n == 0 || n > kMaxQubits) return fail(SPZ_ERR_INVALID_ARGUMENT, "n out of range");
  spz_exec_stats st{};
  std::vector<uint64_t> m;
  std::vector<uint32_t> c;
  int rc = plan_stats(n, ops, nops, flags, &st, nullptr, nullptr, &m, &c);
  if (rc) return rc;
  *count = m.size();
  for (size_t i = 0; i < m.size() && i < capacity; ++i) {
    local_mask[i] = m[i];
    pass_ops[i] = c[i];
  }
  return SPZ_OK;
}

int spz_plan_schedule(uint32_t n, const spz_op* ops, size_t nops, uint32_t flags, uint32_t* order, uint32_t* pass,
                      size_t capacity, size_t* count) {
  if (!count || (capacity && (!order || !pass))) return fail(SPZ_ERR_NULL, "NULL argument");
  if (nops && !ops) return fail(SPZ_ERR_NULL, "ops is NULL");
  if (n == 0 || n > kMaxQubits) return fail(SPZ_ERR_INVALID_ARGUMENT, "n out of range");
  spz_exec_stats st{};
  std::vector<uint32_t> o, p;
  int rc = plan_stats(n, ops, nops, flags, &st, &o, &p);
  if (rc) return rc;
  *count = o.size();
  for (size_t i = 0; i < o.size() && i < capacity; ++i) {
    order[i] = o[i];
    pass[i] = p[i];
  }
  return SPZ_OK;
}

// core.rs:184-191: for j = len-1 .. 0: H(targets[j]); for k = j-1 .. 0:
// CP(-pi / 2^(j-k)) with control targets[j], target targets[k].
int spz_iqft(spz_state_t h, const uint32_t* targets, uint32_t ntargets) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  if (ntargets && !targets) return fail(SPZ_ERR_NULL, "targets is NULL");
  std::vector<spz_op> ops;
  for (int64_t j = (int64_t)ntargets - 1; j >= 0; --j) {
    spz_op op{};
    op.gate.kind = SPZ_GATE_H;
    op.target = targets[j];
    ops.push_back(op);
    for (int64_t k = j - 1; k >= 0; --k) {
      spz_op cp{};
      cp.gate.kind = SPZ_GATE_P;
      cp.gate.p[0] = -3.14159265358979323846 / std::ldexp(1.0, (int)(j - k));
      cp.target = targets[k];
      cp.controls_kind = SPZ_CONTROLS_SINGLE;
      if (targets[j] >= 64) return fail(SPZ_ERR_INVALID_ARGUMENT, "target qubit out of range");
      cp.controls = 1ull << targets[j];
      ops.push_back(cp);
    }
  }
  return execute(h, ops.data(), ops.size(), nullptr, SPZ_EXEC_DEFAULT, nullptr);
}

int spz_program_create(uint32_t n, const spz_op* ops, size_t nops, uint32_t flags, spz_program_t* out) {
  if (!out || (nops && !ops)) return fail(SPZ_ERR_NULL, "NULL argument");
  if (n == 0 || n > kMaxQubits) return fail(SPZ_ERR_INVALID_ARGUMENT, "n out of range");
  spz_program_t p = new (std::nothrow) spz_program_s();
  if (!p) return fail(SPZ_ERR_OUT_OF_MEMORY, "host allocation failed");
  p->n = n;
  cudaError_t e = cudaGetDevice(&p->device);
  int rc = e == cudaSuccess ? build_program(p, ops, nops, flags) : cuda_fail(e, "cudaGetDevice");
  if (rc) {
    free_program(p);
    return rc;
  }
  *out = p;
  return SPZ_OK;
}

int spz_program_run(spz_program_t p, spz_state_t h) {
  if (!p || !h) return fail(SPZ_ERR_NULL, "NULL argument");
  if (h->n != p->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "the state's qubit count differs from the program's");
  if (p->passes.empty()) return SPZ_OK;
  if (!p->exec || p->exec_re != h->re || p->exec_im != h->im) {
    int rc = capture_program(p, h);
    if (rc) return rc;
  }
  SPZ_CUDA(cudaGraphLaunch(p->exec, h->stream));
  return SPZ_OK;
}

int spz_program_stats(spz_program_t p, spz_exec_stats* stats) {
  if (!p || !stats) return fail(SPZ_ERR_NULL, "NULL argument");
  *stats = p->stats;
  return SPZ_OK;
}

int spz_program_destroy(spz_program_t p) {
  if (p && p->capture) cudaStreamSynchronize(p->capture);
  free_program(p);
  return SPZ_OK;
}

}  // extern "C"
