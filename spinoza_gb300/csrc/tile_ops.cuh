// Gate ops on a tile of amplitudes held in shared memory, shared by the fused
// circuit executor (circuit.cu) and the batched engine (batch.cu).  A gate
// descriptor G provides: pos[] / npos (sorted tile-offset bits inserted as
// zeros by the enumeration: target and local controls), l_ones (local bits
// set: controls, and the target of a diagonal gate that acts on its 1 half),
// tbit / tbit2 (the target's tile bit; SWAP's second), and the gate's Coef c.
#pragma once

#include "common.cuh"
#include "gate_math.cuh"

namespace spz {

// Every tile op reads its descriptor once, into registers, before its loop:
// the loop body then touches only shared memory (and, for phase ops, the
// phase table through L1).

// m -> tile offset with zero bits inserted at the op's sorted local positions
// (NPOS of them; -1 = any number, read from the descriptor), then l_ones set.
// Inserting a zero at p is e + (e & ~(2^p - 1)); ascending order keeps the
// lower insertions in place.
template <int NPOS, class G>
struct Enumerator {
  uint32_t hm[NPOS > 0 ? NPOS : 1];
  uint32_t ones;
  __device__ __forceinline__ explicit Enumerator(const G& g) {
#pragma unroll
    for (int j = 0; j < NPOS; ++j) hm[j] = ~((1u << g.pos[j]) - 1u);
    ones = g.l_ones;
  }
  __device__ __forceinline__ uint32_t operator()(uint32_t m) const {
    uint32_t e = m;
#pragma unroll
    for (int j = 0; j < NPOS; ++j) e += e & hm[j];
    return e | ones;
  }
};

template <class G>
struct Enumerator<-1, G> {
  const uint8_t* pos;
  int npos;
  uint32_t ones;
  __device__ __forceinline__ explicit Enumerator(const G& g) : pos(g.pos), npos(g.npos), ones(g.l_ones) {}
  __device__ __forceinline__ uint32_t operator()(uint32_t m) const {
    uint32_t e = m;
    for (int j = 0; j < npos; ++j) e += e & ~((1u << pos[j]) - 1u);
    return e | ones;
  }
};

// Shared-memory layout of a tile: amplitude e lives at SW::at(e).
// NoSwizzle keeps e.  NibbleSwizzle flips the low four bits of e when bit 4
// is set: the 16 lanes of a half-warp that read s0 (or s1) of a pair op with
// its target at tile bit 0-3 then hit 16 distinct 8-byte bank slots instead
// of 8 twice (a 2-way conflict); accesses whose low four bits run through all
// values in a half-warp are unaffected.  An involution.
struct NoSwizzle {
  __device__ __forceinline__ static uint32_t at(uint32_t e) { return e; }
};
struct NibbleSwizzle {
  __device__ __forceinline__ static uint32_t at(uint32_t e) { return e ^ ((0u - ((e >> 4) & 1u)) & 15u); }
};

// Unroll factor of the per-pair loops (independent iterations in flight per
// thread); 2 measured no faster than 1 on the 30-qubit brickwork.
#ifndef SPZ_TILE_UNROLL
#define SPZ_TILE_UNROLL 1
#endif
constexpr int kTileUnroll = SPZ_TILE_UNROLL;

// Dispatch on the op's insertion count: 0-3 specialised, more generic.
#define SPZ_BY_NPOS(npos, CALL) \
  switch (npos) {               \
    case 0: CALL(0); break;     \
    case 1: CALL(1); break;     \
    case 2: CALL(2); break;     \
    case 3: CALL(3); break;     \
    default: CALL(-1); break;   \
  }

// Pairs handled per loop iteration and thread.  The pairs of one op are
// disjoint, but the compiler cannot prove that the next pair's shared-memory
// loads do not alias this pair's stores, so unrolling alone cannot overlap
// them; the batched loop loads kTileBatch pairs, computes them, then stores.
// Measured on the 30-qubit brickwork with 2: fast mode 4% slower (80
// registers instead of 72), exact mode 0.7% faster; 4 spills.  So 1.
#ifndef SPZ_TILE_BATCH
#define SPZ_TILE_BATCH 1
#endif
constexpr int kTileBatch = SPZ_TILE_BATCH;

template <int KIND, int NPOS, class G, class SW = NoSwizzle>
__device__ __forceinline__ void tile_pair(const G& g, double* sre, double* sim, uint32_t npairs) {
  const Enumerator<NPOS, G> E(g);
  const uint32_t tbit = g.tbit;
  const Coef c = g.c;
  if constexpr (kTileBatch > 1) {
    const uint32_t step = blockDim.x;
    for (uint32_t m0 = threadIdx.x; m0 < npairs; m0 += kTileBatch * step) {
      uint32_t s0[kTileBatch], s1[kTileBatch];
      double a[kTileBatch], b[kTileBatch], x[kTileBatch], d[kTileBatch];
#pragma unroll
      for (int u = 0; u < kTileBatch; ++u) {
        const uint32_t m = m0 + u * step;
        const uint32_t e0 = E(m < npairs ? m : m0);
        s0[u] = SW::at(e0);
        s1[u] = SW::at(e0 | tbit);
        a[u] = sre[s0[u]]; b[u] = sim[s0[u]]; x[u] = sre[s1[u]]; d[u] = sim[s1[u]];
      }
#pragma unroll
      for (int u = 0; u < kTileBatch; ++u) {
        if constexpr (KIND >= FK_LAZY_H) fast_pair<KIND>(c, a[u], b[u], x[u], d[u]);
        else gate_pair<KIND>(c, a[u], b[u], x[u], d[u]);
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
      const uint32_t s0 = SW::at(e0), s1 = SW::at(e0 | tbit);
      double a = sre[s0], b = sim[s0], x = sre[s1], d = sim[s1];
      if constexpr (KIND >= FK_LAZY_H) fast_pair<KIND>(c, a, b, x, d);
      else gate_pair<KIND>(c, a, b, x, d);
      sre[s0] = a; sim[s0] = b; sre[s1] = x; sim[s1] = d;
    }
  }
}

template <int KIND, class G, class SW = NoSwizzle>
__device__ __forceinline__ void tile_pair_any(const G& g, double* sre, double* sim, uint32_t npairs) {
#define SPZ_CALL(N) tile_pair<KIND, N, G, SW>(g, sre, sim, npairs)
  SPZ_BY_NPOS(g.npos, SPZ_CALL)
#undef SPZ_CALL
}

template <int KIND, int NPOS, class G, class SW = NoSwizzle>
__device__ __forceinline__ void tile_diag(const G& g, double* sre, double* sim, uint32_t nelem, int global_one) {
  const Enumerator<NPOS, G> E(g);
  const uint32_t tbit = g.tbit;
  const Coef c = g.c;
  for (uint32_t m = threadIdx.x; m < nelem; m += blockDim.x) {
    const uint32_t e0 = E(m);
    const bool one = global_one >= 0 ? global_one != 0 : (e0 & tbit) != 0;
    const uint32_t e = SW::at(e0);
    double r = sre[e], i = sim[e];
    gate_diag<KIND>(c, one, r, i);
    sre[e] = r; sim[e] = i;
  }
}

template <int KIND, class G, class SW = NoSwizzle>
__device__ __forceinline__ void tile_diag_any(const G& g, double* sre, double* sim, uint32_t nelem,
                                              int global_one) {
#define SPZ_CALL(N) tile_diag<KIND, N, G, SW>(g, sre, sim, nelem, global_one)
  SPZ_BY_NPOS(g.npos, SPZ_CALL)
#undef SPZ_CALL
}

template <int NPOS, class G, class SW = NoSwizzle>
__device__ __forceinline__ void tile_swap(const G& g, double* sre, double* sim, uint32_t nw) {
  const Enumerator<NPOS, G> E(g);
  const uint32_t t1 = g.tbit, t2 = g.tbit2;
  for (uint32_t m = threadIdx.x; m < nw; m += blockDim.x) {
    const uint32_t b0 = E(m);
    const uint32_t i = SW::at(b0 | t2), j = SW::at(b0 | t1);
    const double r = sre[i], q = sim[i];
    sre[i] = sre[j]; sim[i] = sim[j];
    sre[j] = r; sim[j] = q;
  }
}

template <class G, class SW = NoSwizzle>
__device__ __forceinline__ void tile_swap_any(const G& g, double* sre, double* sim, uint32_t nw) {
#define SPZ_CALL(N) tile_swap<N, G, SW>(g, sre, sim, nw)
  SPZ_BY_NPOS(g.npos, SPZ_CALL)
#undef SPZ_CALL
}

}  // namespace spz
