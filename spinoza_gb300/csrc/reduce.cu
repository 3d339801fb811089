// Measurement, probability and expectation reductions, and sampling.
// Replaces spinoza/src/measurement.rs:12-92 (measure_qubit) and the
// reductions of spinoza/src/core.rs:65-264 (reservoir sampling,
// qubit_expectation_value, xyz_expectation_value).
//
// All sums are deterministic: a fixed grid (a function of the size only),
// each thread folding its strided elements in a fixed order, a fixed warp-
// shuffle + shared-memory tree per block, then one block folding the block
// partials in a fixed tree.  Results are identical from run to run.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace spz {

constexpr int kRedThreads = 256;
constexpr int kMaxRedBlocks = kNumSMs * 8;  // 1216 partials per quantity

__device__ __forceinline__ double block_sum(double v, double* smem) {
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
  return r;  // valid in thread 0
}

// Fold nq rows of `nblocks` partials each: out[q] = sum of partials[q][*].
__global__ void finalize_kernel(const double* __restrict__ partials, int nblocks, int nq, double* __restrict__ out) {
  __shared__ double smem[32];
  for (int q = 0; q < nq; ++q) {
    double v = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) v = dadd(v, partials[(size_t)q * nblocks + b]);
    v = block_sum(v, smem);
    if (threadIdx.x == 0) out[q] = v;
  }
}

enum RedMode { RED_PROB0 = 0, RED_X = 1, RED_Y = 2, RED_Z = 3, RED_NORM = 4 };

// Per-pair functionals over the pairs (s0, s1 = s0 | tbit) with s0 enumerated
// by inserting a zero at the target bit.  With tbit == 0 (RED_NORM) every
// amplitude is one "pair" element s0.
template <int MODE>
__global__ void __launch_bounds__(kRedThreads) pair_reduce_kernel(const double* __restrict__ re,
                                                                  const double* __restrict__ im, uint64_t nwork,
                                                                  int t, double* __restrict__ partials) {
  __shared__ double smem[32];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t tbit = 1ull << t, lowmask = tbit - 1;
  double acc = 0.0;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwork; w += stride) {
    if constexpr (MODE == RED_NORM) {
      const double a = re[w], b = im[w];
      acc = dadd(acc, dfma(a, a, dmul(b, b)));
    } else {
      const uint64_t s0 = ((w & ~lowmask) << 1) | (w & lowmask);
      const double a = re[s0], b = im[s0];
      if constexpr (MODE == RED_PROB0) {
        acc = dadd(acc, dfma(a, a, dmul(b, b)));
      } else {
        const uint64_t s1 = s0 | tbit;
        const double c = re[s1], d = im[s1];
        if constexpr (MODE == RED_X) {  // Re<psi|X psi> per pair: 2 (a c + b d)
          acc = dadd(acc, dmul(2.0, dfma(a, c, dmul(b, d))));
        } else if constexpr (MODE == RED_Y) {  // 2 (a d - b c)
          acc = dadd(acc, dmul(2.0, dfma(a, d, dmul(dneg(b), c))));
        } else {  // Z: |s0|^2 - |s1|^2
          acc = dadd(acc, dsub(dfma(a, a, dmul(b, b)), dfma(c, c, dmul(d, d))));
        }
      }
    }
  }
  const double s = block_sum(acc, smem);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// Launch a pair reduction, fold the partials into d_out[0] (device).
template <int MODE>
static int pair_reduce_to_device(spz_state_t h, int t, double* d_partials, double* d_out) {
  const uint64_t nwork = MODE == RED_NORM ? h->N : h->N / 2;
  const int blocks = std::min<int>(grid_for(nwork, kRedThreads, 8), kMaxRedBlocks);
  pair_reduce_kernel<MODE><<<blocks, kRedThreads, 0, h->stream>>>(h->re, h->im, nwork, t, d_partials);
  finalize_kernel<<<1, 1024, 0, h->stream>>>(d_partials, blocks, 1, d_out);
  SPZ_CHECK_LAUNCH("pair_reduce_kernel");
  return SPZ_OK;
}

// Read `count` doubles from the device into host memory (synchronises).
static int read_back(spz_state_t h, const double* d_src, double* host, size_t count) {
  void* pinned;
  int rc = ensure_host_scratch(h, count * sizeof(double), &pinned);
  if (rc) return rc;
  SPZ_CUDA(cudaMemcpyAsync(pinned, d_src, count * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  SPZ_CUDA(cudaStreamSynchronize(h->stream));
  std::copy((double*)pinned, (double*)pinned + count, host);
  return SPZ_OK;
}

static int reduce_scalar(spz_state_t h, int mode, int t, double* out) {
  void* scratch;
  int rc = ensure_dev_scratch(h, (kMaxRedBlocks + 8) * sizeof(double), &scratch);
  if (rc) return rc;
  double* partials = (double*)scratch;
  double* slot = partials + kMaxRedBlocks;
  switch (mode) {
    case RED_PROB0: rc = pair_reduce_to_device<RED_PROB0>(h, t, partials, slot); break;
    case RED_X: rc = pair_reduce_to_device<RED_X>(h, t, partials, slot); break;
    case RED_Y: rc = pair_reduce_to_device<RED_Y>(h, t, partials, slot); break;
    case RED_Z: rc = pair_reduce_to_device<RED_Z>(h, t, partials, slot); break;
    default: rc = pair_reduce_to_device<RED_NORM>(h, 0, partials, slot); break;
  }
  if (rc) return rc;
  return read_back(h, slot, out, 1);
}

int norm_sqr_to_device(spz_state_t h, double* d_out) {
  void* scratch;
  int rc = ensure_dev_scratch(h, 64 * 1024 * sizeof(double), &scratch);
  if (rc) return rc;
  return pair_reduce_to_device<RED_NORM>(h, 0, (double*)scratch, d_out);
}

int prob0_device(spz_state_t h, uint32_t target, double* out) { return reduce_scalar(h, RED_PROB0, (int)target, out); }

// ------------------------------------------------------------ collapse
// measurement.rs:39-86: keep the measured half scaled by 1/sqrt(p), zero the other.
__global__ void collapse_kernel(double* __restrict__ re, double* __restrict__ im, uint64_t nwork, int t,
                                int outcome, double scale) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t tbit = 1ull << t, lowmask = tbit - 1;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwork; w += stride) {
    const uint64_t s0 = ((w & ~lowmask) << 1) | (w & lowmask);
    const uint64_t s1 = s0 | tbit;
    const uint64_t keep = outcome ? s1 : s0, drop = outcome ? s0 : s1;
    re[keep] = dmul(re[keep], scale);
    im[keep] = dmul(im[keep], scale);
    re[drop] = 0.0;
    im[drop] = 0.0;
  }
}

int collapse_device(spz_state_t h, uint32_t target, int outcome, double scale) {
  collapse_kernel<<<grid_for(h->N / 2), kThreads, 0, h->stream>>>(h->re, h->im, h->N / 2, (int)target, outcome,
                                                                   scale);
  SPZ_CHECK_LAUNCH("collapse_kernel");
  return SPZ_OK;
}

// measure_qubit (measurement.rs:12-92) with an explicit draw.
// Outcome and scale from prob0 on the device (same arithmetic as measure_qubit).
__global__ void measure_decide_kernel(double* meas, int t, double u) {
  const double prob0 = meas[t];
  const int val = u < 1.0 - prob0 ? 1 : 0;
  meas[64 + t] = val == 0 ? 1.0 / sqrt(prob0) : 1.0 / sqrt(1.0 - prob0);
  reinterpret_cast<int32_t*>(meas + kMeasOutcomeOffset)[t] = val;
}

// Collapse with outcome and scale read from the device; with reset, the kept
// 1 half lands on the 0 half (collapse followed by X, which only moves).
__global__ void collapse_meas_kernel(double* __restrict__ re, double* __restrict__ im, uint64_t nwork, int t,
                                     const double* __restrict__ meas, int reset) {
  const int outcome = reinterpret_cast<const int32_t*>(meas + kMeasOutcomeOffset)[t];
  const double scale = meas[64 + t];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t tbit = 1ull << t, lowmask = tbit - 1;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwork; w += stride) {
    const uint64_t s0 = ((w & ~lowmask) << 1) | (w & lowmask);
    const uint64_t s1 = s0 | tbit;
    const uint64_t keep = outcome ? s1 : s0;
    const double kr = dmul(re[keep], scale), ki = dmul(im[keep], scale);
    const bool to0 = !outcome || reset;
    re[s0] = to0 ? kr : 0.0;
    im[s0] = to0 ? ki : 0.0;
    re[s1] = to0 ? 0.0 : kr;
    im[s1] = to0 ? 0.0 : ki;
  }
}

int measure_on_device(spz_state_t h, uint32_t target, int reset, double u) {
  if (target >= h->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "target qubit out of range");
  if (!h->meas) {
    SPZ_CUDA(dev_alloc(&h->meas, (kMeasOutcomeOffset + 64) * sizeof(double)));
    SPZ_CUDA(cudaMemsetAsync(h->meas, 0, (kMeasOutcomeOffset + 64) * sizeof(double), h->stream));
  }
  void* scratch;
  int rc = ensure_dev_scratch(h, (kMaxRedBlocks + 8) * sizeof(double), &scratch);
  if (rc) return rc;
  rc = pair_reduce_to_device<RED_PROB0>(h, (int)target, (double*)scratch, h->meas + target);
  if (rc) return rc;
  measure_decide_kernel<<<1, 1, 0, h->stream>>>(h->meas, (int)target, u);
  collapse_meas_kernel<<<grid_for(h->N / 2), kThreads, 0, h->stream>>>(h->re, h->im, h->N / 2, (int)target, h->meas,
                                                                       reset);
  SPZ_CHECK_LAUNCH("collapse_meas_kernel");
  return SPZ_OK;
}

int measure_qubit(spz_state_t h, uint32_t target, int reset, int forced, double u, uint8_t* outcome,
                  double* prob0_out) {
  if (target >= h->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "target qubit out of range");
  if (forced < -1 || forced > 1) return fail(SPZ_ERR_INVALID_ARGUMENT, "forced must be -1, 0 or 1");
  double prob0;
  int rc = prob0_device(h, target, &prob0);
  if (rc) return rc;
  const uint8_t val = forced >= 0 ? (uint8_t)forced : (uint8_t)(u < 1.0 - prob0 ? 1 : 0);
  double scale;
  if (val == 0) {
    scale = 1.0 / std::sqrt(prob0);
  } else {
    const double prob1 = 1.0 - prob0;
    scale = 1.0 / std::sqrt(prob1);
  }
  rc = collapse_device(h, target, val, scale);
  if (rc) return rc;
  if (val == 1 && reset) {  // measurement.rs:87-89
    spz_gate x{};
    x.kind = SPZ_GATE_X;
    GateApp a;
    rc = make_gate_app(h->n, x, target, 0, 0, &a);
    if (!rc) rc = launch_gate(h, a);
    if (rc) return rc;
  }
  if (outcome) *outcome = val;
  if (prob0_out) *prob0_out = prob0;
  return SPZ_OK;
}

// ------------------------------------------------------------ Pauli sums
// Diagonal terms (x_mask == 0): sum_x |psi_x|^2 D(x), D(x) = sum_k c_k (-1)^popc(x & z_k).
struct DiagTerms {
  int nterms;
  double coeff[64];
  uint64_t zmask[64];
};

__global__ void __launch_bounds__(kRedThreads) diag_pauli_kernel(const double* __restrict__ re,
                                                                 const double* __restrict__ im, uint64_t N,
                                                                 DiagTerms T, double* __restrict__ partials) {
  __shared__ double smem[32];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  double acc = 0.0;
  for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < N; x += stride) {
    const double a = re[x], b = im[x];
    const double p = dfma(a, a, dmul(b, b));
    double dsum = 0.0;
    for (int k = 0; k < T.nterms; ++k) {
      const double ck = (__popcll(x & T.zmask[k]) & 1) ? dneg(T.coeff[k]) : T.coeff[k];
      dsum = dadd(dsum, ck);
    }
    acc = dfma(p, dsum, acc);
  }
  const double s = block_sum(acc, smem);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// Terms sharing one x_mask != 0.  Pairs (x, y = x ^ xmask) with x's lowest
// x_mask bit 0; w = conj(psi_x) psi_y.  For ny = popc(x_mask & z_mask):
// even ny: term = i^ny (s_y + s_x) Re w; odd ny: term = -i^(ny-1) (s_y - s_x) Im w,
// with s_x = (-1)^popc(x & z_mask).
struct XTerms {
  int nterms;
  uint64_t xmask;
  int lowbit;
  double coeff[64];
  uint64_t zmask[64];
  int ny[64];
};

__global__ void __launch_bounds__(kRedThreads) x_pauli_kernel(const double* __restrict__ re,
                                                              const double* __restrict__ im, uint64_t nwork,
                                                              XTerms T, double* __restrict__ partials) {
  __shared__ double smem[32];
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t lowmask = (1ull << T.lowbit) - 1;
  double acc = 0.0;
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < nwork; w += stride) {
    const uint64_t x = ((w & ~lowmask) << 1) | (w & lowmask);
    const uint64_t y = x ^ T.xmask;
    const double a = re[x], b = im[x], c = re[y], d = im[y];
    const double wre = dfma(a, c, dmul(b, d));
    const double wim = dfma(a, d, dmul(dneg(b), c));
    for (int k = 0; k < T.nterms; ++k) {
      const int sx = (__popcll(x & T.zmask[k]) & 1) ? -1 : 1;
      const int sy = (__popcll(y & T.zmask[k]) & 1) ? -1 : 1;
      const int ny = T.ny[k] & 3;
      double v;
      if ((ny & 1) == 0) {
        const int f = (sx + sy) * (ny == 0 ? 1 : -1);  // i^0 = 1, i^2 = -1
        v = f == 0 ? 0.0 : (f > 0 ? (f == 2 ? dmul(2.0, wre) : wre) : (f == -2 ? dmul(-2.0, wre) : dneg(wre)));
      } else {
        const int f = (sy - sx) * (ny == 1 ? -1 : 1);  // Re(i (...)) = -Im, Re(-i (...)) = +Im
        v = f == 0 ? 0.0 : (f > 0 ? dmul(2.0, wim) : dmul(-2.0, wim));
      }
      acc = dfma(T.coeff[k], v, acc);
    }
  }
  const double s = block_sum(acc, smem);
  if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// ------------------------------------------------ fused Pauli-sum tile passes
// One pass loads a tile of 2^k amplitudes (all values of k local qubits) into
// shared memory and accumulates, per thread:
//  * (first pass only) the diagonal terms: with w_k = parity(x & z_k), the
//    diagonal part is D(x) = C + sum_j T_j[w bits 8j..8j+7], T_j 256-entry tables
//    of -2 sum c_k over the set bits, so a whole Ising-type chain costs a few
//    FP64 operations per amplitude; energy += |psi_x|^2 D(x);
//  * every X/Y-type term whose X-mask lies in the tile: per pair (x, x ^ xmask)
//    the pair's contribution to Re<psi|P|psi>, one accumulator per term.
// Each term's accumulators are reduced once at the end (fixed order).
constexpr int kPtMaxTerms = 16;   // X-type terms per pass
constexpr int kPtMaxDiag = 64;    // diagonal terms (8 chunks of 8)
constexpr int kPtK = 12, kPtLow = 3, kPtThreads = 512;

struct PtTerm {
  uint32_t xl;      // X-mask in local bits
  int32_t lowbit;   // lowest bit of xl
  uint64_t z;       // Z-mask (qubits)
  int32_t ny;       // Y count
  int32_t simple;   // pure X string (z = 0, ny = 0): 2 Re w
};

struct PtArgs {
  const double* re;
  const double* im;
  uint64_t ntiles;
  int k, c, nhigh;
  uint8_t lpos[kPtK];
  int ndiag;                 // diagonal terms handled in this pass (0 or all)
  uint64_t dz[kPtMaxDiag];   // their Z-masks
  const double* dtab;        // nchunks x 256 table entries
  // The chunk index w(x) = sum_j parity(x & dz_j) << j is linear over GF(2):
  // w(base | e) = w(base) ^ L0[e & 63] ^ L1[e >> 6] for the tile offset e.
  uint8_t lz[kPtMaxDiag / 8][2][64];
  double dconst;             // C = sum of the diagonal coefficients
  int nt;
  PtTerm t[kPtMaxTerms];
  double* partials;          // (nt + 1) x gridDim.x
};

__global__ void __launch_bounds__(kPtThreads) pauli_tile_kernel(PtArgs A) {
  extern __shared__ double sm[];
  const uint32_t T = 1u << A.k;
  double* sre = sm;
  double* sim = sm + T;
  uint64_t* rowoff = reinterpret_cast<uint64_t*>(sm + 2 * T);
  double* red = sm + 2 * T + (T >> kPtLow) + 1;
  const uint32_t cmask = (1u << A.c) - 1;
  for (uint32_t r = threadIdx.x; r < (1u << A.nhigh); r += blockDim.x) {
    uint64_t off = 0;
    for (int j = 0; j < A.nhigh; ++j)
      if ((r >> j) & 1) off |= 1ull << A.lpos[A.c + j];
    rowoff[r] = off;
  }
  const int nch = (A.ndiag + 7) / 8;
  double* stab = red + 32;                                          // nch x 256 chunk tables
  uint8_t* slz = reinterpret_cast<uint8_t*>(stab + (size_t)nch * 256);  // nch x 2 x 64
  for (int j = threadIdx.x; j < nch * 256; j += blockDim.x) stab[j] = A.dtab[j];
  for (int j = threadIdx.x; j < nch * 128; j += blockDim.x) slz[j] = (&A.lz[0][0][0])[j];
  double acc[kPtMaxTerms + 1];
#pragma unroll
  for (int j = 0; j <= kPtMaxTerms; ++j) acc[j] = 0.0;
  __syncthreads();
  for (uint64_t tile = blockIdx.x; tile < A.ntiles; tile += gridDim.x) {
    const uint64_t base = deposit(tile, A.lpos, A.k);
    for (uint32_t e2 = threadIdx.x; e2 < T / 2; e2 += blockDim.x) {
      const uint32_t e = 2 * e2;
      const uint64_t gi = base | rowoff[e >> A.c] | (e & cmask);
      *reinterpret_cast<double2*>(sre + e) = *reinterpret_cast<const double2*>(A.re + gi);
      *reinterpret_cast<double2*>(sim + e) = *reinterpret_cast<const double2*>(A.im + gi);
    }
    __syncthreads();
    if (A.ndiag) {
      uint32_t wb[kPtMaxDiag / 8];  // the tile base's part of each chunk index
#pragma unroll
      for (int ch = 0; ch < kPtMaxDiag / 8; ++ch) {
        wb[ch] = 0;
        if (ch < nch) {
          const int jn = min(8, A.ndiag - ch * 8);
          for (int j = 0; j < jn; ++j) wb[ch] |= (uint32_t)(__popcll(base & A.dz[ch * 8 + j]) & 1) << j;
        }
      }
      for (uint32_t e = threadIdx.x; e < T; e += blockDim.x) {
        double d = A.dconst;
        const uint32_t e0 = e & 63, e1 = (e >> 6) & 63;
#pragma unroll
        for (int ch = 0; ch < kPtMaxDiag / 8; ++ch) {
          if (ch >= nch) break;
          const uint32_t w = wb[ch] ^ slz[ch * 128 + e0] ^ slz[ch * 128 + 64 + e1];
          d = dadd(d, stab[ch * 256 + w]);
        }
        const double a = sre[e], b = sim[e];
        acc[kPtMaxTerms] = dfma(dfma(a, a, dmul(b, b)), d, acc[kPtMaxTerms]);
      }
    }
#pragma unroll
    for (int t = 0; t < kPtMaxTerms; ++t) {
      if (t >= A.nt) break;
      const PtTerm P = A.t[t];
      const uint32_t lowmask = (1u << P.lowbit) - 1;
      for (uint32_t m = threadIdx.x; m < T / 2; m += blockDim.x) {
        const uint32_t x = ((m & ~lowmask) << 1) | (m & lowmask);
        const uint32_t y = x ^ P.xl;
        const double a = sre[x], b = sim[x], c = sre[y], d = sim[y];
        if (P.simple) {  // 2 Re(conj(psi_x) psi_y); the factor 2 is applied at the end
          acc[t] = dfma(a, c, acc[t]);
          acc[t] = dfma(b, d, acc[t]);
        } else {
          const uint64_t gx = base | rowoff[x >> A.c] | (x & cmask);
          const uint64_t gy = base | rowoff[y >> A.c] | (y & cmask);
          const int sx = (__popcll(gx & P.z) & 1) ? -1 : 1;
          const int sy = (__popcll(gy & P.z) & 1) ? -1 : 1;
          const int ny = P.ny & 3;
          const double wre = dfma(a, c, dmul(b, d)), wim = dfma(a, d, dmul(dneg(b), c));
          int f;
          double v;
          if ((ny & 1) == 0) {
            f = (sx + sy) * (ny == 0 ? 1 : -1);
            v = wre;
          } else {
            f = (sy - sx) * (ny == 1 ? -1 : 1);
            v = wim;
          }
          // half of f * v (f is -2, 0 or 2): the factor 2 is applied at the end
          if (f > 0) acc[t] = dadd(acc[t], v);
          else if (f < 0) acc[t] = dsub(acc[t], v);
        }
      }
    }
    __syncthreads();
  }
  // one fixed-order block reduction per accumulator; row t < nt: term t, row nt: diagonal
#pragma unroll
  for (int s = 0; s <= kPtMaxTerms; ++s) {
    if (s < kPtMaxTerms && s >= A.nt) continue;
    const int row = s == kPtMaxTerms ? A.nt : s;
    double v = acc[s];
    for (int off = 16; off > 0; off >>= 1) v = dadd(v, __shfl_down_sync(0xffffffffu, v, off));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
      double r = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
      for (int off = 16; off > 0; off >>= 1) r = dadd(r, __shfl_down_sync(0xffffffffu, r, off));
      if (lane == 0) A.partials[(size_t)row * gridDim.x + blockIdx.x] = r;
    }
    __syncthreads();
  }
}

// Tile-pass evaluation; returns false (nothing launched) when the terms do not
// fit its limits, so the caller uses the per-group kernels.
static int pauli_tiles(spz_state_t h, const spz_pauli_term* terms, size_t nterms, double* out, bool* done) {
  *done = false;
  const uint32_t n = h->n;
  const int k = std::min<int>((int)n, kPtK);
  const int c = std::min<int>(kPtLow, k);
  std::vector<size_t> diag, xt;
  for (size_t i = 0; i < nterms; ++i) (terms[i].x_mask ? xt : diag).push_back(i);
  if (diag.size() > (size_t)kPtMaxDiag) return SPZ_OK;
  for (size_t i : xt)
    if (__builtin_popcountll(terms[i].x_mask) > k - c) return SPZ_OK;
  // passes: greedy local sets covering the X-masks
  struct Pass { std::vector<int> local; std::vector<size_t> terms; bool diag; };
  std::vector<Pass> passes;
  std::vector<int> done_t(xt.size(), 0);
  size_t left = xt.size();
  bool first = true;
  while (left > 0 || first) {
    uint64_t L = (1ull << c) - 1;
    int nl = c;
    Pass P;
    P.diag = first && !diag.empty();
    for (size_t j = 0; j < xt.size() && (int)P.terms.size() < kPtMaxTerms; ++j) {
      if (done_t[j]) continue;
      const uint64_t need = terms[xt[j]].x_mask & ~L;
      const int add = __builtin_popcountll(need);
      if (nl + add <= k) {
        L |= need;
        nl += add;
        P.terms.push_back(xt[j]);
        done_t[j] = 1;
        left--;
      }
    }
    for (int q = 0; q < (int)n && nl < k; ++q)
      if (!((L >> q) & 1)) { L |= 1ull << q; nl++; }
    for (int q = 0; q < (int)n; ++q)
      if ((L >> q) & 1) P.local.push_back(q);
    first = false;
    if (P.diag || !P.terms.empty()) passes.push_back(std::move(P));
    if (left == 0) break;
  }
  // diagonal tables
  const size_t nd = diag.size();
  const size_t nchunks = (nd + 7) / 8;
  std::vector<double> tab(std::max<size_t>(1, nchunks) * 256, 0.0);
  double dconst = 0.0;
  for (size_t j = 0; j < nd; ++j) dconst += terms[diag[j]].coeff;
  for (size_t ch = 0; ch < nchunks; ++ch)
    for (int v = 0; v < 256; ++v) {
      double s = 0.0;
      for (int b = 0; b < 8 && ch * 8 + b < nd; ++b)
        if ((v >> b) & 1) s += -2.0 * terms[diag[ch * 8 + b]].coeff;
      tab[ch * 256 + v] = s;
    }
  const int blocks = (int)std::min<uint64_t>(1ull << (n - k), (uint64_t)kNumSMs * 3);
  const size_t slots_per_pass = (size_t)(kPtMaxTerms + 1) * blocks;
  const size_t nres = passes.size() * (kPtMaxTerms + 1);
  void* scratch;
  int rc = ensure_dev_scratch(h, (tab.size() + passes.size() * slots_per_pass + nres) * sizeof(double), &scratch);
  if (rc) return rc;
  double* dtab = (double*)scratch;
  double* dpart = dtab + tab.size();
  double* dres = dpart + passes.size() * slots_per_pass;
  SPZ_CUDA(cudaMemcpyAsync(dtab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  {  // the shared-memory opt-in, once per device (a per-device kernel attribute)
    static std::mutex attr_mu;
    static bool attr[kMaxDevices] = {};
    if (h->device < 0 || h->device >= kMaxDevices) return fail(SPZ_ERR_INVALID_ARGUMENT, "device index out of range");
    std::lock_guard<std::mutex> lock(attr_mu);
    if (!attr[h->device]) {
      SPZ_CUDA(cudaFuncSetAttribute(pauli_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)((2 << kPtK) + (1 << (kPtK - kPtLow)) + 64 + (kPtMaxDiag / 8) * (256 + 16)) * 8));
      attr[h->device] = true;
    }
  }
  for (size_t p = 0; p < passes.size(); ++p) {
    const Pass& P = passes[p];
    PtArgs A{};
    A.re = h->re;
    A.im = h->im;
    A.k = (int)P.local.size();
    A.c = c;
    A.nhigh = A.k - c;
    for (int j = 0; j < A.k; ++j) A.lpos[j] = (uint8_t)P.local[j];
    A.ntiles = 1ull << (n - A.k);
    int where[64];
    for (int q = 0; q < 64; ++q) where[q] = -1;
    for (size_t j = 0; j < P.local.size(); ++j) where[P.local[j]] = (int)j;
    if (P.diag) {
      A.ndiag = (int)nd;
      for (size_t j = 0; j < nd; ++j) A.dz[j] = terms[diag[j]].z_mask;
      A.dtab = dtab;
      A.dconst = dconst;
      // column of tile-offset bit b in chunk ch: the chunk's terms whose Z-mask
      // holds the local qubit lpos[b]
      for (int ch = 0; ch < (int)((nd + 7) / 8); ++ch) {
        uint32_t col[12] = {};
        const int jn = std::min<int>(8, (int)nd - ch * 8);
        for (int b = 0; b < A.k && b < 12; ++b)
          for (int j = 0; j < jn; ++j) col[b] |= (uint32_t)((A.dz[ch * 8 + j] >> A.lpos[b]) & 1) << j;
        for (int v = 0; v < 64; ++v) {
          uint32_t w0 = 0, w1 = 0;
          for (int b = 0; b < 6; ++b) {
            if ((v >> b) & 1) {
              w0 ^= col[b];
              w1 ^= col[b + 6];
            }
          }
          A.lz[ch][0][v] = (uint8_t)w0;
          A.lz[ch][1][v] = (uint8_t)w1;
        }
      }
    }
    A.nt = (int)P.terms.size();
    for (int t = 0; t < A.nt; ++t) {
      const spz_pauli_term& tm = terms[P.terms[t]];
      PtTerm& pt = A.t[t];
      for (int q = 0; q < 64; ++q)
        if ((tm.x_mask >> q) & 1) pt.xl |= 1u << where[q];
      pt.lowbit = __builtin_ctz(pt.xl);
      pt.z = tm.z_mask;
      pt.ny = __builtin_popcountll(tm.x_mask & tm.z_mask);
      pt.simple = tm.z_mask == 0;
    }
    A.partials = dpart + p * slots_per_pass;
    const uint32_t T = 1u << A.k;
    const size_t nch = P.diag ? (nd + 7) / 8 : 0;
    const size_t smem = (2 * T + (T >> kPtLow) + 1 + 32 + nch * 256 + nch * 16) * sizeof(double);
    const int threads = (int)std::min<uint32_t>(kPtThreads, std::max<uint32_t>(32, T / 2));
    const int nb = (int)std::min<uint64_t>(A.ntiles, (uint64_t)blocks);
    pauli_tile_kernel<<<nb, threads, smem, h->stream>>>(A);
    finalize_kernel<<<1, 1024, 0, h->stream>>>(A.partials, nb, A.nt + 1, dres + p * (kPtMaxTerms + 1));
    SPZ_CHECK_LAUNCH("pauli_tile_kernel");
  }
  std::vector<double> res(nres);
  rc = read_back(h, dres, res.data(), nres);
  if (rc) return rc;
  double total = 0.0;
  for (size_t p = 0; p < passes.size(); ++p) {
    const Pass& P = passes[p];
    const double* r = res.data() + p * (kPtMaxTerms + 1);
    for (size_t t = 0; t < P.terms.size(); ++t) total += terms[P.terms[t]].coeff * 2.0 * r[t];
    if (P.diag) total += r[P.terms.size()];
  }
  *out = total;
  *done = true;
  return SPZ_OK;
}

int pauli_expectation(spz_state_t h, const spz_pauli_term* terms, size_t nterms, double* out) {
  if (nterms && !terms) return fail(SPZ_ERR_NULL, "terms is NULL");
  for (size_t k = 0; k < nterms; ++k)
    if (h->n < 64 && ((terms[k].x_mask | terms[k].z_mask) >> h->n) != 0)
      return fail(SPZ_ERR_INVALID_ARGUMENT, "Pauli term acts on a qubit out of range");
  if (nterms == 0) {
    *out = 0.0;
    return SPZ_OK;
  }
  bool done = false;
  int rc0 = pauli_tiles(h, terms, nterms, out, &done);
  if (rc0 || done) return rc0;
  // Fallback: diagonal terms, then one pass per distinct x_mask (chunks of 64 terms).
  std::vector<std::vector<size_t>> groups;
  std::vector<uint64_t> group_x;
  for (size_t k = 0; k < nterms; ++k) {
    size_t g = 0;
    for (; g < groups.size(); ++g)
      if (group_x[g] == terms[k].x_mask && groups[g].size() < 64) break;
    if (g == groups.size()) {
      groups.emplace_back();
      group_x.push_back(terms[k].x_mask);
    }
    groups[g].push_back(k);
  }
  void* scratch;
  const size_t ng = groups.size();
  int rc = ensure_dev_scratch(h, ((ng + 1) * kMaxRedBlocks + ng + 8) * sizeof(double), &scratch);
  if (rc) return rc;
  double* partials = (double*)scratch;
  double* slots = partials + (ng + 1) * kMaxRedBlocks;
  for (size_t g = 0; g < ng; ++g) {
    double* part = partials + g * kMaxRedBlocks;
    if (group_x[g] == 0) {
      DiagTerms T{};
      T.nterms = (int)groups[g].size();
      for (int j = 0; j < T.nterms; ++j) {
        T.coeff[j] = terms[groups[g][j]].coeff;
        T.zmask[j] = terms[groups[g][j]].z_mask;
      }
      const int blocks = std::min<int>(grid_for(h->N, kRedThreads, 8), kMaxRedBlocks);
      diag_pauli_kernel<<<blocks, kRedThreads, 0, h->stream>>>(h->re, h->im, h->N, T, part);
      finalize_kernel<<<1, 1024, 0, h->stream>>>(part, blocks, 1, slots + g);
    } else {
      XTerms T{};
      T.nterms = (int)groups[g].size();
      T.xmask = group_x[g];
      T.lowbit = __builtin_ctzll(group_x[g]);
      for (int j = 0; j < T.nterms; ++j) {
        const spz_pauli_term& tm = terms[groups[g][j]];
        T.coeff[j] = tm.coeff;
        T.zmask[j] = tm.z_mask;
        T.ny[j] = __builtin_popcountll(tm.x_mask & tm.z_mask);
      }
      const uint64_t nwork = h->N / 2;
      const int blocks = std::min<int>(grid_for(nwork, kRedThreads, 8), kMaxRedBlocks);
      x_pauli_kernel<<<blocks, kRedThreads, 0, h->stream>>>(h->re, h->im, nwork, T, part);
      finalize_kernel<<<1, 1024, 0, h->stream>>>(part, blocks, 1, slots + g);
    }
    SPZ_CHECK_LAUNCH("pauli kernel");
  }
  std::vector<double> vals(ng);
  if (ng) {
    rc = read_back(h, slots, vals.data(), ng);
    if (rc) return rc;
  }
  double total = 0.0;
  for (size_t g = 0; g < ng; ++g) total += vals[g];
  *out = total;
  return SPZ_OK;
}

// ------------------------------------------------------------ sampling
// Fixed blocked cumulative order (bit-identical to the oracle's restatement):
// p_i = re*re + im*im; sub-chunks of 32 amplitudes, chunks of 8 sub-chunks,
// super-chunks of 1024 chunks; every total is a sequential sum of the level
// below; bases are exclusive sequential scans; per shot: target = u * total,
// the first chunk whose end exceeds it, then inside the chunk the first
// sub-chunk whose running end exceeds it, then the first element.  A shot
// walks at most 8 sub-totals and 32 elements (instead of up to 256 elements).
constexpr uint64_t kSub = 32, kChunk = 256, kSuper = 1024;

__device__ __forceinline__ double prob_exact(const double* re, const double* im, uint64_t i) {
  const double r = re[i], m = im[i];
  return dadd(dmul(r, r), dmul(m, m));
}

// One warp covers 32 chunks; data is staged through shared memory 32
// amplitudes of each chunk at a time (coalesced loads), so each lane folds one
// sub-chunk per step: its sub-total, then the chunk total from the sub-totals.
__global__ void __launch_bounds__(128) chunk_total_kernel(const double* __restrict__ re,
                                                          const double* __restrict__ im, uint64_t nchunks,
                                                          uint64_t cs, uint64_t ss, double* __restrict__ totals,
                                                          double* __restrict__ subs) {
  __shared__ double tile[4][32][33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t warps_total = (uint64_t)gridDim.x * 4;
  const uint64_t ns = cs / ss;
  for (uint64_t c0 = ((uint64_t)blockIdx.x * 4 + warp) * 32; c0 < nchunks; c0 += warps_total * 32) {
    double t = 0.0;
    for (uint64_t j0 = 0; j0 < cs; j0 += ss) {
      for (int i = 0; i < 32; ++i) {
        const uint64_t c = c0 + i;
        if (c < nchunks && (uint64_t)lane < ss) tile[warp][i][lane] = prob_exact(re, im, c * cs + j0 + lane);
      }
      __syncwarp();
      if (c0 + lane < nchunks) {
        double u = 0.0;
        for (uint64_t j = 0; j < ss; ++j) u = dadd(u, tile[warp][lane][j]);
        subs[(c0 + lane) * ns + j0 / ss] = u;
        t = dadd(t, u);
      }
      __syncwarp();
    }
    if (c0 + lane < nchunks) totals[c0 + lane] = t;
  }
}

// One thread per super-chunk: super total (sequential) .
__global__ void super_total_kernel(const double* __restrict__ ct, uint64_t nchunks, uint64_t nsuper,
                                   double* __restrict__ st) {
  const uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (s >= nsuper) return;
  double t = 0.0;
  const uint64_t end = (s + 1) * kSuper < nchunks ? (s + 1) * kSuper : nchunks;
  for (uint64_t c = s * kSuper; c < end; ++c) t = dadd(t, ct[c]);
  st[s] = t;
}

// Single thread: super bases (exclusive sequential scan) and the total.
__global__ void super_base_kernel(const double* __restrict__ st, uint64_t nsuper, double* __restrict__ sb,
                                  double* __restrict__ total) {
  double b = 0.0;
  for (uint64_t s = 0; s < nsuper; ++s) {
    sb[s] = b;
    b = dadd(b, st[s]);
  }
  *total = b;
}

// One thread per super-chunk: chunk bases and chunk ends.
__global__ void chunk_base_kernel(const double* __restrict__ ct, const double* __restrict__ sb,
                                  const double* __restrict__ total, uint64_t nchunks, uint64_t nsuper,
                                  double* __restrict__ cb, double* __restrict__ ce) {
  const uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (s >= nsuper) return;
  double pre = 0.0;
  const uint64_t end = (s + 1) * kSuper < nchunks ? (s + 1) * kSuper : nchunks;
  for (uint64_t c = s * kSuper; c < end; ++c) {
    const double base = dadd(sb[s], pre);
    cb[c] = base;
    if (c > 0) ce[c - 1] = base;
    pre = dadd(pre, ct[c]);
  }
  if (end == nchunks) ce[nchunks - 1] = *total;
}

__global__ void sample_kernel(const double* __restrict__ re, const double* __restrict__ im, uint64_t nchunks,
                              uint64_t cs, uint64_t ss, const double* __restrict__ subs,
                              const double* __restrict__ cb, const double* __restrict__ ce,
                              const double* __restrict__ total_p, const double* __restrict__ u, uint64_t nshots,
                              uint64_t* __restrict__ out) {
  const uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (k >= nshots) return;
  const double total = *total_p;
  double target = dmul(u[k], total);
  if (target >= total) target = nextafter(total, 0.0);
  uint64_t lo = 0, hi = nchunks - 1;
  while (lo < hi) {
    const uint64_t mid = lo + (hi - lo) / 2;
    if (ce[mid] > target) hi = mid; else lo = mid + 1;
  }
  const uint64_t c = lo, ns = cs / ss;
  double r = cb[c];
  uint64_t kk = ns;
  for (uint64_t q = 0; q < ns; ++q) {
    const double rn = dadd(r, subs[c * ns + q]);
    if (rn > target) {
      kk = q;
      break;
    }
    r = rn;
  }
  uint64_t outcome = ~0ull;
  if (kk < ns) {
    uint64_t last_pos = ~0ull;
    for (uint64_t j = 0; j < ss; ++j) {
      const uint64_t i = c * cs + kk * ss + j;
      const double pj = prob_exact(re, im, i);
      if (pj > 0.0) last_pos = i;
      r = dadd(r, pj);
      if (r > target) {
        outcome = i;
        break;
      }
    }
    if (outcome == ~0ull) outcome = last_pos;
  }
  if (outcome == ~0ull) {  // the last index of the chunk with p > 0, or its first
    outcome = c * cs;
    for (uint64_t j = cs; j-- > 0;)
      if (prob_exact(re, im, c * cs + j) > 0.0) {
        outcome = c * cs + j;
        break;
      }
  }
  out[k] = outcome;
}

int sample(spz_state_t h, const double* u, size_t nshots, uint64_t* out) {
  if (!u || !out) return fail(SPZ_ERR_NULL, "NULL argument");
  if (nshots == 0) return SPZ_OK;
  const uint64_t cs = std::min<uint64_t>(h->N, kChunk);
  const uint64_t ss = std::min<uint64_t>(cs, kSub);
  const uint64_t nchunks = h->N / cs;
  const uint64_t nsuper = (nchunks + kSuper - 1) / kSuper;
  // scratch: subs[N/ss] ct[nchunks] cb[nchunks] ce[nchunks] st[nsuper] sb[nsuper] total[1] u[nshots] out[nshots]
  const size_t doubles = h->N / ss + 3 * nchunks + 2 * nsuper + 8 + 2 * nshots;
  void* scratch;
  int rc = ensure_dev_scratch(h, doubles * sizeof(double), &scratch);
  if (rc) return rc;
  double* subs = (double*)scratch;
  double* ct = subs + h->N / ss;
  double* cb = ct + nchunks;
  double* ce = cb + nchunks;
  double* st = ce + nchunks;
  double* sb = st + nsuper;
  double* total = sb + nsuper;
  double* du = total + 8;
  uint64_t* dout = (uint64_t*)(du + nshots);
  SPZ_CUDA(cudaMemcpyAsync(du, u, nshots * sizeof(double), copy_kind(u, true), h->stream));
  const int cblocks = (int)std::min<uint64_t>((nchunks + 127) / 128, (uint64_t)kNumSMs * 16);
  chunk_total_kernel<<<cblocks, 128, 0, h->stream>>>(h->re, h->im, nchunks, cs, ss, ct, subs);
  super_total_kernel<<<(unsigned)((nsuper + 127) / 128), 128, 0, h->stream>>>(ct, nchunks, nsuper, st);
  super_base_kernel<<<1, 1, 0, h->stream>>>(st, nsuper, sb, total);
  chunk_base_kernel<<<(unsigned)((nsuper + 127) / 128), 128, 0, h->stream>>>(ct, sb, total, nchunks, nsuper, cb, ce);
  sample_kernel<<<(unsigned)((nshots + 255) / 256), 256, 0, h->stream>>>(h->re, h->im, nchunks, cs, ss, subs, cb,
                                                                         ce, total, du, nshots, dout);
  SPZ_CHECK_LAUNCH("sampling kernels");
  double host_total;
  rc = read_back(h, total, &host_total, 1);
  if (rc) return rc;
  if (!(host_total > 0.0)) return fail(SPZ_ERR_INVALID_ARGUMENT, "state has zero norm");
  SPZ_CUDA(cudaMemcpyAsync(out, dout, nshots * sizeof(uint64_t), copy_kind(out, false), h->stream));
  SPZ_CUDA(cudaStreamSynchronize(h->stream));
  return SPZ_OK;
}

}  // namespace spz

using namespace spz;

extern "C" {

int spz_prob0(spz_state_t h, uint32_t target, double* prob0) {
  if (!h || !prob0) return fail(SPZ_ERR_NULL, "NULL argument");
  if (int rc0 = settle(h)) return rc0;
  if (target >= h->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "target qubit out of range");
  return prob0_device(h, target, prob0);
}

int spz_measure_qubit(spz_state_t h, uint32_t target, int reset, int forced, double u, uint8_t* outcome,
                      double* prob0) {
  if (!h || !outcome) return fail(SPZ_ERR_NULL, "NULL argument");
  if (int rc0 = settle(h)) return rc0;
  return measure_qubit(h, target, reset, forced, u, outcome, prob0);
}

int spz_qubit_expectation_value(spz_state_t h, uint32_t target, double* out) {
  if (!h || !out) return fail(SPZ_ERR_NULL, "NULL argument");
  if (int rc0 = settle(h)) return rc0;
  if (target >= h->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "target qubit out of range");
  double p0;
  int rc = prob0_device(h, target, &p0);
  if (rc) return rc;
  *out = 2.0 * p0 - 1.0;  // core.rs:217
  return SPZ_OK;
}

int spz_xyz_expectation_value(spz_state_t h, char observable, const uint32_t* targets, uint32_t ntargets,
                              double* out) {
  if (!h || (ntargets && (!targets || !out))) return fail(SPZ_ERR_NULL, "NULL argument");
  if (int rc0 = settle(h)) return rc0;
  int mode;
  switch (observable) {
    case 'x': mode = RED_X; break;
    case 'y': mode = RED_Y; break;
    case 'z': mode = RED_Z; break;
    default: return fail(SPZ_ERR_INVALID_ARGUMENT, "observable must be 'x', 'y' or 'z' (core.rs:223-225)");
  }
  for (uint32_t i = 0; i < ntargets; ++i)
    if (targets[i] >= h->n) return fail(SPZ_ERR_INVALID_ARGUMENT, "target qubit out of range");
  for (uint32_t i = 0; i < ntargets; ++i) {
    int rc = reduce_scalar(h, mode, (int)targets[i], &out[i]);
    if (rc) return rc;
  }
  return SPZ_OK;
}

int spz_pauli_expectation(spz_state_t h, const spz_pauli_term* terms, size_t nterms, double* out) {
  if (!h || !out) return fail(SPZ_ERR_NULL, "NULL argument");
  if (int rc0 = settle(h)) return rc0;
  return pauli_expectation(h, terms, nterms, out);
}

int spz_norm_sqr(spz_state_t h, double* out) {
  if (!h || !out) return fail(SPZ_ERR_NULL, "NULL argument");
  if (int rc0 = settle(h)) return rc0;
  return reduce_scalar(h, RED_NORM, 0, out);
}

int spz_sample(spz_state_t h, const double* u, size_t nshots, uint64_t* out) {
  if (!h) return fail(SPZ_ERR_NULL, "handle is NULL");
  if (int rc0 = settle(h)) return rc0;
  return sample(h, u, nshots, out);
}

}  // extern "C"
