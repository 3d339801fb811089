// The fused executor's tile geometry and gate descriptor, shared by the
// circuit executor (circuit.cu) and the fused adjoint sweep (adjoint.cu).
#pragma once

#include <vector>

#include "common.cuh"

namespace spz {

#ifndef SPZ_TILE_K
#define SPZ_TILE_K 10
#endif
constexpr int kTileMaxK = SPZ_TILE_K;  // 2^10 amplitudes x 16 B = 16 KiB of shared memory
constexpr int kTileLowBits = 3;   // qubits 0..2 always local: 64-byte contiguous rows
// Small blocks, many of them: every op in a pass ends with a block barrier, so
// the FP64 pipe stays busier with many independent small blocks per SM than
// with a few large ones.  Measured on the 30-qubit brickwork, fast mode, share
// of the DFMA issue rate: 2^12 tiles x 256 threads x 3 blocks 0.81; 2^11 x 128
// x 6 0.84; 2^10 x 64 x 12 0.86 (exact mode 0.86-0.87 for all three).  With
// 32-bit row offsets a block needs 16.5 KiB (+1 KiB the runtime reserves), so
// 13 fit an SM's 228 KiB; 13 against 12 measured the same on the 30-qubit
// brickwork (fast 4,472 / 4,476 ms, exact 8,360 / 8,355 ms per step).
#ifndef SPZ_TILE_THREADS
#define SPZ_TILE_THREADS 64
#endif
#ifndef SPZ_TILE_MIN_BLOCKS
#define SPZ_TILE_MIN_BLOCKS 13  // 13 x (16 KiB tile + 0.5 KiB row table + 1 KiB reserved) <= 228 KiB
#endif
constexpr int kTileThreads = SPZ_TILE_THREADS;

enum TileMode { TM_PAIR = 0, TM_DIAG_LOCAL = 1, TM_DIAG_GLOBAL = 2, TM_SWAP = 3, TM_PHASE = 4, TM_LAZY2 = 5 };

struct TileGate {
  int32_t kind;
  int32_t mode;
  uint32_t tbit;    // local bit of the target (SWAP: first qubit)
  uint32_t tbit2;   // SWAP: local bit of the second qubit
  uint32_t l_ones;  // local bits that must be 1 (controls; plus the target for Z/P on s1)
  int32_t npos;     // number of local positions inserted by the enumeration
  uint8_t pos[16];  // sorted local bit positions inserted as zeros
  uint64_t g_ones;  // non-local bits the tile base must have set
  uint64_t g_zeros; // non-local bits the tile base must have clear
  uint64_t g_tbit;  // TM_DIAG_GLOBAL: the non-local target bit
  Coef c;
  // TM_PHASE: amplitude x (with x & half_bit, if half_bit != 0) is multiplied by
  // table[sum_j parity(x & pmask[j]) << j] (complex, ptab .. ptab + 2^pm - 1).
  uint64_t half_bit;
  uint64_t pmask[kPhaseMaxTerms];  // parity masks over the global index
  uint32_t pemask[kPhaseMaxTerms]; // their local part, as bits of the tile offset e
  int32_t pm;
  uint32_t ptab;
  int32_t cond;  // >= 0: applies only if that qubit's device-side measurement read 1
  uint32_t e_mask;  // pos[0 .. npos - 1] as a bit mask of the tile offset
  // TM_LAZY2 (fast mode): two lazy rotations with phase entries, `kind` on
  // tbit (coefficient c.cs) then `kind2` on tbit2 (c.sn), fused over blocks
  // of four amplitudes.  pmask / pemask [0 .. pm1) are the first op's phase
  // masks, [pm1 .. pm) the second's; the table holds three entries per index
  // (w1, w2, w1' w2), w1' being the first op's entry with its masks' tbit2
  // parities flipped.
  int32_t kind2;
  int32_t pm1;
  // SPZ_EXEC_SHUFFLE: > this gate's index, the end of a run of gates that the
  // block applies with warp shuffles (circuit.cu, tile_run_shfl); 0 otherwise.
  int32_t run_end;
};

// The descriptor of gate g inside a tile pass whose local qubits are `local`
// (sorted); not for fast-mode phase ops.
TileGate make_tile_gate(const GateApp& g, const std::vector<int>& local);

}  // namespace spz
