/*
 * spinoza_gb300 — C ABI of the GB300-native FP64 state-vector engine.
 *
 * This is the drop-in boundary for Spinoza's gate-application path
 * (QuState/spinoza v0.5.1).  Every entry point replaces one function of the
 * reference's public Rust API; the citation above each declaration gives the
 * reference file:line (paths relative to the reference repository).
 *
 * Conventions
 *   - The state lives in HBM as two FP64 arrays (SoA): reals[2^n], imags[2^n],
 *     exactly the layout of `State { reals, imags, n }` (spinoza/src/core.rs:20-27).
 *   - A handle owns (or wraps) the two device arrays and one CUDA stream.  All
 *     work on a handle is issued on that stream; calls on one handle must be
 *     serialised by the caller (the reference borrows `&mut State`).  A handle
 *     belongs to the device that was current when it was created; make that
 *     device current (cudaSetDevice) before calls on it.  Handles on different
 *     devices or threads may be used concurrently.
 *   - Every function returns an int status (SPZ_OK == 0).  Nothing throws across
 *     the ABI.  Where the reference panics (bad qubit index, unsupported gate,
 *     n == 0) this library returns an error code and leaves the state untouched.
 *   - Host pointers passed for bulk data (upload/download, uniforms, outputs) may
 *     be pageable or pinned host memory, or device memory (UVA, cudaMemcpyDefault).
 *   - Random draws are explicit inputs (uniforms in [0,1)), so every result is
 *     reproducible; the reference draws from an unseeded thread_rng.
 */
#ifndef SPINOZA_GB300_H
#define SPINOZA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum spz_status {
  SPZ_OK = 0,
  SPZ_ERR_INVALID_ARGUMENT = 1, /* qubit out of range, duplicate qubits, n == 0, ...   */
  SPZ_ERR_UNSUPPORTED = 2,      /* gate/control combination without a definition      */
  SPZ_ERR_OUT_OF_MEMORY = 3,    /* device or pinned-host allocation failed             */
  SPZ_ERR_CUDA = 4,             /* a CUDA runtime call failed (see spz_last_error)     */
  SPZ_ERR_NULL = 5,             /* a required pointer argument was NULL                */
  SPZ_ERR_TIMEOUT = 6           /* a bounded device-side wait expired                  */
};

/* Human-readable text of the last error raised on the calling thread. */
const char* spz_last_error(void);
/* Library version string ("spinoza_gb300 <semver> sm_103a"). */
const char* spz_version(void);

/* ----------------------------------------------------------------- gates */
/* Gate kinds; same variants and order as `enum Gate` (spinoza/src/gates.rs:45-74). */
enum spz_gate_kind {
  SPZ_GATE_H = 0,
  SPZ_GATE_M = 1,       /* measurement; only valid inside spz_circuit_execute       */
  SPZ_GATE_X = 2,
  SPZ_GATE_Y = 3,
  SPZ_GATE_Z = 4,
  SPZ_GATE_P = 5,       /* p[0] = angle                                             */
  SPZ_GATE_RX = 6,      /* p[0] = angle                                             */
  SPZ_GATE_RY = 7,      /* p[0] = angle                                             */
  SPZ_GATE_RZ = 8,      /* p[0] = angle                                             */
  SPZ_GATE_SWAP = 9,    /* q0, q1 = the two swapped qubits                          */
  SPZ_GATE_U = 10,      /* p[0..2] = theta, phi, lambda                             */
  SPZ_GATE_UNITARY = 11,/* dense unitary: applied by spz_apply_unitary, not as an op */
  SPZ_GATE_BITFLIP = 12 /* p[0] = probability, p[1] = uniform draw: X iff p[1] <= p[0] */
};

/* A gate with its payload, the C form of the Rust `Gate` enum. */
typedef struct spz_gate {
  int32_t kind;  /* enum spz_gate_kind */
  uint32_t q0;   /* SWAP: first qubit  */
  uint32_t q1;   /* SWAP: second qubit */
  uint32_t pad_;
  double p[3];
} spz_gate;

/* ----------------------------------------------------------------- state */
typedef struct spz_state_s* spz_state_t;

/* Largest qubit count a handle accepts (2 x 2^34 x 8 B = 256 GiB of HBM). */
#define SPZ_MAX_QUBITS 34

/* State::new(n): allocate 2 x 2^n FP64 on the current device and set |0...0>.
 * Replaces spinoza/src/core.rs:32-42 (asserts n > 0). */
int spz_state_create(uint32_t n, spz_state_t* out);

/* Wrap caller-owned device arrays (e.g. torch tensors) without copying.  The
 * arrays must hold 2^n doubles each, 16-byte aligned; the caller keeps them
 * alive until spz_state_destroy.  The contents are left as they are. */
int spz_state_wrap(uint32_t n, double* d_reals, double* d_imags, spz_state_t* out);

/* Release the handle (and its arrays when it owns them). */
int spz_state_destroy(spz_state_t h);

/* Issue all later work of this handle on `stream` (a cudaStream_t; NULL = the
 * handle's own stream; pass cudaStreamLegacy for the legacy default stream). */
int spz_state_set_stream(spz_state_t h, void* stream);

/* Wait until all work issued on the handle's stream has finished. */
int spz_state_synchronize(spz_state_t h);

/* n, and the device pointers of the two arrays. */
int spz_state_num_qubits(spz_state_t h, uint32_t* n);
int spz_state_device_arrays(spz_state_t h, double** d_reals, double** d_imags);

/* Copy 2^n reals and imags in (host -> device) / out (device -> host).
 * The Rust State exposes `pub reals, pub imags` (spinoza/src/core.rs:22-24);
 * these two calls are how a caller reads or replaces them. */
int spz_state_upload(spz_state_t h, const double* reals, const double* imags);
int spz_state_download(spz_state_t h, double* reals, double* imags);

/* Reset to |0...0> (the content of State::new). */
int spz_state_reset_zero(spz_state_t h);

/* dst <- src (same n).  Replaces `State: Clone` (spinoza/src/core.rs:18). */
int spz_state_copy(spz_state_t dst, spz_state_t src);

/* Fill with a seeded synthetic state.  dist 0: reals/imags i.i.d. uniform in
 * [-1,1) from the counter-based splitmix64 stream (bit-reproducible on the
 * host); dist 1: i.i.d. N(0,1) by Box-Muller over the same stream.  When
 * `normalise` is non-zero the state is scaled to unit norm. */
int spz_state_fill_random(spz_state_t h, uint64_t seed, int dist, int normalise);

/* Lazy per-gate mode (opt-in; no reference counterpart).  With enable != 0,
 * spz_apply applies uncontrolled H, RX and RY as the gate divided by a real
 * scalar (1/sqrt 2, or the larger in magnitude of cos and sin of theta/2): 4
 * FP64 instructions per amplitude pair instead of the reference's 8-12
 * (h_apply_strat2 gates.rs:547-562, rx_apply_target :713-725,
 * ry_apply_strategy2 :1116-1119), which makes them bound by HBM instead of by
 * FP64 issue on GB300; uncontrolled RZ becomes P (the 1 half only) times a
 * phase.  The handle carries the product of those scalars and phases as a
 * pending factor and folds it into the arrays (one scaling pass) before
 * anything reads them: download, device_arrays, copy, measurement,
 * expectations, sampling, circuit execution, adjoint differentiation.  Every
 * other gate runs exactly as in the default mode (a linear gate commutes with
 * the factor).  Results equal the default mode's up to rounding, not bit for
 * bit.  Code that reads wrapped arrays (spz_state_wrap) itself must call
 * spz_state_settle first.  enable == 0 settles and returns to the reference's
 * arithmetic, the default. */
int spz_state_set_lazy(spz_state_t h, int enable);

/* Fold the lazy mode's pending factor into the arrays now (nothing to do when
 * there is none). */
int spz_state_settle(spz_state_t h);

/* Tile geometry of the fused passes that spz_circuit_execute,
 * spz_circuit_execute_host and spz_iqft run on this handle: 2^tile_qubits
 * amplitudes per shared-memory tile (4..10; 0 = 10) and threads per block
 * (32 or 64; 0 = 64).  A tunable with no reference counterpart (the reference
 * fixes its serial/parallel threshold, gates.rs:14): the exact mode's results
 * are identical for every choice; the fast mode's equal up to rounding. */
int spz_state_set_tile(spz_state_t h, int tile_qubits, int threads);

/* --------------------------------------------------------- gate application */
/* apply(gate, &mut State, target): uncontrolled gate.
 * Replaces spinoza/src/gates.rs:215-232.  SWAP takes its qubits from the gate
 * (gates.rs:1376); BitFlipNoise applies X iff gate.p[1] <= gate.p[0]
 * (gates.rs:1365-1374, with the draw made explicit). */
int spz_apply(spz_state_t h, const spz_gate* gate, uint32_t target);

/* c_apply(gate, &mut State, control, target).  Replaces gates.rs:257-269.
 * Accepts every 1-qubit gate kind, including Z (controlled-Z), which the
 * reference's match arm lacks (gates.rs:258-268). */
int spz_c_apply(spz_state_t h, const spz_gate* gate, uint32_t control, uint32_t target);

/* cc_apply(gate, &mut State, c0, c1, target).  Replaces gates.rs:272-277
 * (the reference only defines X; this library accepts every 1-qubit gate). */
int spz_cc_apply(spz_state_t h, const spz_gate* gate, uint32_t control0, uint32_t control1,
                 uint32_t target);

/* mc_apply(gate, &mut State, controls, zeros, target).  Replaces
 * gates.rs:290-320.  The gate acts on `target` for basis states whose control
 * qubits all read 1, except the qubits listed in `zeros`, which must read 0.
 * `zeros` may be NULL (nzeros == 0); every entry of `zeros` must also appear in
 * `controls`. */
int spz_mc_apply(spz_state_t h, const spz_gate* gate, const uint32_t* controls,
                 uint32_t ncontrols, const uint32_t* zeros, uint32_t nzeros, uint32_t target);

/* transform_u / c_transform_u (spinoza/src/gates.rs:1427-1487) and
 * unitaries::apply_unitary (spinoza/src/unitaries.rs): apply a 2^m x 2^m complex
 * matrix (row-major, separate real and imaginary arrays, like `Unitary`) to
 * qubits target .. target+m-1 (bit target+j of an index is bit j of the row /
 * column), only where `control` reads 1 when control >= 0.  m in 1..12; the
 * control must lie outside the block.  Uses one state-sized work vector. */
int spz_apply_unitary(spz_state_t h, const double* u_reals, const double* u_imags, uint32_t m,
                      uint32_t target, int32_t control);

/* ---------------------------------------------------------------- circuits */
/* Control kinds of a transformation; same variants as `enum Controls`
 * (spinoza/src/circuit.rs:55-69). */
enum spz_controls_kind {
  SPZ_CONTROLS_NONE = 0,
  SPZ_CONTROLS_SINGLE = 1,
  SPZ_CONTROLS_ONES = 2,
  SPZ_CONTROLS_MIXED = 3
};

/* One QuantumTransformation (circuit.rs:113-120) in flat form.  For M the
 * measurement draw is gate.p[0] (outcome 1 iff p[0] < 1 - prob0). */
typedef struct spz_op {
  spz_gate gate;
  uint32_t target;
  int32_t controls_kind; /* enum spz_controls_kind           */
  uint64_t controls;     /* bit q set: qubit q is a control  */
  uint64_t zeros;        /* MIXED: controls that must read 0 */
} spz_op;

/* QubitTracker (circuit.rs:122-164): which qubits were measured, and the values. */
typedef struct spz_tracker {
  uint64_t measured;
  uint64_t values;
} spz_tracker;

/* Execution flags. */
#define SPZ_EXEC_DEFAULT 0u      /* fused executor: runs of gates per shared-memory tile  */
#define SPZ_EXEC_UNFUSED 1u      /* one kernel per gate (the plain per-gate path)         */
#define SPZ_EXEC_TIME_PASSES 4u  /* time every pass with CUDA events (synchronises once)  */
#define SPZ_EXEC_FAST 8u         /* fused, with arithmetic rewritten to need fewer FP64
                                    instructions (lazy scaling, phase pushing); equal to
                                    the exact mode up to rounding, not bit-identical     */
#define SPZ_EXEC_TMA 32u         /* fused tile passes load each tile with the Tensor
                                    Memory Accelerator (gathers of four 64-byte rows)
                                    instead of thread loads; same results               */
#define SPZ_EXEC_TMA_PREFETCH 64u /* as SPZ_EXEC_TMA, and the next tile is fetched while
                                    the current one computes (two tile buffers)          */
#define SPZ_EXEC_SHUFFLE 128u    /* fused tile passes apply runs of gates on the five
                                    lowest tile qubits with warp shuffles, amplitudes in
                                    registers and no block barrier between the gates of
                                    a run; same results                                 */

/* Execution counters filled by spz_circuit_execute (may be NULL). */
typedef struct spz_exec_stats {
  uint64_t gates;          /* gates applied                                         */
  uint64_t passes;         /* passes over the state (kernel launches)               */
  uint64_t tile_passes;    /* of which fused shared-memory tile passes              */
  uint64_t bytes_moved;    /* HBM bytes the passes read + wrote                     */
  uint64_t algorithmic_bytes; /* sum over gates of the unfused bytes                */
  uint64_t fp64_ops;       /* FP64-pipe instructions the gates' arithmetic needs    */
  double tile_ms;          /* SPZ_EXEC_TIME_PASSES: device time of the tile passes  */
  double plain_ms;         /* SPZ_EXEC_TIME_PASSES: device time of plain gate passes */
  uint64_t shuffle_gates;  /* SPZ_EXEC_SHUFFLE: ops applied in warp-shuffle runs     */
  uint64_t io_slab_passes; /* spz_circuit_execute_host: passes run slab by slab with
                              the host copies overlapped                          */
} spz_exec_stats;

/* QuantumCircuit::execute (circuit.rs:552-600): apply `ops` in order.
 * `tracker` carries the QubitTracker across calls (may be NULL when the list has
 * no M and no classically controlled gate).  A Single control on an already
 * measured qubit becomes a classical control (circuit.rs:570-578). */
int spz_circuit_execute(spz_state_t h, const spz_op* ops, size_t nops, spz_tracker* tracker,
                        uint32_t flags, spz_exec_stats* stats);

/* QuantumCircuit::execute on a state held in host memory, the reference's own
 * setting (`State { reals, imags }`, core.rs:20-42, mutated in place by
 * circuit.rs:552-600): the input arrays (2^n doubles each, n = the handle's)
 * are uploaded into the handle, the circuit runs, and the result is written
 * to the output arrays before the call returns; pass the same arrays for the
 * reference's in-place behaviour.  For page-locked arrays (cudaHostAlloc /
 * cudaHostRegister) the upload is cut into 8 slabs that the leading tile
 * passes consume as they arrive (every leading pass that keeps the slab
 * qubits non-local runs slab by slab) and the download follows the trailing
 * passes slab by slab (every trailing pass that keeps three consecutive
 * qubits non-local runs slab by slab), on a second stream; pageable arrays
 * are copied whole before and after.  Same flags, tracker and stats as
 * spz_circuit_execute (stats->io_slab_passes counts the slab-by-slab passes). */
int spz_circuit_execute_host(spz_state_t h, const double* in_reals, const double* in_imags, double* out_reals,
                             double* out_imags, const spz_op* ops, size_t nops, spz_tracker* tracker,
                             uint32_t flags, spz_exec_stats* stats);

/* Compiled circuits: plan `ops` once for n qubits (fused passes; fast-mode
 * lowering with SPZ_EXEC_FAST; descriptors uploaded to device memory the
 * program owns) and run it on any n-qubit state as a replayed CUDA graph: a
 * run costs no planning and no host work beyond one graph launch on the
 * state's stream (asynchronous; spz_state_synchronize waits).  The graph is
 * captured on the first run for a given state and again when the state
 * changes.  Programs hold no measurements (SPZ_ERR_UNSUPPORTED); a Single
 * control is always a quantum control.  Extension: the reference plans nothing
 * ahead (QuantumCircuit::execute, circuit.rs:552-600, walks the list each time). */
typedef struct spz_program_s* spz_program_t;
int spz_program_create(uint32_t n, const spz_op* ops, size_t nops, uint32_t flags, spz_program_t* out);
int spz_program_run(spz_program_t p, spz_state_t h);
int spz_program_stats(spz_program_t p, spz_exec_stats* stats);
int spz_program_destroy(spz_program_t p);

/* Plan `ops` for an n-qubit state without running anything (host only; no
 * device is needed): fills the counters spz_circuit_execute would, taking every
 * measurement outcome as 0.  For inspecting how a circuit is fused. */
int spz_plan_stats(uint32_t n, const spz_op* ops, size_t nops, uint32_t flags, spz_exec_stats* stats);

/* The passes spz_circuit_execute would launch (host only), one entry per
 * pass as counted in spz_exec_stats.passes: local_mask[k] = the local qubits
 * of a fused tile pass (0 for a plain one-gate pass or a measurement's two
 * passes), pass_ops[k] = the device ops it applies (after the fast-mode
 * lowering and fusion; 1 for a plain gate, 0 for a measurement's passes).
 * *count receives the number of passes; at most `capacity` are written.
 * For inspecting the plan (tile sizes, copy-overlap geometry). */
int spz_plan_passes(uint32_t n, const spz_op* ops, size_t nops, uint32_t flags, uint64_t* local_mask,
                    uint32_t* pass_ops, size_t capacity, size_t* count);

/* The order in which spz_circuit_execute would apply `ops` (host only):
 * order[k] is the index of the k-th applied op and pass[k] the pass (kernel
 * launch) that applies it; skipped ops do not appear.  *count receives the
 * number of entries; at most `capacity` are written. */
int spz_plan_schedule(uint32_t n, const spz_op* ops, size_t nops, uint32_t flags, uint32_t* order,
                      uint32_t* pass, size_t capacity, size_t* count);

/* iqft(&mut State, targets) (spinoza/src/core.rs:184-191). */
int spz_iqft(spz_state_t h, const uint32_t* targets, uint32_t ntargets);

/* ------------------------------------------------------------- measurement */
/* measure_qubit(&mut State, target, reset, v) -> u8 (measurement.rs:12-92).
 * forced: -1 draws the outcome from `u` (1 iff u < 1 - prob0), 0/1 forces it.
 * *outcome receives the value; *prob0 (may be NULL) the probability of 0. */
int spz_measure_qubit(spz_state_t h, uint32_t target, int reset, int forced, double u,
                      uint8_t* outcome, double* prob0);

/* Probability that `target` reads 0 (the first pass of measurement.rs:16-29). */
int spz_prob0(spz_state_t h, uint32_t target, double* prob0);

/* qubit_expectation_value(&State, target) = 2 prob0 - 1 (core.rs:198-219). */
int spz_qubit_expectation_value(spz_state_t h, uint32_t target, double* out);

/* xyz_expectation_value(observable, &State, targets) (core.rs:222-264).
 * observable is 'x', 'y' or 'z'; out[i] = Re<psi|O_{targets[i]}|psi>. */
int spz_xyz_expectation_value(spz_state_t h, char observable, const uint32_t* targets,
                              uint32_t ntargets, double* out);

/* Allocation-free form of spz_xyz_expectation_value.  It has no counterpart in
 * the reference.  It is for callers that cannot call cudaMalloc: code that runs
 * inside another framework's memory pool or arena (where a stray cudaMalloc
 * would bypass the pool's accounting or fail against its reservation), or in a
 * process whose device memory budget is fixed up front.  It takes the state as
 * raw device arrays (2^n doubles each) instead of a handle, runs on `stream`
 * (a cudaStream_t, NULL = default stream), writes ntargets results to `out`
 * (host or device memory), and synchronises `stream` before returning.
 * Its scratch is a static 10 KiB device array that every GPU loading the
 * library holds until exit, so at most SPZ_NOALLOC_MAX_TARGETS targets per
 * call; more returns SPZ_ERR_INVALID_ARGUMENT.  ntargets == 0 returns SPZ_OK
 * and launches nothing.  The first call on a device looks up the array's
 * address on that device and keeps it for the life of the process; make that
 * first call before any stream capture, and do not call this function on a
 * device after cudaDeviceReset (the kept address would be stale).  All calls
 * share the array: calls that overlap on the GPU race and must be serialised. */
#define SPZ_NOALLOC_MAX_TARGETS 64
int spz_xyz_expectation_value_noalloc(const double* d_reals, const double* d_imags, uint32_t n,
                                      char observable, const uint32_t* targets, uint32_t ntargets,
                                      double* out, void* stream);

/* A Pauli string coeff * X^x_mask Z^z_mask with Y on bits set in both masks
 * (Y = i X Z per qubit, the phase is accounted for). */
typedef struct spz_pauli_term {
  double coeff;
  uint64_t x_mask;
  uint64_t z_mask;
} spz_pauli_term;

/* <psi|H|psi> for H = sum of Pauli terms, in fused tile passes.  No reference
 * counterpart as one call; the reference builds it from xyz_expectation_value
 * (clone + apply + Re inner product, core.rs:222-264). */
int spz_pauli_expectation(spz_state_t h, const spz_pauli_term* terms, size_t nterms, double* out);

/* Norm squared sum |a_i|^2 (deterministic order). */
int spz_norm_sqr(spz_state_t h, double* out);

/* Sample basis-state outcomes.  For each uniform u[k] in [0,1) the outcome is
 * the inverse of the cumulative distribution of |a_i|^2 in the library's fixed
 * blocked summation order (bit-reproducible).  Serves reservoir_sampling /
 * get_samples (core.rs:67-129, spynoza/src/lib.rs:393-400). */
int spz_sample(spz_state_t h, const double* u, size_t nshots, uint64_t* out);

/* ---------------------------------------------------------- differentiation */
/* Adjoint differentiation of E(theta) = <psi(theta)|H|psi(theta)> with
 * psi(theta) = ops applied to the handle's current state.  Parameterised ops
 * are the rotation gates (P, RX, RY, RZ, and their controlled forms) whose
 * index appears in param_index: param_index[j] = k means d/d(ops[k].gate.p[0])
 * goes to grad[j].  On return the handle holds psi(theta), *energy = E, grad[j]
 * = dE/dtheta_j.  Needs two extra state vectors of device memory.  flags:
 * SPZ_EXEC_DEFAULT, or SPZ_EXEC_FAST (fast-mode forward, and a backward sweep
 * with lazily scaled H / RX / RY inverses and RZ inverses as P: about half the
 * FP64 work, equal to the exact gradients up to rounding).
 * No reference counterpart (new form built on the gate path). */
int spz_adjoint_gradient(spz_state_t h, const spz_op* ops, size_t nops,
                         const uint32_t* param_index, size_t nparams,
                         const spz_pauli_term* terms, size_t nterms, uint32_t flags,
                         double* energy, double* grad);

/* ---------------------------------------------------------------- batching */
/* Many independent parameterised circuits of uneven qubit counts, each with its
 * own Pauli-sum observable: E_i = <0|U_i(theta)^dagger H_i U_i(theta)|0> and
 * dE_i/dtheta for all of them in one persistent launch, replayed as a CUDA
 * graph.  Instances of up to tile_qubits qubits run entirely in shared memory,
 * one CTA each; larger ones stream tiles through HBM workspace.  Wide
 * instances (at least wide_qubits qubits) are spread over many CTAs as work
 * items (one pass over a range of tiles each), ordered by per-instance
 * completion counters inside the same launch; a dependency wait that runs out
 * ends the launch with SPZ_ERR_TIMEOUT.  No reference counterpart (new form). */
typedef struct spz_batch_s* spz_batch_t;

typedef struct spz_batch_instance {
  uint32_t n;             /* qubits (1..30)                                   */
  uint32_t nops;          /* ops of this instance                             */
  uint32_t nparams;       /* parameters of this instance                      */
  uint32_t nterms;        /* Pauli terms of this instance's observable        */
  uint64_t op_offset;     /* first op in `ops`                                */
  uint64_t param_offset;  /* first entry in param_index / theta / grads       */
  uint64_t term_offset;   /* first term in `terms`                            */
} spz_batch_instance;

typedef struct spz_batch_config {
  int32_t tile_qubits;    /* local qubits per shared-memory tile, 4..12 (0 = 9) */
  int32_t threads;        /* threads per CTA, multiple of 32 in 64..1024 (0 = 64) */
  int32_t wide_qubits;    /* instances of at least this many qubits (and more than
                             tile_qubits) are split into work items across CTAs, each
                             with its own psi and lam in HBM; 0 = 18, > 30 = never.
                             Those whose workspace exceeds 60% of free memory, and all
                             of them under SPZ_EXEC_FAST, run one at a time across
                             the GPU instead (fused executor + fused adjoint sweep) */
  int32_t flags;          /* SPZ_EXEC_FAST: the wide instances use the fast adjoint
                             (equal to the exact one up to rounding), one at a time
                             across the GPU; SPZ_BATCH_WIDE_APART: the wide instances
                             run one at a time across the GPU in the exact mode too
                             (no per-instance workspace held for the whole run)      */
  int32_t tiles_per_item; /* tiles per work item of a wide instance (0 = 64)       */
} spz_batch_config;

#define SPZ_BATCH_WIDE_APART 16

typedef struct spz_batch_stats {
  uint64_t instances, resident_instances;
  uint64_t forward_passes, hamiltonian_passes, backward_passes;
  uint64_t ctas, workspace_bytes;
  int32_t tile_qubits, threads;
  uint64_t wide_in_kernel;        /* wide instances run as work items in the launch   */
  uint64_t work_items;            /* entries of the persistent kernel's queue         */
  uint64_t wide_separate;         /* wide instances run one at a time across the GPU  */
  uint64_t wide_workspace_bytes;  /* HBM of the in-launch wide instances' psi and lam */
  int32_t tiles_per_item, pad_;
} spz_batch_stats;

/* Plan and upload a batch.  param_index[param_offset + j] is the op (relative to
 * the instance's op_offset) whose angle p[0] is parameter j; only P, RX, RY and
 * RZ angles can be parameters.  Ops may not contain M or BitFlipNoise. */
int spz_batch_create(const spz_batch_instance* instances, size_t ninstances, const spz_op* ops,
                     const uint32_t* param_index, const spz_pauli_term* terms,
                     const spz_batch_config* config, spz_batch_t* out);
/* theta[param_offset + j]: angles (host); energies[i] and grads[param_offset + j]: outputs (host). */
int spz_batch_run(spz_batch_t b, const double* theta, double* energies, double* grads);
int spz_batch_info(spz_batch_t b, spz_batch_stats* stats);
int spz_batch_destroy(spz_batch_t b);

/* ------------------------------------------------------------------ probes */
/* Measured FP64 FMA issue rate of the current device (FMA/s): the second
 * roofline (beside HBM bandwidth) that bounds dense FP64 gate kernels. */
int spz_probe_fp64_fma_rate(double* fma_per_s);

#ifdef __cplusplus
}
#endif
#endif /* SPINOZA_GB300_H */
