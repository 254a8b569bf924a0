/*
 * krets_gpu.h — C ABI of the GB300 (sm_103a) MNA solve path.
 *
 * This is the drop-in boundary for krets's solver crate.  Each entry point replaces one
 * reference interface (paths inside prokie/krets):
 *
 *   krets_circuit_create   Solver::new(circuit, config)          crates/krets-solver/src/solver.rs:22-25
 *                          + parse-time index layout             crates/krets-parser/src/parser.rs:105-125
 *   krets_op               op::solve                             crates/krets-solver/src/solver/op.rs:15-86
 *   krets_dc               dc::solve                             crates/krets-solver/src/solver/dc.rs:14-124
 *   krets_ac               ac::solve                             crates/krets-solver/src/solver/ac.rs:17-109
 *   krets_tran             transient::solve                      crates/krets-solver/src/solver/transient.rs:14-114
 *   krets_batch_*          (no counterpart: many instances of one topology per launch)
 *   krets_multi_*          (no counterpart: many distinct netlists per launch set)
 *   krets_adjoint_tran     (no counterpart: adjoint sensitivities)
 *   krets_status_string /  Display of krets_solver::Error        crates/krets-solver/src/error.rs:4-36
 *   krets_last_error_message
 *
 * Conventions
 *   - All functions are `extern "C"`, never throw, and return a krets_status (0 = OK).
 *   - Unknown numbering is the reference's: in element file order, I(<id>) first for
 *     Group-2 elements, then each first-seen non-ground node as V(<node>).
 *   - Output buffers are caller-owned.  A pointer may be host memory (pageable or pinned)
 *     or device memory; the library detects which and copies only when it must.
 *   - A krets_circuit owns its device memory and one CUDA stream.  A handle is not
 *     thread-safe; distinct handles are.
 *   - No CPU fallback: every solve runs on the GPU, and an absent or unusable GPU is
 *     reported as KRETS_ERR_CUDA.
 */
#ifndef KRETS_GPU_H
#define KRETS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------------- status codes */
typedef int32_t krets_status;
#define KRETS_OK 0
#define KRETS_ERR_ELEMENT_NOT_FOUND 1    /* Error::ElementNotFound            error.rs:8-9   */
#define KRETS_ERR_MAX_ITERATIONS 2       /* Error::MaximumIterationsExceeded  error.rs:12-13 */
#define KRETS_ERR_INVALID_ELEMENT 3      /* Error::InvalidElementFormat       error.rs:16-17 */
#define KRETS_ERR_UNEXPECTED 4           /* Error::Unexpected                 error.rs:20-21 */
#define KRETS_ERR_DECOMPOSITION_FAILED 5 /* Error::DecompositionFailed        error.rs:24-25 */
#define KRETS_ERR_MATRIX_BUILD 6         /* Error::MatrixBuild                error.rs:28-29 */
#define KRETS_ERR_MATRIX_DECOMPOSITION 7 /* Error::MatrixDecomposition        error.rs:32-33 */
#define KRETS_ERR_NOT_IMPLEMENTED 8      /* the reference panics with todo!() (BJT, NMOS AC) */
#define KRETS_ERR_TIMEOUT 9              /* a bounded device wait ran out                    */
#define KRETS_ERR_CUDA 10                /* a CUDA runtime call failed / no GPU              */
#define KRETS_ERR_INVALID_ARGUMENT 11
#define KRETS_ERR_OUT_OF_MEMORY 12
#define KRETS_ERR_PIVOT_UNSTABLE 13      /* static pivot growth above the limit              */

/* ----------------------------------------------------------------- elements */
#define KRETS_ELEM_R 1 /* resistor          value = ohms                                   */
#define KRETS_ELEM_C 2 /* capacitor         value = farads, flags may hold KRETS_FLAG_G2   */
#define KRETS_ELEM_L 3 /* inductor          value = henries                                */
#define KRETS_ELEM_V 4 /* voltage source    value = dc value, ac = AC amplitude, wave/wp   */
#define KRETS_ELEM_I 5 /* current source    value = amperes                                */
#define KRETS_ELEM_D 6 /* diode             value = saturation current, wp[0] = emission n */
#define KRETS_ELEM_M 7 /* NMOS level 1      wp = {vto, kp, lambda, w, l}; stamps nothing,
                          as the reference's bare-name index lookups never match, unless
                          flags holds KRETS_FLAG_NMOS_RESOLVED                              */
#define KRETS_ELEM_Q 8 /* BJT               parsed only; solving reports NOT_IMPLEMENTED   */

#define KRETS_FLAG_G2 1
/* NMOS: resolve drain / source / gate as their V(<node>) unknowns (the reference looks the
 * bare node names up and stamps nothing: stampable.rs:842-844).  The stamp is then the
 * reference's own entries and values (stampable.rs:846-866, rhs :870-899) with the
 * level-1 g_m, g_ds and i_d of nmosfet.rs:51-103, evaluated at the Newton guess. */
#define KRETS_FLAG_NMOS_RESOLVED 2

#define KRETS_WAVE_NONE 0
#define KRETS_WAVE_PULSE 1 /* wp = {v1, v2, td, tr, tf, pw, per}  voltage_source.rs:70-93 */
#define KRETS_WAVE_SIN 2   /* wp = {off, amp, freq, td, damp, phase_deg}  :52-65          */

/* One flattened element (104 bytes).  p/m/b/g hold MNA unknown indices or -1 (ground, or
 * absent from the index map — the reference then skips that stamp entry). */
typedef struct krets_element {
  int32_t kind;
  int32_t p;     /* V(plus)  (NMOS: drain)  */
  int32_t m;     /* V(minus) (NMOS: source) */
  int32_t b;     /* I(<id>) for Group-2 elements */
  int32_t g;     /* NMOS gate */
  int32_t flags;
  int32_t wave;
  int32_t reserved;
  double value;
  double ac;
  double wp[7];
} krets_element;

/* SolverConfig (crates/krets-solver/src/config.rs:4-36). */
typedef struct krets_config {
  double relative_tolerance;         /* 1e-3  */
  double current_absolute_tolerance; /* 1e-12 */
  double voltage_absolute_tolerance; /* 1e-6  */
  int32_t maximum_iterations;        /* 300   */
  int32_t reserved;
} krets_config;

#define KRETS_METHOD_BE 0 /* backward Euler, as the reference */
#define KRETS_METHOD_TR 1 /* trapezoidal (extension) */

/* Precision of the batched transient/AC engines. */
#define KRETS_PREC_FP64 0  /* FP64 factor and solves (the plain form's arithmetic)          */
#define KRETS_PREC_MIXED 1 /* FP32 factor + solves, iterative refinement with an FP64-class
                              residual (double-float pairs on FP32 pipes for linear circuits,
                              FP64 for nonlinear ones) */
#define KRETS_PREC_DF 2    /* factors computed in FP64, kept and applied as double-float pairs
                              (48-bit significand) on FP32 pipes; linear circuits (nonlinear
                              ones fall back to KRETS_PREC_MIXED) */

typedef struct krets_circuit krets_circuit;

/* Compile the topology (host symbolic pass: fill-reducing ordering, static pivot
 * sequence, fill pattern, stamp-to-slot maps, level schedules) and upload it.
 * `elems` holds nominal values, used to choose pivots.  cfg may be NULL (defaults). */
krets_status krets_circuit_create(const krets_element *elems, int32_t n_elem, int32_t n_unknowns,
                                  const krets_config *cfg, krets_circuit **out);
krets_status krets_circuit_destroy(krets_circuit *c);
krets_status krets_circuit_info(const krets_circuit *c, int32_t mode, int32_t *n, int32_t *nnz_a,
                                int32_t *nnz_lu, int32_t *n_levels, int32_t *n_ulevels);

/* ------------------------------------------------- single-instance analyses (plain form)
 * FP64 throughout, one instance, level-scheduled single-CTA kernels.  These mirror the
 * reference's per-analysis functions; results use the reference unknown numbering. */

/* x_out[n]; iters_out (optional) = Newton iterations. */
krets_status krets_op(krets_circuit *c, double *x_out, int32_t *iters_out);

/* DC sweep of element index `sweep_elem` (must be a V or I source).
 * Points: |(stop-start)/step| + 1 (truncated), x_out[max_points][n]. */
krets_status krets_dc(krets_circuit *c, int32_t sweep_elem, double start, double stop, double step,
                      double *x_out, int32_t max_points, int32_t *n_points);

/* AC sweep: operating point first, frequencies <= 0 skipped.
 * x_out: complex, interleaved re/im, [n_freq][n][2]; *n_kept = points solved. */
krets_status krets_ac(krets_circuit *c, const double *freqs, int32_t n_freq, double *x_out,
                      int32_t *n_kept);

/* Transient: t=0 operating point, then n_steps fixed steps of size h.
 * method KRETS_METHOD_BE/TR; source_lag 1 = the reference's source timing (first Newton
 * iteration sees t_{n-1}), 0 = sources at t_n.  refactor_each_step 1 refactors the
 * matrix every step even for linear circuits (the reference's cost model).
 * x_out[n_steps+1][n]. */
krets_status krets_tran(krets_circuit *c, double h, int32_t n_steps, int32_t method, int32_t source_lag,
                        int32_t refactor_each_step, double *x_out);

/* ------------------------------------------------- batched (persistent) engines
 * `values` [n_inst][n_elem] replaces each element's `value` per instance (Monte Carlo).
 * The engine runs one instance per CTA drawn from a device work queue, keeps the
 * factors and state in shared memory for the whole run, and writes every unknown at
 * every step.  stats_out (optional, host) receives per-instance refinement counts. */
krets_status krets_batch_tran(krets_circuit *c, int32_t n_inst, const double *values, double h,
                              int32_t n_steps, int32_t method, int32_t source_lag, int32_t precision,
                              double *x_out /* [n_inst][n_steps+1][n] */,
                              int32_t *inst_status /* [n_inst] or NULL */);

/* Transient with local-truncation-error step control (extension: krets steps at a fixed
 * h, transient.rs:14-114).  From the operating point at t = 0 to t_stop, FP64, per
 * instance: each attempt solves the companion system at t + h (sources at t + h; Newton
 * for nonlinear circuits), estimates the LTE by divided differences over the last
 * accepted points (BE: h^2 DD2, TR: h^3/2 DD3) and accepts it when
 * max_k |LTE_k| / (lte_tol max(|x_k|, |x_prev,k|) + abstol_k) <= 1 (abstol: the config's
 * current / voltage tolerance).  h then changes by the largest factor of {2, 1.5, 1, 0.75,
 * 0.5} (after an accept) or {0.5, 0.25, 0.125} (after a reject; 0.125 when Newton does not
 * converge) whose predicted ratio stays <= 1/2, within [h_min, h_max]; the first 1 (BE) or
 * 2 (TR) steps are taken at h0 unchecked.  Accepted points: t_out[n_inst][max_points],
 * x_out[n_inst][max_points][n] (row 0 = operating point), n_points[n_inst].  A step below
 * h_min stops the instance (KRETS_ERR_UNEXPECTED); more points than max_points stops it
 * with KRETS_ERR_INVALID_ARGUMENT.  values may be NULL (one instance, nominal values). */
krets_status krets_batch_tran_adaptive(krets_circuit *c, int32_t n_inst, const double *values, double h0,
                                       double t_stop, int32_t method, double lte_tol, double h_min, double h_max,
                                       int32_t max_points, double *t_out, double *x_out, int32_t *n_points,
                                       int32_t *inst_status);

/* Probe-only batched transient: as krets_batch_tran in double-float precision
 * (KRETS_PREC_DF, linear circuits), but each step writes only the unknowns probe[0..n_probe)
 * (MNA indices, e.g. the output node): x_out[n_inst][n_steps+1][n_probe], row 0 = their
 * operating-point values.  The arithmetic is that of krets_batch_tran; only the output
 * traffic differs. */
krets_status krets_batch_tran_probe(krets_circuit *c, int32_t n_inst, const double *values, double h,
                                    int32_t n_steps, int32_t method, int32_t source_lag, int32_t n_probe,
                                    const int32_t *probe, double *x_out, int32_t *inst_status);

/* Batched AC over frequency points of one instance (values NULL) or of several
 * instances: each work item is one (instance, frequency) complex system.
 * precision: FP64 = complex128 factor; MIXED = complex64 factor + complex128 refinement.
 * x_out: [n_inst][n_freq][n][2]; frequencies must be > 0.  MIXED keeps a device buffer in
 * the handle (per CTA of the launch: the frequency-independent coefficients of the
 * instance it is working on), reused by later calls and freed with the handle. */
krets_status krets_batch_ac(krets_circuit *c, int32_t n_inst, const double *values, const double *freqs,
                            int32_t n_freq, int32_t precision, double *x_out, int32_t *item_status);

/* Adjoint sensitivities of a batched linear transient (no counterpart in the reference).
 * Loss per instance: sum over steps n = 1..n_steps of x_out(t_n)^2, out_unknown being the
 * MNA index of the output (e.g. V(out)).  grad_out[n_inst][n_elem] receives dLoss/dvalue for
 * every R, C and L element; for every V and I source it receives dLoss/dalpha, alpha scaling
 * the source's transient value (its waveform, or its DC value) at alpha = 1; 0 for the
 * others.  The forward pass keeps a checkpoint every checkpoint_every steps and the
 * backward sweep recomputes each segment from it; transposed solves reuse the forward LU
 * factors.  gradient = 0 runs the forward pass only (loss).  The operating point at t = 0
 * must be zero (KRETS_ERR_NOT_IMPLEMENTED otherwise). */
krets_status krets_adjoint_tran(krets_circuit *c, int32_t n_inst, const double *values, double h, int32_t n_steps,
                                int32_t method, int32_t out_unknown, int32_t checkpoint_every, int32_t gradient,
                                double *loss_out, double *grad_out);

/* ---- Many distinct linear circuits (R, C, L, V, I) in one launch set (no counterpart in the
 * reference, whose Solver runs one circuit at a time: krets-solver/src/solver.rs:22-52).
 * Circuit c has elements elems[elem_offsets[c] .. elem_offsets[c+1]) numbered over its own
 * n_unknowns[c] unknowns.  krets_multi_create runs the host symbolic pass of every circuit
 * (DC program for the operating point, transient program for method/h) on all host threads
 * and uploads them in one device image. */
typedef struct krets_multi krets_multi;
krets_status krets_multi_create(int32_t n_circuits, const krets_element *elems, const int64_t *elem_offsets,
                                const int32_t *n_unknowns, int32_t method, double h, krets_multi **out);
krets_status krets_multi_destroy(krets_multi *m);
/* info[0..3] = circuits, sum of n, sum of transient LU entries, sum of transient solve levels;
 * info[4..9] = circuits per size class (shared-memory regions from small to large, then
 * global); info[10..15] = microseconds from the start of the last krets_multi_tran launch set
 * to the end of each class. */
krets_status krets_multi_info(const krets_multi *m, int64_t *info, int32_t cap);
/* Operating point then n_steps transient steps of every circuit (transient.rs:14-114 per
 * circuit).  Circuit c writes (n_steps+1) x n_c doubles (row 0 = operating point, original
 * unknown order) at x_out + x_offsets[c] (x_offsets NULL: circuits packed in order).
 * x_out may be host or device memory.  circuit_status (optional) receives each circuit's
 * status. */
krets_status krets_multi_tran(krets_multi *m, int32_t n_steps, int32_t source_lag, double *x_out,
                              const int64_t *x_offsets, int32_t *circuit_status);
krets_status krets_multi_last_timing(const krets_multi *m, float *kernel_ms, float *call_ms);

/* 1 when kernels read and write caller host buffers in place (a GPU sharing the host's page
 * tables, as on Grace systems), 0 when host buffers go through device copies.  Set
 * KRETS_NO_DIRECT_HOST=1 before the first call to force the copies. */
int32_t krets_direct_host_access(void);

/* Batched DC sweep (dc.rs:14-124 per instance): every instance sweeps element `sweep_elem`
 * over the same points, warm-started point to point; values [n_inst][n_elem] replaces the
 * elements' values per instance (the swept element's value is overwritten per point).
 * x_out[n_inst][max_points][n]; *n_points = points per instance; an instance stops at its
 * first failing point (its status in inst_status). */
krets_status krets_batch_dc(krets_circuit *c, int32_t n_inst, const double *values, int32_t sweep_elem,
                            double start, double stop, double step, double *x_out, int32_t max_points,
                            int32_t *n_points, int32_t *inst_status);

/* Batched operating points: x_out[n_inst][n]. */
krets_status krets_batch_op(krets_circuit *c, int32_t n_inst, const double *values, double *x_out,
                            int32_t *inst_status);

/* ------------------------------------------------- diagnostics and timing */
const char *krets_status_string(krets_status s);
const char *krets_last_error_message(void);
/* Device time (CUDA events on the handle's stream) of the last call's main kernel and of
 * the whole last call (copies included), in milliseconds. */
krets_status krets_last_timing(const krets_circuit *c, float *kernel_ms, float *call_ms);
/* The last double-float batched transient launch: info[0] = threads per instance,
 * info[1] = instances per CTA, info[2] = grid, info[3] = how the group size was chosen
 * (1 = timed now by the autotuner, 2 = the autotuner's cached choice for this sparsity
 * signature, 0 = default, too few steps to time; KRETS_GROUP=32|64|128 overrides),
 * info[4] = 1 when the factors were kept in global memory (more instances per SM) instead
 * of shared memory (the autotuner chooses; KRETS_DFD_LU=smem|global overrides). */
krets_status krets_last_launch(const krets_circuit *c, int32_t *info, int32_t cap);
/* Kernel launches issued by this library since load. */
int64_t krets_launch_count(void);
/* Refinement statistics of the last mixed-precision batched call: histogram[k] = number
 * of (instance, step) solves that took k refinement iterations (k < 8), fallbacks =
 * instances that switched to an FP64 refactor, max_rel_correction = largest final
 * correction / |x| seen. */
krets_status krets_last_refine_stats(const krets_circuit *c, int64_t histogram[8], int32_t *fallbacks);

/* Device memory helpers so a caller without a CUDA runtime binding can hold device-
 * resident inputs/outputs (used by the benchmark). */
krets_status krets_device_alloc(size_t bytes, void **ptr);
krets_status krets_device_free(void *ptr);
krets_status krets_memcpy_h2d(void *dst, const void *src, size_t bytes);
krets_status krets_memcpy_d2h(void *dst, const void *src, size_t bytes);
/* Page-lock (pin) a caller's host buffer for the lifetime of a run, and release it.  No
 * counterpart in the reference.  Results of krets_batch_tran with precision
 * KRETS_PREC_DF are copied into host x_out buffers by the copy engines while the next
 * span of steps runs; into pinned memory those copies run at the host link's rate. */
krets_status krets_host_register(void *ptr, size_t bytes);
krets_status krets_host_unregister(void *ptr);
/* Write a scratch buffer larger than L2 (on the given circuit's stream). */
krets_status krets_flush_l2(krets_circuit *c);
krets_status krets_device_synchronize(void);

/* Allocation-free batched transient.  No counterpart in the reference.
 *
 * For callers that are not allowed to allocate device memory while they run: a host
 * program that hands all GPU memory to its own arena at start-up and forbids hidden
 * allocations, a real-time loop whose allocations must all happen before the loop starts,
 * or code that enqueues work while another thread is capturing a CUDA graph in a mode in
 * which cudaMalloc is an error.  krets_batch_tran may allocate temporary device buffers
 * (scratch, staging of host buffers); this entry point does not call cudaMalloc or
 * cudaFree at all.
 *
 *  - values (may be NULL: nominal values), x_out and inst_status must be device pointers
 *    (same shapes as krets_batch_tran).
 *  - precision is KRETS_PREC_FP64, KRETS_PREC_MIXED or KRETS_PREC_DF (anything else is
 *    KRETS_ERR_INVALID_ARGUMENT).  For each, the call picks the same engine, kernels,
 *    refinement tolerance and launch shape as krets_batch_tran, so with the same inputs
 *    the two return identical results.  For KRETS_PREC_DF it uses the group size that the
 *    autotuner of an earlier krets_batch_tran call cached for this circuit (else 128); it
 *    never runs the autotuner itself.
 *  - The circuit must already hold the compiled programs for (method, h): call
 *    krets_batch_tran once with the same time step and method during set-up.  Otherwise
 *    the call fails with KRETS_ERR_INVALID_ARGUMENT.
 *  - Only circuits that run entirely in shared memory are accepted: the operating-point
 *    workspace must fit in one CTA's shared memory, and so must the transient engine's
 *    (the double-float engine's layout for KRETS_PREC_DF, else the warp engine's).
 *    krets_batch_tran runs larger circuits with global-memory workspaces that it
 *    allocates; here they are rejected with KRETS_ERR_INVALID_ARGUMENT.
 *  - Its scratch is a fixed 16 MiB device array inside the library, present on every GPU
 *    that loads the library until the process exits.  Requests that do not fit (too many
 *    instances, a KRETS_PREC_DF waveform table of n_steps + 1 values per PULSE / SIN
 *    source that is too long, or one CTA's FP64 fallback factors too large) are rejected
 *    with KRETS_ERR_INVALID_ARGUMENT; otherwise a smaller array only limits the number of
 *    concurrent CTAs.
 *  - The first call on a device looks up that array's device address (once per device);
 *    make that first call before any stream capture.
 *  - Every call shares the array and clears what must start at zero on entry; calls that
 *    overlap on the GPU (other threads, other handles) race on it.
 *  - The call is synchronous and returns the combined status of all instances. */
krets_status krets_batch_tran_noalloc(krets_circuit *c, int32_t n_inst, const double *values, double h,
                                      int32_t n_steps, int32_t method, int32_t source_lag, int32_t precision,
                                      double *x_out, int32_t *inst_status);

/* ------------------------------------------------- symbolic-pass introspection
 * Builds the static program of a topology for one mode on the host (no GPU needed) and
 * copies array `which` (KRETS_PROG_*) into out[cap]; *len receives its length.  Used by
 * tests to check the ordering, pivot sequence, fill and schedules. */
#define KRETS_PROG_Q 0
#define KRETS_PROG_PROW 1
#define KRETS_PROG_LU_ROWPTR 2
#define KRETS_PROG_LU_COL 3
#define KRETS_PROG_LU_DIAG 4
#define KRETS_PROG_A_ROWPTR 5
#define KRETS_PROG_A_COL 6
#define KRETS_PROG_A_SLOT 7
#define KRETS_PROG_A_CPTR 8
#define KRETS_PROG_A_CONTRIB 9
#define KRETS_PROG_B_CPTR 10
#define KRETS_PROG_B_CONTRIB 11
#define KRETS_PROG_PIV_PTR 12
#define KRETS_PROG_PIV 13
#define KRETS_PROG_UPD 14
#define KRETS_PROG_LEV_PTR 15
#define KRETS_PROG_LEV_ROWS 16
#define KRETS_PROG_ULEV_PTR 17
#define KRETS_PROG_ULEV_ROWS 18
#define KRETS_PROG_EL_POS 19
#define KRETS_PROG_META 20 /* {ordering, n, nnz_a, nnz_lu, n_levels, n_ulevels, factor_flops, tail0, tail_m} */
#define KRETS_PROG_TPROG 21 /* transposed-solve program (transient mode) */
#define KRETS_PROG_TPOFF 22 /* its section offsets (8) and level counts of U^T and L^T */
#define KRETS_PROG_SPROG 23 /* compact step program staged in shared memory */
#define KRETS_PROG_SPOFF 24 /* its section offsets (16), border chunk and row counts */
#define KRETS_PROG_IPROG 25 /* interleaved solve programs (transient mode, single circuit) */
#define KRETS_PROG_IPOFF 26 /* {ip_off[2][4], il_slots[2], imap_off[2], n_il_lrec, n_il_urec, il_ok,
                               lean_off, n_zrow, n_ind, lean_ok, ip_off[4], il_slots, imap_off}:
                               layouts for 64, 128 and (last) 32-thread groups */
#define KRETS_PROG_IMAP 27  /* interleaved factor slot -> CSR slot (-1: zero pad) */
#define KRETS_MODE_DC 0
#define KRETS_MODE_AC 1
#define KRETS_MODE_TRAN 2
/* ordering: -1 = autotune, else a fixed ORDER; ORDER | KRETS_PROG_MULTI builds the program
 * the multi-circuit engine uses (dense trailing block, no factorisation update list), with
 * 0xff | KRETS_PROG_MULTI for autotune. */
#define KRETS_PROG_MULTI 0x100
krets_status krets_symbolic_export(const krets_element *elems, int32_t n_elem, int32_t n_unknowns, int32_t mode,
                                   int32_t method, double h, double freq, int32_t ordering,
                                   int32_t which, int64_t *out, int64_t cap, int64_t *len);

#ifdef __cplusplus
}
#endif
#endif /* KRETS_GPU_H */
