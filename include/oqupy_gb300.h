/*
 * oqupy_gb300 -- C ABI of the GB300 TEMPO / PT-TEMPO / process-tensor engine.
 *
 * Plain pointers and sizes only.  Complex numbers are complex128 stored as
 * interleaved (re, im) doubles.  Matrices are row-major.  Every function
 * returns an otb_status (0 = OK, < 0 = error; otb_last_error() has the text).
 *
 * Ownership: host input buffers are read during the call only (copied to the
 * device).  The library owns the device memory of a handle until
 * *_destroy.  Outputs go to caller-allocated host buffers.
 * Threading: a handle is not thread-safe; distinct handles may be used from
 * distinct threads/streams.  `stream` is a cudaStream_t (NULL = default).
 *
 * Reference interfaces replaced (OQuPy 0.5.0, paths relative to the project):
 *   otb_tempo_*  -> oqupy/backends/tempo_backend.py:577-626
 *                   (TempoBackend.__init__/initialize/compute_step), batched
 *   otb_pt_*     -> oqupy/backends/pt_tempo_backend.py:56-316
 *                   (PtTempoBackend.__init__/initialize/compute_step/
 *                    get_mpo_tensor/update_process_tensor)
 *   otb_dyn_*    -> oqupy/system_dynamics.py:41-182, 631-700
 *                   (compute_dynamics hot loop over a process tensor),
 *                   with controls and time-dependent systems, the runs of
 *                   compute_correlations_nt (:791-990), the sweep of
 *                   compute_dynamics_with_field (:184-476) and the sweeps
 *                   of compute_gradient_and_dynamics (gradient.py:169-437)
 *   otb_mlp_*    -> no reference counterpart (learned screening surrogate)
 */
#ifndef OQUPY_GB300_H
#define OQUPY_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t otb_status;

#define OTB_OK 0
#define OTB_ERR_INVALID_ARG (-1)
#define OTB_ERR_OOM (-2)
#define OTB_ERR_CUDA (-3)
#define OTB_ERR_NO_CONVERGENCE (-4)
#define OTB_ERR_TIMEOUT (-5)
#define OTB_ERR_NONFINITE (-6)
#define OTB_ERR_CHI_OVERFLOW (-7)

/* Both forms split every bond of >= 8 columns by a rank-revealing pivoted
 * Householder QR followed by one-sided Jacobi on the reduced factor, and
 * keep site tensors in complex128; column norms, the descending sort, the
 * tail sums and the epsrel rank decision are FP64 in both.
 * COMPLEX128: QR, Jacobi and every contraction in FP64.
 * MIXED: QR, Jacobi rotations and the contractions (theta, U / carry
 * products, absorb) in double-float arithmetic (pairs of floats, ~48
 * significant bits) on the FP32 pipe; a split whose double-float sweeps do
 * not settle is finished by FP64 sweeps. */
#define OTB_PRECISION_COMPLEX128 0
#define OTB_PRECISION_MIXED 1

/* ------------------------------------------------------------------ TEMPO */

typedef struct otb_tempo otb_tempo;

typedef struct {
  int32_t precision;   /* OTB_PRECISION_* */
  int32_t chi_cap;     /* bond-dimension capacity of every site, chi_cap * D <= 1152 */
  int32_t out_cap;     /* states kept per instance (ring), >= 2 */
  int32_t grid;        /* CTAs per launch, 0 = 3 per SM */
  int32_t block;       /* threads per CTA (64..512, multiple of 32), 0 = 256 */
  int32_t smem_kb;     /* dynamic shared memory per CTA for working matrices
                          (KiB, <= 200), 0 = 56 */
  double qr_cut;       /* relative cut of the rank-revealing QR that precedes
                          the Jacobi SVD of every split of >= 8 columns: the
                          factorisation stops once the remaining block's
                          Frobenius norm is below qr_cut * |R_00| (its squared
                          norm joins the truncation tail).  0 = default:
                          1e-14 (complex128), min(1e-3 epsrel, 1e-9) (mixed) */
} otb_tempo_config;

typedef struct {
  int32_t hs_dim;             /* d; Liouville dimension D = d*d (<= 9) */
  int32_t dkmax;              /* memory length; < 0 = full memory (grows) */
  double epsrel;              /* relative SVD truncation tolerance */
  int32_t n_influences;       /* influence matrices given (dk = 0..n-1) */
  const double* influences;   /* n_influences * D * D complex, [dk][a][r],
                                 coupling eigenbasis; dk=0 is diagonal */
  const double* prop1;        /* D*D: first half-step, eigenbasis-folded  */
  const double* prop2;        /* D*D: second half-step, eigenbasis-folded */
  const double* rho0;         /* D: vectorised initial state */
  int32_t max_sites;          /* site-slot hint (full memory), 0 = auto */
} otb_tempo_instance;

typedef struct {
  int32_t step;       /* completed steps */
  int32_t status;     /* 0 or a negative otb_status */
  int32_t nsites;     /* MPS sites incl. the trailing propagator node */
  int32_t max_bond;   /* largest bond dimension after the last step */
  double log_scale;   /* log of a norm factored out of the MPS (0 here) */
  int32_t splits;     /* truncated SVD splits done so far */
  int32_t sweeps64;   /* FP64 Jacobi sweeps done so far */
  int32_t sweeps32;   /* double-float Jacobi sweeps done so far (mixed) */
  double flops_alg;   /* algorithmic flops done so far: per split of a complex
                         R x N matrix (R >= N) 4 (6 R N^2 + 20 N^3), plus
                         8 flops per complex multiply-add of the contractions */
  int64_t t_begin_ns; /* device clock (ns, %globaltimer) at which the last
                         launch's CTA took this instance, */
  int64_t t_end_ns;   /* ... and at which it finished the launch's steps:
                         the launch's timeline, for critical-path analysis */
} otb_tempo_info;

/* Replaces TempoBackend.__init__ + initialize (tempo_backend.py:583-617). */
otb_status otb_tempo_create(const otb_tempo_config* cfg, int32_t n_instances,
                            const otb_tempo_instance* instances,
                            otb_tempo** out);
void otb_tempo_destroy(otb_tempo* h);
/* Replaces nsteps calls of TempoBackend.compute_step (tempo_backend.py:619-626)
 * for every instance of the handle. */
otb_status otb_tempo_advance(otb_tempo* h, int32_t nsteps, void* stream);
/* Launch shape of the next advances (no reference counterpart: the
 * reference has no launch): block threads per CTA (64..512, 0 = 256),
 * smem_kb dynamic shared memory per CTA (<= 200, 0 = 56), grid CTAs (0 = 3
 * per SM for blocks up to 256 threads, 1 per SM above; capped at the grid
 * the handle's workspace was allocated for).  Used by the per-bond-bucket
 * launch-shape tuner. */
otb_status otb_tempo_set_launch(otb_tempo* h, int32_t block, int32_t smem_kb, int32_t grid);
/* States of steps [first_step, first_step+count) of one instance, each D
 * complex; steps must still be held by the output ring (step 0 = rho0). */
otb_status otb_tempo_read_states(otb_tempo* h, int32_t inst, int32_t first_step,
                                 int32_t count, double* out);
/* All instances, steps [first_step, first_step+count): out[inst][k][D]. */
otb_status otb_tempo_read_all_states(otb_tempo* h, int32_t first_step,
                                     int32_t count, double* out);
otb_status otb_tempo_get_info(otb_tempo* h, int32_t inst, otb_tempo_info* info);
/* Bond dimensions of the current MPS (sites - 1 values); returns the count
 * through *count. */
otb_status otb_tempo_bond_dims(otb_tempo* h, int32_t inst, int32_t* out,
                               int32_t cap, int32_t* count);
/* Influence matrix for one dk (grows storage; full-memory runs append one
 * per step, tempo_backend.py:487-497). */
otb_status otb_tempo_set_influence(otb_tempo* h, int32_t inst, int32_t dk,
                                   const double* mat);
/* Propagators for the next step (time-dependent systems, tempo.py:400-435). */
otb_status otb_tempo_set_propagators(otb_tempo* h, int32_t inst,
                                     const double* prop1, const double* prop2);
/* Propagators of every instance for the next step in one call: p1, p2 hold
 * the instances' D x D matrices packed in instance order (eigenbasis-folded
 * like otb_tempo_set_propagators).  Ordered on `stream` before the next
 * otb_tempo_advance on that stream; from page-locked host memory the copy is
 * asynchronous and the buffers must stay valid until it completes.  The
 * batched form of the per-step propagators(step) call of
 * TempoBackend.compute_step (tempo_backend.py:619-626). */
otb_status otb_tempo_set_all_propagators(otb_tempo* h, const double* prop1,
                                         const double* prop2, void* stream);
/* Influence replacing the oldest window site in the next step only
 * (add_correlation_time, tempo_backend.py:503-517). */
otb_status otb_tempo_set_first_influence(otb_tempo* h, int32_t inst,
                                         const double* mat);
/* Grow the site ring of every instance to at least nslots slots. */
otb_status otb_tempo_reserve_sites(otb_tempo* h, int32_t nslots);

/* --------------------------------------------------------------- PT-TEMPO */

typedef struct otb_pt otb_pt;

typedef struct {
  int32_t precision;   /* OTB_PRECISION_* */
  int32_t chi_cap;     /* bond-dimension capacity of every site, chi_cap * D <= 1152 */
  int32_t grid;        /* CTAs per launch, 0 = 2 per SM */
  double qr_cut;       /* as otb_tempo_config.qr_cut; 0 = default: 1e-14
                          (complex128), min(1e-3 epsrel, 1e-11) (mixed) */
} otb_pt_config;

typedef struct {
  int32_t hs_dim;             /* d (D = d*d <= 9) */
  int32_t num_steps;          /* process-tensor length (>= 2) */
  int32_t dkmax;              /* memory length; num_infl = min(num_steps, dkmax+1) >= 2 */
  double epsrel;
  const double* influences;   /* num_infl * D * D complex, dk = 0..num_infl-1,
                                 coupling eigenbasis, [dk][a][r] */
  const double* neg_influences; /* (num_steps+1) * D * D indexed by step for the
                                   grow-phase dk = -step influences, or NULL */
} otb_pt_instance;

typedef struct {
  int32_t step;       /* 0 = not initialised; num_steps = done */
  int32_t status;
  int32_t num_steps;
  int32_t max_bond;
  int32_t splits;
  int32_t sweeps64;
  int32_t sweepsff;
  int32_t caps_done;
  double flops_alg;
} otb_pt_info;

/* Replaces PtTempoBackend.__init__ (pt_tempo_backend.py:56-93), batched. */
otb_status otb_pt_create(const otb_pt_config* cfg, int32_t n_instances,
                         const otb_pt_instance* instances, otb_pt** out);
void otb_pt_destroy(otb_pt* h);
/* Replaces PtTempoBackend.initialize (first call) and nsteps calls of
 * compute_step (pt_tempo_backend.py:105-282); computes the caps
 * (process_tensor.py:380-406) once the build is complete. */
otb_status otb_pt_advance(otb_pt* h, int32_t nsteps, void* stream);
otb_status otb_pt_get_info(otb_pt* h, int32_t inst, otb_pt_info* info);
/* num_steps+1 bond dimensions (process_tensor.py:367-378). */
otb_status otb_pt_bond_dims(otb_pt* h, int32_t inst, int32_t* out, int32_t cap);
/* Rank-3 PT-MPO tensor of one step, [past bond][future bond][D] complex,
 * already multiplied by d (pt_tempo_backend.py:284-307); dims[0..1] get the
 * bond dimensions, out must hold cap_elems complex values. */
otb_status otb_pt_get_tensor(otb_pt* h, int32_t inst, int32_t step, double* out,
                             int64_t cap_elems, int32_t* dims);
/* Cap vector of one step (process_tensor.py:358-365); *count gets its length. */
otb_status otb_pt_get_cap(otb_pt* h, int32_t inst, int32_t step, double* out,
                          int32_t cap, int32_t* count);

/* ------------------------------------------------------ process-tensor sweep */

/* compute_dynamics over one built process tensor for n_systems systems at
 * once (system_dynamics.py:41-182 with no controls, record_all=True):
 * prop1/prop2 are n_systems * D * D complex half-step propagators (with any
 * transform_in / transform_out of the process tensor folded in: P1 <- Tin^T P1,
 * P2 <- P2 Tout^T), rho0 is n_systems * D, out receives
 * (num_steps+1) * n_systems * D complex.  The num_steps launches are replayed
 * as one CUDA graph. */
otb_status otb_dyn_run(otb_pt* h, int32_t inst, int32_t n_systems,
                       const double* prop1, const double* prop2,
                       const double* rho0, int32_t num_steps, double* out,
                       void* stream);

/* The same sweep with propagators that change from step to step and from
 * system to system: compute_dynamics (system_dynamics.py:41-182) for
 * time-dependent systems and with control operations, and the runs that
 * compute_correlations_nt (system_dynamics.py:791-990) makes, one system
 * slot per run.  props holds n_props pairs (P1 then P2, each D * D complex,
 * transforms folded in as for otb_dyn_run); prop_index (n_systems *
 * num_steps, host) names the pair system h uses at step k; a control
 * operation is folded into the pairs on the host (a post-measurement
 * control C of step k: P1 <- P1 C at step k; a pre-measurement control of
 * step k + 1: P2 <- C P2 at step k; one of step 0: applied to rho0).
 * Indices outside [0, n_props) are rejected before any device work. */
otb_status otb_dyn_run_steps(otb_pt* h, int32_t inst, int32_t n_systems,
                             const double* props, int32_t n_props,
                             const int32_t* prop_index, const double* rho0,
                             int32_t num_steps, double* out, void* stream);

/* A sweep advanced one step per call (compute_dynamics_with_field,
 * system_dynamics.py:184-476, where each step's propagators depend on a
 * field computed from the states so far).  create: n_systems slots on
 * process tensor inst (which must outlive the session), rho0 n_systems * D
 * complex.  step: props holds this step's n_systems pairs (P1 then P2, D * D
 * complex each, transforms and controls folded in as for otb_dyn_run_steps);
 * state_out receives the n_systems * D states after the step.  state: the
 * states of an earlier step (0 .. steps done). */
typedef struct otb_dyn_session otb_dyn_session;
otb_status otb_dyn_session_create(otb_pt* h, int32_t inst, int32_t n_systems,
                                  const double* rho0, otb_dyn_session** out);
otb_status otb_dyn_session_step(otb_dyn_session* s, const double* props,
                                double* state_out, void* stream);
otb_status otb_dyn_session_state(otb_dyn_session* s, int32_t step, double* state_out);
void otb_dyn_session_destroy(otb_dyn_session* s);

/* The forward and adjoint sweeps of compute_gradient_and_dynamics
 * (gradient.py:169-437) for n_systems systems on one process tensor, with
 * propagator pairs as in otb_dyn_run_steps.  num_steps must end where the
 * process tensor's bond closes (its full length).  out_states receives
 * (num_steps+1) * n_systems * D complex (the dynamics); out_cores
 * n_systems * num_steps * D^3 complex: per step n the core
 * C[a][m][e] = sum_{l,r} v_n[l][a] T_n[l][r][m] Y_{n+1}[r][e] of the
 * derivative tensor, v_n the state with its bond leg at the start of step n
 * and Y_{n+1} the adjoint vector (the target swept back through steps
 * num_steps-1 .. n+1); the reference's tensor follows on the host by
 * applying the post-measurement control of step n to leg a, the transposed
 * pre-measurement control of step n+1 to leg e and the process tensor's
 * transforms to leg m. */
otb_status otb_dyn_gradient(otb_pt* h, int32_t inst, int32_t n_systems,
                            const double* props, int32_t n_props,
                            const int32_t* prop_index, const double* rho0,
                            const double* target, int32_t num_steps,
                            double* out_states, double* out_cores, void* stream);

/* ----------------------------------------------- allocation-free TEMPO */

/* No counterpart in the reference.  For callers that cannot allocate device
 * memory through this library -- a host framework whose memory pool owns
 * every device allocation, or code running where cudaMalloc is not allowed:
 * the caller allocates all device buffers below, and the TEMPO step's
 * working memory comes from a fixed device array inside the library
 * (1 MiB, present on every GPU that loads the library until exit), which
 * limits bonds to chi_cap * D <= OTB_TEMPO_STATIC_MAX_CHI_D.
 *
 * One instance, one CTA.  Every call looks up the array's device address
 * for the current device and context (cudaGetSymbolAddress, which allocates
 * nothing); the first call on a device also loads the library's kernels
 * there and should therefore come before any stream capture.  Calls share
 * the array: calls that overlap on the GPU race, so issue them on one
 * stream (or otherwise serialise them).  Nothing in the array needs to
 * start at zero.  The MPS buffer must be zeroed by the caller before the
 * first call; it then carries the instance between calls.  The function
 * calls no cudaMalloc or cudaFree.
 *
 * Failures inside a step (a bond beyond chi_cap, a split that does not
 * converge, a non-finite value) are reported through status_out, written
 * on the stream by every call: [0] status (0 or a negative otb_status),
 * [1] steps completed by this call = rows of states_out written (the rest
 * are left untouched), [2] steps completed by the instance in total,
 * [3] largest bond dimension after the last completed step.  After a
 * nonzero status the MPS buffer holds a partly updated step: later calls
 * complete no step and report the same status until the caller zeroes the
 * buffer, which restarts the instance from rho0. */
#define OTB_TEMPO_STATIC_MAX_CHI_D 128
/* bytes of the MPS buffer: state header, dims, (dkmax+2) site slots */
#define OTB_TEMPO_STATIC_MPS_BYTES(hs_dim, dkmax, chi_cap)                          \
  (256LL + ((((long long)(dkmax) + 2) * 8 + 255) / 256) * 256 +                     \
   ((long long)(dkmax) + 2) * (long long)(chi_cap) * (hs_dim) * (hs_dim) *          \
       (long long)(chi_cap) * 16)

typedef struct {
  int32_t hs_dim;            /* d (D = d*d) */
  int32_t dkmax;             /* memory length (>= 0) */
  double epsrel;
  int32_t chi_cap;           /* bond capacity, chi_cap * D <= 128 */
  int32_t precision;         /* OTB_PRECISION_* */
  const double* influences;  /* device: (dkmax+1) * D * D complex, as otb_tempo_instance */
  const double* props;       /* device: P1 then P2 (eigenbasis-folded), 2 * D * D complex */
  const double* rho0;        /* device: D complex (read on the first call) */
  void* mps;                 /* device: OTB_TEMPO_STATIC_MPS_BYTES bytes, zeroed before
                                the first call */
  int64_t mps_bytes;
  double* states_out;        /* device: nsteps * D complex, states of this call's steps */
  int32_t* status_out;       /* device: 4 int32 (see above), written by every call */
} otb_tempo_static_io;

/* Advance one TEMPO instance by nsteps without allocating. */
otb_status otb_tempo_advance_static(const otb_tempo_static_io* io, int32_t nsteps,
                                    void* stream);

/* -------------------------------------------------- MLP surrogate kernels */

/* No counterpart in the reference (the learned screening part of this
 * project).  All pointers are device pointers owned by the caller; bf16
 * matrices are row-major with K contiguous.
 *
 * C[M][N] = A[M][K] B[N][K]^T on the 5th-generation tensor cores (tcgen05,
 * bf16 in, FP32 accumulate in TMEM), fused epilogue:
 *   0: out = C (+ bias)       1: z = C + bias -> z_out, out = gelu(z)
 *   2: out = C * gelu'(z_in)
 * out_f32 and/or out_bf16 receive the result; *err is set to 1 if a
 * bounded wait on the tensor-core completion barrier timed out. */
otb_status otb_mlp_gemm(const void* A, const void* B, int32_t M, int32_t N, int32_t K,
                        const float* bias, int32_t epilogue, const float* z_in,
                        float* z_out, float* out_f32, void* out_bf16, int32_t* err,
                        void* stream);
/* out[C][R] = in[R][C] (bf16) */
otb_status otb_mlp_transpose_bf16(const void* in, void* out, int32_t R, int32_t C,
                                  void* stream);
otb_status otb_mlp_f32_to_bf16(const float* in, void* out, int64_t n, void* stream);
/* out[c] = sum_r in[r][c] (FP32) */
otb_status otb_mlp_colsum(const float* in, float* out, int32_t R, int32_t C, void* stream);
/* g = 2 (y - t) / n (FP32 and bf16); *loss += sum (y - t)^2 */
otb_status otb_mlp_mse_grad(const float* y, const float* t, float* g_f32, void* g_bf16,
                            int64_t n, double* loss, void* stream);
/* AdamW step on FP32 master weights (bias-corrected, decoupled weight decay);
 * refreshes the bf16 copy when w_bf16 is not NULL */
otb_status otb_mlp_adamw(float* w, const float* g, float* m, float* v, void* w_bf16,
                         int64_t n, float lr, float beta1, float beta2, float eps,
                         float weight_decay, int32_t step, void* stream);

/* Surrogate output baseline (no reference counterpart): adds to y[B][3][nsteps]
 * the Bloch vector of the bath-free system H = Omega/2 sx + eps/2 sz started
 * in (0, 0, 1) at times dt, 2 dt, ..., nsteps dt; omega_eps[B][2] holds
 * (Omega, eps) per point.  Device pointers. */
otb_status otb_mlp_bloch_free_add(float* y, const float* omega_eps, int32_t B, int32_t nsteps,
                                  float dt, void* stream);

/* Measured FMA-pipe throughput of this GPU (TFLOP/s, 2 flops per FMA):
 * precision 0 = FP64 (DFMA), 1 = FP32 (FFMA).  Used as the roofline peak of
 * the Jacobi kernels, which run on these pipes. */
otb_status otb_measure_fma_peak(int32_t precision, double* tflops);

const char* otb_last_error(void);
int32_t otb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* OQUPY_GB300_H */
