// Internal host/device layout of the batched TEMPO engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace otb {

// Static description of one instance (device array, written by the host).
struct InstDev {
  int D;             // Liouville dimension d*d
  int dkmax;         // memory sites dkmax+1 (very large for full memory)
  int cap;           // bond-dimension capacity of every site slot
  int nslots;        // ring slots for MPS sites (>= sites + 1)
  double epsrel;     // relative truncation tolerance
  float qr_delta;    // relative cut of the split's QR (<= 0: default by precision)
  long long site_base;   // element offset of slot 0 in the site arena
  long long dims_base;   // int2 offset of slot 0 in the dims array
  long long infl_base;   // element offset of influence dk=0 (D*D each, row-major [a][r])
  int ninfl;             // influences available (dk = 0 .. ninfl-1)
  int out_cap;           // ring length of the state output buffer
  long long prop_base;   // element offset of P1 (D*D), P2 (D*D), rho0 (D)
  long long out_base;    // element offset of the state output ring (out_cap * D)
  long long ovr_base;    // element offset of the first-site override influence (D*D)
  int out_origin;        // state of step s goes to ring entry (s - out_origin) % out_cap
};

// Mutable per-instance state (device array).
struct InstState {
  int step;        // completed TEMPO steps
  int nsites;      // MPS sites including the trailing propagator node
  int head;        // slot of the oldest site
  int status;      // 0 ok, < 0 error code
  double log_scale;
  int max_bond;    // largest bond dimension seen in the last step
  int ovr_active;  // 1: use the override influence for the first window site
  int splits;      // truncated SVD splits done so far
  int sweeps64;    // FP64 Jacobi sweeps done so far
  int sweeps32;    // double-float Jacobi sweeps done so far (mixed form)
  double flops_alg;  // algorithmic flops done so far (R-SVD count + contractions)
  long long t_begin_ns;  // device clock (globaltimer) when the last launch took this instance
  long long t_end_ns;    // ... and when it finished its steps
};

struct TempoLaunch {
  int n;                     // instances
  const InstDev* inst;
  InstState* state;
  int2* dims;                // (l, r) per slot
  void* sites;               // complex128 arena
  const double* infl;        // complex128 interleaved
  const double* props;       // complex128 interleaved
  double* out;               // complex128 interleaved
  void* work;                // per-CTA workspace (bytes)
  long long work_stride;     // bytes per CTA in `work`
  long long wcap;            // complex elements of one matrix buffer
  int* queue;                // work-queue counter (reset before each launch)
  const int* order;          // instance processing order
  int nsteps;                // steps to advance
  int smem_bytes;            // capacity of the dynamic shared buffer
};

// Per-CTA workspace: three FP64 complex matrices of wcap elements (W, theta
// copy / temporaries, carry) and one double-float complex one (mixed form).
inline long long tempo_work_bytes(long long wcap) { return wcap * (3 * 16 + 16); }

// precision: 0 = complex128 (FP64 Jacobi), 1 = mixed (double-float Jacobi
// on the FP32 pipe; FP64 sites, contractions, rotation angles, norms, rank
// decisions and read-out)
cudaError_t launch_tempo_order(InstState* state, int* order, int n, cudaStream_t stream);
cudaError_t launch_tempo(const TempoLaunch& L, int precision, int grid, int block,
                         int smem_bytes, cudaStream_t stream);
int tempo_smem_bytes(int precision);

// ---------------------------------------------------------------- PT-TEMPO

struct PtDev {
  int D;              // Liouville dimension
  int d;              // Hilbert dimension
  int num_steps;      // MPS length at the end of the build
  int num_infl;       // min(num_steps, dkmax + 1)
  int cap;            // bond-dimension capacity per site
  int has_neg;        // grow-phase influences for dk = -step supplied
  double epsrel;
  float qr_delta;     // relative cut of the split's QR (<= 0: default by precision)
  long long site_base;  // num_steps slots of cap * D * cap
  long long dims_base;  // num_steps int2
  long long infl_base;  // num_infl * D * D, dk = 0 .. num_infl-1
  long long neg_base;   // (num_steps + 1) * D * D, indexed by step
  long long caps_base;  // (num_steps + 1) * cap
};

struct PtState {
  int step;      // 0 = not initialised, then 1 .. num_steps
  int nsites;
  int mpo_len;
  int status;
  int splits;
  int sweeps64;
  int sweepsff;
  int caps_done;
  double flops_alg;
};

struct PtLaunch {
  int n;
  const PtDev* inst;
  PtState* state;
  int2* dims;
  void* sites;
  const double* infl;
  const double* neg;
  double* caps;
  void* work;
  long long work_stride;  // bytes per CTA
  long long wcap;         // complex elements of one matrix buffer
  int* queue;
  const int* order;
  int nsteps;
  int smem_bytes;
};

// Per-CTA PT workspace: four FP64 complex matrices (working matrix, U,
// carry, theta) and one double-float matrix.
inline long long pt_work_bytes(long long wcap) { return wcap * (4 * 16 + 16); }

cudaError_t launch_pt(const PtLaunch& L, int precision, int grid, int block, cudaStream_t stream);

// ------------------------------------------------------- process-tensor sweep

struct DynLaunch {
  int nh;             // systems swept together
  int D;
  int d;
  const double* sites;  // PT sites of one instance (complex128, [l][a][r] per slot)
  long long slot_elems;
  const int2* dims;     // per step (l, r)
  const double* caps;   // (num_steps + 1) * cap
  int cap;
  const double* ptab;   // propagator pairs (P1 then P2, D * D complex each)
  const int* pidx;      // nh * pidx_stride: pair of system h at step k
  int pidx_stride;
  double* vcur;         // nh * cap * D
  double* vnext;
  double* out;          // (num_steps + 1) * nh * D
  double* partial;      // nh * max_chunks * D complex: per-chunk read-out sums
  unsigned int* counter;  // nh counters of finished chunks (zero between steps)
  int max_chunks;
  int k;                // step
  // gradient sweeps (otb_dyn_gradient; null / unused otherwise)
  double* fwd_hist;     // nh * hist_steps * cap * D: v_k at the start of step k
  double* back_hist;    // nh * (hist_steps + 1) * cap * D: adjoint vectors Y_k
  double* deriv;        // nh * hist_steps * D^3: per-step derivative cores
  int hist_steps;
};

cudaError_t launch_dyn_step(const DynLaunch& L, int r, cudaStream_t stream);
cudaError_t launch_dyn_init(const DynLaunch& L, const double* rho0, cudaStream_t stream);
cudaError_t launch_dyn_back_init(const DynLaunch& L, const double* target, cudaStream_t stream);
cudaError_t launch_dyn_back_step(const DynLaunch& L, int l, int r, cudaStream_t stream);
cudaError_t launch_dyn_deriv(const DynLaunch& L, int num_steps, int max_r, cudaStream_t stream);

}  // namespace otb
