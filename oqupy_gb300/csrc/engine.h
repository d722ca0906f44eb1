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
  long long site_base;   // element offset of slot 0 in the site arena
  long long dims_base;   // int2 offset of slot 0 in the dims array
  long long infl_base;   // element offset of influence dk=0 (D*D each, row-major [a][r])
  int ninfl;             // influences available (dk = 0 .. ninfl-1)
  int out_cap;           // ring length of the state output buffer
  long long prop_base;   // element offset of P1 (D*D), P2 (D*D), rho0 (D)
  long long out_base;    // element offset of the state output ring (out_cap * D)
  long long ovr_base;    // element offset of the first-site override influence (D*D)
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
cudaError_t launch_tempo(const TempoLaunch& L, int precision, int grid, int block,
                         cudaStream_t stream);
int tempo_smem_bytes(int precision);

}  // namespace otb
