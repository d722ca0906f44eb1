// Process-tensor sweep (compute_dynamics hot loop), batched over systems.
//
// Reference: compute_dynamics (oqupy/system_dynamics.py:131-165) with
// _apply_system_superoperator (:631-640), _apply_pt_mpos (:654-700) and
// _apply_caps (:643-651).  For a rank-3 PT-MPO tensor T_k[l][r][a] (delta
// between input and output legs, process_tensor.py:346-347) one step of
// system h is
//     u[l][a]  = sum_b P1_hk[a][b] v[l][b]
//     w[r][a]  = sum_l u[l][a] T_k[l][r][a]          (T_k = d * site_k[l][a][r])
//     v'[r][a] = sum_b P2_hk[a][b] w[r][b]
//     rho_h(k+1)[a] = sum_r v'[r][a] cap_{k+1}[r]
// (P1_hk, P2_hk) is entry pidx[h][k] of a table of propagator pairs: a
// time-dependent system has one pair per step, and control operations
// (system_dynamics.py:131-160) are folded into the pairs of their steps on
// the host -- a post-measurement control of step k into P1_hk (P1 post_k),
// a pre-measurement control of step k+1 into P2_hk (pre_{k+1} P2).  One
// launch per step (grid: bond chunks x systems); the host replays the
// launches of a whole sweep as a CUDA graph.  A transform_in / transform_out
// of the process tensor is folded into P1 / P2 on the host.  The read-out
// sum is reproducible bit for bit: a CTA adds its bond chunk's terms in a
// fixed order, and the last CTA of a system to finish (counted after a
// memory fence) adds the chunks' partial sums in chunk order.
#include "common.cuh"
#include "engine.h"

namespace otb {

typedef cx<double> zc;
constexpr int DYN_RB = 32;       // output bond indices per CTA
constexpr int DYN_THREADS = 128;

__global__ void __launch_bounds__(DYN_THREADS) dyn_step_kernel(DynLaunch L) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ int last;
  const int h = blockIdx.y;
  const int k = L.k;
  const int D = L.D;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int2 dm = L.dims[k];
  const int l = dm.x, r = dm.y;
  const zc* A = (const zc*)L.sites + (long long)k * L.slot_elems;
  zc* u = (zc*)dsm;
  zc* w = u + l * D;
  const zc* v = (const zc*)L.vcur + (long long)h * L.cap * D;
  const zc* P1 = (const zc*)L.ptab + (long long)L.pidx[(long long)h * L.pidx_stride + k] * 2 * D * D;
  const zc* P2 = P1 + D * D;
  if (L.fwd_hist && blockIdx.x == 0) {
    // gradient sweep: keep v_k (the state with its bond leg at the start of step k)
    zc* hv = (zc*)L.fwd_hist + ((long long)h * L.hist_steps + k) * L.cap * D;
    for (int idx = tid; idx < l * D; idx += nt) hv[idx] = v[idx];
  }
  for (int idx = tid; idx < l * D; idx += nt) {
    const int ll = idx / D, a = idx - ll * D;
    zc acc = mk<double>(0, 0);
    for (int b = 0; b < D; ++b) cfma(acc, P1[a * D + b], v[ll * D + b]);
    u[idx] = acc;
  }
  __syncthreads();
  const int r0 = blockIdx.x * DYN_RB;
  const int rn = min(DYN_RB, r - r0);
  for (int idx = tid; idx < rn * D; idx += nt) {
    const int a = idx / rn, rr = idx - a * rn;
    zc acc = mk<double>(0, 0);
    for (int ll = 0; ll < l; ++ll) cfma(acc, u[ll * D + a], A[((size_t)ll * D + a) * r + r0 + rr]);
    w[rr * D + a] = cscale(acc, (double)L.d);
  }
  __syncthreads();
  zc* vn = (zc*)L.vnext + (long long)h * L.cap * D;
  const zc* capn = (const zc*)L.caps + (long long)(k + 1) * L.cap;
  zc* cb = w + DYN_RB * D;   // read-out terms of this chunk, [rr][a]
  for (int idx = tid; idx < rn * D; idx += nt) {
    const int rr = idx / D, a = idx - rr * D;
    zc y = mk<double>(0, 0);
    for (int b = 0; b < D; ++b) cfma(y, P2[a * D + b], w[rr * D + b]);
    vn[(size_t)(r0 + rr) * D + a] = y;
    cb[idx] = cmul(y, capn[r0 + rr]);
  }
  __syncthreads();
  zc* part = (zc*)L.partial + (long long)h * L.max_chunks * D;
  if (tid < D) {
    zc acc = mk<double>(0, 0);
    for (int rr = 0; rr < rn; ++rr) acc = acc + cb[rr * D + tid];
    part[blockIdx.x * D + tid] = acc;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) last = (atomicAdd(L.counter + h, 1u) == gridDim.x - 1) ? 1 : 0;
  __syncthreads();
  if (last) {
    if (tid < D) {
      zc acc = mk<double>(0, 0);
      for (int c = 0; c < (int)gridDim.x; ++c) {
        const double2 q = __ldcg(reinterpret_cast<const double2*>(part + c * D + tid));
        acc = acc + mk<double>(q.x, q.y);
      }
      zc* out = (zc*)L.out + (long long)(k + 1) * L.nh * D + (long long)h * D;
      out[tid] = acc;
    }
    if (tid == 0) L.counter[h] = 0u;
  }
}

__global__ void dyn_init_kernel(DynLaunch L, const double* rho0) {
  // v_0 = rho0 (bond dimension 1); rho(0) = rho0 * cap_0[0]
  const int h = blockIdx.x;
  const int D = L.D;
  const zc* r0 = (const zc*)rho0 + (long long)h * D;
  zc* v = (zc*)L.vcur + (long long)h * L.cap * D;
  const zc c0 = ((const zc*)L.caps)[0];
  for (int a = threadIdx.x; a < D; a += blockDim.x) {
    v[a] = r0[a];
    const zc s = cmul(r0[a], c0);
    L.out[2 * ((long long)h * D + a)] = s.x;
    L.out[2 * ((long long)h * D + a) + 1] = s.y;
  }
}

// Adjoint sweep of compute_gradient_and_dynamics (gradient.py:323-425): from
// Y_{k+1} (bond r) to Y_k (bond l) through the transposed step,
//     u[r][c]  = sum_e P2_hk[e][c] Y_{k+1}[r][e]
//     w[l][b]  = sum_r T_k[l][r][b] u[r][b]
//     Y_k[l][a] = sum_b P1_hk[b][a] w[l][b]
// with the same propagator pairs as the forward sweep (controls and
// transforms folded in), so Y_k equals the reference's backward node before
// the pre-measurement control of step k.  Grid: (chunks of DYN_RB left bond
// indices, systems); no reduction across CTAs.
__global__ void __launch_bounds__(DYN_THREADS) dyn_back_step_kernel(DynLaunch L, int l, int r) {
  extern __shared__ __align__(16) unsigned char dsm[];
  const int h = blockIdx.y;
  const int k = L.k;
  const int D = L.D;
  const int tid = threadIdx.x, nt = blockDim.x;
  const zc* A = (const zc*)L.sites + (long long)k * L.slot_elems;
  const zc* P1 = (const zc*)L.ptab + (long long)L.pidx[(long long)h * L.pidx_stride + k] * 2 * D * D;
  const zc* P2 = P1 + D * D;
  const zc* Y = (const zc*)L.back_hist + ((long long)h * (L.hist_steps + 1) + k + 1) * L.cap * D;
  zc* Yk = (zc*)L.back_hist + ((long long)h * (L.hist_steps + 1) + k) * L.cap * D;
  zc* u = (zc*)dsm;              // r * D
  zc* w = u + (size_t)r * D;     // DYN_RB * D
  for (int idx = tid; idx < r * D; idx += nt) {
    const int rr = idx / D, c = idx - rr * D;
    zc acc = mk<double>(0, 0);
    for (int e = 0; e < D; ++e) cfma(acc, P2[e * D + c], Y[rr * D + e]);
    u[idx] = acc;
  }
  __syncthreads();
  const int l0 = blockIdx.x * DYN_RB;
  const int ln = min(DYN_RB, l - l0);
  for (int idx = tid; idx < ln * D; idx += nt) {
    const int li = idx / D, b = idx - li * D;
    const zc* row = A + ((size_t)(l0 + li) * D + b) * r;
    zc acc = mk<double>(0, 0);
    for (int rr = 0; rr < r; ++rr) cfma(acc, row[rr], u[rr * D + b]);
    w[idx] = cscale(acc, (double)L.d);
  }
  __syncthreads();
  for (int idx = tid; idx < ln * D; idx += nt) {
    const int li = idx / D, a = idx - li * D;
    zc acc = mk<double>(0, 0);
    for (int b = 0; b < D; ++b) cfma(acc, P1[b * D + a], w[li * D + b]);
    Yk[(size_t)(l0 + li) * D + a] = acc;
  }
}

// Y_N = the target (bond 1) for every system.
__global__ void dyn_back_init_kernel(DynLaunch L, const double* target) {
  const int h = blockIdx.x;
  const int D = L.D;
  zc* Y = (zc*)L.back_hist + ((long long)h * (L.hist_steps + 1) + L.hist_steps) * L.cap * D;
  const zc* t = (const zc*)target + (long long)h * D;
  for (int a = threadIdx.x; a < D; a += blockDim.x) Y[a] = t[a];
}

// Derivative cores: for every step n and system h,
//     core[n][a][m][e] = sum_{l, r} v_n[l][a] T_n[l][r][m] Y_{n+1}[r][e]
// (T_n = d * site_n, diagonal in its system legs), first
// X[r][a][m] = sum_l v_n[l][a] T_n[l][r][m] in shared memory, then the sum
// over r.  The host maps a core to the reference's derivative tensor (the
// post-measurement control of step n on leg a, the pre-measurement control
// of step n+1 on leg e, the process tensor's transforms on the MPO legs).
// Grid: (steps, systems).
__global__ void __launch_bounds__(DYN_THREADS) dyn_deriv_kernel(DynLaunch L) {
  extern __shared__ __align__(16) unsigned char dsm[];
  const int n = blockIdx.x;
  const int h = blockIdx.y;
  const int D = L.D;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int2 dm = L.dims[n];
  const int l = dm.x, r = dm.y;
  const zc* A = (const zc*)L.sites + (long long)n * L.slot_elems;
  const zc* v = (const zc*)L.fwd_hist + ((long long)h * L.hist_steps + n) * L.cap * D;
  const zc* Y = (const zc*)L.back_hist + ((long long)h * (L.hist_steps + 1) + n + 1) * L.cap * D;
  zc* X = (zc*)dsm;   // r * D * D
  for (int idx = tid; idx < r * D * D; idx += nt) {
    const int rr = idx / (D * D), am = idx - rr * D * D;
    const int a = am / D, m = am - a * D;
    zc acc = mk<double>(0, 0);
    for (int ll = 0; ll < l; ++ll) cfma(acc, v[ll * D + a], A[((size_t)ll * D + m) * r + rr]);
    X[idx] = cscale(acc, (double)L.d);
  }
  __syncthreads();
  zc* out = (zc*)L.deriv + ((long long)h * L.hist_steps + n) * D * D * D;
  for (int idx = tid; idx < D * D * D; idx += nt) {
    const int a = idx / (D * D), me = idx - a * D * D;
    const int m = me / D, e = me - m * D;
    zc acc = mk<double>(0, 0);
    for (int rr = 0; rr < r; ++rr) cfma(acc, X[((size_t)rr * D + a) * D + m], Y[rr * D + e]);
    out[idx] = acc;
  }
}

cudaError_t launch_dyn_back_init(const DynLaunch& L, const double* target, cudaStream_t stream) {
  dyn_back_init_kernel<<<L.nh, 32, 0, stream>>>(L, target);
  return cudaGetLastError();
}

cudaError_t launch_dyn_back_step(const DynLaunch& L, int l, int r, cudaStream_t stream) {
  const int chunks = (l + DYN_RB - 1) / DYN_RB;
  const size_t smem = (size_t)(r * L.D + DYN_RB * L.D) * sizeof(zc);
  dim3 grid(chunks, L.nh);
  dyn_back_step_kernel<<<grid, DYN_THREADS, smem, stream>>>(L, l, r);
  return cudaGetLastError();
}

cudaError_t launch_dyn_deriv(const DynLaunch& L, int num_steps, int max_r, cudaStream_t stream) {
  const size_t smem = (size_t)max_r * L.D * L.D * sizeof(zc);
  cudaError_t e = cudaFuncSetAttribute(dyn_deriv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid(num_steps, L.nh);
  dyn_deriv_kernel<<<grid, DYN_THREADS, smem, stream>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_dyn_step(const DynLaunch& L, int r, cudaStream_t stream) {
  const int chunks = (r + DYN_RB - 1) / DYN_RB;
  const size_t smem = (size_t)(L.cap * L.D + 2 * DYN_RB * L.D) * sizeof(zc);
  dim3 grid(chunks, L.nh);
  dyn_step_kernel<<<grid, DYN_THREADS, smem, stream>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_dyn_init(const DynLaunch& L, const double* rho0, cudaStream_t stream) {
  dyn_init_kernel<<<L.nh, 32, 0, stream>>>(L, rho0);
  return cudaGetLastError();
}

}  // namespace otb
