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
