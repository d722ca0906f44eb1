// Batched TEMPO step kernel (sm_103a).
//
// One CTA advances one TEMPO instance by whole time steps; CTAs pull
// instances from a work queue (longest first), so instances with very
// different memory lengths and bond dimensions share one launch.
//
// Per step (reference: BaseTempoBackend.compute_system_step,
// oqupy/backends/tempo_backend.py:439-575):
//   1. first half-step propagator on the newest site          (:521-529)
//   2. trace out the oldest site once the MPS outgrows the window (:531-537)
//   3. zip-up of the influence MPO, site by site: contraction + truncated
//      SVD, S V^H carried right                   (node_array.py:503-552)
//   4. right-to-left truncated SVD sweep          (node_array.py:274-296)
//   5. second half-step propagator appended as a new site     (:555-558)
//   6. read-out: all sites summed with the all-ones north vector (:560-573)
//
// The reference's MPO sites are rank-4 delta tensors built densely with
// create_delta (util.py:30-57); here the delta structure is used directly:
// theta[(x,a),(r,m)] = I_dk[a,m] * sum_c C[x,c,m] A[c,a,r].  The basis
// rotation the reference applies to the dk=0 site (tempo_backend.py:419-424)
// is folded into the propagators on the host (P1 <- U_dag P1, P2 <- P2 U_sup),
// so every influence here is in the coupling eigenbasis.
//
// Site tensors live in a per-instance ring of fixed-capacity slots, layout
// [l][a][r] (row-major).  That layout is also the column-major (a r) x l
// matrix the right-to-left sweep factorises, so sweep splits need no
// reshuffle.
#include <math.h>

#include "engine.h"
#include "jacobi.cuh"

namespace otb {

constexpr int TEMPO_THREADS = 256;
constexpr int NMAX = 1152;   // max columns of a split (D * cap <= 9 * 128)
constexpr int VMAX = 128;    // max bond dimension held by the read-out vector (chi_cap <= 128)

template <typename T>
struct Bufs {
  cx<T>* sites;
  int2* dims;
  const cx<double>* infl;
  const cx<double>* props;
  cx<double>* out;
  cx<T>* W;    // working matrix (shared or global)
  cx<T>* Wg;   // global fallback for W
  cx<T>* Tg;   // global scratch (theta copy / temporaries)
  cx<T>* Cg;   // carry S V^H
  cx<T>* Ws;   // dynamic shared buffer
  int smem_elems;
};

struct SharedStep {
  InstState st;
  JacobiShared jsh;
  double norm[NMAX];
  int perm[NMAX];
  cx<double> v[2][VMAX];
  int inst;
};

template <typename T>
__device__ __forceinline__ cx<T> to_t(cx<double> a) {
  return mk<T>((T)a.x, (T)a.y);
}
template <typename T>
__device__ __forceinline__ cx<double> to_d(cx<T> a) {
  return mk<double>((double)a.x, (double)a.y);
}

template <typename T, bool RESCALE>
__device__ void tempo_step(const TempoLaunch& L, const InstDev& I, int i, Bufs<T>& b,
                           SharedStep& sh) {
  const int tid = threadIdx.x;
  const int nt = blockDim.x;
  if (tid == 0) sh.st = L.state[i];
  __syncthreads();
  if (sh.st.status != ST_OK) return;
  const int D = I.D;
  const int cap = I.cap;
  const long long slot_elems = (long long)cap * D * cap;
  const int step = sh.st.step + 1;
  const long long window = min((long long)step, (long long)I.dkmax + 1);
  cx<T>* const sites = b.sites + I.site_base;
  int2* const dims = b.dims + I.dims_base;
  const cx<double>* P1 = b.props + I.prop_base;
  const cx<double>* P2 = P1 + D * D;

#define SLOT(k) ((sh.st.head + (k)) % I.nslots)
#define SITE(k) (sites + (long long)SLOT(k) * slot_elems)
#define DIMS(k) (dims[SLOT(k)])

  // 1. first half-step propagator on the newest site: A[l][b][0] = sum_a P1[b][a] A[l][a][0]
  {
    const int k = sh.st.nsites - 1;
    cx<T>* A = SITE(k);
    const int l = DIMS(k).x;
    for (int idx = tid; idx < l * D; idx += nt) {
      const int ll = idx / D, bb = idx - ll * D;
      cx<double> acc = mk<double>(0, 0);
      for (int a = 0; a < D; ++a) cfma(acc, P1[bb * D + a], to_d(A[ll * D + a]));
      b.Tg[idx] = to_t<T>(acc);
    }
    __syncthreads();
    for (int idx = tid; idx < l * D; idx += nt) A[idx] = b.Tg[idx];
    __syncthreads();
  }

  // 2. trace out the oldest site (sum_north = ones) and merge into the next
  if (sh.st.nsites > window) {
    cx<T>* A0 = SITE(0);
    cx<T>* A1 = SITE(1);
    const int r0 = DIMS(0).y;
    const int r1 = DIMS(1).y;
    for (int c = tid; c < r0; c += nt) {
      cx<double> acc = mk<double>(0, 0);
      for (int a = 0; a < D; ++a) acc = acc + to_d(A0[a * r0 + c]);
      sh.v[0][c] = acc;
    }
    __syncthreads();
    for (int idx = tid; idx < D * r1; idx += nt) {
      const int a = idx / r1, rr = idx - a * r1;
      cx<double> acc = mk<double>(0, 0);
      for (int c = 0; c < r0; ++c) cfma(acc, sh.v[0][c], to_d(A1[((long long)c * D + a) * r1 + rr]));
      b.Tg[idx] = to_t<T>(acc);
    }
    __syncthreads();
    for (int idx = tid; idx < D * r1; idx += nt) A1[idx] = b.Tg[idx];
    __syncthreads();
    if (tid == 0) {
      dims[(sh.st.head + 1) % I.nslots] = make_int2(1, r1);
      sh.st.head = (sh.st.head + 1) % I.nslots;
      sh.st.nsites -= 1;
    }
    __syncthreads();
  }

  const int K = sh.st.nsites;
  // 3. zip-up
  int cxd = 1, ccd = 1;
  for (int k = 0; k < K; ++k) {
    cx<T>* A = SITE(k);
    const int2 dA = DIMS(k);
    const int r = dA.y;
    const int dk = K - 1 - k;
    const cx<double>* Im = (k == 0 && sh.st.ovr_active) ? (b.props + I.ovr_base)
                                                         : (b.infl + I.infl_base + (long long)dk * D * D);
    const int m = cxd * D;
    const int n = r * D;
    const cx<T>* C = b.Cg;
    if (k == K - 1) {
      for (int idx = tid; idx < m * n; idx += nt) {
        const int row = idx / n, col = idx - row * n;
        const int x = row / D, a = row - x * D;
        const int rr = col / D, mr = col - rr * D;
        cx<T> acc = mk<T>(0, 0);
        if (k == 0) {
          acc = A[a * r + rr];
        } else {
          for (int c = 0; c < ccd; ++c)
            cfma(acc, C[(long long)x * (ccd * D) + c * D + mr], A[((long long)c * D + a) * r + rr]);
        }
        b.Tg[idx] = cmul(to_t<T>(Im[a * D + mr]), acc);
      }
      __syncthreads();
      for (int idx = tid; idx < m * n; idx += nt) A[idx] = b.Tg[idx];
      if (tid == 0) dims[SLOT(k)] = make_int2(cxd, n);
      __syncthreads();
      break;
    }
    const bool trans = n > m;
    cx<T>* W = ((long long)m * n <= b.smem_elems) ? b.Ws : b.Wg;
    for (int idx = tid; idx < m * n; idx += nt) {
      const int col = idx / m, row = idx - col * m;
      const int x = row / D, a = row - x * D;
      const int rr = col / D, mr = col - rr * D;
      cx<T> acc = mk<T>(0, 0);
      if (k == 0) {
        acc = A[a * r + rr];
      } else {
        for (int c = 0; c < ccd; ++c)
          cfma(acc, C[(long long)x * (ccd * D) + c * D + mr], A[((long long)c * D + a) * r + rr]);
      }
      const cx<T> th = cmul(to_t<T>(Im[a * D + mr]), acc);
      b.Tg[idx] = th;
      if (!trans)
        W[idx] = th;
      else
        W[col + (long long)row * n] = cconj(th);
    }
    __syncthreads();
    const int kk = trans ? jacobi_truncate<T>(W, n, m, n, I.epsrel, sh.norm, sh.perm, &sh.jsh)
                         : jacobi_truncate<T>(W, m, n, m, I.epsrel, sh.norm, sh.perm, &sh.jsh);
    if (sh.jsh.status != ST_OK || kk > cap) {
      if (tid == 0) sh.st.status = (sh.jsh.status != ST_OK) ? sh.jsh.status : ST_CHI_OVERFLOW;
      __syncthreads();
      break;
    }
    const double smax = sh.norm[sh.perm[0]];
    const T cscal = RESCALE ? (T)(1.0 / smax) : (T)1;
    cx<T>* Cn = b.Cg;  // new carry overwrites the old one (old one no longer read)
    if (!trans) {
      // U = W[:, perm] / s  -> site (cxd, D, kk);  carry = U^H theta
      for (int idx = tid; idx < m * kk; idx += nt) {
        const int row = idx / kk, j = idx - row * kk;
        const int pj = sh.perm[j];
        const T inv = (T)(1.0 / sh.norm[pj]);
        A[idx] = cscale(W[(long long)pj * m + row], inv);
      }
      for (int idx = tid; idx < kk * n; idx += nt) {
        const int j = idx / n, col = idx - j * n;
        const int pj = sh.perm[j];
        const cx<T>* u = W + (long long)pj * m;
        const cx<T>* th = b.Tg + (long long)col * m;
        cx<T> acc = mk<T>(0, 0);
        for (int row = 0; row < m; ++row) cjfma(acc, u[row], th[row]);
        Cn[idx] = cscale(acc, (T)(1.0 / sh.norm[pj]) * cscal);
      }
    } else {
      // W = theta^H orthogonalised: U = theta W[:, perm] / s^2, carry = W[:, perm]^H
      for (int idx = tid; idx < m * kk; idx += nt) {
        const int row = idx / kk, j = idx - row * kk;
        const int pj = sh.perm[j];
        const double sj = sh.norm[pj];
        const cx<T>* w = W + (long long)pj * n;
        cx<T> acc = mk<T>(0, 0);
        for (int col = 0; col < n; ++col) cfma(acc, b.Tg[(long long)col * m + row], w[col]);
        A[idx] = cscale(acc, (T)(1.0 / (sj * sj)));
      }
      for (int idx = tid; idx < kk * n; idx += nt) {
        const int j = idx / n, col = idx - j * n;
        Cn[idx] = cscale(cconj(W[(long long)sh.perm[j] * n + col]), cscal);
      }
    }
    if (tid == 0) {
      dims[SLOT(k)] = make_int2(cxd, kk);
      if (RESCALE) sh.st.log_scale += log(smax);
    }
    __syncthreads();
    cxd = kk;
    ccd = r;
  }
  if (sh.st.status != ST_OK) {
    if (tid == 0) L.state[i] = sh.st;
    return;
  }

  // 4. right-to-left sweep
  for (int k = K - 1; k >= 1; --k) {
    cx<T>* A = SITE(k);
    const int2 dA = DIMS(k);
    const int l = dA.x, r = dA.y;
    const int m = D * r, n = l;
    const bool trans = n > m;
    cx<T>* W = ((long long)m * n <= b.smem_elems) ? b.Ws : b.Wg;
    if (!trans) {
      for (int idx = tid; idx < m * n; idx += nt) W[idx] = A[idx];
    } else {
      for (int idx = tid; idx < m * n; idx += nt) {
        const int col = idx / m, row = idx - col * m;
        W[col + (long long)row * n] = cconj(A[idx]);
      }
    }
    __syncthreads();
    const int kk = trans ? jacobi_truncate<T>(W, n, m, n, I.epsrel, sh.norm, sh.perm, &sh.jsh)
                         : jacobi_truncate<T>(W, m, n, m, I.epsrel, sh.norm, sh.perm, &sh.jsh);
    if (sh.jsh.status != ST_OK || kk > cap) {
      if (tid == 0) sh.st.status = (sh.jsh.status != ST_OK) ? sh.jsh.status : ST_CHI_OVERFLOW;
      __syncthreads();
      break;
    }
    const double smax = sh.norm[sh.perm[0]];
    const T cscal = RESCALE ? (T)(1.0 / smax) : (T)1;
    if (!trans) {
      for (int idx = tid; idx < kk * n; idx += nt) {
        const int j = idx / n, col = idx - j * n;
        const int pj = sh.perm[j];
        const cx<T>* u = W + (long long)pj * m;
        const cx<T>* y = A + (long long)col * m;
        cx<T> acc = mk<T>(0, 0);
        for (int row = 0; row < m; ++row) cjfma(acc, u[row], y[row]);
        b.Cg[idx] = cscale(acc, (T)(1.0 / sh.norm[pj]) * cscal);
      }
      __syncthreads();
      for (int idx = tid; idx < m * kk; idx += nt) {
        const int j = idx / m, row = idx - j * m;
        const int pj = sh.perm[j];
        A[idx] = cscale(W[(long long)pj * m + row], (T)(1.0 / sh.norm[pj]));
      }
    } else {
      for (int idx = tid; idx < m * kk; idx += nt) {
        const int j = idx / m, row = idx - j * m;
        const int pj = sh.perm[j];
        const double sj = sh.norm[pj];
        const cx<T>* w = W + (long long)pj * n;
        cx<T> acc = mk<T>(0, 0);
        for (int col = 0; col < n; ++col) cfma(acc, A[(long long)col * m + row], w[col]);
        b.Tg[idx] = cscale(acc, (T)(1.0 / (sj * sj)));
      }
      for (int idx = tid; idx < kk * n; idx += nt) {
        const int j = idx / n, col = idx - j * n;
        b.Cg[idx] = cscale(cconj(W[(long long)sh.perm[j] * n + col]), cscal);
      }
      __syncthreads();
      for (int idx = tid; idx < m * kk; idx += nt) A[idx] = b.Tg[idx];
    }
    if (tid == 0) {
      dims[SLOT(k)] = make_int2(kk, r);
      if (RESCALE) sh.st.log_scale += log(smax);
    }
    __syncthreads();
    // absorb S V^H into site k-1: (l2, D, n) x (kk, n)^T -> (l2, D, kk)
    cx<T>* B = SITE(k - 1);
    const int l2 = DIMS(k - 1).x;
    for (int idx = tid; idx < l2 * D * kk; idx += nt) {
      const int la = idx / kk, j = idx - la * kk;
      const cx<T>* brow = B + (long long)la * n;
      const cx<T>* crow = b.Cg + (long long)j * n;
      cx<T> acc = mk<T>(0, 0);
      for (int c = 0; c < n; ++c) cfma(acc, brow[c], crow[c]);
      b.Tg[idx] = acc;
    }
    __syncthreads();
    for (int idx = tid; idx < l2 * D * kk; idx += nt) B[idx] = b.Tg[idx];
    if (tid == 0) dims[SLOT(k - 1)] = make_int2(l2, kk);
    __syncthreads();
  }
  if (sh.st.status != ST_OK) {
    if (tid == 0) L.state[i] = sh.st;
    return;
  }

  // 5. second half-step propagator as the new last site: A[r][b][0] = P2[b][r]
  {
    cx<T>* A = SITE(K);
    for (int idx = tid; idx < D * D; idx += nt) {
      const int rr = idx / D, bb = idx - rr * D;
      A[idx] = to_t<T>(P2[bb * D + rr]);
    }
    if (tid == 0) {
      dims[SLOT(K)] = make_int2(D, 1);
      sh.st.nsites = K + 1;
    }
    __syncthreads();
  }

  // 6. read-out: v <- sum_{c,a} v[c] A[c][a][r] over all sites, state = P2 v
  {
    int cur = 0;
    if (tid == 0) sh.v[0][0] = mk<double>(1, 0);
    __syncthreads();
    int maxb = 1;
    for (int k = 0; k < K; ++k) {
      const cx<T>* A = SITE(k);
      const int2 dA = DIMS(k);
      const int l = dA.x, r = dA.y;
      maxb = max(maxb, r);
      for (int rr = tid; rr < r; rr += nt) {
        cx<double> acc = mk<double>(0, 0);
        for (int c = 0; c < l; ++c) {
          cx<double> part = mk<double>(0, 0);
          for (int a = 0; a < D; ++a) part = part + to_d(A[((long long)c * D + a) * r + rr]);
          cfma(acc, sh.v[cur][c], part);
        }
        sh.v[cur ^ 1][rr] = acc;
      }
      __syncthreads();
      cur ^= 1;
    }
    if (tid < D) {
      cx<double> acc = mk<double>(0, 0);
      for (int c = 0; c < D; ++c) cfma(acc, P2[tid * D + c], sh.v[cur][c]);
      if (RESCALE) {
        const double f = exp(sh.st.log_scale);
        acc.x *= f;
        acc.y *= f;
      }
      b.out[I.out_base + (long long)(step % I.out_cap) * D + tid] = acc;
    }
    if (tid == 0) {
      sh.st.step = step;
      sh.st.max_bond = maxb;
      sh.st.ovr_active = 0;
      L.state[i] = sh.st;
    }
    __syncthreads();
  }
#undef SLOT
#undef SITE
#undef DIMS
}

template <typename T, bool RESCALE>
__global__ void __launch_bounds__(TEMPO_THREADS) tempo_kernel(TempoLaunch L) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ SharedStep sh;
  Bufs<T> b;
  b.sites = (cx<T>*)L.sites;
  b.dims = L.dims;
  b.infl = (const cx<double>*)L.infl;
  b.props = (const cx<double>*)L.props;
  b.out = (cx<double>*)L.out;
  cx<T>* work = (cx<T>*)L.work + (long long)blockIdx.x * L.work_stride;
  b.Wg = work;
  b.Tg = work + L.wcap;
  b.Cg = work + 2 * L.wcap;
  b.Ws = (cx<T>*)dsm;
  b.smem_elems = L.smem_elems;
  for (;;) {
    if (threadIdx.x == 0) sh.inst = atomicAdd(L.queue, 1);
    __syncthreads();
    const int q = sh.inst;
    __syncthreads();
    if (q >= L.n) break;
    const int i = L.order[q];
    const InstDev I = L.inst[i];
    for (int s = 0; s < L.nsteps; ++s) {
      tempo_step<T, RESCALE>(L, I, i, b, sh);
      __syncthreads();
      if (sh.st.status != ST_OK) break;
    }
  }
}

int tempo_smem_bytes(int precision) {
  // 80 KiB of dynamic shared memory for the working matrix: two CTAs per SM
  // together with the static SharedStep block.
  (void)precision;
  return 80 * 1024;
}

cudaError_t launch_tempo(const TempoLaunch& L, int precision, int grid, int block,
                         cudaStream_t stream) {
  const int smem = tempo_smem_bytes(precision);
  TempoLaunch l2 = L;
  if (precision == 0) {
    l2.smem_elems = smem / (int)sizeof(cx<double>);
    cudaError_t e = cudaFuncSetAttribute(tempo_kernel<double, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    tempo_kernel<double, false><<<grid, block, smem, stream>>>(l2);
  } else {
    l2.smem_elems = smem / (int)sizeof(cx<float>);
    cudaError_t e = cudaFuncSetAttribute(tempo_kernel<float, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    tempo_kernel<float, true><<<grid, block, smem, stream>>>(l2);
  }
  return cudaGetLastError();
}

}  // namespace otb
