// One-sided (Hestenes) Jacobi SVD with the TEMPO relative truncation rule,
// executed by one CTA on a matrix held in shared or global memory.
//
// Replaces, for every bond split on the TEMPO / PT-TEMPO path, the
// truncated SVD the reference obtains from tensornetwork's
// split_node_full_svd(max_truncation_err=epsrel, relative=True)
// (oqupy/backends/node_array.py:262-268, 285-291, 541-547).  The truncation
// rule keeps chi = #{i : sqrt(sum_{j>=i} s_j^2) > epsrel * s_0} over the
// singular values in descending order (stated in the reference at
// oqupy/mps_mpo.py:452-457).
//
// Parallel schedule: round-robin ("circle") tournament over the n columns, so
// each round rotates n/2 disjoint column pairs concurrently.  A pair is owned
// by a group of G lanes (G = 8, 16 or 32 by row count); the three inner
// products are reduced with xor shuffles inside the group.  Column norms,
// the descending sort, the tail sums and the rank decision are always done in
// FP64, also when the matrix itself is FP32.
#pragma once

#include "common.cuh"

namespace otb {

constexpr int JACOBI_MAX_SWEEPS = 60;

struct JacobiShared {
  int flag[2];
  int kept;
  int status;
};

template <typename T>
__device__ __forceinline__ T group_sum(T v, int G) {
  for (int off = G >> 1; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off, 32);
  return v;
}

// Orthogonalise the columns of W (m x n, column-major, leading dimension ld)
// in place: on return W = A V with mutually orthogonal columns.  Afterwards
// norm[j] = ||W_j||_2 (FP64), perm[0..n) lists the columns by descending
// norm, and the return value is the kept rank (>= 1).  Must be called by all
// threads of the CTA.  norm/perm must hold n entries (shared memory).
template <typename T>
__device__ int jacobi_truncate(cx<T>* W, int m, int n, int ld, double epsrel, double* norm,
                               int* perm, JacobiShared* sh) {
  const int tid = threadIdx.x;
  const int nthreads = blockDim.x;
  const int G = (m > 32) ? 32 : ((m > 16) ? 16 : 8);
  const int lane = tid & (G - 1);
  const int group = tid / G;
  const int ngroups = nthreads / G;
  const int np = (n + 1) >> 1;
  const int nn = np << 1;
  const T tol = sqrt((T)m) * num<T>::eps();
  const T bigz = num<T>::big_zeta();

  if (tid == 0) {
    sh->flag[0] = 0;
    sh->status = ST_OK;
  }
  __syncthreads();
  int sweep = 0;
  if (n > 1) {
    for (sweep = 0; sweep < JACOBI_MAX_SWEEPS; ++sweep) {
      for (int round = 0; round < nn - 1; ++round) {
        for (int pb = 0; pb < np; pb += ngroups) {
          const int p = pb + group;
          int a, b;
          if (p == 0) {
            a = nn - 1;
            b = round;
          } else {
            a = (round + p) % (nn - 1);
            b = (round - p + nn - 1) % (nn - 1);
          }
          if (a > b) {
            const int t = a;
            a = b;
            b = t;
          }
          const bool active = (p < np) && (b < n);
          T al = 0, be = 0, gr = 0, gi = 0;
          cx<T>* ca = W + (size_t)a * ld;
          cx<T>* cb = W + (size_t)b * ld;
          if (active) {
            for (int r = lane; r < m; r += G) {
              const cx<T> u = ca[r];
              const cx<T> v = cb[r];
              al = fma(u.x, u.x, fma(u.y, u.y, al));
              be = fma(v.x, v.x, fma(v.y, v.y, be));
              gr = fma(u.x, v.x, fma(u.y, v.y, gr));
              gi = fma(u.x, v.y, fma(-u.y, v.x, gi));
            }
          }
          al = group_sum(al, G);
          be = group_sum(be, G);
          gr = group_sum(gr, G);
          gi = group_sum(gi, G);
          if (active) {
            const T g = sqrt(gr * gr + gi * gi);
            if (al > 0 && be > 0 && g > tol * sqrt(al) * sqrt(be)) {
              const T zeta = (be - al) / (2 * g);
              const T az = fabs(zeta);
              T t = (az > bigz) ? (T)0.5 / az : (T)1 / (az + sqrt((T)1 + zeta * zeta));
              if (zeta < 0) t = -t;
              const T c = (T)1 / sqrt((T)1 + t * t);
              const T s = c * t;
              const T pr = gr / g, pi = gi / g;  // e^{i phi}
              // a' = c a - s e^{-i phi} b ;  b' = s e^{i phi} a + c b
              for (int r = lane; r < m; r += G) {
                const cx<T> u = ca[r];
                const cx<T> v = cb[r];
                cx<T> nu, nv;
                nu.x = c * u.x - s * (pr * v.x + pi * v.y);
                nu.y = c * u.y - s * (pr * v.y - pi * v.x);
                nv.x = c * v.x + s * (pr * u.x - pi * u.y);
                nv.y = c * v.y + s * (pr * u.y + pi * u.x);
                ca[r] = nu;
                cb[r] = nv;
              }
              if (lane == 0) sh->flag[sweep & 1] = 1;
            }
          }
        }
        __syncthreads();
      }
      const int rotated = sh->flag[sweep & 1];
      if (tid == 0) sh->flag[(sweep + 1) & 1] = 0;
      __syncthreads();
      if (!rotated) break;
    }
  }
  // FP64 column norms
  for (int j = tid / 32; j < n; j += nthreads / 32) {
    const int l = tid & 31;
    double acc = 0.0;
    const cx<T>* c = W + (size_t)j * ld;
    for (int r = l; r < m; r += 32) {
      const double x = (double)c[r].x, y = (double)c[r].y;
      acc = fma(x, x, fma(y, y, acc));
    }
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (l == 0) norm[j] = sqrt(acc);
  }
  __syncthreads();
  // descending order, ties broken by column index
  for (int j = tid; j < n; j += nthreads) {
    const double sj = norm[j];
    int rank = 0;
    for (int i = 0; i < n; ++i) {
      const double si = norm[i];
      rank += (si > sj) || (si == sj && i < j);
    }
    perm[rank] = j;
  }
  __syncthreads();
  if (tid == 0) {
    const double thr = epsrel * norm[perm[0]];
    double cum = 0.0;
    int kept = 0;
    bool finite = true;
    for (int r = n - 1; r >= 0; --r) {
      const double s = norm[perm[r]];
      finite = finite && isfinite(s);
      cum += s * s;
      kept += (sqrt(cum) > thr) ? 1 : 0;
    }
    if (kept < 1) kept = 1;
    sh->kept = kept;
    if (!finite)
      sh->status = ST_NONFINITE;
    else if (sweep >= JACOBI_MAX_SWEEPS)
      sh->status = ST_NO_CONVERGENCE;
  }
  __syncthreads();
  return sh->kept;
}

}  // namespace otb
