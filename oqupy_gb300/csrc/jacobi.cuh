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
// the descending sort, the tail sums and the rank decision are always FP64.
//
// Drivers:
//  * complex128 (jacobi_truncate_fp64): FP64 sweeps on the matrix until no
//    pair rotates;
//  * mixed, small splits (jacobi_truncate_mixed): the same sweeps in
//    double-float arithmetic (ff.cuh) on the FP32 pipe, FP64 fallback sweeps
//    if they do not settle;
//  * both forms, >= 8 columns: rank-revealing pivoted Householder QR, then
//    these sweeps on the k rows of R (qr.cuh).
#pragma once

#include "common.cuh"
#include "ff.cuh"

namespace otb {

constexpr int JACOBI_MAX_SWEEPS = 60;

struct JacobiShared {
  double red[33];
  int flag[2];
  float worst[2];   // largest relative off-diagonal rotated in a sweep
  int noise_converged;
  int kept;
  int status;
  int sweeps;     // FP64 sweeps of the last split
  int sweeps32;   // FP32 sweeps of the last split (mixed form)
};

__device__ __forceinline__ int jacobi_group(int rows) { return rows > 128 ? 32 : (rows > 32 ? 16 : 8); }

template <typename T>
__device__ __forceinline__ T group_sum(T v, int G) {
  for (int off = G >> 1; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off, 32);
  return v;
}

// Sweeps of one-sided Jacobi on W (m x n, column-major, leading dim ld).
// With V != nullptr the same rotations are applied to V (n x n, ld ldv).
// Returns the number of sweeps done (JACOBI_MAX_SWEEPS = not converged).
//
// Numerical-zero floor: a column whose squared norm is below
// (16 sqrt(m) eps)^2 times the largest squared column norm holds only
// rounding noise of the other columns; pairs involving such a column are not
// rotated (rotating noise against a real column regenerates noise at the
// stopping threshold and never converges).  The floor changes nothing above
// the rounding level of the decomposition.
template <typename T>
__device__ int jacobi_sweeps(cx<T>* W, int m, int n, int ld, cx<T>* V, int ldv, JacobiShared* sh,
                             int max_sweeps = JACOBI_MAX_SWEEPS, T tol_scale = (T)1) {
  const int tid = threadIdx.x;
  const int nthreads = blockDim.x;
  const int G = jacobi_group(m);
  const int lane = tid & (G - 1);
  const int group = tid / G;
  const int ngroups = nthreads / G;
  const int np = (n + 1) >> 1;
  const int nn = np << 1;
  const T tol = tol_scale * sqrt((T)m) * num<T>::eps();
  const T bigz = num<T>::big_zeta();
  if (tid == 0) {
    sh->flag[0] = 0;
    sh->worst[0] = 0.f;
    sh->noise_converged = 0;
  }
  __syncthreads();
  if (n <= 1) return 0;
  int sweep;
  for (sweep = 0; sweep < max_sweeps; ++sweep) {
    T zfloor;
    {
      // largest squared column norm (a lower bound of s_max^2)
      double mx = 0.0;
      for (int j = tid / 32; j < n; j += nthreads / 32) {
        const int l = tid & 31;
        double acc = 0.0;
        const cx<T>* c = W + (size_t)j * ld;
        for (int r = l; r < m; r += 32) {
          const double x = (double)c[r].x, y = (double)c[r].y;
          acc = fma(x, x, fma(y, y, acc));
        }
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
        mx = fmax(mx, acc);
      }
      for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
      if ((tid & 31) == 0) sh->red[tid >> 5] = mx;
      __syncthreads();
      if (tid == 0) {
        double v = 0.0;
        for (int w = 0; w < nthreads / 32; ++w) v = fmax(v, sh->red[w]);
        sh->red[32] = v;
      }
      __syncthreads();
      const double zf = 16.0 * sqrt((double)m) * (double)num<T>::eps();
      zfloor = (T)(zf * zf * sh->red[32]);
    }
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
          if (al > zfloor && be > zfloor && g > tol * sqrt(al) * sqrt(be)) {
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
            if (lane == 0) {
              const float ratio = (float)(g / (sqrt(al) * sqrt(be)));
              atomicMax((int*)&sh->worst[sweep & 1], __float_as_int(ratio));
            }
            if (V != nullptr) {
              cx<T>* va = V + (size_t)a * ldv;
              cx<T>* vb = V + (size_t)b * ldv;
              for (int r = lane; r < n; r += G) {
                const cx<T> u = va[r];
                const cx<T> v = vb[r];
                cx<T> nu, nv;
                nu.x = c * u.x - s * (pr * v.x + pi * v.y);
                nu.y = c * u.y - s * (pr * v.y - pi * v.x);
                nv.x = c * v.x + s * (pr * u.x - pi * u.y);
                nv.y = c * v.y + s * (pr * u.y + pi * u.x);
                va[r] = nu;
                vb[r] = nv;
              }
            }
            if (lane == 0) sh->flag[sweep & 1] = 1;
          }
        }
      }
      __syncthreads();
    }
    const int rotated = sh->flag[sweep & 1];
    const float worst = sh->worst[sweep & 1];
    if (tid == 0) {
      sh->flag[(sweep + 1) & 1] = 0;
      sh->worst[(sweep + 1) & 1] = 0.f;
    }
    __syncthreads();
    if (!rotated) break;
    // at the sweep cap, rotations below 1e-10 relative are rounding noise
    if (sweep == max_sweeps - 1 && worst < 1e-10f && tid == 0) sh->noise_converged = 1;
  }
  // noise_converged is written by thread 0 in the last sweep and read by every
  // caller thread to choose its next step: publish it before returning
  __syncthreads();
  return sweep;
}

// One-sided Jacobi sweeps in double-float arithmetic on W (m x n, ld).
// Same schedule, stopping test and numerical-zero floor as jacobi_sweeps;
// the inner products are reduced in FF, the rotation parameters are formed
// on the FP32 pipe (see below), and the rotation is applied in FF.  Orthogonality reaches
// about 1e-14 relative, with every per-element operation on the FP32 pipe.
__device__ inline int jacobi_sweeps_ff(cff* W, int m, int n, int ld, JacobiShared* sh) {
  const int tid = threadIdx.x;
  const int nthreads = blockDim.x;
  const int G = jacobi_group(m);
  const int lane = tid & (G - 1);
  const int group = tid / G;
  const int ngroups = nthreads / G;
  const int np = (n + 1) >> 1;
  const int nn = np << 1;
  const float eps_ff = 3.6e-15f;  // ~2^-48, double-float unit roundoff
  // the sloppy FF add and accumulated dot products sit a few units above
  // eps_ff: stopping test at 4x and numerical-zero floor at 32x
  const float tol = 4.f * sqrtf((float)m) * eps_ff;
  if (tid == 0) {
    sh->flag[0] = 0;
    sh->worst[0] = 0.f;
    sh->noise_converged = 0;
  }
  __syncthreads();
  if (n <= 1) return 0;
  int sweep;
  for (sweep = 0; sweep < JACOBI_MAX_SWEEPS; ++sweep) {
    float zfloor;
    {
      float mx = 0.f;
      for (int j = tid / 32; j < n; j += nthreads / 32) {
        const int l = tid & 31;
        float acc = 0.f;
        const cff* c = W + (size_t)j * ld;
        for (int r = l; r < m; r += 32) acc = fmaf(c[r].x.hi, c[r].x.hi, fmaf(c[r].y.hi, c[r].y.hi, acc));
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
        mx = fmaxf(mx, acc);
      }
      for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
      if ((tid & 31) == 0) sh->red[tid >> 5] = (double)mx;
      __syncthreads();
      if (tid == 0) {
        double v = 0.0;
        for (int w = 0; w < nthreads / 32; ++w) v = fmax(v, sh->red[w]);
        sh->red[32] = v;
      }
      __syncthreads();
      const float zf = 32.f * sqrtf((float)m) * eps_ff;
      zfloor = zf * zf * (float)sh->red[32];
    }
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
        // squared norms only steer the angle and the thresholds: FP32 from
        // the high parts; the off-diagonal gamma decides convergence: FF
        float A = 0.f, B = 0.f;
        ff gr = ff_make(0.f, 0.f), gi = gr;
        cff* ca = W + (size_t)a * ld;
        cff* cb = W + (size_t)b * ld;
        if (active) {
          // gamma = u^H v as compensated accumulators (ffp_acc)
          float grh = 0.f, grl = 0.f, gih = 0.f, gil = 0.f;
          for (int r = lane; r < m; r += G) {
            const cff u = ca[r];
            const cff v = cb[r];
            A = fmaf(u.x.hi, u.x.hi, fmaf(u.y.hi, u.y.hi, A));
            B = fmaf(v.x.hi, v.x.hi, fmaf(v.y.hi, v.y.hi, B));
            ffp_acc(u.x.hi, u.x.lo, v.x.hi, v.x.lo, grh, grl);
            ffp_acc(u.y.hi, u.y.lo, v.y.hi, v.y.lo, grh, grl);
            ffp_acc(u.x.hi, u.x.lo, v.y.hi, v.y.lo, gih, gil);
            ffp_acc(-u.y.hi, -u.y.lo, v.x.hi, v.x.lo, gih, gil);
          }
          gr = ffacc_norm(grh, grl);
          gi = ffacc_norm(gih, gil);
        }
        for (int off = G >> 1; off > 0; off >>= 1) {
          A += __shfl_xor_sync(0xffffffffu, A, off, 32);
          B += __shfl_xor_sync(0xffffffffu, B, off, 32);
          gr = ff_add(gr, ff_shfl_xor(gr, off));
          gi = ff_add(gi, ff_shfl_xor(gi, off));
        }
        // Near-degenerate pair: float norms cannot resolve B - A (their
        // relative precision is 1e-7), and an angle from that noise never
        // zeroes gamma.  Recompute the difference in FF for such pairs.
        float dBA = B - A;
        {
          const bool need = active && A > zfloor && B > zfloor && fabsf(dBA) <= 2e-4f * (A + B) &&
                            hypotf(gr.hi, gi.hi) > tol * sqrtf(A) * sqrtf(B);
          if (__any_sync(0xffffffffu, need)) {
            ff d = ff_make(0.f, 0.f);
            if (need) {
              for (int r = lane; r < m; r += G) {
                const cff u = ca[r];
                const cff v = cb[r];
                d = ff_fma(v.x, v.x, ff_fma(v.y, v.y, d));
                d = ff_sub(d, ff_add(ff_mul(u.x, u.x), ff_mul(u.y, u.y)));
              }
            }
            for (int off = G >> 1; off > 0; off >>= 1) d = ff_add(d, ff_shfl_xor(d, off));
            if (need) dBA = d.hi + d.lo;
          }
        }
        if (active) {
          // Rotation parameters on the FP32 pipe.  The angle only needs float
          // accuracy (later sweeps correct it); unitarity is what must hold to
          // FF precision, so c, s come from t through an FF rsqrt
          // (c^2 + s^2 = c^2 (1 + t^2) = 1) and the phase is normalised in FF.
          const float g = hypotf(gr.hi, gi.hi);
          if (A > zfloor && B > zfloor && g > tol * sqrtf(A) * sqrtf(B)) {
            const float zeta = dBA / (2.f * g);
            const float az = fabsf(zeta);
            float t = (az > 1e18f) ? 0.5f / az : 1.f / (az + sqrtf(1.f + zeta * zeta));
            if (zeta < 0.f) t = -t;
            const ff ft = ff_make(t, 0.f);
            const ff fc = ff_rsqrt(ff_add(ff_make(1.f, 0.f), ff_mul(ft, ft)));
            const ff fs = ff_mul(fc, ft);
            const ff ig = ff_make(1.f / g, 0.f);
            const ff px = ff_mul(gr, ig), py = ff_mul(gi, ig);
            const ff nrm = ff_rsqrt(ff_add(ff_mul(px, px), ff_mul(py, py)));
            const ff pr = ff_mul(px, nrm), pi = ff_mul(py, nrm);
            // q = s e^{-i phi}, w = s e^{i phi}
            const ff qx = ff_mul(fs, pr);
            const ff wy = ff_mul(fs, pi);
            const ff qy = ff_make(-wy.hi, -wy.lo);
            for (int r = lane; r < m; r += G) {
              const cff u = ca[r];
              const cff v = cb[r];
              cff nu, nv;
              // each component one compensated accumulation of three products
              float h, l;
              // nu = c u - q v
              h = l = 0.f;
              ffp_acc(fc.hi, fc.lo, u.x.hi, u.x.lo, h, l);
              ffp_acc(-qx.hi, -qx.lo, v.x.hi, v.x.lo, h, l);
              ffp_acc(qy.hi, qy.lo, v.y.hi, v.y.lo, h, l);
              nu.x = ffacc_norm(h, l);
              h = l = 0.f;
              ffp_acc(fc.hi, fc.lo, u.y.hi, u.y.lo, h, l);
              ffp_acc(-qx.hi, -qx.lo, v.y.hi, v.y.lo, h, l);
              ffp_acc(-qy.hi, -qy.lo, v.x.hi, v.x.lo, h, l);
              nu.y = ffacc_norm(h, l);
              // nv = c v + w u, w = (qx, wy)
              h = l = 0.f;
              ffp_acc(fc.hi, fc.lo, v.x.hi, v.x.lo, h, l);
              ffp_acc(qx.hi, qx.lo, u.x.hi, u.x.lo, h, l);
              ffp_acc(-wy.hi, -wy.lo, u.y.hi, u.y.lo, h, l);
              nv.x = ffacc_norm(h, l);
              h = l = 0.f;
              ffp_acc(fc.hi, fc.lo, v.y.hi, v.y.lo, h, l);
              ffp_acc(qx.hi, qx.lo, u.y.hi, u.y.lo, h, l);
              ffp_acc(wy.hi, wy.lo, u.x.hi, u.x.lo, h, l);
              nv.y = ffacc_norm(h, l);
              ca[r] = nu;
              cb[r] = nv;
            }
            if (lane == 0) {
              sh->flag[sweep & 1] = 1;
              atomicMax((int*)&sh->worst[sweep & 1], __float_as_int(g / (sqrtf(A) * sqrtf(B))));
            }
          }
        }
      }
      __syncthreads();
    }
    const int rotated = sh->flag[sweep & 1];
    const float worst = sh->worst[sweep & 1];
    if (tid == 0) {
      sh->flag[(sweep + 1) & 1] = 0;
      sh->worst[(sweep + 1) & 1] = 0.f;
    }
    __syncthreads();
    if (!rotated) break;
    // at the sweep cap, rotations below 1e-10 relative are rounding noise
    if (sweep == JACOBI_MAX_SWEEPS - 1 && worst < 1e-10f && tid == 0) sh->noise_converged = 1;
  }
  __syncthreads();  // publish noise_converged (see jacobi_sweeps)
  return sweep;
}

__device__ inline int jacobi_rank(int n, double epsrel, double* norm, int* perm, JacobiShared* sh,
                                  int sweeps, double tail2);

// FP64 column norms of W, descending order and the kept rank (>= 1).
template <typename T>
__device__ int jacobi_finish(const cx<T>* W, int m, int n, int ld, double epsrel, double* norm,
                             int* perm, JacobiShared* sh, int sweeps, double tail2 = 0.0) {
  const int tid = threadIdx.x;
  const int nthreads = blockDim.x;
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
  return jacobi_rank(n, epsrel, norm, perm, sh, sweeps, tail2);
}

// Descending order of the n values norm[] and the kept rank (>= 1): the
// second half of jacobi_finish, for callers that computed the norms.
__device__ inline int jacobi_rank(int n, double epsrel, double* norm, int* perm, JacobiShared* sh,
                                  int sweeps, double tail2) {
  const int tid = threadIdx.x;
  const int nthreads = blockDim.x;
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
    double cum = tail2;  // squared norm of a block dropped before the sweeps (all in the tail)
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
    sh->sweeps = sweeps;
    sh->status = ST_OK;
    if (!finite)
      sh->status = ST_NONFINITE;
    else if (sweeps >= JACOBI_MAX_SWEEPS && !sh->noise_converged)
      sh->status = ST_NO_CONVERGENCE;
  }
  __syncthreads();
  return sh->kept;
}

// complex128 driver: orthogonalise W (m x n) in place and truncate.
__device__ inline int jacobi_truncate_fp64(cx<double>* W, int m, int n, int ld, double epsrel,
                                           double* norm, int* perm, JacobiShared* sh) {
  const int sw = jacobi_sweeps<double>(W, m, n, ld, nullptr, 0, sh);
  if (threadIdx.x == 0) sh->sweeps32 = 0;
  return jacobi_finish<double>(W, m, n, ld, epsrel, norm, perm, sh, sw);
}

// Mixed driver: W (m x n, FP64, ld m) holds the matrix to split.  It is
// scaled to unit largest entry, converted to double-float in Wff (m x n),
// orthogonalised there, and written back (rescaled) to W in FP64, followed by
// the FP64 finish.  The FF range (float exponent) is why the scaling is done.
__device__ inline int jacobi_truncate_mixed(cx<double>* W, int m, int n, cff* Wff, double epsrel,
                                            double* norm, int* perm, JacobiShared* sh) {
  const int tid = threadIdx.x;
  const int nt = blockDim.x;
  double mx = 0.0;
  for (int idx = tid; idx < m * n; idx += nt) mx = fmax(mx, fmax(fabs(W[idx].x), fabs(W[idx].y)));
  for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if ((tid & 31) == 0) sh->red[tid >> 5] = mx;
  __syncthreads();
  if (tid == 0) {
    double v = 0.0;
    for (int w = 0; w < nt / 32; ++w) v = fmax(v, sh->red[w]);
    sh->red[32] = (v > 0.0) ? v : 1.0;
  }
  __syncthreads();
  const double scale = sh->red[32];
  const double inv = 1.0 / scale;
  for (int idx = tid; idx < m * n; idx += nt) Wff[idx] = cff_from(cscale(W[idx], inv));
  __syncthreads();
  const int sw = jacobi_sweeps_ff(Wff, m, n, m, sh);
  const bool ff_done = sw < JACOBI_MAX_SWEEPS || sh->noise_converged;
  for (int idx = tid; idx < m * n; idx += nt) W[idx] = cscale(cff_to(Wff[idx]), scale);
  __syncthreads();
  // FP64 fallback: if the double-float sweeps did not settle, finish the
  // (nearly orthogonal) matrix with FP64 sweeps; their count is reported
  const int sw64 = ff_done ? 0 : jacobi_sweeps<double>(W, m, n, m, nullptr, 0, sh);
  if (threadIdx.x == 0) sh->sweeps32 = sw;
  const int kk = jacobi_finish<double>(W, m, n, m, epsrel, norm, perm, sh, ff_done ? 0 : sw64);
  if (threadIdx.x == 0) sh->sweeps = ff_done ? 0 : sw64;
  __syncthreads();
  return kk;
}

}  // namespace otb
