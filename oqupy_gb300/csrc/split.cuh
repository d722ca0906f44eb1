// Generic truncated bond split for one CTA, used by the PT-TEMPO build.
//
// X is an m x n complex128 matrix read through an accessor X(row, col).  The
// split orients itself so that the Jacobi columns are the smaller side, runs
// the QR-preconditioned Jacobi (qr.cuh; plain Jacobi, jacobi.cuh, below 8
// columns) in FP64 or double-float, and returns
//   U  (m x kk, column-major, in Tg)      left singular vectors,
//   C  (kk x n, row-major, in Cg)         S V^H (the carry),
// with kk the kept rank of the relative tail rule.  The caller copies U to its
// destination after the call (U never aliases X, so X may be the destination).
#pragma once

#include "qr.cuh"

namespace otb {

typedef cx<double> zc;

constexpr int SPLIT_NMAX = 1152;  // max Jacobi columns (D * cap <= 9 * 128)

struct SplitBufs {
  zc* Wg;      // global working matrix
  zc* Tg;      // global U output / temporaries
  zc* Cg;      // carry
  cff* Wffg;   // global double-float matrix (mixed form)
  unsigned char* smem;
  int smem_bytes;
};

struct SplitShared {
  JacobiShared jsh;
  double norm[SPLIT_NMAX];
  int perm[SPLIT_NMAX];
};

// Returns kk (>= 1); on failure sets *status (nonzero) and returns 0.
template <bool MIXED, class Acc>
__device__ int split_generic(const Acc& X, int m, int n, double epsrel, float qr_delta, int cap, SplitBufs& b,
                             SplitShared& sh, int* status, int* sweeps64, int* sweepsff,
                             double* flops) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const bool trans = n > m;
  const int R = trans ? n : m, N = trans ? m : n;
  size_t used = 0;
  auto take = [&](size_t bytes) -> void* {
    bytes = (bytes + 15) & ~(size_t)15;
    if (used + bytes > (size_t)b.smem_bytes) return nullptr;
    void* p = b.smem + used;
    used += bytes;
    return p;
  };
  // QR / double-float workspace (16 bytes per element in both forms)
  const bool flip = N >= 8;
  cff* Wff = nullptr;
  if (MIXED || flip) {
    Wff = (cff*)take((size_t)R * N * sizeof(cff));
    if (!Wff) Wff = b.Wffg;
  }
  zc* W = (zc*)take((size_t)R * N * sizeof(zc));
  if (!W) W = b.Wg;
  // W = X (R = m) or X^H (R = n), column-major with leading dimension R
  for (int idx = tid; idx < R * N; idx += nt) {
    const int c = idx / R, r = idx - c * R;
    W[idx] = trans ? cconj(X(c, r)) : X(r, c);
  }
  __syncthreads();
  // the QR-preconditioned driver (qr.cuh) returns X^H U (N x kk, ld N)
  // instead of X V (R x N, ld R): the same two branches below, swapped
  zc* Wr = W;
  const size_t spare = (size_t)b.smem_bytes > used ? (size_t)b.smem_bytes - used : 0;
  int kk;
  if (flip && MIXED)
    kk = qr_jacobi_truncate<ff>(W, R, N, Wff, b.smem + used, spare, epsrel, qr_delta, sh.norm, sh.perm,
                                &sh.jsh, &Wr);
  else if (flip)
    kk = qr_jacobi_truncate<double>(W, R, N, reinterpret_cast<zc*>(Wff), b.smem + used, spare, epsrel,
                                    qr_delta, sh.norm, sh.perm, &sh.jsh, &Wr);
  else if (MIXED)
    kk = jacobi_truncate_mixed(W, R, N, Wff, epsrel, sh.norm, sh.perm, &sh.jsh);
  else
    kk = jacobi_truncate_fp64(W, R, N, R, epsrel, sh.norm, sh.perm, &sh.jsh);
  W = Wr;
  *sweeps64 += sh.jsh.sweeps;  // mixed form: FP64 fallback sweeps only
  *sweepsff += MIXED ? sh.jsh.sweeps32 : 0;
  *flops += 4.0 * (6.0 * R * (double)N * N + 20.0 * (double)N * N * N);
  if (sh.jsh.status != ST_OK || kk > cap) {
    if (tid == 0) *status = (sh.jsh.status != ST_OK) ? sh.jsh.status : ST_CHI_OVERFLOW;
    __syncthreads();
    return 0;
  }
  if (!(flip ? !trans : trans)) {
    // U = W[:, perm] / s;  C = U^H X
    for (int idx = tid; idx < m * kk; idx += nt) {
      const int j = idx / m, row = idx - j * m;
      const int pj = sh.perm[j];
      b.Tg[idx] = cscale(W[(size_t)pj * m + row], 1.0 / sh.norm[pj]);
    }
    for (int idx = tid; idx < kk * n; idx += nt) {
      const int j = idx / n, col = idx - j * n;
      const int pj = sh.perm[j];
      const zc* u = W + (size_t)pj * m;
      zc acc = mk<double>(0, 0);
      for (int row = 0; row < m; ++row) cjfma(acc, u[row], X(row, col));
      b.Cg[idx] = cscale(acc, 1.0 / sh.norm[pj]);
    }
  } else {
    // W = X^H V orthogonal: U = X W[:, perm] / s^2, C = W[:, perm]^H
    for (int idx = tid; idx < m * kk; idx += nt) {
      const int j = idx / m, row = idx - j * m;
      const int pj = sh.perm[j];
      const double sj = sh.norm[pj];
      const zc* w = W + (size_t)pj * n;
      zc acc = mk<double>(0, 0);
      for (int col = 0; col < n; ++col) cfma(acc, X(row, col), w[col]);
      b.Tg[idx] = cscale(acc, 1.0 / (sj * sj));
    }
    for (int idx = tid; idx < kk * n; idx += nt) {
      const int j = idx / n, col = idx - j * n;
      b.Cg[idx] = cconj(W[(size_t)sh.perm[j] * n + col]);
    }
  }
  *flops += 8.0 * (double)m * n * kk;
  __syncthreads();
  return kk;
}

}  // namespace otb
