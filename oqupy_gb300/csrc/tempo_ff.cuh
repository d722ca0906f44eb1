// The mixed form's TEMPO step: the same six stages as tempo_step (tempo.cu,
// oqupy/backends/tempo_backend.py:439-575), with the site tensors, the
// carry and theta held in double-float (pairs of floats, ff.cuh) and every
// contraction, QR and Jacobi rotation on the FP32 pipe.  The FP64 pipe (one
// seventy-fourth of the FP32 pipe's throughput on GB300) only sees per-split
// and per-step quantities: the kept singular values and the rank decision,
// the D x D propagators and influences when they are staged into shared
// memory, and the D-entry state written to the output ring.
#pragma once

namespace otb {

// Truncated split of the R x N (R >= N) double-float matrix A = op(src), op
// the identity (A(row,c) = src[c*lds+row]) or the conjugate transpose
// (A(row,c) = conj(src[row*lds+c])).  As split(): *Wout is A V (R x N,
// ld R) or, with *flip (>= QR_MIN_COLS columns), A^H U (N x kept, ld N), with
// sh.norm / sh.perm / the return value as in jacobi_finish; here *Wout is
// double-float and in the units of A.
__device__ __noinline__ int split_ff(const cff* src, int lds, bool src_trans, int R, int N, double epsrel,
                                     float qr_delta, Bufs& b, SharedStep& sh, cff** Wout, bool* flip) {
  const int tid = threadIdx.x, nt = blockDim.x;
  size_t used = 0;
  auto take = [&](size_t bytes) -> void* {
    bytes = (bytes + 15) & ~(size_t)15;
    if (used + bytes > (size_t)b.smem_bytes) return nullptr;
    void* p = b.smem + used;
    used += bytes;
    return p;
  };
  cff* X = (cff*)take((size_t)R * N * sizeof(cff));
  if (!X) X = b.Wffg;
  // power-of-two scale from the largest float magnitude (exact)
  float mx = 0.f;
  for (int idx = tid; idx < R * N; idx += nt) {
    const int c = idx / R, row = idx - c * R;
    const cff x = src_trans ? src[(size_t)row * lds + c] : src[(size_t)c * lds + row];
    mx = fmaxf(mx, fmaxf(fabsf(x.x.hi), fabsf(x.y.hi)));
  }
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if ((tid & 31) == 0) sh.jsh.red[tid >> 5] = mx;
  __syncthreads();
  if (tid == 0) {
    float v = 0.f;
    for (int w = 0; w < nt / 32; ++w) v = fmaxf(v, (float)sh.jsh.red[w]);
    sh.jsh.red[32] = (v > 0.f && isfinite(v)) ? (double)ilogbf(v) : 0.0;
  }
  __syncthreads();
  const int e = (int)sh.jsh.red[32];
  const float down = ldexpf(1.f, -e);
  for (int idx = tid; idx < R * N; idx += nt) {
    const int c = idx / R, row = idx - c * R;
    const cff x = src_trans ? cff_conj(src[(size_t)row * lds + c]) : src[(size_t)c * lds + row];
    X[idx] = cff_ldexp(x, down);
  }
  __syncthreads();
  const double scale = ldexp(1.0, e);
  if (N >= QR_MIN_COLS) {
    *flip = true;
    const size_t spare = (size_t)b.smem_bytes > used ? (size_t)b.smem_bytes - used : 0;
    return qr_jacobi_truncate_ff(X, R, N, scale, reinterpret_cast<cff*>(b.Wg), b.smem + used, spare, epsrel,
                                 qr_delta, sh.norm, sh.perm, &sh.jsh, Wout);
  }
  *flip = false;
  const int sw = jacobi_sweeps_ff(X, R, N, R, &sh.jsh);
  int sw64 = 0;
  if (!(sw < JACOBI_MAX_SWEEPS || sh.jsh.noise_converged)) sw64 = cff_fp64_fallback(X, R, N, R, &sh.jsh);
  if (tid == 0) sh.jsh.sweeps32 = sw;
  cff_column_norms(X, R, N, R, sh.norm);
  for (int j = tid; j < N; j += nt) sh.norm[j] *= scale;
  __syncthreads();
  const int kk = jacobi_rank(N, epsrel, sh.norm, sh.perm, &sh.jsh, sw64, 0.0);
  if (tid == 0) sh.jsh.sweeps = sw64;
  const float up = ldexpf(1.f, e);
  for (int idx = tid; idx < R * N; idx += nt) X[idx] = cff_ldexp(X[idx], up);
  __syncthreads();
  *Wout = X;
  return kk;
}

// The kept columns' scale factors as double-float, in place of their norms:
// 1 / s (wt false) or 1 / s^2 (wt true), one FP64 division per kept column.
__device__ __forceinline__ ff* kept_inverses(SharedStep& sh, int kk, bool wt) {
  ff* sinv = reinterpret_cast<ff*>(sh.norm);
  for (int j = threadIdx.x; j < kk; j += blockDim.x) {
    const int pj = sh.perm[j];
    const double s = sh.norm[pj];
    sinv[pj] = ff_from(wt ? 1.0 / (s * s) : 1.0 / s);
  }
  __syncthreads();
  return sinv;
}

__device__ void tempo_step_ff(const TempoLaunch& L, const InstDev& I, int i, Bufs& b, SharedStep& sh) {
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
  cff* const sites = reinterpret_cast<cff*>(b.sites) + I.site_base;
  int2* const dims = b.dims + I.dims_base;
  const zc* P1 = b.props + I.prop_base;
  const zc* P2 = P1 + D * D;
  cff* const Tf = reinterpret_cast<cff*>(b.Tg);   // theta / temporaries
  cff* const Cf = reinterpret_cast<cff*>(b.Cg);   // carry / read-out vectors
  int splits = 0, sw64 = 0, sw32 = 0;
  double flops = 0.0;
  // the step's propagators in double-float, staged once
  for (int idx = tid; idx < D * D; idx += nt) {
    sh.pf[0][idx] = cff_from(P1[idx]);
    sh.pf[1][idx] = cff_from(P2[idx]);
  }
  __syncthreads();

#define SLOT(k) ((sh.st.head + (k)) % I.nslots)
#define SITE(k) (sites + (long long)SLOT(k) * slot_elems)
#define DIMS(k) (dims[SLOT(k)])

  // 1. first half-step propagator on the newest site
  {
    const int k = sh.st.nsites - 1;
    cff* A = SITE(k);
    const int l = DIMS(k).x;
    for (int idx = tid; idx < l * D; idx += nt) {
      const int ll = idx / D, bb = idx - ll * D;
      ccacc f = ccacc_zero();
      for (int a = 0; a < D; ++a) ccacc_fma(f, sh.pf[0][bb * D + a], A[ll * D + a]);
      Tf[idx] = ccacc_cff(f);
    }
    __syncthreads();
    for (int idx = tid; idx < l * D; idx += nt) A[idx] = Tf[idx];
    __syncthreads();
  }

  // 2. trace out the oldest site (sum_north = ones) and merge into the next
  if (sh.st.nsites > window) {
    cff* A0 = SITE(0);
    cff* A1 = SITE(1);
    const int r0 = DIMS(0).y;
    const int r1 = DIMS(1).y;
    for (int c = tid; c < r0; c += nt) {
      cff acc = A0[c];
      for (int a = 1; a < D; ++a) acc = cff_add(acc, A0[a * r0 + c]);
      Cf[c] = acc;
    }
    __syncthreads();
    for (int idx = tid; idx < D * r1; idx += nt) {
      const int a = idx / r1, rr = idx - a * r1;
      ccacc f = ccacc_zero();
      for (int c = 0; c < r0; ++c) ccacc_fma(f, Cf[c], A1[((long long)c * D + a) * r1 + rr]);
      Tf[idx] = ccacc_cff(f);
    }
    __syncthreads();
    for (int idx = tid; idx < D * r1; idx += nt) A1[idx] = Tf[idx];
    __syncthreads();
    if (tid == 0) {
      dims[(sh.st.head + 1) % I.nslots] = make_int2(1, r1);
      sh.st.head = (sh.st.head + 1) % I.nslots;
      sh.st.nsites -= 1;
    }
    __syncthreads();
  }

  const int K = sh.st.nsites;
  // 3. zip-up: theta[(x,a),(r,m)] = I_dk[a,m] sum_c C[x,c,m] A[c,a,r]
  int cxd = 1, ccd = 1;
  for (int k = 0; k < K; ++k) {
    cff* A = SITE(k);
    const int r = DIMS(k).y;
    const int dk = K - 1 - k;
    const zc* Im = (k == 0 && sh.st.ovr_active) ? (b.props + I.ovr_base)
                                                 : (b.infl + I.infl_base + (long long)dk * D * D);
    for (int idx = tid; idx < D * D; idx += nt) sh.pf[2][idx] = cff_from(Im[idx]);
    __syncthreads();
    const int m = cxd * D;
    const int n = r * D;
    const bool last = (k == K - 1);
    // theta into Tf: column-major (ld m) for a split, site layout for the last site
    for (int idx = tid; idx < m * n; idx += nt) {
      int row, col;
      if (last) {
        row = idx / n;
        col = idx - row * n;
      } else {
        col = idx / m;
        row = idx - col * m;
      }
      const int x = row / D, a = row - x * D;
      const int rr = col / D, mr = col - rr * D;
      ccacc f = ccacc_zero();
      if (k == 0) {
        ccacc_fma(f, sh.pf[2][a * D + mr], A[a * r + rr]);
      } else {
        ccacc g = ccacc_zero();
        for (int c = 0; c < ccd; ++c)
          ccacc_fma(g, Cf[(long long)x * (ccd * D) + c * D + mr], A[((long long)c * D + a) * r + rr]);
        ccacc_fma(f, sh.pf[2][a * D + mr], ccacc_cff(g));
      }
      Tf[idx] = ccacc_cff(f);
    }
    __syncthreads();
    if (last) {
      for (int idx = tid; idx < m * n; idx += nt) A[idx] = Tf[idx];
      if (tid == 0) dims[SLOT(k)] = make_int2(cxd, n);
      __syncthreads();
      break;
    }
    const bool trans = n > m;
    cff* W;
    bool flip;
    const int kk = trans ? split_ff(Tf, m, true, n, m, I.epsrel, I.qr_delta, b, sh, &W, &flip)
                         : split_ff(Tf, m, false, m, n, I.epsrel, I.qr_delta, b, sh, &W, &flip);
    {
      const double R = trans ? n : m, N = trans ? m : n;
      flops += 8.0 * m * n * ccd + 4.0 * (6.0 * R * N * N + 20.0 * N * N * N);
    }
    ++splits;
    sw64 += sh.jsh.sweeps;
    sw32 += sh.jsh.sweeps32;
    if (sh.jsh.status != ST_OK || kk > cap) {
      if (tid == 0) sh.st.status = (sh.jsh.status != ST_OK) ? sh.jsh.status : ST_CHI_OVERFLOW;
      __syncthreads();
      break;
    }
    // W = theta V (U S, ld m) or W = theta^H U (V S, ld n), by orientation and driver
    const bool wt = flip ? !trans : trans;
    const ff* sinv = kept_inverses(sh, kk, wt);
    if (!wt) {
      // U = W[:, perm] / s -> site (cxd, D, kk);  carry = U^H theta
      for (int idx = tid; idx < m * kk; idx += nt) {
        const int row = idx / kk, j = idx - row * kk;
        const int pj = sh.perm[j];
        A[idx] = cff_scale(W[(long long)pj * m + row], sinv[pj]);
      }
      for (int idx = tid; idx < kk * n; idx += nt) {
        const int j = idx / n, col = idx - j * n;
        const int pj = sh.perm[j];
        const cff* u = W + (long long)pj * m;
        const cff* th = Tf + (long long)col * m;
        ccacc f = ccacc_zero();
        for (int row = 0; row < m; ++row) ccacc_fmaj(f, u[row], th[row]);
        Cf[idx] = cff_scale(ccacc_cff(f), sinv[pj]);
      }
    } else {
      // U = theta W[:, perm] / s^2 -> site;  carry = W[:, perm]^H
      for (int idx = tid; idx < m * kk; idx += nt) {
        const int row = idx / kk, j = idx - row * kk;
        const int pj = sh.perm[j];
        const cff* w = W + (long long)pj * n;
        ccacc f = ccacc_zero();
        for (int col = 0; col < n; ++col) ccacc_fma(f, Tf[(long long)col * m + row], w[col]);
        A[idx] = cff_scale(ccacc_cff(f), sinv[pj]);
      }
      for (int idx = tid; idx < kk * n; idx += nt) {
        const int j = idx / n, col = idx - j * n;
        Cf[idx] = cff_conj(W[(long long)sh.perm[j] * n + col]);
      }
    }
    if (tid == 0) dims[SLOT(k)] = make_int2(cxd, kk);
    __syncthreads();
    cxd = kk;
    ccd = r;
  }

  // 4. right-to-left sweep: site k as the column-major (D r) x l matrix
  if (sh.st.status == ST_OK) {
    for (int k = K - 1; k >= 1; --k) {
      cff* A = SITE(k);
      const int2 dA = DIMS(k);
      const int l = dA.x, r = dA.y;
      const int m = D * r, n = l;
      const bool trans = n > m;
      cff* W;
      bool flip;
      const int kk = trans ? split_ff(A, m, true, n, m, I.epsrel, I.qr_delta, b, sh, &W, &flip)
                           : split_ff(A, m, false, m, n, I.epsrel, I.qr_delta, b, sh, &W, &flip);
      {
        const double R = trans ? n : m, N = trans ? m : n;
        flops += 4.0 * (6.0 * R * N * N + 20.0 * N * N * N) + 8.0 * DIMS(k - 1).x * D * (double)kk * n;
      }
      ++splits;
      sw64 += sh.jsh.sweeps;
      sw32 += sh.jsh.sweeps32;
      if (sh.jsh.status != ST_OK || kk > cap) {
        if (tid == 0) sh.st.status = (sh.jsh.status != ST_OK) ? sh.jsh.status : ST_CHI_OVERFLOW;
        __syncthreads();
        break;
      }
      const bool wt = flip ? !trans : trans;
      const ff* sinv = kept_inverses(sh, kk, wt);
      if (!wt) {
        // carry = U^H A (U = W / s), then U -> site k (kk, D, r)
        for (int idx = tid; idx < kk * n; idx += nt) {
          const int j = idx / n, col = idx - j * n;
          const int pj = sh.perm[j];
          const cff* u = W + (long long)pj * m;
          const cff* y = A + (long long)col * m;
          ccacc f = ccacc_zero();
          for (int row = 0; row < m; ++row) ccacc_fmaj(f, u[row], y[row]);
          Cf[idx] = cff_scale(ccacc_cff(f), sinv[pj]);
        }
        __syncthreads();
        for (int idx = tid; idx < m * kk; idx += nt) {
          const int j = idx / m, row = idx - j * m;
          const int pj = sh.perm[j];
          A[idx] = cff_scale(W[(long long)pj * m + row], sinv[pj]);
        }
      } else {
        // U = A W[:, perm] / s^2 -> Tf, carry = W[:, perm]^H, then Tf -> site k
        for (int idx = tid; idx < m * kk; idx += nt) {
          const int j = idx / m, row = idx - j * m;
          const int pj = sh.perm[j];
          const cff* w = W + (long long)pj * n;
          ccacc f = ccacc_zero();
          for (int col = 0; col < n; ++col) ccacc_fma(f, A[(long long)col * m + row], w[col]);
          Tf[idx] = cff_scale(ccacc_cff(f), sinv[pj]);
        }
        for (int idx = tid; idx < kk * n; idx += nt) {
          const int j = idx / n, col = idx - j * n;
          Cf[idx] = cff_conj(W[(long long)sh.perm[j] * n + col]);
        }
        __syncthreads();
        for (int idx = tid; idx < m * kk; idx += nt) A[idx] = Tf[idx];
      }
      if (tid == 0) dims[SLOT(k)] = make_int2(kk, r);
      __syncthreads();
      // absorb S V^H into site k-1: (l2, D, n) x (kk, n)^T -> (l2, D, kk)
      cff* B = SITE(k - 1);
      const int l2 = DIMS(k - 1).x;
      for (int idx = tid; idx < l2 * D * kk; idx += nt) {
        const int la = idx / kk, j = idx - la * kk;
        const cff* brow = B + (long long)la * n;
        const cff* crow = Cf + (long long)j * n;
        ccacc f = ccacc_zero();
        for (int c = 0; c < n; ++c) ccacc_fma(f, brow[c], crow[c]);
        Tf[idx] = ccacc_cff(f);
      }
      __syncthreads();
      for (int idx = tid; idx < l2 * D * kk; idx += nt) B[idx] = Tf[idx];
      if (tid == 0) dims[SLOT(k - 1)] = make_int2(l2, kk);
      __syncthreads();
    }
  }
  if (sh.st.status != ST_OK) {
    if (tid == 0) L.state[i] = sh.st;
    return;
  }

  // 5. second half-step propagator as the new last site: A[r][b][0] = P2[b][r]
  {
    cff* A = SITE(K);
    for (int idx = tid; idx < D * D; idx += nt) {
      const int rr = idx / D, bb = idx - rr * D;
      A[idx] = sh.pf[1][bb * D + rr];
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
    cff* const vv[2] = {Cf, Cf + cap};
    if (tid == 0) {
      cff one;
      one.x = ff_make(1.f, 0.f);
      one.y = ff_make(0.f, 0.f);
      vv[0][0] = one;
    }
    __syncthreads();
    int maxb = 1;
    for (int k = 0; k < K; ++k) {
      const cff* A = SITE(k);
      const int2 dA = DIMS(k);
      const int l = dA.x, r = dA.y;
      maxb = max(maxb, r);
      for (int rr = tid; rr < r; rr += nt) {
        ccacc f = ccacc_zero();
        for (int c = 0; c < l; ++c) {
          cff part = A[((long long)c * D) * r + rr];
          for (int a = 1; a < D; ++a) part = cff_add(part, A[((long long)c * D + a) * r + rr]);
          ccacc_fma(f, vv[cur][c], part);
        }
        vv[cur ^ 1][rr] = ccacc_cff(f);
      }
      __syncthreads();
      cur ^= 1;
    }
    if (tid < D) {
      zc acc = mk<double>(0, 0);
      for (int c = 0; c < D; ++c) cfma(acc, P2[tid * D + c], cff_to(vv[cur][c]));
      b.out[I.out_base + (long long)((step - I.out_origin) % I.out_cap) * D + tid] = acc;
    }
    if (tid == 0) {
      sh.st.step = step;
      sh.st.max_bond = maxb;
      sh.st.ovr_active = 0;
      sh.st.splits += splits;
      sh.st.sweeps64 += sw64;
      sh.st.sweeps32 += sw32;
      sh.st.flops_alg += flops;
      L.state[i] = sh.st;
    }
    __syncthreads();
  }
#undef SLOT
#undef SITE
#undef DIMS
}

}  // namespace otb
