// Rank-revealing QR preconditioner + one-sided Jacobi on the reduced factor:
// the truncated bond split of both precision forms for splits of >= 8
// columns (smaller splits run plain Jacobi, jacobi.cuh).
//
// Replaces, like jacobi.cuh, the truncated SVD that the reference obtains
// from tensornetwork's split_node_full_svd(max_truncation_err=epsrel,
// relative=True) (oqupy/backends/node_array.py:262-268, 285-291, 541-547),
// with the rank rule chi = #{i : sqrt(sum_{j>=i} s_j^2) > epsrel * s_0}
// (oqupy/mps_mpo.py:452-457).
//
// The oriented matrix A (R x N, R >= N) is factorised A P = Q R by
// Householder QR with column pivoting, stopped at the first step k whose
// remaining block has Frobenius norm below delta |R_00|.  One-sided Jacobi
// then orthogonalises the columns of Z = P R[0:k, :]^H (N x k): the pivoted
// R is graded, so Z converges in few sweeps, and it has only k columns.
// With Z V = W orthogonal, A ~= (Q V) Sigma (W / Sigma)^H, so W = A^H U Sigma:
// the caller receives the conjugate-side factor (N x k, ld N).  The dropped
// block's squared norm belongs to the tail of every kept index and is added
// to the tail sums, so the rank decision is that of the full decomposition up
// to delta.
//
// Arithmetic (template parameter T):
//   double -- complex128 form: FP64 throughout; delta at the factorisation's
//             own backward-error level (1e-14 by default);
//   ff     -- mixed form: double-float (ff.cuh) on the FP32 pipe; delta
//             min(1e-3 epsrel, 1e-9) by default.
// Norms, the descending sort, the tail sums and the rank decision are FP64 in
// both (jacobi_finish).
//
// Synchronisation: one __syncthreads per QR column.  No columns are
// exchanged: column p_i chosen at step i keeps its storage; a short list of
// the unchosen columns is exchanged instead.  The pivot, the remaining mass
// and the reflector scalars are computed redundantly by every warp from data
// no thread writes during the step (partial norms and the column list are
// double-buffered by step parity; the diagonal R_ii is stored one step late,
// when no warp reads that column any more).
#pragma once

#include "jacobi.cuh"

namespace otb {

template <typename T>
struct QA;

// Householder scalars of a column x (rows i..) with head x0 and squared norm
// n2: v0 = e (|x0| + |x|), alpha = -e |x| (the new diagonal), beta =
// 1 / (|x| (|x| + |x0|)) (H = I - beta v v^H), inv = 1 / v0, tau = beta |v0|^2
// (the unit-diagonal form), e = x0 / |x0| (1 for x0 = 0); a zero column gives
// H = I.
template <typename E, typename S>
struct Refl {
  E v0, alpha, inv;
  S beta;
  double tau;
};

template <>
struct QA<double> {
  typedef cx<double> E;  // element of the working matrix
  typedef double S;      // accurate real scalar
  static constexpr bool kFF = false;
  static __device__ __forceinline__ E from(cx<double> z) { return z; }
  static __device__ __forceinline__ cx<double> to(const E& e) { return e; }
  static __device__ __forceinline__ S zero() { return 0.0; }
  static __device__ __forceinline__ S fromd(double d) { return d; }
  static __device__ __forceinline__ double tod(S s) { return s; }
  static __device__ __forceinline__ S add(S a, S b) { return a + b; }
  static __device__ __forceinline__ S mul(S a, S b) { return a * b; }
  static __device__ __forceinline__ S shfl(S v, int off) { return __shfl_xor_sync(0xffffffffu, v, off, 32); }
  static __device__ __forceinline__ S abs2_acc(const E& x, S acc) { return fma(x.x, x.x, fma(x.y, x.y, acc)); }
  static __device__ __forceinline__ float abs2f(const E& x) { return (float)fma(x.x, x.x, x.y * x.y); }
  // (wr, wi) += conj(a) x
  static __device__ __forceinline__ void dotj(S& wr, S& wi, const E& a, const E& x) {
    wr = fma(a.x, x.x, fma(a.y, x.y, wr));
    wi = fma(a.x, x.y, fma(-a.y, x.x, wi));
  }
  static __device__ __forceinline__ S fin(S v) { return v; }
  // x - a (bx + i by)
  static __device__ __forceinline__ E sub_scaled(const E& x, const E& a, S bx, S by) {
    return mk<double>(x.x - fma(a.x, bx, -a.y * by), x.y - fma(a.x, by, a.y * bx));
  }
  static __device__ __forceinline__ E conj(const E& x) { return mk<double>(x.x, -x.y); }
  static __device__ __forceinline__ E zeroE() { return mk<double>(0.0, 0.0); }
  static __device__ __forceinline__ E oneE() { return mk<double>(1.0, 0.0); }
  static __device__ __forceinline__ E mulc(const E& a, const E& b) { return cmul(a, b); }
  // FP64: evaluated by one lane of each warp and broadcast (the FP64 pipe is
  // the narrow one)
  static constexpr bool kAllLanes = false;
  static __device__ __forceinline__ Refl<E, S> reflector(S n2, const E& x0) {
    Refl<E, S> r;
    const double nrm = sqrt(fmax(n2, 0.0));
    const double a0 = sqrt(x0.x * x0.x + x0.y * x0.y);
    const double ex = (a0 > 0.0) ? x0.x / a0 : 1.0, ey = (a0 > 0.0) ? x0.y / a0 : 0.0;
    const double m = a0 + nrm;
    r.v0 = mk<double>(ex * m, ey * m);
    r.alpha = mk<double>(-ex * nrm, -ey * nrm);
    r.inv = (m > 0.0) ? mk<double>(ex / m, -ey / m) : mk<double>(0.0, 0.0);
    r.beta = (nrm > 0.0) ? 1.0 / (nrm * m) : 0.0;
    r.tau = (nrm > 0.0) ? m / nrm : 0.0;
    return r;
  }
  static __device__ __forceinline__ Refl<E, S> bcast(Refl<E, S> r) {
    r.v0.x = __shfl_sync(0xffffffffu, r.v0.x, 0);
    r.v0.y = __shfl_sync(0xffffffffu, r.v0.y, 0);
    r.alpha.x = __shfl_sync(0xffffffffu, r.alpha.x, 0);
    r.alpha.y = __shfl_sync(0xffffffffu, r.alpha.y, 0);
    r.inv.x = __shfl_sync(0xffffffffu, r.inv.x, 0);
    r.inv.y = __shfl_sync(0xffffffffu, r.inv.y, 0);
    r.beta = __shfl_sync(0xffffffffu, r.beta, 0);
    r.tau = __shfl_sync(0xffffffffu, r.tau, 0);
    return r;
  }
};

template <>
struct QA<ff> {
  typedef cff E;
  typedef ff S;
  static constexpr bool kFF = true;
  static __device__ __forceinline__ E from(cx<double> z) { return cff_from(z); }
  static __device__ __forceinline__ cx<double> to(const E& e) { return cff_to(e); }
  static __device__ __forceinline__ S zero() { return ff_make(0.f, 0.f); }
  static __device__ __forceinline__ S fromd(double d) { return ff_from(d); }
  static __device__ __forceinline__ double tod(S s) { return ff_to(s); }
  static __device__ __forceinline__ S add(S a, S b) { return ff_add(a, b); }
  static __device__ __forceinline__ S mul(S a, S b) { return ff_mul(a, b); }
  static __device__ __forceinline__ S shfl(S v, int off) { return ff_shfl_xor(v, off); }
  static __device__ __forceinline__ S abs2_acc(const E& x, S acc) { return ff_fma(x.x, x.x, ff_fma(x.y, x.y, acc)); }
  static __device__ __forceinline__ float abs2f(const E& x) { return fmaf(x.x.hi, x.x.hi, x.y.hi * x.y.hi); }
  // wr + i wi += conj(a) x as compensated accumulators (ffp_acc): the
  // (hi, lo) pair is left unnormalised inside a loop; fin() normalises it
  static __device__ __forceinline__ void dotj(S& wr, S& wi, const E& a, const E& x) {
    ffp_acc(a.x.hi, a.x.lo, x.x.hi, x.x.lo, wr.hi, wr.lo);
    ffp_acc(a.y.hi, a.y.lo, x.y.hi, x.y.lo, wr.hi, wr.lo);
    ffp_acc(a.x.hi, a.x.lo, x.y.hi, x.y.lo, wi.hi, wi.lo);
    ffp_acc(-a.y.hi, -a.y.lo, x.x.hi, x.x.lo, wi.hi, wi.lo);
  }
  static __device__ __forceinline__ S fin(S v) { return ffacc_norm(v.hi, v.lo); }
  // x - a (bx + i by), each component one compensated accumulation
  static __device__ __forceinline__ E sub_scaled(const E& x, const E& a, S bx, S by) {
    E r;
    float h = x.x.hi, l = x.x.lo;
    ffp_acc(-a.x.hi, -a.x.lo, bx.hi, bx.lo, h, l);
    ffp_acc(a.y.hi, a.y.lo, by.hi, by.lo, h, l);
    r.x = ffacc_norm(h, l);
    h = x.y.hi;
    l = x.y.lo;
    ffp_acc(-a.x.hi, -a.x.lo, by.hi, by.lo, h, l);
    ffp_acc(-a.y.hi, -a.y.lo, bx.hi, bx.lo, h, l);
    r.y = ffacc_norm(h, l);
    return r;
  }
  static __device__ __forceinline__ E conj(const E& x) {
    E r = x;
    r.y.hi = -r.y.hi;
    r.y.lo = -r.y.lo;
    return r;
  }
  static __device__ __forceinline__ E zeroE() {
    E r;
    r.x = ff_make(0.f, 0.f);
    r.y = r.x;
    return r;
  }
  static __device__ __forceinline__ E oneE() {
    E r;
    r.x = ff_make(1.f, 0.f);
    r.y = ff_make(0.f, 0.f);
    return r;
  }
  static __device__ __forceinline__ E mulc(const E& a, const E& b) {
    E r;
    r.x = ff_sub(ff_mul(a.x, b.x), ff_mul(a.y, b.y));
    r.y = ff_add(ff_mul(a.x, b.y), ff_mul(a.y, b.x));
    return r;
  }
  // double-float on the FP32 pipe: evaluated by every lane (n2 and x0 are
  // the same in all lanes), no FP64 instruction and no broadcast
  static constexpr bool kAllLanes = true;
  static __device__ __forceinline__ Refl<E, S> reflector(S n2, const E& x0) {
    Refl<E, S> r;
    const ff z = ff_make(0.f, 0.f);
    const ff nrm = ff_sqrt(n2);
    const ff a0 = ff_sqrt(ff_fma(x0.x, x0.x, ff_mul(x0.y, x0.y)));
    ff ex = ff_make(1.f, 0.f), ey = z;
    if (a0.hi > 0.f) {
      const ff ia = ff_recip(a0);
      ex = ff_mul(x0.x, ia);
      ey = ff_mul(x0.y, ia);
    }
    const ff m = ff_add(a0, nrm);
    r.v0.x = ff_mul(ex, m);
    r.v0.y = ff_mul(ey, m);
    r.alpha.x = ff_make(-ff_mul(ex, nrm).hi, -ff_mul(ex, nrm).lo);
    r.alpha.y = ff_make(-ff_mul(ey, nrm).hi, -ff_mul(ey, nrm).lo);
    r.inv.x = z;
    r.inv.y = z;
    r.beta = z;
    r.tau = 0.0;
    if (m.hi > 0.f) {
      const ff im = ff_recip(m);
      r.inv.x = ff_mul(ex, im);
      const ff t = ff_mul(ey, im);
      r.inv.y = ff_make(-t.hi, -t.lo);
    }
    if (nrm.hi > 0.f) {
      r.beta = ff_recip(ff_mul(nrm, m));
      r.tau = ff_to(ff_mul(m, ff_recip(nrm)));
    }
    return r;
  }
  static __device__ __forceinline__ Refl<E, S> bcast(Refl<E, S> r) { return r; }
};

// Default relative cut of the QR (the remaining block's Frobenius norm over
// |R_00|) for each arithmetic.
__device__ __forceinline__ float qr_default_delta(bool ffarith, double epsrel) {
  return ffarith ? (float)fmin(1e-3 * epsrel, 1e-9) : 1e-14f;
}

// Householder QR with column pivoting of X (R x N, column-major ld R), in
// place, without column exchanges.  Workspace: cn holds 2 N floats (partial
// squared column norms by column, double-buffered by step parity), lists
// 2 N shorts (by step parity: positions 0..i-1 the columns chosen at steps
// 0..i-1, positions i..N-1 the unchosen ones).  Returns k and writes
// colstep[j] (N ints, in cn's storage, valid after the call) = the step at
// which column j was chosen, N for never; for i < k, X[j * R + i] = R[i][j]
// for every column j with colstep[j] >= i (colstep[j] == i: the diagonal of
// step i).  *tail2 is the remaining squared mass at the stop (0 when all N
// steps ran).
template <typename T>
__device__ int qrcp_inplace(typename QA<T>::E* X, int R, int N, float delta, float* cn, short* lists,
                            float* tail2) {
  typedef QA<T> Q;
  typedef typename Q::E E;
  typedef typename Q::S S;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane32 = tid & 31, warp = tid >> 5, nw = nt >> 5;
  for (int j = warp; j < N; j += nw) {
    float acc = 0.f;
    const E* c = X + (size_t)j * R;
    for (int r = lane32; r < R; r += 32) acc += Q::abs2f(c[r]);
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (lane32 == 0) cn[j] = acc;
  }
  for (int j = tid; j < N; j += nt) lists[j] = (short)j;
  __syncthreads();
  float r00 = 0.f, t2 = 0.f;
  int k = N;
  int pend_p = -1;  // thread 0: column and value of the previous step's diagonal
  E pend_a = Q::zeroE();
  for (int i = 0; i < N; ++i) {
    const float* cur = cn + (i & 1) * N;
    float* nxt = cn + ((i + 1) & 1) * N;
    const short* Lc = lists + (i & 1) * N;
    short* Ln = lists + ((i + 1) & 1) * N;
    // (a) pivot (largest partial norm, lowest list position on ties) and
    // remaining mass over the unchosen columns, by every warp; the xor
    // butterfly leaves bitwise-identical results in every lane, and every
    // warp reduces the same data in the same order
    float bv = -1.f, sum = 0.f;
    int bq = N;
    for (int q = i + lane32; q < N; q += 32) {
      const float v = cur[Lc[q]];
      sum += v;
      if (v > bv) {
        bv = v;
        bq = q;
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, bv, off);
      const int oq = __shfl_xor_sync(0xffffffffu, bq, off);
      if (ov > bv || (ov == bv && oq < bq)) {
        bv = ov;
        bq = oq;
      }
      sum += __shfl_xor_sync(0xffffffffu, sum, off);
    }
    if (i == 0) {
      r00 = bv;
    } else if (sum < delta * delta * r00) {
      k = i;
      t2 = sum;
      break;
    }
    const int pos = bq;
    const int p = Lc[pos];
    // next step's list (the other parity buffer, read by no one in this
    // step): history through position i, the unchosen columns after it
    for (int q = i - 1 + tid; q < N; q += nt) {
      if (q >= 0) Ln[q] = (q == i) ? (short)p : ((q == pos) ? Lc[i] : Lc[q]);
    }
    // the previous step's diagonal: its column is read by no one any more
    if (tid == 0 && pend_p >= 0) X[(size_t)pend_p * R + (i - 1)] = pend_a;
    // (b) reflector of column p, rows i..R-1 (column p is not written in
    // this step): H = I - beta v v^H, v = x - alpha e_i, alpha = -e |x|,
    // v_i = e (|x_i| + |x|), beta = 1 / (|x| (|x| + |x_i|)), e = x_i / |x_i|
    const E* v = X + (size_t)p * R;
    S n2 = Q::zero();
    for (int r = i + lane32; r < R; r += 32) n2 = Q::abs2_acc(v[r], n2);
    for (int off = 16; off > 0; off >>= 1) n2 = Q::add(n2, Q::shfl(n2, off));
    Refl<E, S> rf;
    if (Q::kAllLanes || lane32 == 0) rf = Q::reflector(n2, v[i]);
    rf = Q::bcast(rf);
    if (tid == 0) {
      pend_p = p;
      pend_a = rf.alpha;
    }
    const E v0 = rf.v0;
    const S beta = rf.beta;
    // (c) apply H to the other unchosen columns (list positions i..N-1 but
    // pos), refresh their partial norms (rows > i) in the other buffer
    const int G = jacobi_group(R - i);
    const int gl = tid & (G - 1), group = tid / G, ngroups = nt / G;
    const int nrest = N - i - 1;
    for (int tb = 0; tb < nrest; tb += ngroups) {
      const int t = tb + group;
      const bool act = t < nrest;
      const int q = i + t + ((i + t >= pos) ? 1 : 0);
      const int j = act ? Lc[q] : p;
      E* cj = X + (size_t)j * R;
      S wr = Q::zero(), wi = Q::zero();
      if (act) {
        for (int r = i + gl; r < R; r += G) Q::dotj(wr, wi, (r == i) ? v0 : v[r], cj[r]);
      }
      wr = Q::fin(wr);
      wi = Q::fin(wi);
      for (int off = G >> 1; off > 0; off >>= 1) {
        wr = Q::add(wr, Q::shfl(wr, off));
        wi = Q::add(wi, Q::shfl(wi, off));
      }
      float s2 = 0.f;
      if (act) {
        const S bx = Q::mul(beta, wr), by = Q::mul(beta, wi);
        for (int r = i + gl; r < R; r += G) {
          const E x = Q::sub_scaled(cj[r], (r == i) ? v0 : v[r], bx, by);
          cj[r] = x;
          if (r > i) s2 += Q::abs2f(x);
        }
      }
      for (int off = G >> 1; off > 0; off >>= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, off, 32);
      if (act && gl == 0) nxt[j] = s2;
    }
    __syncthreads();
  }
  if (tid == 0 && pend_p >= 0) X[(size_t)pend_p * R + (k - 1)] = pend_a;
  // a stop at step k leaves warps that may still be reading cn in that
  // step's pivot search
  __syncthreads();
  // colstep from the final list (buffer k & 1), over cn's storage
  const short* L = lists + (k & 1) * N;
  int* colstep = reinterpret_cast<int*>(cn);
  for (int q = tid; q < N; q += nt) colstep[L[q]] = (q < k) ? q : N;
  __syncthreads();
  *tail2 = t2;
  return k;
}

// Unpivoted Householder QR of Z (M x K, M >= K, column-major ld), in place,
// one __syncthreads per column: on return the upper triangle of Z[0:K, :]
// holds R, below the diagonal column i holds its reflector w_i scaled to
// w_i[i] = 1 (implicit), and tau[i] (FP64) makes H_i = I - tau_i w_i w_i^H,
// Z = H_0 H_1 ... H_{K-1} [R; 0].  The reflector scalars are computed by
// every warp from column i, which no thread writes during step i; column
// i's scaling and diagonal are written in step i + 1, when no warp reads it.
template <typename T>
__device__ void householder_unit(typename QA<T>::E* Z, int M, int K, int ld, double* tau) {
  typedef QA<T> Q;
  typedef typename Q::E E;
  typedef typename Q::S S;
  const int tid = threadIdx.x, nt = blockDim.x, lane32 = tid & 31;
  E pinv = Q::zeroE(), palpha = Q::zeroE();   // previous column's 1 / v_i and diagonal
  for (int i = 0; i < K; ++i) {
    if (i > 0) {
      E* c = Z + (size_t)(i - 1) * ld;
      for (int r = i + tid; r < M; r += nt) c[r] = Q::mulc(c[r], pinv);
      if (tid == 0) c[i - 1] = palpha;
    }
    const E* v = Z + (size_t)i * ld;
    S n2 = Q::zero();
    for (int r = i + lane32; r < M; r += 32) n2 = Q::abs2_acc(v[r], n2);
    for (int off = 16; off > 0; off >>= 1) n2 = Q::add(n2, Q::shfl(n2, off));
    Refl<E, S> rf;
    if (Q::kAllLanes || lane32 == 0) rf = Q::reflector(n2, v[i]);
    rf = Q::bcast(rf);
    if (tid == 0) tau[i] = rf.tau;
    pinv = rf.inv;
    palpha = rf.alpha;
    const E v0 = rf.v0;
    const S beta = rf.beta;
    const int G = jacobi_group(M - i);
    const int gl = tid & (G - 1), group = tid / G, ngroups = nt / G;
    const int nrest = K - i - 1;
    for (int tb = 0; tb < nrest; tb += ngroups) {
      const int t = tb + group;
      const bool act = t < nrest;
      E* cj = Z + (size_t)(act ? i + 1 + t : i) * ld;
      S wr = Q::zero(), wi = Q::zero();
      if (act) {
        for (int r = i + gl; r < M; r += G) Q::dotj(wr, wi, (r == i) ? v0 : v[r], cj[r]);
      }
      wr = Q::fin(wr);
      wi = Q::fin(wi);
      for (int off = G >> 1; off > 0; off >>= 1) {
        wr = Q::add(wr, Q::shfl(wr, off));
        wi = Q::add(wi, Q::shfl(wi, off));
      }
      if (act) {
        const S bx = Q::mul(beta, wr), by = Q::mul(beta, wi);
        for (int r = i + gl; r < M; r += G) cj[r] = Q::sub_scaled(cj[r], (r == i) ? v0 : v[r], bx, by);
      }
    }
    __syncthreads();
  }
  if (K > 0) {
    E* c = Z + (size_t)(K - 1) * ld;
    for (int r = K + tid; r < M; r += nt) c[r] = Q::mulc(c[r], pinv);
    if (tid == 0) c[K - 1] = palpha;
  }
  __syncthreads();
}

// Y <- Q Y for the first ncols columns of Y (M x ncols, ld ldy), Q = H_0 ...
// H_{K-1} as stored by householder_unit: reflectors applied last-first, one
// __syncthreads each.
template <typename T>
__device__ void apply_q_unit(const typename QA<T>::E* Z, int M, int K, int ld, const double* tau,
                             typename QA<T>::E* Y, int ncols, int ldy) {
  typedef QA<T> Q;
  typedef typename Q::E E;
  typedef typename Q::S S;
  const int tid = threadIdx.x, nt = blockDim.x;
  const E one = Q::oneE();
  for (int i = K - 1; i >= 0; --i) {
    const E* w = Z + (size_t)i * ld;
    const S ti = Q::fromd(tau[i]);
    const int G = jacobi_group(M - i);
    const int gl = tid & (G - 1), group = tid / G, ngroups = nt / G;
    for (int jb = 0; jb < ncols; jb += ngroups) {
      const int j = jb + group;
      const bool act = j < ncols;
      E* y = Y + (size_t)(act ? j : 0) * ldy;
      S sr = Q::zero(), si = Q::zero();
      if (act) {
        for (int r = i + gl; r < M; r += G) Q::dotj(sr, si, (r == i) ? one : w[r], y[r]);
      }
      sr = Q::fin(sr);
      si = Q::fin(si);
      for (int off = G >> 1; off > 0; off >>= 1) {
        sr = Q::add(sr, Q::shfl(sr, off));
        si = Q::add(si, Q::shfl(si, off));
      }
      if (act) {
        const S bx = Q::mul(ti, sr), by = Q::mul(ti, si);
        for (int r = i + gl; r < M; r += G) y[r] = Q::sub_scaled(y[r], (r == i) ? one : w[r], bx, by);
      }
    }
    __syncthreads();
  }
}

// The split driver.  W (R x N, FP64, ld R) holds the oriented matrix and is
// scratch afterwards; X (R x N elements of QA<T>::E) is the QR workspace; zs /
// zs_bytes is spare shared memory for the Jacobi operand.  delta <= 0 selects
// the default cut.  Returns the kept rank; *Wout (FP64, N x k, ld N, in X's
// storage) holds V_A Sigma with norm / perm describing its columns as in
// jacobi_finish.
template <typename T>
__device__ int qr_jacobi_truncate(cx<double>* W, int R, int N, typename QA<T>::E* X, unsigned char* zs,
                                  size_t zs_bytes, double epsrel, float delta, double* norm, int* perm,
                                  JacobiShared* sh, cx<double>** Wout) {
  typedef QA<T> Q;
  typedef typename Q::E E;
  constexpr bool FF = Q::kFF;
  const int tid = threadIdx.x;
  const int nt = blockDim.x;
  // scale by a power of two so that the largest entry is of order one (exact
  // in FP64; keeps the double-float exponents in range)
  double mx = 0.0;
  for (int idx = tid; idx < R * N; idx += nt) mx = fmax(mx, fmax(fabs(W[idx].x), fabs(W[idx].y)));
  for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if ((tid & 31) == 0) sh->red[tid >> 5] = mx;
  __syncthreads();
  if (tid == 0) {
    double v = 0.0;
    for (int w = 0; w < nt / 32; ++w) v = fmax(v, sh->red[w]);
    sh->red[32] = (v > 0.0 && isfinite(v)) ? ldexp(1.0, ilogb(v)) : 1.0;
  }
  __syncthreads();
  const double scale = sh->red[32];
  const double inv = 1.0 / scale;
  for (int idx = tid; idx < R * N; idx += nt) X[idx] = Q::from(cscale(W[idx], inv));
  __syncthreads();
  // QR bookkeeping in the (not yet used) norm / perm arrays: partial norms
  // (2 N floats) then colstep (N ints) in norm[], column lists (2 N shorts)
  // in perm[]
  float* cn = reinterpret_cast<float*>(norm);
  if (!(delta > 0.f)) delta = qr_default_delta(FF, epsrel);
  float tail2;
  const int k = qrcp_inplace<T>(X, R, N, delta, cn, reinterpret_cast<short*>(perm), &tail2);
  const int* colstep = reinterpret_cast<const int*>(norm);
  // Z = P R[0:k, :]^H: row q (original column q of A), column i
  E* Z = ((size_t)N * k * sizeof(E) <= zs_bytes) ? reinterpret_cast<E*>(zs) : reinterpret_cast<E*>(W);
  for (int idx = tid; idx < N * k; idx += nt) {
    const int i = idx / N, q = idx - i * N;
    Z[idx] = (colstep[q] >= i) ? Q::conj(X[(size_t)q * R + i]) : Q::zeroE();
  }
  __syncthreads();
  int sw, sw64 = 0;
  bool done;
  cx<double>* O = reinterpret_cast<cx<double>*>(X);
  if (k >= 8 && 2 * k <= N) {
    // Second (unpivoted) QR, Z = Q2 [R2; 0]: the Jacobi runs on the k x k R2
    // instead of the N rows of Z, the rank is decided from R2's singular
    // values (those of Z), and W = Q2 [W2; 0] is formed for the kept columns
    // only, in sorted order.  X's storage: [0, N kk) the kept columns,
    // [N k, N k + k^2) R2, then tau (k doubles): N k + k^2 + k <= R N for
    // 2 k <= N <= R.
    E* R2 = X + (size_t)N * k;
    double* tau = reinterpret_cast<double*>(X + (size_t)N * k + (size_t)k * k);
    householder_unit<T>(Z, N, k, N, tau);
    for (int idx = tid; idx < k * k; idx += nt) {
      const int c = idx / k, r = idx - c * k;
      R2[idx] = (r <= c) ? Z[(size_t)c * N + r] : Q::zeroE();
    }
    __syncthreads();
    cx<double>* R2d = reinterpret_cast<cx<double>*>(R2);
    if (FF) {
      sw = jacobi_sweeps_ff(reinterpret_cast<cff*>(R2), k, k, k, sh);
      done = sw < JACOBI_MAX_SWEEPS || sh->noise_converged;
      for (int idx = tid; idx < k * k; idx += nt) R2d[idx] = cscale(Q::to(R2[idx]), scale);
      __syncthreads();
      if (!done) sw64 = jacobi_sweeps<double>(R2d, k, k, k, nullptr, 0, sh);
    } else {
      sw64 = jacobi_sweeps<double>(R2d, k, k, k, nullptr, 0, sh);
      sw = 0;
      for (int idx = tid; idx < k * k; idx += nt) R2d[idx] = cscale(R2d[idx], scale);
      __syncthreads();
    }
    if (tid == 0) sh->sweeps32 = sw;
    const int kk = jacobi_finish<double>(R2d, k, k, k, epsrel, norm, perm, sh, sw64,
                                         (double)tail2 * scale * scale);
    if (tid == 0) sh->sweeps = sw64;
    E* Y = X;
    for (int idx = tid; idx < N * kk; idx += nt) {
      const int j = idx / N, r = idx - j * N;
      Y[idx] = (r < k) ? Q::from(cscale(R2d[(size_t)perm[j] * k + r], inv)) : Q::zeroE();
    }
    __syncthreads();
    apply_q_unit<T>(Z, N, k, N, tau, Y, kk, N);
    for (int idx = tid; idx < N * kk; idx += nt) O[idx] = cscale(Q::to(Y[idx]), scale);
    // the kept columns are stored sorted: norms in that order, identity perm
    for (int j = tid; j < kk; j += nt) tau[j] = norm[perm[j]];
    __syncthreads();
    for (int j = tid; j < kk; j += nt) {
      norm[j] = tau[j];
      perm[j] = j;
    }
    __syncthreads();
    *Wout = O;
    return kk;
  }
  if (FF) {
    sw = jacobi_sweeps_ff(reinterpret_cast<cff*>(Z), N, k, N, sh);
    done = sw < JACOBI_MAX_SWEEPS || sh->noise_converged;
    for (int idx = tid; idx < N * k; idx += nt) O[idx] = cscale(Q::to(Z[idx]), scale);
    __syncthreads();
    // FP64 fallback: if the double-float sweeps did not settle, finish the
    // (nearly orthogonal) matrix with FP64 sweeps; their count is reported
    if (!done) {
      sw64 = jacobi_sweeps<double>(O, N, k, N, nullptr, 0, sh);
      done = true;
    }
  } else {
    sw64 = jacobi_sweeps<double>(reinterpret_cast<cx<double>*>(Z), N, k, N, nullptr, 0, sh);
    sw = 0;
    for (int idx = tid; idx < N * k; idx += nt) O[idx] = cscale(Q::to(Z[idx]), scale);
    __syncthreads();
  }
  if (tid == 0) sh->sweeps32 = sw;
  const int kk = jacobi_finish<double>(O, N, k, N, epsrel, norm, perm, sh, sw64, (double)tail2 * scale * scale);
  if (tid == 0) sh->sweeps = sw64;
  __syncthreads();
  *Wout = O;
  return kk;
}

// ---------------------------------------------------------------------------
// Double-float input and output (the mixed form's TEMPO step keeps sites,
// carries and theta in double-float): no FP64 instruction per matrix element.
// ---------------------------------------------------------------------------

// x * 2^e for a double-float complex x: exact (two float multiplications by
// a power of two) unless it leaves the float range.
__device__ __forceinline__ cff cff_ldexp(cff x, float p2) {
  x.x.hi *= p2;
  x.x.lo *= p2;
  x.y.hi *= p2;
  x.y.lo *= p2;
  return x;
}

// FP64 norms of the n columns of W (m rows, ld), accumulated in double-float.
__device__ inline void cff_column_norms(const cff* W, int m, int n, int ld, double* norm) {
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int j = tid / 32; j < n; j += nt / 32) {
    const int l = tid & 31;
    ff acc = ff_make(0.f, 0.f);
    const cff* c = W + (size_t)j * ld;
    for (int r = l; r < m; r += 32) acc = ff_fma(c[r].x, c[r].x, ff_fma(c[r].y, c[r].y, acc));
    for (int off = 16; off > 0; off >>= 1) acc = ff_add(acc, ff_shfl_xor(acc, off));
    if (l == 0) norm[j] = ff_to(ff_sqrt(acc));
  }
  __syncthreads();
}

// FP64 sweeps on a double-float matrix whose double-float sweeps did not
// settle: converted in place (both 16-byte elements), swept, converted back.
__device__ inline int cff_fp64_fallback(cff* W, int m, int n, int ld, JacobiShared* sh) {
  const int tid = threadIdx.x, nt = blockDim.x;
  cx<double>* Wd = reinterpret_cast<cx<double>*>(W);
  for (int j = 0; j < n; ++j)
    for (int r = tid; r < m; r += nt) {
      const size_t q = (size_t)j * ld + r;
      Wd[q] = cff_to(W[q]);
    }
  __syncthreads();
  const int sw = jacobi_sweeps<double>(Wd, m, n, ld, nullptr, 0, sh);
  for (int j = 0; j < n; ++j)
    for (int r = tid; r < m; r += nt) {
      const size_t q = (size_t)j * ld + r;
      W[q] = cff_from(Wd[q]);
    }
  __syncthreads();
  return sw;
}

// The split driver on a double-float input already in X (R x N, ld R,
// scaled by 1 / scale, a power of two), with Zbuf (R x N) as spare global
// storage and zs / zs_bytes spare shared memory.  Returns the kept rank;
// *Wout (double-float, N x kk or N x k, ld N, in original units) holds
// V_A Sigma with norm / perm as in jacobi_finish (the k <= N / 2 branch
// stores its kept columns sorted, perm the identity).
__device__ inline int qr_jacobi_truncate_ff(cff* X, int R, int N, double scale, cff* Zbuf, unsigned char* zs,
                                            size_t zs_bytes, double epsrel, float delta, double* norm,
                                            int* perm, JacobiShared* sh, cff** Wout) {
  typedef QA<ff> Q;
  const int tid = threadIdx.x;
  const int nt = blockDim.x;
  const float up = (float)scale;    // power of two in float range for the data this path sees
  float* cn = reinterpret_cast<float*>(norm);
  if (!(delta > 0.f)) delta = qr_default_delta(true, epsrel);
  float tail2;
  const int k = qrcp_inplace<ff>(X, R, N, delta, cn, reinterpret_cast<short*>(perm), &tail2);
  const int* colstep = reinterpret_cast<const int*>(norm);
  cff* Z = ((size_t)N * k * sizeof(cff) <= zs_bytes) ? reinterpret_cast<cff*>(zs) : Zbuf;
  for (int idx = tid; idx < N * k; idx += nt) {
    const int i = idx / N, q = idx - i * N;
    Z[idx] = (colstep[q] >= i) ? Q::conj(X[(size_t)q * R + i]) : Q::zeroE();
  }
  __syncthreads();
  const double t2 = (double)tail2 * scale * scale;
  if (k >= 8 && 2 * k <= N) {
    // second QR, Jacobi on the k x k R2, kept columns transformed back
    // (as in qr_jacobi_truncate)
    cff* R2 = X + (size_t)N * k;
    double* tau = reinterpret_cast<double*>(X + (size_t)N * k + (size_t)k * k);
    householder_unit<ff>(Z, N, k, N, tau);
    for (int idx = tid; idx < k * k; idx += nt) {
      const int c = idx / k, r = idx - c * k;
      R2[idx] = (r <= c) ? Z[(size_t)c * N + r] : Q::zeroE();
    }
    __syncthreads();
    const int sw = jacobi_sweeps_ff(R2, k, k, k, sh);
    int sw64 = 0;
    if (!(sw < JACOBI_MAX_SWEEPS || sh->noise_converged)) sw64 = cff_fp64_fallback(R2, k, k, k, sh);
    if (tid == 0) sh->sweeps32 = sw;
    cff_column_norms(R2, k, k, k, norm);
    for (int j = tid; j < k; j += nt) norm[j] *= scale;
    __syncthreads();
    const int kk = jacobi_rank(k, epsrel, norm, perm, sh, sw64, t2);
    if (tid == 0) sh->sweeps = sw64;
    cff* Y = X;
    for (int idx = tid; idx < N * kk; idx += nt) {
      const int j = idx / N, r = idx - j * N;
      Y[idx] = (r < k) ? R2[(size_t)perm[j] * k + r] : Q::zeroE();
    }
    __syncthreads();
    apply_q_unit<ff>(Z, N, k, N, tau, Y, kk, N);
    for (int idx = tid; idx < N * kk; idx += nt) Y[idx] = cff_ldexp(Y[idx], up);
    for (int j = tid; j < kk; j += nt) tau[j] = norm[perm[j]];
    __syncthreads();
    for (int j = tid; j < kk; j += nt) {
      norm[j] = tau[j];
      perm[j] = j;
    }
    __syncthreads();
    *Wout = Y;
    return kk;
  }
  const int sw = jacobi_sweeps_ff(Z, N, k, N, sh);
  int sw64 = 0;
  if (!(sw < JACOBI_MAX_SWEEPS || sh->noise_converged)) sw64 = cff_fp64_fallback(Z, N, k, N, sh);
  if (tid == 0) sh->sweeps32 = sw;
  cff_column_norms(Z, N, k, N, norm);
  for (int j = tid; j < k; j += nt) norm[j] *= scale;
  __syncthreads();
  const int kk = jacobi_rank(k, epsrel, norm, perm, sh, sw64, t2);
  if (tid == 0) sh->sweeps = sw64;
  for (int idx = tid; idx < N * k; idx += nt) Z[idx] = cff_ldexp(Z[idx], up);
  __syncthreads();
  *Wout = Z;
  return kk;
}

}  // namespace otb
