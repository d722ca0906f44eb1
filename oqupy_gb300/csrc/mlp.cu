// BF16 tensor-core GEMM (tcgen05, sm_103a) and the elementwise kernels of
// the MLP surrogate (forward, backward, AdamW).
//
//   C[M][N] = A[M][K] * B[N][K]^T      A, B bf16, K contiguous ("K-major")
//
// One CTA (128 threads) computes a 128 x 128 tile.  Per 64-wide K chunk the
// CTA stages A and B into shared memory in the canonical no-swizzle K-major
// layout of the 5th-generation tensor core -- 8-row x 16-byte core matrices,
// the two core matrices of a 16-deep K step 128 B apart (leading byte
// offset), successive 8-row groups 1024 B apart (stride byte offset) -- and
// one elected thread issues four tcgen05.mma (M=128, N=128, K=16, bf16 in,
// FP32 accumulate) into a 128-column TMEM accumulator, then tcgen05.commit to
// an mbarrier.  Every wait on that mbarrier is bounded; on timeout the kernel
// records an error, still frees its TMEM and returns.  The epilogue reads the
// accumulator with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = tile
// rows) and applies the fused bias / GELU / GELU-gradient step.
#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>

#include "../../include/oqupy_gb300.h"
#include "capi_util.h"

namespace otb {

constexpr int TC_BM = 128, TC_BN = 128, TC_BK = 64;
constexpr int TC_THREADS = 128;
constexpr long long TC_WAIT_LIMIT = 1LL << 26;

enum : int {
  EPI_NONE = 0,       // out = acc (+ bias)
  EPI_GELU = 1,       // z = acc + bias -> z_out (FP32), out = gelu(z)
  EPI_GELU_GRAD = 2,  // out = acc * gelu'(z_in)
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// tcgen05 shared-memory matrix descriptor, no swizzle, K-major
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of the 5th-generation tensor core
  return d;                // base offset 0, layout: no swizzle
}

// instruction descriptor: kind::f16, A/B bf16, D f32, both K-major
__host__ __device__ constexpr uint32_t make_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ float gelu_f(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad_f(float x) {
  return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// stage a 128 x 64 bf16 tile (rows r0.., k k0..) of a row-major [R][K]
// matrix into the core-matrix layout: core (rg, kg) at (rg * 8 + kg) * 128 B
__device__ __forceinline__ void stage_tile(unsigned char* dst, const __nv_bfloat16* src, int R, int K,
                                           int r0, int k0) {
  for (int chunk = threadIdx.x; chunk < TC_BM * (TC_BK / 8); chunk += blockDim.x) {
    const int rr = chunk / (TC_BK / 8), kc = chunk % (TC_BK / 8);
    const int row = r0 + rr, kk = k0 + kc * 8;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (row < R) {
      const __nv_bfloat16* p = src + (size_t)row * K + kk;
      if (kk + 8 <= K && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
        v = *reinterpret_cast<const uint4*>(p);
      } else {
        union {
          uint4 u;
          __nv_bfloat16 h[8];
        } tmp;
        for (int e = 0; e < 8; ++e) tmp.h[e] = (kk + e < K) ? p[e] : __float2bfloat16(0.f);
        v = tmp.u;
      }
    }
    const int rg = rr >> 3, r8 = rr & 7;
    *reinterpret_cast<uint4*>(dst + (size_t)(rg * (TC_BK / 8) + kc) * 128 + r8 * 16) = v;
  }
}

// Same tile as stage_tile, with 16-byte cp.async copies (global -> shared,
// no register round trip) for every aligned full chunk; ragged or unaligned
// chunks (K % 8 != 0, tile edges) are zero-padded through registers.
__device__ __forceinline__ void stage_tile_async(unsigned char* dst, const __nv_bfloat16* src, int R, int K,
                                                 int r0, int k0) {
  for (int chunk = threadIdx.x; chunk < TC_BM * (TC_BK / 8); chunk += blockDim.x) {
    const int rr = chunk / (TC_BK / 8), kc = chunk % (TC_BK / 8);
    const int row = r0 + rr, kk = k0 + kc * 8;
    const int rg = rr >> 3, r8 = rr & 7;
    unsigned char* d = dst + (size_t)(rg * (TC_BK / 8) + kc) * 128 + r8 * 16;
    const __nv_bfloat16* p = src + (size_t)row * K + kk;
    if (row < R && kk + 8 <= K && ((reinterpret_cast<uintptr_t>(p) & 15) == 0)) {
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(d)), "l"(p) : "memory");
    } else {
      union {
        uint4 u;
        __nv_bfloat16 h[8];
      } tmp;
      tmp.u = make_uint4(0, 0, 0, 0);
      if (row < R)
        for (int e = 0; e < 8; ++e)
          if (kk + e < K) tmp.h[e] = p[e];
      *reinterpret_cast<uint4*>(d) = tmp.u;
    }
  }
}

__device__ __forceinline__ bool tc_wait_phase(uint64_t* mbar, int phase) {
  uint32_t done = 0;
  for (long long it = 0; it < TC_WAIT_LIMIT && !done; ++it) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(phase));
  }
  return done != 0;
}

// Two-stage pipeline version of tc_gemm_kernel: while the tensor core runs
// the four MMAs of chunk k, the CTA's cp.async copies of chunk k+1 land in
// the other buffer.  A buffer is refilled only after the mbarrier reports
// the MMAs that read it complete (at most one MMA batch is outstanding at
// any wait, so the phase parity identifies it).  All waits are bounded.
__global__ void __launch_bounds__(TC_THREADS)
    tc_gemm_pipe_kernel(const __nv_bfloat16* __restrict__ A, const __nv_bfloat16* __restrict__ B, int M, int N,
                        int K, const float* __restrict__ bias, int epi, const float* __restrict__ zin,
                        float* __restrict__ zout, float* __restrict__ outf, __nv_bfloat16* __restrict__ outb,
                        int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char tc_dsm[];
  unsigned char* sA[2] = {tc_dsm, tc_dsm + TC_BM * TC_BK * 2};
  unsigned char* sB[2] = {tc_dsm + 2 * TC_BM * TC_BK * 2, tc_dsm + 2 * TC_BM * TC_BK * 2 + TC_BN * TC_BK * 2};
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_err;
  __shared__ int s_drain;  // phase parity of an MMA batch still in flight after a timed-out wait
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * TC_BN;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(TC_BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
    s_err = 0;
    s_drain = -1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = make_idesc(TC_BM, TC_BN);

  const int nk = (K + TC_BK - 1) / TC_BK;
  stage_tile_async(sA[0], A, M, K, m0, 0);
  stage_tile_async(sB[0], B, N, K, n0, 0);
  asm volatile("cp.async.commit_group;" ::: "memory");
  int issued = 0;   // MMA batches committed so far (batch j completes phase j & 1)
  for (int kc = 0; kc < nk; ++kc) {
    const int buf = kc & 1;
    if (kc >= 1) {
      // batch kc - 1 read the other buffer: wait for it before refilling, and
      // so that no more than one batch is outstanding at any parity wait
      if (tid == 0 && !s_err && !tc_wait_phase(&mbar, (kc - 1) & 1)) {
        s_err = 1;
        s_drain = (kc - 1) & 1;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      __syncthreads();
      if (s_err) break;
    }
    if (kc + 1 < nk) {
      stage_tile_async(sA[buf ^ 1], A, M, K, m0, (kc + 1) * TC_BK);
      stage_tile_async(sB[buf ^ 1], B, N, K, n0, (kc + 1) * TC_BK);
      asm volatile("cp.async.commit_group;" ::: "memory");
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      for (int ks = 0; ks < TC_BK / 16; ++ks) {
        const uint64_t ad = make_desc(smem_u32(sA[buf]) + ks * 2 * 128, 128, (TC_BK / 8) * 128);
        const uint64_t bd = make_desc(smem_u32(sB[buf]) + ks * 2 * 128, 128, (TC_BK / 8) * 128);
        const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&mbar)));
    }
    ++issued;
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  // the last committed batch: every earlier one was waited for in the loop
  if (tid == 0 && !s_err && issued > 0 && !tc_wait_phase(&mbar, (issued - 1) & 1)) {
    s_err = 1;
    s_drain = (issued - 1) & 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");

  if (!s_err) {
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < TC_BN; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      if (row < M) {
        for (int j = 0; j < 16; ++j) {
          const int col = n0 + c0 + j;
          if (col >= N) break;
          float v = __uint_as_float(r[j]);
          const size_t o = (size_t)row * N + col;
          if (epi == EPI_GELU_GRAD) {
            v *= gelu_grad_f(zin[o]);
          } else {
            if (bias) v += bias[col];
            if (epi == EPI_GELU) {
              if (zout) zout[o] = v;
              v = gelu_f(v);
            }
          }
          if (outf) outf[o] = v;
          if (outb) outb[o] = __float2bfloat16(v);
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(err, 1);
    // one more bounded wait for the batch still in flight, so that it is
    // not writing the accumulator when the columns are released
    if (s_drain >= 0) tc_wait_phase(&mbar, s_drain);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_BN));
  }
}

__global__ void __launch_bounds__(TC_THREADS)
    tc_gemm_kernel(const __nv_bfloat16* __restrict__ A, const __nv_bfloat16* __restrict__ B, int M,
                   int N, int K, const float* __restrict__ bias, int epi, const float* __restrict__ zin,
                   float* __restrict__ zout, float* __restrict__ outf, __nv_bfloat16* __restrict__ outb,
                   int* __restrict__ err) {
  __shared__ __align__(1024) unsigned char sA[TC_BM * TC_BK * 2];
  __shared__ __align__(1024) unsigned char sB[TC_BN * TC_BK * 2];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_err;
  __shared__ int s_drain;  // phase parity of an MMA batch still in flight after a timed-out wait
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * TC_BN;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(TC_BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
    s_err = 0;
    s_drain = -1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = make_idesc(TC_BM, TC_BN);

  int phase = 0;
  const int nk = (K + TC_BK - 1) / TC_BK;
  for (int kc = 0; kc < nk && !s_err; ++kc) {
    stage_tile(sA, A, M, K, m0, kc * TC_BK);
    stage_tile(sB, B, N, K, n0, kc * TC_BK);
    asm volatile("fence.proxy.async.shared::cta;");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      for (int ks = 0; ks < TC_BK / 16; ++ks) {
        // a 16-deep K step spans core-matrix columns 2 ks and 2 ks + 1
        const uint64_t ad = make_desc(smem_u32(sA) + ks * 2 * 128, 128, (TC_BK / 8) * 128);
        const uint64_t bd = make_desc(smem_u32(sB) + ks * 2 * 128, 128, (TC_BK / 8) * 128);
        const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&mbar)));
    }
    // bounded wait for the MMAs of this chunk (they read sA / sB)
    uint32_t done = 0;
    for (long long it = 0; it < TC_WAIT_LIMIT && !done; ++it) {
      asm volatile(
          "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
          " selp.u32 %0, 1, 0, p;\n}\n"
          : "=r"(done)
          : "r"(smem_u32(&mbar)), "r"(phase));
    }
    if (!done) {
      s_err = 1;
      s_drain = phase;
    }
    phase ^= 1;
    asm volatile("tcgen05.fence::after_thread_sync;");
    __syncthreads();
  }

  if (!s_err) {
    // epilogue: warp w reads TMEM lanes 32 w .. 32 w + 31 (tile rows)
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < TC_BN; c0 += 16) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      if (row < M) {
        for (int j = 0; j < 16; ++j) {
          const int col = n0 + c0 + j;
          if (col >= N) break;
          float v = __uint_as_float(r[j]);
          const size_t o = (size_t)row * N + col;
          if (epi == EPI_GELU_GRAD) {
            v *= gelu_grad_f(zin[o]);
          } else {
            if (bias) v += bias[col];
            if (epi == EPI_GELU) {
              if (zout) zout[o] = v;
              v = gelu_f(v);
            }
          }
          if (outf) outf[o] = v;
          if (outb) outb[o] = __float2bfloat16(v);
        }
      }
    }
  } else if (tid == 0) {
    atomicExch(err, 1);
    // one more bounded wait for the batch still in flight, so that it is
    // not writing the accumulator when the columns are released
    if (s_drain >= 0) tc_wait_phase(&mbar, s_drain);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_BN));
  }
}

// out[c][r] = in[r][c] (bf16), 32 x 32 tiles through shared memory
__global__ void transpose_bf16_kernel(const __nv_bfloat16* __restrict__ in, __nv_bfloat16* __restrict__ out,
                                      int R, int C) {
  __shared__ __nv_bfloat16 t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    t[i][threadIdx.x] = (r < R && c < C) ? in[(size_t)r * C + c] : __float2bfloat16(0.f);
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (c < C && r < R) out[(size_t)c * R + r] = t[threadIdx.x][i];
  }
}

__global__ void f32_to_bf16_kernel(const float* __restrict__ in, __nv_bfloat16* __restrict__ out, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16(in[i]);
}

// column sums of a row-major [R][C] FP32 matrix (bias gradients)
__global__ void colsum_kernel(const float* __restrict__ in, float* __restrict__ out, int R, int C) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  float s = 0.f;
  for (int r = 0; r < R; ++r) s += in[(size_t)r * C + c];
  out[c] = s;
}

// mean-squared-error gradient dY = 2 (Y - T) / (R C) (FP32 and bf16); loss
// partial sums accumulated into *loss
__global__ void mse_grad_kernel(const float* __restrict__ y, const float* __restrict__ t, float* __restrict__ gf,
                                __nv_bfloat16* __restrict__ gb, long long n, float scale, double* loss) {
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float d = y[i] - t[i];
    acc += (double)d * d;
    const float g = 2.f * d * scale;
    gf[i] = g;
    gb[i] = __float2bfloat16(g);
  }
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, acc);
}

// AdamW on FP32 master weights; refreshes the bf16 copy
__global__ void adamw_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                             float* __restrict__ v, __nv_bfloat16* __restrict__ wb, long long n, float lr, float b1,
                             float b2, float eps, float wd, float c1, float c2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float wi = w[i] * (1.f - lr * wd);
    wi -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
  }
}

// y[b][c * nsteps + t] += Bloch component c at time (t + 1) dt of the system
// without the bath: precession of (0, 0, 1) about (Omega, 0, eps) at angular
// frequency w = sqrt(Omega^2 + eps^2) (Rodrigues' rotation).
__global__ void bloch_free_add_kernel(float* __restrict__ y, const float* __restrict__ oe, int B, int nsteps,
                                      float dt) {
  const long long total = (long long)B * nsteps;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(i / nsteps), t = (int)(i - (long long)b * nsteps);
    const float om = oe[2 * b], ep = oe[2 * b + 1];
    const float w = sqrtf(om * om + ep * ep);
    const float nx = w > 0.f ? om / w : 0.f, nz = w > 0.f ? ep / w : 1.f;
    float s, c;
    sincosf(w * dt * (float)(t + 1), &s, &c);
    float* row = y + (size_t)b * 3 * nsteps;
    row[t] += nx * nz * (1.f - c);
    row[nsteps + t] += -nx * s;
    row[2 * nsteps + t] += c + nz * nz * (1.f - c);
  }
}

}  // namespace otb

using namespace otb;

extern "C" otb_status otb_mlp_gemm(const void* A, const void* B, int32_t M, int32_t N, int32_t K,
                                   const float* bias, int32_t epilogue, const float* z_in, float* z_out,
                                   float* out_f32, void* out_bf16, int32_t* err, void* stream) {
  if (!A || !B || !err || M <= 0 || N <= 0 || K <= 0 || epilogue < 0 || epilogue > 2)
    return set_error(OTB_ERR_INVALID_ARG, "bad gemm arguments");
  if (epilogue == EPI_GELU_GRAD && !z_in) return set_error(OTB_ERR_INVALID_ARG, "gelu-grad needs z_in");
  dim3 grid((N + TC_BN - 1) / TC_BN, (M + TC_BM - 1) / TC_BM);
  constexpr int smem = 2 * (TC_BM + TC_BN) * TC_BK * 2;   // two A + B stages, 64 KiB
  static bool attr_set = false;
  if (!attr_set) {
    if (!check_cuda(cudaFuncSetAttribute(tc_gemm_pipe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                    "tc gemm smem"))
      return OTB_ERR_CUDA;
    attr_set = true;
  }
  tc_gemm_pipe_kernel<<<grid, TC_THREADS, smem, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)A, (const __nv_bfloat16*)B, M, N, K, bias, epilogue, z_in, z_out, out_f32,
      (__nv_bfloat16*)out_bf16, err);
  if (!check_cuda(cudaGetLastError(), "tc gemm")) return OTB_ERR_CUDA;
  return OTB_OK;
}

extern "C" otb_status otb_mlp_transpose_bf16(const void* in, void* out, int32_t R, int32_t C, void* stream) {
  if (!in || !out || R <= 0 || C <= 0) return set_error(OTB_ERR_INVALID_ARG, "bad transpose arguments");
  dim3 grid((C + 31) / 32, (R + 31) / 32), block(32, 8);
  transpose_bf16_kernel<<<grid, block, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)in, (__nv_bfloat16*)out,
                                                                  R, C);
  if (!check_cuda(cudaGetLastError(), "transpose")) return OTB_ERR_CUDA;
  return OTB_OK;
}

extern "C" otb_status otb_mlp_f32_to_bf16(const float* in, void* out, int64_t n, void* stream) {
  if (!in || !out || n < 0) return set_error(OTB_ERR_INVALID_ARG, "bad conversion arguments");
  if (n == 0) return OTB_OK;
  f32_to_bf16_kernel<<<1024, 256, 0, (cudaStream_t)stream>>>(in, (__nv_bfloat16*)out, n);
  if (!check_cuda(cudaGetLastError(), "f32->bf16")) return OTB_ERR_CUDA;
  return OTB_OK;
}

extern "C" otb_status otb_mlp_colsum(const float* in, float* out, int32_t R, int32_t C, void* stream) {
  if (!in || !out || R <= 0 || C <= 0) return set_error(OTB_ERR_INVALID_ARG, "bad colsum arguments");
  colsum_kernel<<<(C + 127) / 128, 128, 0, (cudaStream_t)stream>>>(in, out, R, C);
  if (!check_cuda(cudaGetLastError(), "colsum")) return OTB_ERR_CUDA;
  return OTB_OK;
}

extern "C" otb_status otb_mlp_mse_grad(const float* y, const float* t, float* g_f32, void* g_bf16, int64_t n,
                                       double* loss, void* stream) {
  if (!y || !t || !g_f32 || !g_bf16 || !loss || n <= 0) return set_error(OTB_ERR_INVALID_ARG, "bad mse arguments");
  mse_grad_kernel<<<1024, 256, 0, (cudaStream_t)stream>>>(y, t, g_f32, (__nv_bfloat16*)g_bf16, n,
                                                          1.f / (float)n, loss);
  if (!check_cuda(cudaGetLastError(), "mse")) return OTB_ERR_CUDA;
  return OTB_OK;
}

extern "C" otb_status otb_mlp_adamw(float* w, const float* g, float* m, float* v, void* w_bf16, int64_t n, float lr,
                                    float beta1, float beta2, float eps, float weight_decay, int32_t step,
                                    void* stream) {
  if (!w || !g || !m || !v || n <= 0 || step < 1) return set_error(OTB_ERR_INVALID_ARG, "bad adamw arguments");
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  adamw_kernel<<<1024, 256, 0, (cudaStream_t)stream>>>(w, g, m, v, (__nv_bfloat16*)w_bf16, n, lr, beta1, beta2, eps,
                                                       weight_decay, c1, c2);
  if (!check_cuda(cudaGetLastError(), "adamw")) return OTB_ERR_CUDA;
  return OTB_OK;
}

extern "C" otb_status otb_mlp_bloch_free_add(float* y, const float* omega_eps, int32_t B, int32_t nsteps, float dt,
                                            void* stream) {
  if (!y || !omega_eps || B <= 0 || nsteps <= 0 || !(dt > 0.f))
    return set_error(OTB_ERR_INVALID_ARG, "bad bloch arguments");
  bloch_free_add_kernel<<<1024, 256, 0, (cudaStream_t)stream>>>(y, omega_eps, B, nsteps, dt);
  if (!check_cuda(cudaGetLastError(), "bloch free add")) return OTB_ERR_CUDA;
  return OTB_OK;
}
