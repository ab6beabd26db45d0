// ft_gemm_tc.cuh -- the surrogate's training GEMMs on the fifth-generation
// tensor cores (tcgen05.mma, FP32 accumulators in tensor memory).
//
// C[M x N] = A[M x K] B[K x N] with BF16 operands read through arbitrary
// strides (the forward layers, the backward dX = dZ W and the weight
// gradients dW = dZ^T H of the MLP, see ft_mlp.cu), and the same fused
// epilogues as the warp-level kernel it replaces: bias + SiLU (pre-activation
// and BF16 activation out), plain store (optionally + bias), and the SiLU
// gradient.  Included by ft_mlp.cu after its tcgen05 helpers.
//
// One CTA of four warps computes a 128-row tile of C over the whole N
// (N <= 128, padded to a multiple of 16) and a K range: per 64-column chunk
// of K every thread stages its share of the A and B chunks into shared memory
// as K-major core-matrix images without swizzle (element (r, k) at byte
// (r / 8) * 1024 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2), one thread
// issues the chunk's K = 16 MMAs (M = 128) and commits them to an mbarrier,
// and every thread waits on it before the next chunk overwrites the images.
// The epilogue reads the accumulator rows back with tcgen05.ld (warp w owns
// TMEM lanes 32 w .. 32 w + 31, one row per thread).  Weight gradients
// (K = the batch) split K over CTAs and add the FP32 partial tiles in a fixed
// order afterwards, so training stays bitwise reproducible.
#pragma once

namespace tcg {
constexpr int kThreads = 128;
constexpr int kBK = 64;                       // K columns per staged chunk
constexpr uint32_t kA = 0;                    // [128 x 64] BF16 image, 16 KB
constexpr uint32_t kB = kA + 128 * kBK * 2;   // [<=128 x 64] BF16 image, 16 KB
constexpr uint32_t kBar = kB + 128 * kBK * 2; // mbarrier, TMEM base, abort flag
constexpr uint32_t kSmem = kBar + 16 + 1024;  // + alignment slack of the base
}  // namespace tcg

// 16 bytes (8 BF16 values along K) of the core-matrix image: value j is
// element (r, k0 + j) of the operand whose element (r, k) sits at
// src[r * sr + k * sk]; zero outside r < rows, k < K.
__device__ __forceinline__ uint4 tcg_gather8(const bf16 *src, long long sr, long long sk, int r,
                                             int rows, int k0, int K) {
  uint4 v = make_uint4(0u, 0u, 0u, 0u);
  if (r >= rows || k0 >= K) return v;
  const bf16 *p = src + (long long)r * sr + (long long)k0 * sk;
  if (sk == 1 && k0 + 8 <= K && ((reinterpret_cast<uintptr_t>(p) & 15) == 0))
    return *reinterpret_cast<const uint4 *>(p);
  bf16 *e = reinterpret_cast<bf16 *>(&v);
#pragma unroll
  for (int j = 0; j < 8; ++j)
    if (k0 + j < K) e[j] = p[(long long)j * sk];
  return v;
}

// Stage rows [0, rows_pad) x K chunk [k0, k0 + 64) of an operand into an image.
// Consecutive threads take consecutive rows of one 8-column group, so the
// strided (transposed) reads coalesce across the warp.
__device__ __forceinline__ void tcg_stage(unsigned char *img, const bf16 *src, long long sr,
                                          long long sk, int r0, int rows, int rows_pad, int k0,
                                          int K) {
  const int chunks = rows_pad * (tcg::kBK / 8);
  for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
    const int q = c / rows_pad, r = c - q * rows_pad;  // 8-column group, row
    const uint4 v = tcg_gather8(src, sr, sk, r0 + r, rows, k0 + 8 * q, K);
    *reinterpret_cast<uint4 *>(img + (r >> 3) * 1024 + q * 128 + (r & 7) * 16) = v;
  }
}

// EPI as k_gemm (kEpiStore, kEpiBias, kEpiBiasSilu, kEpiSiluGrad).  part !=
// null: write the FP32 tile of K slice blockIdx.y to part[slice][M][N]
// instead (the sum runs in k_splitk_reduce).
template <int EPI>
__global__ void __launch_bounds__(tcg::kThreads) k_gemm_tc(const GemmArgs g, int Npad, int kslice,
                                                           float *part, int *err) {
  extern __shared__ __align__(128) unsigned char tcg_raw[];
  unsigned char *sm = tcg_raw + ((1024 - (smem_u32(tcg_raw) & 1023)) & 1023);
  const int t = threadIdx.x, warp = t >> 5;
  const uint32_t bar = smem_u32(sm + tcg::kBar);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + tcg::kBar + 8);
  volatile int *abort = reinterpret_cast<volatile int *>(sm + tcg::kBar + 12);
  const int m0 = blockIdx.x * 128;
  const int kb = blockIdx.y * kslice, ke = min(g.K, kb + kslice);
  const uint32_t ncols = Npad <= 32 ? 32u : (Npad <= 64 ? 64u : 128u);
  if (t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t idesc = umma_idesc_bf16(128, Npad);
  uint32_t phase = 0;
  bool ok = true;
  for (int k0 = kb; k0 < ke && ok; k0 += tcg::kBK) {
    tcg_stage(sm + tcg::kA, g.A, g.sam, g.sak, m0, g.M, 128, k0, ke);
    tcg_stage(sm + tcg::kB, g.B, g.sbn, g.sbk, 0, g.N, Npad, k0, ke);
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    if (t == 0) {
      tc_fence_after();
      const int steps = (min(tcg::kBK, ke - k0) + 15) / 16;
      const uint32_t sa = smem_u32(sm + tcg::kA), sb = smem_u32(sm + tcg::kB);
      for (int kk = 0; kk < steps; ++kk)
        umma_bf16(tmem, umma_sdesc(sa + 256 * kk, 128, 1024), umma_sdesc(sb + 256 * kk, 128, 1024),
                  idesc, (k0 > kb || kk > 0) ? 1u : 0u);
      umma_commit(bar);
    }
    // every thread waits for the chunk's MMAs before the images are reused
    if (!mbar_wait(bar, phase, abort)) ok = false;
    phase ^= 1u;
    tc_fence_after();
    __syncthreads();
    if (*abort) ok = false;
  }
  if (ok && kb < ke) {
    // epilogue: row m0 + 32 warp + lane, columns in chunks of 16
    const int r = 32 * warp + (t & 31);
    const long long i = (long long)m0 + r;
    for (int c0 = 0; c0 < Npad; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
      if (i >= g.M) continue;
      if (part) {
        float *dst = part + ((long long)blockIdx.y * g.M + i) * g.N;
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (c0 + j < g.N) dst[c0 + j] = v[j];
        continue;
      }
      if constexpr (EPI == kEpiBiasSilu) {
#pragma unroll
        for (int j = 0; j < 16; j += 2) {
          const int c = c0 + j;
          if (c >= g.N) break;
          const float v0 = v[j] + g.bias[c], v1 = v[j + 1] + g.bias[c + 1];
          g.Z[i * g.N + c] = v0;
          g.Z[i * g.N + c + 1] = v1;
          *reinterpret_cast<uint32_t *>(g.H + i * g.N + c) = silu_bf16x2(v0, v1);
        }
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int c = c0 + j;
          if (c >= g.N) break;
          if (EPI == kEpiStore) {
            g.C[i * g.scm + (long long)c * g.scn] = v[j];
          } else if (EPI == kEpiBias) {
            g.C[i * g.scm + (long long)c * g.scn] = v[j] + g.bias[c];
          } else {  // kEpiSiluGrad
            g.dZ[i * g.N + c] = __float2bfloat16_rn(v[j] * dsilu(g.Zp[i * g.N + c]));
          }
        }
      }
    }
  }
  if (!ok && t == 0) atomicOr(err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols)
                 : "memory");
}

// C = sum over the K slices of the partial tiles, in slice order
__global__ void k_splitk_reduce(const float *part, int slices, int M, int N, float *C,
                                long long scm, long long scn) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)M * N) return;
  const long long i = idx / N, c = idx - i * N;
  float s = 0.f;
  for (int k = 0; k < slices; ++k) s += part[(long long)k * M * N + idx];
  C[i * scm + c * scn] = s;
}
