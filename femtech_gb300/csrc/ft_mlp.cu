// ft_mlp.cu -- BF16 tensor-core MLP for the constitutive surrogate: training
// data from the plain GOH law, forward / backward GEMMs, Adam, prediction.
//
// GEMMs use the warp-level BF16 tensor-core MMA (m16n8k16, FP32 accumulate)
// with fused epilogues (bias + SiLU, SiLU derivative); every reduction (bias
// gradients, the batch dimension of weight gradients) runs in a fixed order,
// so training is bitwise reproducible.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "ft_common.h"
#include "ft_mlp.cuh"
#include "ftgpu.h"

namespace ftgpu {

int record_error(int code, const char *msg);  // ft_api.cu: sets ftgpu_last_error()

typedef __nv_bfloat16 bf16;

// ---------------- counter-based random numbers ----------------
__host__ __device__ inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__device__ inline double urand(uint64_t seed, uint64_t i, int k) {
  return (mix64(seed ^ mix64(i * 64 + k)) >> 11) * (1.0 / 9007199254740992.0);
}
__device__ inline double nrand(uint64_t seed, uint64_t i, int k) {  // Box-Muller
  double u1 = urand(seed, i, 2 * k) + 1e-300, u2 = urand(seed, i, 2 * k + 1);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

// Training sample i: a random rotation Q (unit quaternion), principal
// stretches in [lo, hi], U = Q diag(l) Q^T, a random unit fibre; target = the
// scaled residual of the plain law's isochoric PK2 over its linearisation.
__global__ void k_mlp_gen(long long n, uint64_t seed, double lo, double hi, MatP<double> mp,
                          SurrogateLaw law, bf16 *X, float *T) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double q[4], qn = 0;
  for (int k = 0; k < 4; ++k) {
    q[k] = nrand(seed, i, k);
    qn += q[k] * q[k];
  }
  qn = 1.0 / sqrt(qn);
  for (int k = 0; k < 4; ++k) q[k] *= qn;
  const double w = q[0], x = q[1], y = q[2], z = q[3];
  const double Q[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)},
                          {2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)},
                          {2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)}};
  double l[3];
  for (int k = 0; k < 3; ++k) l[k] = lo + (hi - lo) * urand(seed, i, 10 + k);
  double a0[3], an = 0;
  for (int k = 0; k < 3; ++k) {
    a0[k] = nrand(seed, i, 20 + k);
    an += a0[k] * a0[k];
  }
  an = 1.0 / sqrt(an);
  for (int k = 0; k < 3; ++k) a0[k] *= an;
  double D[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += Q[r][k] * l[k] * Q[c][k];
      D[r][c] = s - (r == c ? 1.0 : 0.0);
    }
  const double Jm1 = jm1_of(D);
  Sym6<double> Si, Sv;
  mat_hgo_parts<double, true>(mp, D, Jm1, a0, Si, Sv);
  Sym6<double> e2 = two_E(D);
  double E[6] = {0.5 * e2.xx, 0.5 * e2.yy, 0.5 * e2.zz, 0.5 * e2.yz, 0.5 * e2.xz, 0.5 * e2.xy};
  float xf[kMlpUsedIn];
  double Slin[6], scale;
  surrogate_features(E, a0, law, xf, Slin, scale);
  const double S[6] = {Si.xx, Si.yy, Si.zz, Si.yz, Si.xz, Si.xy};
  for (int k = 0; k < kMlpIn; ++k) X[i * kMlpIn + k] = __float2bfloat16_rn(k < kMlpUsedIn ? xf[k] : 0.f);
  for (int k = 0; k < kMlpOut; ++k) T[i * kMlpOut + k] = k < 6 ? float((S[k] - Slin[k]) / scale) : 0.f;
}

// ---------------- generic BF16 tensor-core GEMM ----------------
// C(M x N) = A(M x K) B(K x N); element (i,k) of A at A[i*sam + k*sak], (k,j)
// of B at B[k*sbk + j*sbn].  One warp computes a 16 x 32 tile with four
// m16n8k16 MMAs per 16-wide K step; a block is 4 warps (64 x 32).
enum { kEpiStore = 0, kEpiBiasSilu = 1, kEpiBias = 2, kEpiSiluGrad = 3 };

__device__ inline uint32_t pack2(bf16 lo, bf16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// The activation of every forward path (training, both inference kernels):
// SiLU on BF16 pairs, h = z / 2 rounded to BF16, then h + h tanh(h) with a
// BF16-pair tanh and fused multiply-add -- one MUFU operation per two values.
// The activations are stored in BF16 anyway; training with the same rounding
// makes the trained network exact for the fast inference arithmetic.
__device__ __forceinline__ uint32_t silu_h_bf16x2(float h0, float h1) {
  uint32_t hp, th, out;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(hp) : "f"(h1), "f"(h0));  // h0 low, h1 high
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(th) : "r"(hp));
  asm("fma.rn.bf16x2 %0, %1, %2, %1;" : "=r"(out) : "r"(hp), "r"(th));
  return out;
}
__device__ __forceinline__ uint32_t silu_bf16x2(float z0, float z1) {
  return silu_h_bf16x2(0.5f * z0, 0.5f * z1);
}

// derivative of the exact SiLU at the FP32 pre-activation (backward pass)
__device__ inline float dsilu(float z) {
  const float s = 1.f / (1.f + __expf(-z));
  return s * (1.f + z * (1.f - s));
}

struct GemmArgs {
  int M, N, K;
  const bf16 *A;
  long long sam, sak;
  const bf16 *B;
  long long sbk, sbn;
  float *C;          // kEpiStore / kEpiBias: output (f32)
  long long scm, scn;
  const float *bias; // kEpiBiasSilu / kEpiBias
  float *Z;          // kEpiBiasSilu: pre-activation out, [M][N]
  bf16 *H;           // kEpiBiasSilu: activation out, [M][N]
  const float *Zp;   // kEpiSiluGrad: pre-activation of the layer below, [M][N]
  bf16 *dZ;          // kEpiSiluGrad: gradient out, [M][N]
};

template <int EPI>
__global__ void __launch_bounds__(128) k_gemm(const GemmArgs g) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gq = lane >> 2, tq = lane & 3;
  const long long m0 = (long long)blockIdx.x * 64 + warp * 16;
  const int n0 = blockIdx.y * 32;
  const bf16 zero = __float2bfloat16_rn(0.f);
  auto Aat = [&](long long i, int k) -> bf16 {
    return (i < g.M && k < g.K) ? g.A[i * g.sam + k * g.sak] : zero;
  };
  auto Bat = [&](int k, int j) -> bf16 {
    return (k < g.K && j < g.N) ? g.B[(long long)k * g.sbk + (long long)j * g.sbn] : zero;
  };
  float acc[4][4];
#pragma unroll
  for (int j = 0; j < 4; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
  for (int k0 = 0; k0 < g.K; k0 += 16) {
    const uint32_t a0 = pack2(Aat(m0 + gq, k0 + 2 * tq), Aat(m0 + gq, k0 + 2 * tq + 1));
    const uint32_t a1 = pack2(Aat(m0 + gq + 8, k0 + 2 * tq), Aat(m0 + gq + 8, k0 + 2 * tq + 1));
    const uint32_t a2 = pack2(Aat(m0 + gq, k0 + 2 * tq + 8), Aat(m0 + gq, k0 + 2 * tq + 9));
    const uint32_t a3 = pack2(Aat(m0 + gq + 8, k0 + 2 * tq + 8), Aat(m0 + gq + 8, k0 + 2 * tq + 9));
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int nn = n0 + 8 * j + gq;
      const uint32_t b0 = pack2(Bat(k0 + 2 * tq, nn), Bat(k0 + 2 * tq + 1, nn));
      const uint32_t b1 = pack2(Bat(k0 + 2 * tq + 8, nn), Bat(k0 + 2 * tq + 9, nn));
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
          "{%8,%9}, {%0,%1,%2,%3};\n"
          : "+f"(acc[j][0]), "+f"(acc[j][1]), "+f"(acc[j][2]), "+f"(acc[j][3])
          : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }
  }
  if constexpr (EPI == kEpiBiasSilu) {  // column pairs (c, c + 1) -> one BF16 pair (N is even)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int hp = 0; hp < 2; ++hp) {
        const long long i = m0 + gq + 8 * hp;
        const int c = n0 + 8 * j + 2 * tq;
        if (i >= g.M || c >= g.N) continue;
        const float v0 = acc[j][2 * hp] + g.bias[c], v1 = acc[j][2 * hp + 1] + g.bias[c + 1];
        g.Z[i * g.N + c] = v0;
        g.Z[i * g.N + c + 1] = v1;
        *reinterpret_cast<uint32_t *>(g.H + i * g.N + c) = silu_bf16x2(v0, v1);
      }
  } else {
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const long long i = m0 + gq + (h >= 2 ? 8 : 0);
        const int c = n0 + 8 * j + 2 * tq + (h & 1);
        if (i >= g.M || c >= g.N) continue;
        float v = acc[j][h];
        if (EPI == kEpiStore) {
          g.C[i * g.scm + (long long)c * g.scn] = v;
        } else if (EPI == kEpiBias) {
          g.C[i * g.scm + (long long)c * g.scn] = v + g.bias[c];
        } else {  // kEpiSiluGrad
          g.dZ[i * g.N + c] = __float2bfloat16_rn(v * dsilu(g.Zp[i * g.N + c]));
        }
      }
  }
}

// column sums of an [M][N] bf16 matrix (bias gradients), fixed-order tree
__global__ void k_colsum(const bf16 *dZ, long long M, int N, float *out) {
  __shared__ float red[256];
  const int c = blockIdx.x;
  float s = 0.f;
  for (long long i = threadIdx.x; i < M; i += blockDim.x) s += __bfloat162float(dZ[i * N + c]);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = red[0];
}

// MSE over the used outputs: dY = 2 (Y - T) / (n_used * M), per-row loss partials
__global__ void k_mse(const float *Y, const float *T, long long M, bf16 *dY, float *rowloss) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M) return;
  float l = 0.f;
  const float sc = 2.f / (float(kMlpUsedOut) * float(M));
  for (int k = 0; k < kMlpOut; ++k) {
    const float d = k < kMlpUsedOut ? Y[i * kMlpOut + k] - T[i * kMlpOut + k] : 0.f;
    l += d * d;
    dY[i * kMlpOut + k] = __float2bfloat16_rn(sc * d);
  }
  rowloss[i] = l;
}

__global__ void k_sum(const float *v, long long n, float *out) {
  __shared__ float red[256];
  float s = 0.f;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) s += v[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// sum of squares of the used target columns, FP64, one partial per block
// (summed on the host in block order, so the result is reproducible)
__global__ void k_target_sumsq(const float *T, long long n, double *out) {
  __shared__ double red[256];
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n * kMlpOut;
       i += (long long)gridDim.x * blockDim.x)
    if ((i % kMlpOut) < kMlpUsedOut) s += double(T[i]) * double(T[i]);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

__global__ void k_scale(float *v, long long n, float a) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    v[i] *= a;
}

// features of host-given strains (for ftgpu_surrogate_predict): BF16 rows,
// the linear part and the output scale, as the element kernel forms them
__global__ void k_predict_features(long long n, const double *E, const double *a0,
                                   SurrogateLaw law, bf16 *X, double *Slin, double *scale) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double e[6], a[3], sl[6], sc;
  for (int k = 0; k < 6; ++k) e[k] = E[6 * i + k];
  for (int k = 0; k < 3; ++k) a[k] = a0[3 * i + k];
  float xf[kMlpUsedIn];
  surrogate_features(e, a, law, xf, sl, sc);
  for (int k = 0; k < kMlpIn; ++k) X[i * kMlpIn + k] = __float2bfloat16_rn(k < kMlpUsedIn ? xf[k] : 0.f);
  for (int k = 0; k < 6; ++k) Slin[6 * i + k] = sl[k];
  scale[i] = sc;
}

__global__ void k_predict_combine(long long n, const float *Y, double *Slin, const double *scale) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < 6; ++k) Slin[6 * i + k] += scale[i] * double(Y[i * kMlpOut + k]);
}

// Adam on the FP32 master parameters, then the BF16 weight copies
__global__ void k_adam(float *P, const float *G, float *Mo, float *V, int n, float lr, float b1,
                       float b2, float eps, float c1, float c2, bf16 *Wb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = G[i];
  const float m = b1 * Mo[i] + (1.f - b1) * g;
  const float v = b2 * V[i] + (1.f - b2) * g * g;
  Mo[i] = m;
  V[i] = v;
  const float p = P[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
  P[i] = p;
  Wb[i] = __float2bfloat16_rn(p);
}

__global__ void k_to_bf16(const float *P, int n, bf16 *Wb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) Wb[i] = __float2bfloat16_rn(P[i]);
}

// ---------------- fused inference ----------------
// Persistent blocks of 8 warps; the weights are staged once per block in
// shared memory with rows padded by 8 bf16 (row stride 68 words: the 8 x 4
// lanes of a B-fragment load hit 32 distinct banks).  A warp owns 16 rows and
// keeps them in registers through all four layers: the FP32 accumulator
// fragments of one layer (pairs of n8 tiles) are exactly the BF16 A fragments
// of the next layer's k16 chunks.
constexpr int kLdW0 = kMlpIn + 8, kLdW = kMlpHid + 8;
constexpr size_t kInferSmem =
    sizeof(bf16) * ((size_t)kMlpHid * kLdW0 + 2 * (size_t)kMlpHid * kLdW + (size_t)kMlpOut * kLdW) +
    sizeof(float) * (3 * kMlpHid + kMlpOut);

__device__ inline void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// one hidden layer 128 -> 128: a (8 k-chunks) -> bias + SiLU -> next (8 k-chunks)
__device__ inline void hidden_layer(const uint32_t (&a)[8][4], uint32_t (&nx)[8][4],
                                    const bf16 *W, const float *b, int gq, int tq) {
#pragma unroll
  for (int kc = 0; kc < 8; ++kc) {  // output n-tiles 2kc and 2kc+1
    float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
    const bf16 *r0 = W + (16 * kc + gq) * kLdW + 2 * tq;
    const bf16 *r1 = W + (16 * kc + 8 + gq) * kLdW + 2 * tq;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      mma16816(c0, a[k], *reinterpret_cast<const uint32_t *>(r0 + 16 * k),
               *reinterpret_cast<const uint32_t *>(r0 + 16 * k + 8));
      mma16816(c1, a[k], *reinterpret_cast<const uint32_t *>(r1 + 16 * k),
               *reinterpret_cast<const uint32_t *>(r1 + 16 * k + 8));
    }
    const float bA0 = b[16 * kc + 2 * tq], bA1 = b[16 * kc + 2 * tq + 1];
    const float bB0 = b[16 * kc + 8 + 2 * tq], bB1 = b[16 * kc + 8 + 2 * tq + 1];
    nx[kc][0] = silu_bf16x2(c0[0] + bA0, c0[1] + bA1);
    nx[kc][1] = silu_bf16x2(c0[2] + bA0, c0[3] + bA1);
    nx[kc][2] = silu_bf16x2(c1[0] + bB0, c1[1] + bB1);
    nx[kc][3] = silu_bf16x2(c1[2] + bB0, c1[3] + bB1);
  }
}

__global__ void __launch_bounds__(256) k_mlp_infer(const bf16 *__restrict__ X, long long n,
                                                   const bf16 *__restrict__ Wg,
                                                   const float *__restrict__ P,
                                                   float *__restrict__ Y) {
  extern __shared__ __align__(16) unsigned char sm[];
  bf16 *W0 = reinterpret_cast<bf16 *>(sm);
  bf16 *W1 = W0 + kMlpHid * kLdW0;
  bf16 *W2 = W1 + kMlpHid * kLdW;
  bf16 *W3 = W2 + kMlpHid * kLdW;
  float *bs = reinterpret_cast<float *>(W3 + kMlpOut * kLdW);
  for (int i = threadIdx.x; i < kMlpHid * kMlpIn; i += blockDim.x)
    W0[(i / kMlpIn) * kLdW0 + i % kMlpIn] = Wg[kOffW0 + i];
  for (int i = threadIdx.x; i < kMlpHid * kMlpHid; i += blockDim.x) {
    W1[(i / kMlpHid) * kLdW + i % kMlpHid] = Wg[kOffW1 + i];
    W2[(i / kMlpHid) * kLdW + i % kMlpHid] = Wg[kOffW2 + i];
  }
  for (int i = threadIdx.x; i < kMlpOut * kMlpHid; i += blockDim.x)
    W3[(i / kMlpHid) * kLdW + i % kMlpHid] = Wg[kOffW3 + i];
  for (int i = threadIdx.x; i < kMlpHid; i += blockDim.x) {
    bs[i] = P[kOffB0 + i];
    bs[kMlpHid + i] = P[kOffB1 + i];
    bs[2 * kMlpHid + i] = P[kOffB2 + i];
  }
  if (threadIdx.x < kMlpOut) bs[3 * kMlpHid + threadIdx.x] = P[kOffB3 + threadIdx.x];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gq = lane >> 2, tq = lane & 3;
  const long long tiles = (n + 15) / 16;
  for (long long tile = (long long)blockIdx.x * 8 + warp; tile < tiles;
       tile += (long long)gridDim.x * 8) {
    const long long r0 = tile * 16 + gq, r1 = r0 + 8;
    // layer 0 (K = 16): A fragment straight from the input rows
    uint32_t a0[4];
    a0[0] = r0 < n ? *reinterpret_cast<const uint32_t *>(X + r0 * kMlpIn + 2 * tq) : 0u;
    a0[1] = r1 < n ? *reinterpret_cast<const uint32_t *>(X + r1 * kMlpIn + 2 * tq) : 0u;
    a0[2] = r0 < n ? *reinterpret_cast<const uint32_t *>(X + r0 * kMlpIn + 8 + 2 * tq) : 0u;
    a0[3] = r1 < n ? *reinterpret_cast<const uint32_t *>(X + r1 * kMlpIn + 8 + 2 * tq) : 0u;
    uint32_t h[8][4], g[8][4];
#pragma unroll
    for (int kc = 0; kc < 8; ++kc) {
      float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
      const bf16 *w0 = W0 + (16 * kc + gq) * kLdW0 + 2 * tq;
      const bf16 *w1 = W0 + (16 * kc + 8 + gq) * kLdW0 + 2 * tq;
      mma16816(c0, a0, *reinterpret_cast<const uint32_t *>(w0),
               *reinterpret_cast<const uint32_t *>(w0 + 8));
      mma16816(c1, a0, *reinterpret_cast<const uint32_t *>(w1),
               *reinterpret_cast<const uint32_t *>(w1 + 8));
      const float bA0 = bs[16 * kc + 2 * tq], bA1 = bs[16 * kc + 2 * tq + 1];
      const float bB0 = bs[16 * kc + 8 + 2 * tq], bB1 = bs[16 * kc + 8 + 2 * tq + 1];
      h[kc][0] = silu_bf16x2(c0[0] + bA0, c0[1] + bA1);
      h[kc][1] = silu_bf16x2(c0[2] + bA0, c0[3] + bA1);
      h[kc][2] = silu_bf16x2(c1[0] + bB0, c1[1] + bB1);
      h[kc][3] = silu_bf16x2(c1[2] + bB0, c1[3] + bB1);
    }
    hidden_layer(h, g, W1, bs + kMlpHid, gq, tq);
    hidden_layer(g, h, W2, bs + 2 * kMlpHid, gq, tq);
    // output layer (N = 8)
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    const bf16 *w3 = W3 + gq * kLdW + 2 * tq;
#pragma unroll
    for (int k = 0; k < 8; ++k)
      mma16816(c, h[k], *reinterpret_cast<const uint32_t *>(w3 + 16 * k),
               *reinterpret_cast<const uint32_t *>(w3 + 16 * k + 8));
    const float b0 = bs[3 * kMlpHid + 2 * tq], b1 = bs[3 * kMlpHid + 2 * tq + 1];
    if (r0 < n) {
      Y[r0 * kMlpOut + 2 * tq] = c[0] + b0;
      Y[r0 * kMlpOut + 2 * tq + 1] = c[1] + b1;
    }
    if (r1 < n) {
      Y[r1 * kMlpOut + 2 * tq] = c[2] + b0;
      Y[r1 * kMlpOut + 2 * tq + 1] = c[3] + b1;
    }
  }
}

// ---------------- fused inference on the 5th-generation tensor cores ----------------
// A persistent, warp-specialised kernel: one CTA per SM stages the weights
// once and keeps three 128-row tiles in flight, one per *slot* (13 warps: the
// register file is split over the SM's four schedulers, and 4 warps of 128
// registers fill one scheduler's share).  Slot s owns an
// input image, an activation image and TMEM columns [128 s, 128 s + 128); row r
// of its tile is TMEM lane r.  Warps 4s .. 4s+3 are the slot's epilogue (warp
// 4s + q reaches lanes 32 q .. 32 q + 31); warp 12 issues every MMA from one
// thread.  Per layer the slot's epilogue makes its operand visible and
// arrives on full[s]; the MMA thread waits on full[s], issues the layer
// (tcgen05.mma, M = 128, K = 16 per instruction, BF16 x BF16 -> FP32) and
// commits to done[s]; the epilogue waits on done[s], reads the accumulator
// (tcgen05.ld), applies SiLU and writes the BF16 activations as the next
// layer's A operand.  While one slot runs its epilogue the tensor core serves
// the others.  The biases ride in the MMAs: every activation image carries
// two constant columns of ones (columns 128, 129 of a K = 144 image; input
// columns 14, 15, unused features) against the bias split into a BF16 high
// part and the BF16 rounding of the rest (b = hi + lo to 2^-16) in the weight
// images -- one more K = 16 MMA per hidden layer (the tensor core is mostly
// idle) instead of a 128-column TMEM store per row and layer.  W0..W2 and
// b0..b2 are staged times 1/2 (exact), so an accumulator holds h = z / 2 and
// SiLU(z) = z sigmoid(z) = h + h tanh(h) is evaluated on BF16 pairs: one
// MUFU tanh and one FMA per two values.
// Every wait is bounded; a wait that gives
// up raises a shared abort flag that ends all roles, and the error word.
//
// Shared-memory operand images are K-major without swizzle: 8-row x 16-byte
// core matrices, element (r, k) of an image with K columns at byte
//   (r / 8) * 16 K + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// i.e. leading-dimension (K-direction) byte offset 128 and stride-dimension
// (8-row group) byte offset 16 K in the matrix descriptors.
namespace tc {
constexpr int kSlots = 3;
constexpr int kMmaWarp = 4 * kSlots;               // warp 12
constexpr int kThreads = 32 * (kMmaWarp + 1);      // 416: at most 4 warps per SMSP
constexpr int kKH = kMlpHid + 16;                  // hidden K plus the bias columns (144)
constexpr uint32_t kSBOH = 16 * kKH;               // 8-row group stride of a K = 144 image
constexpr uint32_t kW0 = 0;                        // [128 x 16]     4 KB (bias in columns 14, 15)
constexpr uint32_t kW1 = kW0 + 128 * 16 * 2;       // [128 x 144]   36 KB
constexpr uint32_t kW2 = kW1 + 128 * kKH * 2;      // [128 x 144]   36 KB
constexpr uint32_t kW3 = kW2 + 128 * kKH * 2;      // [16 x 144]   4.5 KB (rows 8..15 zero)
constexpr uint32_t kXs = kW3 + 16 * kKH * 2;       // per slot [128 x 16]    4 KB
constexpr uint32_t kHs = kXs + kSlots * 4096;      // per slot [128 x 144]  36 KB
constexpr uint32_t kBar = kHs + kSlots * 128 * kKH * 2;  // full[], done[], TMEM base, abort
constexpr uint32_t kSmem = kBar + 72 + 128;        // + alignment slack of the base
constexpr uint32_t kTmemCols = 512;               // 128 per slot, rounded to a power of 2
constexpr int kWaitLimit = 1 << 21;                // try_wait rounds before giving up
}  // namespace tc

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: start, leading / stride byte offsets,
// descriptor version 1 (bits 46-47), no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t umma_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) |
         ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}

// instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// D (+)= A B^T for one K = 16 step
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   bar)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// bounded wait for the completion of phase `parity` of an mbarrier; gives up
// (false) after kWaitLimit rounds or when another role raised *abort
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int *abort) {
  for (int it = 0; it < tc::kWaitLimit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (*abort) return false;
  }
  *abort = 1;
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// 32 consecutive FP32 accumulator columns of this thread's TMEM lane (the
// wait for the load is part of the same statement, so no use can precede it)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// A row-major BF16 weight matrix [rows x Ks] (times `scale`) into a K-major
// core-matrix image with K = Ks + 16 whose columns Ks, Ks + 1 hold the bias
// (times `scale`) as a BF16 high part and the BF16 rounding of the rest; rows
// up to rows_pad zero.  For the K = 16 input layer (Ks = 16) the bias goes
// into columns 14, 15 instead (bcol), replacing weights of unused features.
__device__ __forceinline__ void stage_kmajor_bias(unsigned char *img, const bf16 *src,
                                                  const float *b, int rows, int rows_pad, int Ks,
                                                  int Ki, int bcol, float scale) {
  // chunk d of the image (16 bytes) is row 8 g + rr, columns 8 q .. 8 q + 7,
  // with d = (g * (Ki / 8) + q) * 8 + rr: consecutive threads write
  // consecutive chunks, rows_pad * Ki / 8 chunks in all
  const int per_group = Ki;  // chunks per 8-row group: (Ki / 8) * 8
  for (int d = threadIdx.x; d < rows_pad * (Ki / 8); d += blockDim.x) {
    const int g = d / per_group, rem = d - g * per_group;
    const int q = rem >> 3, r = 8 * g + (rem & 7), k0 = 8 * q;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (r < rows) {
      bf16 *e = reinterpret_cast<bf16 *>(&v);
      if (k0 + 8 <= Ks && (bcol >= k0 + 8 || bcol + 1 < k0)) {
        v = *reinterpret_cast<const uint4 *>(src + (long long)r * Ks + k0);
        if (scale != 1.f) {
#pragma unroll
          for (int j = 0; j < 8; ++j) e[j] = __float2bfloat16_rn(__bfloat162float(e[j]) * scale);
        }
      } else {
        const float bs = b[r] * scale;
        const bf16 hi = __float2bfloat16_rn(bs);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int k = k0 + j;
          float w = 0.f;
          if (k == bcol)
            w = __bfloat162float(hi);
          else if (k == bcol + 1)
            w = bs - __bfloat162float(hi);
          else if (k < Ks)
            w = __bfloat162float(src[(long long)r * Ks + k]) * scale;
          e[j] = __float2bfloat16_rn(w);
        }
      }
    }
    *reinterpret_cast<uint4 *>(img + 16 * d) = v;
  }
}

// SiLU of one 32-column accumulator chunk of this thread's lane into row r of
// the activation image (columns c0 .. c0 + 31)
__device__ __forceinline__ void tc_silu_chunk(uint32_t taddr, unsigned char *hs, int r, int c0) {
  float v[32];
  tmem_ld32(taddr, v);
  uint32_t pk[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) pk[j] = silu_h_bf16x2(v[2 * j], v[2 * j + 1]);
  unsigned char *dst = hs + (r / 8) * tc::kSBOH + (r % 8) * 16 + (c0 / 8) * 128;
#pragma unroll
  for (int i = 0; i < 4; ++i)
    *reinterpret_cast<uint4 *>(dst + i * 128) =
        make_uint4(pk[4 * i], pk[4 * i + 1], pk[4 * i + 2], pk[4 * i + 3]);
}

// issue one layer of a slot: D (+)= A B^T over K = 16 steps
__device__ __forceinline__ void tc_issue_layer(int layer, uint32_t tmem_d, uint32_t sX,
                                               uint32_t sH, uint32_t sW0, uint32_t sW1,
                                               uint32_t sW2, uint32_t sW3) {
  constexpr uint32_t id128 = umma_idesc_bf16(128, 128), id16 = umma_idesc_bf16(128, 16);
  if (layer == 0) {  // the bias comes with the input's constant columns
    umma_bf16(tmem_d, umma_sdesc(sX, 128, 256), umma_sdesc(sW0, 128, 256), id128, 0u);
    return;
  }
  const uint32_t sW = layer == 1 ? sW1 : (layer == 2 ? sW2 : sW3);
  const uint32_t id = layer == 3 ? id16 : id128;
#pragma unroll
  for (int kk = 0; kk < tc::kKH / 16; ++kk)  // 8 steps of weights, 1 of bias columns
    umma_bf16(tmem_d, umma_sdesc(sH + 256 * kk, 128, tc::kSBOH),
              umma_sdesc(sW + 256 * kk, 128, tc::kSBOH), id, kk > 0 ? 1u : 0u);
}

__global__ void __maxnreg__(128)
    k_mlp_infer_tc(const bf16 *__restrict__ X, long long n, const bf16 *__restrict__ Wg,
                   const float *__restrict__ P, float *__restrict__ Y, int *err) {
  extern __shared__ __align__(128) unsigned char tc_raw[];
  unsigned char *sm = tc_raw + ((128 - (smem_u32(tc_raw) & 127)) & 127);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const uint32_t full0 = smem_u32(sm + tc::kBar), done0 = full0 + 8 * tc::kSlots;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + tc::kBar + 64);
  volatile int *abort = reinterpret_cast<volatile int *>(sm + tc::kBar + 68);

  // weights with their biases, once per CTA (layers 0..2 times 1/2, see above)
  stage_kmajor_bias(sm + tc::kW0, Wg + kOffW0, P + kOffB0, kMlpHid, kMlpHid, kMlpIn, kMlpIn,
                    kMlpIn - 2, 0.5f);
  stage_kmajor_bias(sm + tc::kW1, Wg + kOffW1, P + kOffB1, kMlpHid, kMlpHid, kMlpHid, tc::kKH,
                    kMlpHid, 0.5f);
  stage_kmajor_bias(sm + tc::kW2, Wg + kOffW2, P + kOffB2, kMlpHid, kMlpHid, kMlpHid, tc::kKH,
                    kMlpHid, 0.5f);
  stage_kmajor_bias(sm + tc::kW3, Wg + kOffW3, P + kOffB3, kMlpOut, 16, kMlpHid, tc::kKH,
                    kMlpHid, 1.f);
  // the constant columns of every slot's activation image: ones in columns
  // 128, 129, zeros in 130..143 (the epilogues write columns 0..127 only)
  for (int d = t; d < tc::kSlots * 128; d += blockDim.x) {
    const int sl = d / 128, r = d - sl * 128;
    unsigned char *row = sm + tc::kHs + sl * 128 * tc::kKH * 2 + (r / 8) * tc::kSBOH + (r % 8) * 16;
    *reinterpret_cast<uint4 *>(row + 16 * 128) = make_uint4(0x3F803F80u, 0u, 0u, 0u);
    *reinterpret_cast<uint4 *>(row + 17 * 128) = make_uint4(0u, 0u, 0u, 0u);
  }
  if (t == 0) {
    for (int sl = 0; sl < tc::kSlots; ++sl) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 128;" ::"r"(full0 + 8 * sl) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(done0 + 8 * sl) : "memory");
    }
    *abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(tc::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tmem_slot;
  const uint32_t sW0 = smem_u32(sm + tc::kW0), sW1 = smem_u32(sm + tc::kW1);
  const uint32_t sW2 = smem_u32(sm + tc::kW2), sW3 = smem_u32(sm + tc::kW3);
  const long long tiles = (n + 127) / 128, stride = (long long)tc::kSlots * gridDim.x;

  if (warp < tc::kMmaWarp) {
    // ---- epilogue of slot s: tiles first, first + stride, ...
    const int s = warp >> 2, q = warp & 3, r = 32 * q + lane;
    const uint32_t tl = tbase + ((uint32_t)(32 * q) << 16) + 128u * s;
    const uint32_t full = full0 + 8 * s, done = done0 + 8 * s;
    unsigned char *xs = sm + tc::kXs + 4096 * s, *hs = sm + tc::kHs + 128 * tc::kKH * 2 * s;
    const long long first = (long long)tc::kSlots * blockIdx.x + s;
    uint32_t j = 0;  // steps (layers) completed: the parity of the next wait
    uint4 xa = make_uint4(0u, 0u, 0u, 0u), xb = xa;
    if (first < tiles && first * 128 + r < n) {
      const uint4 *src = reinterpret_cast<const uint4 *>(X + (first * 128 + r) * kMlpIn);
      xa = src[0];
      xb = src[1];
    }
    bool ok = true;
    for (long long tile = first; tile < tiles && ok; tile += stride) {
      const long long row = tile * 128 + r;
      // layer 0 operand: the input row with ones in the bias columns 14, 15
      unsigned char *xd = xs + (r / 8) * 256 + (r % 8) * 16;
      *reinterpret_cast<uint4 *>(xd) = xa;
      *reinterpret_cast<uint4 *>(xd + 128) = make_uint4(xb.x, xb.y, xb.z, 0x3F803F80u);
      {  // the next tile's rows, loaded while this one runs
        const long long nrow = (tile + stride) * 128 + r;
        xa = make_uint4(0u, 0u, 0u, 0u);
        xb = xa;
        if (tile + stride < tiles && nrow < n) {
          const uint4 *src = reinterpret_cast<const uint4 *>(X + nrow * kMlpIn);
          xa = src[0];
          xb = src[1];
        }
      }
      fence_proxy_async_smem();
      tc_fence_before();
      mbar_arrive(full);
      for (int l = 0; l < 4; ++l) {
        ok = mbar_wait(done, j & 1u, abort);
        ++j;
        tc_fence_after();
        ok = __all_sync(0xffffffffu, ok);  // warp-uniform before the .sync.aligned TMEM ops
        if (!ok) break;
        if (l < 3) {
#pragma unroll 1
          for (int c = 0; c < 4; ++c) tc_silu_chunk(tl + 32 * c, hs, r, 32 * c);
          fence_proxy_async_smem();
          tc_fence_before();
          mbar_arrive(full);
        } else {
          float o[16];
          tmem_ld16(tl, o);
          if (row < n) {
            float4 *yd = reinterpret_cast<float4 *>(Y + row * kMlpOut);
            yd[0] = make_float4(o[0], o[1], o[2], o[3]);
            yd[1] = make_float4(o[4], o[5], o[6], o[7]);
          }
        }
      }
    }
    if (!ok && lane == 0) atomicOr(err, kErrWait);
  } else if (lane == 0) {
    // ---- the MMA issuer: slots round-robin, one layer per visit
    long long nt[tc::kSlots];
    uint32_t js[tc::kSlots];
    for (int sl = 0; sl < tc::kSlots; ++sl) {
      const long long f = (long long)tc::kSlots * blockIdx.x + sl;
      nt[sl] = f < tiles ? (tiles - 1 - f) / stride + 1 : 0;
      js[sl] = 0;
    }
    bool ok = true, any = true;
    while (ok && any) {
      any = false;
      for (int sl = 0; sl < tc::kSlots && ok; ++sl) {
        if ((long long)js[sl] >= 4 * nt[sl]) continue;
        any = true;
        ok = mbar_wait(full0 + 8 * sl, js[sl] & 1u, abort);
        if (!ok) break;
        tc_fence_after();
        tc_issue_layer((int)(js[sl] & 3u), tbase + 128u * sl,
                       smem_u32(sm + tc::kXs + 4096 * sl),
                       smem_u32(sm + tc::kHs + 128 * tc::kKH * 2 * sl),
                       sW0, sW1, sW2, sW3);
        umma_commit(done0 + 8 * sl);
        ++js[sl];
      }
    }
    if (!ok) {
      atomicOr(err, kErrWait);
      // the MMAs already issued (bounded): the last commit of every slot
      for (int sl = 0; sl < tc::kSlots; ++sl)
        if (js[sl] > 0) mbar_wait(done0 + 8 * sl, (js[sl] - 1) & 1u, abort);
    }
  }
  // every MMA has completed (or a wait gave up): free TMEM
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase),
                 "r"(tc::kTmemCols)
                 : "memory");
}

#include "ft_gemm_tc.cuh"

}  // namespace ftgpu

using namespace ftgpu;

// ------------------------------------------------------------------------
struct ftgpu_surrogate {
  int device = 0;
  cudaStream_t stream = nullptr;
  SurrogateLaw law;
  MatP<double> mp;
  float *P = nullptr, *G = nullptr, *Mo = nullptr, *V = nullptr;  // FP32 master, grad, Adam
  bf16 *Wb = nullptr;                                             // BF16 copy (same layout)
  bf16 *X = nullptr;                                              // training inputs [n][16]
  float *T = nullptr;                                             // targets [n][8]
  long long nsamples = 0;
  // activations of one batch
  long long cap = 0;
  float *Z1 = nullptr, *Z2 = nullptr, *Z3 = nullptr, *Y = nullptr, *rowloss = nullptr, *loss = nullptr;
  bf16 *H1 = nullptr, *H2 = nullptr, *H3 = nullptr, *dY = nullptr, *dZ1 = nullptr, *dZ2 = nullptr,
       *dZ3 = nullptr;
  long long adam_t = 0;
  int *derr = nullptr;  // device error word of standalone inference calls
  float *part = nullptr;  // split-K partial tiles of the weight gradients
  long long part_cap = 0;
  int tensor_cores = 1;   // training GEMMs: 1 tcgen05 (k_gemm_tc), 0 mma.sync (k_gemm)
  std::string err;
  ~ftgpu_surrogate() {
    for (void *p : {(void *)P, (void *)G, (void *)Mo, (void *)V, (void *)Wb, (void *)X, (void *)T,
                    (void *)Z1, (void *)Z2, (void *)Z3, (void *)Y, (void *)rowloss, (void *)loss,
                    (void *)H1, (void *)H2, (void *)H3, (void *)dY, (void *)dZ1, (void *)dZ2,
                    (void *)dZ3, (void *)derr, (void *)part})
      if (p) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

// CUDA failures of the surrogate calls: the call and the CUDA error text
// become ftgpu_last_error()
#define SCK(x)                                                                      \
  do {                                                                              \
    const cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) {                                                        \
      cudaGetLastError();                                                           \
      return record_error(FTGPU_ERR_CUDA,                                           \
                          (std::string(#x) + ": " + cudaGetErrorString(e_)).c_str()); \
    }                                                                               \
  } while (0)

template <class T>
int dalloc(T **p, size_t n) {
  if (*p) cudaFree(*p);
  *p = nullptr;
  if (cudaMalloc((void **)p, n * sizeof(T) + 16) != cudaSuccess) {
    cudaGetLastError();
    return FTGPU_ERR_ALLOC;
  }
  return 0;
}

int ensure_batch(ftgpu_surrogate *s, long long B) {
  if (B <= s->cap) return 0;
  int r = 0;
  r |= dalloc(&s->Z1, B * kMlpHid) | dalloc(&s->Z2, B * kMlpHid) | dalloc(&s->Z3, B * kMlpHid);
  r |= dalloc(&s->H1, B * kMlpHid) | dalloc(&s->H2, B * kMlpHid) | dalloc(&s->H3, B * kMlpHid);
  r |= dalloc(&s->dZ1, B * kMlpHid) | dalloc(&s->dZ2, B * kMlpHid) | dalloc(&s->dZ3, B * kMlpHid);
  r |= dalloc(&s->Y, B * kMlpOut) | dalloc(&s->dY, B * kMlpOut) | dalloc(&s->rowloss, B);
  r |= dalloc(&s->loss, 1);
  // split-K partial tiles of the weight gradients: K slices of 256 rows, tiles <= 128 x 128
  const long long pc = ((B + 255) / 256) * 128 * 128;
  if (pc > s->part_cap) {
    r |= dalloc(&s->part, pc);
    s->part_cap = pc;
  }
  if (r) return FTGPU_ERR_ALLOC;
  s->cap = B;
  return 0;
}

// One training GEMM: on the tensor cores (k_gemm_tc: 128-row tiles, weight
// gradients split over K in slices of 256 batch rows and summed in slice
// order), or on the warp-level mma.sync kernel (the cross-check path).
template <int EPI>
int gemm(ftgpu_surrogate *s, cudaStream_t st, const GemmArgs &g) {
  if (!s->tensor_cores) {
    dim3 grid((unsigned)((g.M + 63) / 64), (unsigned)((g.N + 31) / 32));
    k_gemm<EPI><<<grid, 128, 0, st>>>(g);
    return cudaGetLastError() == cudaSuccess ? 0 : FTGPU_ERR_CUDA;
  }
  const int Npad = (g.N + 15) / 16 * 16;
  if (Npad > 128 || g.M <= 0 || g.K <= 0) return FTGPU_ERR_INPUT;
  const int mt = (g.M + 127) / 128;
  int slices = 1, kslice = g.K;
  if (EPI == kEpiStore && mt == 1 && g.K > 512) {
    kslice = 256;
    slices = (g.K + kslice - 1) / kslice;
    if ((long long)slices * g.M * g.N > s->part_cap) return FTGPU_ERR_INPUT;
  }
  k_gemm_tc<EPI><<<dim3((unsigned)mt, (unsigned)slices), tcg::kThreads, tcg::kSmem, st>>>(
      g, Npad, kslice, slices > 1 ? s->part : nullptr, s->derr);
  if (slices > 1) {
    const long long n = (long long)g.M * g.N;
    k_splitk_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(s->part, slices, g.M, g.N, g.C,
                                                                g.scm, g.scn);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : FTGPU_ERR_CUDA;
}

GemmArgs ga(int M, int N, int K, const bf16 *A, long long sam, long long sak, const bf16 *B,
            long long sbk, long long sbn) {
  GemmArgs g;
  memset(&g, 0, sizeof(g));
  g.M = M; g.N = N; g.K = K; g.A = A; g.sam = sam; g.sak = sak; g.B = B; g.sbk = sbk; g.sbn = sbn;
  return g;
}

// forward of B rows of X: Z1/H1, Z2/H2, Z3/H3 and Y
int forward(ftgpu_surrogate *s, const bf16 *X, long long B) {
  const bf16 *W = s->Wb;
  const float *P = s->P;
  GemmArgs g = ga((int)B, kMlpHid, kMlpIn, X, kMlpIn, 1, W + kOffW0, 1, kMlpIn);
  g.bias = P + kOffB0; g.Z = s->Z1; g.H = s->H1;
  int r = gemm<kEpiBiasSilu>(s, s->stream, g);
  g = ga((int)B, kMlpHid, kMlpHid, s->H1, kMlpHid, 1, W + kOffW1, 1, kMlpHid);
  g.bias = P + kOffB1; g.Z = s->Z2; g.H = s->H2;
  r |= gemm<kEpiBiasSilu>(s, s->stream, g);
  g = ga((int)B, kMlpHid, kMlpHid, s->H2, kMlpHid, 1, W + kOffW2, 1, kMlpHid);
  g.bias = P + kOffB2; g.Z = s->Z3; g.H = s->H3;
  r |= gemm<kEpiBiasSilu>(s, s->stream, g);
  g = ga((int)B, kMlpOut, kMlpHid, s->H3, kMlpHid, 1, W + kOffW3, 1, kMlpHid);
  g.bias = P + kOffB3; g.C = s->Y; g.scm = kMlpOut; g.scn = 1;
  r |= gemm<kEpiBias>(s, s->stream, g);
  return r;
}

// loss and all parameter gradients of one batch (X, T) into G
int backward(ftgpu_surrogate *s, const bf16 *X, const float *T, long long B) {
  const bf16 *W = s->Wb;
  float *G = s->G;
  cudaStream_t st = s->stream;
  int r = 0;
  k_mse<<<(unsigned)((B + 255) / 256), 256, 0, st>>>(s->Y, T, B, s->dY, s->rowloss);
  k_sum<<<1, 256, 0, st>>>(s->rowloss, B, s->loss);
  // layer 3: dW3 = dY^T H3, db3, dZ3 = (dY W3) * silu'(Z3)
  GemmArgs g = ga(kMlpOut, kMlpHid, (int)B, s->dY, 1, kMlpOut, s->H3, kMlpHid, 1);
  g.C = G + kOffW3; g.scm = kMlpHid; g.scn = 1;
  r |= gemm<kEpiStore>(s, st, g);
  k_colsum<<<kMlpOut, 256, 0, st>>>(s->dY, B, kMlpOut, G + kOffB3);
  g = ga((int)B, kMlpHid, kMlpOut, s->dY, kMlpOut, 1, W + kOffW3, kMlpHid, 1);
  g.Zp = s->Z3; g.dZ = s->dZ3;
  r |= gemm<kEpiSiluGrad>(s, st, g);
  // layer 2
  g = ga(kMlpHid, kMlpHid, (int)B, s->dZ3, 1, kMlpHid, s->H2, kMlpHid, 1);
  g.C = G + kOffW2; g.scm = kMlpHid; g.scn = 1;
  r |= gemm<kEpiStore>(s, st, g);
  k_colsum<<<kMlpHid, 256, 0, st>>>(s->dZ3, B, kMlpHid, G + kOffB2);
  g = ga((int)B, kMlpHid, kMlpHid, s->dZ3, kMlpHid, 1, W + kOffW2, kMlpHid, 1);
  g.Zp = s->Z2; g.dZ = s->dZ2;
  r |= gemm<kEpiSiluGrad>(s, st, g);
  // layer 1
  g = ga(kMlpHid, kMlpHid, (int)B, s->dZ2, 1, kMlpHid, s->H1, kMlpHid, 1);
  g.C = G + kOffW1; g.scm = kMlpHid; g.scn = 1;
  r |= gemm<kEpiStore>(s, st, g);
  k_colsum<<<kMlpHid, 256, 0, st>>>(s->dZ2, B, kMlpHid, G + kOffB1);
  g = ga((int)B, kMlpHid, kMlpHid, s->dZ2, kMlpHid, 1, W + kOffW1, kMlpHid, 1);
  g.Zp = s->Z1; g.dZ = s->dZ1;
  r |= gemm<kEpiSiluGrad>(s, st, g);
  // layer 0
  g = ga(kMlpHid, kMlpIn, (int)B, s->dZ1, 1, kMlpHid, X, kMlpIn, 1);
  g.C = G + kOffW0; g.scm = kMlpIn; g.scn = 1;
  r |= gemm<kEpiStore>(s, st, g);
  k_colsum<<<kMlpHid, 256, 0, st>>>(s->dZ1, B, kMlpHid, G + kOffB0);
  if (cudaGetLastError() != cudaSuccess) return FTGPU_ERR_CUDA;
  return r;
}

}  // namespace

namespace ftgpu {

// fused inference on the tensor cores (tcgen05, the in-loop path); device
// errors (a wait that gave up) are or-ed into *err
int surrogate_infer(ftgpu_surrogate *s, const uint16_t *X, long long n, float *Y,
                    cudaStream_t st, int *err) {
  static bool attr_set[64] = {false};
  if (n <= 0) return 0;
  if (s->device >= 0 && s->device < 64 && !attr_set[s->device]) {
    const cudaError_t e = cudaFuncSetAttribute(
        k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::kSmem);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return record_error(FTGPU_ERR_CUDA, (std::string("tensor-core inference shared memory: ") +
                                           cudaGetErrorString(e)).c_str());
    }
    attr_set[s->device] = true;
  }
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
  const long long tiles = (n + 127) / 128;
  const long long grid =
      std::max<long long>(1, std::min<long long>((long long)sms, (tiles + tc::kSlots - 1) / tc::kSlots));
  k_mlp_infer_tc<<<(unsigned)grid, tc::kThreads, tc::kSmem, st>>>(reinterpret_cast<const bf16 *>(X), n,
                                                          s->Wb, s->P, Y, err);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return record_error(FTGPU_ERR_CUDA, (std::string("tensor-core inference launch: ") +
                                         cudaGetErrorString(e)).c_str());
  return 0;
}

// the same on the warp-level mma.sync path (kept as a cross-check)
int surrogate_infer_mma(ftgpu_surrogate *s, const uint16_t *X, long long n, float *Y,
                        cudaStream_t st) {
  static bool attr_set[64] = {false};
  if (n <= 0) return 0;
  if (s->device >= 0 && s->device < 64 && !attr_set[s->device]) {
    if (cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kInferSmem) != cudaSuccess)
      return FTGPU_ERR_CUDA;
    attr_set[s->device] = true;
  }
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
  const long long tiles = (n + 15) / 16;
  long long grid = std::min<long long>((long long)sms * 2, (tiles + 7) / 8);
  if (grid < 1) grid = 1;
  k_mlp_infer<<<(unsigned)grid, 256, kInferSmem, st>>>(reinterpret_cast<const bf16 *>(X), n, s->Wb,
                                                       s->P, Y);
  return cudaGetLastError() == cudaSuccess ? 0 : FTGPU_ERR_CUDA;
}

SurrogateLaw surrogate_law(const ftgpu_surrogate *s) { return s->law; }
int surrogate_device(const ftgpu_surrogate *s) { return s->device; }

}  // namespace ftgpu

extern "C" {

int ftgpu_surrogate_create(ftgpu_surrogate **out, int device, const double *props,
                           unsigned long long seed) {
  if (!out || !props) return FTGPU_ERR_INPUT;
  *out = nullptr;
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || device < 0 || device >= nd) {
    cudaGetLastError();
    return FTGPU_ERR_NODEVICE;
  }
  SCK(cudaSetDevice(device));
  auto s = std::make_unique<ftgpu_surrogate>();
  s->device = device;
  SCK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  memset(&s->mp, 0, sizeof(s->mp));
  for (int k = 0; k < 9; ++k) s->mp.p[k] = props[k];
  s->mp.K = props[2] + 2.0 * props[1] / 3.0;
  s->mp.mat = 7;
  s->law.mu = props[1];
  s->law.k1 = props[3];
  s->law.k2 = props[4];
  s->law.kappa = props[7];
  s->law.s0 = props[1] + props[3];
  s->law.out_scale = 1.0;
  s->law.trust_e2 = 0.04;
  int r = dalloc(&s->P, kMlpParams) | dalloc(&s->G, kMlpParams) | dalloc(&s->Mo, kMlpParams) |
          dalloc(&s->V, kMlpParams) | dalloc(&s->Wb, kMlpParams) | dalloc(&s->derr, 1);
  if (r) return FTGPU_ERR_ALLOC;
  // Kaiming-uniform-style init (fan-in scaled), seeded, on the host
  std::vector<float> p(kMlpParams, 0.f);
  auto init = [&](int off, int rows, int cols, int used_cols) {
    const double b = sqrt(6.0 / used_cols) * 0.5;
    for (int i = 0; i < rows; ++i)
      for (int j = 0; j < cols; ++j) {
        const double u = (mix64(seed ^ mix64((uint64_t)(off + i * cols + j))) >> 11) *
                         (1.0 / 9007199254740992.0);
        p[off + i * cols + j] = j < used_cols ? float((2 * u - 1) * b) : 0.f;
      }
  };
  init(kOffW0, kMlpHid, kMlpIn, kMlpUsedIn);
  init(kOffW1, kMlpHid, kMlpHid, kMlpHid);
  init(kOffW2, kMlpHid, kMlpHid, kMlpHid);
  init(kOffW3, kMlpOut, kMlpHid, kMlpHid);
  for (int j = kMlpUsedOut; j < kMlpOut; ++j)
    for (int i = 0; i < kMlpHid; ++i) p[kOffW3 + j * kMlpHid + i] = 0.f;
  SCK(cudaMemcpy(s->P, p.data(), kMlpParams * 4, cudaMemcpyHostToDevice));
  SCK(cudaMemset(s->Mo, 0, kMlpParams * 4));
  SCK(cudaMemset(s->V, 0, kMlpParams * 4));
  k_to_bf16<<<(kMlpParams + 255) / 256, 256, 0, s->stream>>>(s->P, kMlpParams, s->Wb);
  SCK(cudaStreamSynchronize(s->stream));
  *out = s.release();
  return FTGPU_OK;
}

int ftgpu_surrogate_destroy(ftgpu_surrogate *s) {
  if (s) {
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    delete s;
  }
  return FTGPU_OK;
}

int ftgpu_surrogate_generate(ftgpu_surrogate *s, long long n, unsigned long long seed,
                             double stretch_lo, double stretch_hi) {
  if (!s || n <= 0 || !(stretch_lo > 0) || !(stretch_hi > stretch_lo)) return FTGPU_ERR_INPUT;
  SCK(cudaSetDevice(s->device));
  int r = dalloc(&s->X, n * kMlpIn) | dalloc(&s->T, n * kMlpOut);
  if (r) return FTGPU_ERR_ALLOC;
  // targets relative to s0 |E|^2 first, then normalised to unit RMS; the RMS
  // becomes the law's out_scale
  s->law.out_scale = 1.0;
  k_mlp_gen<<<(unsigned)((n + 127) / 128), 128, 0, s->stream>>>(n, seed, stretch_lo, stretch_hi,
                                                                 s->mp, s->law, s->X, s->T);
  SCK(cudaGetLastError());
  constexpr int kParts = 1024;
  double *dss = nullptr;
  if (dalloc(&dss, kParts)) return FTGPU_ERR_ALLOC;
  k_target_sumsq<<<kParts, 256, 0, s->stream>>>(s->T, n, dss);
  std::vector<double> part(kParts);
  SCK(cudaMemcpyAsync(part.data(), dss, kParts * sizeof(double), cudaMemcpyDeviceToHost,
                      s->stream));
  SCK(cudaStreamSynchronize(s->stream));
  cudaFree(dss);
  double ss = 0.0;
  for (double v : part) ss += v;
  const double rms = sqrt(ss / (double(n) * kMlpUsedOut));
  if (!(rms > 0.0) || !std::isfinite(rms)) return FTGPU_ERR_INPUT;
  s->law.out_scale = rms;
  k_scale<<<1024, 256, 0, s->stream>>>(s->T, n * kMlpOut, float(1.0 / rms));
  SCK(cudaGetLastError());
  SCK(cudaStreamSynchronize(s->stream));
  s->nsamples = n;
  return FTGPU_OK;
}

int ftgpu_surrogate_train(ftgpu_surrogate *s, int epochs, int batch, double lr,
                          double *final_loss) {
  if (!s || s->nsamples <= 0 || batch <= 0 || epochs <= 0) return FTGPU_ERR_STATE;
  SCK(cudaSetDevice(s->device));
  int r = ensure_batch(s, batch);
  if (r) return r;
  const long long nb = s->nsamples / batch;
  double last = 0.0;
  const long long total = nb * epochs;
  SCK(cudaMemsetAsync(s->derr, 0, sizeof(int), s->stream));
  for (int ep = 0; ep < epochs; ++ep) {
    double acc = 0.0;
    for (long long b = 0; b < nb; ++b) {
      const bf16 *X = s->X + b * batch * kMlpIn;
      const float *T = s->T + b * batch * kMlpOut;
      r = forward(s, X, batch);
      r |= backward(s, X, T, batch);
      if (r) return r;
      ++s->adam_t;
      // cosine-decayed learning rate over the whole run
      const double frac = double(s->adam_t) / double(total + 1);
      const float lr_t = float(lr * 0.5 * (1.0 + cos(3.141592653589793 * std::min(frac, 1.0))));
      const float b1 = 0.9f, b2 = 0.999f;
      const float c1 = 1.f - powf(b1, (float)s->adam_t), c2 = 1.f - powf(b2, (float)s->adam_t);
      k_adam<<<(kMlpParams + 255) / 256, 256, 0, s->stream>>>(s->P, s->G, s->Mo, s->V, kMlpParams,
                                                              lr_t, b1, b2, 1e-8f, c1, c2, s->Wb);
      if (b == nb - 1) {
        float hl = 0.f;
        SCK(cudaMemcpyAsync(&hl, s->loss, 4, cudaMemcpyDeviceToHost, s->stream));
        SCK(cudaStreamSynchronize(s->stream));
        acc = hl / (double(batch) * kMlpUsedOut);
      }
    }
    last = acc;
  }
  SCK(cudaStreamSynchronize(s->stream));
  int e = 0;
  SCK(cudaMemcpy(&e, s->derr, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) return record_error(FTGPU_ERR_CUDA, "tensor-core training GEMM gave up waiting");
  if (final_loss) *final_loss = last;
  return FTGPU_OK;
}

// training GEMMs on tcgen05 (tensor_cores = 1, the default) or on the
// warp-level mma.sync kernel (0)
int ftgpu_surrogate_gemm_path(ftgpu_surrogate *s, int tensor_cores) {
  if (!s || (tensor_cores != 0 && tensor_cores != 1)) return FTGPU_ERR_INPUT;
  s->tensor_cores = tensor_cores;
  return FTGPU_OK;
}

// raw network outputs for host features x[n][16] (float) -> y[n][8]
int ftgpu_surrogate_forward(ftgpu_surrogate *s, long long n, const float *x, float *y) {
  if (!s || n <= 0 || !x || !y) return FTGPU_ERR_INPUT;
  SCK(cudaSetDevice(s->device));
  int r = ensure_batch(s, n);
  if (r) return r;
  std::vector<bf16> xb(n * kMlpIn);
  for (long long i = 0; i < n * kMlpIn; ++i) xb[i] = __float2bfloat16_rn(x[i]);
  bf16 *dX = nullptr;
  if (dalloc(&dX, n * kMlpIn)) return FTGPU_ERR_ALLOC;
  SCK(cudaMemcpy(dX, xb.data(), n * kMlpIn * 2, cudaMemcpyHostToDevice));
  SCK(cudaMemset(s->derr, 0, sizeof(int)));
  r = forward(s, dX, n);
  SCK(cudaStreamSynchronize(s->stream));
  int e = 0;
  SCK(cudaMemcpy(&e, s->derr, sizeof(int), cudaMemcpyDeviceToHost));
  if (!r && e) r = record_error(FTGPU_ERR_CUDA, "tensor-core training GEMM gave up waiting");
  SCK(cudaMemcpy(y, s->Y, n * kMlpOut * 4, cudaMemcpyDeviceToHost));
  cudaFree(dX);
  return r;
}

// the same outputs through the fused inference kernel of the explicit loop
// (tensor_cores = 1: tcgen05 with TMEM accumulators; 0: warp-level mma.sync)
static int surrogate_infer_host(ftgpu_surrogate *s, long long n, const float *x, float *y,
                                int tensor_cores) {
  if (!s || n <= 0 || !x || !y) return FTGPU_ERR_INPUT;
  SCK(cudaSetDevice(s->device));
  std::vector<bf16> xb(n * kMlpIn);
  for (long long i = 0; i < n * kMlpIn; ++i) xb[i] = __float2bfloat16_rn(x[i]);
  bf16 *dX = nullptr;
  float *dY = nullptr;
  if (dalloc(&dX, n * kMlpIn) || dalloc(&dY, n * kMlpOut)) return FTGPU_ERR_ALLOC;
  SCK(cudaMemcpy(dX, xb.data(), n * kMlpIn * 2, cudaMemcpyHostToDevice));
  SCK(cudaMemset(s->derr, 0, sizeof(int)));
  int r = tensor_cores
              ? surrogate_infer(s, reinterpret_cast<const uint16_t *>(dX), n, dY, s->stream, s->derr)
              : surrogate_infer_mma(s, reinterpret_cast<const uint16_t *>(dX), n, dY, s->stream);
  SCK(cudaStreamSynchronize(s->stream));
  int e = 0;
  SCK(cudaMemcpy(&e, s->derr, sizeof(int), cudaMemcpyDeviceToHost));
  if (!r && e) r = record_error(FTGPU_ERR_CUDA, "tensor-core inference gave up waiting");
  SCK(cudaMemcpy(y, dY, n * kMlpOut * 4, cudaMemcpyDeviceToHost));
  cudaFree(dX);
  cudaFree(dY);
  return r;
}

int ftgpu_surrogate_infer(ftgpu_surrogate *s, long long n, const float *x, float *y) {
  return surrogate_infer_host(s, n, x, y, 1);
}

int ftgpu_surrogate_infer_mma(ftgpu_surrogate *s, long long n, const float *x, float *y) {
  return surrogate_infer_host(s, n, x, y, 0);
}

// loss and parameter gradient of one batch given on the host (gradient checks)
int ftgpu_surrogate_gradient(ftgpu_surrogate *s, long long n, const float *x, const float *t,
                             float *grad, double *loss) {
  if (!s || n <= 0 || !x || !t) return FTGPU_ERR_INPUT;
  SCK(cudaSetDevice(s->device));
  int r = ensure_batch(s, n);
  if (r) return r;
  std::vector<bf16> xb(n * kMlpIn);
  for (long long i = 0; i < n * kMlpIn; ++i) xb[i] = __float2bfloat16_rn(x[i]);
  bf16 *dX = nullptr;
  float *dT = nullptr;
  if (dalloc(&dX, n * kMlpIn) || dalloc(&dT, n * kMlpOut)) return FTGPU_ERR_ALLOC;
  SCK(cudaMemcpy(dX, xb.data(), n * kMlpIn * 2, cudaMemcpyHostToDevice));
  SCK(cudaMemcpy(dT, t, n * kMlpOut * 4, cudaMemcpyHostToDevice));
  SCK(cudaMemset(s->derr, 0, sizeof(int)));
  r = forward(s, dX, n);
  r |= backward(s, dX, dT, n);
  SCK(cudaStreamSynchronize(s->stream));
  int e = 0;
  SCK(cudaMemcpy(&e, s->derr, sizeof(int), cudaMemcpyDeviceToHost));
  if (!r && e) r = record_error(FTGPU_ERR_CUDA, "tensor-core training GEMM gave up waiting");
  float hl = 0.f;
  SCK(cudaMemcpy(&hl, s->loss, 4, cudaMemcpyDeviceToHost));
  if (loss) *loss = hl / (double(n) * kMlpUsedOut);
  if (grad) SCK(cudaMemcpy(grad, s->G, kMlpParams * 4, cudaMemcpyDeviceToHost));
  cudaFree(dX);
  cudaFree(dT);
  return r;
}

int ftgpu_surrogate_params(ftgpu_surrogate *s, float *get, const float *set) {
  if (!s) return FTGPU_ERR_INPUT;
  SCK(cudaSetDevice(s->device));
  if (set) {
    SCK(cudaMemcpy(s->P, set, kMlpParams * 4, cudaMemcpyHostToDevice));
    k_to_bf16<<<(kMlpParams + 255) / 256, 256, 0, s->stream>>>(s->P, kMlpParams, s->Wb);
    SCK(cudaStreamSynchronize(s->stream));
  }
  if (get) SCK(cudaMemcpy(get, s->P, kMlpParams * 4, cudaMemcpyDeviceToHost));
  return FTGPU_OK;
}

// training samples back to the host (first n): x[n][16] as float, t[n][8]
int ftgpu_surrogate_samples(ftgpu_surrogate *s, long long n, float *x, float *t) {
  if (!s || n <= 0 || n > s->nsamples) return FTGPU_ERR_INPUT;
  std::vector<bf16> xb(n * kMlpIn);
  SCK(cudaMemcpy(xb.data(), s->X, n * kMlpIn * 2, cudaMemcpyDeviceToHost));
  if (x)
    for (long long i = 0; i < n * kMlpIn; ++i) x[i] = __bfloat162float(xb[i]);
  if (t) SCK(cudaMemcpy(t, s->T, n * kMlpOut * 4, cudaMemcpyDeviceToHost));
  return FTGPU_OK;
}

int ftgpu_surrogate_num_params(void) { return kMlpParams; }

int ftgpu_surrogate_output_scale(ftgpu_surrogate *s, double *out_scale) {
  if (!s || !out_scale) return FTGPU_ERR_INPUT;
  *out_scale = s->law.out_scale;
  return FTGPU_OK;
}

// isochoric PK2 (Voigt) predicted for Green strains E[n][6] (tensor shears) and
// fibres a0[n][3]: the element kernel's features, fused inference, S_lin +
// scale * NN, all on the device
int ftgpu_surrogate_predict(ftgpu_surrogate *s, long long n, const double *E, const double *a0,
                            double *S) {
  if (!s || n <= 0 || !E || !a0 || !S) return FTGPU_ERR_INPUT;
  SCK(cudaSetDevice(s->device));
  double *dE = nullptr, *dA = nullptr, *dS = nullptr, *dsc = nullptr;
  bf16 *dX = nullptr;
  float *dY = nullptr;
  int r = dalloc(&dE, 6 * n) | dalloc(&dA, 3 * n) | dalloc(&dS, 6 * n) | dalloc(&dsc, n) |
          dalloc(&dX, n * kMlpIn) | dalloc(&dY, n * kMlpOut);
  if (!r) {
    SCK(cudaMemcpy(dE, E, 6 * n * sizeof(double), cudaMemcpyHostToDevice));
    SCK(cudaMemcpy(dA, a0, 3 * n * sizeof(double), cudaMemcpyHostToDevice));
    const unsigned g = (unsigned)((n + 127) / 128);
    k_predict_features<<<g, 128, 0, s->stream>>>(n, dE, dA, s->law, dX, dS, dsc);
    SCK(cudaMemset(s->derr, 0, sizeof(int)));
    r = surrogate_infer(s, reinterpret_cast<const uint16_t *>(dX), n, dY, s->stream, s->derr);
    k_predict_combine<<<g, 128, 0, s->stream>>>(n, dY, dS, dsc);
    SCK(cudaStreamSynchronize(s->stream));
    SCK(cudaMemcpy(S, dS, 6 * n * sizeof(double), cudaMemcpyDeviceToHost));
  } else {
    r = FTGPU_ERR_ALLOC;
  }
  cudaFree(dE);
  cudaFree(dA);
  cudaFree(dS);
  cudaFree(dsc);
  cudaFree(dX);
  cudaFree(dY);
  return r;
}

}  // extern "C"
