// ft_injury.cuh -- per-step injury criteria of the brain drivers on the GPU
// (examples/ex5/ex5.cpp:1311-1430, CalculateInjuryCriterions): principal
// strains of the listed elements, running extremes, sticky threshold flags and
// the largest 95th percentiles of MPS and of MPS x strain rate, by an exact
// radix selection.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "ft_common.h"

namespace ftgpu {

// running state (FP64 values; element ids are the reference's)
struct InjuryState {
  double max_strain, max_strain_time, min_strain, min_strain_time;
  double max_shear, max_shear_time, max_psxsr, max_psxsr_time;
  int max_strain_elem, min_strain_elem, max_shear_elem, max_psxsr_elem;
  double mps95, mps95_time, mpsxsr95, mpsxsr95_time;
  int mps95_count, mpsxsr95_count;
  long long steps;
};

// flags per injury element (bits)
enum { kInjMps15 = 1, kInjMps30 = 2, kInjPsr120 = 4, kInjPsxsr28 = 8, kInjInMps95 = 16,
       kInjInMpsxsr95 = 32 };

// per-block partial extremes of one step: value, the caller's list position
// (tie-break) and the compact index of the element
struct InjuryPart {
  double v[4];  // max strain, min strain, max shear, max psxsr
  int j[4];     // list position
  int c[4];     // compact index
};

constexpr int kInjThreads = 256;
constexpr int kRadixBins = 256;

// The listed elements are kept in group order ("compact" index c): element e
// (group order) is listed when cidx[e] >= 0; upos[c] is its position in the
// caller's list (ties go to the smaller position, as in the reference's loop)
// and eref[c] its reference id.
template <class R>
struct InjuryArgs {
  const int *cidx;       // [E] compact index or -1
  const int *upos;       // [n]
  const int *eref;       // [n]
  R *ps_old, *psxsr;     // [n] compact order
  uint8_t *flags;        // [n] compact order
  InjuryPart *part;      // [patches] block extremes of the step
  InjuryPart *part2;     // [reduction blocks] second level
  unsigned *done_blocks; // finished reduction blocks (reset by the last one)
  InjuryState *state;
  const Clock *clock;    // clock[0] of the step (single instance)
  unsigned *hist;        // [2 selections][passes][256], then [2] counters
  unsigned *count;       // [2] elements at or above a new maximum
  int n, parity, npart;
};

// principal strains of the symmetric strain in the trigonometric form of
// CalculateStrain.cpp:38-74
template <class T>
__device__ __forceinline__ void principal_strains(T xx, T yy, T zz, T yz, T xz, T xy, T &mx,
                                                  T &mn, T &sh) {
  const T a = xx, b = xy, c = xz, d = yy, e = yz, f = zz;
  const T p1 = b * b + c * c + e * e;
  T e1, e2, e3;
  if (p1 == T(0)) {
    e1 = a;
    e2 = d;
    e3 = f;
  } else {
    T I1 = a + d + f;
    const T I2 = a * (d + f) + d * f - b * b - c * c - e * e;
    const T I3 = a * d * f + T(2) * b * c * e - b * b * f - c * c * d - e * e * a;
    const T Q = (T(3) * I2 - I1 * I1) / T(9);
    const T Rr = (T(2) * I1 * I1 * I1 - T(9) * I1 * I2 + T(27) * I3) / T(54);
    const T theta = acos(Rr / sqrt(-Q * Q * Q));
    const T sq = T(2) * sqrt(-Q);
    const T kPi = T(3.141592653589793);
    I1 = I1 / T(3);
    e1 = sq * cos(theta / T(3)) + I1;
    e2 = sq * cos((theta + T(2) * kPi) / T(3)) + I1;
    e3 = sq * cos((theta + T(4) * kPi) / T(3)) + I1;
  }
  const T hi = fmax(e3, fmax(e2, e1)), lo = fmin(e3, fmin(e2, e1));
  sh = T(0.5) * (hi - lo);
  mx = hi > T(0) ? hi : T(0);
  mn = lo < T(0) ? lo : T(0);
}

// order-preserving unsigned keys of floating-point values
__device__ __forceinline__ uint32_t fkey(float x) {
  const uint32_t b = __float_as_uint(x);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}
__device__ __forceinline__ uint64_t fkey(double x) {
  const uint64_t b = (uint64_t)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double fkey_inv(uint64_t k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

// better (value, list index) of two candidates for extreme k (k = 1 is a
// minimum): the better value, then the smaller list index
template <class V>
__device__ __forceinline__ bool inj_better(int k, V bv, int bj, V av, int aj) {
  return (k == 1) ? (bv < av || (bv == av && bj < aj)) : (bv > av || (bv == av && bj < aj));
}

// Best of each extreme over a range of partials, then over the threads of a
// block (fixed tree); the result in slot 0 of the shared arrays.
__device__ __forceinline__ void inj_block_best(const InjuryPart *part, int lo, int hi,
                                               double (*sv)[256], int (*sj)[256],
                                               int (*sc)[256]) {
  double v[4] = {-1e300, 1e300, -1e300, -1e300};
  int jj[4] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff}, cc[4] = {-1, -1, -1, -1};
  for (int b = lo + threadIdx.x; b < hi; b += blockDim.x) {
    const InjuryPart p = part[b];
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (inj_better(k, p.v[k], p.j[k], v[k], jj[k])) {
        v[k] = p.v[k];
        jj[k] = p.j[k];
        cc[k] = p.c[k];
      }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    sv[k][threadIdx.x] = v[k];
    sj[k][threadIdx.x] = jj[k];
    sc[k][threadIdx.x] = cc[k];
  }
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h)
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (inj_better(k, sv[k][threadIdx.x + h], sj[k][threadIdx.x + h], sv[k][threadIdx.x],
                       sj[k][threadIdx.x])) {
          sv[k][threadIdx.x] = sv[k][threadIdx.x + h];
          sj[k][threadIdx.x] = sj[k][threadIdx.x + h];
          sc[k][threadIdx.x] = sc[k][threadIdx.x + h];
        }
    __syncthreads();
  }
}

constexpr int kInjReduceSpan = 256;  // partials per reduction block

// The step's extremes from the per-patch partials into the running state: each
// block reduces kInjReduceSpan partials into part2[block]; the last block to
// finish (counter in count[2]) reduces those in block order and updates the
// state: a strictly better value takes the element and the time (the
// reference's ordered loop with strict comparisons).  The last block also
// clears the radix histograms and counters of the step.
template <class R>
__global__ void __launch_bounds__(256) k_injury_reduce(const InjuryArgs<R> A) {
  __shared__ double sv[4][256];
  __shared__ int sj[4][256], sc[4][256];
  __shared__ bool last;
  const int lo = blockIdx.x * kInjReduceSpan, hi = min(lo + kInjReduceSpan, A.npart);
  inj_block_best(A.part, lo, hi, sv, sj, sc);
  if (threadIdx.x == 0) {
    InjuryPart q;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      q.v[k] = sv[k][0];
      q.j[k] = sj[k][0];
      q.c[k] = sc[k][0];
    }
    A.part2[blockIdx.x] = q;
    __threadfence();
    last = atomicAdd(A.done_blocks, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  inj_block_best(A.part2, 0, gridDim.x, sv, sj, sc);
  for (int i = threadIdx.x; i < 2 * 8 * kRadixBins + 2; i += blockDim.x) A.hist[i] = 0;
  if (threadIdx.x != 0) return;
  *A.done_blocks = 0;
  const Clock ck = A.clock[A.parity];
  if (ck.done) return;
  const double t = ck.time + ck.dt;
  InjuryState s = *A.state;
  double *val[4] = {&s.max_strain, &s.min_strain, &s.max_shear, &s.max_psxsr};
  double *tim[4] = {&s.max_strain_time, &s.min_strain_time, &s.max_shear_time,
                    &s.max_psxsr_time};
  int *el[4] = {&s.max_strain_elem, &s.min_strain_elem, &s.max_shear_elem, &s.max_psxsr_elem};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int c = sc[k][0];
    if (c < 0) continue;
    const bool upd = (k == 1) ? (*val[k] > sv[k][0]) : (*val[k] < sv[k][0]);
    if (upd) {
      *val[k] = sv[k][0];
      *el[k] = A.eref[c];
      *tim[k] = t;
    }
  }
  ++s.steps;
  *A.state = s;
}

// Radix selection of the value of rank k = (int)(0.95 n) - 1 (rank 0 if
// negative) of sel = 0: ps_old, 1: psxsr, 8 bits per pass from the most
// significant byte.  Every pass first recovers the digits fixed so far from
// the histograms of the previous passes (the same in every block).
// The digits fixed by the first `pass` histograms of a selection, recovered
// by every block (blockDim.x == kRadixBins: thread t owns bin t): per pass a
// block-wide scan of the 256 counts finds the bin holding the remaining rank
// (the first bin whose cumulative count exceeds it).  The result is in
// *prefix after the final barrier; `stage` is unused scratch kept for the
// callers' layout.
template <class K>
__device__ __forceinline__ void block_radix_prefix(const unsigned *hist, int pass, int n,
                                                   unsigned *stage, K *prefix) {
  (void)stage;
  constexpr int KB = sizeof(K) * 8;
  __shared__ unsigned wsum[kRadixBins / 32];
  __shared__ unsigned s_krem, s_below;
  __shared__ int s_d;
  __shared__ K s_pref;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  if (t == 0) {
    int k = (int)(n * 0.95) - 1;
    if (k < 0) k = 0;
    s_krem = (unsigned)k;
    s_pref = 0;
  }
  for (int q = 0; q < pass; ++q) {
    const unsigned c = hist[q * kRadixBins + t];
    unsigned x = c;  // inclusive scan within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    if (t == 0) {
      s_d = 0;
      s_below = 0;
    }
    __syncthreads();
    unsigned off = 0;
#pragma unroll
    for (int v = 0; v < kRadixBins / 32; ++v) off += v < w ? wsum[v] : 0u;
    const unsigned incl = x + off, excl = incl - c, krem = s_krem;
    if (excl <= krem && krem < incl) {
      s_d = t;
      s_below = excl;
    }
    __syncthreads();
    if (t == 0) {
      s_krem = krem - s_below;
      s_pref |= (K)s_d << (KB - 8 * (q + 1));
    }
    __syncthreads();
  }
  if (t == 0) *prefix = s_pref;
  __syncthreads();
}

// Histogram of the next digit of the keys that share the digits fixed so far.
// The values cluster (strains of one tissue), so most keys fall into a few
// bins: lanes of a warp with the same bin are merged (__match_any_sync) and one
// of them adds the count to its warp's own sub-histogram.
template <class R>
__global__ void __launch_bounds__(kInjThreads) k_radix_hist(const InjuryArgs<R> A, int pass) {
  const int sel = blockIdx.y;  // 0: MPS, 1: MPS x rate
  typedef typename std::conditional<sizeof(R) == 8, uint64_t, uint32_t>::type K;
  constexpr int KB = sizeof(K) * 8;
  constexpr int kWarps = kInjThreads / 32;
  if (A.clock[A.parity].done) return;
  unsigned *hist = A.hist + (sel * (KB / 8)) * kRadixBins;
  __shared__ unsigned sh[kWarps][kRadixBins];
  __shared__ unsigned stage[(KB / 8) * kRadixBins];
  __shared__ K s_prefix;
  for (int i = threadIdx.x; i < kWarps * kRadixBins; i += blockDim.x) (&sh[0][0])[i] = 0;
  block_radix_prefix<K>(hist, pass, A.n, stage, &s_prefix);  // digits fixed so far
  const K prefix = s_prefix;
  const R *val = sel == 0 ? A.ps_old : A.psxsr;
  const K mask = pass == 0 ? K(0) : (K)(~K(0)) << (KB - 8 * pass);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // the same trip count for every lane of a warp (for __match_any_sync)
  for (long long base = (long long)blockIdx.x * blockDim.x; base < A.n;
       base += (long long)gridDim.x * blockDim.x) {
    const long long j = base + threadIdx.x;
    unsigned bin = 0xffffffffu;
    if (j < A.n) {
      const K key = fkey(val[j]);
      if ((key & mask) == prefix) bin = (unsigned)(key >> (KB - 8 * (pass + 1))) & 0xffu;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, bin);
    if (bin != 0xffffffffu && lane == __ffs(peers) - 1) atomicAdd(&sh[warp][bin], __popc(peers));
  }
  __syncthreads();
  unsigned *out = hist + pass * kRadixBins;
  for (int i = threadIdx.x; i < kRadixBins; i += blockDim.x) {
    unsigned c = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) c += sh[w][i];
    if (c) atomicAdd(&out[i], c);
  }
}

// The selected values; where one beats its running maximum, the listed
// elements at or above it are marked (flag bit) and counted.  Both selections
// in one pass per element, so each flag byte is written by one thread.
template <class R>
__global__ void __launch_bounds__(kInjThreads) k_radix_list(const InjuryArgs<R> A) {
  typedef typename std::conditional<sizeof(R) == 8, uint64_t, uint32_t>::type K;
  constexpr int KB = sizeof(K) * 8;
  if (A.clock[A.parity].done) return;
  __shared__ unsigned stage[(KB / 8) * kRadixBins];
  __shared__ K s_prefix[2];
  for (int sel = 0; sel < 2; ++sel)
    block_radix_prefix<K>(A.hist + (sel * (KB / 8)) * kRadixBins, KB / 8, A.n, stage,
                          &s_prefix[sel]);
  const R v0 = fkey_inv(s_prefix[0]), v1 = fkey_inv(s_prefix[1]);
  const bool up0 = double(v0) > A.state->mps95, up1 = double(v1) > A.state->mpsxsr95;
  if (!up0 && !up1) return;
  unsigned c0 = 0, c1 = 0;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < A.n; j += gridDim.x * blockDim.x) {
    uint8_t f = A.flags[j];
    if (up0) {
      const bool in = A.ps_old[j] >= v0;
      f = in ? (f | kInjInMps95) : (f & (uint8_t)~kInjInMps95);
      c0 += in;
    }
    if (up1) {
      const bool in = A.psxsr[j] >= v1;
      f = in ? (f | kInjInMpsxsr95) : (f & (uint8_t)~kInjInMpsxsr95);
      c1 += in;
    }
    A.flags[j] = f;
  }
  if (c0) atomicAdd(&A.count[0], c0);
  if (c1) atomicAdd(&A.count[1], c1);
}

// Running maxima of the two percentiles (after k_radix_list of both).
template <class R>
__global__ void __launch_bounds__(kRadixBins) k_radix_final(const InjuryArgs<R> A) {
  typedef typename std::conditional<sizeof(R) == 8, uint64_t, uint32_t>::type K;
  constexpr int KB = sizeof(K) * 8;
  const Clock ck = A.clock[A.parity];
  if (ck.done) return;
  __shared__ unsigned stage[(KB / 8) * kRadixBins];
  __shared__ K s_prefix[2];
  for (int sel = 0; sel < 2; ++sel)
    block_radix_prefix<K>(A.hist + (sel * (KB / 8)) * kRadixBins, KB / 8, A.n, stage,
                          &s_prefix[sel]);
  if (threadIdx.x != 0) return;
  const double t = ck.time + ck.dt;
  InjuryState s = *A.state;
  for (int sel = 0; sel < 2; ++sel) {
    const double v = double(fkey_inv(s_prefix[sel]));
    double &mx = sel == 0 ? s.mps95 : s.mpsxsr95;
    if (v > mx) {
      mx = v;
      (sel == 0 ? s.mps95_time : s.mpsxsr95_time) = t;
      (sel == 0 ? s.mps95_count : s.mpsxsr95_count) = (int)A.count[sel];
    }
  }
  *A.state = s;
}

}  // namespace ftgpu
