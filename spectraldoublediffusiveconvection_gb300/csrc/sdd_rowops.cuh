// Row operations shared by the nonlinear-term, transform and diagnostics kernels: parity suffix sums
// along a row of modes, and exact power-of-two balancing of rows that share one complex FFT.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sdd {

// S[m] = sum_{m' >= m, m' = m mod 2} v[m'] for m < M.  Called by every thread of the block; returns after a
// barrier (S and the block's shared totals are then free to reuse), the caller syncs before reading S.
// Each parity's values go in chunks of 32 (one warp-wide suffix scan per chunk, all chunks of both parities
// at once over the block's warps); chunk c then adds the carried total of the chunks above it,
// carry_c = T_{c+1} + (T_{c+2} + (... + T_last)), the association of a sequential carry from the top chunk
// down, so the sums are those of one warp scanning the chunks one after another.
constexpr int kSuffixChunks = 64;   // per parity: M <= 4096
template <typename T>
__device__ void parity_suffix(const T* v, T* S, int M) {
  __shared__ T tot[2][kSuffixChunks];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int cnt0 = (M + 1) / 2, cnt1 = M / 2;
  const int nc0 = (cnt0 + 31) / 32, nc1 = (cnt1 + 31) / 32;
  for (int item = warp; item < nc0 + nc1; item += nw) {
    const int p = item < nc0 ? 0 : 1;
    const int c = item - (p ? nc0 : 0);
    const int cnt = p ? cnt1 : cnt0;
    const int t = c * 32 + lane;
    T x = (t < cnt) ? v[p + 2 * t] : (T)0;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      T y = __shfl_down_sync(0xffffffffu, x, off);
      if (lane + off < 32) x += y;
    }
    if (t < cnt) S[p + 2 * t] = x;
    if (lane == 0) tot[p][c] = x;
  }
  __syncthreads();
  for (int item = warp; item < nc0 + nc1; item += nw) {
    const int p = item < nc0 ? 0 : 1;
    const int c = item - (p ? nc0 : 0);
    const int cnt = p ? cnt1 : cnt0, nc = p ? nc1 : nc0;
    T carry = (T)0;
    for (int cc = nc - 1; cc > c; --cc) carry = tot[p][cc] + carry;
    const int t = c * 32 + lane;
    if (t < cnt) S[p + 2 * t] = S[p + 2 * t] + carry;
  }
  __syncthreads();
}

// Exact power-of-two balancing of the rows that share one complex FFT.  The two rows of a pair ride in
// the real and imaginary parts, and the FFT's rounding error scales with the larger of the two: an
// unbalanced pair (|komega| ~ 1e3 next to |JT_psi| ~ 1e-2) would leave the small row with an error of
// eps*1e3.  Each row is therefore scaled by 2^-e, e = exponent of its max |value| (exact), before the
// transform and scaled back after it.  The maxima are taken on the IEEE bit patterns (for non-negative
// values the unsigned order is the numeric order), i.e. with integer instructions: on GB300 the FP64
// pipe is the scarce resource of these kernels.
template <typename T> struct Bits;
template <> struct Bits<double> {
  using U = unsigned long long;
  static __device__ __forceinline__ U absbits(double x) { return (U)__double_as_longlong(x) & 0x7fffffffffffffffull; }
  static __device__ __forceinline__ double val(U u) { return __longlong_as_double((long long)u); }
};
template <> struct Bits<float> {
  using U = unsigned int;
  static __device__ __forceinline__ U absbits(float x) { return __float_as_uint(x) & 0x7fffffffu; }
  static __device__ __forceinline__ float val(U u) { return __uint_as_float(u); }
};

template <typename T>
__device__ __forceinline__ void pow2_scale(T mx, T* s, T* inv) {
  if (!(mx > (T)0) || !isfinite(mx)) {
    *s = (T)1;
    *inv = (T)1;
    return;
  }
  int e;
  frexp(mx, &e);
  *s = ldexp((T)1, -e);
  *inv = ldexp((T)1, e);
}

// Block-wide max of K per-thread |value| bit patterns; writes the scale and inverse scale of each into
// sc[0..K), sc[K..2K).  red must hold K*32 words of U.  Ends with __syncthreads().
template <typename T, int K>
__device__ __forceinline__ void block_max_scales(typename Bits<T>::U (&v)[K], typename Bits<T>::U* red, T* sc) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int t = 0; t < K; ++t) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const typename Bits<T>::U o = __shfl_xor_sync(0xffffffffu, v[t], off);
      v[t] = o > v[t] ? o : v[t];
    }
    if (lane == 0) red[t * 32 + warp] = v[t];
  }
  __syncthreads();
  if (threadIdx.x < K) {
    typename Bits<T>::U m = 0;
    for (int w = 0; w < nw; ++w) m = red[threadIdx.x * 32 + w] > m ? red[threadIdx.x * 32 + w] : m;
    pow2_scale(Bits<T>::val(m), sc + threadIdx.x, sc + K + threadIdx.x);
  }
  __syncthreads();
}

}  // namespace sdd
