// Shared-memory FFT building blocks for the theta transforms.
//
// The reference's transforms (Transforms.py:73-129) are scipy DCT-II/III and DST-II/III on the
// midpoint grid theta_i = pi(2i+1)/(2P).  Here every one of them is reduced to
//   DCT3:  f_i = sum_{k<P} x_k cos(k theta_i)            (inverse direction)
//   DCT2:  y_k = sum_{i<P} f_i cos(k theta_i)            (forward direction)
// and both are evaluated for two real rows at once with one complex FFT of length P (Makhoul's
// even/odd reordering; the pair rides in the real and imaginary parts):
//   DCT3: W_k = V_A(k) + i V_B(k),  V(k) = 0.5 e^{i pi k/2P} (x_k - i x_{P-k}) (k>=1), V(0) = x_0,
//         v = IDFT(W) (unnormalised),  f_{2n} = v_n,  f_{2n+1} = v_{P-1-n}  (A = Re, B = Im)
//   DCT2: z_n = f_A[src(n)] + i f_B[src(n)],  Z = DFT(z),
//         y_A[k] = c (Z_k + Z_{-k})_re/2 + s (Z_k - Z_{-k})_im/2,
//         y_B[k] = c (Z_k + Z_{-k})_im/2 - s (Z_k - Z_{-k})_re/2,   (c, s) = (cos, sin)(pi k/2P).
// The DCT twiddle table holds 0.5 (cos, sin)(pi k/2P), the factor 1/2 of both formulas folded in.
// Sine transforms use sin(w theta_i) = (-1)^i cos((P-w) theta_i).
// The complex FFT is a Stockham autosort FFT (natural order in and out) with radix-2/3/4/5/7 passes,
// ping-ponging between two shared-memory buffers; twiddles come from a table exp(-2 pi i k/L) built on
// the host.
#pragma once
#include <cuda_runtime.h>
#include "sdd_internal.cuh"

namespace sdd {

template <typename T> struct Cplx;
template <> struct Cplx<double> { using type = double2; };
template <> struct Cplx<float> { using type = float2; };

template <typename C> __device__ __forceinline__ C cmk(decltype(C::x) a, decltype(C::x) b) {
  C r; r.x = a; r.y = b; return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return cmk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return cmk<C>(a.x - b.x, a.y - b.y); }
// Every multiply-add is an explicit fma (the translation units that include this file are compiled
// without automatic contraction), so the rounding of a transform does not depend on the kernel it is
// inlined into.
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  return cmk<C>(fma(a.x, b.x, -(a.y * b.y)), fma(a.x, b.y, a.y * b.x));
}
// multiply by -i (forward) or +i (inverse)
template <typename C, bool INV> __device__ __forceinline__ C cmul_mi(C a) {
  return INV ? cmk<C>(-a.y, a.x) : cmk<C>(a.y, -a.x);
}

template <typename T, bool INV>
__device__ __forceinline__ typename Cplx<T>::type tw_at(const typename Cplx<T>::type* w, int idx) {
  typename Cplx<T>::type t = w[idx];
  if (INV) t.y = -t.y;
  return t;
}

// In-register radix-R DFT of v[0..R-1] (R a compile-time constant); w is the length-L twiddle table.
template <typename T, bool INV, int R>
__device__ __forceinline__ void butterfly(typename Cplx<T>::type (&v)[R], const typename Cplx<T>::type* w, int L) {
  using C = typename Cplx<T>::type;
  if constexpr (R == 2) {
    C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if constexpr (R == 4) {
    C t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    C t2 = cadd(v[1], v[3]), t3 = cmul_mi<C, INV>(csub(v[1], v[3]));
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  } else if constexpr (R == 3) {
    const T h = (T)0.86602540378443864676;  // sqrt(3)/2
    C s = cadd(v[1], v[2]);
    C d = csub(v[1], v[2]);
    C t = cmk<C>(fma((T)-0.5, s.x, v[0].x), fma((T)-0.5, s.y, v[0].y));
    C u = cmul_mi<C, INV>(d);  // -i d forward
    v[0] = cadd(v[0], s);
    v[1] = cmk<C>(fma(h, u.x, t.x), fma(h, u.y, t.y));
    v[2] = cmk<C>(fma(-h, u.x, t.x), fma(-h, u.y, t.y));
  } else {  // small prime radix (5, 7): direct DFT with roots of unity from the table
    C o[R];
    const int step = L / R;
#pragma unroll
    for (int q = 0; q < R; ++q) {
      C acc = v[0];
#pragma unroll
      for (int r = 1; r < R; ++r) acc = cadd(acc, cmul(v[r], tw_at<T, INV>(w, ((q * r) % R) * step)));
      o[q] = acc;
    }
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = o[q];
  }
}

// One Stockham pass of radix R over nf FFTs of length L stored back to back (stride L); fnb, fns divide by
// nb = L / R and by Ns, tws = L / (Ns R) (precomputed per stage).
template <typename T, bool INV, int R>
__device__ __forceinline__ void fft_pass_r(const typename Cplx<T>::type* __restrict__ in,
                                           typename Cplx<T>::type* __restrict__ out, int L, int nf, int Ns,
                                           const typename Cplx<T>::type* w, FastDiv fnb, FastDiv fns, int tws) {
  using C = typename Cplx<T>::type;
  const int nb = L / R;
  const int total = nf * nb;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int f = (int)fast_div((unsigned)t, fnb);
    const int j = t - f * nb;
    const C* src = in + f * L;
    C* dst = out + f * L;
    const int jq = (int)fast_div((unsigned)j, fns);
    const int k = j - jq * Ns;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = src[j + r * nb];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], tw_at<T, INV>(w, k * r * tws));
    }
    butterfly<T, INV, R>(v, w, L);
    const int idxD = jq * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) dst[idxD + r * Ns] = v[r];
  }
}

template <typename T, bool INV>
__device__ __forceinline__ void fft_pass(const typename Cplx<T>::type* __restrict__ in,
                                         typename Cplx<T>::type* __restrict__ out, int L, int nf, int R, int Ns,
                                         const typename Cplx<T>::type* w, FastDiv fnb, FastDiv fns, int tws) {
  switch (R) {
    case 4: fft_pass_r<T, INV, 4>(in, out, L, nf, Ns, w, fnb, fns, tws); break;
    case 2: fft_pass_r<T, INV, 2>(in, out, L, nf, Ns, w, fnb, fns, tws); break;
    case 3: fft_pass_r<T, INV, 3>(in, out, L, nf, Ns, w, fnb, fns, tws); break;
    case 5: fft_pass_r<T, INV, 5>(in, out, L, nf, Ns, w, fnb, fns, tws); break;
    default: fft_pass_r<T, INV, 7>(in, out, L, nf, Ns, w, fnb, fns, tws); break;
  }
}

// Full FFT of nf rows in buffer a (b is scratch of the same size).  Returns the buffer holding the
// result.  Must be called by all threads of the block; ends with a __syncthreads().
template <typename T, bool INV>
__device__ typename Cplx<T>::type* fft_rows(typename Cplx<T>::type* a, typename Cplx<T>::type* b, int nf,
                                            const StageArgs& st, const typename Cplx<T>::type* w) {
  using C = typename Cplx<T>::type;
  C* in = a;
  C* out = b;
  int Ns = 1;
  for (int s = 0; s < st.nst; ++s) {
    const int R = st.rad[s];
    fft_pass<T, INV>(in, out, st.L, nf, R, Ns, w, st.nb[s], st.ns[s], st.tws[s]);
    __syncthreads();
    Ns *= R;
    C* tmp = in; in = out; out = tmp;
  }
  return in;
}

// Makhoul source index of reordered slot n (forward direction): v_n = f_{src(n)}.
__device__ __forceinline__ int makhoul_src(int n, int P) {
  return (n < (P + 1) / 2) ? 2 * n : 2 * (P - 1 - n) + 1;
}

}  // namespace sdd
