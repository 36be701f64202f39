// Row kernels of the nonlinear term, the right-hand-side assembly, the theta recurrences and the
// standalone theta transforms.
//
// k_fx_rows: one CTA per (radial row n, shell).  It forms the nine spectral rows of
// Matrix_Operators.py:631-740 (Derivatives, with J_theta_RT :437 and A2_SINE_R2 :476 evaluated as
// parity suffix sums along the row), transforms them to the 3/2-padded grid (:776-786), forms the
// products of :791-793 (NLIN_FX) or :884-887 (NLIN_DFX), and transforms four product rows back
// (:797-802).  The radial derivative Dr@(JT_psi*omega) of :791 is moved through the (theta-only) DST:
// the kernel outputs DST(JT_psi*omega) and the rhs kernel applies Dr to it in spectral space, so the
// row kernel has no cross-row dependency.
#include <cuda_runtime.h>
#include "sdd_internal.cuh"
#include "sdd_fft.cuh"
#include "sdd_rowops.cuh"

namespace sdd {

// shared memory of k_fx_rows in units of T: RA, RB (5P complex each), W, E (P complex each), RG (9P),
// kf (P), operator rows (2 kMaxNr), reduction words (9*32 of 8 bytes), scales (32)
size_t fx_smem_bytes(int M, int P, int prec) {
  (void)M;
  const size_t es = prec == SDD_PREC_MIXED ? sizeof(float) : sizeof(double);
  return (34 * (size_t)P + 2 + 2 * kMaxNr + 32) * es + 9 * 32 * 8;
}

// DCT3 input x_k of transform t of the nine fields (see the header comment of sdd_fft.cuh); kf[k] = k.
// Fields: 0 JT_psi, 1 komega, 2 kDpsi, 3 DT, 4 DC (cosine type); 5 omega, 6 Dpsi, 7 kT, 8 kC (sine type).
template <typename T>
__device__ __forceinline__ T fx_x(int t, int k, int M, int P, const T* kf, const T* JP, const T* OM,
                                  const T* DP, const T* DTv, const T* DCv, const T* Tv, const T* Sv) {
  if (t < 5) {
    if (k >= M) return (T)0;
    switch (t) {
      case 0: return JP[k];
      case 1: return k >= 1 ? kf[k] * OM[k - 1] : (T)0;
      case 2: return k >= 1 ? kf[k] * DP[k - 1] : (T)0;
      case 3: return DTv[k];
      default: return DCv[k];
    }
  }
  const int w = P - k;  // wavenumber
  if (k == 0 || w > M - 1) return (T)0;
  switch (t) {
    case 5: return OM[w - 1];
    case 6: return DP[w - 1];
    case 7: return -(kf[w] * Tv[w]);
    default: return -(kf[w] * Sv[w]);
  }
}

// Runs body(rd) with rd(e) = element e of shell b's state as T: FP32 kernels read the caller's FP32 copy
// when there is one (the previous mixed step wrote it with the same rounding), else the FP64 state is
// converted (an FP64-pipe instruction per element).  The choice is made once, outside the loops, so the
// compiler cannot turn it into a per-element select that executes both loads and the conversion.
template <typename T, typename F>
__device__ __forceinline__ void with_x(const FxArgs& a, int b, F&& body) {
  if (sizeof(T) == 4 && a.X32) {
    const float* x = a.X32 + (size_t)b * a.x32_stride;
    body([x](size_t e) { return (T)__ldg(x + e); });
  } else {
    const double* x = a.X + (size_t)b * a.x_stride;
    body([x](size_t e) { return (T)__ldg(x + e); });
  }
}

// Arithmetic shared by the fused and the split nonlinear-term kernels.  This file is compiled without
// automatic fma contraction and every multiply-add below is an explicit fma, so both kernels round
// identically.
// J_theta_RT (:437-472) and A2_SINE_R2 (:476-526) at mode k along a row: jp, and om updated from D2 psi.
template <typename T>
__device__ __forceinline__ void jp_om(int k, int M, const T* kf, const T* pv, const T* Sc, T ir4n, T& jp, T& om) {
  const T s1 = (k + 1 < M) ? Sc[k + 1] : (T)0;
  jp = (k == 0) ? s1 : fma(kf[k + 1], pv[k - 1], (T)2 * s1);
  const T s2 = (k + 2 < M) ? Sc[k + 2] : (T)0;
  om = fma(-kf[k + 1], ir4n * fma(kf[k + 2], pv[k], (T)2 * s2), om);
}
// W_k of a DCT3 pair (rows A, B with scales sa, sb): s_A V_A(k) + i s_B V_B(k), V(k) = e_k (x_k - i x_{P-k}).
template <typename T, typename C>
__device__ __forceinline__ C dct3_pack(C e, T xa, T xar, T xb, T xbr, T sa, T sb) {
  const T a1 = fma(e.x, xa, e.y * xar), a2 = fma(e.y, xa, -(e.x * xar));
  const T b1 = fma(e.x, xb, e.y * xbr), b2 = fma(e.y, xb, -(e.x * xbr));
  return cmk<C>(fma(sa, a1, -(sb * b2)), fma(sa, a2, sb * b1));
}
// y_A, y_B of a DCT2 pair from Z_k, Z_{-k} and e_k = 0.5 (cos, sin)(pi k/2P).
template <typename T, typename C>
__device__ __forceinline__ void dct2_unpack(C Zk, C Zm, C e, T& ya, T& yb) {
  ya = fma(e.x, Zk.x + Zm.x, e.y * (Zk.y - Zm.y));
  yb = fma(e.x, Zk.y + Zm.y, -(e.y * (Zk.x - Zm.x)));
}
// Grid products at point i (:791-793 for MODE 0, :884-887 for MODE 1 with base fields bs):
// pair 0 = (Q, R) (sine type), pair 1 = (NT, NS) (cosine type).
template <typename T, int MODE>
__device__ __forceinline__ void grid_products(int pair, const T* RG, const T* bs, int i, int P, T& v0, T& v1) {
  const T JT = RG[i], DPg = RG[6 * P + i];
  if (pair == 0) {
    const T kO = RG[P + i], kDP = RG[2 * P + i], O = RG[5 * P + i];
    if (MODE != 1) {
      v0 = JT * O;
      v1 = fma(kDP, O, DPg * kO);
    } else {
      const T aJT = bs[i], akO = bs[P + i], akDP = bs[2 * P + i], aO = bs[5 * P + i], aDP = bs[6 * P + i];
      v0 = fma(aJT, O, JT * aO);
      v1 = fma(akDP, O, aDP * kO) + fma(kDP, aO, DPg * akO);
    }
  } else {
    const T DTg = RG[3 * P + i], DCg = RG[4 * P + i], kT = RG[7 * P + i], kC = RG[8 * P + i];
    if (MODE != 1) {
      v0 = fma(JT, DTg, -(DPg * kT));
      v1 = fma(JT, DCg, -(DPg * kC));
    } else {
      const T aJT = bs[i], aDT = bs[3 * P + i], aDC = bs[4 * P + i], aDP = bs[6 * P + i];
      const T akT = bs[7 * P + i], akC = bs[8 * P + i];
      v0 = fma(JT, aDT, -(DPg * akT)) + fma(aJT, DTg, -(aDP * kT));
      v1 = fma(JT, aDC, -(DPg * akC)) + fma(aJT, DCg, -(aDP * kC));
    }
  }
}

// MODE 0: NLIN_FX (optionally storing the grid fields); 1: NLIN_DFX with base fields from the cache;
// 2: grid fields only (fills the cache).
template <typename T, int MODE>
__global__ void __launch_bounds__(kFxRowThreads) k_fx_rows(FxArgs a) {
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = a.M, nr = a.nr, P = a.P;
  const int n = blockIdx.x, b = blockIdx.y;
  if (a.active && !a.active[b]) return;
  const int tid = threadIdx.x, bd = blockDim.x;

  C* RA = reinterpret_cast<C*>(smem_raw);
  C* RB = RA + 5 * P;
  C* Wt = RB + 5 * P;
  C* Et = Wt + P;
  T* RG = reinterpret_cast<T*>(Et + P);
  T* kf = RG + 9 * P;          // kf[k] = k, k < P + 2
  T* opr = kf + P + 2;
  T* scl = opr + 2 * kMaxNr;   // 9 scales + 9 inverse scales (inverse transforms), reused for 4+4
  using U = typename Bits<T>::U;
  U* red = reinterpret_cast<U*>(scl + 32);   // 9*32 reduction words
  T* pv = RG;
  T* Tv = pv + M;
  T* Sv = Tv + M;
  T* DP = Sv + M;
  T* OM = DP + M;
  T* DTv = OM + M;
  T* DCv = DTv + M;
  T* JP = DCv + M;
  T* Sc = JP + M;
  const C* wg = reinterpret_cast<const C*>(a.ops.w);
  const C* eg = reinterpret_cast<const C*>(a.ops.e);
  for (int i = tid; i < P; i += bd) {
    Wt[i] = wg[i];
    Et[i] = eg[i];
  }
  for (int i = tid; i < P + 2; i += bd) kf[i] = (T)i;
  const T* Drg = reinterpret_cast<const T*>(a.ops.Dr);
  const T* D2g = reinterpret_cast<const T*>(a.ops.D2r2);
  for (int m = tid; m < nr; m += bd) {
    opr[m] = Drg[n * nr + m];
    opr[nr + m] = D2g[n * nr + m];
  }
  const T ir4n = reinterpret_cast<const T*>(a.ops.ir4r2)[n];
  __syncthreads();

  // ---- 1. radial contractions of row n (Derivatives, :698-729) and the row values ----
  const int N = M * nr;
  // mixed plans with tensor cores: the four contractions were formed by k_deriv_tc ([op][n][k] blocks)
  const T* Dt = (sizeof(T) == 4 && a.deriv_t) ? reinterpret_cast<const T*>(a.deriv) + (size_t)b * a.deriv_stride
                                              : nullptr;
  with_x<T>(a, b, [&](auto xr) {
  for (int k = tid; k < M; k += bd) {
    const size_t ps = (size_t)k * nr, ts = N + (size_t)k * nr, ss = 2 * (size_t)N + (size_t)k * nr;
    const bool psi_on = !(a.sym && (k % 2 == 0));
    const bool ts_on = !(a.sym && (k % 2 == 1));
    T dp = 0, d2 = 0, dtv = 0, dcv = 0, pn = 0, tn = 0, sn = 0;
    if (psi_on) {
      if (Dt) {
        dp = Dt[(size_t)n * M + k];
        d2 = Dt[((size_t)nr + n) * M + k];
      } else {
        for (int m = 0; m < nr; ++m) {
          const T x = xr(ps + m);
          dp = fma(opr[m], x, dp);
          d2 = fma(opr[nr + m], x, d2);
        }
      }
      pn = xr(ps + n);
    }
    if (ts_on) {
      if (Dt) {
        dtv = Dt[((size_t)2 * nr + n) * M + k];
        dcv = Dt[((size_t)3 * nr + n) * M + k];
      } else {
        for (int m = 0; m < nr; ++m) {
          dtv = fma(opr[m], xr(ts + m), dtv);
          dcv = fma(opr[m], xr(ss + m), dcv);
        }
      }
      tn = xr(ts + n);
      sn = xr(ss + n);
    }
    pv[k] = pn;
    Tv[k] = tn;
    Sv[k] = sn;
    DP[k] = dp;
    OM[k] = d2;
    DTv[k] = dtv;
    DCv[k] = dcv;
  }
  });
  __syncthreads();
  parity_suffix<T>(pv, Sc, M);
  __syncthreads();
  // J_theta_RT (:437-472) and A2_SINE_R2 (:476-526) along the row
  for (int k = tid; k < M; k += bd) jp_om<T>(k, M, kf, pv, Sc, ir4n, JP[k], OM[k]);
  __syncthreads();
  // ---- 2. nine inverse transforms as five paired DCT3s (:776-786) ----
  // the nine DCT3 input rows, materialised once (in RB, free until the FFT), with their maxima
  T* XV = reinterpret_cast<T*>(RB);
  {
    U mb[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) {
      mb[t] = 0;
      for (int k = tid; k < P; k += bd) {
        const T v = fx_x<T>(t, k, M, P, kf, JP, OM, DP, DTv, DCv, Tv, Sv);
        XV[t * P + k] = v;
        const U u = Bits<T>::absbits(v);
        mb[t] = u > mb[t] ? u : mb[t];
      }
    }
    block_max_scales<T, 9>(mb, red, scl);
  }
  // W_k = s_A V_A(k) + i s_B V_B(k),  V(k) = 0.5 e^{i pi k/2P} (x_k - i x_{P-k}),  V(0) = x_0;
  // Et holds 0.5 e^{i pi k/2P}.
  for (int idx = tid; idx < 5 * P; idx += bd) {
    const int p = idx / P;
    const int k = idx - p * P;
    const int ta = 2 * p, tb = 2 * p + 1;
    const T sa = scl[ta], sb = (tb < 9) ? scl[tb] : (T)0;
    const T xa = XV[ta * P + k], xb = (tb < 9) ? XV[tb * P + k] : (T)0;
    if (k == 0) {
      RA[idx] = cmk<C>(sa * xa, sb * xb);
    } else {
      const T xar = XV[ta * P + P - k], xbr = (tb < 9) ? XV[tb * P + P - k] : (T)0;
      RA[idx] = dct3_pack<T, C>(Et[k], xa, xar, xb, xbr, sa, sb);
    }
  }
  __syncthreads();
  C* res = fft_rows<T, true>(RA, RB, 5, a.st, Wt);
  for (int idx = tid; idx < 9 * P; idx += bd) {
    const int t = idx / P;
    const int i = idx - t * P;
    const int src = (i & 1) ? (P - 1 - (i >> 1)) : (i >> 1);
    const C v = res[(t >> 1) * P + src];
    T val = ((t & 1) ? v.y : v.x) * scl[9 + t];
    if (t >= 5 && (i & 1)) val = -val;
    RG[idx] = val;
  }
  __syncthreads();

  if (MODE != 1 && a.base != nullptr) {
    T* bc = reinterpret_cast<T*>(a.base) + (size_t)b * a.base_stride + (size_t)n * 9 * P;
    for (int idx = tid; idx < 9 * P; idx += bd) bc[idx] = RG[idx];
  }
  if (MODE == 2) return;

  // ---- 3. grid products (:791-793 or :884-887); sine outputs pre-multiplied by (-1)^i ----
  T* PR = reinterpret_cast<T*>(RA);
  const T* bs = (MODE == 1) ? reinterpret_cast<const T*>(a.base) + (size_t)b * a.base_stride +
                                  (size_t)n * 9 * P
                            : nullptr;
  U m4[4] = {0, 0, 0, 0};
  for (int i = tid; i < P; i += bd) {
    T Q, Rr, NT, NS;
    grid_products<T, MODE>(0, RG, bs, i, P, Q, Rr);
    grid_products<T, MODE>(1, RG, bs, i, P, NT, NS);
    const T sg = (i & 1) ? (T)-1 : (T)1;
    PR[i] = sg * Q;
    PR[P + i] = sg * Rr;
    PR[2 * P + i] = NT;
    PR[3 * P + i] = NS;
    const U u0 = Bits<T>::absbits(Q), u1 = Bits<T>::absbits(Rr), u2 = Bits<T>::absbits(NT),
            u3 = Bits<T>::absbits(NS);
    m4[0] = u0 > m4[0] ? u0 : m4[0];
    m4[1] = u1 > m4[1] ? u1 : m4[1];
    m4[2] = u2 > m4[2] ? u2 : m4[2];
    m4[3] = u3 > m4[3] ? u3 : m4[3];
  }
  block_max_scales<T, 4>(m4, red, scl);   // scl[0..4) scales, scl[4..8) inverses

  // ---- 4. four forward transforms as two paired DCT2s (:797-802) ----
  for (int idx = tid; idx < 2 * P; idx += bd) {
    const int p = idx / P;
    const int nn = idx - p * P;
    const int src = makhoul_src(nn, P);
    RB[idx] = cmk<C>(scl[2 * p] * PR[(2 * p) * P + src], scl[2 * p + 1] * PR[(2 * p + 1) * P + src]);
  }
  __syncthreads();
  C* Z = fft_rows<T, false>(RB, RA, 2, a.st, Wt);
  double* o = a.out4 + (size_t)b * a.out_stride;
  const T two_P = (T)2 / (T)P, one_P = (T)1 / (T)P;
  for (int idx = tid; idx < 2 * M; idx += bd) {
    const int p = idx / M;
    const int s = idx - p * M;
    T ya = 0, yb = 0;
    bool zero = false;
    int k;
    if (p == 0) {            // sine pair: slot s <-> wavenumber s+1, read at k = P-1-s
      zero = (s == M - 1) || (a.sym && (s % 2 == 0));
      k = P - 1 - s;
    } else {
      zero = a.sym && (s % 2 == 1);
      k = s;
    }
    if (!zero) {
      dct2_unpack<T, C>(Z[p * P + k], Z[p * P + ((P - k) % P)], Et[k], ya, yb);
      const T sc = (p == 1 && k == 0) ? one_P : two_P;
      ya *= sc * scl[4 + 2 * p];
      yb *= sc * scl[4 + 2 * p + 1];
    }
    const size_t q0 = (size_t)(2 * p) * N + (size_t)s * nr + n;
    o[q0] = (double)ya;
    o[q0 + N] = (double)yb;
    if (sizeof(T) == 4 && p == 0 && a.q32) a.q32[(size_t)b * M * a.nr + (size_t)s * a.nr + n] = (float)ya;
  }
}

// ---- split nonlinear term: the same arithmetic over 7 CTAs per radial row ------------------------
// k_fx_rows runs a row's five paired inverse and two paired forward transforms one after the other on
// one SM, so a single shell occupies only nr SMs.  For small batches the work is split:
//   k_fx_grid (nr x 5 CTAs per shell): CTA (n, p) forms the DCT3 input rows t = 2p, 2p+1 of row n (with
//     the radial contractions those two fields need), runs their paired inverse transform and writes the
//     two grid rows to grid[shell][n][t][P] (the layout of the base-state cache);
//   k_fx_prod (nr x 2 CTAs per shell): CTA (n, p) forms product pair p on the grid of row n (p = 0: the
//     sine-type Q, R; p = 1: the cosine-type NT, NS) and runs their paired forward transform into out4.
// Per element the operations and their order are those of k_fx_rows, so the results are identical.
constexpr int kFxSplitThreads = 256;
constexpr size_t kFxDerivStageMaxBytes = 110 * 1024;   // two derivative CTAs per SM

// FP32 grid kernels of the fused right-hand side keep FP64 copies of the row's psi, T, S and psi's parity
// suffix sums (4 M doubles) for the linear parts, after the T-typed arrays.
__host__ __device__ inline size_t fx_grid_lin64_offset(int M, int P, int prec) {
  const size_t es = prec == SDD_PREC_MIXED ? sizeof(float) : sizeof(double);
  return (((8 * (size_t)P + P + 2 + 9 * (size_t)M + 32) * es + 2 * 32 * 8) + 15) / 16 * 16;
}
size_t fx_grid_smem_bytes(int M, int P, int prec) {
  return fx_grid_lin64_offset(M, P, prec) + (prec == SDD_PREC_MIXED ? 4 * (size_t)M * sizeof(double) : 0);
}
size_t fx_prod_smem_bytes(int P, int prec) {
  const size_t es = prec == SDD_PREC_MIXED ? sizeof(float) : sizeof(double);
  return (8 * (size_t)P + 2 * (size_t)P + 32) * es + 2 * 32 * 8;
}

// Radial contractions of the split path (Derivatives, Matrix_Operators.py:698-729), one CTA per (mode,
// shell): Dr psi_k, D2r2 psi_k, Dr T_k, Dr S_k for every radial row n, each a sequential fma chain over the
// columns in the order of the fused kernel's (so both paths round identically).  With the fused
// right-hand side a fifth block, D2s psi_k in FP64, follows the four T-typed blocks (per shell:
// 4 M nr T then M nr doubles).
// sum over the TPR lanes of a row group (the order of the chains' group_sum)
template <int TPR>
__device__ __forceinline__ double lane_group_sum(double v) {
#pragma unroll
  for (int off = 1; off < TPR; off <<= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// One asynchronous global -> shared copy of an element of 4, 8 or 16 bytes (the issuing thread does not
// wait for the data: a loop of such copies has all its loads in flight at once).
template <int BYTES>
__device__ __forceinline__ void cp_async_bytes(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (BYTES == 16) asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem));
  else if constexpr (BYTES == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem));
  else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem));
}
template <typename E>
__device__ __forceinline__ void cp_async_elem(E* smem, const E* gmem) {
  static_assert(sizeof(E) == 4 || sizeof(E) == 8 || sizeof(E) == 16, "element size");
  cp_async_bytes<(int)sizeof(E)>(smem, gmem);
}
__device__ __forceinline__ void cp_async_all_done() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_all;\n" ::: "memory");
}

// Shared memory for a staged pending correction (FixArgs::stage): the G blocks of the mode's three chains
// (2 nr + nr + nr columns of ldl) and, per chain, d_{c-1} and the carry terms of its chunk c (at most
// nch - 1 vectors of 2 nr / nr / nr doubles).
__host__ __device__ inline size_t fix_stage_doubles(int nr, int ldl, int nch) {
  return (size_t)4 * nr * ldl + (size_t)(nch > 1 ? nch - 1 : 0) * 4 * nr;
}

// The asynchronous copies of a staged correction of mode k into st (16-byte aligned): the G blocks of the
// three chains at st, st + 2 nr ldl, st + 3 nr ldl; then per chain f, from st + 4 nr ldl + c o_f
// (o = 0, 2 nr, 3 nr), the c vectors d_{c-1}, part_{c,0}, ..., part_{c,c-2} of m_f doubles each.  The
// caller commits and waits.
__device__ __forceinline__ void stage_pending_fix(const FxArgs& a, int b, int k, double* st) {
  const FixArgs& x = a.fix;
  const int M = a.M, nr = a.nr, ldl = x.ldl;
  const int jj = M - 1 - k, par = jj & 1, c = (jj >> 1) / x.kc;
  if (c < 1) return;
  for (int f = 0; f < 3; ++f) {
    const bool a4 = f == 0;
    if (a.sym && !(a4 ? par == 0 : par == 1)) continue;
    const int m = a4 ? 2 * nr : nr;
    const int o = a4 ? 0 : (f == 1 ? 2 * nr : 3 * nr);
    const double* G = (a4 ? x.GA4 : (f == 1 ? x.GT : x.GS)) + (size_t)jj * m * ldl;
    double* Gs = st + (size_t)o * ldl;
    for (int e = threadIdx.x; e < m * ldl / 2; e += blockDim.x)   // m ldl is even (ldl even)
      cp_async_bytes<16>(Gs + 2 * e, G + 2 * e);
    const size_t chain = (size_t)(f * 2 + par);
    const double* d = x.dbuf + (size_t)b * x.d_stride + chain * x.nch * x.ldd + (size_t)(c - 1) * x.ldd;
    const double* prow = x.pbuf + (size_t)b * x.p_stride + (chain * x.np + (size_t)(c - 1) * (c - 2) / 2) * x.ldd;
    double* Ts = st + (size_t)4 * nr * ldl + (size_t)c * o;
    for (int e = threadIdx.x; e < c * m; e += blockDim.x) {
      const int v = e / m, i = e - v * m;
      cp_async_bytes<8>(Ts + e, v == 0 ? d + i : prow + (size_t)(v - 1) * x.ldd + i);
    }
  }
}

// The pending correction of mode k (see FixArgs) on xd (the mode's FP64 psi, T, S rows, in shared memory),
// the three fields at once, each by its own 128 threads (threads 128 f .. 128 f + 127; the CTA has 384):
// s_c = d_{c-1} + part_{c,0} + ... in index order, then xd += G_jj s_c with rows split over TPR lanes as
// k_mode_mv<TPR, true> (the same bits); the corrected rows are written back to the state (and its FP32
// copy).  sc holds the three carried states (4 nr doubles).  st: the staged G blocks and terms
// (stage_pending_fix, landed), or null to read them from global memory.
template <int TPR>
__device__ void apply_pending_fix(const FxArgs& a, int b, int k, double* xd, double* sc, const double* st) {
  const FixArgs& x = a.fix;
  const int M = a.M, nr = a.nr, ldl = x.ldl;
  const int jj = M - 1 - k, par = jj & 1, c = (jj >> 1) / x.kc;
  if (c < 1) return;                                   // uniform over the CTA
  const size_t N = (size_t)M * nr;
  const int f = threadIdx.x >> 7, t = threadIdx.x & 127;
  const bool a4 = f == 0;
  const bool on = f < 3 && !(a.sym && !(a4 ? par == 0 : par == 1));
  const int m = a4 ? 2 * nr : nr;
  const int o = a4 ? 0 : (f == 1 ? 2 * nr : 3 * nr);
  double* s = sc + o;
  if (on) {
    const size_t chain = (size_t)(f * 2 + par);
    const int nt = c - 1;
    if (st) {
      const double* Ts = st + (size_t)4 * nr * ldl + (size_t)c * o;
      for (int e = t; e < m; e += 128) {
        double v = Ts[e];                              // d_{c-1} + part_0 + ... + part_{c-2} in index order
        for (int u = 0; u < nt; ++u) v += Ts[(size_t)(u + 1) * m + e];
        s[e] = v;
      }
    } else {
      const double* d = x.dbuf + (size_t)b * x.d_stride + chain * x.nch * x.ldd;
      const double* prow = x.pbuf + (size_t)b * x.p_stride + (chain * x.np + (size_t)(c - 1) * (c - 2) / 2) * x.ldd;
      for (int e = t; e < m; e += 128) {
        // d_{c-1} + part_0 + ... + part_{c-2} in index order, the terms loaded eight at a time (a load
        // after each addition would wait out one L2 round trip per term)
        double v = d[(size_t)(c - 1) * x.ldd + e];
        for (int u0 = 0; u0 < nt; u0 += 8) {
          double tv[8];
#pragma unroll
          for (int k = 0; k < 8; ++k) tv[k] = (u0 + k < nt) ? prow[(size_t)(u0 + k) * x.ldd + e] : 0.0;
#pragma unroll
          for (int k = 0; k < 8; ++k)
            if (u0 + k < nt) v += tv[k];
        }
        s[e] = v;
      }
    }
  }
  __syncthreads();
  if (on) {
    const double* G = st ? st + (size_t)o * ldl : (a4 ? x.GA4 : (f == 1 ? x.GT : x.GS)) + (size_t)jj * m * ldl;
    const int i = t / TPR, q = t % TPR;
    for (int r0 = 0; r0 < nr; r0 += 128 / TPR) {
      const int r = r0 + i;
      const int rr = r < nr ? r : 0;
      double acc = 0.0;
#pragma unroll 16
      for (int col = q; col < m; col += TPR) acc = fma(G[(size_t)col * ldl + rr], s[col], acc);
      acc = lane_group_sum<TPR>(acc);
      if (r < nr && q == 0) {
        const double v = xd[f * nr + r] + acc;
        xd[f * nr + r] = v;
        const size_t o = (size_t)b * a.x_stride + (size_t)f * N + (size_t)k * nr + r;
        x.X[o] = v;
        if (x.X32) x.X32[(size_t)b * a.x32_stride + (size_t)f * N + (size_t)k * nr + r] = (float)v;
      }
    }
  }
  __syncthreads();
}

// T-typed Dr, D2r2 and the mode's rows; then (FP64) the corrected rows and carried states of a pending fix
// (7 nr); then the fused right-hand side's D2s (nr^2) and the mode's FP64 psi row (nr); then, 16-byte
// aligned, the staged correction (stage_doubles, fix_stage_doubles, or 0)
__host__ __device__ inline size_t fx_deriv_stage_offset(int nr, int prec, bool fix, bool fuse) {
  const size_t es = prec == SDD_PREC_MIXED ? sizeof(float) : sizeof(double);
  const size_t t = ((2 * (size_t)nr * nr + 3 * (size_t)nr) * es + 15) / 16 * 16;
  return (t + (fix ? 7 * (size_t)nr * sizeof(double) : 0) + (fuse ? ((size_t)nr * nr + nr) * sizeof(double) : 0) +
          15) / 16 * 16;
}
size_t fx_deriv_smem_bytes(int nr, int prec, bool fix, bool fuse, size_t stage_doubles) {
  return fx_deriv_stage_offset(nr, prec, fix, fuse) + stage_doubles * sizeof(double);
}


template <typename T>
__global__ void __launch_bounds__(384) k_fx_deriv(FxArgs a, T* deriv, size_t deriv_stride) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = a.M, nr = a.nr;
  const int k = blockIdx.x, b = blockIdx.y;
  if (a.active && !a.active[b]) return;
  T* ops = reinterpret_cast<T*>(smem_raw);     // Dr, D2r2 (nr x nr each, row-major)
  T* xv = ops + 2 * nr * nr;                  // psi_k, T_k, S_k
  // with a pending correction: the mode's FP64 rows (corrected here) and a carried state
  double* xd = reinterpret_cast<double*>(smem_raw + ((2 * (size_t)nr * nr + 3 * (size_t)nr) * sizeof(T) + 15) / 16 * 16);
  double* sc = xd + 3 * nr;
  double* D2sm = xd + (a.fix.on ? 7 * nr : 0);        // fused right-hand side: A2_SINE's D2 (FP64)
  const T* Drg = reinterpret_cast<const T*>(a.ops.Dr);
  const T* D2g = reinterpret_cast<const T*>(a.ops.D2r2);
  double* stg = (a.fix.on && a.fix.stage)
                    ? reinterpret_cast<double*>(smem_raw + fx_deriv_stage_offset(nr, sizeof(T) == 4 ? SDD_PREC_MIXED
                                                                                                    : SDD_PREC_FP64,
                                                                                 true, a.fuse_rhs != 0))
                    : nullptr;
  // the operators (and the rows, G blocks and carry terms of a pending fix) stream in asynchronously: one
  // L2 round trip, not one per element each thread copies
  if (stg) stage_pending_fix(a, b, k, stg);
  for (int e = threadIdx.x; e < nr * nr; e += blockDim.x) {
    cp_async_elem(ops + e, Drg + e);
    cp_async_elem(ops + nr * nr + e, D2g + e);
    if (a.fuse_rhs) cp_async_elem(D2sm + e, a.rl.D2s + e);
  }
  const int N = M * nr;
  if (a.fix.on) {
    for (int e = threadIdx.x; e < 3 * nr; e += blockDim.x) {
      const int f = e / nr, m = e - f * nr;
      cp_async_elem(xd + e, a.fix.X + (size_t)b * a.x_stride + (size_t)f * N + (size_t)k * nr + m);
    }
    cp_async_all_done();
    __syncthreads();
    if (nr <= 32) apply_pending_fix<4>(a, b, k, xd, sc, stg);
    else apply_pending_fix<2>(a, b, k, xd, sc, stg);
    for (int e = threadIdx.x; e < 3 * nr; e += blockDim.x) xv[e] = (T)xd[e];
  } else {
    with_x<T>(a, b, [&](auto xr) {
      for (int e = threadIdx.x; e < 3 * nr; e += blockDim.x) {
        const int f = e / nr, m = e - f * nr;
        xv[e] = xr((size_t)f * N + (size_t)k * nr + m);
      }
    });
    if (a.fuse_rhs)
      for (int e = threadIdx.x; e < nr; e += blockDim.x)
        cp_async_elem(D2sm + nr * nr + e, a.X + (size_t)b * a.x_stride + (size_t)k * nr + e);
    cp_async_all_done();
  }
  __syncthreads();
  T* D = deriv + (size_t)b * deriv_stride;
  const int nops = a.fuse_rhs ? 5 : 4;
  const int op0 = a.deriv_t ? 4 : 0;    // tensor cores: only the pending correction and the FP64 block here
  for (int e = threadIdx.x + op0 * nr; e < nops * nr; e += blockDim.x) {
    const int op = e / nr, n = e - op * nr;
    if (op < 4) {
      const T* row = ops + (op == 1 ? nr * nr : 0) + (size_t)n * nr;
      const T* x = xv + (op < 2 ? 0 : (op - 1) * nr);
      T acc = 0;
      for (int m = 0; m < nr; ++m) acc = fma(row[m], x[m], acc);
      D[((size_t)op * M + k) * nr + n] = acc;
    } else {   // A2_SINE's D2 psi for the fused right-hand side (FP64; the order of k_rhs's dot)
      const double* row = D2sm + (size_t)n * nr;
      double acc = 0;
      if (a.fix.on) {          // the corrected rows (this kernel wrote them: not through the read-only path)
        for (int m = 0; m < nr; ++m) acc = fma(row[m], xd[m], acc);
      } else {
        const double* ps = D2sm + nr * nr;     // the mode's FP64 psi row
        for (int m = 0; m < nr; ++m) acc = fma(row[m], ps[m], acc);
      }
      reinterpret_cast<double*>(D)[(size_t)4 * M * nr * sizeof(T) / 8 + (size_t)k * nr + n] = acc;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kFxSplitThreads) k_fx_grid(FxArgs a, T* grid, size_t grid_stride) {
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = a.M, nr = a.nr, P = a.P;
  const int n = blockIdx.x, pr = blockIdx.y, b = blockIdx.z;
  if (a.active && !a.active[b]) return;
  const int tid = threadIdx.x, bd = blockDim.x;
  const int ta = 2 * pr, tb = 2 * pr + 1;      // tb = 9 (absent) for the last pair

  C* RA = reinterpret_cast<C*>(smem_raw);
  C* RB = RA + P;
  C* Wt = RB + P;
  C* Et = Wt + P;
  T* kf = reinterpret_cast<T*>(Et + P);   // kf[k] = k, k < P + 2
  T* pv = kf + P + 2;
  T* Tv = pv + M;
  T* Sv = Tv + M;
  T* DP = Sv + M;
  T* OM = DP + M;
  T* DTv = OM + M;
  T* DCv = DTv + M;
  T* JP = DCv + M;
  T* Sc = JP + M;
  T* scl = Sc + M;
  using U = typename Bits<T>::U;
  U* red = reinterpret_cast<U*>(scl + 32);
  const C* wg = reinterpret_cast<const C*>(a.ops.w);
  const C* eg = reinterpret_cast<const C*>(a.ops.e);
  for (int i = tid; i < P; i += bd) {               // asynchronous: in flight while the row loads
    cp_async_elem(Wt + i, wg + i);
    cp_async_elem(Et + i, eg + i);
  }
  for (int i = tid; i < P + 2; i += bd) kf[i] = (T)i;
  const T ir4n = reinterpret_cast<const T*>(a.ops.ir4r2)[n];
  // (no barrier: the row loads below do not read the tables; the one after them covers both)

  // which row quantities the pair's two fields need (fields: 0 JT_psi, 1 komega, 2 kDpsi, 3 DT, 4 DC,
  // 5 omega, 6 Dpsi, 7 kT, 8 kC)
  const bool need_psi = pr == 0 || pr == 2;            // pv (JT_psi, omega's A2 term) and D2 psi (omega)
  // The linear parts of the fused right-hand sides.  FP64 kernels split them over three pairs: pair 2 the T
  // and S parts, and psi's part by modes between pair 0 (k < M/2) and pair 4, whose one field leaves it the
  // least work (it forms psi's parity sums for that alone): so no pair carries all of psi's part beside its
  // own rows.  FP32 kernels form all three in pair 0 from FP64 copies of the row.
  const bool lin = a.fuse_rhs && (pr == 0 || (sizeof(T) == 8 && (pr == 2 || pr == 4)));
  const bool lin_psi = lin && (pr == 0 || pr == 4);
  const bool lin_ts = lin && (pr == 2 || sizeof(T) == 4);
  const int kp0 = (sizeof(T) == 8 && pr == 4) ? M / 2 : 0;   // psi's part: modes [kp0, kp1) of this pair
  const int kp1 = (sizeof(T) == 8 && pr == 0) ? M / 2 : M;
  double* pv64 = nullptr;
  if (sizeof(T) == 4 && lin)
    pv64 = reinterpret_cast<double*>(smem_raw + fx_grid_lin64_offset(M, P, SDD_PREC_MIXED));
  const int N = M * nr;
  const double* Xs = a.X + (size_t)b * a.x_stride;
  const T* Dv = reinterpret_cast<const T*>(a.deriv) + (size_t)b * a.deriv_stride;   // k_fx_deriv
  // the psi part's FP64 D2 psi (k_fx_deriv's fifth block) for this thread's first mode, loaded with the row
  const double* D2p = reinterpret_cast<const double*>(Dv) + (size_t)4 * M * nr * sizeof(T) / 8;
  double d2s0 = 0.0;
  if (lin_psi && tid >= kp0 && tid < kp1 && !(a.sym && (tid % 2 == 0))) d2s0 = D2p[(size_t)tid * nr + n];
  // the linear parts' per-row scalars, also loaded with the row (read after the parity sums)
  double lRa = 0.0, lRas = 0.0, lir2 = 0.0, lrsq = 0.0, ldT0 = 0.0, lgr = 0.0;
  if (lin) {
    lRa = a.rl.Ra[b];
    lRas = a.rl.Ra_s[b];
    lir2 = a.rl.ir2s[n];
    lrsq = a.rl.rsq[n];
    ldT0 = a.rl.dT0[n];
    lgr = a.rl.gr[n];
  }
  with_x<T>(a, b, [&](auto xr) {
  for (int k = tid; k < M; k += bd) {
    const bool psi_on = !(a.sym && (k % 2 == 0));
    const bool ts_on = !(a.sym && (k % 2 == 1));
    T dp = 0, d2 = 0, dtv = 0, dcv = 0, pn = 0, tn = 0, sn = 0;
    // k_fx_deriv writes [op][k][n]; k_deriv_tc (deriv_t) the transposed [op][n][k]
    const size_t o0 = a.deriv_t ? (size_t)n * M + k : (size_t)k * nr + n;
    const size_t ob = (size_t)M * nr;
    if (psi_on) {
      dp = Dv[o0];
      d2 = Dv[ob + o0];
      pn = xr((size_t)k * nr + n);
    }
    if (ts_on) {
      dtv = Dv[2 * ob + o0];
      dcv = Dv[3 * ob + o0];
      tn = xr(N + (size_t)k * nr + n);
      sn = xr(2 * (size_t)N + (size_t)k * nr + n);
    }
    pv[k] = pn;
    Tv[k] = tn;
    Sv[k] = sn;
    DP[k] = dp;
    OM[k] = d2;
    DTv[k] = dtv;
    DCv[k] = dcv;
    if (pv64) {
      pv64[k] = psi_on ? __ldg(Xs + (size_t)k * nr + n) : 0.0;
      pv64[2 * M + k] = ts_on ? __ldg(Xs + N + (size_t)k * nr + n) : 0.0;
      pv64[3 * M + k] = ts_on ? __ldg(Xs + 2 * N + (size_t)k * nr + n) : 0.0;
    }
  }
  });
  cp_async_all_done();
  __syncthreads();
  if (need_psi || lin_psi) {
    parity_suffix<T>(pv, Sc, M);                       // (ends with a barrier)
    if (pv64) parity_suffix<double>(pv64, pv64 + M, M);
    // one loop: the linear parts of the right-hand sides at row n (k_rhs's expressions, Main.py:262-280, in
    // FP64) and J_theta_RT / A2_SINE_R2 of the row, independent per k
    const double* pvd = pv64 ? pv64 : reinterpret_cast<const double*>(pv);
    const double* Scd = pv64 ? pv64 + M : reinterpret_cast<const double*>(Sc);
    const double* Tvd = pv64 ? pv64 + 2 * M : reinterpret_cast<const double*>(Tv);
    const double* Svd = pv64 ? pv64 + 3 * M : reinterpret_cast<const double*>(Sv);
    const RhsArgs& r = a.rl;
    const double dt = r.dt, dtPr = r.dt * r.Pr;
    const double Ra = lRa, Ras = lRas;
    const double ir2 = lir2, rsq = lrsq, dT0 = ldT0, gr = lgr;
    double* R = lin ? r.rhs + (size_t)b * r.rhs_stride : nullptr;
    for (int k = tid; k < M; k += bd) {
      if (need_psi) jp_om<T>(k, M, kf, pv, Sc, ir4n, JP[k], OM[k]);
      if (lin) {
        const double pk = pvd[k];
        const size_t o = (size_t)k * nr + n;
        if (lin_psi && k >= kp0 && k < kp1) {
          const double s2 = (k + 2 < M) ? Scd[k + 2] : 0.0;
          const bool psi_on = !(a.sym && (k % 2 == 0));
          const double d2s = k == tid ? d2s0 : (psi_on ? D2p[(size_t)k * nr + n] : 0.0);
          const double Om = d2s - (double)(k + 1) * ir2 * ((k + 2.0) * pk + 2.0 * s2);
          const double grv = (k < M - 1) ? (-(double)(k + 1) * gr) * (Ra * Tvd[k + 1] - Ras * Svd[k + 1]) : 0.0;
          R[o] = Om + dtPr * grv;
        }
        if (lin_ts) {
          const double pkm = k > 0 ? pvd[k - 1] : 0.0;
          const double s1 = (k + 1 < M) ? Scd[k + 1] : 0.0;
          const double JPk = (k == 0) ? 1.0 * s1 : (k + 1.0) * pkm + 2.0 * s1;
          const double psiT0 = dT0 * JPk;
          R[N + o] = rsq * Tvd[k] - dt * psiT0;
          R[2 * N + o] = rsq * Svd[k] - dt * psiT0;
        }
      }
    }
    __syncthreads();
  }
  // the pair's two DCT3 input rows (in RB, free until the FFT) and their maxima
  T* XV = reinterpret_cast<T*>(RB);
  {
    U mb[2] = {0, 0};
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int t = ta + u;
      if (t < 9)
        for (int k = tid; k < P; k += bd) {
          const T v = fx_x<T>(t, k, M, P, kf, JP, OM, DP, DTv, DCv, Tv, Sv);
          XV[u * P + k] = v;
          const U w = Bits<T>::absbits(v);
          mb[u] = w > mb[u] ? w : mb[u];
        }
    }
    block_max_scales<T, 2>(mb, red, scl);
  }
  const T sa = scl[0], sb = (tb < 9) ? scl[1] : (T)0;
  for (int k = tid; k < P; k += bd) {
    const T xa = XV[k], xb = (tb < 9) ? XV[P + k] : (T)0;
    if (k == 0) {
      RA[k] = cmk<C>(sa * xa, sb * xb);
    } else {
      const T xar = XV[P - k], xbr = (tb < 9) ? XV[P + P - k] : (T)0;
      RA[k] = dct3_pack<T, C>(Et[k], xa, xar, xb, xbr, sa, sb);
    }
  }
  __syncthreads();
  C* res = fft_rows<T, true>(RA, RB, 1, a.st, Wt);
  T* g = grid + (size_t)b * grid_stride + (size_t)n * 9 * P;
  const int nt = (tb < 9) ? 2 : 1;
  for (int idx = tid; idx < nt * P; idx += bd) {
    const int u = idx / P;
    const int i = idx - u * P;
    const int t = ta + u;
    const int src = (i & 1) ? (P - 1 - (i >> 1)) : (i >> 1);
    const C v = res[src];
    T val = (u ? v.y : v.x) * scl[2 + u];
    if (t >= 5 && (i & 1)) val = -val;
    g[(size_t)t * P + i] = val;
  }
}

template <typename T, int MODE>
__global__ void __launch_bounds__(kFxSplitThreads) k_fx_prod(FxArgs a, const T* grid, size_t grid_stride) {
  using C = typename Cplx<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = a.M, nr = a.nr, P = a.P;
  const int n = blockIdx.x, p = blockIdx.y, b = blockIdx.z;
  if (a.active && !a.active[b]) return;
  const int tid = threadIdx.x, bd = blockDim.x;
  C* RA = reinterpret_cast<C*>(smem_raw);
  C* RB = RA + P;
  C* Wt = RB + P;
  C* Et = Wt + P;
  T* PR = reinterpret_cast<T*>(Et + P);
  T* scl = PR + 2 * P;
  using U = typename Bits<T>::U;
  U* red = reinterpret_cast<U*>(scl + 32);
  const C* wg = reinterpret_cast<const C*>(a.ops.w);
  const C* eg = reinterpret_cast<const C*>(a.ops.e);
  for (int i = tid; i < P; i += bd) {               // asynchronous: in flight while the products load
    cp_async_elem(Wt + i, wg + i);
    cp_async_elem(Et + i, eg + i);
  }
  const T* RG = grid + (size_t)b * grid_stride + (size_t)n * 9 * P;
  const T* bs = (MODE == 1) ? reinterpret_cast<const T*>(a.base) + (size_t)b * a.base_stride + (size_t)n * 9 * P
                            : nullptr;
  U m2[2] = {0, 0};
#pragma unroll 2
  for (int i = tid; i < P; i += bd) {               // (unrolled: both iterations' grid loads in flight)
    T v0, v1;
    grid_products<T, MODE>(p, RG, bs, i, P, v0, v1);
    if (p == 0) {
      const T sg = (i & 1) ? (T)-1 : (T)1;
      PR[i] = sg * v0;
      PR[P + i] = sg * v1;
    } else {
      PR[i] = v0;
      PR[P + i] = v1;
    }
    const U u0 = Bits<T>::absbits(v0), u1 = Bits<T>::absbits(v1);
    m2[0] = u0 > m2[0] ? u0 : m2[0];
    m2[1] = u1 > m2[1] ? u1 : m2[1];
  }
  block_max_scales<T, 2>(m2, red, scl);   // scl[0..2) scales, scl[2..4) inverses
  for (int nn = tid; nn < P; nn += bd) {
    const int src = makhoul_src(nn, P);
    RB[nn] = cmk<C>(scl[0] * PR[src], scl[1] * PR[P + src]);
  }
  cp_async_all_done();
  __syncthreads();
  C* Z = fft_rows<T, false>(RB, RA, 1, a.st, Wt);
  const int N = M * nr;
  double* o = a.out4 + (size_t)b * a.out_stride;
  const T two_P = (T)2 / (T)P, one_P = (T)1 / (T)P;
  for (int s = tid; s < M; s += bd) {
    T ya = 0, yb = 0;
    bool zero;
    int k;
    if (p == 0) {            // sine pair: slot s <-> wavenumber s+1, read at k = P-1-s
      zero = (s == M - 1) || (a.sym && (s % 2 == 0));
      k = P - 1 - s;
    } else {
      zero = a.sym && (s % 2 == 1);
      k = s;
    }
    if (!zero) {
      dct2_unpack<T, C>(Z[k], Z[(P - k) % P], Et[k], ya, yb);
      const T sc = (p == 1 && k == 0) ? one_P : two_P;
      ya *= sc * scl[2];
      yb *= sc * scl[3];
    }
    const size_t q0 = (size_t)(2 * p) * N + (size_t)s * nr + n;
    o[q0] = (double)ya;
    o[q0 + N] = (double)yb;
    if (sizeof(T) == 4 && p == 0 && a.q32) a.q32[(size_t)b * M * a.nr + (size_t)s * a.nr + n] = (float)ya;
  }
}

// ---- right-hand sides of the three implicit solves (Main.py:262-280) ---------------------------
__global__ void __launch_bounds__(kFxThreads) k_rhs(RhsArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = a.M, nr = a.nr;
  const int n = blockIdx.x, b = blockIdx.y;
  if (a.active && !a.active[b]) return;
  const int tid = threadIdx.x, bd = blockDim.x;
  double* sm = reinterpret_cast<double*>(smem_raw);
  double* pv = sm;
  double* Sc = pv + M;
  double* D2p = Sc + M;
  double* DrQ = D2p + M;
  double* Tv = DrQ + M;
  double* Sv = Tv + M;
  double* opr = Sv + M;  // Dr row n, D2s row n
  // kd[k] = k: the mode numbers as doubles, read instead of converted (a conversion is an FP64-pipe
  // instruction on this GPU); the same exact values, so the same bits
  double* kd = opr + 2 * nr;
  for (int m = tid; m < nr; m += bd) {
    opr[m] = a.Dr[n * nr + m];
    opr[nr + m] = a.D2s[n * nr + m];
  }
  for (int k = tid; k < M + 3; k += bd) kd[k] = (double)k;
  __syncthreads();
  const int N = M * nr;
  const double* Xs = a.X + (size_t)b * a.x_stride;
  const double* O4 = a.linear ? nullptr : a.out4 + (size_t)b * a.out_stride;
  for (int k = tid; k < M; k += bd) {
    const bool psi_on = !(a.sym && (k % 2 == 0));
    const bool ts_on = !(a.sym && (k % 2 == 1));
    const double* ps = Xs + (size_t)k * nr;
    double d2 = 0, pn = 0, q = 0;
    if (psi_on) {
      for (int m = 0; m < nr; ++m) d2 = fma(opr[nr + m], __ldg(ps + m), d2);
      pn = __ldg(ps + n);
    }
    if (O4 && a.q32) {         // FP32 nonlinear term: Dr Q in FP32 (the order of the chains' fused_g)
      const float* qs = a.q32 + (size_t)b * M * nr + (size_t)k * nr;
      const float* drn = a.Dr32 + (size_t)n * nr;
      float d = 0.0f;
      for (int m = 0; m < nr; ++m) d = fmaf(__ldg(drn + m), __ldg(qs + m), d);
      q = (double)d;
    } else if (O4) {
      const double* qs = O4 + (size_t)k * nr;
      for (int m = 0; m < nr; ++m) q = fma(opr[m], __ldg(qs + m), q);
    }
    pv[k] = pn;
    D2p[k] = d2;
    DrQ[k] = q;
    Tv[k] = ts_on ? __ldg(Xs + N + (size_t)k * nr + n) : 0.0;
    Sv[k] = ts_on ? __ldg(Xs + 2 * N + (size_t)k * nr + n) : 0.0;
  }
  __syncthreads();
  parity_suffix<double>(pv, Sc, M);
  __syncthreads();
  const double dt = a.dt, dtPr = a.dt * a.Pr;
  const double Ra = a.Ra[b], Ras = a.Ra_s[b];
  const double ir2 = a.ir2s[n], rsq = a.rsq[n], dT0 = a.dT0[n], gr = a.gr[n];
  double* R = a.rhs + (size_t)b * a.rhs_stride;
  for (int k = tid; k < M; k += bd) {
    const double s1 = (k + 1 < M) ? Sc[k + 1] : 0.0;
    const double k1 = kd[k + 1], k2 = kd[k + 2];
    const double JP = (k == 0) ? 1.0 * s1 : k1 * pv[k - 1] + 2.0 * s1;    // J_theta_RT
    const double s2 = (k + 2 < M) ? Sc[k + 2] : 0.0;
    const double Om = D2p[k] - k1 * ir2 * (k2 * pv[k] + 2.0 * s2);       // A2_SINE
    const double grv = (k < M - 1) ? (-k1 * gr) * (Ra * Tv[k + 1] - Ras * Sv[k + 1]) : 0.0;
    double nxp = 0, nxt = 0, nxs = 0;
    if (O4) {
      const size_t o = (size_t)k * nr + n;
      nxp = -dt * (DrQ[k] - O4[N + o]);
      nxt = -dt * O4[2 * N + o];
      nxs = -dt * O4[3 * N + o];
    }
    const double psiT0 = dT0 * JP;                                              // DT0_theta
    const size_t o = (size_t)k * nr + n;
    if (a.cnab2) {
      // explicit terms per unit time at this step, and the Adams-Bashforth 2 extrapolation
      const size_t ko = (size_t)k * nr + n;
      const double ep = (O4 ? -(DrQ[k] - O4[N + ko]) : 0.0) + a.Pr * grv;
      const double et = (O4 ? -O4[2 * N + ko] : 0.0) - psiT0;
      const double es = (O4 ? -O4[3 * N + ko] : 0.0) - psiT0;
      double* H = a.hist + (size_t)b * a.rhs_stride;
      double xp = ep, xt = et, xs = es;
      if (a.hist_valid) {
        xp = fma(1.5, ep, -0.5 * H[o]);
        xt = fma(1.5, et, -0.5 * H[N + o]);
        xs = fma(1.5, es, -0.5 * H[2 * N + o]);
      }
      H[o] = ep;
      H[N + o] = et;
      H[2 * N + o] = es;
      R[o] = fma(dt, xp, 2.0 * Om);
      R[N + o] = fma(dt, xt, 2.0 * (rsq * Tv[k]));
      R[2 * N + o] = fma(dt, xs, 2.0 * (rsq * Sv[k]));
      continue;
    }
    R[o] = nxp + (Om + dtPr * grv);
    R[N + o] = nxt + (rsq * Tv[k] - dt * psiT0);
    R[2 * N + o] = nxs + (rsq * Sv[k] - dt * psiT0);
  }
}

// The same right-hand sides in FP32, for Jacobian products inside GMRES solves whose tolerance is far
// above FP32 rounding: X from its FP32 copy, D2s and Dr Q in FP32, the nonlinear-term outputs rounded once,
// written to rhs32.  FP64 arithmetic (and FP64<->FP32 conversion) runs on the GPU's narrow FP64 pipe; here
// only the conversions of the nonlinear-term outputs and of the per-CTA scalars remain on it.  (Staging the
// psi and Q rows in shared memory was measured slower: the 66 KB per CTA cut the resident CTAs that hide
// the latency of these row reads.)
__global__ void __launch_bounds__(kFxThreads) k_rhs32(RhsArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ float scal[8];
  const int M = a.M, nr = a.nr;
  const int n = blockIdx.x, b = blockIdx.y;
  if (a.active && !a.active[b]) return;
  const int tid = threadIdx.x, bd = blockDim.x;
  float* sm = reinterpret_cast<float*>(smem_raw);
  float* pv = sm;
  float* Sc = pv + M;
  float* D2p = Sc + M;
  float* DrQ = D2p + M;
  float* Tv = DrQ + M;
  float* Sv = Tv + M;
  float* opr = Sv + M;                      // Dr row n, D2s row n
  for (int m = tid; m < nr; m += bd) {
    opr[m] = a.Dr32[n * nr + m];
    opr[nr + m] = a.D2s32[n * nr + m];
  }
  if (tid == 0) {
    scal[0] = (float)a.dt;
    scal[1] = (float)(a.dt * a.Pr);
    scal[2] = (float)a.Ra[b];
    scal[3] = (float)a.Ra_s[b];
    scal[4] = (float)a.ir2s[n];
    scal[5] = (float)a.rsq[n];
    scal[6] = (float)a.dT0[n];
    scal[7] = (float)a.gr[n];
  }
  const int N = M * nr;
  const float* Xs = a.X32 + (size_t)b * a.x32_stride;
  const double* O4 = a.linear ? nullptr : a.out4 + (size_t)b * a.out_stride;
  __syncthreads();                          // opr / scal are visible
  for (int k = tid; k < M; k += bd) {
    const bool psi_on = !(a.sym && (k % 2 == 0));
    const bool ts_on = !(a.sym && (k % 2 == 1));
    const float* ps = Xs + (size_t)k * nr;
    float d2 = 0.0f, pn = 0.0f, q = 0.0f;
    if (psi_on) {
      for (int m = 0; m < nr; ++m) d2 = fmaf(opr[nr + m], __ldg(ps + m), d2);
      pn = __ldg(ps + n);
    }
    if (O4) {
      const float* qs = a.q32 + (size_t)b * M * nr + (size_t)k * nr;
      for (int m = 0; m < nr; ++m) q = fmaf(opr[m], __ldg(qs + m), q);
    }
    pv[k] = pn;
    D2p[k] = d2;
    DrQ[k] = q;
    Tv[k] = ts_on ? __ldg(Xs + N + (size_t)k * nr + n) : 0.0f;
    Sv[k] = ts_on ? __ldg(Xs + 2 * N + (size_t)k * nr + n) : 0.0f;
  }
  __syncthreads();
  parity_suffix<float>(pv, Sc, M);
  __syncthreads();
  const float dt = scal[0], dtPr = scal[1], Ra = scal[2], Ras = scal[3];
  const float ir2 = scal[4], rsq = scal[5], dT0 = scal[6], gr = scal[7];
  float* R = a.rhs32 + (size_t)b * a.rhs_stride;
  for (int k = tid; k < M; k += bd) {
    // k as a float without an int->float conversion: the bits of 2^23 + k, minus 2^23 (exact for k < 2^23)
    const float k1 = (__int_as_float(0x4B000000 | k) - 8388608.0f) + 1.0f;
    const float s1 = (k + 1 < M) ? Sc[k + 1] : 0.0f;
    const float JP = (k == 0) ? s1 : k1 * pv[k - 1] + 2.0f * s1;                                // J_theta_RT
    const float s2 = (k + 2 < M) ? Sc[k + 2] : 0.0f;
    const float Om = D2p[k] - k1 * ir2 * ((k1 + 1.0f) * pv[k] + 2.0f * s2);                    // A2_SINE
    const float grv = (k < M - 1) ? (-k1 * gr) * (Ra * Tv[k + 1] - Ras * Sv[k + 1]) : 0.0f;
    float nxp = 0.0f, nxt = 0.0f, nxs = 0.0f;
    const size_t o = (size_t)k * nr + n;
    if (O4) {
      nxp = -dt * (DrQ[k] - (float)O4[N + o]);
      nxt = -dt * (float)O4[2 * N + o];
      nxs = -dt * (float)O4[3 * N + o];
    }
    const float psiT0 = dT0 * JP;                                                            // DT0_theta
    R[o] = nxp + (Om + dtPr * grv);
    R[N + o] = nxt + (rsq * Tv[k] - dt * psiT0);
    R[2 * N + o] = nxs + (rsq * Sv[k] - dt * psiT0);
  }
}

// ---- standalone theta recurrences (J_theta_RT, A2_SINE_R2, A2_SINE, DT0_theta) ------------------
struct ThetaArgs {
  int op, M, nr, sym;
  const double* D2;
  const double* ir;
  const double* dT0;
  const double* g;
  double* f;
};

__global__ void __launch_bounds__(kFxThreads) k_theta_op(ThetaArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = a.M, nr = a.nr;
  const int n = blockIdx.x, b = blockIdx.y;
  const int tid = threadIdx.x, bd = blockDim.x;
  double* sm = reinterpret_cast<double*>(smem_raw);
  double* pv = sm;
  double* Sc = pv + M;
  double* D2p = Sc + M;
  double* opr = D2p + M;
  const bool a2 = (a.op == 1 || a.op == 2);
  if (a2)
    for (int m = tid; m < nr; m += bd) opr[m] = a.D2[n * nr + m];
  __syncthreads();
  const double* g = a.g + (size_t)b * M * nr;
  for (int k = tid; k < M; k += bd) {
    const bool on = !(a.sym && (k % 2 == 0));
    double d2 = 0, pn = 0;
    if (on) {
      const double* ps = g + (size_t)k * nr;
      if (a2)
        for (int m = 0; m < nr; ++m) d2 = fma(opr[m], __ldg(ps + m), d2);
      pn = __ldg(ps + n);
    }
    pv[k] = pn;
    D2p[k] = d2;
  }
  __syncthreads();
  parity_suffix<double>(pv, Sc, M);
  __syncthreads();
  double* f = a.f + (size_t)b * M * nr;
  for (int k = tid; k < M; k += bd) {
    const double s1 = (k + 1 < M) ? Sc[k + 1] : 0.0;
    const double s2 = (k + 2 < M) ? Sc[k + 2] : 0.0;
    double v;
    if (a2) {
      v = D2p[k] - (double)(k + 1) * (a.ir[n] * ((k + 2.0) * pv[k] + 2.0 * s2));
      if (a.sym && (k % 2 == 0)) v = 0.0;
    } else {
      const double jp = (k == 0) ? 1.0 * s1 : (k + 1.0) * pv[k - 1] + 2.0 * s1;
      v = (a.op == 3) ? a.dT0[n] * jp : jp;
      if (a.sym && (k % 2 == 1)) v = 0.0;
    }
    f[(size_t)k * nr + n] = v;
  }
}

// ---- standalone batched transforms (Transforms.py) -------------------------------------------
struct TrArgs {
  int kind, rows, n_in, n_out, L;
  StageArgs st;
  const double2* w;
  const double2* e;
  const double* in;
  double* out;
};

constexpr int kTrPairs = 2;

__global__ void __launch_bounds__(kFxThreads) k_transform(TrArgs a) {
  using C = double2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int L = a.L;
  C* RA = reinterpret_cast<C*>(smem_raw);
  C* RB = RA + kTrPairs * L;
  C* Wt = RB + kTrPairs * L;
  C* Et = Wt + L;
  double* scl = reinterpret_cast<double*>(Et + L);   // 4 scales + 4 inverses
  unsigned long long* red = reinterpret_cast<unsigned long long*>(scl + 8);   // 4*32
  const int tid = threadIdx.x, bd = blockDim.x;
  for (int i = tid; i < L; i += bd) {
    Wt[i] = a.w[i];
    Et[i] = a.e[i];
  }
  const int r0 = blockIdx.x * 2 * kTrPairs;
  const bool inverse = (a.kind == SDD_IDCT || a.kind == SDD_IDST);
  const bool sine = (a.kind == SDD_IDST || a.kind == SDD_DST);
  const int n_in = a.n_in, n_out = a.n_out;
  {  // per-row power-of-two balance of the pairs (see pow2_scale)
    unsigned long long m[4] = {0, 0, 0, 0};
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const int r = r0 + h;
      if (r < a.rows)
        for (int i = tid; i < n_in; i += bd) {
          const unsigned long long u = Bits<double>::absbits(a.in[(size_t)r * n_in + i]);
          m[h] = u > m[h] ? u : m[h];
        }
    }
    block_max_scales<double, 4>(m, red, scl);
  }
  if (inverse) {
    for (int idx = tid; idx < kTrPairs * L; idx += bd) {
      const int p = idx / L;
      const int k = idx - p * L;
      C V[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = r0 + 2 * p + h;
        double x = 0, xr = 0;
        if (r < a.rows) {
          const double* src = a.in + (size_t)r * n_in;
          for (int pass = 0; pass < 2; ++pass) {
            const int kk = pass == 0 ? k : L - k;
            double v = 0;
            if (pass == 1 && k == 0) break;
            if (!sine) {
              v = (kk < n_in) ? src[kk] : 0.0;
            } else if (kk == 0) {
              v = (L < n_in) ? 0.5 * src[L] : 0.0;
            } else {
              const int w = L - kk;
              v = (w <= n_in - 1) ? src[w] : 0.0;
            }
            if (pass == 0) x = v; else xr = v;
          }
          x *= scl[2 * p + h];
          xr *= scl[2 * p + h];
        }
        if (k == 0) {
          V[h] = make_double2(x, 0.0);
        } else {
          const C e = Et[k];
          V[h] = make_double2(fma(e.x, x, e.y * xr), fma(e.y, x, -(e.x * xr)));
        }
      }
      RA[idx] = make_double2(V[0].x - V[1].y, V[0].y + V[1].x);
    }
    __syncthreads();
    C* res = fft_rows<double, true>(RA, RB, kTrPairs, a.st, Wt);
    for (int idx = tid; idx < 2 * kTrPairs * L; idx += bd) {
      const int t = idx / L;
      const int i = idx - t * L;
      const int r = r0 + t;
      if (r >= a.rows) continue;
      const int src = (i & 1) ? (L - 1 - (i >> 1)) : (i >> 1);
      const C v = res[(t >> 1) * L + src];
      double val = ((t & 1) ? v.y : v.x) * scl[4 + t];
      if (sine && (i & 1)) val = -val;
      a.out[(size_t)r * n_out + i] = val;
    }
  } else {
    for (int idx = tid; idx < kTrPairs * L; idx += bd) {
      const int p = idx / L;
      const int nn = idx - p * L;
      const int src = makhoul_src(nn, L);
      double v[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = r0 + 2 * p + h;
        double x = (r < a.rows) ? a.in[(size_t)r * n_in + src] * scl[2 * p + h] : 0.0;
        if (sine && (src & 1)) x = -x;
        v[h] = x;
      }
      RA[idx] = make_double2(v[0], v[1]);
    }
    __syncthreads();
    C* Z = fft_rows<double, false>(RA, RB, kTrPairs, a.st, Wt);
    for (int idx = tid; idx < 2 * kTrPairs * n_out; idx += bd) {
      const int t = idx / n_out;
      const int s = idx - t * n_out;
      const int r = r0 + t;
      if (r >= a.rows) continue;
      double y = 0;
      if (!(sine && s == 0)) {
        const int k = sine ? L - s : s;
        const int p = t >> 1;
        const C Zk = Z[p * L + k];
        const C Zm = Z[p * L + ((L - k) % L)];
        const C e = Et[k];
        if ((t & 1) == 0)
          y = fma(e.x, Zk.x + Zm.x, e.y * (Zk.y - Zm.y));
        else
          y = fma(e.x, Zk.y + Zm.y, -(e.y * (Zk.x - Zm.x)));
        y *= ((!sine && k == 0) ? 1.0 / L : 2.0 / L) * scl[4 + t];
      }
      a.out[(size_t)r * n_out + s] = y;
    }
  }
}

// ---- F in state layout from the four spectral outputs (NLIN_FX/NLIN_DFX drop-ins) --------------
struct FinishArgs {
  int M, nr;
  const double* Dr;
  const double* out4;
  size_t out_stride;
  double* F;
  size_t f_stride;
};

__global__ void __launch_bounds__(kFxThreads) k_fx_finish(FinishArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* opr = reinterpret_cast<double*>(smem_raw);
  const int M = a.M, nr = a.nr, n = blockIdx.x, b = blockIdx.y;
  for (int m = threadIdx.x; m < nr; m += blockDim.x) opr[m] = a.Dr[n * nr + m];
  __syncthreads();
  const int N = M * nr;
  const double* O4 = a.out4 + (size_t)b * a.out_stride;
  double* F = a.F + (size_t)b * a.f_stride;
  for (int k = threadIdx.x; k < M; k += blockDim.x) {
    const double* qs = O4 + (size_t)k * nr;
    double q = 0;
    for (int m = 0; m < nr; ++m) q = fma(opr[m], qs[m], q);
    const size_t o = (size_t)k * nr + n;
    F[o] = q - O4[N + o];
    F[N + o] = O4[2 * N + o];
    F[2 * N + o] = O4[3 * N + o];
  }
}

// ---- launchers ---------------------------------------------------------------------------------
// The tensor-core contractions of a mixed launch (a.deriv_t): every state row of the batch at once.
static cudaError_t launch_tc_for(const FxArgs& a, int batch, cudaStream_t s) {
  TcArgs t;
  t.M = a.M; t.nr = a.nr; t.sym = a.sym; t.KP = a.tcKP; t.NP = a.tcNP;
  t.rows = batch * 3 * a.M;
  t.X32 = a.X32; t.x32_stride = a.x32_stride;
  t.X = a.X; t.x_stride = a.x_stride;
  t.active = a.active;
  t.B = a.tcB;
  t.out = reinterpret_cast<float*>(a.deriv);
  t.out_stride = a.deriv_stride;
  t.err = a.tc_err;
  return launch_deriv_tc(t, s);
}

// The most dynamic shared memory a k_fx_rows launch of precision prec can take: the opt-in limit less the
// kernel's static shared memory (the parity scans' chunk totals), over its three modes.
size_t fx_rows_max_dynamic_smem(int prec) {
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  size_t stat = 0;
  auto take = [&](const void* f) {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, f) == cudaSuccess) stat = fa.sharedSizeBytes > stat ? fa.sharedSizeBytes : stat;
    else cudaGetLastError();
  };
  if (prec == SDD_PREC_MIXED) {
    take(reinterpret_cast<const void*>(k_fx_rows<float, 0>));
    take(reinterpret_cast<const void*>(k_fx_rows<float, 1>));
    take(reinterpret_cast<const void*>(k_fx_rows<float, 2>));
  } else {
    take(reinterpret_cast<const void*>(k_fx_rows<double, 0>));
    take(reinterpret_cast<const void*>(k_fx_rows<double, 1>));
    take(reinterpret_cast<const void*>(k_fx_rows<double, 2>));
  }
  return (size_t)optin > stat ? (size_t)optin - stat : 0;
}

template <typename T, int MODE>
static cudaError_t launch_fx_t(const FxArgs& a, int batch, cudaStream_t s) {
  const size_t smem = fx_smem_bytes(a.M, a.P, sizeof(T) == 4 ? SDD_PREC_MIXED : SDD_PREC_FP64);
  static unsigned long long done = 0;
  cudaError_t e = ensure_smem_attr(k_fx_rows<T, MODE>, &done);
  if (e != cudaSuccess) return e;
  if (sizeof(T) == 4 && a.deriv_t && (e = launch_tc_for(a, batch, s)) != cudaSuccess) return e;
  e = launch_kernel(k_fx_rows<T, MODE>, dim3(a.nr, batch), dim3(kFxRowThreads), smem, s, a);
  ktimer_mark(SDD_K_FX_ROWS, s);
  return e;
}

template <typename T, int MODE>
static cudaError_t launch_fx_split_t(const FxArgs& a, int batch, cudaStream_t s) {
  const int prec = sizeof(T) == 4 ? SDD_PREC_MIXED : SDD_PREC_FP64;
  // grid rows go to the caller's cache when one is given (modes 0 and 2), else to the scratch
  T* grid = reinterpret_cast<T*>((MODE != 1 && a.base) ? a.base : a.grid);
  const size_t gs = (MODE != 1 && a.base) ? a.base_stride : a.grid_stride;
  cudaError_t e;
  {
    static unsigned long long done = 0;   // large nr with a pending correction can pass 48 KB
    if ((e = ensure_smem_attr(k_fx_deriv<T>, &done)) != cudaSuccess) return e;
  }
  // with tensor cores the per-mode kernel only applies a pending chain correction and forms the fused
  // right-hand side's FP64 block; the contractions follow on the corrected state
  const bool tc = sizeof(T) == 4 && a.deriv_t;
  if (!tc || a.fix.on || a.fuse_rhs) {
    // a pending correction's G blocks and terms are staged with the operators while the CTA still fits
    // twice on an SM (the per-mode CTAs of one shell outnumber the SMs)
    FxArgs ad = a;
    size_t sd = a.fix.on ? fix_stage_doubles(a.nr, a.fix.ldl, a.fix.nch) : 0;
    if (fx_deriv_smem_bytes(a.nr, prec, a.fix.on != 0, a.fuse_rhs != 0, sd) > kFxDerivStageMaxBytes) sd = 0;
    ad.fix.stage = sd > 0 ? 1 : 0;
    e = launch_kernel(k_fx_deriv<T>, dim3(a.M, batch), dim3(a.fix.on ? 384 : 256),
                      fx_deriv_smem_bytes(a.nr, prec, a.fix.on != 0, a.fuse_rhs != 0, sd), s, ad,
                      reinterpret_cast<T*>(a.deriv), a.deriv_stride);
    ktimer_mark(SDD_K_FX_DERIV, s);
    if (e != cudaSuccess) return e;
  }
  if (tc && (e = launch_tc_for(a, batch, s)) != cudaSuccess) return e;
  {
    static unsigned long long done = 0;
    if ((e = ensure_smem_attr(k_fx_grid<T>, &done)) != cudaSuccess) return e;
    e = launch_kernel(k_fx_grid<T>, dim3(a.nr, 5, batch), dim3(kFxSplitThreads), fx_grid_smem_bytes(a.M, a.P, prec),
                   s, a, grid, gs);
    ktimer_mark(SDD_K_FX_GRID, s);
    if (e != cudaSuccess || MODE == 2) return e;
  }
  constexpr int PM = MODE == 1 ? 1 : 0;
  static unsigned long long done = 0;
  if ((e = ensure_smem_attr(k_fx_prod<T, PM>, &done)) != cudaSuccess) return e;
  e = launch_kernel(k_fx_prod<T, PM>, dim3(a.nr, 2, batch), dim3(kFxSplitThreads), fx_prod_smem_bytes(a.P, prec), s,
                 a, (const T*)grid, gs);
  ktimer_mark(SDD_K_FX_PROD, s);
  return e;
}

static int fx_sm_count() {
  static const int sms = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
  return sms;
}

// The split path is taken when forced (split = 2) or, automatically, while the fused kernel would leave
// most SMs idle (nr * batch CTAs below half the SMs); it needs a grid scratch (or none: mode 2 and
// cached mode 0 write the cache).  A batch that shares the GPU with other launches (the captured
// multi-group graphs) is better served by the fused kernel; its autotuner sets the choice per plan.
bool fx_split_rule(int split, int nr, int batch) {
  if (split == 1) return false;
  return split == 2 || 2 * nr * batch <= fx_sm_count();
}

bool fx_uses_split(const FxArgs& a, int batch, int mode) {
  const bool has_grid = (mode != 1 && a.base) || a.grid;
  if (!has_grid || !a.deriv) return false;
  return fx_split_rule(a.split, a.nr, batch);
}

cudaError_t launch_fx(const FxArgs& a_in, int batch, int mode, int prec, cudaStream_t s) {
  FxArgs a = a_in;
  // mixed plans with tensor-core tables: the radial contractions go to k_deriv_tc (needs the deriv scratch)
  a.deriv_t = (prec == SDD_PREC_MIXED && a.tcB && a.deriv) ? 1 : 0;
  if (fx_uses_split(a, batch, mode)) {
    if (prec == SDD_PREC_MIXED) {
      if (mode == 0) return launch_fx_split_t<float, 0>(a, batch, s);
      if (mode == 1) return launch_fx_split_t<float, 1>(a, batch, s);
      return launch_fx_split_t<float, 2>(a, batch, s);
    }
    if (mode == 0) return launch_fx_split_t<double, 0>(a, batch, s);
    if (mode == 1) return launch_fx_split_t<double, 1>(a, batch, s);
    return launch_fx_split_t<double, 2>(a, batch, s);
  }
  if (prec == SDD_PREC_MIXED) {
    if (mode == 0) return launch_fx_t<float, 0>(a, batch, s);
    if (mode == 1) return launch_fx_t<float, 1>(a, batch, s);
    return launch_fx_t<float, 2>(a, batch, s);
  }
  if (mode == 0) return launch_fx_t<double, 0>(a, batch, s);
  if (mode == 1) return launch_fx_t<double, 1>(a, batch, s);
  return launch_fx_t<double, 2>(a, batch, s);
}

cudaError_t launch_rhs(const RhsArgs& a, int batch, cudaStream_t s) {
  if (a.rhs32) {   // needs X32, D2s32, Dr32 and (with a nonlinear term) q32
    if (!a.X32 || !a.D2s32 || !a.Dr32 || (!a.linear && !a.q32)) return cudaErrorInvalidValue;
    const size_t smem32 = (6 * (size_t)a.M + 2 * (size_t)a.nr) * sizeof(float);
    static unsigned long long done32 = 0;
    cudaError_t e = ensure_smem_attr(k_rhs32, &done32);
    if (e != cudaSuccess) return e;
    const cudaError_t er = launch_kernel(k_rhs32, dim3(a.nr, batch), dim3(kFxThreads), smem32, s, a);
    ktimer_mark(SDD_K_RHS, s);
    if (er != cudaSuccess) return er;
    return cudaGetLastError();
  }
  const size_t smem = (7 * (size_t)a.M + 3 + 2 * (size_t)a.nr) * sizeof(double);
  static unsigned long long done = 0;
  cudaError_t e = ensure_smem_attr(k_rhs, &done);
  if (e != cudaSuccess) return e;
  const cudaError_t er = launch_kernel(k_rhs, dim3(a.nr, batch), dim3(kFxThreads), smem, s, a);
  ktimer_mark(SDD_K_RHS, s);
  if (er != cudaSuccess) return er;
  return cudaGetLastError();
}

cudaError_t launch_theta_op(int op, int M, int nr, int sym, const double* D2, const double* ir,
                            const double* dT0, const double* g, double* f, int batch, cudaStream_t s) {
  ThetaArgs a{op, M, nr, sym, D2, ir, dT0, g, f};
  const size_t smem = (3 * (size_t)M + (size_t)nr) * sizeof(double);
  static unsigned long long done = 0;
  cudaError_t e = ensure_smem_attr(k_theta_op, &done);
  if (e != cudaSuccess) return e;
  k_theta_op<<<dim3(nr, batch), kFxThreads, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fx_finish(int M, int nr, const double* Dr, const double* out4, size_t out_stride,
                             double* F, size_t f_stride, int batch, cudaStream_t s) {
  FinishArgs a{M, nr, Dr, out4, out_stride, F, f_stride};
  k_fx_finish<<<dim3(nr, batch), kFxThreads, nr * sizeof(double), s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_transform(int kind, int rows, int n_in, int n_out, const FftPlan* fp,
                             const double* in, double* out, cudaStream_t s) {
  TrArgs a;
  a.kind = kind;
  a.rows = rows;
  a.n_in = n_in;
  a.n_out = n_out;
  a.L = fp->L;
  a.st = stage_args(fp);
  a.w = fp->w64;
  a.e = fp->e64;
  a.in = in;
  a.out = out;
  const size_t smem = (2 * kTrPairs + 2) * (size_t)fp->L * sizeof(double2) + (4 * 32 + 8) * 8;
  static unsigned long long done = 0;
  cudaError_t e = ensure_smem_attr(k_transform, &done);
  if (e != cudaSuccess) return e;
  const int grid = (rows + 2 * kTrPairs - 1) / (2 * kTrPairs);
  k_transform<<<grid, kFxThreads, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace sdd
