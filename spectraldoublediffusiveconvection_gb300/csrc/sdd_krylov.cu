// Device Krylov kernels for the matrix-free Newton-GMRES of Main.py:523-536 (the reference calls
// scipy.sparse.linalg.lgmres on a LinearOperator wrapping PDFX).  Here: restarted GMRES(m) with
// classical Gram-Schmidt, the pass repeated for a column only where the first one cancelled w below
// kReorthEta of its norm, FP64 throughout, one Krylov space per shell of a batch.
//
// Reductions are deterministic: every dot product is a fixed-order two-level sum (per-CTA partials over
// fixed element chunks, then a fixed-order sum of the partials), so a shell's result does not depend
// on the other shells in the batch.
//
// Vector layout: V[i][b][ld]: Krylov vector i of shell b has n used doubles at stride ld (n = 3*N_fm*nr
// for Newton, n+1 with the continuation parameter appended for the bordered arclength system).
//
// FP32 basis (the VT = float instances): the Krylov vectors are stored rounded to FP32 and the
// Gram-Schmidt products run in FP32 arithmetic (per-thread FP32 partial sums over a few elements, the
// cross-thread sums in FP64); w, the norms, the Hessenberg matrix and the rotations stay FP64.  For inner
// solves whose tolerance (relative 1e-4 in Newton) is far above FP32 rounding: the outer residual is FP64,
// so the converged state is unchanged in accuracy.  The FP64 products are bound by the FP64 multiply-add
// rate (one per element of V), the FP32 ones by the bytes of V, half as many.
#include <cuda_runtime.h>

#include <algorithm>

#include "sdd_krylov.cuh"

namespace sdd {

constexpr int kDotThreads = 256;

// part[(b*(nv) + i)*nchunk + c] = sum over chunk c of V_i[b] . w[b],  i < nv.
// The chunk of w sits in registers (kDotPer elements per thread); the vectors go kDotVecs at a time, so
// each thread has kDotVecs * kDotPer independent loads in flight and a block reduction serves kDotVecs
// dot products (the products are FP64-throughput bound on this GPU, about 5 TB/s of V).  Each partial is
// a fixed-order sum: per thread over its elements in index order, then the warp's transposed shuffle
// tree (warp_sum4), then the warps in order.
constexpr int kDotPer = kDotChunk / kDotThreads;
constexpr int kSubPer = kSubChunk / kDotThreads;
static_assert(kSubChunk % kDotThreads == 0, "update chunk must be a multiple of the block");
constexpr int kDotVecs = 4;
static_assert(kDotChunk % kDotThreads == 0, "dot chunk must be a multiple of the block");

// Warp sums of four values per lane in 6 FP64 additions per lane instead of 4 x 5: the first two shuffle
// levels exchange halves of the set (lanes with bit 4 set keep vectors 2-3, then lanes with bit 3 set
// keep the odd one), the last three are a plain tree.  Lanes 8v..8v+7 return the sum of vector v.
__device__ __forceinline__ double warp_sum4(const double (&sv)[4], int lane) {
  const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0;
  double k0 = h16 ? sv[2] : sv[0], k1 = h16 ? sv[3] : sv[1];
  const double s0 = h16 ? sv[0] : sv[2], s1 = h16 ? sv[1] : sv[3];
  k0 += __shfl_xor_sync(0xffffffffu, s0, 16);
  k1 += __shfl_xor_sync(0xffffffffu, s1, 16);
  double k = h8 ? k1 : k0;
  const double t = h8 ? k0 : k1;
  k += __shfl_xor_sync(0xffffffffu, t, 8);
  k += __shfl_xor_sync(0xffffffffu, k, 4);
  k += __shfl_xor_sync(0xffffffffu, k, 2);
  k += __shfl_xor_sync(0xffffffffu, k, 1);
  return k;
}

// warp_sum4 in FP32 (the FP32 basis's projections: conversions and FP64 additions hold the FP64 pipe, the
// FP32 ones do not); the same lane pattern.
__device__ __forceinline__ float warp_sum4f(const float (&sv)[4], int lane) {
  const bool h16 = (lane & 16) != 0, h8 = (lane & 8) != 0;
  float k0 = h16 ? sv[2] : sv[0], k1 = h16 ? sv[3] : sv[1];
  const float s0 = h16 ? sv[0] : sv[2], s1 = h16 ? sv[1] : sv[3];
  k0 += __shfl_xor_sync(0xffffffffu, s0, 16);
  k1 += __shfl_xor_sync(0xffffffffu, s1, 16);
  float k = h8 ? k1 : k0;
  const float t = h8 ? k0 : k1;
  k += __shfl_xor_sync(0xffffffffu, t, 8);
  k += __shfl_xor_sync(0xffffffffu, k, 4);
  k += __shfl_xor_sync(0xffffffffu, k, 2);
  k += __shfl_xor_sync(0xffffffffu, k, 1);
  return k;
}

// The last CTA of a shell to finish (ticket[b], one counter per shell, zero between launches) sums the
// shell's partials in chunk order and writes h: the reduction of k_dot_reduce, without its launch.
__device__ __forceinline__ bool last_chunk_of_shell(int* ticket, int b, int nblocks) {
  __shared__ int s_last;
  __syncthreads();                                   // this CTA's partials are written
  if (threadIdx.x == 0) {
    __threadfence();
    const int last = atomicAdd(ticket + b, 1) == nblocks - 1;
    if (last) {
      __threadfence();
      ticket[b] = 0;                                 // ready for the next launch
    }
    s_last = last;
  }
  __syncthreads();
  return s_last != 0;
}

__device__ __forceinline__ void reduce_partials(const double* part, int b, int nv, int nchunk, double* h, int ldh,
                                                int accumulate) {
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    double t = 0.0;
    const volatile double* p = part + ((size_t)b * nv + i) * nchunk;
    for (int c = 0; c < nchunk; ++c) t += p[c];
    if (accumulate) h[(size_t)b * ldh + i] += t;
    else h[(size_t)b * ldh + i] = t;
  }
}

// blockIdx.z selects the vectors [z vpb, (z+1) vpb) of the CTA (vpb a multiple of kDotVecs): small batches
// spread the vectors over more CTAs; every partial is summed the same way whatever the split.
template <typename VT>
__global__ void __launch_bounds__(kDotThreads) k_dot_partials(const VT* __restrict__ V, size_t vstride_i,
                                                             const double* __restrict__ w, int n, int ld, int nv,
                                                             int chunk, double* part,
                                                             const int* __restrict__ active, int* ticket,
                                                             double* h, int ldh, int accumulate, int vpb) {
  __shared__ double red[kDotVecs][kDotThreads / 32];
  const int c = blockIdx.x, b = blockIdx.y, nchunk = gridDim.x;
  const int ib = blockIdx.z * vpb, ie = min(nv, ib + vpb);
  if (active && !active[b]) {                         // skipped shell: zero partials (its results are unused)
    for (int i = ib + threadIdx.x; i < ie; i += blockDim.x) part[((size_t)b * nv + i) * nchunk + c] = 0.0;
  } else {
    const int e0 = c * chunk;
    const double* wb = w + (size_t)b * ld;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    VT wr[kDotPer];
#pragma unroll
    for (int k = 0; k < kDotPer; ++k) {
      const int e = e0 + threadIdx.x + k * kDotThreads;
      wr[k] = e < n ? (VT)wb[e] : (VT)0;
    }
    for (int i0 = ib; i0 < ie; i0 += kDotVecs) {
      VT sp[kDotVecs];
#pragma unroll
      for (int u = 0; u < kDotVecs; ++u) {
        sp[u] = (VT)0;
        if (i0 + u < ie) {
          const VT* vb = V + (size_t)(i0 + u) * vstride_i + (size_t)b * ld;
#pragma unroll
          for (int k = 0; k < kDotPer; ++k) {
            const int e = e0 + threadIdx.x + k * kDotThreads;
            if (e < n) sp[u] = fma(vb[e], wr[k], sp[u]);
          }
        }
      }
      static_assert(kDotVecs == 4, "warp_sum4 reduces four vectors");
      double ws;
      if constexpr (sizeof(VT) == 4) {
        ws = (double)warp_sum4f(sp, lane);             // the warp's 256 products in FP32, then FP64
      } else {
        ws = warp_sum4(sp, lane);
      }
      if ((lane & 7) == 0) red[lane >> 3][warp] = ws;
      __syncthreads();
      if (threadIdx.x < kDotVecs && i0 + threadIdx.x < ie) {
        double t = 0.0;
        for (int q = 0; q < kDotThreads / 32; ++q) t += red[threadIdx.x][q];
        part[((size_t)b * nv + i0 + threadIdx.x) * nchunk + c] = t;
      }
      __syncthreads();
    }
  }
  if (ticket && last_chunk_of_shell(ticket, b, nchunk * gridDim.z))
    reduce_partials(part, b, nv, nchunk, h, ldh, accumulate);
}

// w[b] -= sum_{i<nv} V_i[b] coef[b*ldc + i] for the shells with sub_mask[b] (per element, the products summed
// in index order), then nrm2[b] = |w[b]|^2 for the shells with norm_mask[b] (0 for the others): per thread over its elements
// in index order, the warp tree of k_dot_partials, the warps in order, the chunks of kSubChunk elements in
// order.  The chunks are a quarter of the dot products' (the update's dependent multiply-adds over the
// basis dominate, so one shell's update spreads over four times the CTAs).  With reo != nullptr the shell's
// last CTA also sets the second-pass flag of column j: active and |w'|^2 < eta^2 (|w'|^2 + |h|^2), where
// |w|^2 = |w'|^2 + |h|^2 for an orthonormal basis.
template <typename VT>
__global__ void __launch_bounds__(kDotThreads) k_sub_norm(const VT* __restrict__ V, size_t vstride_i, double* w,
                                                         const double* __restrict__ coef, int ldc, int n, int ld,
                                                         int nv, const int* __restrict__ sub_mask,
                                                         const int* __restrict__ norm_mask, double* part,
                                                         int* ticket, double* nrm2, GmresState gs, int j,
                                                         double eta2, int set_reo) {
  __shared__ double red[kDotVecs][kDotThreads / 32];
  __shared__ VT cs[kMaxRestart + 1];                   // the coefficients in the basis's precision
  const int c = blockIdx.x, b = blockIdx.y, nchunk = gridDim.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int e0 = c * kSubChunk;
  double* wb = w + (size_t)b * ld;
  const bool sub = !sub_mask || sub_mask[b];
  const bool nrm = !norm_mask || norm_mask[b];
  const double* cb = coef + (size_t)b * ldc;
  for (int i = threadIdx.x; i < nv && i <= kMaxRestart; i += blockDim.x) cs[i] = (VT)cb[i];
  __syncthreads();
  double sv[kDotVecs] = {0.0, 0.0, 0.0, 0.0};
  // per element the products summed in index order; the thread's elements side by side, so that their
  // loads of one basis vector are in flight together
  VT t[kSubPer];
#pragma unroll
  for (int k = 0; k < kSubPer; ++k) t[k] = (VT)0;
  if (sub) {
    const VT* vb = V + (size_t)b * ld + e0 + threadIdx.x;
    const int kmax = min(kSubPer, max(0, (n - e0 - (int)threadIdx.x + kDotThreads - 1) / kDotThreads));
    if (kmax == kSubPer) {
#pragma unroll 4
      for (int i = 0; i < nv; ++i) {
#pragma unroll
        for (int k = 0; k < kSubPer; ++k) t[k] += vb[(size_t)i * vstride_i + k * kDotThreads] * cs[i];
      }
    } else {
      for (int i = 0; i < nv; ++i)
        for (int k = 0; k < kmax; ++k) t[k] += vb[(size_t)i * vstride_i + k * kDotThreads] * cs[i];
    }
  }
#pragma unroll
  for (int k = 0; k < kSubPer; ++k) {
    const int e = e0 + threadIdx.x + k * kDotThreads;
    if (e < n) {
      double x = wb[e];
      if (sub) {
        x -= (double)t[k];
        wb[e] = x;
      }
      if (nrm) sv[0] = fma(x, x, sv[0]);
    }
  }
  const double ws = warp_sum4(sv, lane);
  if ((lane & 7) == 0) red[lane >> 3][warp] = ws;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < kDotThreads / 32; ++q) t += red[0][q];
    part[(size_t)b * nchunk + c] = nrm ? t : 0.0;
  }
  if (last_chunk_of_shell(ticket, b, nchunk) && threadIdx.x == 0) {
    double t = 0.0;
    const volatile double* p = part + (size_t)b * nchunk;
    for (int q = 0; q < nchunk; ++q) t += p[q];
    nrm2[b] = t;
    if (set_reo) {
      int r = 0;
      if (gs.active[b]) {
        const double* hc = gs.hcol + (size_t)b * (gs.m + 1);
        double h2 = 0.0;
        for (int i = 0; i <= j; ++i) h2 = fma(hc[i], hc[i], h2);
        r = t < eta2 * (t + h2) ? 1 : 0;
      }
      gs.reo[b] = r;
    }
  }
}

// h[b*ldh + i] (+)= sum_c part[(b*nv+i)*nchunk + c]
__global__ void k_dot_reduce(const double* __restrict__ part, int nv, int nchunk, double* __restrict__ h,
                             int ldh, int accumulate) {
  const int b = blockIdx.x;
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    double t = 0.0;
    const double* p = part + ((size_t)b * nv + i) * nchunk;
    for (int c = 0; c < nchunk; ++c) t += p[c];
    if (accumulate) h[(size_t)b * ldh + i] += t;
    else h[(size_t)b * ldh + i] = t;
  }
}

// x[b] += sum_{i<k_b} V_i[b] * y[b*ldy + i]  (the sum in the basis's precision)
template <typename VT>
__global__ void k_add_combination(const VT* __restrict__ V, size_t vstride_i, double* __restrict__ x,
                                  const double* __restrict__ y, int ldy, const int* __restrict__ kb, int n,
                                  int ld) {
  __shared__ VT ys[kMaxRestart];
  const int b = blockIdx.y;
  const int k = min(kb[b], kMaxRestart);
  const double* yb = y + (size_t)b * ldy;
  for (int i = threadIdx.x; i < k; i += blockDim.x) ys[i] = (VT)yb[i];
  __syncthreads();
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    VT s = (VT)0;
    for (int i = 0; i < k; ++i) s += V[(size_t)i * vstride_i + (size_t)b * ld + e] * ys[i];
    x[(size_t)b * ld + e] += (double)s;
  }
}

// out[b] = a[b] * scale[b]  (scale may be per shell); out32 / out2 (nullable): FP32 and FP64 copies
__global__ void k_scale(const double* __restrict__ a, const double* __restrict__ scale, double* __restrict__ out,
                        int n, int ld, float* __restrict__ out32, double* __restrict__ out2) {
  const int b = blockIdx.y;
  const double s = scale[b];
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const double v = a[(size_t)b * ld + e] * s;
    out[(size_t)b * ld + e] = v;
    if (out32) out32[(size_t)b * ld + e] = (float)v;
    if (out2) out2[(size_t)b * ld + e] = v;
  }
}

// FP32 basis: out[b] = fl32(a[b] * scale[b]); out32 (nullable) the same FP32 values, out2 (nullable) them
// in FP64 (the vector the next product reads is exactly the stored basis vector)
__global__ void k_scale_to32(const double* __restrict__ a, const double* __restrict__ scale, float* __restrict__ out,
                             int n, int ld, float* __restrict__ out32, double* __restrict__ out2) {
  const int b = blockIdx.y;
  const double s = scale[b];
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const float v = (float)(a[(size_t)b * ld + e] * s);
    out[(size_t)b * ld + e] = v;
    if (out32) out32[(size_t)b * ld + e] = v;
    if (out2) out2[(size_t)b * ld + e] = (double)v;
  }
}

// out[e] = (double)in[e]
__global__ void k_widen(const float* __restrict__ in, double* __restrict__ out, size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    out[e] = (double)in[e];
}

// out = a - b
__global__ void k_sub(const double* __restrict__ a, const double* __restrict__ bb, double* __restrict__ out,
                      size_t n) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    out[e] = a[e] - bb[e];
}

// X[b] (stride ldx) -= dx[b] (stride ld) where mask[b] != 0
__global__ void k_masked_sub(double* __restrict__ X, const double* __restrict__ dx, const int* __restrict__ mask,
                             int n, int ldx, int ld) {
  const int b = blockIdx.y;
  if (!mask[b]) return;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x)
    X[(size_t)b * ldx + e] -= dx[(size_t)b * ld + e];
}

// Start of a GMRES cycle.  nrm2[b] = ||r_b||^2.  Sets beta, g = [beta,0..], inv = 1/beta, and the
// per-shell activity flag (active while the shell is being solved and beta is above its target).
__global__ void k_cycle_start(GmresState s, const double* __restrict__ nrm2, int B) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const double beta = sqrt(nrm2[b]);
  s.beta[b] = beta;
  double* g = s.g + (size_t)b * (s.m + 1);
  for (int i = 0; i <= s.m; ++i) g[i] = 0.0;
  g[0] = beta;
  const int act = s.solve[b] && beta > s.target[b] && beta > 0.0;
  s.active[b] = act;
  s.kb[b] = 0;
  s.inv[b] = (act && beta > 0.0) ? 1.0 / beta : 0.0;
  s.resid[b] = beta;
}

// After Gram-Schmidt for column j: hcol + h2 [b][0..j] hold the projections, nrm2[b] = ||w||^2.  Stores the
// column in H, applies the previous Givens rotations, makes the new one, updates g and the residual estimate.
__global__ void __launch_bounds__(32) k_arnoldi_finish(GmresState s, const double* __restrict__ nrm2, int j,
                                                        int B) {
  // one warp per shell: the lanes stage the column (hcol + h2) and the previous rotations in shared memory,
  // lane 0 applies the rotations (the rotated entry of row i + 1 carried in a register, the only dependent
  // chain) and makes the new one, the lanes write the column back
  __shared__ double col[kMaxRestart + 1], csv[kMaxRestart], snv[kMaxRestart];
  const int b = blockIdx.x, lane = threadIdx.x;
  if (b >= B) return;
  const int m = s.m;
  double* H = s.H + (size_t)b * (m + 1) * m;   // H[row*m + col]
  const double* hc = s.hcol + (size_t)b * (m + 1);
  const double* hd = s.h2 + (size_t)b * (m + 1);
  double* cs = s.cs + (size_t)b * m;
  double* sn = s.sn + (size_t)b * m;
  double* g = s.g + (size_t)b * (m + 1);
  if (!s.active[b]) {
    if (lane == 0) s.inv[b] = 0.0;
    return;
  }
  for (int i = lane; i <= j; i += 32) col[i] = hc[i] + hd[i];
  for (int i = lane; i < j; i += 32) {
    csv[i] = cs[i];
    snv[i] = sn[i];
  }
  __syncwarp();
  if (lane == 0) {
    const double hnext = sqrt(nrm2[b]);
    double a = col[0];
    for (int i = 0; i < j; ++i) {
      const double c = col[i + 1];
      col[i] = fma(csv[i], a, snv[i] * c);
      a = fma(-snv[i], a, csv[i] * c);
    }
    const double c = hnext;
    const double r = hypot(a, c);
    double cj = 1.0, sj = 0.0;
    if (r > 0.0) {
      cj = a / r;
      sj = c / r;
    }
    cs[j] = cj;
    sn[j] = sj;
    H[j * m + j] = r;
    H[(j + 1) * m + j] = 0.0;
    g[j + 1] = -sj * g[j];
    g[j] = cj * g[j];
    const double res = fabs(g[j + 1]);
    s.resid[b] = res;
    s.kb[b] = j + 1;
    const bool breakdown = !(hnext > 1e-300 * s.beta[b]);
    int act = 1;
    if (res <= s.target[b] || breakdown || j + 1 == m) act = 0;
    s.active[b] = act;
    s.inv[b] = (act && hnext > 0.0) ? 1.0 / hnext : 0.0;
  }
  __syncwarp();
  for (int i = lane; i < j; i += 32) H[i * m + j] = col[i];
}

// Back substitution R y = g over the first kb[b] columns.
__global__ void k_solve_y(GmresState s, int B) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const int m = s.m, k = s.kb[b];
  const double* H = s.H + (size_t)b * (m + 1) * m;
  const double* g = s.g + (size_t)b * (m + 1);
  double* y = s.y + (size_t)b * m;
  for (int i = k - 1; i >= 0; --i) {
    double t = g[i];
    for (int c = i + 1; c < k; ++c) t -= H[i * m + c] * y[c];
    const double d = H[i * m + i];
    y[i] = d != 0.0 ? t / d : 0.0;
  }
}

// ---- pseudo-arclength continuation helpers (Main.py:829-837, 910-917) ------------------------------
// g[b][k][n] = dtPr * (-(k+1)) gr[n] T[b][k+1][n] for k < M-1, 0 for k = M-1: the psi right-hand side of
// PDFmu (kGR_RT applied to T, Matrix_Operators.py:97-128); symmetric plans drop the odd T slots.
__global__ void k_grk_T(const double* __restrict__ X, int ldx, double* __restrict__ g, int M, int nr,
                        const double* __restrict__ gr, double dtPr, int sym) {
  const int b = blockIdx.y;
  const int N = M * nr;
  const double* T = X + (size_t)b * ldx + N;
  double* gb = g + (size_t)b * 3 * N;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 3 * N; e += gridDim.x * blockDim.x) {
    double v = 0.0;
    if (e < N) {
      const int k = e / nr, n = e - k * nr;
      if (k < M - 1 && !(sym && ((k + 1) & 1))) v = dtPr * ((-(double)(k + 1) * gr[n]) * T[(size_t)(k + 1) * nr + n]);
    }
    gb[e] = v;
  }
}

// out[b][0..N) += v[b][n] * Jmu[b][0..N)  (psi block; Jmu stride ldj);  out[b][n] = delta*dot[b] + (1-delta)*mudot[b]*v[b][n]
__global__ void k_border(const double* __restrict__ v, double* __restrict__ out, int n, int ld,
                         const double* __restrict__ Jmu, int ldj, int Npsi, const double* __restrict__ dot,
                         const double* __restrict__ mudot, double delta) {
  const int b = blockIdx.y;
  const double vl = v[(size_t)b * ld + n];
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < Npsi; e += gridDim.x * blockDim.x)
    out[(size_t)b * ld + e] += vl * Jmu[(size_t)b * ldj + e];
  if (blockIdx.x == 0 && threadIdx.x == 0) out[(size_t)b * ld + n] = delta * dot[b] + (1.0 - delta) * mudot[b] * vl;
}

// dst[b][e] (stride ldd) = a * src[b][e] (stride lds), e < n; optionally dst[b][n] = last[b]
__global__ void k_copy_scaled(const double* __restrict__ src, int lds, double* __restrict__ dst, int ldd, int n,
                              double a, const double* __restrict__ last) {
  const int b = blockIdx.y;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x)
    dst[(size_t)b * ldd + e] = a * src[(size_t)b * lds + e];
  if (last && blockIdx.x == 0 && threadIdx.x == 0) dst[(size_t)b * ldd + n] = last[b];
}

// y[b] (stride ldy) = x0[b] (stride ldx0) + c[b] * d[b] (stride ldd), e < n
__global__ void k_axpy_shell(const double* __restrict__ x0, int ldx0, const double* __restrict__ d, int ldd,
                             const double* __restrict__ c, double* __restrict__ y, int ldy, int n) {
  const int b = blockIdx.y;
  const double cb = c[b];
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x)
    y[(size_t)b * ldy + e] = x0[(size_t)b * ldx0 + e] + cb * d[(size_t)b * ldd + e];
}

// ---- host wrappers ------------------------------------------------------------------------------
static int grid_x(int n) {
  int g = (n + 255) / 256;
  return g < 1 ? 1 : (g > 1024 ? 1024 : g);
}

static int sm_count_dev() {
  static int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

template <typename VT>
static cudaError_t krylov_dots_t(const VT* V, size_t vstride_i, const double* w, int n, int ld, int nv, int B,
                                 double* part, double* h, int ldh, int accumulate, cudaStream_t st, const int* active,
                                 int* ticket) {
  const int nchunk = (n + kDotChunk - 1) / kDotChunk;
  // with the one-launch reduction, spread the vectors over CTAs until the launch has ~2 CTAs per SM
  int nvg = 1;
  if (ticket) {
    const int want = (2 * sm_count_dev() + B * nchunk - 1) / (B * nchunk);
    nvg = std::max(1, std::min((nv + kDotVecs - 1) / kDotVecs, want));
  }
  int vpb = (nv + nvg - 1) / nvg;
  vpb = (vpb + kDotVecs - 1) / kDotVecs * kDotVecs;
  nvg = (nv + vpb - 1) / vpb;
  k_dot_partials<VT><<<dim3(nchunk, B, nvg), kDotThreads, 0, st>>>(V, vstride_i, w, n, ld, nv, kDotChunk, part,
                                                                   active, ticket, h, ldh, accumulate, vpb);
  if (!ticket) k_dot_reduce<<<B, 64, 0, st>>>(part, nv, nchunk, h, ldh, accumulate);
  return cudaGetLastError();
}
cudaError_t krylov_dots(const double* V, size_t vstride_i, const double* w, int n, int ld, int nv, int B,
                        double* part, double* h, int ldh, int accumulate, cudaStream_t st, const int* active,
                        int* ticket) {
  return krylov_dots_t(V, vstride_i, w, n, ld, nv, B, part, h, ldh, accumulate, st, active, ticket);
}
cudaError_t krylov_dots(const float* V, size_t vstride_i, const double* w, int n, int ld, int nv, int B,
                        double* part, double* h, int ldh, int accumulate, cudaStream_t st, const int* active,
                        int* ticket) {
  return krylov_dots_t(V, vstride_i, w, n, ld, nv, B, part, h, ldh, accumulate, st, active, ticket);
}

template <typename VT>
static cudaError_t krylov_sub_norm_t(const VT* V, size_t vstride_i, double* w, const double* coef, int ldc, int n,
                                     int ld, int nv, int B, const int* sub_mask, const int* norm_mask, double* part,
                                     int* ticket, double* nrm2, const GmresState* reo_of, int j, double eta,
                                     cudaStream_t st) {
  if (!ticket || nv > kMaxRestart + 1) return cudaErrorInvalidValue;
  const int nchunk = (n + kSubChunk - 1) / kSubChunk;
  GmresState gs{};
  if (reo_of) gs = *reo_of;
  k_sub_norm<VT><<<dim3(nchunk, B), kDotThreads, 0, st>>>(V, vstride_i, w, coef, ldc, n, ld, nv, sub_mask, norm_mask,
                                                          part, ticket, nrm2, gs, j, eta * eta, reo_of ? 1 : 0);
  return cudaGetLastError();
}
cudaError_t krylov_sub_norm(const double* V, size_t vstride_i, double* w, const double* coef, int ldc, int n, int ld,
                            int nv, int B, const int* sub_mask, const int* norm_mask, double* part, int* ticket,
                            double* nrm2, const GmresState* reo_of, int j, double eta, cudaStream_t st) {
  return krylov_sub_norm_t(V, vstride_i, w, coef, ldc, n, ld, nv, B, sub_mask, norm_mask, part, ticket, nrm2, reo_of,
                           j, eta, st);
}
cudaError_t krylov_sub_norm(const float* V, size_t vstride_i, double* w, const double* coef, int ldc, int n, int ld,
                            int nv, int B, const int* sub_mask, const int* norm_mask, double* part, int* ticket,
                            double* nrm2, const GmresState* reo_of, int j, double eta, cudaStream_t st) {
  return krylov_sub_norm_t(V, vstride_i, w, coef, ldc, n, ld, nv, B, sub_mask, norm_mask, part, ticket, nrm2, reo_of,
                           j, eta, st);
}

cudaError_t krylov_add_combination(const double* V, size_t vstride_i, double* x, const double* y, int ldy,
                                   const int* kb, int n, int ld, int B, cudaStream_t st) {
  k_add_combination<double><<<dim3(grid_x(n), B), 256, 0, st>>>(V, vstride_i, x, y, ldy, kb, n, ld);
  return cudaGetLastError();
}
cudaError_t krylov_add_combination(const float* V, size_t vstride_i, double* x, const double* y, int ldy,
                                   const int* kb, int n, int ld, int B, cudaStream_t st) {
  k_add_combination<float><<<dim3(grid_x(n), B), 256, 0, st>>>(V, vstride_i, x, y, ldy, kb, n, ld);
  return cudaGetLastError();
}

cudaError_t krylov_scale(const double* a, const double* scale, double* out, int n, int ld, int B, cudaStream_t st,
                         float* out32, double* out2) {
  k_scale<<<dim3(grid_x(n), B), 256, 0, st>>>(a, scale, out, n, ld, out32, out2);
  return cudaGetLastError();
}
cudaError_t krylov_scale(const double* a, const double* scale, float* out, int n, int ld, int B, cudaStream_t st,
                         float* out32, double* out2) {
  k_scale_to32<<<dim3(grid_x(n), B), 256, 0, st>>>(a, scale, out, n, ld, out32, out2);
  return cudaGetLastError();
}

cudaError_t krylov_widen(const float* in, double* out, size_t n, cudaStream_t st) {
  k_widen<<<grid_x((int)(n > (1u << 30) ? (1u << 30) : n)), 256, 0, st>>>(in, out, n);
  return cudaGetLastError();
}

cudaError_t krylov_sub(const double* a, const double* b, double* out, size_t n, cudaStream_t st) {
  k_sub<<<grid_x((int)(n > (1u << 30) ? (1u << 30) : n)), 256, 0, st>>>(a, b, out, n);
  return cudaGetLastError();
}

cudaError_t krylov_masked_sub(double* X, const double* dx, const int* mask, int n, int ldx, int ld, int B,
                              cudaStream_t st) {
  k_masked_sub<<<dim3(grid_x(n), B), 256, 0, st>>>(X, dx, mask, n, ldx, ld);
  return cudaGetLastError();
}

cudaError_t krylov_cycle_start(const GmresState& s, const double* nrm2, int B, cudaStream_t st) {
  k_cycle_start<<<(B + 63) / 64, 64, 0, st>>>(s, nrm2, B);
  return cudaGetLastError();
}

cudaError_t krylov_arnoldi_finish(const GmresState& s, const double* nrm2, int j, int B, cudaStream_t st) {
  if (s.m > kMaxRestart || j >= s.m) return cudaErrorInvalidValue;
  k_arnoldi_finish<<<B, 32, 0, st>>>(s, nrm2, j, B);
  return cudaGetLastError();
}

cudaError_t contin_grk_T(const double* X, int ldx, double* g, int M, int nr, const double* gr, double dtPr, int sym,
                         int B, cudaStream_t st) {
  k_grk_T<<<dim3(grid_x(3 * M * nr), B), 256, 0, st>>>(X, ldx, g, M, nr, gr, dtPr, sym);
  return cudaGetLastError();
}

cudaError_t contin_border(const double* v, double* out, int n, int ld, const double* Jmu, int ldj, int Npsi,
                          const double* dot, const double* mudot, double delta, int B, cudaStream_t st) {
  k_border<<<dim3(grid_x(Npsi), B), 256, 0, st>>>(v, out, n, ld, Jmu, ldj, Npsi, dot, mudot, delta);
  return cudaGetLastError();
}

cudaError_t krylov_copy_scaled(const double* src, int lds, double* dst, int ldd, int n, double a, const double* last,
                               int B, cudaStream_t st) {
  k_copy_scaled<<<dim3(grid_x(n), B), 256, 0, st>>>(src, lds, dst, ldd, n, a, last);
  return cudaGetLastError();
}

cudaError_t krylov_axpy_shell(const double* x0, int ldx0, const double* d, int ldd, const double* c, double* y,
                              int ldy, int n, int B, cudaStream_t st) {
  k_axpy_shell<<<dim3(grid_x(n), B), 256, 0, st>>>(x0, ldx0, d, ldd, c, y, ldy, n);
  return cudaGetLastError();
}

cudaError_t krylov_solve_y(const GmresState& s, int B, cudaStream_t st) {
  k_solve_y<<<(B + 63) / 64, 64, 0, st>>>(s, B);
  return cudaGetLastError();
}

}  // namespace sdd
