// Mode-coupled implicit solves: the back-substitution chains of
//   A4_BSub_TSTEP_V2   (Matrix_Operators.py:1115-1194)  -- psi: (A^2 - dt Pr A^4) psi = g
//   NAB2_BSub_TSTEP_V2 (Matrix_Operators.py:1033-1086)  -- T, S: (r^2 - dt r^2 Lap) f = g
// In the sin/cos basis each operator couples mode j to j+2, j+4, ... so a solve is two sequential
// chains (one per mode parity) of N_fm/2 steps; each step is a dense nr x nr matvec with a pre-inverted
// block (plus, for psi, one D2 matvec of the running sum f_e).
//
// One CTA per (shell, field, parity).  4 threads per matrix row (partial sums combined with two warp
// shuffles), 2 barriers per step.  The Linv block of step s+2 is copied global->shared with cp.async
// while step s runs (3-slot ring), so the L2 latency of the 7-18 KB blocks stays off the chain.
// FP64 throughout.
#include <cuda_runtime.h>
#include "sdd_internal.cuh"

namespace sdd {

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void copy_block(double* dst, const double* src, int ndouble) {
  const int nchunk = ndouble / 2;  // ndouble is even (ldl even)
  for (int c = threadIdx.x; c < nchunk; c += blockDim.x) cp_async16(dst + 2 * c, src + 2 * c);
}

// sum over the 4 threads of a row group
__device__ __forceinline__ double group4_sum(double v) {
  v += __shfl_xor_sync(0xffffffffu, v, 1);
  v += __shfl_xor_sync(0xffffffffu, v, 2);
  return v;
}

__global__ void k_chain(ChainArgs a) {
  extern __shared__ __align__(16) double csm[];
  const int field = a.field0 + (blockIdx.x >> 1);
  const int par = blockIdx.x & 1;  // first jj of the chain
  const int b = blockIdx.y;
  const int M = a.M, nr = a.nr, ldl = a.ldl;
  const bool a4 = (field == 0);
  const size_t foff = (size_t)field * a.field_off;
  const double* g = a.g + (size_t)b * a.g_stride + foff;
  double* f = a.f + (size_t)b * a.f_stride + foff;
  const double* sub = a.sub ? a.sub + (size_t)b * a.sub_stride + foff : nullptr;
  const int tid = threadIdx.x;
  const int i = tid >> 2, q = tid & 3;
  const bool row_ok = i < nr;
  const int nsteps = (M - par + 1) / 2;

  // symmetric: only the "evens" loops run (A4 jj = 0,2,..; NAB2 jj = 1,3,..); other rows stay 0.
  const bool active = !a.sym || (a4 ? par == 0 : par == 1);
  if (!active) {
    for (int s = 0; s < nsteps; ++s) {
      const int row = M - 1 - (par + 2 * s);
      for (int c = tid; c < nr; c += blockDim.x) f[(size_t)row * nr + c] = 0.0;
    }
    return;
  }

  const int blk = nr * ldl;
  double* Lb0 = csm;
  double* D2 = csm + 3 * blk;
  double* fe = D2 + (a4 ? nr * nr : 0);
  double* bfe = fe + nr;
  double* fprev = bfe + nr;
  double* w = fprev + nr;
  const double* Linv = a4 ? a.LinvA4 : (field == 1 ? a.LinvT : a.LinvS);

  copy_block(Lb0, Linv + (size_t)par * blk, blk);
  cp_async_commit();
  if (nsteps > 1) copy_block(Lb0 + blk, Linv + (size_t)(par + 2) * blk, blk);
  cp_async_commit();
  if (a4)
    for (int c = tid; c < nr * nr; c += blockDim.x) D2[c] = a.D2A4[c];
  for (int c = tid; c < nr; c += blockDim.x) {
    fe[c] = 0.0;
    bfe[c] = 0.0;
    fprev[c] = 0.0;
  }
  __syncthreads();

  const double ir2 = (a4 && row_ok) ? a.ir2A4[i] : 0.0;
  const double ir4 = (a4 && row_ok) ? a.ir4A4[i] : 0.0;
  const double dtc = a4 ? a.dtA4 : (field == 1 ? a.dtT : a.dtS);

  for (int s = 0; s < nsteps; ++s) {
    const int jj = par + 2 * s;
    const int row = M - 1 - jj;  // A4: row; NAB2: cosine mode j
    const double* cur = Lb0 + (s % 3) * blk;
    if (a4) {
      const double j = (double)(M - jj);
      const double bj = -j * (j + 1.0);
      const double bjt = -2.0 * j;
      const bool first = row >= M - 2;
      if (!first && q == 0 && row_ok) fe[i] += fprev[i];
      __syncthreads();
      if (s + 2 < nsteps) copy_block(Lb0 + ((s + 2) % 3) * blk, Linv + (size_t)(jj + 4) * blk, blk);
      cp_async_commit();
      double u = 0.0;
      if (!first && row_ok)
        for (int c = q; c < nr; c += 4) u += D2[i * nr + c] * fe[c];
      u = group4_sum(u);
      if (q == 0 && row_ok) {
        const double gi = g[(size_t)row * nr + i];
        if (first) {
          w[i] = gi;
        } else {
          const double L1f = u + bj * ir4 * fe[i];
          const double bt = dtc * bjt * (L1f + ir4 * bfe[i]) - bjt * ir2 * fe[i];
          w[i] = gi + bt;
        }
      }
      cp_async_wait<2>();
      __syncthreads();
      double y = 0.0;
      if (row_ok)
        for (int c = q; c < nr; c += 4) y += cur[i * ldl + c] * w[c];
      y = group4_sum(y);
      if (q == 0 && row_ok) {
        fprev[i] = y;
        f[(size_t)row * nr + i] = sub ? y - sub[(size_t)row * nr + i] : y;
        bfe[i] += first ? bj * y : bj * y + bjt * fe[i];
      }
    } else {
      const int j = row;
      if (q == 0 && row_ok) {
        if (j < M - 2) {
          double bk = -2.0 * (j + 2.0);
          bk = -dtc * bk;
          fe[i] += bk * fprev[i];  // fe holds b
        }
        const double gi = g[(size_t)j * nr + i];
        w[i] = (j == 0) ? gi - 0.5 * fe[i] : gi - fe[i];
      }
      if (s + 2 < nsteps) copy_block(Lb0 + ((s + 2) % 3) * blk, Linv + (size_t)(jj + 4) * blk, blk);
      cp_async_commit();
      cp_async_wait<2>();
      __syncthreads();
      double y = 0.0;
      if (row_ok)
        for (int c = q; c < nr; c += 4) y += cur[i * ldl + c] * w[c];
      y = group4_sum(y);
      if (q == 0 && row_ok) {
        fprev[i] = y;
        f[(size_t)j * nr + i] = sub ? y - sub[(size_t)j * nr + i] : y;
      }
      __syncthreads();
    }
  }
  cp_async_wait<0>();
}

cudaError_t launch_chain(const ChainArgs& a, int batch, int nfields, cudaStream_t s) {
  const int blk = a.nr * a.ldl;
  const size_t smem = (3 * (size_t)blk + (size_t)a.nr * a.nr + 4 * (size_t)a.nr) * sizeof(double);
  static unsigned long long done = 0;
  cudaError_t e = ensure_smem_attr(k_chain, &done);
  if (e != cudaSuccess) return e;
  const int threads = ((4 * a.nr + 31) / 32) * 32;
  k_chain<<<dim3(2 * nfields, batch), threads, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace sdd
