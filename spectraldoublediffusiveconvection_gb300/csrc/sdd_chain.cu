// Mode-coupled implicit solves: the back-substitution chains of
//   A4_BSub_TSTEP_V2   (Matrix_Operators.py:1115-1194)  -- psi: (A^2 - dt Pr A^4) psi = g
//   NAB2_BSub_TSTEP_V2 (Matrix_Operators.py:1033-1086)  -- T, S: (r^2 - dt r^2 Lap) f = g
// In the sin/cos basis each operator couples mode j to j+2, j+4, ... so a solve is two sequential
// chains (one per mode parity) of N_fm/2 steps; each step is a dense nr x nr matvec with a pre-inverted
// block (plus, for psi, one D2 matvec of the running sum f_e).
//
// Cost model (measured on GB300): an FP64 warp instruction occupies its SM sub-partition (SMSP) for 64
// cycles whatever the number of active lanes, and a dependent FP64 chain also advances one instruction
// per 64 cycles.  A chain is therefore bound by the FP64 warp-instructions each SMSP issues per step.
// Two layouts, picked by the launcher:
//   TPR = 4 (nr <= 32) or 2 (nr <= 64), 4 warps: every matrix row is split over TPR lanes and the rows
//     over 4 warps, one per SMSP; a matvec costs ~nr/TPR DFMA + log2(TPR) DADD per warp.  Lowest latency
//     for one chain on an otherwise idle SM (single shells, small batches).
//   TPR = 1, ceil(nr/32) warps: one lane per row, nr DFMA per matvec and no reduction adds.  Fewest FP64
//     instructions per chain, used when a batch puts several chains on every SM.
// Linv and D2 are stored transposed (column c contiguous, leading dimension ldl); the Linv block of step
// s+2 streams global->shared with cp.async while step s runs (3-slot ring); the chain's right-hand
// sides are staged in shared memory up front; per-step scalars come from a table built with the plan.
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

// sum over the TPR lanes of a row group (aligned groups inside one warp)
template <int TPR>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
  for (int off = 1; off < TPR; off <<= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}

// y_i = sum_c AT[c*ld + i] x[c] over the columns c = q (mod TPR) of the lane, then summed over the group.
// One accumulator: a dependent DFMA costs an SMSP the same 64 cycles as an independent one, so a second
// accumulator would only add a DADD.
template <int TPR>
__device__ __forceinline__ double col_dot(const double* AT, int ld, const double* x, int nr, int i, int q) {
  double s0 = 0.0;
  for (int c = q; c < nr; c += TPR) s0 = fma(AT[c * ld + i], x[c], s0);
  return group_sum<TPR>(s0);
}

__device__ __forceinline__ void chain_sync() {
  if (blockDim.x <= 32) __syncwarp();
  else __syncthreads();
}

template <int TPR>
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
  const int i = tid / TPR, q = tid % TPR;
  const bool row_ok = i < nr;
  const bool lead = row_ok && q == 0;     // the lane that owns row i's elementwise state
  const int ir = row_ok ? i : 0;
  const int nsteps = (M - par + 1) / 2;

  // symmetric: only the "evens" loops run (A4 jj = 0,2,..; NAB2 jj = 1,3,..); other rows stay 0.
  const bool active = !a.sym || (a4 ? par == 0 : par == 1);
  if (!active) {
    for (int e = tid; e < nsteps * nr; e += blockDim.x) {
      const int s = e / nr, c = e - s * nr;
      f[(size_t)(M - 1 - (par + 2 * s)) * nr + c] = 0.0;
    }
    return;
  }

  const int blk = nr * ldl;
  double* Lb0 = csm;
  double* D2 = csm + 3 * blk;                 // transposed, ld = ldl
  double* gs = D2 + (a4 ? blk : 0);           // the chain's right-hand sides, step-ordered
  double* cf = gs + (size_t)nsteps * nr;      // per-step scalars (4 per step)
  double* fe = cf + 4 * (size_t)nsteps;
  double* bfe = fe + nr;
  double* w = bfe + nr;
  const double* Linv = a4 ? a.LinvA4 : (field == 1 ? a.LinvT : a.LinvS);
  const double* coef = a4 ? a.coefA4 : (field == 1 ? a.coefT : a.coefS);   // [M][4] indexed by jj

  copy_block(Lb0, Linv + (size_t)par * blk, blk);
  cp_async_commit();
  if (nsteps > 1) copy_block(Lb0 + blk, Linv + (size_t)(par + 2) * blk, blk);
  cp_async_commit();
  if (a4) {
    copy_block(D2, a.D2A4, blk);
    cp_async_commit();
    cp_async_wait<0>();
  }
  for (int e = tid; e < nsteps * nr; e += blockDim.x) {
    const int s = e / nr, c = e - s * nr;
    gs[e] = g[(size_t)(M - 1 - (par + 2 * s)) * nr + c];
  }
  for (int e = tid; e < 4 * nsteps; e += blockDim.x) cf[e] = coef[(size_t)(par + 2 * (e >> 2)) * 4 + (e & 3)];
  for (int c = tid; c < nr; c += blockDim.x) {
    fe[c] = 0.0;
    bfe[c] = 0.0;
  }
  __syncthreads();

  const double ir2 = a4 ? a.ir2A4[ir] : 0.0;
  const double ir4 = a4 ? a.ir4A4[ir] : 0.0;
  double fprev = 0.0;

  for (int s = 0; s < nsteps; ++s) {
    const int jj = par + 2 * s;
    const int row = M - 1 - jj;
    const double* cur = Lb0 + (s % 3) * blk;
    const double gi = gs[s * nr + ir];
    if (a4) {
      // cf = (c1 = dt*bjt, k1 = c1*bj, bj, bjt) of sine mode j = M - jj
      const double c1 = cf[4 * s], k1 = cf[4 * s + 1], bj = cf[4 * s + 2], bjt = cf[4 * s + 3];
      const bool first = row >= M - 2;
      if (!first && lead) fe[i] += fprev;
      chain_sync();
      if (s + 2 < nsteps) copy_block(Lb0 + ((s + 2) % 3) * blk, Linv + (size_t)(jj + 4) * blk, blk);
      cp_async_commit();
      double wi = gi;
      if (!first) {
        // w = g + dt bjt ((D2 + bj IR4) f_e + IR4 bf_e) - bjt IR2 f_e      (Matrix_Operators.py:1155-1157)
        //   = g + c1 (D2 f_e) + IR4 (k1 f_e + c1 bf_e) - bjt IR2 f_e
        const double fei = fe[ir];
        const double t = fma(ir4, fma(k1, fei, c1 * bfe[ir]), fma(-bjt * ir2, fei, gi));
        const double u = col_dot<TPR>(D2, ldl, fe, nr, ir, q);
        wi = fma(c1, u, t);
      }
      if (lead) w[i] = wi;
      cp_async_wait<2>();
      chain_sync();
      const double bpre = fma(bjt, fe[ir], bfe[ir]);
      const double y = col_dot<TPR>(cur, ldl, w, nr, ir, q);
      if (lead) {
        fprev = y;
        f[(size_t)row * nr + i] = y;
        bfe[i] = fma(bj, y, first ? bfe[i] : bpre);
      }
    } else {
      // b += 2 dt (j+2) f_{j+2};  f_j = Linv (g_j - b), row j = 0 uses 0.5 b  (Matrix_Operators.py:1058-1083)
      // cf = (cb = 2 dt (j+2), hb = 0.5 for j == 0 else 1, -, -) of cosine mode j = M - 1 - jj
      const double cb = cf[4 * s], hb = cf[4 * s + 1];
      if (lead) {
        double bi = fe[i];                       // fe holds b
        if (row < M - 2) bi = fma(cb, fprev, bi);
        fe[i] = bi;
        w[i] = fma(-hb, bi, gi);
      }
      if (s + 2 < nsteps) copy_block(Lb0 + ((s + 2) % 3) * blk, Linv + (size_t)(jj + 4) * blk, blk);
      cp_async_commit();
      cp_async_wait<2>();
      chain_sync();
      const double y = col_dot<TPR>(cur, ldl, w, nr, ir, q);
      if (lead) {
        fprev = y;
        f[(size_t)row * nr + i] = y;
      }
      chain_sync();
    }
  }
  cp_async_wait<0>();
  if (sub) {  // Newton residual: f -= sub over the chain's rows (the block's own writes are visible)
    __syncthreads();
    for (int e = tid; e < nsteps * nr; e += blockDim.x) {
      const int s = e / nr, c = e - s * nr;
      const size_t o = (size_t)(M - 1 - (par + 2 * s)) * nr + c;
      f[o] -= sub[o];
    }
  }
}

size_t chain_smem_bytes(int M, int nr, int ldl) {
  const size_t blk = (size_t)nr * ldl;
  const size_t ns = (size_t)((M + 1) / 2);
  return (4 * blk + ns * nr + 4 * ns + 3 * (size_t)nr) * sizeof(double);
}

// One CTA per chain.  When the batch leaves SMs idle (2*nfields*batch <= #SMs) the 4-warp split-row
// layout gives the shortest chain; otherwise the one-lane-per-row layout issues the fewest FP64
// instructions and several chains share every SM.
cudaError_t launch_chain(const ChainArgs& a, int batch, int nfields, cudaStream_t s) {
  const size_t smem = chain_smem_bytes(a.M, a.nr, a.ldl);
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  const dim3 grid(2 * nfields, batch);
  cudaError_t e;
  if (2 * nfields * batch <= sms && a.nr <= 32) {
    static unsigned long long done = 0;
    if ((e = ensure_smem_attr(k_chain<4>, &done)) != cudaSuccess) return e;
    k_chain<4><<<grid, 128, smem, s>>>(a);
  } else if (2 * nfields * batch <= sms) {
    static unsigned long long done = 0;
    if ((e = ensure_smem_attr(k_chain<2>, &done)) != cudaSuccess) return e;
    k_chain<2><<<grid, 128, smem, s>>>(a);
  } else {
    static unsigned long long done = 0;
    if ((e = ensure_smem_attr(k_chain<1>, &done)) != cudaSuccess) return e;
    k_chain<1><<<grid, ((a.nr + 31) / 32) * 32, smem, s>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace sdd
