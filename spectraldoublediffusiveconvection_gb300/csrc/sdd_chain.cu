// Mode-coupled implicit solves: the back-substitution chains of
//   A4_BSub_TSTEP_V2   (Matrix_Operators.py:1115-1194)  -- psi: (A^2 - dt Pr A^4) psi = g
//   NAB2_BSub_TSTEP_V2 (Matrix_Operators.py:1033-1086)  -- T, S: (r^2 - dt r^2 Lap) f = g
// In the sin/cos basis each operator couples mode j to j+2, j+4, ... so a solve is two sequential
// chains (one per mode parity) of N_fm/2 steps.
//
// Restructured for a short critical path (exact algebra; checked against the reference formulation to
// ~3e-16):
//   h_j = Linv_j g_j for every mode first (k_hpre, all SMs in parallel, off the chains), then
//   psi:  f_j = h_j + A_j f_e + B_j bf_e,  A_j = Linv_j (dt bjt D2 + diag(alpha_j)),  B_j = Linv_j diag(beta_j),
//         alpha_j = dt bjt bj IR4 - bjt IR2,  beta_j = dt bjt IR4   (b_test of :1155, expanded)
//         f_e += f_j,  bf_e += bj f_j + bjt f_e   (:1153, :1159)
//   T, S: b += 2 dt (j+2) f_{j+2},  f_j = h_j - (j==0 ? 0.5 : 1) Linv_j b   (:1058-1083)
// so each chain step is ONE dependent matvec ([A_j B_j] over 2 nr columns, or Linv_j) plus three
// elementwise updates.
//
// Cost model (measured on GB300): an FP64 warp instruction occupies its SM sub-partition (SMSP) for 64
// cycles whatever the number of active lanes, and a dependent FP64 chain also advances one instruction
// per 64 cycles.  A chain is therefore bound by the FP64 warp-instructions each SMSP issues per step.
// Two layouts, picked by the launcher:
//   TPR = 4 (nr <= 32) or 2 (nr <= 64), 4 warps: every matrix row is split over TPR lanes and the rows
//     over 4 warps, one per SMSP.  Lowest latency for one chain on an otherwise idle SM.
//   TPR = 1, ceil(nr/32) warps: one lane per row, no reduction adds.  Fewest FP64 instructions per
//     chain, used when a batch puts several chains on every SM.
// Matrices are stored transposed (column c contiguous, leading dimension ldl); the block of step s+2
// streams global->shared with cp.async while step s runs (3-slot ring).  FP64 throughout.
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
  const double* h = a.g + (size_t)b * a.g_stride + foff;       // h_j = Linv_j g_j (k_hpre)
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

  const int ncol = a4 ? 2 * nr : nr;           // columns of the step matrix ([A B] or Linv)
  const int blk = ncol * ldl;
  double* Lb0 = csm;                           // 3-slot ring of step matrices
  double* hs = csm + 3 * blk;                  // the chain's h rows, step-ordered
  double* cf = hs + (size_t)nsteps * nr;       // per-step scalars (4 per step)
  double* x2 = cf + 4 * (size_t)nsteps;        // matvec operand: A4 [f_e; bf_e], NAB2 b
  const double* Mat = a4 ? a.ABA4 : (field == 1 ? a.LinvT : a.LinvS);
  const double* coef = a4 ? a.coefA4 : (field == 1 ? a.coefT : a.coefS);   // [M][4] indexed by jj

  copy_block(Lb0, Mat + (size_t)par * blk, blk);
  cp_async_commit();
  if (nsteps > 1) copy_block(Lb0 + blk, Mat + (size_t)(par + 2) * blk, blk);
  cp_async_commit();
  for (int e = tid; e < nsteps * nr; e += blockDim.x) {
    const int s = e / nr, c = e - s * nr;
    hs[e] = h[(size_t)(M - 1 - (par + 2 * s)) * nr + c];
  }
  for (int e = tid; e < 4 * nsteps; e += blockDim.x) cf[e] = coef[(size_t)(par + 2 * (e >> 2)) * 4 + (e & 3)];
  for (int c = tid; c < 2 * nr; c += blockDim.x) x2[c] = 0.0;
  __syncthreads();

  double fprev = 0.0;
  for (int s = 0; s < nsteps; ++s) {
    const int jj = par + 2 * s;
    const int row = M - 1 - jj;
    const double* cur = Lb0 + (s % 3) * blk;
    const double hi = hs[s * nr + ir];
    if (!a4) {   // b += 2 dt (j+2) f_{j+2}   (cf = (2 dt (j+2), 0.5 or 1, -, -))
      if (row < M - 2 && lead) x2[i] = fma(cf[4 * s], fprev, x2[i]);
    }
    if (s + 2 < nsteps) copy_block(Lb0 + ((s + 2) % 3) * blk, Mat + (size_t)(jj + 4) * blk, blk);
    cp_async_commit();
    cp_async_wait<2>();
    chain_sync();                              // block s landed; x2 of this step visible
    double fi;
    if (a4) {
      // f = h + [A B] [f_e; bf_e]   (cf = (dt bjt, dt bjt bj, bj, bjt)); the first step has f_e = bf_e = 0
      double acc = 0.0;
      if (s > 0)
        for (int c = q; c < ncol; c += TPR) acc = fma(cur[c * ldl + ir], x2[c], acc);
      fi = hi + group_sum<TPR>(acc);
    } else {
      double acc = 0.0;
      for (int c = q; c < nr; c += TPR) acc = fma(cur[c * ldl + ir], x2[c], acc);
      fi = fma(-cf[4 * s + 1], group_sum<TPR>(acc), hi);
    }
    chain_sync();                              // all lanes done reading x2 before it is updated
    if (lead) {
      f[(size_t)row * nr + i] = fi;
      if (a4) {
        const double bj = cf[4 * s + 2], bjt = cf[4 * s + 3];
        const double fe = x2[i];
        x2[nr + i] = fma(bj, fi, fma(bjt, fe, x2[nr + i]));   // bf_e += bj f + bjt f_e
        x2[i] = fe + fi;                                       // f_e += f (used from the next step on)
      }
    }
    fprev = fi;
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
  const size_t blk = (size_t)2 * nr * ldl;
  const size_t ns = (size_t)((M + 1) / 2);
  return (3 * blk + ns * nr + 4 * ns + 2 * (size_t)nr) * sizeof(double);
}

// h[field][row] = Linv_field[jj] g[field][row], row = M-1-jj, for all modes and the fields [field0,
// field0+nfields): one warp per (field, mode), lanes = rows, fully parallel over the GPU.
__global__ void k_hpre(ChainArgs a, int nfields) {
  const int warps = blockDim.x >> 5;
  const int wid = blockIdx.x * warps + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  const int M = a.M, nr = a.nr, ldl = a.ldl;
  if (wid >= nfields * M) return;
  const int fl = wid / M, jj = wid - fl * M;
  const int field = a.field0 + fl;
  const int b = blockIdx.y;
  const int row = M - 1 - jj;
  const size_t foff = (size_t)field * a.field_off;
  const double* g = a.g + (size_t)b * a.g_stride + foff + (size_t)row * nr;
  double* hout = a.h + (size_t)b * a.h_stride + foff + (size_t)row * nr;
  const double* L = (field == 0 ? a.LinvA4 : (field == 1 ? a.LinvT : a.LinvS)) + (size_t)jj * nr * ldl;
  for (int i = lane; i < nr; i += 32) {
    double acc = 0.0;
    for (int c = 0; c < nr; ++c) acc = fma(__ldg(L + (size_t)c * ldl + i), __ldg(g + c), acc);
    hout[i] = acc;
  }
}

// One CTA per chain.  When the batch leaves SMs idle (2*nfields*batch <= #SMs) the 4-warp split-row
// layout gives the shortest chain; otherwise the one-lane-per-row layout issues the fewest FP64
// instructions and several chains share every SM.  a.g holds the right-hand sides; a.h receives
// h = Linv g (k_hpre) and is what the chains read.
cudaError_t launch_chain(const ChainArgs& a_in, int batch, int nfields, cudaStream_t s) {
  ChainArgs a = a_in;
  const int hw = 4;
  k_hpre<<<dim3((nfields * a.M + hw - 1) / hw, batch), 32 * hw, 0, s>>>(a, nfields);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  a.g = a.h;
  a.g_stride = a.h_stride;
  const size_t smem = chain_smem_bytes(a.M, a.nr, a.ldl);
  static const int sms = [] {  // thread-safe one-time initialisation (host threads may launch concurrently)
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
  const dim3 grid(2 * nfields, batch);
  const bool split = a.layout == 4 || (a.layout == 0 && 2 * nfields * batch <= sms);
  if (split && a.nr <= 32) {
    static unsigned long long done = 0;
    if ((e = ensure_smem_attr(k_chain<4>, &done)) != cudaSuccess) return e;
    k_chain<4><<<grid, 128, smem, s>>>(a);
  } else if (split) {
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
