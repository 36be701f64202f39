// Mode-coupled implicit solves: the back-substitution chains of
//   A4_BSub_TSTEP_V2   (Matrix_Operators.py:1115-1194)  -- psi: (A^2 - dt Pr A^4) psi = g
//   NAB2_BSub_TSTEP_V2 (Matrix_Operators.py:1033-1086)  -- T, S: (r^2 - dt r^2 Lap) f = g
// In the sin/cos basis each operator couples mode j to j+2, j+4, ... so a solve is two sequential
// chains (one per mode parity) of N_fm/2 steps.
//
// Restructured for a short critical path (exact algebra; checked against the reference formulation to
// ~3e-16):
//   h_j = Linv_j g_j for every mode first (k_mode_mv, all SMs in parallel, off the chains), then
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
// Layouts, picked by the launcher:
//   TPR = 4 (nr <= 32) or 2 (nr <= 64), 4 warps: every matrix row is split over TPR lanes and the rows
//     over 4 warps, one per SMSP.  Lowest latency for one chain on an otherwise idle SM.
//   TPR = 1, ceil(nr/32) warps: one lane per row, no reduction adds.  Fewest FP64 instructions per
//     chain, used when a batch puts several chains on every SM.
//   chunked (layouts 2 and 3): the S = N_fm/2 steps of a chain are cut into nch chunks of kc steps that
//     run concurrently, each from a zero carried state (its own CTA; h = Linv g from k_mode_mv).  The
//     chain's carried state s (psi: [f_e; bf_e], 2 nr; T/S: b, nr) enters every later step linearly, so
//     with the plan's precomputed Phi_c (state over a whole chunk) and G_jj (state -> f_jj):
//       layout 2: s_1 = d_0,  s_{c+1} = Phi_c s_c + d_c   (carry_run, by the chain's last-finishing chunk CTA)
//       layout 3: s_c = d_{c-1} + sum_{i<=c-2} P_{c,i} d_i, P_{c,i} = Phi_{c-1}...Phi_{i+1} precomputed,
//                 every product at once (k_carry_par), the row sums in the corrections
//       f_jj += G_jj s_c(jj)                    (k_mode_mv, all modes in parallel)
//     The critical path drops from S dependent steps to kc + (nch - 2) carried matvecs + one matvec
//     (layout 2), or kc steps + one product + one matvec (layout 3, shorter chunks).
// Matrices are stored transposed (column c contiguous, leading dimension ldl); the block of step s+2
// streams global->shared with cp.async while step s runs (3-slot ring).  FP64 throughout.
#include <cuda_runtime.h>
#include <algorithm>

#include "sdd_internal.cuh"

namespace sdd {

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
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

__device__ __forceinline__ void chain_sync() {
  if (blockDim.x <= 32) __syncwarp();
  else __syncthreads();
}

// g of mode `row` for the fused right-hand side, element n (see ChainArgs::fuse_rhs): the roundings of
// k_rhs, psi: (-dt (Dr Q - R)) + lin, T: (-dt NT) + lin, S: (-dt NS) + lin.
// Dr and the Q row may be given in shared memory (Drs: nr x nr row-major, Qs: nr); nullptr reads global.
__device__ __forceinline__ double fused_g(const ChainArgs& a, int b, int field, int row, int n,
                                         const double* Drs = nullptr, const double* Qs = nullptr) {
  const int M = a.M, nr = a.nr;
  const size_t N = (size_t)M * nr;
  const double* o4 = a.out4 + (size_t)b * a.out_stride;
  double nl;
  if (field == 0) {
    double dq = 0.0;
    if (a.q32) {            // FP32 nonlinear term: Dr Q in FP32, the order of k_rhs
      const float* qs = a.q32 + (size_t)b * M * nr + (size_t)row * nr;
      const float* drn = a.Dr32 + (size_t)n * nr;
      float d = 0.0f;
      for (int c = 0; c < nr; ++c) d = fmaf(__ldg(drn + c), __ldg(qs + c), d);
      dq = (double)d;
    } else {
      const double* qs = Qs ? Qs : o4 + (size_t)row * nr;
      const double* drn = (Drs ? Drs : a.Dr) + (size_t)n * nr;
      for (int c = 0; c < nr; ++c) dq = fma(drn[c], qs[c], dq);
    }
    nl = __dmul_rn(-a.dt, __dsub_rn(dq, o4[N + (size_t)row * nr + n]));
  } else {
    nl = __dmul_rn(-a.dt, o4[(size_t)(field + 1) * N + (size_t)row * nr + n]);
  }
  return __dadd_rn(nl, a.lin[(size_t)b * a.g_stride + (size_t)field * a.field_off + (size_t)row * nr + n]);
}

// One chain (field, parity) of one shell: steps [s0, s1) of the S = (M - par + 1)/2 chain steps.
// CHUNK = false: the whole chain (s0 = 0, s1 = S).  CHUNK = true: chunk blockIdx.z of a.kc steps,
// started from a zero carried state; its end state goes to dbuf (psi: [f_e; bf_e]; T/S: b + k_next f_last,
// the b the next chunk's first step uses).  Both read h = Linv g (k_mode_mv) through a.g.
template <int TPR, int R>
__device__ void carry_run(const ChainArgs& a, int field, int par, int b, double* csm);

template <int TPR, bool CHUNK, int CR = 0>
__global__ void k_chain(ChainArgs a) {
  extern __shared__ __align__(16) double csm[];
  const int field = a.field0 + (blockIdx.x >> 1);
  const int par = blockIdx.x & 1;  // first jj of the chain
  const int b = blockIdx.y;
  if (a.active && !a.active[b]) return;
  const int M = a.M, nr = a.nr, ldl = a.ldl;
  const bool a4 = (field == 0);
  const size_t foff = (size_t)field * a.field_off;
  double* f = a.f + (size_t)b * a.f_stride + foff;
  const double* sub = a.sub ? a.sub + (size_t)b * a.sub_stride + foff : nullptr;
  const int tid = threadIdx.x;
  const int i = tid / TPR, q = tid % TPR;
  const bool row_ok = i < nr;
  const bool lead = row_ok && q == 0;     // the lane that owns row i's elementwise state
  const int ir = row_ok ? i : 0;
  const int S = (M - par + 1) / 2;
  const int chunk = CHUNK ? (int)blockIdx.z : 0;
  const int s0 = CHUNK ? chunk * a.kc : 0;
  const int s1 = CHUNK ? min(S, s0 + a.kc) : S;
  if (s0 >= S) return;
  const int nsteps = s1 - s0;
  double* dout = CHUNK ? a.dbuf + (size_t)b * a.d_stride + ((size_t)(field * 2 + par) * a.nch + chunk) * a.ldd
                       : nullptr;

  // symmetric: only the "evens" loops run (A4 jj = 0,2,..; NAB2 jj = 1,3,..); other rows stay 0.
  const bool active = !a.sym || (a4 ? par == 0 : par == 1);
  float* f32 = a.f32 ? a.f32 + (size_t)b * a.f32_stride + foff : nullptr;   // final values only (no sub)
  if (!active) {
    for (int e = tid; e < nsteps * nr; e += blockDim.x) {
      const int s = e / nr, c = e - s * nr;
      f[(size_t)(M - 1 - (par + 2 * (s0 + s))) * nr + c] = 0.0;
      if (f32) f32[(size_t)(M - 1 - (par + 2 * (s0 + s))) * nr + c] = 0.0f;
    }
    if (CHUNK)
      for (int e = tid; e < a.ldd; e += blockDim.x) dout[e] = 0.0;
    return;
  }

  const int ncol = a4 ? 2 * nr : nr;           // columns of the step matrix ([A B] or Linv)
  const int blk = ncol * ldl;
  double* Lb0 = csm;                           // 3-slot ring of step matrices
  double* cf = csm + 3 * blk;                  // per-step scalars (4 per step, one step past the chunk)
  double* x2 = cf + 4 * (size_t)(nsteps + 1);  // 2 buffers of the matvec operand: A4 [f_e; bf_e], NAB2 b
  const double* Mat = a4 ? a.ABA4 : (field == 1 ? a.LinvT : a.LinvS);
  const double* coef = a4 ? a.coefA4 : (field == 1 ? a.coefT : a.coefS);   // [M][4] indexed by jj
  const int jj0 = par + 2 * s0;

  copy_block(Lb0, Mat + (size_t)jj0 * blk, blk);
  cp_async_commit();
  if (nsteps > 1) copy_block(Lb0 + blk, Mat + (size_t)(jj0 + 2) * blk, blk);
  cp_async_commit();
  for (int e = tid; e < 4 * (nsteps + 1); e += blockDim.x) {
    const int jj = jj0 + 2 * (e >> 2);
    cf[e] = jj < M ? coef[(size_t)jj * 4 + (e & 3)] : 0.0;
  }
  for (int c = tid; c < 4 * nr; c += blockDim.x) x2[c] = 0.0;
  // h_j = Linv_j g_j (k_mode_mv) of row ir, two steps ahead in registers (off the chain's critical path;
  // no shared-memory copy of the chain's h rows, so long chains leave room for other CTAs on the SM)
  const double* hrow = a.g + (size_t)b * a.g_stride + foff + ir;
  auto h_at = [&](int s) { return s < nsteps ? hrow[(size_t)(M - 1 - (par + 2 * (s0 + s))) * nr] : 0.0; };
  double hn0 = h_at(0), hn1 = h_at(1);

  // The lead lane of row i keeps the row's carried state in registers and publishes it to the other
  // buffer of x2 for the next step's matvec: one barrier per step.
  //   psi:  f = h + [A B] [f_e; bf_e];  f_e += f,  bf_e += bj f + bjt f_e   (cf = (dt bjt, dt bjt bj, bj, bjt))
  //   T/S:  f = h - w Linv b;  then b += k' f with k' = 2 dt (j'+2) of the next step   (cf = (k, w, -, -))
  double fe = 0.0, bfe = 0.0;                  // psi: f_e_i, bf_e_i;  T/S: b_i in fe
  for (int s = 0; s < nsteps; ++s) {
    const int jj = jj0 + 2 * s;
    const int row = M - 1 - jj;
    const double* cur = Lb0 + (s % 3) * blk;
    const double* xs = x2 + (s & 1) * 2 * nr;
    double* xn = x2 + ((s + 1) & 1) * 2 * nr;
    cp_async_wait<1>();
    chain_sync();                              // block s landed; this step's x2 visible; step s-1 done
    if (s + 2 < nsteps) copy_block(Lb0 + ((s + 2) % 3) * blk, Mat + (size_t)(jj + 4) * blk, blk);
    cp_async_commit();
    const double hi = hn0;
    hn0 = hn1;
    hn1 = h_at(s + 2);
    double fi;
    if (a4) {
      const double pre = fma(cf[4 * s + 3], fe, bfe);   // bf_e + bjt f_e, off the matvec's path
      double acc = (q == 0) ? hi : 0.0;
      if (TPR == 1) {                          // one lane per row: two interleaved partial sums
        double acc1 = 0.0;
        if (s > 0) {
          int c = 0;
#pragma unroll 4
          for (; c + 1 < ncol; c += 2) {
            acc = fma(cur[c * ldl + ir], xs[c], acc);
            acc1 = fma(cur[(c + 1) * ldl + ir], xs[c + 1], acc1);
          }
          if (c < ncol) acc = fma(cur[c * ldl + ir], xs[c], acc);
        }
        acc += acc1;
      } else if (s > 0) {
#pragma unroll 8
        for (int c = q; c < ncol; c += TPR) acc = fma(cur[c * ldl + ir], xs[c], acc);
      }
      fi = group_sum<TPR>(acc);
      fe += fi;
      bfe = fma(cf[4 * s + 2], fi, pre);
      if (lead) {
        xn[i] = fe;
        xn[nr + i] = bfe;
      }
    } else {
      double acc = 0.0;
      if (TPR == 1) {                          // one lane per row: two interleaved partial sums
        double acc1 = 0.0;
        int c = 0;
#pragma unroll 4
        for (; c + 1 < nr; c += 2) {
          acc = fma(cur[c * ldl + ir], xs[c], acc);
          acc1 = fma(cur[(c + 1) * ldl + ir], xs[c + 1], acc1);
        }
        if (c < nr) acc = fma(cur[c * ldl + ir], xs[c], acc);
        acc += acc1;
      } else {
#pragma unroll 8
        for (int c = q; c < nr; c += TPR) acc = fma(cur[c * ldl + ir], xs[c], acc);
      }
      fi = fma(-cf[4 * s + 1], group_sum<TPR>(acc), hi);
      fe = fma(cf[4 * (s + 1)], fi, fe);       // the b of the next step (of the next chunk after the last)
      if (lead) xn[i] = fe;
    }
    if (lead) {
      f[(size_t)row * nr + i] = fi;
      if (f32 && chunk == 0) f32[(size_t)row * nr + i] = (float)fi;   // later chunks: final after the correction
    }
  }
  cp_async_wait<0>();
  if (CHUNK && chunk + 1 < a.nch && lead) {    // end state of the chunk from a zero start
    dout[i] = fe;
    if (a4) dout[nr + i] = bfe;
  }
  if (sub) {  // Newton residual: f -= sub over the chunk's rows (the block's own writes are visible)
    __syncthreads();
    for (int e = tid; e < nsteps * nr; e += blockDim.x) {
      const int s = e / nr, c = e - s * nr;
      const size_t o = (size_t)(M - 1 - (par + 2 * (s0 + s))) * nr + c;
      f[o] -= sub[o];
    }
  }
  if (CHUNK && a.nch > 2 && a.carry_seq) {
    // the last chunk of this chain to finish runs the carried-state recurrence (no extra launch)
    __shared__ int s_last;
    __syncthreads();                                   // this chunk's end state before the ticket (see k_carry_par)
    int* cnt = a.counter + (size_t)b * 6 + (field * 2 + par);
    if (tid == 0) {
      __threadfence();
      const int last = atomicAdd(cnt, 1) == a.nch - 1;
      if (last) {
        __threadfence();
        *cnt = 0;                                      // ready for the next launch
      }
      s_last = last;
    }
    __syncthreads();
    if (!s_last) return;
    carry_run<(TPR == 4 ? 2 : 1), CR>(a, field, par, b, csm);
  } else if (CHUNK && a.nch == 2 && a.carry_seq) {    // s_1 = d_0 only: the chain's first chunk copies it
    if (chunk == 0 && lead) {
      double* cb = a.cbuf + (size_t)b * a.d_stride + ((size_t)(field * 2 + par) * a.nch + 1) * a.ldd;
      cb[i] = fe;
      if (a4) cb[nr + i] = bfe;
    }
  }
}

// Layouts 10 and 11: the chunked chains of layouts 2 and 3 with each chunk in the reference's order of
// operations (the step of ref_chain below: per psi step D2 f_e, then Linv_j (g_j + b); per T/S step
// Linv_j (g_j - w b)), so that no h = Linv g pre-pass runs: each chunk starts from a zero carried state
// exactly as in layouts 2 and 3 (the carried state [f_e; bf_e] or b is the same quantity), writes the same
// end state (psi: f_e after its last f, bf_e), and the same carries and corrections follow.  g is the full
// right-hand side, or with fuse_rhs formed by the CTA itself before its chain from the linear parts and the
// nonlinear-term outputs (fused_g, the roundings of k_rhs: the same bits), so that the single shell's step
// needs no right-hand-side kernel either.  One CTA per (field, parity, chunk, shell), rows over TPR lanes.
template <int TPR, int CR>
__global__ void k_chain_cref(ChainArgs a) {
  extern __shared__ __align__(16) double csm[];
  const int field = a.field0 + (blockIdx.x >> 1);
  const int par = blockIdx.x & 1;
  const int b = blockIdx.y;
  if (a.active && !a.active[b]) return;
  const int M = a.M, nr = a.nr, ldl = a.ldl;
  const bool a4 = (field == 0);
  const size_t foff = (size_t)field * a.field_off;
  double* f = a.f + (size_t)b * a.f_stride + foff;
  const double* sub = a.sub ? a.sub + (size_t)b * a.sub_stride + foff : nullptr;
  const int tid = threadIdx.x;
  const int i = tid / TPR, q = tid % TPR;
  const bool row_ok = i < nr;
  const bool lead = row_ok && q == 0;
  const int ir = row_ok ? i : 0;
  const int S = (M - par + 1) / 2;
  const int chunk = (int)blockIdx.z;
  const int s0 = chunk * a.kc;
  const int s1 = min(S, s0 + a.kc);
  if (s0 >= S) return;
  const int nsteps = s1 - s0;
  double* dout = a.dbuf + (size_t)b * a.d_stride + ((size_t)(field * 2 + par) * a.nch + chunk) * a.ldd;
  const bool active = !a.sym || (a4 ? par == 0 : par == 1);
  float* f32 = a.f32 ? a.f32 + (size_t)b * a.f32_stride + foff : nullptr;   // final values only (no sub)
  if (!active) {
    for (int e = tid; e < nsteps * nr; e += blockDim.x) {
      const int st = e / nr, c = e - st * nr;
      f[(size_t)(M - 1 - (par + 2 * (s0 + st))) * nr + c] = 0.0;
      if (f32) f32[(size_t)(M - 1 - (par + 2 * (s0 + st))) * nr + c] = 0.0f;
    }
    for (int e = tid; e < a.ldd; e += blockDim.x) dout[e] = 0.0;
    return;
  }
  const int blk = nr * ldl;
  double* Lb0 = csm;                                   // 3-slot ring of Linv blocks
  double* D2s = Lb0 + 3 * blk;                         // psi: D2 (transposed)
  double* cf = D2s + (a4 ? blk : 0);                   // per-step scalars, 4 per step, one step past the chunk
  double* xv = cf + 4 * (size_t)(nsteps + 1);          // 2 buffers of f_e (psi)
  double* yv = xv + 2 * nr;                            // 2 buffers of the Linv matvec's operand
  double* gs = yv + 2 * nr;                            // fuse_rhs: g of the chunk's steps, then Dr (psi)
  double* Drs = gs + (size_t)nsteps * nr;
  const bool stage_dr = a.fuse_rhs && a4 && !a.q32;
  const double* Mat = a4 ? a.LinvA4 : (field == 1 ? a.LinvT : a.LinvS);
  const double* coef = a4 ? a.coefA4 : (field == 1 ? a.coefT : a.coefS);
  const int jj0 = par + 2 * s0;
  copy_block(Lb0, Mat + (size_t)jj0 * blk, blk);
  if (a4) copy_block(D2s, a.D2A4, blk);
  if (stage_dr)
    for (int e = tid; e < nr * nr; e += blockDim.x) cp_async8(Drs + e, a.Dr + e);
  cp_async_commit();
  if (nsteps > 1) copy_block(Lb0 + blk, Mat + (size_t)(jj0 + 2) * blk, blk);
  cp_async_commit();
  for (int e = tid; e < 4 * (nsteps + 1); e += blockDim.x) {
    const int jj = jj0 + 2 * (e >> 2);
    cf[e] = jj < M ? coef[(size_t)jj * 4 + (e & 3)] : 0.0;
  }
  const double ir4 = a4 ? a.ir4A4[ir] : 0.0, ir2 = a4 ? a.ir2A4[ir] : 0.0;
  if (a.fuse_rhs) {
    if (stage_dr) cp_async_wait<1>();                  // Dr landed (with the first Linv block and D2)
    __syncthreads();
    for (int e = tid; e < nsteps * nr; e += blockDim.x) {
      const int st = e / nr, n = e - st * nr;
      gs[e] = fused_g(a, b, field, M - 1 - (par + 2 * (s0 + st)), n, stage_dr ? Drs : nullptr);
    }
    __syncthreads();
  }
  const double* grow = a.g + (size_t)b * a.g_stride + foff + ir;
  auto g_at = [&](int st) {
    if (st >= nsteps) return 0.0;
    return a.fuse_rhs ? gs[st * nr + ir] : grow[(size_t)(M - 1 - (par + 2 * (s0 + st))) * nr];
  };
  double gn0 = g_at(0), gn1 = g_at(1);
  double fe = 0.0, bfe = 0.0, fprev = 0.0;             // psi: f_e_i, bf_e_i; T/S: b_i in fe
  for (int st = 0; st < nsteps; ++st) {
    const int jj = jj0 + 2 * st;
    const int row = M - 1 - jj;
    const double* cur = Lb0 + (st % 3) * blk;
    double* yb = yv + (st & 1) * nr;
    cp_async_wait<1>();
    chain_sync();                                      // Linv_jj (and D2) landed; step st-1 done
    if (st + 2 < nsteps) copy_block(Lb0 + ((st + 2) % 3) * blk, Mat + (size_t)(jj + 4) * blk, blk);
    cp_async_commit();
    const double gi = gn0;
    gn0 = gn1;
    gn1 = g_at(st + 2);
    if (a4) {
      const double bj = cf[4 * st + 2], bjt = cf[4 * st + 3], c1 = cf[4 * st];
      double y = gi;
      if (st > 0) {
        fe += fprev;                                   // f_e += f_{j+2}
        double* xb = xv + (st & 1) * nr;
        if (lead) xb[i] = fe;
        chain_sync();
        double z = 0.0;
#pragma unroll 8
        for (int c = q; c < nr; c += TPR) z = fma(D2s[c * ldl + ir], xb[c], z);
        z = group_sum<TPR>(z);
        const double L1f = fma(bj * ir4, fe, z);      // (D2 + bj IR4) f_e
        const double tt = fma(ir4, bfe, L1f);          // + IR4 bf_e
        const double bt = fma(c1, tt, -(bjt * ir2 * fe));
        y = gi + bt;
      }
      if (lead) yb[i] = y;
      chain_sync();
      double acc = 0.0;
#pragma unroll 8
      for (int c = q; c < nr; c += TPR) acc = fma(cur[c * ldl + ir], yb[c], acc);
      const double fi = group_sum<TPR>(acc);
      bfe = st > 0 ? fma(bj, fi, fma(bjt, fe, bfe)) : fma(bj, fi, bfe);
      fprev = fi;
      if (lead) {
        f[(size_t)row * nr + i] = fi;
        if (f32 && chunk == 0) f32[(size_t)row * nr + i] = (float)fi;   // later chunks: after the correction
      }
    } else {
      const double y = fma(-cf[4 * st + 1], fe, gi);  // g - w b
      if (lead) yb[i] = y;
      chain_sync();
      double acc = 0.0;
#pragma unroll 8
      for (int c = q; c < nr; c += TPR) acc = fma(cur[c * ldl + ir], yb[c], acc);
      const double fi = group_sum<TPR>(acc);
      fe = fma(cf[4 * (st + 1)], fi, fe);             // the b of the next step (of the next chunk after the last)
      if (lead) {
        f[(size_t)row * nr + i] = fi;
        if (f32 && chunk == 0) f32[(size_t)row * nr + i] = (float)fi;
      }
    }
  }
  cp_async_wait<0>();
  if (a4) fe += fprev;                                 // the carried f_e after the chunk's last f
  if (chunk + 1 < a.nch && lead) {                     // end state of the chunk from a zero start
    dout[i] = fe;
    if (a4) dout[nr + i] = bfe;
  }
  if (sub) {  // Newton residual: f -= sub over the chunk's rows (the block's own writes are visible)
    __syncthreads();
    for (int e = tid; e < nsteps * nr; e += blockDim.x) {
      const int st = e / nr, c = e - st * nr;
      const size_t o = (size_t)(M - 1 - (par + 2 * (s0 + st))) * nr + c;
      f[o] -= sub[o];
    }
  }
  if (a.nch > 2 && a.carry_seq) {
    // the last chunk of this chain to finish runs the carried-state recurrence (no extra launch)
    __shared__ int s_last;
    __syncthreads();
    int* cnt = a.counter + (size_t)b * 6 + (field * 2 + par);
    if (tid == 0) {
      __threadfence();
      const int last = atomicAdd(cnt, 1) == a.nch - 1;
      if (last) {
        __threadfence();
        *cnt = 0;                                      // ready for the next launch
      }
      s_last = last;
    }
    __syncthreads();
    if (!s_last) return;
    carry_run<(TPR == 4 ? 2 : 1), CR>(a, field, par, b, csm);
  } else if (a.nch == 2 && a.carry_seq) {              // s_1 = d_0 only: the chain's first chunk copies it
    if (chunk == 0 && lead) {
      double* cb = a.cbuf + (size_t)b * a.d_stride + ((size_t)(field * 2 + par) * a.nch + 1) * a.ldd;
      cb[i] = fe;
      if (a4) cb[nr + i] = bfe;
    }
  }
}

// Layouts 6, 7 and 8: the chains in the reference's own order of operations, without the h = Linv g pre-pass:
//   psi (Matrix_Operators.py:1139-1164):  f_e += f_{j+2};  L1f = D2 f_e + bj IR4 f_e;
//          b = dt bjt (L1f + IR4 bf_e) - bjt IR2 f_e;  f_j = Linv_j (g_j + b);  bf_e += bj f_j + bjt f_e
//   T, S (Matrix_Operators.py:1056-1083):  b += 2 dt (j+2) f_{j+2};  f_j = Linv_j (g_j - w b)
// Per mode 4 nr^2 multiply-adds instead of the 7 nr^2 of the pre-pass form (h, then [A B] for psi and
// Linv b for T/S), at the price of a second dependent matvec per psi step: the form for batches that fill
// the GPU, where the FP64 work and not a chain's latency sets the time.  g is the full right-hand side (not
// the fused form).
//
// ref_chain runs one chain (field, parity) of shell b on `nt` threads (whole warps) of a CTA, thread t of
// them, rows split over TPR lanes, synchronising on named barrier `bar` (nt > 32) or the warp; its own
// shared memory `sm` (ref_group_doubles): a 3-slot cp.async ring of Linv blocks, D2 (psi), the per-step
// scalars and two operand buffers.  Every cp.async of the chain is issued and waited for by the chain's own
// threads, so chains sharing a CTA never wait on one another.
__device__ __forceinline__ void group_sync(int bar, int nt) {
  if (nt <= 32) __syncwarp();
  else asm volatile("bar.sync %0, %1;\n" ::"r"(bar), "r"(nt) : "memory");
}

__device__ __forceinline__ void copy_block_g(double* dst, const double* src, int ndouble, int t, int nt) {
  const int nchunk = ndouble / 2;  // ndouble is even (ldl even)
  for (int c = t; c < nchunk; c += nt) cp_async16(dst + 2 * c, src + 2 * c);
}

__host__ __device__ inline size_t ref_group_doubles(int M, int nr, int ldl, bool a4) {
  const size_t blk = (size_t)nr * ldl;
  const size_t ns = (size_t)((M + 1) / 2);
  return (a4 ? 4 : 3) * blk + 4 * (ns + 1) + (a4 ? 4 : 2) * (size_t)nr;
}

template <int TPR>
__device__ __forceinline__ void ref_chain(const ChainArgs& a, int field, int par, int b, int t, int nt, int bar,
                                          double* sm) {
  const int M = a.M, nr = a.nr, ldl = a.ldl;
  const bool a4 = (field == 0);
  const size_t foff = (size_t)field * a.field_off;
  double* f = a.f + (size_t)b * a.f_stride + foff;
  const double* sub = a.sub ? a.sub + (size_t)b * a.sub_stride + foff : nullptr;
  float* f32 = a.f32 ? a.f32 + (size_t)b * a.f32_stride + foff : nullptr;
  const int i = t / TPR, q = t % TPR;
  const bool row_ok = i < nr;
  const bool lead = row_ok && q == 0;
  const int ir = row_ok ? i : 0;
  const int S = (M - par + 1) / 2;
  if (a.sym && !(a4 ? par == 0 : par == 1)) {          // symmetric: the other parity's rows are zero
    for (int e = t; e < S * nr; e += nt) {
      const int st = e / nr, c = e - st * nr;
      f[(size_t)(M - 1 - (par + 2 * st)) * nr + c] = 0.0;
      if (f32) f32[(size_t)(M - 1 - (par + 2 * st)) * nr + c] = 0.0f;
    }
    return;
  }
  const int blk = nr * ldl;
  double* Lb0 = sm;                                    // 3-slot ring of Linv blocks
  double* D2s = Lb0 + 3 * blk;                         // psi: D2 (transposed), nr x ldl
  double* cf = D2s + (a4 ? blk : 0);                   // per-step scalars, 4 per step
  double* xv = cf + 4 * (size_t)(S + 1);               // 2 buffers of f_e (psi)
  double* yv = xv + (a4 ? 2 * nr : 0);                 // 2 buffers of the Linv matvec's operand
  const double* Mat = a4 ? a.LinvA4 : (field == 1 ? a.LinvT : a.LinvS);
  const double* coef = a4 ? a.coefA4 : (field == 1 ? a.coefT : a.coefS);
  copy_block_g(Lb0, Mat + (size_t)par * blk, blk, t, nt);
  if (a4) copy_block_g(D2s, a.D2A4, blk, t, nt);
  cp_async_commit();
  if (S > 1) copy_block_g(Lb0 + blk, Mat + (size_t)(par + 2) * blk, blk, t, nt);
  cp_async_commit();
  for (int e = t; e < 4 * (S + 1); e += nt) {
    const int jj = par + 2 * (e >> 2);
    cf[e] = jj < M ? coef[(size_t)jj * 4 + (e & 3)] : 0.0;
  }
  const double ir4 = a4 ? a.ir4A4[ir] : 0.0, ir2 = a4 ? a.ir2A4[ir] : 0.0;
  const double* grow = a.g + (size_t)b * a.g_stride + foff + ir;
  auto g_at = [&](int st) { return st < S ? grow[(size_t)(M - 1 - (par + 2 * st)) * nr] : 0.0; };
  double gn0 = g_at(0), gn1 = g_at(1);
  double fe = 0.0, bfe = 0.0, fprev = 0.0;             // psi: f_e_i, bf_e_i; T/S: b_i in fe
  for (int st = 0; st < S; ++st) {
    const int jj = par + 2 * st;
    const int row = M - 1 - jj;
    const double* cur = Lb0 + (st % 3) * blk;
    double* yb = yv + (st & 1) * nr;
    cp_async_wait<1>();
    group_sync(bar, nt);                               // Linv_jj (and D2) landed; step st-1 done
    if (st + 2 < S) copy_block_g(Lb0 + ((st + 2) % 3) * blk, Mat + (size_t)(jj + 4) * blk, blk, t, nt);
    cp_async_commit();
    const double gi = gn0;
    gn0 = gn1;
    gn1 = g_at(st + 2);
    if (a4) {
      const double bj = cf[4 * st + 2], bjt = cf[4 * st + 3], c1 = cf[4 * st];
      double y = gi;
      if (st > 0) {
        fe += fprev;                                   // f_e += f_{j+2}
        double* xb = xv + (st & 1) * nr;
        if (lead) xb[i] = fe;
        group_sync(bar, nt);
        double z = 0.0;
#pragma unroll 8
        for (int c = q; c < nr; c += TPR) z = fma(D2s[c * ldl + ir], xb[c], z);
        z = group_sum<TPR>(z);
        const double L1f = fma(bj * ir4, fe, z);      // (D2 + bj IR4) f_e
        const double tt = fma(ir4, bfe, L1f);          // + IR4 bf_e
        const double bt = fma(c1, tt, -(bjt * ir2 * fe));
        y = gi + bt;
      }
      if (lead) yb[i] = y;
      group_sync(bar, nt);
      double acc = 0.0;
#pragma unroll 8
      for (int c = q; c < nr; c += TPR) acc = fma(cur[c * ldl + ir], yb[c], acc);
      const double fi = group_sum<TPR>(acc);
      bfe = st > 0 ? fma(bj, fi, fma(bjt, fe, bfe)) : fma(bj, fi, bfe);
      fprev = fi;
      if (lead) {
        f[(size_t)row * nr + i] = fi;
        if (f32) f32[(size_t)row * nr + i] = (float)fi;
      }
    } else {
      const double y = fma(-cf[4 * st + 1], fe, gi);  // g - w b
      if (lead) yb[i] = y;
      group_sync(bar, nt);
      double acc = 0.0;
#pragma unroll 8
      for (int c = q; c < nr; c += TPR) acc = fma(cur[c * ldl + ir], yb[c], acc);
      const double fi = group_sum<TPR>(acc);
      fe = fma(cf[4 * (st + 1)], fi, fe);             // the b of the next step
      if (lead) {
        f[(size_t)row * nr + i] = fi;
        if (f32) f32[(size_t)row * nr + i] = (float)fi;
      }
    }
  }
  cp_async_wait<0>();
  if (sub) {  // Newton residual: f -= sub (the group's own writes are visible after the barrier)
    group_sync(bar, nt);
    for (int e = t; e < S * nr; e += nt) {
      const int st = e / nr, c = e - st * nr;
      const size_t o = (size_t)(M - 1 - (par + 2 * st)) * nr + c;
      f[o] -= sub[o];
    }
  }
}

// Layouts 6 / 7: one chain per CTA (field, parity, shell), rows over TPR = 2 / 4 lanes.
template <int TPR>
__global__ void k_chain_ref(ChainArgs a) {
  extern __shared__ __align__(16) double csm[];
  const int b = blockIdx.y;
  if (a.active && !a.active[b]) return;
  ref_chain<TPR>(a, a.field0 + (blockIdx.x >> 1), blockIdx.x & 1, b, threadIdx.x, blockDim.x, 0, csm);
}

// Layout 8: the three chains of one (parity, shell) in one CTA, each on its own warps: psi on wp warps with
// rows over 2 lanes (two dependent matvecs of nr/2 multiply-adds per lane and step), T and S on wt warps each
// with one lane per row (one matvec of nr multiply-adds).  Every warp then carries about the same dependent
// FP64 work per step, and a CTA puts one warp on each SM sub-partition (nr <= 32: 2 + 1 + 1 warps), where
// one CTA per (field, parity, shell) leaves the T/S warps idle half the time and stacks psi warps on shared
// sub-partitions.  Named barriers 1-3, one per chain.
__global__ void k_chain_shell(ChainArgs a, int wp, int wt) {
  extern __shared__ __align__(16) double csm[];
  const int par = blockIdx.x, b = blockIdx.y;
  if (a.active && !a.active[b]) return;
  const int w = threadIdx.x >> 5;
  const size_t sp = ref_group_doubles(a.M, a.nr, a.ldl, true), sg = ref_group_doubles(a.M, a.nr, a.ldl, false);
  if (w < wp) ref_chain<2>(a, 0, par, b, threadIdx.x, 32 * wp, 1, csm);
  else if (w < wp + wt) ref_chain<1>(a, 1, par, b, threadIdx.x - 32 * wp, 32 * wt, 2, csm + sp);
  else ref_chain<1>(a, 2, par, b, threadIdx.x - 32 * (wp + wt), 32 * wt, 3, csm + sp + sg);
}

// Layout 9: the pre-pass form (f_j = h_j + A_j f_e + B_j bf_e for psi, f_j = h_j - w Linv_j b for T and S;
// h = Linv g from k_mode_mv / k_mode_mv32, so the fused and the FP32 right-hand sides work) with the three
// chains of one (parity, shell) in one CTA, each on its own warps, named barrier and cp.async ring: psi rows
// over 2 lanes (one matvec of 2 nr columns: nr multiply-adds per lane and step), T and S one lane per row
// (nr multiply-adds).  The arithmetic of each chain is that of k_chain<2> (psi) and k_chain<1> (T, S).
__host__ __device__ inline size_t pre_group_doubles(int M, int nr, int ldl, bool a4) {
  const size_t blk = (size_t)(a4 ? 2 * nr : nr) * ldl;
  const size_t ns = (size_t)((M + 1) / 2);
  return 3 * blk + 4 * (ns + 1) + 4 * (size_t)nr;
}

template <int TPR>
__device__ __forceinline__ void pre_chain(const ChainArgs& a, int field, int par, int b, int t, int nt, int bar,
                                          double* sm) {
  const int M = a.M, nr = a.nr, ldl = a.ldl;
  const bool a4 = (field == 0);
  const size_t foff = (size_t)field * a.field_off;
  double* f = a.f + (size_t)b * a.f_stride + foff;
  const double* sub = a.sub ? a.sub + (size_t)b * a.sub_stride + foff : nullptr;
  float* f32 = a.f32 ? a.f32 + (size_t)b * a.f32_stride + foff : nullptr;
  const int i = t / TPR, q = t % TPR;
  const bool row_ok = i < nr;
  const bool lead = row_ok && q == 0;
  const int ir = row_ok ? i : 0;
  const int S = (M - par + 1) / 2;
  if (a.sym && !(a4 ? par == 0 : par == 1)) {          // symmetric: the other parity's rows are zero
    for (int e = t; e < S * nr; e += nt) {
      const int st = e / nr, c = e - st * nr;
      f[(size_t)(M - 1 - (par + 2 * st)) * nr + c] = 0.0;
      if (f32) f32[(size_t)(M - 1 - (par + 2 * st)) * nr + c] = 0.0f;
    }
    return;
  }
  const int ncol = a4 ? 2 * nr : nr;
  const int blk = ncol * ldl;
  double* Lb0 = sm;                                    // 3-slot ring of step matrices
  double* cf = sm + 3 * blk;                           // per-step scalars, 4 per step, one step past the end
  double* x2 = cf + 4 * (size_t)(S + 1);               // 2 buffers of the matvec operand ([f_e; bf_e] or b)
  const double* Mat = a4 ? a.ABA4 : (field == 1 ? a.LinvT : a.LinvS);
  const double* coef = a4 ? a.coefA4 : (field == 1 ? a.coefT : a.coefS);
  copy_block_g(Lb0, Mat + (size_t)par * blk, blk, t, nt);
  cp_async_commit();
  if (S > 1) copy_block_g(Lb0 + blk, Mat + (size_t)(par + 2) * blk, blk, t, nt);
  cp_async_commit();
  for (int e = t; e < 4 * (S + 1); e += nt) {
    const int jj = par + 2 * (e >> 2);
    cf[e] = jj < M ? coef[(size_t)jj * 4 + (e & 3)] : 0.0;
  }
  for (int c = t; c < 4 * nr; c += nt) x2[c] = 0.0;
  const double* hrow = a.g + (size_t)b * a.g_stride + foff + ir;
  auto h_at = [&](int st) { return st < S ? hrow[(size_t)(M - 1 - (par + 2 * st)) * nr] : 0.0; };
  double hn0 = h_at(0), hn1 = h_at(1);
  double fe = 0.0, bfe = 0.0;                          // psi: f_e_i, bf_e_i;  T/S: b_i in fe
  for (int st = 0; st < S; ++st) {
    const int jj = par + 2 * st;
    const int row = M - 1 - jj;
    const double* cur = Lb0 + (st % 3) * blk;
    const double* xs = x2 + (st & 1) * 2 * nr;
    double* xn = x2 + ((st + 1) & 1) * 2 * nr;
    cp_async_wait<1>();
    group_sync(bar, nt);                               // block st landed; this step's x2 visible
    if (st + 2 < S) copy_block_g(Lb0 + ((st + 2) % 3) * blk, Mat + (size_t)(jj + 4) * blk, blk, t, nt);
    cp_async_commit();
    const double hi = hn0;
    hn0 = hn1;
    hn1 = h_at(st + 2);
    double fi;
    if (a4) {
      const double pre = fma(cf[4 * st + 3], fe, bfe);   // bf_e + bjt f_e, off the matvec's path
      double acc = (q == 0) ? hi : 0.0;
      if (TPR == 1) {
        double acc1 = 0.0;
        if (st > 0) {
          int c = 0;
#pragma unroll 4
          for (; c + 1 < ncol; c += 2) {
            acc = fma(cur[c * ldl + ir], xs[c], acc);
            acc1 = fma(cur[(c + 1) * ldl + ir], xs[c + 1], acc1);
          }
          if (c < ncol) acc = fma(cur[c * ldl + ir], xs[c], acc);
        }
        acc += acc1;
      } else if (st > 0) {
#pragma unroll 8
        for (int c = q; c < ncol; c += TPR) acc = fma(cur[c * ldl + ir], xs[c], acc);
      }
      fi = group_sum<TPR>(acc);
      fe += fi;
      bfe = fma(cf[4 * st + 2], fi, pre);
      if (lead) {
        xn[i] = fe;
        xn[nr + i] = bfe;
      }
    } else {
      double acc = 0.0;
      if (TPR == 1) {
        double acc1 = 0.0;
        int c = 0;
#pragma unroll 4
        for (; c + 1 < nr; c += 2) {
          acc = fma(cur[c * ldl + ir], xs[c], acc);
          acc1 = fma(cur[(c + 1) * ldl + ir], xs[c + 1], acc1);
        }
        if (c < nr) acc = fma(cur[c * ldl + ir], xs[c], acc);
        acc += acc1;
      } else {
#pragma unroll 8
        for (int c = q; c < nr; c += TPR) acc = fma(cur[c * ldl + ir], xs[c], acc);
      }
      fi = fma(-cf[4 * st + 1], group_sum<TPR>(acc), hi);
      fe = fma(cf[4 * (st + 1)], fi, fe);             // the b of the next step
      if (lead) xn[i] = fe;
    }
    if (lead) {
      f[(size_t)row * nr + i] = fi;
      if (f32) f32[(size_t)row * nr + i] = (float)fi;
    }
  }
  cp_async_wait<0>();
  if (sub) {  // Newton residual: f -= sub (the group's own writes are visible after the barrier)
    group_sync(bar, nt);
    for (int e = t; e < S * nr; e += nt) {
      const int st = e / nr, c = e - st * nr;
      const size_t o = (size_t)(M - 1 - (par + 2 * st)) * nr + c;
      f[o] -= sub[o];
    }
  }
}

__global__ void k_chain_shell_pre(ChainArgs a, int wp, int wt) {
  extern __shared__ __align__(16) double csm[];
  const int par = blockIdx.x, b = blockIdx.y;
  if (a.active && !a.active[b]) return;
  const int w = threadIdx.x >> 5;
  const size_t sp = pre_group_doubles(a.M, a.nr, a.ldl, true), sg = pre_group_doubles(a.M, a.nr, a.ldl, false);
  if (w < wp) pre_chain<2>(a, 0, par, b, threadIdx.x, 32 * wp, 1, csm);
  else if (w < wp + wt) pre_chain<1>(a, 1, par, b, threadIdx.x - 32 * wp, 32 * wt, 2, csm + sp);
  else pre_chain<1>(a, 2, par, b, threadIdx.x - 32 * (wp + wt), 32 * wt, 3, csm + sp + sg);
}

static size_t chain_shell_pre_smem_bytes(int M, int nr, int ldl) {
  return (pre_group_doubles(M, nr, ldl, true) + 2 * pre_group_doubles(M, nr, ldl, false)) * sizeof(double);
}

static size_t chain_ref_smem_bytes(int M, int nr, int ldl) {
  return ref_group_doubles(M, nr, ldl, true) * sizeof(double);
}

static size_t chain_shell_smem_bytes(int M, int nr, int ldl) {
  return (ref_group_doubles(M, nr, ldl, true) + 2 * ref_group_doubles(M, nr, ldl, false)) * sizeof(double);
}

size_t chain_smem_bytes(int M, int nr, int ldl) {
  const size_t blk = (size_t)2 * nr * ldl;
  const size_t ns = (size_t)((M + 1) / 2);
  return (3 * blk + 4 * (ns + 1) + 4 * (size_t)nr) * sizeof(double);
}

static size_t chunk_smem_bytes(int kc, int nr, int ldl) {
  const size_t blk = (size_t)2 * nr * ldl;
  return (3 * blk + 4 * ((size_t)kc + 1) + 4 * (size_t)nr) * sizeof(double);
}

// k_chain_cref: the Linv ring and D2 (4 nr ldl), the step scalars and operand buffers, and with fuse_rhs
// the chunk's g (kc nr) and Dr (nr nr)
static size_t chunk_ref_smem_bytes(int kc, int nr, int ldl, bool fuse) {
  const size_t blk = (size_t)nr * ldl;
  return (4 * blk + 4 * ((size_t)kc + 1) + 4 * (size_t)nr + (fuse ? (size_t)kc * nr + (size_t)nr * nr : 0)) *
         sizeof(double);
}

// Carried states of the chunked chains: s_1 = d_0, s_{c+1} = Phi_c s_c + d_c (c = 1 .. nch-2) of one chain,
// run by the CTA of that chain's chunks that finishes last (see k_chain).  Rows of Phi split over TPR
// lanes.  Phi_c streams into an R-slot shared-memory ring, R - 1 matrices ahead of the one in use (R = 0:
// read through L2).  One barrier per step: the copy into the slot of Phi_{c-1} is issued after the step-c
// barrier, when every thread is done with it.  The other chunks' end states are read through L2.
template <int TPR, int R>
__device__ void carry_run(const ChainArgs& a, int field, int par, int b, double* csm) {
  const bool a4 = (field == 0);
  const int m = a4 ? 2 * a.nr : a.nr;
  const int ldm = a4 ? a.ldmA : a.ldmT;
  const int nch = a.nch;
  const size_t blk = (size_t)m * ldm;
  const double* Phi = (a4 ? a.PhiA4 : (field == 1 ? a.PhiT : a.PhiS)) + (size_t)par * nch * blk;
  const size_t slot = (size_t)(field * 2 + par) * nch;
  const double* d = a.dbuf + (size_t)b * a.d_stride + slot * a.ldd;
  double* cb = a.cbuf + (size_t)b * a.d_stride + slot * a.ldd;
  double* ring = csm;                                  // R * blk
  double* st = csm + (size_t)R * blk;                  // 2 x ldd state buffers
  const int tid = threadIdx.x;
  const int q = tid % TPR;
  const int rows_per_pass = blockDim.x / TPR;
  const int last = nch - 2;                            // Phi_1 .. Phi_last are used
  constexpr int RR = R > 0 ? R : 1;

  __syncthreads();                                     // the chunk's shared memory is free
  if (R > 0) {
#pragma unroll
    for (int k = 1; k < RR; ++k) {                     // Phi_1 .. Phi_{R-1}
      if (k <= last) copy_block(ring + (size_t)((k - 1) % RR) * blk, Phi + (size_t)k * blk, (int)blk);
      cp_async_commit();
    }
  }
  for (int e = tid; e < m; e += blockDim.x) {
    const double v = __ldcg(d + e);                    // s_1 = d_0
    st[e] = v;
    cb[a.ldd + e] = v;
  }
  for (int c = 1; c <= last; ++c) {
    const double* cur_in = st + ((c - 1) & 1) * a.ldd;
    double* nxt = st + (c & 1) * a.ldd;
    const double* P = R > 0 ? ring + (size_t)((c - 1) % RR) * blk : Phi + (size_t)c * blk;
    if (R > 0) cp_async_wait<(R > 1 ? R - 2 : 0)>();
    __syncthreads();                                   // Phi_c landed, s_c visible, step c-1 done
    if (R > 0) {
      const int k = c + R - 1;                         // into the slot of Phi_{c-1}
      if (k <= last) copy_block(ring + (size_t)((k - 1) % RR) * blk, Phi + (size_t)k * blk, (int)blk);
      cp_async_commit();
    }
    const double* dc = d + (size_t)c * a.ldd;
    double* cout = cb + (size_t)(c + 1) * a.ldd;
    for (int r0 = 0; r0 < m; r0 += rows_per_pass) {
      const int r = r0 + tid / TPR;
      const int rr = r < m ? r : 0;
      double acc = 0.0;
#pragma unroll 8
      for (int col = q; col < m; col += TPR) acc = fma(P[(size_t)col * ldm + rr], cur_in[col], acc);
      acc = group_sum<TPR>(acc);
      if (r < m && q == 0) {
        const double v = acc + __ldcg(dc + r);
        nxt[r] = v;
        cout[r] = v;
      }
    }
  }
  cp_async_wait<0>();
}

// y = P x for one m x m block P (transposed, leading dimension ldm) and x, both in shared memory; rows
// over 128/TPR lane groups, columns split over the TPR lanes of a group.
template <int TPR>
__device__ __forceinline__ void block_mv(const double* P, int ldm, const double* x, int m, double* y) {
  const int q = threadIdx.x % TPR;
  for (int r0 = 0; r0 < m; r0 += 128 / TPR) {
    const int r = r0 + threadIdx.x / TPR;
    const int rr = r < m ? r : 0;
    double acc = 0.0;
#pragma unroll 8
    for (int col = q; col < m; col += TPR) acc = fma(P[(size_t)col * ldm + rr], x[col], acc);
    acc = group_sum<TPR>(acc);
    if (r < m && q == 0) y[r] = acc;
  }
}

size_t carry_par_smem_bytes(int nr, int ldmA) { return (size_t)2 * nr * ldmA * sizeof(double); }

// Parallel carry of the chunked chains (layouts 3 and 11).  One CTA of 128 threads per (chain, shell, product
// (j, i)), i <= j - 2: part_{j,i} = P_{j,i} d_i, with P_{j,i} staged in shared memory by one round of
// cp.async (every load in flight at once).  The corrections sum each row (carried_state):
//   s_j = d_{j-1} + part_{j,0} + part_{j,1} + ... + part_{j,j-2},
// the exact algebra of s_{c+1} = Phi_c s_c + d_c.
__global__ void __launch_bounds__(128) k_carry_par(ChainArgs a) {
  extern __shared__ __align__(16) double psm[];
  __shared__ double xs[2 * kMaxNr];
  const int field = a.field0 + (blockIdx.x >> 1), par = blockIdx.x & 1;
  const int b = blockIdx.y, pidx = blockIdx.z;
  const bool a4 = field == 0;
  if (a.sym && !(a4 ? par == 0 : par == 1)) return;    // inactive chain: its carried states are not read
  if (a.active && !a.active[b]) return;
  int j = 2;
  while (j * (j - 1) / 2 <= pidx) ++j;                 // row j holds products (j-1)(j-2)/2 .. j(j-1)/2 - 1
  const int i = pidx - (j - 1) * (j - 2) / 2;
  const int m = a4 ? 2 * a.nr : a.nr;
  const int ldm = a4 ? a.ldmA : a.ldmT;
  const size_t chain = (size_t)(field * 2 + par);
  const double* d = a.dbuf + (size_t)b * a.d_stride + chain * a.nch * a.ldd;
  double* part = a.pbuf + (size_t)b * a.p_stride + chain * a.np * a.ldd;
  const double* P = (a4 ? a.PA4 : (field == 1 ? a.PT : a.PS)) + ((size_t)par * a.np + pidx) * m * ldm;
  copy_block(psm, P, m * ldm);                         // m * ldm is even (ldm even)
  cp_async_commit();
  for (int e = threadIdx.x; e < m; e += blockDim.x) xs[e] = d[(size_t)i * a.ldd + e];
  cp_async_wait<0>();
  __syncthreads();
  double* y = part + (size_t)pidx * a.ldd;
  if (a4) {
    if (m <= 64) block_mv<2>(psm, ldm, xs, m, y);
    else block_mv<1>(psm, ldm, xs, m, y);
  } else {
    if (m <= 32) block_mv<4>(psm, ldm, xs, m, y);
    else block_mv<2>(psm, ldm, xs, m, y);
  }
}

// Element e of the carried state s_c (c >= 1) of chain `chain` under layouts 3 / 11: d_{c-1} plus the row's
// products (k_carry_par), summed in index order.
__device__ __forceinline__ double carried_state(const ChainArgs& a, int b, size_t chain, int c, int e) {
  const double* d = a.dbuf + (size_t)b * a.d_stride + chain * a.nch * a.ldd;
  double v = d[(size_t)(c - 1) * a.ldd + e];
  if (c >= 2) {
    const double* row = a.pbuf + (size_t)b * a.p_stride + (chain * a.np + (size_t)(c - 1) * (c - 2) / 2) * a.ldd;
    const int nt = c - 1;                              // in index order, the terms loaded eight at a time
    for (int u0 = 0; u0 < nt; u0 += 8) {
      double tv[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) tv[k] = (u0 + k < nt) ? row[(size_t)(u0 + k) * a.ldd + e] : 0.0;
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (u0 + k < nt) v += tv[k];
    }
  }
  return v;
}

// Independent per-mode matvecs, one CTA of 128 threads per (field, mode, shell); matrix rows split over
// TPR lanes (TPR = 4 for nr <= 32, 2 for nr <= 64), every lane's column loads independent of each other:
//   FIX = false:  h_jj = Linv_jj g_jj                          (the chains' right-hand sides)
//   FIX = true:   f_jj += G_jj s_c(jj) for the modes of chunks c >= 1   (chunked chains' correction)
// Shared memory of k_mode_mv: the matrix block (m x ldl), then the layout-3 terms of s_c ((nch + 1) 2 nr)
// or the fused right-hand side's Dr and Q row (nr^2 + nr) and g (nr).
size_t mode_mv_smem_bytes(const ChainArgs& a, bool fix) {
  const size_t blk = (size_t)(fix ? 2 * a.nr : a.nr) * a.ldl;
  const size_t rest = fix ? (a.carry_seq ? 0 : ((size_t)a.nch + 1) * 2 * a.nr)
                          : (size_t)a.nr * a.nr + 2 * (size_t)a.nr;
  return (blk + rest) * sizeof(double);
}

template <int TPR, bool FIX>
__global__ void __launch_bounds__(128) k_mode_mv(ChainArgs a) {
  extern __shared__ __align__(16) double msm[];
  const int M = a.M, nr = a.nr, ldl = a.ldl;
  const int fl = blockIdx.x / M, jj = blockIdx.x - fl * M;
  const int field = a.field0 + fl;
  const int b = blockIdx.y;
  if (a.active && !a.active[b]) return;
  const int row = M - 1 - jj;
  const size_t foff = (size_t)field * a.field_off;
  const bool a4 = field == 0;
  const double* A;
  const double* x;
  double* y;
  int m;
  if (FIX) {
    const int par = jj & 1, c = (jj >> 1) / a.kc;
    if (c == 0 || (a.sym && !(a4 ? par == 0 : par == 1))) return;
    m = a4 ? 2 * nr : nr;
    A = (a4 ? a.GA4 : (field == 1 ? a.GT : a.GS)) + (size_t)jj * m * ldl;
    copy_block(msm, A, m * ldl);                       // the block streams in while s_c is formed
    cp_async_commit();
    A = msm;
    y = a.f + (size_t)b * a.f_stride + foff + (size_t)row * nr;
    const size_t chain = (size_t)(field * 2 + par);
    if (a.carry_seq) {
      x = a.cbuf + (size_t)b * a.d_stride + (chain * a.nch + c) * a.ldd;
    } else {
      // s_c: the row's terms loaded in parallel into shared memory, then summed in index order
      double* tsm = msm + (size_t)2 * nr * ldl;          // c * m doubles, then m for s_c
      const double* d = a.dbuf + (size_t)b * a.d_stride + chain * a.nch * a.ldd;
      const double* prow = a.pbuf + (size_t)b * a.p_stride + (chain * a.np + (size_t)(c - 1) * (c - 2) / 2) * a.ldd;
      for (int e = threadIdx.x; e < c * m; e += blockDim.x) {
        const int t = e / m, k = e - t * m;
        tsm[e] = t == 0 ? d[(size_t)(c - 1) * a.ldd + k] : prow[(size_t)(t - 1) * a.ldd + k];
      }
      __syncthreads();
      double* xs = tsm + (size_t)c * m;
      for (int e = threadIdx.x; e < m; e += blockDim.x) {
        double v = tsm[e];
        for (int t = 1; t < c; ++t) v += tsm[(size_t)t * m + e];
        xs[e] = v;
      }
      __syncthreads();
      x = xs;
    }
  } else {
    m = nr;
    A = (a4 ? a.LinvA4 : (field == 1 ? a.LinvT : a.LinvS)) + (size_t)jj * nr * ldl;
    copy_block(msm, A, nr * ldl);                      // the block streams in while g is formed
    cp_async_commit();
    A = msm;
    x = a.g + (size_t)b * a.g_stride + foff + (size_t)row * nr;
    y = a.h + (size_t)b * a.h_stride + foff + (size_t)row * nr;
    if (a.fuse_rhs) {
      double* Drs = msm + (size_t)nr * ldl;            // Dr (nr x nr), the Q row, then g
      double* Qs = Drs + (size_t)nr * nr;
      double* gsm = Qs + nr;
      if (a4 && !a.q32) {
        // asynchronous copies (the Linv block's are in flight too): one L2 round trip for all of them
        const double* q4 = a.out4 + (size_t)b * a.out_stride + (size_t)row * nr;
        for (int e = threadIdx.x; e < nr * nr; e += blockDim.x) cp_async8(Drs + e, a.Dr + e);
        for (int e = threadIdx.x; e < nr; e += blockDim.x) cp_async8(Qs + e, q4 + e);
        cp_async_commit();
        cp_async_wait<0>();
        __syncthreads();
      }
      for (int n = threadIdx.x; n < nr; n += blockDim.x) gsm[n] = fused_g(a, b, field, row, n, Drs, Qs);
      x = gsm;
    }
  }
  cp_async_wait<0>();
  __syncthreads();
  const int i = threadIdx.x / TPR, q = threadIdx.x % TPR;
  for (int r0 = 0; r0 < nr; r0 += 128 / TPR) {
    const int r = r0 + i;
    const int rr = r < nr ? r : 0;
    double acc = 0.0;
#pragma unroll 8
    for (int col = q; col < m; col += TPR) acc = fma(A[(size_t)col * ldl + rr], x[col], acc);
    acc = group_sum<TPR>(acc);
    if (r < nr && q == 0) {
      if (FIX) {
        const double v = y[r] + acc;
        y[r] = v;
        if (a.f32) a.f32[(size_t)b * a.f32_stride + foff + (size_t)row * nr + r] = (float)v;
      } else {
        y[r] = acc;
      }
    }
  }
}

// The same matvecs with one warp per (field, mode, shell) and one lane per row: the fewest FP64
// instructions, for launches that share the GPU with many others (lane-per-row chain layout).
template <bool FIX, int TPR>
__global__ void __launch_bounds__(128) k_mode_mv_warp(ChainArgs a, int nfields) {
  const int M = a.M, nr = a.nr, ldl = a.ldl;
  const int wid = blockIdx.x * 4 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (wid >= nfields * M) return;
  const int fl = wid / M, jj = wid - fl * M;
  const int field = a.field0 + fl;
  const int b = blockIdx.y;
  if (a.active && !a.active[b]) return;
  const int row = M - 1 - jj;
  const size_t foff = (size_t)field * a.field_off;
  const bool a4 = field == 0;
  const double* A;
  const double* x;
  double* y;
  int m;
  if (FIX) {
    const int par = jj & 1, c = (jj >> 1) / a.kc;
    if (c == 0 || (a.sym && !(a4 ? par == 0 : par == 1))) return;
    m = a4 ? 2 * nr : nr;
    A = (a4 ? a.GA4 : (field == 1 ? a.GT : a.GS)) + (size_t)jj * m * ldl;
    y = a.f + (size_t)b * a.f_stride + foff + (size_t)row * nr;
    if (a.carry_seq) {
      x = a.cbuf + (size_t)b * a.d_stride + ((size_t)(field * 2 + par) * a.nch + c) * a.ldd;
    } else {   // s_c summed per lane in the index order of k_mode_mv
      __shared__ double ssm[4][2 * kMaxNr];
      double* sw = ssm[threadIdx.x >> 5];
      for (int e = lane; e < m; e += 32) sw[e] = carried_state(a, b, (size_t)(field * 2 + par), c, e);
      __syncwarp();
      x = sw;
    }
  } else {
    m = nr;
    A = (a4 ? a.LinvA4 : (field == 1 ? a.LinvT : a.LinvS)) + (size_t)jj * nr * ldl;
    x = a.g + (size_t)b * a.g_stride + foff + (size_t)row * nr;
    y = a.h + (size_t)b * a.h_stride + foff + (size_t)row * nr;
    if (a.fuse_rhs) {
      __shared__ double gsm[4][kMaxNr];
      double* gw = gsm[threadIdx.x >> 5];
      for (int n = lane; n < nr; n += 32) gw[n] = fused_g(a, b, field, row, n);
      __syncwarp();
      x = gw;
    }
  }
  for (int r = lane; r < nr; r += 32) {
    // the TPR column-strided partial sums of k_mode_mv, combined in its shuffle-tree order: both kernels
    // give the same bits, so the launcher may pick either by size
    double acc[TPR];
#pragma unroll
    for (int q = 0; q < TPR; ++q) acc[q] = 0.0;
    int col = 0;
    for (; col + TPR <= m; col += TPR) {
#pragma unroll
      for (int q = 0; q < TPR; ++q) acc[q] = fma(__ldg(A + (size_t)(col + q) * ldl + r), x[col + q], acc[q]);
    }
#pragma unroll
    for (int q = 0; q < TPR; ++q)
      if (col + q < m) acc[q] = fma(__ldg(A + (size_t)(col + q) * ldl + r), x[col + q], acc[q]);
    double v;
    if (TPR == 4) v = (acc[0] + acc[1]) + (acc[2 % TPR] + acc[3 % TPR]);
    else v = acc[0] + acc[1 % TPR];
    if (FIX) {
      const double w = y[r] + v;
      y[r] = w;
      if (a.f32) a.f32[(size_t)b * a.f32_stride + foff + (size_t)row * nr + r] = (float)w;
    } else {
      y[r] = v;
    }
  }
}

// h = Linv g in FP32 from the FP32 right-hand sides (k_rhs32) and the FP32 copies of the Linv blocks: one
// warp per (field, mode) and group of up to kMv32Shells shells, one lane per row.  The lane keeps its row
// of the block in registers for all shells of the group (the block is read once per group, not once per
// shell); each shell's g row is loaded once per lane and broadcast by shuffles.  h is stored in FP64 for
// the chains.  NP: passes of 32 rows (nr <= 32 NP).
constexpr int kMv32Shells = 16;

template <int NP>
__global__ void __launch_bounds__(128) k_mode_mv32(ChainArgs a, int nfields, int batch) {
  const int M = a.M, nr = a.nr, ldl = a.ldl;
  const int wid = blockIdx.x * 4 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (wid >= nfields * M) return;
  const int fl = wid / M, jj = wid - fl * M;
  const int field = a.field0 + fl;
  const size_t foff = (size_t)field * a.field_off + (size_t)(M - 1 - jj) * nr;   // this mode's row
  const float* A = (field == 0 ? a.Linv32A4 : (field == 1 ? a.Linv32T : a.Linv32S)) + (size_t)jj * nr * ldl;
  const int b0 = blockIdx.y * kMv32Shells;
  const int b1 = min(batch, b0 + kMv32Shells);
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    const int r = p * 32 + lane;
    const bool rok = r < nr;
    float Ar[32 * NP];
#pragma unroll
    for (int c = 0; c < 32 * NP; ++c) Ar[c] = (rok && c < nr) ? __ldg(A + (size_t)c * ldl + r) : 0.0f;
    for (int b = b0; b < b1; ++b) {
      if (a.active && !a.active[b]) continue;
      const float* x = a.g32 + (size_t)b * a.g_stride + foff;
      float xv[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) xv[q] = (q * 32 + lane < nr) ? x[q * 32 + lane] : 0.0f;
      float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
#pragma unroll
      for (int c = 0; c < 32 * NP; c += 4) {
        s0 = fmaf(Ar[c], __shfl_sync(0xffffffffu, xv[c / 32], c % 32), s0);
        s1 = fmaf(Ar[c + 1], __shfl_sync(0xffffffffu, xv[(c + 1) / 32], (c + 1) % 32), s1);
        s2 = fmaf(Ar[c + 2], __shfl_sync(0xffffffffu, xv[(c + 2) / 32], (c + 2) % 32), s2);
        s3 = fmaf(Ar[c + 3], __shfl_sync(0xffffffffu, xv[(c + 3) / 32], (c + 3) % 32), s3);
      }
      if (rok) a.h[(size_t)b * a.h_stride + foff + r] = (double)((s0 + s1) + (s2 + s3));
    }
  }
}

template <bool FIX>
static cudaError_t launch_mode_mv(const ChainArgs& a, int batch, int nfields, cudaStream_t s, bool per_warp) {
  if (!FIX && a.g32) {   // FP32 right-hand sides: the FP32 matvecs, whatever the chain layout
    if (!a.Linv32A4 || !a.Linv32T || !a.Linv32S || a.fuse_rhs) return cudaErrorInvalidValue;
    const dim3 grid((nfields * a.M + 3) / 4, (batch + kMv32Shells - 1) / kMv32Shells);
    const cudaError_t e = a.nr <= 32 ? launch_kernel(k_mode_mv32<1>, grid, dim3(128), 0, s, a, nfields, batch)
                                     : launch_kernel(k_mode_mv32<2>, grid, dim3(128), 0, s, a, nfields, batch);
    ktimer_mark(SDD_K_MODE_H, s);
    return e;
  }
  if (per_warp) {
    const dim3 wg((nfields * a.M + 3) / 4, batch);
    const cudaError_t e = a.nr <= 32 ? launch_kernel(k_mode_mv_warp<FIX, 4>, wg, dim3(128), 0, s, a, nfields)
                                     : launch_kernel(k_mode_mv_warp<FIX, 2>, wg, dim3(128), 0, s, a, nfields);
    ktimer_mark(FIX ? SDD_K_MODE_FIX : SDD_K_MODE_H, s);
    return e;
  }
  const dim3 grid(nfields * a.M, batch);
  const size_t sm = mode_mv_smem_bytes(a, FIX);
  cudaError_t e;
  if (a.nr <= 32) {
    static unsigned long long done = 0;
    if ((e = ensure_smem_attr(k_mode_mv<4, FIX>, &done, true)) != cudaSuccess) return e;
    e = launch_kernel(k_mode_mv<4, FIX>, grid, dim3(128), sm, s, a);
  } else {
    static unsigned long long done = 0;
    if ((e = ensure_smem_attr(k_mode_mv<2, FIX>, &done, true)) != cudaSuccess) return e;
    e = launch_kernel(k_mode_mv<2, FIX>, grid, dim3(128), sm, s, a);
  }
  ktimer_mark(FIX ? SDD_K_MODE_FIX : SDD_K_MODE_H, s);
  return e;
}

// The per-mode matvecs run one per CTA (rows split over lanes: the most lanes per matvec, for launches
// that leave the GPU idle) until there are more than kMvPerCtaMax of them, then four per CTA, one per warp
// (the fewest instructions; same bits).
constexpr int kMvPerCtaMax = 2048;
static bool mv_per_warp(const ChainArgs& a, int batch, int nfields) {
  return (long long)nfields * a.M * batch > kMvPerCtaMax;
}

static int sm_count() {
  static const int sms = [] {  // thread-safe one-time initialisation (host threads may launch concurrently)
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
  return sms;
}

static cudaError_t launch_chunked(const ChainArgs& a_in, int batch, int nfields, cudaStream_t s, bool ref = false) {
  cudaError_t e;
  const bool pw = mv_per_warp(a_in, batch, nfields);
  ChainArgs a = a_in;
  if (!ref) {               // the pre-pass form: h = Linv g, read by the chunks
    if ((e = launch_mode_mv<false>(a_in, batch, nfields, s, pw)) != cudaSuccess) return e;
    a.g = a.h;
    a.g_stride = a.h_stride;
  }
  if (!a.carry_seq) {   // layouts 3 / 11: chunks, then the products in parallel, then the corrections
    const dim3 grid(2 * nfields, batch, a.nch);
    const size_t smem = ref ? chunk_ref_smem_bytes(a.kc, a.nr, a.ldl, a.fuse_rhs) : chunk_smem_bytes(a.kc, a.nr, a.ldl);
    if (ref) {
      if (a.nr <= 32) {
        static unsigned long long done = 0;
        if ((e = ensure_smem_attr(k_chain_cref<4, 0>, &done)) != cudaSuccess) return e;
        if ((e = launch_kernel(k_chain_cref<4, 0>, grid, dim3(128), smem, s, a)) != cudaSuccess) return e;
      } else {
        static unsigned long long done = 0;
        if ((e = ensure_smem_attr(k_chain_cref<2, 0>, &done)) != cudaSuccess) return e;
        if ((e = launch_kernel(k_chain_cref<2, 0>, grid, dim3(128), smem, s, a)) != cudaSuccess) return e;
      }
    } else if (a.nr <= 32) {
      static unsigned long long done = 0;
      if ((e = ensure_smem_attr(k_chain<4, true, 0>, &done)) != cudaSuccess) return e;
      if ((e = launch_kernel(k_chain<4, true, 0>, grid, dim3(128), smem, s, a)) != cudaSuccess) return e;
    } else {
      static unsigned long long done = 0;
      if ((e = ensure_smem_attr(k_chain<2, true, 0>, &done)) != cudaSuccess) return e;
      if ((e = launch_kernel(k_chain<2, true, 0>, grid, dim3(128), smem, s, a)) != cudaSuccess) return e;
    }
    ktimer_mark(SDD_K_CHAIN, s);
    if (a.nch < 2) return cudaSuccess;
    if (a.np > 0) {
      static unsigned long long done = 0;
      if ((e = ensure_smem_attr(k_carry_par, &done, true)) != cudaSuccess) return e;
      if ((e = launch_kernel(k_carry_par, dim3(2 * nfields, batch, a.np), dim3(128),
                             carry_par_smem_bytes(a.nr, a.ldmA), s, a)) != cudaSuccess)
        return e;
      ktimer_mark(SDD_K_CHAIN_CARRY, s);
    }
    if (a.defer_fix) return cudaSuccess;   // the next step's nonlinear term applies the correction
    return launch_mode_mv<true>(a, batch, nfields, s, pw);
  }
  // The carry ring of the psi chain (m = 2 nr) sets the shared memory of every chunk CTA of the launch,
  // though only the last-finishing CTA of each chain runs the carry: the ring is made as deep (4, 2 or 0
  // slots: the carry then reads Phi through L2) as still lets all the launch's chunk CTAs be resident at
  // once, so that a large batch's chunks do not run in waves for the carry's sake.  The carry's arithmetic
  // is the same at every depth.
  const int mmax = a.field0 == 0 ? 2 * a.nr : a.nr;
  const int ldmax = a.field0 == 0 ? a.ldmA : a.ldmT;
  const size_t blkb = (size_t)mmax * ldmax * sizeof(double);
  const size_t st = 2 * (size_t)a.ldd * sizeof(double);
  const size_t base = ref ? chunk_ref_smem_bytes(a.kc, a.nr, a.ldl, a.fuse_rhs) : chunk_smem_bytes(a.kc, a.nr, a.ldl);
  const dim3 grid(2 * nfields, batch, a.nch);
  const long ctas = (long)grid.x * grid.y * grid.z;
  const int t = a.nr <= 32 ? 0 : 1;                    // rows over 4 lanes (nr <= 32) or 2
  using Kern = void (*)(ChainArgs);
  static const Kern kern[2][2][3] = {
      {{k_chain<4, true, 0>, k_chain<4, true, 2>, k_chain<4, true, 4>},
       {k_chain<2, true, 0>, k_chain<2, true, 2>, k_chain<2, true, 4>}},
      {{k_chain_cref<4, 0>, k_chain_cref<4, 2>, k_chain_cref<4, 4>},
       {k_chain_cref<2, 0>, k_chain_cref<2, 2>, k_chain_cref<2, 4>}}};
  static unsigned long long done[2][2][3] = {};
  const int r = ref ? 1 : 0;
  int di = 0;
  size_t smem = std::max(base, st);
  for (int d = 2; d >= 1; --d) {                        // depth 4, then 2
    const int depth = 2 * d;
    const size_t sm = std::max(base, depth * blkb + st);
    if (sm > 200 * 1024) continue;
    if ((e = ensure_smem_attr(kern[r][t][d], &done[r][t][d])) != cudaSuccess) return e;
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern[r][t][d], 128, sm)) != cudaSuccess) return e;
    if ((long)per_sm * sm_count() >= ctas) {
      di = d;
      smem = sm;
      break;
    }
  }
  if ((e = ensure_smem_attr(kern[r][t][di], &done[r][t][di])) != cudaSuccess) return e;
  if ((e = launch_kernel(kern[r][t][di], grid, dim3(128), smem, s, a)) != cudaSuccess) return e;
  ktimer_mark(SDD_K_CHAIN, s);
  if (a.nch < 2) return cudaSuccess;
  return launch_mode_mv<true>(a, batch, nfields, s, pw);
}

// One CTA per chain.  When the batch leaves SMs idle (2*nfields*batch <= #SMs) the 4-warp split-row
// layout gives the shortest chain; otherwise rows split over 2 lanes in 2 warps (layout 5, nr <= 32):
// fewer FP64 instructions per step than 4 lanes (one shuffle-add level, half the warps repeating the
// per-row updates), and two chains share an SM's sub-partitions (64-shell batch: 0.60 vs 0.63 ms per
// step, and 0.79 with one lane per row).  Layout 2 (chunked: nch CTAs per chain, a short
// carried-state recurrence and a parallel correction) is chosen automatically while all its CTAs fit
// on the GPU at two per SM.  a.g holds the right-hand sides; a.h receives h = Linv g (k_mode_mv), which
// is what the chains read.
// The layout-3 / 11 correction f += G_jj s_c on its own (a correction left pending by the last step of a
// sequence; a.f is the state, a.f32 its FP32 copy or null).
cudaError_t launch_chunk_fix(const ChainArgs& a_in, int batch, int nfields, cudaStream_t s) {
  ChainArgs a = a_in;
  const ChunkSet& c = a.cset[1];
  a.kc = c.kc; a.nch = c.nch; a.np = c.np;
  a.GA4 = c.GA4; a.GT = c.GT; a.GS = c.GS;
  a.PA4 = c.PA4; a.PT = c.PT; a.PS = c.PS;
  a.carry_seq = 0;
  if (a.nch < 2) return cudaSuccess;
  return launch_mode_mv<true>(a, batch, nfields, s, mv_per_warp(a, batch, nfields));
}

int resolve_chain_layout(const ChainArgs& a, int batch, int nfields) {
  const int sms = sm_count();
  static const int optin = [] {   // less a margin for the chain kernels' static shared memory (a few words)
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return n - 256;
  }();
  int layout = a.layout;
  const ChunkSet& c2 = a.cset[0];
  const ChunkSet& c3 = a.cset[1];
  // layout 8 needs all three fields of a step with full right-hand sides, and its three rings in one CTA
  if (layout == 8 && (nfields != 3 || a.field0 != 0 || a.fuse_rhs || a.g32 ||
                      chain_shell_smem_bytes(a.M, a.nr, a.ldl) > (size_t)optin))
    layout = 6;
  // layout 9 needs all three fields and its three rings in one CTA
  if (layout == 9 && (nfields != 3 || a.field0 != 0 || chain_shell_pre_smem_bytes(a.M, a.nr, a.ldl) > (size_t)optin))
    layout = 5;
  // layouts 10 / 11 (chunks in the reference's order) need an FP64 right-hand side (full or fused): else 2 / 3
  if ((layout == 10 || layout == 11) && (a.g32 || !a.D2A4)) layout -= 8;
  if (layout == 0 && c3.nch > 1 && c3.GA4 && 2 * nfields * batch * c3.nch <= 2 * sms) layout = 3;
  if (layout == 0 && c2.nch > 1 && c2.GA4 && 2 * nfields * batch * c2.nch <= 2 * sms) layout = 2;
  // chosen chunks run in the reference's order where the full FP64 right-hand side is there (no pre-pass)
  if (a.layout == 0 && (layout == 2 || layout == 3) && !a.fuse_rhs && !a.g32 && a.D2A4) layout += 8;
  // layouts 6 / 7 need the full right-hand side in FP64: with the fused or the FP32 one, the pre-pass form
  if ((layout == 6 || layout == 7) && (a.fuse_rhs || a.g32)) layout = 5;
  if ((layout == 6 || layout == 7) && chain_ref_smem_bytes(a.M, a.nr, a.ldl) > (size_t)optin) layout = 2;
  if (layout != 2 && layout != 3 && layout < 6 && chain_smem_bytes(a.M, a.nr, a.ldl) > (size_t)optin)
    layout = 2;   // whole chain too long for shared memory
  // a launch that fills the SMs: the reference-order chains (4 nr^2 multiply-adds per mode instead of 7), a
  // step's three chains per CTA where they fit (64 shells N_r=30 N_theta=256: 287 us against 301 us)
  if (layout == 0) {
    if (2 * nfields * batch <= sms) layout = 4;
    else if (a.fuse_rhs || a.g32) layout = 5;
    else if (nfields == 3 && a.field0 == 0 && chain_shell_smem_bytes(a.M, a.nr, a.ldl) <= (size_t)optin) layout = 8;
    else layout = 6;
  }
  if (layout == 5 && a.nr > 32) layout = 4;
  return layout;
}

cudaError_t launch_chain(const ChainArgs& a_in, int batch, int nfields, cudaStream_t s) {
  ChainArgs a = a_in;
  const int layout = resolve_chain_layout(a, batch, nfields);
  if (layout == 9) {                  // the pre-pass form, three chains per CTA
    if (nfields != 3 || a.field0 != 0) return cudaErrorInvalidValue;
    cudaError_t e = launch_mode_mv<false>(a, batch, nfields, s, mv_per_warp(a, batch, nfields));   // h = Linv g
    if (e != cudaSuccess) return e;
    a.g = a.h;
    a.g_stride = a.h_stride;
    const int wp = (2 * a.nr + 31) / 32, wt = (a.nr + 31) / 32;
    static unsigned long long done = 0;
    if ((e = ensure_smem_attr(k_chain_shell_pre, &done)) != cudaSuccess) return e;
    e = launch_kernel(k_chain_shell_pre, dim3(2, batch), dim3(32 * (wp + 2 * wt)),
                      chain_shell_pre_smem_bytes(a.M, a.nr, a.ldl), s, a, wp, wt);
    ktimer_mark(SDD_K_CHAIN, s);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
  }
  if (layout == 8) {                  // the reference's order, three chains per CTA
    if (a.fuse_rhs || a.g32 || !a.D2A4 || nfields != 3 || a.field0 != 0) return cudaErrorInvalidValue;
    const int wp = (2 * a.nr + 31) / 32, wt = (a.nr + 31) / 32;
    static unsigned long long done = 0;
    cudaError_t e;
    if ((e = ensure_smem_attr(k_chain_shell, &done)) != cudaSuccess) return e;
    e = launch_kernel(k_chain_shell, dim3(2, batch), dim3(32 * (wp + 2 * wt)), chain_shell_smem_bytes(a.M, a.nr, a.ldl),
                      s, a, wp, wt);
    ktimer_mark(SDD_K_CHAIN, s);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
  }
  if (layout == 6 || layout == 7) {   // the reference's order, no h pre-pass (full right-hand sides only)
    if (a.fuse_rhs || a.g32 || !a.D2A4) return cudaErrorInvalidValue;
    const int tpr = layout == 6 ? 2 : 4;
    const int threads = ((a.nr * tpr + 31) / 32) * 32;
    const size_t smem = chain_ref_smem_bytes(a.M, a.nr, a.ldl);
    cudaError_t e;
    if (tpr == 2) {
      static unsigned long long done = 0;
      if ((e = ensure_smem_attr(k_chain_ref<2>, &done)) != cudaSuccess) return e;
      e = launch_kernel(k_chain_ref<2>, dim3(2 * nfields, batch), dim3(threads), smem, s, a);
    } else {
      static unsigned long long done = 0;
      if ((e = ensure_smem_attr(k_chain_ref<4>, &done)) != cudaSuccess) return e;
      e = launch_kernel(k_chain_ref<4>, dim3(2 * nfields, batch), dim3(threads), smem, s, a);
    }
    ktimer_mark(SDD_K_CHAIN, s);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
  }
  const ChunkSet& c2 = a.cset[0];
  const ChunkSet& c3 = a.cset[1];
  if (layout == 2 || layout == 3 || layout == 10 || layout == 11) {
    const bool ref = layout >= 10;
    const ChunkSet& c = (layout == 3 || layout == 11) ? c3 : c2;
    if (!c.GA4 || c.kc < 1 || c.nch < 1) return cudaErrorInvalidValue;
    a.kc = c.kc; a.nch = c.nch; a.np = c.np;
    a.GA4 = c.GA4; a.GT = c.GT; a.GS = c.GS;
    a.PhiA4 = c.PhiA4; a.PhiT = c.PhiT; a.PhiS = c.PhiS;
    a.PA4 = c.PA4; a.PT = c.PT; a.PS = c.PS;
    a.carry_seq = layout == 2 || layout == 10;
    return launch_chunked(a, batch, nfields, s, ref);
  }
  const bool split = layout == 4;
  if (layout == 5 && a.nr <= 32) {   // rows split over 2 lanes, 2 warps per chain
    cudaError_t e = launch_mode_mv<false>(a, batch, nfields, s, mv_per_warp(a, batch, nfields));
    if (e != cudaSuccess) return e;
    a.g = a.h;
    a.g_stride = a.h_stride;
    static unsigned long long done = 0;
    if ((e = ensure_smem_attr(k_chain<2, false>, &done)) != cudaSuccess) return e;
    if ((e = launch_kernel(k_chain<2, false>, dim3(2 * nfields, batch), dim3(64), chain_smem_bytes(a.M, a.nr, a.ldl),
                           s, a)) != cudaSuccess)
      return e;
    ktimer_mark(SDD_K_CHAIN, s);
    return cudaGetLastError();
  }
  cudaError_t e = launch_mode_mv<false>(a, batch, nfields, s, mv_per_warp(a, batch, nfields));   // h = Linv g
  if (e != cudaSuccess) return e;
  a.g = a.h;
  a.g_stride = a.h_stride;
  const size_t smem = chain_smem_bytes(a.M, a.nr, a.ldl);
  const dim3 grid(2 * nfields, batch);
  if (split && a.nr <= 32) {
    static unsigned long long done = 0;
    if ((e = ensure_smem_attr(k_chain<4, false>, &done)) != cudaSuccess) return e;
    if ((e = launch_kernel(k_chain<4, false>, grid, dim3(128), smem, s, a)) != cudaSuccess) return e;
  } else if (split) {
    static unsigned long long done = 0;
    if ((e = ensure_smem_attr(k_chain<2, false>, &done)) != cudaSuccess) return e;
    if ((e = launch_kernel(k_chain<2, false>, grid, dim3(128), smem, s, a)) != cudaSuccess) return e;
  } else {
    static unsigned long long done = 0;
    if ((e = ensure_smem_attr(k_chain<1, false>, &done)) != cudaSuccess) return e;
    if ((e = launch_kernel(k_chain<1, false>, grid, dim3(((a.nr + 31) / 32) * 32), smem, s, a)) != cudaSuccess) return e;
  }
  ktimer_mark(SDD_K_CHAIN, s);
  return cudaGetLastError();
}

}  // namespace sdd
