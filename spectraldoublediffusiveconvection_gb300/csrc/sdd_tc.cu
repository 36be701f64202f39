// Radial-derivative contractions of the mixed-precision nonlinear term on the 5th-generation tensor cores:
// 3xTF32 split products issued with tcgen05.mma, accumulators in tensor memory (TMEM).
//
// Derivatives (Matrix_Operators.py:698-729) applies the interior Chebyshev operators to every mode of the
// state: Dr psi_k, (D^2/r^2) psi_k (A2_SINE_R2 :498), Dr T_k and Dr S_k.  Over a batch these are one
// product with a tall operand: the state rows (shell b, field f, mode k), each a radial vector of nr values
// contiguous in memory (the reference's layout, Matrix_Operators.py:530-575), times the transposed
// operators.  Per 128-row tile:
//   D[128 x N] = A[128 x KP] B[KP x N],   B = [Dr^T | (D^2/r^2)^T], N = 2 NP,  KP, NP = nr rounded up to 8,
// with every FP32 operand split into TF32 hi and lo parts, a = a_hi + a_lo, and the product formed as
// a_lo b_hi + a_hi b_lo + a_hi b_hi (three MMAs per K step of 8, FP32 accumulation): the classic 3xTF32
// scheme, which recovers FP32-level accuracy from TF32 tensor-core products (the a_lo b_lo term, ~2^-22
// relative, is dropped).  Rows of T and S use only the Dr half of D.
//
// Layout.  A and B sit in shared memory in the canonical no-swizzle K-major layout of the tensor cores:
// core matrices of 8 rows x 16 bytes (4 TF32), stored as 128 contiguous bytes; the core matrices of one
// 8-row group follow each other along K (leading-dimension byte offset 128), and 8-row groups are KP*32
// bytes apart (stride-dimension byte offset).  A is split on the fly while it is staged (the hi/lo split
// needs the value in a register, so a bulk tensor copy could not be used; the rows are nr*4 bytes long,
// which is not a multiple of 16 either); B is split once on the host and copied in ready-made.
// The accumulator of a 128-row tile is 128 TMEM lanes x N columns; warp w of the CTA reads lanes
// 32w..32w+31 back (tcgen05.ld 32x32b), thread = tile row, and stores the row's outputs transposed,
// out[shell][op][n][k] (k contiguous), so that the 32 lanes of a warp store 32 consecutive modes.
//
// Each CTA is persistent over tiles, holds one TMEM allocation for its lifetime and waits for its MMAs on an
// mbarrier with a bounded spin (a wait that runs out sets *err, fills the tile's outputs with NaN and stops
// the CTA after its TMEM is released).
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>

#include "sdd_internal.cuh"

namespace sdd {

constexpr int kTcThreads = 128;   // 4 warps: one per 32-lane quarter of TMEM
constexpr int kTcRows = 128;      // MMA M

__host__ __device__ inline uint32_t tc_canon_off(int r, int k, int KP) {
  return (uint32_t)((r >> 3) * (KP * 32) + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

size_t tc_smem_bytes(int KP, int NP) {
  const size_t a = (size_t)kTcRows * KP * 4, b = (size_t)2 * NP * KP * 4;
  size_t n = 3 * a + 2 * b + 64;   // A hi, A lo, the raw FP32 rows of a tile, B hi, B lo, barrier + TMEM slot
  // at most three CTAs per SM with 128 TMEM columns each (five with 64): TMEM (512 columns) never runs out
  const size_t floor_bytes = (2 * NP > 64) ? (size_t)60 * 1024 : (size_t)46 * 1024;
  return n < floor_bytes ? floor_bytes : n;
}

static __device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor of a tcgen05 operand: start address, leading / stride dimension byte
// offsets (all >> 4), the descriptor version bit 46 of the sm_100 family, no swizzle.
static __device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32 (bits 7-9, 10-12 = 2), both
// K-major (bits 15, 16 = 0), N >> 3 at bit 17, M >> 4 at bit 24.
static __device__ __forceinline__ uint32_t tc_idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

static __device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

static __device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                              uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

static __device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits until the mbarrier's phase with this parity has completed, for at most limit_ns.
static __device__ __forceinline__ bool mbar_wait_bounded(uint32_t addr, uint32_t parity, uint64_t limit_ns) {
  const uint64_t t0 = globaltimer_ns();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
    if (globaltimer_ns() - t0 > limit_ns) return false;
    __nanosleep(64);
  }
}

static __device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_u32(smem)), "l"(gmem));
}

static __device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__global__ void __launch_bounds__(kTcThreads, 1) k_deriv_tc(TcArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const int KP = a.KP, NP = a.NP, N = 2 * NP, M = a.M, nr = a.nr;
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t abytes = (uint32_t)kTcRows * KP * 4, bbytes = (uint32_t)N * KP * 4;
  unsigned char* Ahi = smem_raw;
  unsigned char* Alo = Ahi + abytes;
  unsigned char* Bhi = Alo + abytes;
  unsigned char* Blo = Bhi + bbytes;
  float* raw = reinterpret_cast<float*>(Blo + bbytes);          // the tile's rows as loaded, [128][nr]
  uint64_t* mbar = reinterpret_cast<uint64_t*>(reinterpret_cast<unsigned char*>(raw) + abytes);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 1);
  __shared__ int s_timeout;
  const uint32_t ncols = N > 64 ? 128u : 64u;

  // operator tiles (split on the host, canonical layout): one 16-byte copy per thread and step
  {
    const uint4* src = reinterpret_cast<const uint4*>(a.B);
    uint4* dst = reinterpret_cast<uint4*>(Bhi);
    for (uint32_t i = tid; i < 2 * bbytes / 16; i += kTcThreads) dst[i] = __ldg(src + i);
  }
  if (tid == 0) {
    s_timeout = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t idesc = tc_idesc_tf32(kTcRows, N);
  const uint32_t sbo = (uint32_t)KP * 32;
  const int rows3 = 3 * M;
  const int ntiles = (a.rows + kTcRows - 1) / kTcRows;
  uint32_t phase = 0;

  // The rows of a tile go to `raw` in contiguous segments (one per shell the tile touches: a shell's rows
  // are contiguous).  FP32 input: cp.async, issued for the next tile as soon as this tile's rows are split,
  // so the loads overlap this tile's MMAs and epilogue.  FP64 input: converted through registers.
  auto stage = [&](int t) {
    for (int r0 = 0; r0 < kTcRows;) {
      const int R = t * kTcRows + r0;
      if (R >= a.rows) break;
      const int b = R / rows3, fk = R - b * rows3;
      const int cnt = min(min(kTcRows - r0, rows3 - fk), a.rows - R);
      float* dst = raw + (size_t)r0 * nr;
      if (a.X32) {
        const float* src = a.X32 + (size_t)b * a.x32_stride + (size_t)fk * nr;
        for (int e = tid; e < cnt * nr; e += kTcThreads) cp_async4(dst + e, src + e);
      } else {
        const double* src = a.X + (size_t)b * a.x_stride + (size_t)fk * nr;
        for (int e = tid; e < cnt * nr; e += kTcThreads) dst[e] = (float)__ldg(src + e);
      }
      r0 += cnt;
    }
    asm volatile("cp.async.commit_group;\n" ::);
  };
  if ((int)blockIdx.x < ntiles) stage(blockIdx.x);

  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    // ---- stage A.  1: this tile's rows have landed in `raw` ----
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncthreads();
    // 2: thread = tile row (kTcThreads == kTcRows): split into TF32 hi / lo, zero in the padding and in
    // rows the symmetric subspace leaves out; 16-byte stores (one core-matrix row each) ----
    const int r = tid;
    const int R = tile * kTcRows + r;
    int b = 0, f = 0, kk = 0;
    bool valid = R < a.rows, load = false;
    if (valid) {
      b = R / rows3;
      const int fk = R - b * rows3;
      f = fk / M;
      kk = fk - f * M;
      valid = !a.active || a.active[b];
      load = valid && !(a.sym && (f == 0 ? (kk % 2 == 0) : (kk % 2 == 1)));
    }
    const float* xr = raw + (size_t)r * nr;     // stride nr words between threads: conflict-free for odd nr
    for (int k4 = 0; k4 < KP / 4; ++k4) {
      uint32_t h[4], l[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = 4 * k4 + j;
        const float v = (load && k < nr) ? xr[k] : 0.f;
        h[j] = tf32_rna(v);
        l[j] = tf32_rna(v - __uint_as_float(h[j]));
      }
      const uint32_t off = tc_canon_off(r, 4 * k4, KP);
      *reinterpret_cast<uint4*>(Ahi + off) = make_uint4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<uint4*>(Alo + off) = make_uint4(l[0], l[1], l[2], l[3]);
    }
    // the tensor cores read shared memory through the async proxy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    // `raw` is free again: the next tile's rows stream in while this tile's products run
    if (tile + (int)gridDim.x < ntiles) stage(tile + gridDim.x);
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t ah = smem_u32(Ahi), al = smem_u32(Alo), bh = smem_u32(Bhi), bl = smem_u32(Blo);
      for (int s = 0; s < KP / 8; ++s) {
        const uint32_t ko = (uint32_t)s * 256;   // two core matrices (8 TF32) along K per MMA
        tc_mma(tmem, tc_desc(al + ko, 128, sbo), tc_desc(bh + ko, 128, sbo), idesc, s > 0);
        tc_mma(tmem, tc_desc(ah + ko, 128, sbo), tc_desc(bl + ko, 128, sbo), idesc, 1);
        tc_mma(tmem, tc_desc(ah + ko, 128, sbo), tc_desc(bh + ko, 128, sbo), idesc, 1);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_u32(mbar))
                   : "memory");
    }
    const bool ok = mbar_wait_bounded(smem_u32(mbar), phase, 200000000ull);   // 0.2 s
    phase ^= 1u;
    if (!ok) s_timeout = 1;
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool timed_out = s_timeout != 0;

    // ---- epilogue: TMEM lanes 32 warp .. 32 warp + 31 = tile rows (this thread's row); store transposed ----
    float* ob = a.out + (size_t)b * a.out_stride + kk;
    const int ncol_used = f == 0 ? N : NP;
    for (int c0 = 0; c0 < N; c0 += 16) {
      uint32_t v[16];
      if (!timed_out) {
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      }
      if (valid) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = c0 + j;
          if (col >= ncol_used) continue;
          const int op = f == 0 ? (col < NP ? 0 : 1) : f + 1;
          const int n = col < NP ? col : col - NP;
          if (n < nr) ob[((size_t)op * nr + n) * M] = timed_out ? __int_as_float(0x7fc00000) : __uint_as_float(v[j]);
        }
      }
    }
    if (timed_out) {
      if (tid == 0 && a.err) atomicExch(a.err, 1);
      break;
    }
    // the next tile's MMAs overwrite the accumulator: every TMEM read of this tile comes first
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");   // a prefetch left in flight by a timed-out tile
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (s_timeout) {
    // MMAs may still be in flight: give them time to finish before the accumulator is released
    if (tid == 0) mbar_wait_bounded(smem_u32(mbar), phase ^ 1u, 200000000ull);
    __syncthreads();
  }
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
  }
}

static int tc_sm_count() {
  static const int sms = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
  return sms;
}

cudaError_t launch_deriv_tc(const TcArgs& a, cudaStream_t s) {
  if (a.KP % 8 != 0 || a.NP % 8 != 0 || a.KP < 8 || 2 * a.NP > 128 || a.nr > a.KP || a.nr > a.NP || !a.B ||
      !a.out || (!a.X32 && !a.X))
    return cudaErrorInvalidValue;
  const size_t smem = tc_smem_bytes(a.KP, a.NP);
  static unsigned long long done = 0;
  cudaError_t e = ensure_smem_attr(k_deriv_tc, &done);
  if (e != cudaSuccess) return e;
  const int ntiles = (a.rows + kTcRows - 1) / kTcRows;
  // persistent: as many CTAs as fit on an SM at once (their shared memory bounds the count; at most 4)
  static int smem_sm = 0, smem_rsv = 0;
  if (!smem_sm) {
    int dev = 0;
    cudaGetDevice(&dev);
    int v = 0, r = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&r, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    smem_rsv = r;
    smem_sm = v > 0 ? v : 1;
  }
  int per_sm = smem_sm / (int)(smem + 1024 + smem_rsv);   // 1 KB of static shared memory per CTA
  per_sm = per_sm < 1 ? 1 : (per_sm > 4 ? 4 : per_sm);
  const int slots = per_sm * tc_sm_count();
  const int grid = ntiles < slots ? ntiles : slots;
  e = launch_kernel(k_deriv_tc, dim3(grid), dim3(kTcThreads), smem, s, a);
  ktimer_mark(SDD_K_DERIV_TC, s);
  return e;
}

// The operator tiles of a plan: [hi | lo] of B = [Dr ; D^2/r^2] (N = 2 NP rows of KP), each in the canonical
// layout, values rounded to TF32 (nearest, ties away from zero, on the 13 dropped bits) from FP64: b_hi the
// rounded value, b_lo the rounded remainder b - b_hi.
static float tf32_round_host(double x) {
  float f = (float)x;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) != 0x7f800000u) {
    u += 0x1000u;
    u &= 0xffffe000u;
  }
  std::memcpy(&f, &u, 4);
  return f;
}

void build_tc_operator(const double* Dr, const double* D2r2, int nr, int KP, int NP, float* out) {
  const int N = 2 * NP;
  const size_t half = (size_t)N * KP;
  for (size_t i = 0; i < 2 * half; ++i) out[i] = 0.f;
  for (int row = 0; row < N; ++row) {
    const int n = row < NP ? row : row - NP;
    if (n >= nr) continue;
    const double* src = row < NP ? Dr : D2r2;
    for (int k = 0; k < nr; ++k) {
      const double v = src[(size_t)n * nr + k];
      const float hi = tf32_round_host(v);
      const float lo = tf32_round_host(v - (double)hi);
      const size_t o = tc_canon_off(row, k, KP) / 4;
      out[o] = hi;
      out[half + o] = lo;
    }
  }
}

}  // namespace sdd
