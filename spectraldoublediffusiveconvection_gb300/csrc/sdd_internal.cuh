// Internal declarations shared by the CUDA translation units of libsdd_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/sdd_gb300.h"

namespace sdd {

constexpr int kMaxStages = 16;   // FFT stages (radices) per length
constexpr int kMaxRadix = 7;     // largest radix handled by the butterflies (2,3,4,5,7)
constexpr int kMaxNr = 64;       // interior radial points supported by the chain kernel
constexpr int kMaxM = 1024;      // theta modes supported
constexpr int kFxThreads = 256;  // threads of the rhs / theta / transform row kernels
constexpr int kFxRowThreads = 512;  // threads of the nonlinear-term row kernel

void set_cuda_error(cudaError_t e);

// Kernel launch through cudaLaunchKernelEx with the launch error returned.  (Programmatic dependent
// launch was measured here and dropped: inside the captured step graphs it made a step 1.4x slower.)
template <typename... KArgs, typename... Args>
inline cudaError_t launch_kernel(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                 Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = nullptr;
  cfg.numAttrs = 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Per-kernel timing for sdd_step_kernel_profile: while a KernelTimer is installed on the calling thread,
// every launcher records an event after each launch, tagged with the kernel's id (SDD_K_* in the public
// header).  Off (one thread-local load per launch) otherwise, and always off during graph capture.
struct KernelTimer {
  static constexpr int kMax = 64;
  cudaEvent_t ev[kMax];
  int id[kMax];
  int n;
};
extern thread_local KernelTimer* g_ktimer;
inline void ktimer_mark(int id, cudaStream_t s) {
  KernelTimer* t = g_ktimer;
  if (t && t->n < KernelTimer::kMax && cudaEventRecord(t->ev[t->n], s) == cudaSuccess) t->id[t->n++] = id;
}

// Raises a kernel's dynamic shared-memory limit to the device's opt-in maximum once per device, so
// launches do not pay a cudaFuncSetAttribute call each.  max_carveout: also prefer the largest
// shared-memory share of the L1/shared storage, for kernels whose many CTAs must be resident at once.
template <typename F>
inline cudaError_t ensure_smem_attr(F* fn, unsigned long long* done_mask, bool max_carveout = false) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (__atomic_load_n(done_mask, __ATOMIC_ACQUIRE) & bit) return cudaSuccess;
  int optin = 0;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(fn));
  if (e != cudaSuccess) return e;
  // the dynamic limit may not exceed the opt-in maximum less the kernel's static shared memory
  e = cudaFuncSetAttribute(reinterpret_cast<const void*>(fn), cudaFuncAttributeMaxDynamicSharedMemorySize,
                           optin - (int)fa.sharedSizeBytes);
  if (e == cudaSuccess && max_carveout)
    e = cudaFuncSetAttribute(reinterpret_cast<const void*>(fn), cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
  if (e == cudaSuccess) __atomic_fetch_or(done_mask, bit, __ATOMIC_ACQ_REL);
  return e;
}

// Twiddle tables and radix plan of one complex FFT length L (used for DCT-II/III of length L).
struct FftPlan {
  int L = 0;
  int nst = 0;
  int rad[kMaxStages] = {0};
  double2* w64 = nullptr;   // exp(-2 pi i k / L), k < L
  double2* e64 = nullptr;   // 0.5 exp(+i pi k / (2L)), k < L
  float2* w32 = nullptr;
  float2* e32 = nullptr;
};

// Returns a cached device FFT plan for length L (nullptr if L has a prime factor > kMaxRadix).
const FftPlan* get_fft_plan(int L);

// Kernel argument blocks -----------------------------------------------------------------------

// Division of n < 2^31 by an invariant d >= 1 with one multiply-high and a shift (Granlund and Montgomery,
// "Division by invariant integers using multiplication", 1994): with l = ceil(log2 d) and p = 31 + l,
// m = ceil(2^p / d) < 2^32 and floor(n / d) = floor(n m / 2^p), because m d - 2^p < d <= 2^l and
// n < 2^31 keep the error below one.  m = 0 encodes d = 1.
struct FastDiv {
  unsigned m;
  int s;                     // p - 32
};
inline FastDiv make_fastdiv(unsigned d) {
  if (d <= 1) return FastDiv{0u, 0};
  int l = 0;
  while ((1ull << l) < d) ++l;
  const int p = 31 + l;
  return FastDiv{(unsigned)(((1ull << p) + d - 1) / d), p - 32};
}
__device__ __forceinline__ unsigned fast_div(unsigned n, FastDiv f) { return f.m ? (__umulhi(n, f.m) >> f.s) : n; }

struct StageArgs {           // radices passed by value, with each stage's divisors precomputed
  int L, nst;
  int rad[kMaxStages];
  int tws[kMaxStages];       // twiddle stride L / (Ns R) of the stage
  FastDiv nb[kMaxStages];    // division by L / R (butterflies per transform)
  FastDiv ns[kMaxStages];    // division by Ns (product of the earlier radices)
};

inline StageArgs stage_args(const FftPlan* fp) {
  StageArgs st{};
  st.L = fp->L;
  st.nst = fp->nst;
  int Ns = 1;
  for (int i = 0; i < kMaxStages; ++i) {
    st.rad[i] = fp->rad[i];
    if (i < fp->nst) {
      const int R = fp->rad[i];
      st.tws[i] = fp->L / (Ns * R);
      st.nb[i] = make_fastdiv((unsigned)(fp->L / R));
      st.ns[i] = make_fastdiv((unsigned)Ns);
      Ns *= R;
    }
  }
  return st;
}

struct FxOps {               // FP64 or FP32 copies of the operators the nonlinear term needs
  const void* Dr;            // nr*nr
  const void* D2r2;          // nr*nr
  const void* ir4r2;         // nr
  const void* w;             // FFT twiddles (complex, P)
  const void* e;             // DCT twiddles (complex, P)
};

struct RhsArgs {
  int M, nr, sym, linear;
  double dt, Pr;
  const double* Dr;          // nr*nr
  const double* D2s;         // nr*nr (A2_SINE)
  const double* ir2s, *rsq, *dT0, *gr;
  const double* X;           // state (or perturbation) the linear terms act on
  size_t x_stride;
  const double* out4;        // FX spectral outputs (ignored when linear)
  size_t out_stride;
  const double* Ra, *Ra_s;   // per shell
  double* rhs;               // [shell][3][M][nr]
  size_t rhs_stride;
  // mixed plans: Q (out4's first block) also in FP32, [shell][M][nr]; then Dr Q is an FP32 contraction
  // (part of the FP32 nonlinear term) with Dr32, converted to FP64 once
  const float* q32;
  const float* Dr32;
  const int* active;         // nullable: per-shell flags; kernels skip shells whose flag is 0
  // FP32 right-hand sides (Jacobian products of Newton solves whose GMRES tolerance is far above FP32
  // rounding): k_rhs32 reads the FP32 copy X32 of X and writes rhs32 [shell][3][M][nr] instead of rhs
  const float* X32;
  size_t x32_stride;         // floats between shells in X32
  float* rhs32;
  const float* D2s32;        // nr*nr (A2_SINE) in FP32
  // Crank-Nicolson / Adams-Bashforth 2 (cnab2 != 0; the plan's operators are those of dt/2, dt above is
  // the full step): rhs = 2 lin + dt (3/2 E - 1/2 E_prev) with E the explicit terms per unit time
  // (psi: -(Dr Q - R) + Pr gr_k(Ra T - Ra_s S); T/S: -N - psi_T0), lin = A2_SINE(psi), r^2 T, r^2 S.
  // hist [shell][3][M][nr] (stride rhs_stride) holds E_prev on entry when hist_valid (else the explicit
  // part is Euler, dt E) and E of this step on exit.
  int cnab2;
  int hist_valid;
  double* hist;
};

// A chunk correction of the state left pending by the previous time step (layouts 3 / 11, sdd_step): the split
// nonlinear term's k_fx_deriv applies X[jj] += G_jj s_c(jj) to its mode before using it, with the
// arithmetic of k_mode_mv<TPR, true> (the same bits), and writes the corrected rows back (and their FP32
// copy).  The previous step's chunk end states and carry products are still in dbuf / pbuf: this step's
// chains overwrite them only after the nonlinear term.
struct FixArgs {
  int on;
  int kc, nch, np, ldd, ldl;
  const double* GA4, *GT, *GS;
  const double* dbuf, *pbuf;
  size_t d_stride, p_stride;
  double* X;                 // the state being corrected in place (the nonlinear term's input)
  float* X32;                // nullable: its FP32 copy
  int stage;                 // set by the launcher: the mode's G blocks and carried-state terms are staged
                             // in shared memory when they fit (fix_stage_doubles)
};

struct FxArgs {
  int M, nr, P, sym;
  StageArgs st;
  FxOps ops;
  const double* X;           // state whose nonlinear term (FX) or perturbation (DFX) is formed
  size_t x_stride;           // doubles between shells in X
  const float* X32;          // nullable: X rounded to FP32, read by the FP32 kernels instead of converting X
  size_t x32_stride;         // floats between shells in X32
  float* q32;                // nullable (FP32 kernels): Q also written in FP32, [shell][M][nr]
  const int* active;         // nullable: per-shell flags; kernels skip shells whose flag is 0 (their
                             // outputs are left as they were: Krylov solves mask those shells out)
  void* base;                // base-state grid cache [shell][nr][9][P] (T precision), nullable
  size_t base_stride;        // elements between shells in base
  double* out4;              // [shell][4][M][nr] : Qhat, Rhat, NJ_T hat, NJ_S hat
  size_t out_stride;         // doubles between shells in out4
  double* fx_out;            // optional: write F directly in state layout [shell][3][M][nr]
  size_t fx_stride;
  void* grid;                // nullable: grid-field scratch [shell][nr][9][P] (T precision) of the split path
  size_t grid_stride;        // elements between shells in grid
  int split;                 // 0 auto, 1 fused row kernel, 2 split (needs grid or a cache)
  void* deriv;               // split path: radial derivatives [shell][5][M][nr] (T): Dr psi, D2r2 psi, Dr T, Dr S
                             // (and, with fuse_rhs, D2s psi in FP64 as the fifth block)
  size_t deriv_stride;       // elements between shells in deriv
  // fuse_rhs (FP64 split path): k_fx_grid writes the linear parts of the three right-hand sides into
  // rl.rhs (the terms of k_rhs that do not involve the nonlinear term); the chains' h kernel adds the
  // nonlinear parts from out4.  rl carries the operators, parameters and the rhs buffer.
  int fuse_rhs;
  RhsArgs rl;
  FixArgs fix;               // split path: a pending correction of X (see FixArgs)
  // mixed plans: the FP32 radial contractions on the tensor cores (k_deriv_tc, 3xTF32).  tcB: the plan's
  // split operator tiles (nullable: CUDA-core FP32 contractions); tcKP / tcNP: nr rounded up to 8.  When
  // they are used, deriv's four FP32 blocks hold the transposed layout [op][n][k] (deriv_t, set by
  // launch_fx) and the row kernels read them instead of contracting.
  const float* tcB;
  int tcKP, tcNP;
  int* tc_err;               // nullable: set by a tensor-core kernel whose wait timed out
  int deriv_t;
};

// k_deriv_tc: the four radial contractions of Derivatives for every state row of a batch, 3xTF32 on the
// tensor cores, into out[shell][op][n][k] (op 0 Dr psi, 1 (D^2/r^2) psi, 2 Dr T, 3 Dr S; FP32).
struct TcArgs {
  int M, nr, sym, KP, NP;
  int rows;                  // batch * 3 * M state rows
  const float* X32;          // the state in FP32 (nullable: X is converted)
  size_t x32_stride;
  const double* X;
  size_t x_stride;
  const int* active;         // nullable: per-shell flags; rows of shells whose flag is 0 are skipped
  const float* B;            // [hi | lo] operator tiles (build_tc_operator), 16-byte aligned
  float* out;
  size_t out_stride;         // floats between shells in out
  int* err;                  // nullable: set to 1 when a wait for the tensor cores timed out
};



// Tables of one chunking of the chains (see k_chain): chunk length kc, nch chunks per chain, the
// corrections G_jj of every mode and the carried-state maps, either per chunk (Phi_c, the sequential
// carry of layout 2) or as the products P_{j,i} = Phi_{j-1} ... Phi_{i+1}, i <= j - 2 (np per chain,
// row j after row j-1; the parallel carry of layout 3).
struct ChunkSet {
  int kc, nch, np;
  const double* GA4, *GT, *GS;        // [M][m cols][ldl] transposed G_jj (m = 2 nr for psi, nr for T/S)
  const double* PhiA4, *PhiT, *PhiS;  // [2 parity][nch][m cols][ldm] transposed Phi_c
  const double* PA4, *PT, *PS;        // [2 parity][np][m cols][ldm] transposed P_{j,i}
};

struct ChainArgs {
  int M, nr, ldl, sym;
  int field0;                // first field handled (blockIdx.x/2 + field0)
  int layout;                // 1 one lane per row, 4 rows split over 4 warps, 2/3 chunked, 6/7 the reference's
                             // order (resolved by the host)
  size_t field_off;          // doubles between field blocks (N_fm*nr, or 0 when g/f point at one block)
  const double* g;           // rhs [shell][3][M][nr]
  size_t g_stride;
  double* f;                 // solution [shell][3][M][nr]
  size_t f_stride;
  float* f32;                // nullable: the final solution also rounded to FP32 (the next mixed step's X32)
  size_t f32_stride;
  const double* sub;         // nullable: f -= sub (Newton residual), same layout
  size_t sub_stride;
  const double* LinvA4, *LinvT, *LinvS;  // [M][nr cols][ldl] transposed blocks
  const double* ABA4;        // [M][2 nr cols][ldl]: transposed [A_j B_j] of the psi chain
  const double* D2A4;        // [nr cols][ldl]: transposed D2 of the psi operator (layouts 6 and 7)
  double* h;                 // [shell][3][M][nr] h = Linv g
  size_t h_stride;           // doubles between shells in h
  const double* ir2A4, *ir4A4;
  const double* coefA4;      // [M][4] per jj: (dt bjt, dt bjt bj, bj, bjt), dt = Pr*dt, j = M - jj
  const double* coefT, *coefS;  // [M][4] per jj: (2 dt (j+2), 0.5 if j == 0 else 1, 0, 0), j = M-1-jj
  double dtA4, dtT, dtS;     // Pr*dt, dt, Tau*dt
  // fuse_rhs: g is not read; the h kernel forms g from the linear parts in `lin` and the nonlinear-term
  // outputs in out4 (psi: -dt (Dr Q - R) + lin; T, S: -dt N + lin), exactly as k_rhs would
  int fuse_rhs;
  const double* lin;         // [shell][3][M][nr] linear parts (k_fx_grid), stride g_stride
  const double* out4;        // [shell][4][M][nr]
  size_t out_stride;
  const double* Dr;          // nr*nr (FP64)
  const float* q32, *Dr32;   // mixed plans: Dr Q in FP32 (see RhsArgs)
  double dt;                 // the step's dt
  // chunked (parallel-in-modes) chains, layout 2: every chain of S = N_fm/2 steps is cut into nch chunks
  // of kc steps.  Chunk c runs from a zero carried state (f_local, end state d_c); the carried states
  // s_c at the chunk starts follow s_{c+1} = Phi_c s_c + d_c; then f += G_jj s_c for the chunk's modes.
  int kc, nch;               // chunk length (steps) and chunks per chain
  int ldmA, ldmT;            // leading dimensions of Phi for the psi (m = 2 nr) and T/S (m = nr) states
  int ldd;                   // doubles per (field, parity, chunk) slot of dbuf / cbuf (>= 2 nr, even)
  const double* GA4, *GT, *GS;        // [M][m cols][ldl] transposed G_jj (m = 2 nr for psi, nr for T/S)
  const double* PhiA4, *PhiT, *PhiS;  // [2 parity][nch][m cols][ldm] transposed Phi_c
  double* dbuf;              // [shell][3][2][nch][ldd] chunk end states from a zero start
  double* cbuf;              // [shell][3][2][nch][ldd] carried states at the chunk starts (c >= 1)
  size_t d_stride;           // doubles per shell in dbuf / cbuf
  int* counter;              // [shell][6] chunks finished per chain (the last one runs the carry), zeroed
  // layouts 3 / 11 (parallel carry): the chunks only write their end states; k_carry_par forms
  // part_{j,i} = P_{j,i} d_i for every product in parallel and the corrections sum
  // s_j = d_{j-1} + sum_i part_{j,i} (index order)
  int carry_seq;             // 1: the last-finishing chunk CTA runs the sequential carry (layouts 2 / 10)
  int np;                    // products per chain
  const double* PA4, *PT, *PS;
  double* pbuf;              // [shell][6][np][ldd] products P_{j,i} d_i
  size_t p_stride;           // doubles per shell in pbuf
  ChunkSet cset[2];          // the chunkings of layouts 2 and 3 (launch_chain copies one into the fields above)
  int defer_fix;             // layouts 3 / 11: leave the correction to the next step's nonlinear term (FixArgs)
  const int* active;         // nullable: per-shell flags; kernels skip shells whose flag is 0
  // nullable: FP32 right-hand sides (k_rhs32, stride g_stride): h = Linv g is then formed in FP32 with the
  // FP32 copies of the Linv blocks (k_mode_mv32) and stored in FP64 for the chains
  const float* g32;
  const float* Linv32A4, *Linv32T, *Linv32S;
};

struct DiagArgs {
  int M, nr, sym, L;         // L = 3 M: the kinetic-energy grid
  StageArgs st;              // FFT of length L
  const double2* w;          // FFT twiddles of length L
  const double2* e;          // DCT twiddles of length L
  const double* Dr;          // nr*nr interior D
  const double* ir;          // nr  1/R interior
  const double* tw;          // L   trapezoid weight * sin(theta_i) on the L-point midpoint grid
  const double* wr;          // nr  trapezoid weights over the interior radii
  const double* nuw;         // ceil(M/2)*nr  Nusselt weights of the even modes
  double ke_scale;           // 1/(2V), V = (2/3)(r_o^3 - r_i^3)
  const double* X;           // states [shell][3][M][nr]
  size_t x_stride;
  double* part;              // [shell][nr] per-radius kinetic-energy sums
  double* out;               // [shell][4]
};

// launchers (return cudaError_t of the launch)
cudaError_t launch_diag(const DiagArgs& a, int batch, cudaStream_t s);
size_t diag_rows_smem_bytes(int M, int L);
cudaError_t launch_fx(const FxArgs& a, int batch, int mode, int prec, cudaStream_t s);
cudaError_t launch_deriv_tc(const TcArgs& a, cudaStream_t s);
size_t tc_smem_bytes(int KP, int NP);
// [hi | lo] tiles of B = [Dr ; D^2/r^2] (2 NP rows of KP) in the tensor cores' canonical shared-memory
// layout: 2 * 2 NP * KP floats
void build_tc_operator(const double* Dr, const double* D2r2, int nr, int KP, int NP, float* out);
// whether launch_fx takes the split path for these arguments
bool fx_uses_split(const FxArgs& a, int batch, int mode);
// the largest dynamic shared memory a k_fx_rows launch of this precision can take on the current device
size_t fx_rows_max_dynamic_smem(int prec);
// the split-or-fused rule alone (split: 0 automatic, 1 fused, 2 split), for a plan whose scratch is not yet
// reserved
bool fx_split_rule(int split, int nr, int batch);
cudaError_t launch_rhs(const RhsArgs& a, int batch, cudaStream_t s);
cudaError_t launch_chain(const ChainArgs& a, int batch, int nfields, cudaStream_t s);
// the chain layout (1, 2, 3 or 4) launch_chain runs for a.layout (0 = automatic) and this launch size
int resolve_chain_layout(const ChainArgs& a, int batch, int nfields);
cudaError_t launch_chunk_fix(const ChainArgs& a, int batch, int nfields, cudaStream_t s);
cudaError_t launch_theta_op(int op, int M, int nr, int sym, const double* D2, const double* ir,
                            const double* dT0, const double* g, double* f, int batch,
                            cudaStream_t s);
cudaError_t launch_transform(int kind, int rows, int n_in, int n_out, const FftPlan* fp,
                             const double* in, double* out, cudaStream_t s);
size_t fx_smem_bytes(int M, int P, int prec);

}  // namespace sdd
