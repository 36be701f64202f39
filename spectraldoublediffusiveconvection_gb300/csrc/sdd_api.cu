// C ABI of libsdd_gb300: plans (device-resident operators), FFT tables, workspaces, entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <atomic>
#include <mutex>
#include <vector>

#include "sdd_internal.cuh"
#include "sdd_krylov.cuh"

namespace sdd {
cudaError_t launch_fx_finish(int M, int nr, const double* Dr, const double* out4, size_t out_stride,
                             double* F, size_t f_stride, int batch, cudaStream_t s);

static thread_local int g_last_cuda = 0;
thread_local KernelTimer* g_ktimer = nullptr;
void set_cuda_error(cudaError_t e) { g_last_cuda = (int)e; }

#define SDD_CUDA(call)                         \
  do {                                         \
    cudaError_t e_ = (call);                   \
    if (e_ != cudaSuccess) {                   \
      set_cuda_error(e_);                      \
      (void)cudaGetLastError(); /* not left for the caller's next runtime call */ \
      return e_ == cudaErrorMemoryAllocation ? SDD_ERR_NOMEM : SDD_ERR_CUDA; \
    }                                          \
  } while (0)

// ---- FFT plans (per device, per length) --------------------------------------------------------
static bool factor_length(int L, int* rad, int* nst) {
  int n = 0, r = L;
  while (r % 4 == 0) { if (n >= kMaxStages) return false; rad[n++] = 4; r /= 4; }
  while (r % 2 == 0) { if (n >= kMaxStages) return false; rad[n++] = 2; r /= 2; }
  const int odd[3] = {3, 5, 7};
  for (int f : odd)
    while (r % f == 0) { if (n >= kMaxStages) return false; rad[n++] = f; r /= f; }
  if (r != 1) return false;
  *nst = n;
  return true;
}

static std::mutex g_fft_mu;
static std::map<std::pair<int, int>, FftPlan*> g_fft;

const FftPlan* get_fft_plan(int L) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(g_fft_mu);
  auto key = std::make_pair(dev, L);
  auto it = g_fft.find(key);
  if (it != g_fft.end()) return it->second;
  FftPlan* fp = new FftPlan();
  fp->L = L;
  if (L < 1 || !factor_length(L, fp->rad, &fp->nst)) { delete fp; return nullptr; }
  std::vector<double2> w(L), e(L);
  std::vector<float2> wf(L), ef(L);
  const double pi = 3.14159265358979323846264338327950288;
  for (int k = 0; k < L; ++k) {
    const double a = 2.0 * pi * (double)k / (double)L;
    w[k] = make_double2(std::cos(a), -std::sin(a));
    const double b = pi * (double)k / (2.0 * (double)L);
    e[k] = make_double2(0.5 * std::cos(b), 0.5 * std::sin(b));
    wf[k] = make_float2((float)w[k].x, (float)w[k].y);
    ef[k] = make_float2((float)e[k].x, (float)e[k].y);
  }
  bool ok = cudaMalloc(&fp->w64, L * sizeof(double2)) == cudaSuccess &&
            cudaMalloc(&fp->e64, L * sizeof(double2)) == cudaSuccess &&
            cudaMalloc(&fp->w32, L * sizeof(float2)) == cudaSuccess &&
            cudaMalloc(&fp->e32, L * sizeof(float2)) == cudaSuccess;
  ok = ok && cudaMemcpy(fp->w64, w.data(), L * sizeof(double2), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(fp->e64, e.data(), L * sizeof(double2), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(fp->w32, wf.data(), L * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(fp->e32, ef.data(), L * sizeof(float2), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    cudaFree(fp->w64); cudaFree(fp->e64); cudaFree(fp->w32); cudaFree(fp->e32);
    delete fp;
    return nullptr;
  }
  g_fft[key] = fp;
  return fp;
}

}  // namespace sdd

using namespace sdd;

// ---- plan ---------------------------------------------------------------------------------------
// One instantiated graph of `pairs` step pairs A -> B -> A (B the plan's xtmp), keyed by everything the
// captured launches bake in.
struct StepGraph {
  cudaGraphExec_t exec;
  const double* A;
  const double* Ra;
  const double* Ras;
  int batch, linear, pairs, layout, fx_split;
  unsigned long long last_use;
};
constexpr int kStepGraphs = 8;
// CUDA graphs of the GMRES products: the launches of one Jacobian (or bordered) product, keyed by what they
// bake in (the kind of product, the batch, every pointer it reads or writes, the plan's kernel choices)
struct MvGraph {
  cudaGraphExec_t exec;
  int kind, batch, layout, fx_split, use_tc;
  const void* ptr[7];               // v, out, active, v32, Ra, Ras, base
  unsigned long long last_use;
};
constexpr int kMvGraphs = 8;
constexpr int kGraphMinSteps = 8;   // sdd_step replays captured graphs from this many steps on
// The Arnoldi loop reads the shells' activity flags kFlagLag columns late, so that the host never waits on
// the column the GPU is computing: the columns run past the last active one are fully masked (no shell takes
// part) and are not counted as Jacobian products.
constexpr int kFlagLag = 2;

struct sdd_plan {
  int M, nr, P, ldl, sym, prec, device;
  int chain_layout;
  int fx_split;                     // 0 auto, 1 fused row kernel, 2 split over 7 CTAs per row
  double dt, Pr, Tau;
  const FftPlan* fft;
  // FP64 operators
  double *Dr, *D2r2, *ir4r2, *D2s, *ir2s, *D2A4, *ir2A4, *ir4A4, *rsq, *dT0, *gr;
  double *LinvA4, *LinvT, *LinvS;
  double *ABA4;                     // transposed [A_j B_j] of the psi chain
  double *coefA4, *coefT, *coefS;   // per-step scalars of the chains
  // chunked chains: cs[0] the chunking of layout 2 (sequential carry), cs[1] of layout 3 (parallel
  // carry); leading dimensions; workspaces sized for the larger chunk and product counts
  ChunkSet cs[2];
  int ldmA, ldmT, ldd, nch_alloc, np_alloc;
  // host copies of what the chunk tables are built from, for sdd_plan_set_chunk_length: the psi step
  // matrices [A B] (M x 2nr x ldl), Linv_T, Linv_S (M nr nr), the per-step scalars (4 M each)
  double *h_AB, *h_LinvT, *h_LinvS, *h_cA, *h_cT, *h_cS;
  double *dbuf, *cbuf;              // [B][3][2][nch_alloc][ldd] chunk end states / carried states
  int* dcnt;                        // [B][6] chunk counters of the sequential carry
  double* pbuf;                     // [B][6][np_alloc][ldd] products of the parallel carry
  // FP32 copies used by the mixed-precision nonlinear term
  float *Dr32, *D2r232, *ir4r232;
  // mixed plans: FP32 copies for the FP32 right-hand sides and h matvecs of Newton's Jacobian products
  float* D2s32;
  float* Linv32[3];                 // LinvA4, LinvT, LinvS in their transposed layout
  // mixed plans: the radial contractions on the tensor cores (k_deriv_tc): split operator tiles
  float* tcB;                       // [hi | lo] of [Dr ; D^2/r^2], tensor-core layout (build_tc_operator)
  int tcKP, tcNP;                   // nr rounded up to 8
  int use_tc;                       // 1: k_deriv_tc forms the FP32 contractions (sdd_plan_set_tensor_cores)
  int* tc_err;                      // device word set by a tensor-core kernel whose wait timed out
  // workspace
  int ws_batch;
  double* out4;     // [B][4][M][nr]
  double* rhs;      // [B][3][M][nr]
  double* xtmp;     // [B][3][M][nr]
  double* hbuf;     // [B][3][M][nr] h = Linv g of the chains
  float* x32[2];    // mixed plans: [B][3][M][nr] FP32 copies of sdd_step's output buffer and of xtmp
  float* q32;       // mixed plans: [B][M][nr] FP32 copy of the nonlinear term's Q block
  float* g32;       // mixed plans: [B][3][M][nr] FP32 right-hand sides (k_rhs32)
  void* base_tmp;   // [B][nr][9][P] (T precision), for DFX without a caller cache
  void* gridbuf;    // [B][nr][9][P] (T precision), grid fields of the split nonlinear-term path
  void* derivbuf;   // [B] x (5 M nr doubles of room), radial derivatives of the split path: 4 M nr of the
                    // precision, then M nr doubles (D2s psi of the fused right-hand side)
  // Krylov / Newton / continuation workspace (grown on demand)
  int sv_B, sv_m;
  double reorth_eta;  // second Gram-Schmidt pass where |w'| < reorth_eta |w| (sdd_plan_set_reorth_eta)
  int kv_last_B;      // batch of the last GMRES solve (the layout sdd_krylov_basis reads)
  int kv_basis32;     // the last GMRES solve kept its basis in FP32 (in kv_V's storage)
  double *kv_V, *kv_w, *kv_r, *kv_part, *kv_nrm2, *kv_small, *kv_dot;
  int* kv_ismall;
  int* kv_ticket;     // [B] per-shell CTA counters of the one-launch reductions (zero between launches)
  double* h_dbl;      // pinned host scalars
  int* h_int;         // pinned host flags: kFlagLag + 1 slots of B
  cudaEvent_t flag_ev[kFlagLag + 1];   // one per slot: its flags have arrived
  cudaEvent_t wait_ev;                 // the solvers' host waits (blocking: the waiting thread sleeps)
  double *sv_F, *sv_x, *sv_X0, *sv_Xd, *sv_t, *sv_G, *sv_Jmu, *sv_g, *sv_base64, *sv_dev;
  float* sv_base32;
  float* kv_v32;      // mixed plans: [B][ld] FP32 copy of the Krylov vector the next product is applied to
  // diagnostics (sdd_diagnostics): FFT plan of length 3M and weight tables; part = per-radius sums
  const FftPlan* dfft;
  double *dg_ir, *dg_tw, *dg_wr, *dg_nuw, *dg_part, *dg_out;
  double ke_scale;
  // CUDA graphs of repeated time steps (sdd_step): A -> xtmp -> A pairs, A = the caller's output
  StepGraph graphs[kStepGraphs];
  MvGraph mv_graphs[kMvGraphs];
  long long mv_count[3];            // GMRES products: captured into a graph, replayed from one, run directly
  int mv_graphs_off;                // 1: run the GMRES products kernel by kernel (sdd_plan_set_product_graphs)
  double* kv_vin;     // [B][ld] the Krylov vector the next product reads (a fixed address for its graph)
  unsigned long long graph_clock;
  cudaStream_t cap_stream;          // private capture stream (created on first use)
  cudaStream_t branch_stream;       // sdd_batch_step: this plan's branch of a batched call (created on first use)
  cudaEvent_t branch_ev[2];         // sdd_batch_step: the fork (recorded on the caller's stream) and the join
};

// Workspace allocations (sdd_plan_reserve and the Krylov workspace) go through ws_malloc, so that a test can
// make them fail on the host (sdd_debug_fail_allocations) and check that SDD_ERR_NOMEM reaches the caller.
static std::atomic<long long> g_alloc_left{-1};   // allocations that still succeed; -1: no limit
static cudaError_t ws_malloc(void** ptr, size_t bytes, bool pinned_host = false) {
  long long left = g_alloc_left.load();
  while (left >= 0) {
    if (left == 0) {
      *ptr = nullptr;
      return cudaErrorMemoryAllocation;
    }
    if (g_alloc_left.compare_exchange_weak(left, left - 1)) break;
  }
  return pinned_host ? cudaMallocHost(ptr, bytes) : cudaMalloc(ptr, bytes);
}
template <typename T>
static cudaError_t ws_malloc(T** ptr, size_t bytes, bool pinned_host = false) {
  return ws_malloc(reinterpret_cast<void**>(ptr), bytes, pinned_host);
}

extern "C" {

const char* sdd_error_string(int status) {
  switch (status) {
    case SDD_OK: return "ok";
    case SDD_ERR_ARG: return "invalid argument";
    case SDD_ERR_ODD_NFM: return "The number of Fourier modes is not even";
    case SDD_ERR_UNSUPPORTED: return "size not supported by the GB300 kernels";
    case SDD_ERR_CUDA: return "CUDA runtime error";
    case SDD_ERR_NOMEM: return "device allocation failed";
    case SDD_ERR_NOT_CONVERGED: return "iteration did not converge";
    default: return "unknown status";
  }
}

int sdd_last_cuda_error(void) { return g_last_cuda; }
int sdd_version(void) { return 100; }

int sdd_transform(int kind, int rows, int n_in, int n_out, const double* in, double* out, void* stream) {
  if (kind < SDD_IDCT || kind > SDD_DST || rows < 0 || n_in < 1 || n_out < 1 || !in || !out)
    return SDD_ERR_ARG;
  if (rows == 0) return SDD_OK;
  const bool inverse = kind == SDD_IDCT || kind == SDD_IDST;
  if (!inverse && n_out > n_in) return SDD_ERR_ARG;
  const int L = inverse ? n_out : n_in;
  const FftPlan* fp = get_fft_plan(L);
  if (!fp) return SDD_ERR_UNSUPPORTED;
  const size_t smem = 6 * (size_t)L * sizeof(double2) + (4 * 32 + 8) * sizeof(double);
  if (smem > 227 * 1024) return SDD_ERR_UNSUPPORTED;
  cudaError_t e = launch_transform(kind, rows, n_in, n_out, fp, in, out, (cudaStream_t)stream);
  SDD_CUDA(e);
  return SDD_OK;
}

static int upload(double** dst, const double* src, size_t n) {
  if (!src) return SDD_ERR_ARG;
  SDD_CUDA(cudaMalloc(dst, n * sizeof(double)));
  SDD_CUDA(cudaMemcpy(*dst, src, n * sizeof(double), cudaMemcpyHostToDevice));
  return SDD_OK;
}
static int upload32(float** dst, const double* src, size_t n) {
  std::vector<float> h(n);
  for (size_t i = 0; i < n; ++i) h[i] = (float)src[i];
  SDD_CUDA(cudaMalloc(dst, n * sizeof(float)));
  SDD_CUDA(cudaMemcpy(*dst, h.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  return SDD_OK;
}
// Linv blocks (and D2_A4 with M = 1) go to the device transposed, column c of a block contiguous with
// leading dimension ldl (even, so every block starts on a 16-byte boundary for cp.async).
static int upload_linv(double** dst, const double* src, int M, int nr, int ldl) {
  if (!src) return SDD_ERR_ARG;
  std::vector<double> h((size_t)M * nr * ldl, 0.0);
  for (int m = 0; m < M; ++m)
    for (int i = 0; i < nr; ++i)
      for (int c = 0; c < nr; ++c) h[((size_t)m * nr + c) * ldl + i] = src[((size_t)m * nr + i) * nr + c];
  SDD_CUDA(cudaMalloc(dst, h.size() * sizeof(double)));
  SDD_CUDA(cudaMemcpy(*dst, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
  return SDD_OK;
}
// The same transposed layout rounded to FP32.
static int upload_linv32(float** dst, const double* src, int M, int nr, int ldl) {
  if (!src) return SDD_ERR_ARG;
  std::vector<float> h((size_t)M * nr * ldl, 0.0f);
  for (int m = 0; m < M; ++m)
    for (int i = 0; i < nr; ++i)
      for (int c = 0; c < nr; ++c) h[((size_t)m * nr + c) * ldl + i] = (float)src[((size_t)m * nr + i) * nr + c];
  SDD_CUDA(cudaMalloc(dst, h.size() * sizeof(float)));
  SDD_CUDA(cudaMemcpy(*dst, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
  return SDD_OK;
}

static void clear_mv_graphs(sdd_plan* p);

static void solver_free(sdd_plan* p) {
  clear_mv_graphs(p);               // they bake in the solver workspace
  cudaFree(p->kv_vin);
  p->kv_vin = nullptr;
  double* d[] = {p->kv_V, p->kv_w, p->kv_r, p->kv_part, p->kv_nrm2, p->kv_small, p->kv_dot, p->sv_F, p->sv_x,
                 p->sv_X0, p->sv_Xd, p->sv_t, p->sv_G, p->sv_Jmu, p->sv_g, p->sv_base64, p->sv_dev};
  for (double* x : d) cudaFree(x);
  cudaFree(p->sv_base32);
  cudaFree(p->kv_v32);
  cudaFree(p->kv_ismall);
  cudaFree(p->kv_ticket);
  cudaFreeHost(p->h_dbl);
  cudaFreeHost(p->h_int);
  for (cudaEvent_t& e : p->flag_ev) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  if (p->wait_ev) cudaEventDestroy(p->wait_ev);
  p->wait_ev = nullptr;
  p->kv_V = p->kv_w = p->kv_r = p->kv_part = p->kv_nrm2 = p->kv_small = p->kv_dot = nullptr;
  p->sv_F = p->sv_x = p->sv_X0 = p->sv_Xd = p->sv_t = p->sv_G = p->sv_Jmu = p->sv_g = p->sv_base64 = nullptr;
  p->sv_dev = nullptr;
  p->sv_base32 = nullptr;
  p->kv_v32 = nullptr;
  p->kv_ismall = nullptr;
  p->kv_ticket = nullptr;
  p->h_dbl = nullptr;
  p->h_int = nullptr;
  p->sv_B = p->sv_m = 0;
}

static void clear_mv_graphs(sdd_plan* p) {
  for (MvGraph& g : p->mv_graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
  }
}

static void clear_step_graphs(sdd_plan* p) {
  for (int i = 0; i < kStepGraphs; ++i) {
    if (p->graphs[i].exec) cudaGraphExecDestroy(p->graphs[i].exec);
    p->graphs[i].exec = nullptr;
  }
  clear_mv_graphs(p);
}

static void free_chunk_set(ChunkSet& c) {
  const double* t[] = {c.GA4, c.GT, c.GS, c.PhiA4, c.PhiT, c.PhiS, c.PA4, c.PT, c.PS};
  for (const double* x : t) cudaFree(const_cast<double*>(x));
  c = ChunkSet{};
}

static void free_plan(sdd_plan* p) {
  if (!p) return;
  delete[] p->h_AB; delete[] p->h_LinvT; delete[] p->h_LinvS;
  delete[] p->h_cA; delete[] p->h_cT; delete[] p->h_cS;
  clear_step_graphs(p);
  if (p->cap_stream) cudaStreamDestroy(p->cap_stream);
  if (p->branch_stream) cudaStreamDestroy(p->branch_stream);
  for (cudaEvent_t e : p->branch_ev)
    if (e) cudaEventDestroy(e);
  double* d[] = {p->Dr, p->D2r2, p->ir4r2, p->D2s, p->ir2s, p->D2A4, p->ir2A4, p->ir4A4, p->rsq, p->dT0,
                 p->gr, p->LinvA4, p->LinvT, p->LinvS, p->out4, p->rhs, p->xtmp, p->coefA4, p->coefT, p->coefS, p->ABA4, p->hbuf,
                 p->dbuf, p->cbuf, p->pbuf,
                 p->dg_ir, p->dg_tw, p->dg_wr, p->dg_nuw, p->dg_part, p->dg_out};
  for (double* x : d) cudaFree(x);
  for (ChunkSet& c : p->cs) free_chunk_set(c);
  cudaFree(p->Dr32); cudaFree(p->D2r232); cudaFree(p->ir4r232); cudaFree(p->D2s32);
  cudaFree(p->tcB); cudaFree(p->tc_err);
  for (float* x : p->Linv32) cudaFree(x);
  cudaFree(p->x32[0]); cudaFree(p->x32[1]); cudaFree(p->q32); cudaFree(p->g32);
  cudaFree(p->base_tmp);
  cudaFree(p->gridbuf);
  cudaFree(p->derivbuf);
  cudaFree(p->dcnt);
  solver_free(p);
  delete p;
}

// Tables of the chunked chains.  Within a chunk that starts with carried state s, the state before step
// k is Psi_k s + (its value from a zero start) and f_k = (zero-start f_k) + G_k s, with
//   psi (s = [f_e; bf_e], m = 2 nr):  G_k = C_k Psi_k, C_k = [A_k B_k];
//     Psi_{k+1} = [[I, 0], [bjt I, I]] Psi_k + [I; bj I] G_k   (f_e += f, bf_e += bj f + bjt f_e)
//   T/S (s = b, m = nr):  G_k = -w_k Linv_k Psi_k,  Psi_{k+1} = Psi_k + k_{k+1} G_k   (b += k f before
//     the next step, k = 2 dt (j+2) of that step, w = 0.5 for j = 0 else 1)
// with Psi = I at the chunk start, and Phi_c = Psi after the chunk's last step.  G is stored transposed
// per mode ([jj][m cols][ldl]) and Phi per (parity, chunk) ([m cols][ldm]).
static void matmul_rows(const double* A, const double* B, double* C, int n, int k, int m) {  // C = A B
  for (int i = 0; i < n; ++i) {
    double* c = C + (size_t)i * m;
    for (int j = 0; j < m; ++j) c[j] = 0.0;
    for (int l = 0; l < k; ++l) {
      const double a = A[(size_t)i * k + l];
      const double* b = B + (size_t)l * m;
      for (int j = 0; j < m; ++j) c[j] += a * b[j];
    }
  }
}

// Products of the parallel carry: P_{j,i} = Phi_{j-1} ... Phi_{i+1} for 2 <= j < nch, 0 <= i <= j-2,
// built as P_{j,j-2} = Phi_{j-1}, P_{j,i} = Phi_{j-1} P_{j-1,i}; stored transposed like Phi, row j after
// row j-1.  PhiT holds the Phi_c of both parities ([par][c][m cols][ldm]).
static void carry_products(const std::vector<double>& PhiT, int nch, int m, int ldm, std::vector<double>& out) {
  const int np = (nch - 1) * (nch - 2) / 2;
  const size_t blk = (size_t)m * ldm;
  out.assign((size_t)2 * std::max(np, 1) * blk, 0.0);
  std::vector<double> Phi((size_t)m * m), Q((size_t)m * m), R((size_t)m * m);
  std::vector<std::vector<double>> prev, cur;   // row-major P_{j-1,i}, P_{j,i}
  for (int par = 0; par < 2; ++par) {
    prev.clear();
    for (int j = 2; j < nch; ++j) {
      const double* src = PhiT.data() + ((size_t)par * nch + (j - 1)) * blk;   // Phi_{j-1}, transposed
      for (int i = 0; i < m; ++i)
        for (int col = 0; col < m; ++col) Phi[(size_t)i * m + col] = src[(size_t)col * ldm + i];
      cur.assign(j - 1, std::vector<double>());
      for (int i = 0; i <= j - 2; ++i) {
        if (i == j - 2) {
          cur[i] = Phi;
        } else {
          cur[i].resize((size_t)m * m);
          matmul_rows(Phi.data(), prev[i].data(), cur[i].data(), m, m, m);
        }
        double* dst = out.data() + ((size_t)par * np + (size_t)(j - 1) * (j - 2) / 2 + i) * blk;
        for (int r = 0; r < m; ++r)
          for (int col = 0; col < m; ++col) dst[(size_t)col * ldm + r] = cur[i][(size_t)r * m + col];
      }
      prev.swap(cur);
    }
  }
}

// One chunking of the three chains' tables (see matmul_rows above for G and Phi): products for the
// parallel carry (layout 3), else the per-chunk maps Phi_c (layout 2).
static int build_chunk_set(sdd_plan* p, int kc, bool products, const double* AB, const double* LinvT,
                           const double* LinvS, const double* cA, const double* cT, const double* cS,
                           ChunkSet* cs) {
  const int M = p->M, nr = p->nr, ldl = p->ldl, S = M / 2;
  const int nch = (S + kc - 1) / kc;
  cs->kc = kc;
  cs->nch = nch;
  cs->np = products ? (nch - 1) * (nch - 2) / 2 : 0;
  std::vector<double> Pr;
  {  // psi
    const int m = 2 * nr, ldm = p->ldmA;
    std::vector<double> G((size_t)M * m * ldl, 0.0), Phi((size_t)2 * nch * m * ldm, 0.0);
    std::vector<double> Psi((size_t)m * m), Gs((size_t)nr * m), C((size_t)nr * m);
    for (int par = 0; par < 2; ++par)
      for (int c = 0; c < nch; ++c) {
        std::fill(Psi.begin(), Psi.end(), 0.0);
        for (int i = 0; i < m; ++i) Psi[(size_t)i * m + i] = 1.0;
        for (int s = c * kc; s < std::min(S, (c + 1) * kc); ++s) {
          const int jj = par + 2 * s;
          const double* blk = AB + (size_t)jj * 2 * nr * ldl;
          for (int i = 0; i < nr; ++i)
            for (int col = 0; col < m; ++col) C[(size_t)i * m + col] = blk[(size_t)col * ldl + i];
          matmul_rows(C.data(), Psi.data(), Gs.data(), nr, m, m);
          for (int i = 0; i < nr; ++i)
            for (int col = 0; col < m; ++col) G[((size_t)jj * m + col) * ldl + i] = Gs[(size_t)i * m + col];
          const double bj = cA[4 * jj + 2], bjt = cA[4 * jj + 3];
          for (int i = 0; i < nr; ++i)
            for (int col = 0; col < m; ++col) {
              const double top = Psi[(size_t)i * m + col], g = Gs[(size_t)i * m + col];
              Psi[(size_t)(nr + i) * m + col] += bjt * top + bj * g;
              Psi[(size_t)i * m + col] = top + g;
            }
        }
        if (c + 1 < nch)
          for (int i = 0; i < m; ++i)
            for (int col = 0; col < m; ++col)
              Phi[(((size_t)par * nch + c) * m + col) * ldm + i] = Psi[(size_t)i * m + col];
      }
    int st;
    double* g = nullptr;
    double* t = nullptr;
    if ((st = upload(&g, G.data(), G.size()))) return st;
    cs->GA4 = g;
    if (products) {
      carry_products(Phi, nch, m, ldm, Pr);
      if ((st = upload(&t, Pr.data(), Pr.size()))) return st;
      cs->PA4 = t;
    } else {
      if ((st = upload(&t, Phi.data(), Phi.size()))) return st;
      cs->PhiA4 = t;
    }
  }
  for (int fld = 1; fld <= 2; ++fld) {  // T, S
    const int m = nr, ldm = p->ldmT;
    const double* Linv = fld == 1 ? LinvT : LinvS;
    const double* cf = fld == 1 ? cT : cS;
    std::vector<double> G((size_t)M * m * ldl, 0.0), Phi((size_t)2 * nch * m * ldm, 0.0);
    std::vector<double> Psi((size_t)m * m), Gs((size_t)nr * m);
    for (int par = 0; par < 2; ++par)
      for (int c = 0; c < nch; ++c) {
        std::fill(Psi.begin(), Psi.end(), 0.0);
        for (int i = 0; i < m; ++i) Psi[(size_t)i * m + i] = 1.0;
        for (int s = c * kc; s < std::min(S, (c + 1) * kc); ++s) {
          const int jj = par + 2 * s;
          matmul_rows(Linv + (size_t)jj * nr * nr, Psi.data(), Gs.data(), nr, nr, m);
          const double w = cf[4 * jj + 1];
          for (double& x : Gs) x *= -w;
          for (int i = 0; i < nr; ++i)
            for (int col = 0; col < m; ++col) G[((size_t)jj * m + col) * ldl + i] = Gs[(size_t)i * m + col];
          const double knext = (s + 1 < S) ? cf[4 * (jj + 2)] : 0.0;
          for (size_t e = 0; e < Psi.size(); ++e) Psi[e] += knext * Gs[e];
        }
        if (c + 1 < nch)
          for (int i = 0; i < m; ++i)
            for (int col = 0; col < m; ++col)
              Phi[(((size_t)par * nch + c) * m + col) * ldm + i] = Psi[(size_t)i * m + col];
      }
    int st;
    double* g = nullptr;
    double* t = nullptr;
    if ((st = upload(&g, G.data(), G.size()))) return st;
    (fld == 1 ? cs->GT : cs->GS) = g;
    if (products) {
      carry_products(Phi, nch, m, ldm, Pr);
      if ((st = upload(&t, Pr.data(), Pr.size()))) return st;
      (fld == 1 ? cs->PT : cs->PS) = t;
    } else {
      if ((st = upload(&t, Phi.data(), Phi.size()))) return st;
      (fld == 1 ? cs->PhiT : cs->PhiS) = t;
    }
  }
  return SDD_OK;
}

// Chunk lengths.  Layout 2 (sequential carry: kc local steps, then nch - 2 carried matvecs of twice the
// width, on one SM per chain): kc ~ sqrt(2S).  Layout 3 (parallel carry: kc local steps, then all
// (nch-1)(nch-2)/2 products at once, spread over the GPU): kc ~ sqrt(S/2), shorter chunks.
static int chunk_len(int S, int layout) {
  const double k = layout == 3 ? std::sqrt(0.5 * S) : std::sqrt(2.0 * S);
  return std::max(layout == 3 ? 2 : 4, std::min(layout == 3 ? 16 : 32, (int)std::lround(k)));
}

static int build_chunk_tables(sdd_plan* p, const double* AB, const double* LinvT, const double* LinvS,
                              const double* cA, const double* cT, const double* cS) {
  const int S = p->M / 2, nr = p->nr;
  p->ldmA = 2 * nr;
  p->ldmT = nr + (nr & 1);
  p->ldd = 2 * nr;
  int st;
  if ((st = build_chunk_set(p, chunk_len(S, 2), false, AB, LinvT, LinvS, cA, cT, cS, &p->cs[0])) ||
      (st = build_chunk_set(p, chunk_len(S, 3), true, AB, LinvT, LinvS, cA, cT, cS, &p->cs[1])))
    return st;
  p->nch_alloc = std::max(p->cs[0].nch, p->cs[1].nch);
  p->np_alloc = std::max(p->cs[1].np, 1);
  return SDD_OK;
}

// Diagnostics tables (Main.py:41-134): 1/R and trapezoid weights over the interior radii, trapezoid
// weight * sin(theta) on the 3M-point midpoint grid, Nusselt weights of the even modes, 1/(2V).  Left out
// (diagnostics unsupported) when the descriptor has no radii or 3M has no FFT plan.
static int build_diag_tables(sdd_plan* p, const sdd_plan_desc* d) {
  if (!d->nu_w || !d->r_int) return SDD_OK;
  const int M = p->M, nr = p->nr, L = 3 * M;
  const FftPlan* fp = get_fft_plan(L);
  int optin = 0;
  SDD_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device));
  if (!fp || diag_rows_smem_bytes(M, L) > (size_t)optin) return SDD_OK;
  std::vector<double> ir(nr), wr(nr, 0.0), tw(L), nuw((size_t)((M + 1) / 2) * nr);
  const double* x = d->r_int;
  for (int n = 0; n < nr; ++n) ir[n] = 1.0 / x[n];
  for (int n = 0; n + 1 < nr; ++n) {   // trapezoid over x = R[1:-1]
    const double hh = 0.5 * (x[n + 1] - x[n]);
    wr[n] += hh;
    wr[n + 1] += hh;
  }
  const double h = M_PI / L;          // midpoint grid theta_i = pi (2i+1) / (2L)
  for (int i = 0; i < L; ++i) {
    const double th = M_PI * (2.0 * i + 1.0) / (2.0 * L);
    const double w = (i == 0 || i == L - 1) ? 0.5 * h : h;
    tw[i] = w * std::sin(th);
  }
  for (int kk = 0; kk < (M + 1) / 2; ++kk) {
    const double k = 2.0 * kk;
    for (int m = 0; m < nr; ++m) nuw[(size_t)kk * nr + m] = d->nu_w[m] / (1.0 - k * k);
  }
  int st;
  if ((st = upload(&p->dg_ir, ir.data(), nr)) || (st = upload(&p->dg_wr, wr.data(), nr)) ||
      (st = upload(&p->dg_tw, tw.data(), L)) || (st = upload(&p->dg_nuw, nuw.data(), nuw.size())))
    return st;
  p->ke_scale = 0.5 / ((2.0 / 3.0) * (d->r_o * d->r_o * d->r_o - d->r_i * d->r_i * d->r_i));
  p->dfft = fp;
  return SDD_OK;
}

int sdd_plan_create(const sdd_plan_desc* d, sdd_plan** out) {
  if (!d || !out) return SDD_ERR_ARG;
  *out = nullptr;
  if (d->N_fm < 2 || d->nr < 1) return SDD_ERR_ARG;
  if (d->N_fm % 2 != 0) return SDD_ERR_ODD_NFM;
  if (d->nr > kMaxNr || d->N_fm > kMaxM) return SDD_ERR_UNSUPPORTED;
  if (d->precision != SDD_PREC_FP64 && d->precision != SDD_PREC_MIXED) return SDD_ERR_ARG;
  const int M = d->N_fm, nr = d->nr, P = (3 * M) / 2;
  int dev = 0;
  SDD_CUDA(cudaGetDevice(&dev));
  // the fused row kernel's dynamic shared memory within what the device leaves beside its static part; the
  // FP64 kernel is also needed by the mixed plan's Newton residual
  if (fx_smem_bytes(M, P, d->precision) > fx_rows_max_dynamic_smem(d->precision)) return SDD_ERR_UNSUPPORTED;
  if (fx_smem_bytes(M, P, SDD_PREC_FP64) > fx_rows_max_dynamic_smem(SDD_PREC_FP64)) return SDD_ERR_UNSUPPORTED;
  const FftPlan* fp = get_fft_plan(P);
  if (!fp) return SDD_ERR_UNSUPPORTED;
  sdd_plan* p = new sdd_plan();
  std::memset(p, 0, sizeof(*p));
  p->M = M; p->nr = nr; p->P = P; p->ldl = nr + (nr & 1); p->sym = d->symmetric ? 1 : 0;
  p->prec = d->precision; p->device = dev;
  p->reorth_eta = kReorthEta;
  p->dt = d->dt; p->Pr = d->Pr; p->Tau = d->Tau;
  p->fft = fp;
  const size_t nn = (size_t)nr * nr, nm = (size_t)M * nr * nr;
  int st = SDD_OK;
  if ((st = upload(&p->Dr, d->Dr, nn)) || (st = upload(&p->D2r2, d->D2_r2, nn)) ||
      (st = upload(&p->ir4r2, d->ir4_r2, nr)) || (st = upload(&p->D2s, d->D2_sine, nn)) ||
      (st = upload(&p->ir2s, d->ir2_sine, nr)) || (st = upload_linv(&p->D2A4, d->D2_A4, 1, nr, p->ldl)) ||
      (st = upload(&p->ir2A4, d->ir2_A4, nr)) || (st = upload(&p->ir4A4, d->ir4_A4, nr)) ||
      (st = upload(&p->rsq, d->rsq, nr)) || (st = upload(&p->dT0, d->dT0, nr)) ||
      (st = upload(&p->gr, d->gr, nr)) || (st = upload_linv(&p->LinvA4, d->Linv_A4, M, nr, p->ldl)) ||
      (st = upload_linv(&p->LinvT, d->Linv_T, M, nr, p->ldl)) ||
      (st = upload_linv(&p->LinvS, d->Linv_S, M, nr, p->ldl)) ||
      (st = upload32(&p->Dr32, d->Dr, nn)) || (st = upload32(&p->D2r232, d->D2_r2, nn)) ||
      (st = upload32(&p->ir4r232, d->ir4_r2, nr))) {
    free_plan(p);
    return st;
  }
  if (p->prec == SDD_PREC_MIXED &&
      ((st = upload32(&p->D2s32, d->D2_sine, nn)) ||
       (st = upload_linv32(&p->Linv32[0], d->Linv_A4, M, nr, p->ldl)) ||
       (st = upload_linv32(&p->Linv32[1], d->Linv_T, M, nr, p->ldl)) ||
       (st = upload_linv32(&p->Linv32[2], d->Linv_S, M, nr, p->ldl)))) {
    free_plan(p);
    return st;
  }
  if (p->prec == SDD_PREC_MIXED) {   // 3xTF32 operator tiles of the tensor-core contractions
    p->tcKP = p->tcNP = (nr + 7) / 8 * 8;
    std::vector<float> tb((size_t)2 * 2 * p->tcNP * p->tcKP);
    build_tc_operator(d->Dr, d->D2_r2, nr, p->tcKP, p->tcNP, tb.data());
    cudaError_t e = cudaMalloc(&p->tcB, tb.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(p->tcB, tb.data(), tb.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&p->tc_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(p->tc_err, 0, sizeof(int));
    if (e != cudaSuccess) {
      set_cuda_error(e);
      cudaGetLastError();
      free_plan(p);
      return e == cudaErrorMemoryAllocation ? SDD_ERR_NOMEM : SDD_ERR_CUDA;
    }
    p->use_tc = 1;
  }
  {  // per-step scalars of the chains (Matrix_Operators.py:1143-1159 and 1056-1083)
    std::vector<double> cA((size_t)M * 4), cT((size_t)M * 4), cS((size_t)M * 4);
    const double dA = d->Pr * d->dt, dT = d->dt, dS = d->Tau * d->dt;
    for (int jj = 0; jj < M; ++jj) {
      const double j = (double)(M - jj);
      const double bj = -j * (j + 1.0), bjt = -2.0 * j;
      cA[4 * jj] = dA * bjt;
      cA[4 * jj + 1] = dA * bjt * bj;
      cA[4 * jj + 2] = bj;
      cA[4 * jj + 3] = bjt;
      const double jc = (double)(M - 1 - jj);
      cT[4 * jj] = -dT * (-2.0 * (jc + 2.0));
      cS[4 * jj] = -dS * (-2.0 * (jc + 2.0));
      cT[4 * jj + 1] = cS[4 * jj + 1] = (M - 1 - jj == 0) ? 0.5 : 1.0;
      cT[4 * jj + 2] = cT[4 * jj + 3] = cS[4 * jj + 2] = cS[4 * jj + 3] = 0.0;
    }
    if ((st = upload(&p->coefA4, cA.data(), cA.size())) || (st = upload(&p->coefT, cT.data(), cT.size())) ||
        (st = upload(&p->coefS, cS.data(), cS.size()))) {
      free_plan(p);
      return st;
    }
    // psi chain step matrices (exact algebra of b_test, Matrix_Operators.py:1149-1157):
    //   A_j = Linv_j (c1 D2 + diag(alpha)), B_j = Linv_j diag(beta),
    //   c1 = dt bjt, alpha = c1 bj IR4 - bjt IR2, beta = c1 IR4;  stored transposed, [A B] per mode.
    const int ldl = p->ldl;
    std::vector<double> AB((size_t)M * 2 * nr * ldl, 0.0);
    std::vector<double> LD((size_t)nr * nr);
    for (int jj = 0; jj < M; ++jj) {
      const double c1 = cA[4 * jj], bj = cA[4 * jj + 2], bjt = cA[4 * jj + 3];
      const double* L = d->Linv_A4 + (size_t)jj * nr * nr;
      for (int i = 0; i < nr; ++i)
        for (int c = 0; c < nr; ++c) {
          double acc = 0.0;
          for (int k = 0; k < nr; ++k) acc += L[i * nr + k] * d->D2_A4[k * nr + c];
          LD[(size_t)i * nr + c] = acc;
        }
      double* blk = AB.data() + (size_t)jj * 2 * nr * ldl;
      for (int c = 0; c < nr; ++c) {
        const double alpha = c1 * bj * d->ir4_A4[c] - bjt * d->ir2_A4[c];
        const double beta = c1 * d->ir4_A4[c];
        for (int i = 0; i < nr; ++i) {
          blk[(size_t)c * ldl + i] = c1 * LD[(size_t)i * nr + c] + L[i * nr + c] * alpha;
          blk[(size_t)(nr + c) * ldl + i] = L[i * nr + c] * beta;
        }
      }
    }
    if ((st = upload(&p->ABA4, AB.data(), AB.size())) ||
        (st = build_chunk_tables(p, AB.data(), d->Linv_T, d->Linv_S, cA.data(), cT.data(), cS.data())) ||
        (st = build_diag_tables(p, d))) {
      free_plan(p);
      return st;
    }
    auto keep = [](const double* src, size_t n) {
      double* h = new double[n];
      std::memcpy(h, src, n * sizeof(double));
      return h;
    };
    p->h_AB = keep(AB.data(), AB.size());
    p->h_LinvT = keep(d->Linv_T, nm);
    p->h_LinvS = keep(d->Linv_S, nm);
    p->h_cA = keep(cA.data(), cA.size());
    p->h_cT = keep(cT.data(), cT.size());
    p->h_cS = keep(cS.data(), cS.size());
  }
  *out = p;
  return SDD_OK;
}

int sdd_plan_destroy(sdd_plan* p) {
  if (!p) return SDD_ERR_ARG;
  free_plan(p);
  return SDD_OK;
}

// Chunk length of chunk set `set` (0: the sequential-carry chunks of layouts 2 / 10, 1: the parallel-carry
// chunks of layouts 3 / 11): the set's tables are rebuilt on the host from the plan's copies and uploaded; the
// carry workspace follows on the next step (sdd_plan_reserve).  kc = 0 restores the plan's rule.
int sdd_plan_set_chunk_length(sdd_plan* p, int set, int kc) {
  if (!p || set < 0 || set > 1 || kc < 0 || !p->h_AB) return SDD_ERR_ARG;
  const int S = p->M / 2;
  if (kc == 0) kc = chunk_len(S, set == 1 ? 3 : 2);
  const int nch = (S + kc - 1) / kc;
  // at least two steps per chunk; the parallel carry's products grow as nch^2 / 2: at most 32 chunks
  if (kc < 2 || kc > S || (set == 1 && nch > 32) || nch > 64) return SDD_ERR_ARG;
  if (p->cs[set].kc == kc) return SDD_OK;
  clear_step_graphs(p);                    // the graphs bake in the tables' pointers
  SDD_CUDA(cudaDeviceSynchronize());      // no launch may still read the old tables
  ChunkSet c{};
  int st = build_chunk_set(p, kc, set == 1, p->h_AB, p->h_LinvT, p->h_LinvS, p->h_cA, p->h_cT, p->h_cS, &c);
  if (st) {
    free_chunk_set(c);
    return st;
  }
  free_chunk_set(p->cs[set]);
  p->cs[set] = c;
  const int nch_alloc = std::max(p->cs[0].nch, p->cs[1].nch), np_alloc = std::max(p->cs[1].np, 1);
  if (nch_alloc > p->nch_alloc || np_alloc > p->np_alloc) {
    p->nch_alloc = std::max(p->nch_alloc, nch_alloc);
    p->np_alloc = std::max(p->np_alloc, np_alloc);
    const int b = p->ws_batch;
    p->ws_batch = 0;                       // regrow the chunk workspace for the batch already reserved
    if (b > 0 && (st = sdd_plan_reserve(p, b))) return st;
  }
  return SDD_OK;
}

int sdd_plan_set_fx_split(sdd_plan* p, int mode) {
  if (!p || mode < 0 || mode > 2) return SDD_ERR_ARG;
  if (p->fx_split != mode) clear_step_graphs(p);
  p->fx_split = mode;
  return SDD_OK;
}

int sdd_plan_set_tensor_cores(sdd_plan* p, int on) {
  if (!p || on < 0 || on > 1) return SDD_ERR_ARG;
  if (on && !p->tcB) return SDD_ERR_UNSUPPORTED;
  if (p->use_tc != on) clear_step_graphs(p);   // the captured graphs hold the other kernels
  p->use_tc = on;
  return SDD_OK;
}

int sdd_plan_tensor_core_status(const sdd_plan* p, int* timed_out) {
  if (!p || !timed_out) return SDD_ERR_ARG;
  *timed_out = 0;
  if (p->tc_err) SDD_CUDA(cudaMemcpy(timed_out, p->tc_err, sizeof(int), cudaMemcpyDeviceToHost));
  return SDD_OK;
}

int sdd_plan_set_product_graphs(sdd_plan* p, int on) {
  if (!p || on < 0 || on > 1) return SDD_ERR_ARG;
  p->mv_graphs_off = !on;
  return SDD_OK;
}

int sdd_plan_product_graph_stats(const sdd_plan* p, long long* captured, long long* replayed, long long* direct) {
  if (!p || !captured || !replayed || !direct) return SDD_ERR_ARG;
  *captured = p->mv_count[0];
  *replayed = p->mv_count[1];
  *direct = p->mv_count[2];
  return SDD_OK;
}

int sdd_plan_set_reorth_eta(sdd_plan* p, double eta) {
  if (!p || !(eta >= 0.0)) return SDD_ERR_ARG;
  p->reorth_eta = eta;
  return SDD_OK;
}

int sdd_krylov_basis(const sdd_plan* p, int shell, int max_cols, double* out, int* ncols, void* stream) {
  if (!p || !out || !ncols || max_cols < 1 || shell < 0 || shell >= p->kv_last_B || !p->kv_V) return SDD_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int B = p->kv_last_B;
  int kb = 0;
  SDD_CUDA(cudaMemcpyAsync(&kb, p->kv_ismall + 2 * (size_t)B + shell, sizeof(int), cudaMemcpyDeviceToHost, s));
  SDD_CUDA(cudaStreamSynchronize(s));
  const size_t n = (size_t)3 * p->M * p->nr, ld = n + 1, vs = (size_t)B * ld;
  const int c = kb < max_cols ? kb : max_cols;
  for (int j = 0; j < c; ++j) {
    if (p->kv_basis32) {   // FP32 basis: widened to FP64 on the way out
      const float* src = reinterpret_cast<const float*>(p->kv_V) + (size_t)j * vs + (size_t)shell * ld;
      SDD_CUDA(krylov_widen(src, out + (size_t)j * n, n, s));
    } else {
      SDD_CUDA(cudaMemcpyAsync(out + (size_t)j * n, p->kv_V + (size_t)j * vs + (size_t)shell * ld,
                               n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    }
  }
  *ncols = c;
  return SDD_OK;
}

int sdd_plan_set_chain_layout(sdd_plan* p, int layout) {
  if (!p || layout < 0 || layout > 11) return SDD_ERR_ARG;
  if (p->chain_layout != layout) clear_step_graphs(p);
  p->chain_layout = layout;
  return SDD_OK;
}

static ChainArgs chain_args(const sdd_plan* p, const double* g, double* f, const double* sub);
static ChainArgs step_chain_args(const sdd_plan* p, int batch);

int sdd_plan_chain_choice(const sdd_plan* p, int batch, int* layout, int* kc, int* nch) {
  if (!p || batch < 1 || !layout || !kc || !nch) return SDD_ERR_ARG;
  const ChainArgs a = step_chain_args(p, batch);
  *layout = resolve_chain_layout(a, batch, 3);
  const bool chunked = *layout == 2 || *layout == 3 || *layout == 10 || *layout == 11;
  const int set = (*layout == 3 || *layout == 11) ? 1 : 0;
  *kc = chunked ? p->cs[set].kc : 0;
  *nch = chunked ? p->cs[set].nch : 1;
  return SDD_OK;
}

size_t sdd_plan_base_cache_elems(const sdd_plan* p) { return p ? (size_t)9 * p->nr * p->P : 0; }

static size_t shell_elems(const sdd_plan* p) { return (size_t)3 * p->M * p->nr; }


int sdd_plan_reserve(sdd_plan* p, int max_batch) {
  if (!p || max_batch < 1) return SDD_ERR_ARG;
  if (max_batch <= p->ws_batch) return SDD_OK;
  clear_step_graphs(p);   // the graphs bake in the workspace pointers
  cudaFree(p->out4); cudaFree(p->rhs); cudaFree(p->xtmp); cudaFree(p->base_tmp); cudaFree(p->hbuf);
  cudaFree(p->dbuf); cudaFree(p->cbuf); cudaFree(p->gridbuf); cudaFree(p->derivbuf);
  cudaFree(p->dg_part); cudaFree(p->dg_out); cudaFree(p->dcnt); cudaFree(p->pbuf);
  cudaFree(p->x32[0]); cudaFree(p->x32[1]); cudaFree(p->q32); cudaFree(p->g32);
  p->x32[0] = p->x32[1] = nullptr;
  p->q32 = p->g32 = nullptr;
  p->dg_part = p->dg_out = nullptr;
  p->dcnt = nullptr;
  p->pbuf = nullptr;
  p->out4 = p->rhs = p->xtmp = p->hbuf = p->dbuf = p->cbuf = nullptr;
  p->base_tmp = p->gridbuf = p->derivbuf = nullptr;
  p->ws_batch = 0;
  const size_t se = shell_elems(p);
  const size_t be = sdd_plan_base_cache_elems(p);
  SDD_CUDA(ws_malloc(&p->out4, (size_t)max_batch * 4 * p->M * p->nr * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->rhs, (size_t)max_batch * se * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->xtmp, (size_t)max_batch * se * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->hbuf, (size_t)max_batch * se * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->base_tmp, (size_t)max_batch * be * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->gridbuf, (size_t)max_batch * be * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->derivbuf, (size_t)max_batch * 5 * p->M * p->nr * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->dg_part, (size_t)max_batch * p->nr * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->dg_out, (size_t)max_batch * 4 * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->dcnt, (size_t)max_batch * 6 * sizeof(int)));
  SDD_CUDA(cudaMemset(p->dcnt, 0, (size_t)max_batch * 6 * sizeof(int)));
  const size_t de = (size_t)6 * p->nch_alloc * p->ldd;
  SDD_CUDA(ws_malloc(&p->dbuf, (size_t)max_batch * de * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->cbuf, (size_t)max_batch * de * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->pbuf, (size_t)max_batch * 6 * p->np_alloc * p->ldd * sizeof(double)));
  if (p->prec == SDD_PREC_MIXED) {
    for (float*& x : p->x32) SDD_CUDA(ws_malloc(&x, (size_t)max_batch * se * sizeof(float)));
    SDD_CUDA(ws_malloc(&p->q32, (size_t)max_batch * p->M * p->nr * sizeof(float)));
    SDD_CUDA(ws_malloc(&p->g32, (size_t)max_batch * se * sizeof(float)));
  }
  p->ws_batch = max_batch;
  return SDD_OK;
}

}  // extern "C"

// ---- internal launch helpers ---------------------------------------------------------------------
static FxArgs fx_args(const sdd_plan* p, int prec, const double* X, void* base, double* out4) {
  FxArgs a;
  std::memset(&a, 0, sizeof(a));
  a.M = p->M; a.nr = p->nr; a.P = p->P; a.sym = p->sym;
  a.st = stage_args(p->fft);
  if (prec == SDD_PREC_MIXED) {
    a.ops.Dr = p->Dr32; a.ops.D2r2 = p->D2r232; a.ops.ir4r2 = p->ir4r232;
    a.ops.w = p->fft->w32; a.ops.e = p->fft->e32;
  } else {
    a.ops.Dr = p->Dr; a.ops.D2r2 = p->D2r2; a.ops.ir4r2 = p->ir4r2;
    a.ops.w = p->fft->w64; a.ops.e = p->fft->e64;
  }
  a.X = X; a.x_stride = shell_elems(p);
  a.base = base; a.base_stride = sdd_plan_base_cache_elems(p);
  a.out4 = out4; a.out_stride = (size_t)4 * p->M * p->nr;
  a.grid = p->gridbuf; a.grid_stride = sdd_plan_base_cache_elems(p);
  a.split = p->fx_split;
  // per shell: 4 M nr elements of the precision, then M nr doubles (the fused rhs's D2s psi)
  a.deriv = p->derivbuf;
  a.deriv_stride = (size_t)(prec == SDD_PREC_MIXED ? 6 : 5) * p->M * p->nr;
  if (prec == SDD_PREC_MIXED && p->use_tc) {
    a.tcB = p->tcB;
    a.tcKP = p->tcKP;
    a.tcNP = p->tcNP;
    a.tc_err = p->tc_err;
  }
  return a;
}

static RhsArgs rhs_args(const sdd_plan* p, const double* X, const double* out4, const double* Ra,
                        const double* Ras, double* rhs, int linear) {
  RhsArgs a;
  std::memset(&a, 0, sizeof(a));
  a.M = p->M; a.nr = p->nr; a.sym = p->sym; a.linear = linear;
  a.dt = p->dt; a.Pr = p->Pr;
  a.Dr = p->Dr; a.D2s = p->D2s; a.ir2s = p->ir2s; a.rsq = p->rsq; a.dT0 = p->dT0; a.gr = p->gr;
  a.X = X; a.x_stride = shell_elems(p);
  a.out4 = out4; a.out_stride = (size_t)4 * p->M * p->nr;
  a.Ra = Ra; a.Ra_s = Ras;
  a.rhs = rhs; a.rhs_stride = shell_elems(p);
  return a;
}

static ChainArgs chain_args(const sdd_plan* p, const double* g, double* f, const double* sub) {
  ChainArgs a;
  std::memset(&a, 0, sizeof(a));
  a.M = p->M; a.nr = p->nr; a.ldl = p->ldl; a.sym = p->sym; a.field0 = 0; a.layout = p->chain_layout;
  a.field_off = (size_t)p->M * p->nr;
  a.g = g; a.g_stride = shell_elems(p);
  a.f = f; a.f_stride = shell_elems(p);
  a.sub = sub; a.sub_stride = shell_elems(p);
  a.LinvA4 = p->LinvA4; a.LinvT = p->LinvT; a.LinvS = p->LinvS;
  a.ABA4 = p->ABA4; a.D2A4 = p->D2A4; a.ir2A4 = p->ir2A4; a.ir4A4 = p->ir4A4;
  a.h = p->hbuf;
  a.h_stride = shell_elems(p);
  a.coefA4 = p->coefA4; a.coefT = p->coefT; a.coefS = p->coefS;
  a.dtA4 = p->Pr * p->dt; a.dtT = p->dt; a.dtS = p->Tau * p->dt;
  a.ldmA = p->ldmA; a.ldmT = p->ldmT; a.ldd = p->ldd;
  a.cset[0] = p->cs[0];
  a.cset[1] = p->cs[1];
  a.dbuf = p->dbuf; a.cbuf = p->cbuf; a.counter = p->dcnt;
  a.d_stride = (size_t)6 * p->nch_alloc * p->ldd;
  a.pbuf = p->pbuf;
  a.p_stride = (size_t)6 * p->np_alloc * p->ldd;
  return a;
}

static int check_plan(sdd_plan* p, int batch) {
  if (!p || batch < 1) return SDD_ERR_ARG;
  int dev = 0;
  SDD_CUDA(cudaGetDevice(&dev));
  if (dev != p->device) return SDD_ERR_ARG;
  return sdd_plan_reserve(p, batch);
}

// One application of Phi (the step map) or its Jacobian to X (or dv), into out.
// mode 0: FX (nonlinear term of X); 1: DFX about the base in `base`; 2: linear only.
// Same as apply_step with explicit strides (doubles between shells) of the input X, the output and sub.
// With the split nonlinear term, the right-hand sides are not assembled by k_rhs: the grid kernel writes
// their linear parts (FP64 in both precisions) and the chains' h kernel adds the nonlinear parts (same
// roundings).
// ev (nullable): four events recorded around the nonlinear term, the rhs and the chains.
// The pending correction of layouts 3 / 11 (chunk set 1) of a state X (and its FP32 copy x32, nullable),
// for FixArgs.
static FixArgs fix_args(const sdd_plan* p, const double* X, const float* x32) {
  FixArgs f;
  std::memset(&f, 0, sizeof(f));
  const ChunkSet& c = p->cs[1];
  f.on = 1;
  f.kc = c.kc; f.nch = c.nch; f.np = c.np; f.ldd = p->ldd; f.ldl = p->ldl;
  f.GA4 = c.GA4; f.GT = c.GT; f.GS = c.GS;
  f.dbuf = p->dbuf; f.pbuf = p->pbuf;
  f.d_stride = (size_t)6 * p->nch_alloc * p->ldd;
  f.p_stride = (size_t)6 * p->np_alloc * p->ldd;
  f.X = const_cast<double*>(X);
  f.X32 = const_cast<float*>(x32);
  return f;
}

// x32_in / x32_out (mixed time steps only): the FP32 copy of X the nonlinear term reads instead of
// converting X, and the one the chains write beside out for the next step (nullable).  defer: leave a
// layout-3 / 11 chain correction pending (sdd_step); fix_in: X carries the previous step's pending correction,
// applied by the nonlinear term's first kernel.  v32 (mixed plans, mode 1, nullable): an FP32 copy of X
// (stride ldx), read by the FP32 nonlinear term instead of converting X (the same values); with v32_rhs
// the right-hand sides and h = Linv g are then formed in FP32 as well (k_rhs32, k_mode_mv32), for Jacobian
// products inside a GMRES solve whose tolerance is far above FP32 rounding.
static int apply_step_ld(sdd_plan* p, int batch, const double* Ra, const double* Ras, const double* X, size_t ldx,
                         double* out, size_t ldo, const double* sub, size_t lds, int mode, void* base, int prec,
                         cudaStream_t s, cudaEvent_t* ev = nullptr, const float* x32_in = nullptr,
                         float* x32_out = nullptr, const int* active = nullptr, int defer = 0, int fix_in = 0,
                         const float* v32 = nullptr, bool v32_rhs = true) {
  RhsArgs ra = rhs_args(p, X, p->out4, Ra, Ras, p->rhs, mode == 2);
  ra.x_stride = ldx;
  ra.active = active;
  if (prec == SDD_PREC_MIXED && mode != 2) {   // the FP32 nonlinear term's Q, for an FP32 Dr Q
    ra.q32 = p->q32;
    ra.Dr32 = p->Dr32;
  }
  bool fuse = false;
  if (ev) SDD_CUDA(cudaEventRecord(ev[0], s));
  if (mode != 2) {
    FxArgs fa = fx_args(p, prec, X, base, p->out4);
    fa.x_stride = ldx;
    fa.active = active;
    if (prec == SDD_PREC_MIXED && mode == 0) {
      fa.X32 = x32_in;
      fa.x32_stride = shell_elems(p);
    }
    if (prec == SDD_PREC_MIXED && mode == 1 && v32) {   // the Krylov vector's FP32 copy: no conversions
      fa.X32 = v32;
      fa.x32_stride = ldx;
    }
    if (prec == SDD_PREC_MIXED) fa.q32 = p->q32;
    const int fm = mode == 1 ? 1 : 0;
    fuse = fx_uses_split(fa, batch, fm);
    if (fix_in) {
      if (!fuse || mode != 0) return SDD_ERR_ARG;   // only the split path's derivative kernel applies it
      fa.fix = fix_args(p, X, x32_in);
    }
    if (fuse) {
      fa.fuse_rhs = 1;
      fa.rl = ra;
    }
    SDD_CUDA(launch_fx(fa, batch, fm, prec, s));
  }
  if (ev) SDD_CUDA(cudaEventRecord(ev[1], s));
  const bool rhs32 = v32 && v32_rhs && mode == 1 && prec == SDD_PREC_MIXED && !fuse && p->g32 && ra.q32;
  if (rhs32) {
    ra.X32 = v32;
    ra.x32_stride = ldx;
    ra.rhs32 = p->g32;
    ra.D2s32 = p->D2s32;
  }
  if (!fuse) SDD_CUDA(launch_rhs(ra, batch, s));
  if (ev) SDD_CUDA(cudaEventRecord(ev[2], s));
  ChainArgs ca = chain_args(p, p->rhs, out, sub);
  ca.f_stride = ldo;
  ca.sub_stride = lds;
  ca.active = active;
  ca.defer_fix = defer && mode == 0 && !sub;
  if (rhs32) {
    ca.g32 = p->g32;
    ca.Linv32A4 = p->Linv32[0]; ca.Linv32T = p->Linv32[1]; ca.Linv32S = p->Linv32[2];
  }
  if (prec == SDD_PREC_MIXED && mode == 0 && !sub) {
    ca.f32 = x32_out;
    ca.f32_stride = shell_elems(p);
  }
  if (fuse) {
    ca.fuse_rhs = 1;
    ca.lin = p->rhs;
    ca.out4 = p->out4;
    ca.out_stride = (size_t)4 * p->M * p->nr;
    ca.Dr = p->Dr;
    ca.q32 = ra.q32;
    ca.Dr32 = ra.Dr32;
    ca.dt = p->dt;
  }
  SDD_CUDA(launch_chain(ca, batch, 3, s));
  if (ev) SDD_CUDA(cudaEventRecord(ev[3], s));
  return SDD_OK;
}

static int apply_step(sdd_plan* p, int batch, const double* Ra, const double* Ras, const double* X,
                      double* out, const double* sub, int mode, void* base, int prec, cudaStream_t s,
                      const float* x32_in = nullptr, float* x32_out = nullptr, int defer = 0, int fix_in = 0) {
  const size_t n = shell_elems(p);
  return apply_step_ld(p, batch, Ra, Ras, X, n, out, n, sub, n, mode, base, prec, s, nullptr, x32_in, x32_out,
                       nullptr, defer, fix_in);
}

// The chain arguments of a plain step of `batch` shells as sdd_step launches them: the right-hand side fused
// into the split nonlinear term when the step runs that form, so that the layout resolves as in the step.
// The step reserves its scratch (the grid and derivative buffers the split form needs) before it launches,
// so the rule is applied as if they were there.
static ChainArgs step_chain_args(const sdd_plan* p, int batch) {
  ChainArgs ca = chain_args(p, nullptr, nullptr, nullptr);
  ca.fuse_rhs = fx_split_rule(p->fx_split, p->nr, batch) ? 1 : 0;
  return ca;
}

// Whether sdd_step's steps leave the chains' correction to the next step's nonlinear term: layout 3 or 11
// (chunk set 1, parallel carries) with the split nonlinear term, non-linear steps.
static bool step_defers_fix(sdd_plan* p, int batch, int linear) {
  if (linear || p->cs[1].nch < 2) return false;
  const ChainArgs ca = step_chain_args(p, batch);
  const int layout = resolve_chain_layout(ca, batch, 3);
  return ca.fuse_rhs && (layout == 3 || layout == 11);
}

// The correction left pending by the last step of a sequence, on the state X (and its FP32 copy).
static int finish_fix(sdd_plan* p, int batch, double* X, float* x32, cudaStream_t s) {
  ChainArgs ca = chain_args(p, nullptr, X, nullptr);
  ca.f32 = x32;
  ca.f32_stride = shell_elems(p);
  SDD_CUDA(launch_chunk_fix(ca, batch, 3, s));
  return SDD_OK;
}

extern "C" {

int sdd_nlin_fx(sdd_plan* p, int batch, const double* X, double* F, double* base_cache, void* stream) {
  int st = check_plan(p, batch);
  if (st) return st;
  if (!X || !F) return SDD_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  FxArgs fa = fx_args(p, SDD_PREC_FP64, X, base_cache, p->out4);
  SDD_CUDA(launch_fx(fa, batch, 0, SDD_PREC_FP64, s));
  SDD_CUDA(launch_fx_finish(p->M, p->nr, p->Dr, p->out4, (size_t)4 * p->M * p->nr, F, shell_elems(p),
                            batch, s));
  return SDD_OK;
}

int sdd_nlin_dfx(sdd_plan* p, int batch, const double* dv, const double* X, const double* base_cache,
                 double* out, void* stream) {
  int st = check_plan(p, batch);
  if (st) return st;
  if (!dv || !out || (!X && !base_cache)) return SDD_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  void* base = const_cast<double*>(base_cache);
  if (!base) {
    FxArgs ga = fx_args(p, SDD_PREC_FP64, X, p->base_tmp, p->out4);
    SDD_CUDA(launch_fx(ga, batch, 2, SDD_PREC_FP64, s));
    base = p->base_tmp;
  }
  FxArgs fa = fx_args(p, SDD_PREC_FP64, dv, base, p->out4);
  SDD_CUDA(launch_fx(fa, batch, 1, SDD_PREC_FP64, s));
  SDD_CUDA(launch_fx_finish(p->M, p->nr, p->Dr, p->out4, (size_t)4 * p->M * p->nr, out, shell_elems(p),
                            batch, s));
  return SDD_OK;
}

int sdd_a4_bsub(sdd_plan* p, int batch, const double* g, double* f, void* stream) {
  if (!g || !f) return SDD_ERR_ARG;
  int st = check_plan(p, batch);
  if (st) return st;
  ChainArgs a = chain_args(p, g, f, nullptr);
  a.g_stride = a.f_stride = (size_t)p->M * p->nr;
  a.field0 = 0;
  a.field_off = 0;
  SDD_CUDA(launch_chain(a, batch, 1, (cudaStream_t)stream));
  return SDD_OK;
}

int sdd_nab2_bsub(sdd_plan* p, int field, int batch, const double* g, double* f, void* stream) {
  if (!g || !f || (field != 1 && field != 2)) return SDD_ERR_ARG;
  int st = check_plan(p, batch);
  if (st) return st;
  const size_t N = (size_t)p->M * p->nr;
  ChainArgs a = chain_args(p, g, f, nullptr);
  a.g_stride = a.f_stride = N;
  a.field0 = field;
  a.field_off = 0;
  SDD_CUDA(launch_chain(a, batch, 1, (cudaStream_t)stream));
  return SDD_OK;
}

int sdd_theta_op(sdd_plan* p, int op, int batch, const double* g, double* f, void* stream) {
  if (!p || batch < 1 || !g || !f || op < 0 || op > 3) return SDD_ERR_ARG;
  const double* D2 = op == 1 ? p->D2r2 : p->D2s;
  const double* ir = op == 1 ? p->ir4r2 : p->ir2s;
  SDD_CUDA(launch_theta_op(op, p->M, p->nr, p->sym, D2, ir, p->dT0, g, f, batch, (cudaStream_t)stream));
  return SDD_OK;
}

// The instantiated graph of `pairs` step pairs A -> xtmp -> A, captured on first use on the plan's private
// stream (thread-local capture mode, so other host threads are unaffected).  Returns nullptr when it
// cannot be built; the caller then launches the steps one by one.
static cudaGraphExec_t step_graph(sdd_plan* p, int batch, const double* Ra, const double* Ras, double* A, int pairs,
                                  int linear) {
  StepGraph* slot = nullptr;
  for (int i = 0; i < kStepGraphs; ++i) {
    StepGraph& g = p->graphs[i];
    if (g.exec && g.A == A && g.Ra == Ra && g.Ras == Ras && g.batch == batch && g.linear == linear &&
        g.pairs == pairs && g.layout == p->chain_layout && g.fx_split == p->fx_split) {
      g.last_use = ++p->graph_clock;
      return g.exec;
    }
    if (!slot || !g.exec || (slot->exec && g.last_use < slot->last_use)) slot = &g;
  }
  if (!p->cap_stream && cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
    p->cap_stream = nullptr;
    cudaGetLastError();
    return nullptr;
  }
  cudaStream_t cs = p->cap_stream;
  if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  int st = SDD_OK;
  // mixed: A's FP32 copy is current (the graph runs after a step into A); each step writes the other's.
  // With deferred corrections every step applies its input's pending one and leaves its own.
  float* a32 = linear ? nullptr : p->x32[0];
  float* t32 = linear ? nullptr : p->x32[1];
  const int dfix = step_defers_fix(p, batch, linear) ? 1 : 0;
  for (int i = 0; i < pairs && st == SDD_OK; ++i) {
    st = apply_step(p, batch, Ra, Ras, A, p->xtmp, nullptr, linear ? 2 : 0, nullptr, p->prec, cs, a32, t32, dfix,
                    dfix);
    if (st == SDD_OK)
      st = apply_step(p, batch, Ra, Ras, p->xtmp, A, nullptr, linear ? 2 : 0, nullptr, p->prec, cs, t32, a32, dfix,
                      dfix);
  }
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(cs, &graph);
  cudaGraphExec_t exec = nullptr;
  if (st != SDD_OK || ec != cudaSuccess || !graph || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
  if (graph) cudaGraphDestroy(graph);
  cudaGetLastError();
  if (!exec) return nullptr;
  if (slot->exec) cudaGraphExecDestroy(slot->exec);
  *slot = StepGraph{exec, A, Ra, Ras, batch, linear, pairs, p->chain_layout, p->fx_split, ++p->graph_clock};
  return exec;
}

int sdd_step(sdd_plan* p, int batch, const double* Ra, const double* Ras, const double* X_in, double* X_out,
             int nsteps, int linear, void* stream) {
  int st = check_plan(p, batch);
  if (st) return st;
  if (!Ra || !Ras || !X_in || !X_out || nsteps < 0) return SDD_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = (size_t)batch * shell_elems(p) * sizeof(double);
  if (nsteps == 0) {
    if (X_out != X_in) SDD_CUDA(cudaMemcpyAsync(X_out, X_in, bytes, cudaMemcpyDeviceToDevice, s));
    return SDD_OK;
  }
  // ping-pong so that the last step lands in X_out; mixed plans keep an FP32 copy of each step's output
  // for the next step's nonlinear term (the caller's X_in has none)
  const double* cur = X_in;
  const float* cur32 = nullptr;
  // layout 3 or 11 with the split nonlinear term: each step's chain correction is applied by the next step's
  // first kernel (one launch fewer per step); the last one runs on its own at the end
  const int dfix = step_defers_fix(p, batch, linear) ? 1 : 0;
  cudaStreamCaptureStatus cst = cudaStreamCaptureStatusNone;
  SDD_CUDA(cudaStreamIsCapturing(s, &cst));
  const bool graphs = cst == cudaStreamCaptureStatusNone && nsteps >= kGraphMinSteps && X_out != p->xtmp;
  for (int it = 0; it < nsteps; ++it) {
    const int left = nsteps - it;  // steps remaining including this one
    if (graphs && it > 0 && cur == X_out && left % 2 == 0) {
      // the remaining steps are A -> xtmp -> A pairs: replay captured graphs of 8 pairs, then of 1 pair
      const int npairs = left / 2;
      cudaGraphExec_t g8 = npairs >= 8 ? step_graph(p, batch, Ra, Ras, X_out, 8, linear) : nullptr;
      cudaGraphExec_t g1 = step_graph(p, batch, Ra, Ras, X_out, 1, linear);
      if (g1 && (g8 || npairs < 8)) {
        int done = 0;
        for (; g8 && done + 8 <= npairs; done += 8) SDD_CUDA(cudaGraphLaunch(g8, s));
        for (; done < npairs; ++done) SDD_CUDA(cudaGraphLaunch(g1, s));
        return dfix ? finish_fix(p, batch, X_out, linear ? nullptr : p->x32[0], s) : SDD_OK;
      }
    }
    double* dst = (left % 2 == 1) ? X_out : p->xtmp;
    if (dst == cur) dst = (dst == X_out) ? p->xtmp : X_out;  // never write the input in place
    float* dst32 = linear ? nullptr : p->x32[dst == p->xtmp ? 1 : 0];
    st = apply_step(p, batch, Ra, Ras, cur, dst, nullptr, linear ? 2 : 0, nullptr, p->prec, s, cur32, dst32, dfix,
                    dfix && it > 0);
    if (st) return st;
    cur = dst;
    cur32 = dst32;
  }
  if (dfix && (st = finish_fix(p, batch, const_cast<double*>(cur), const_cast<float*>(cur32), s))) return st;
  if (cur != X_out) SDD_CUDA(cudaMemcpyAsync(X_out, cur, bytes, cudaMemcpyDeviceToDevice, s));
  return SDD_OK;
}

// Several plans' shells advanced in one call (the C form of a batch of uneven shells: one plan per shape
// group): every group runs sdd_step on its plan's own branch stream, forked from and joined back into the
// caller's stream by events, so the groups run concurrently and the call is stream-ordered like sdd_step.
// On a stream that is being captured the fork and join become graph dependencies (one graph with a branch
// per group).  A plan may appear once per call (its workspace serves one stream at a time).
int sdd_batch_step(const sdd_batch_group* groups, int ngroups, int nsteps, int linear, void* stream) {
  if (!groups || ngroups < 1 || nsteps < 0) return SDD_ERR_ARG;
  for (int g = 0; g < ngroups; ++g) {
    const sdd_batch_group& q = groups[g];
    if (!q.plan || q.batch < 1 || !q.Ra || !q.Ra_s || !q.X_in || !q.X_out) return SDD_ERR_ARG;
    for (int h = 0; h < g; ++h)
      if (groups[h].plan == q.plan) return SDD_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  for (int g = 0; g < ngroups; ++g) {
    sdd_plan* p = groups[g].plan;
    if (!p->branch_stream) SDD_CUDA(cudaStreamCreateWithFlags(&p->branch_stream, cudaStreamNonBlocking));
    for (cudaEvent_t& e : p->branch_ev)
      if (!e) SDD_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  cudaEvent_t fork = groups[0].plan->branch_ev[0];
  SDD_CUDA(cudaEventRecord(fork, s));
  int st = SDD_OK;
  for (int g = 0; g < ngroups && st == SDD_OK; ++g) {
    const sdd_batch_group& q = groups[g];
    cudaStream_t bs = q.plan->branch_stream;
    cudaError_t e = cudaStreamWaitEvent(bs, fork, 0);
    if (e != cudaSuccess) {
      set_cuda_error(e);
      st = SDD_ERR_CUDA;
      break;
    }
    st = sdd_step(q.plan, q.batch, q.Ra, q.Ra_s, q.X_in, q.X_out, nsteps, linear, bs);
    // the join is recorded whatever the step returned, so that the caller's stream (and a capture on it)
    // never ends with a branch left open
    e = cudaEventRecord(q.plan->branch_ev[1], bs);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, q.plan->branch_ev[1], 0);
    if (e != cudaSuccess && st == SDD_OK) {
      set_cuda_error(e);
      st = SDD_ERR_CUDA;
    }
  }
  return st;
}

// Crank-Nicolson / Adams-Bashforth 2 step (no counterpart in the reference, which steps IMEX Euler): the plan
// holds the operators of dt/2, the step is dt = 2 plan dt.  psi' = A4_BSub_{dt/2}(2 A2 psi + dt E~) - psi,
// T' = NAB2_BSub_{dt/2}(2 r^2 T + dt E~_T) - T (and S with Tau), E~ = 3/2 E - 1/2 E_prev (E when !hist_valid).
int sdd_step_cnab2(sdd_plan* p, int batch, const double* Ra, const double* Ras, const double* X_in, double* X_out,
                   double* hist, int hist_valid, void* stream) {
  int st = check_plan(p, batch);
  if (st) return st;
  if (!Ra || !Ras || !X_in || !X_out || !hist || X_in == X_out || hist == X_in || hist == X_out) return SDD_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  FxArgs fa = fx_args(p, p->prec, X_in, nullptr, p->out4);
  if (p->prec == SDD_PREC_MIXED) fa.q32 = p->q32;
  SDD_CUDA(launch_fx(fa, batch, 0, p->prec, s));
  RhsArgs ra = rhs_args(p, X_in, p->out4, Ra, Ras, p->rhs, 0);
  ra.dt = 2.0 * p->dt;
  if (p->prec == SDD_PREC_MIXED) {
    ra.q32 = p->q32;
    ra.Dr32 = p->Dr32;
  }
  ra.cnab2 = 1;
  ra.hist_valid = hist_valid ? 1 : 0;
  ra.hist = hist;
  SDD_CUDA(launch_rhs(ra, batch, s));
  ChainArgs ca = chain_args(p, p->rhs, X_out, X_in);   // the chains' "f -= sub": minus the old state
  SDD_CUDA(launch_chain(ca, batch, 3, s));
  return SDD_OK;
}

int sdd_pfx(sdd_plan* p, int batch, const double* Ra, const double* Ras, const double* X, double* F,
            double* base_cache, void* stream) {
  int st = check_plan(p, batch);
  if (st) return st;
  if (!Ra || !Ras || !X || !F || X == F) return SDD_ERR_ARG;
  // the residual is always FP64 (also for mixed plans)
  return apply_step(p, batch, Ra, Ras, X, F, X, 0, base_cache, SDD_PREC_FP64, (cudaStream_t)stream);
}

int sdd_pdfx(sdd_plan* p, int batch, const double* Ra, const double* Ras, const double* dv, const double* X,
             const double* base_cache, double* out, void* stream) {
  int st = check_plan(p, batch);
  if (st) return st;
  if (!Ra || !Ras || !dv || !out || dv == out || (!X && !base_cache)) return SDD_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  void* base = const_cast<double*>(base_cache);
  if (!base) {
    FxArgs ga = fx_args(p, SDD_PREC_FP64, X, p->base_tmp, p->out4);
    SDD_CUDA(launch_fx(ga, batch, 2, SDD_PREC_FP64, s));
    base = p->base_tmp;
  }
  return apply_step(p, batch, Ra, Ras, dv, out, dv, 1, base, SDD_PREC_FP64, s);
}

}  // extern "C"

// ---- Krylov workspace, generic GMRES, Newton and pseudo-arclength continuation ----------------------
// Vectors of the solvers have stride ld = n + 1 per shell (n = 3*N_fm*nr): the Newton solves use the first
// n doubles, the bordered continuation system all n + 1 (the last is the continuation parameter).
static int solver_reserve(sdd_plan* p, int B, int m) {
  if (p->sv_B >= B && p->sv_m >= m) return SDD_OK;
  solver_free(p);
  const size_t n = shell_elems(p), ld = n + 1, be = sdd_plan_base_cache_elems(p);
  const int nchunk = (int)((ld + kDotChunk - 1) / kDotChunk);
  const size_t vb = (size_t)B * ld * sizeof(double);
  SDD_CUDA(ws_malloc(&p->kv_V, (size_t)(m + 1) * vb));
  SDD_CUDA(ws_malloc(&p->kv_w, vb));
  SDD_CUDA(cudaMemset(p->kv_w, 0, vb));   // shells a masked matvec skips keep finite values here
  SDD_CUDA(ws_malloc(&p->kv_r, vb));
  const size_t nsub = (ld + kSubChunk - 1) / kSubChunk;       // partials of the fused update-and-norm
  SDD_CUDA(ws_malloc(&p->kv_part, (size_t)B * std::max((size_t)(m + 1) * nchunk, nsub) * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->kv_nrm2, (size_t)B * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->kv_dot, (size_t)B * sizeof(double)));
  const size_t small = (size_t)B * ((size_t)(m + 1) * m + 3 * (m + 1) + 3 * m + 4);
  SDD_CUDA(ws_malloc(&p->kv_small, small * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->kv_ismall, (size_t)5 * B * sizeof(int)));
  SDD_CUDA(ws_malloc(&p->kv_ticket, (size_t)B * sizeof(int)));
  SDD_CUDA(ws_malloc(&p->kv_vin, vb));
  SDD_CUDA(cudaMemset(p->kv_ticket, 0, (size_t)B * sizeof(int)));
  SDD_CUDA(ws_malloc(&p->h_dbl, (size_t)2 * B * sizeof(double), true));
  SDD_CUDA(ws_malloc(&p->h_int, (size_t)(kFlagLag + 1) * B * sizeof(int), true));
  // blocking-sync events: a solver thread waiting for the GPU sleeps instead of spinning, so that many
  // solver threads (a server's workers) do not take the host cores from each other
  for (cudaEvent_t& e : p->flag_ev)
    SDD_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming | cudaEventBlockingSync));
  SDD_CUDA(cudaEventCreateWithFlags(&p->wait_ev, cudaEventDisableTiming | cudaEventBlockingSync));
  double** v[] = {&p->sv_F, &p->sv_x, &p->sv_Xd, &p->sv_t, &p->sv_G};
  for (double** q : v) SDD_CUDA(ws_malloc(q, vb));
  SDD_CUDA(ws_malloc(&p->sv_X0, (size_t)B * n * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->sv_Jmu, (size_t)B * n * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->sv_g, (size_t)B * n * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->sv_base64, (size_t)B * be * sizeof(double)));
  SDD_CUDA(ws_malloc(&p->sv_base32, (size_t)B * be * sizeof(float)));
  if (p->prec == SDD_PREC_MIXED) SDD_CUDA(ws_malloc(&p->kv_v32, (size_t)B * ld * sizeof(float)));
  SDD_CUDA(ws_malloc(&p->sv_dev, (size_t)8 * B * sizeof(double)));
  p->sv_B = B;
  p->sv_m = m;
  return SDD_OK;
}

static GmresState gmres_state(sdd_plan* p, int B, int m) {
  GmresState s;
  s.m = m;
  double* q = p->kv_small;
  s.H = q; q += (size_t)B * (m + 1) * m;
  s.hcol = q; q += (size_t)B * (m + 1);
  s.h2 = q; q += (size_t)B * (m + 1);
  s.g = q; q += (size_t)B * (m + 1);
  s.cs = q; q += (size_t)B * m;
  s.sn = q; q += (size_t)B * m;
  s.y = q; q += (size_t)B * m;
  s.beta = q; q += B;
  s.inv = q; q += B;
  s.resid = q; q += B;
  s.target = q; q += B;
  int* iq = p->kv_ismall;
  s.active = iq; iq += B;
  s.solve = iq; iq += B;
  s.kb = iq; iq += B;
  s.reo = p->kv_ismall + (size_t)4 * B;   // (block 3 is the Newton update mask)
  return s;
}

// Device matvec on B shells: out = A v (vectors of stride ld); shells whose flag in `active` (device,
// nullable) is 0 may be skipped, their part of out left as it was.  v32 (nullable): v rounded to FP32,
// same strides, for matvecs that work in FP32.
using MatVec = std::function<int(const double* v, double* out, const int* active, const float* v32, cudaStream_t st)>;

// What a product graph bakes in besides its operands: its kind (0: never captured) and the parameter / base
// state pointers the product reads.
struct MvSpec {
  int kind;
  const void* Ra;
  const void* Ras;
  const void* base;
};

// Runs A on stream s.  A product of a nonzero kind is captured once per key on the plan's private stream
// (thread-local capture: other host threads are unaffected) and replayed as one graph launch; a product
// that cannot be captured runs its launches directly.
static int run_mv(sdd_plan* p, const MatVec& A, const MvSpec& spec, int B, const double* v, double* out,
                  const int* active, const float* v32, cudaStream_t s) {
  auto direct = [&]() {
    ++p->mv_count[2];
    return A(v, out, active, v32, s);
  };
  if (!spec.kind || p->mv_graphs_off) return direct();
  const void* key[7] = {v, out, active, v32, spec.Ra, spec.Ras, spec.base};
  MvGraph* slot = nullptr;
  for (MvGraph& g : p->mv_graphs) {
    if (g.exec && g.kind == spec.kind && g.batch == B && g.layout == p->chain_layout && g.fx_split == p->fx_split &&
        g.use_tc == p->use_tc && std::equal(key, key + 7, g.ptr)) {
      g.last_use = ++p->graph_clock;
      ++p->mv_count[1];
      SDD_CUDA(cudaGraphLaunch(g.exec, s));
      return SDD_OK;
    }
    if (!slot || !g.exec || (slot->exec && g.last_use < slot->last_use)) slot = &g;
  }
  if (!p->cap_stream && cudaStreamCreateWithFlags(&p->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
    p->cap_stream = nullptr;
    cudaGetLastError();
    return direct();
  }
  cudaStream_t cs = p->cap_stream;
  if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return direct();
  }
  const int st = A(v, out, active, v32, cs);
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(cs, &graph);
  cudaGraphExec_t exec = nullptr;
  if (st != SDD_OK || ec != cudaSuccess || !graph || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) exec = nullptr;
  if (graph) cudaGraphDestroy(graph);
  cudaGetLastError();
  if (st != SDD_OK || !exec) return direct();   // not capturable: the launches themselves
  if (slot->exec) cudaGraphExecDestroy(slot->exec);
  slot->exec = exec;
  slot->kind = spec.kind;
  slot->batch = B;
  slot->layout = p->chain_layout;
  slot->fx_split = p->fx_split;
  slot->use_tc = p->use_tc;
  std::copy(key, key + 7, slot->ptr);
  slot->last_use = ++p->graph_clock;
  ++p->mv_count[0];
  SDD_CUDA(cudaGraphLaunch(exec, s));
  return SDD_OK;
}

// The solvers' host waits: until the work queued on s so far is done, sleeping on a blocking event.
static int solver_wait(sdd_plan* p, cudaStream_t s) {
  SDD_CUDA(cudaEventRecord(p->wait_ev, s));
  SDD_CUDA(cudaEventSynchronize(p->wait_ev));
  return SDD_OK;
}

// Restarted GMRES(m), classical Gram-Schmidt with a conditional second pass, for the shells with
// solve[b] != 0: A x = rhs, x starts at 0, inner stop |r_b| <= target[b] (absolute).  x, rhs have stride
// ld with nu used doubles.  resid (host) receives the final residual estimates.
static int gmres_solve(sdd_plan* p, const MatVec& A, const MvSpec& spec, const double* rhs, double* x, int B, int nu,
                       int ld, int m, int max_restarts, const std::vector<double>& target,
                       const std::vector<int>& solve, cudaStream_t s, int* matvecs, std::vector<double>& resid,
                       bool basis32 = false) {
  GmresState G = gmres_state(p, B, m);
  p->kv_last_B = B;
  p->kv_basis32 = basis32 ? 1 : 0;
  const size_t vs = (size_t)B * ld;
  // the FP32 basis lives in the FP64 basis's storage (half of it)
  float* V32 = reinterpret_cast<float*>(p->kv_V);
  auto dots = [&](double* h, int nv, const int* mask) {
    return basis32 ? krylov_dots(V32, vs, p->kv_w, nu, ld, nv, B, p->kv_part, h, m + 1, 0, s, mask, p->kv_ticket)
                   : krylov_dots(p->kv_V, vs, p->kv_w, nu, ld, nv, B, p->kv_part, h, m + 1, 0, s, mask, p->kv_ticket);
  };
  auto sub_norm = [&](const double* h, int nv, const int* sub_mask, const GmresState* reo_of, int j) {
    return basis32 ? krylov_sub_norm(V32, vs, p->kv_w, h, m + 1, nu, ld, nv, B, sub_mask, G.active, p->kv_part,
                                     p->kv_ticket, p->kv_nrm2, reo_of, j, p->reorth_eta, s)
                   : krylov_sub_norm(p->kv_V, vs, p->kv_w, h, m + 1, nu, ld, nv, B, sub_mask, G.active, p->kv_part,
                                     p->kv_ticket, p->kv_nrm2, reo_of, j, p->reorth_eta, s);
  };
  auto to_basis = [&](const double* src, int col) {
    return basis32 ? krylov_scale(src, G.inv, V32 + (size_t)col * vs, nu, ld, B, s, p->kv_v32, p->kv_vin)
                   : krylov_scale(src, G.inv, p->kv_V + (size_t)col * vs, nu, ld, B, s, p->kv_v32, p->kv_vin);
  };
  int st;
  resid.assign(B, 0.0);
  SDD_CUDA(cudaMemcpyAsync(G.target, target.data(), B * sizeof(double), cudaMemcpyHostToDevice, s));
  SDD_CUDA(cudaMemcpyAsync(G.solve, solve.data(), B * sizeof(int), cudaMemcpyHostToDevice, s));
  SDD_CUDA(cudaMemsetAsync(x, 0, vs * sizeof(double), s));
  std::vector<int> again(solve);
  for (int cyc = 0; cyc < max_restarts; ++cyc) {
    const double* r = rhs;
    if (cyc > 0) {                                   // r = rhs - A x
      if ((st = run_mv(p, A, spec, B, x, p->kv_w, G.solve, nullptr, s))) return st;
      ++*matvecs;
      SDD_CUDA(krylov_sub(rhs, p->kv_w, p->kv_r, vs, s));
      r = p->kv_r;
    }
    SDD_CUDA(krylov_dots(r, 0, r, nu, ld, 1, B, p->kv_part, p->kv_nrm2, 1, 0, s, nullptr, p->kv_ticket));
    SDD_CUDA(krylov_cycle_start(G, p->kv_nrm2, B, s));
    SDD_CUDA(to_basis(r, 0));
    for (int j = 0; j < m; ++j) {
      // kv_vin (and kv_v32 in FP32) hold V_j: a fixed address, so one captured graph serves every column
      if ((st = run_mv(p, A, spec, B, p->kv_vin, p->kv_w, G.active, p->kv_v32, s))) return st;
      ++*matvecs;
      // shells whose Arnoldi process has stopped skip the Gram-Schmidt work (krylov_arnoldi_finish ignores them);
      // each pass is two launches: the projections, then the update with the new norm (and after the first
      // pass the flag of the shells that repeat it: those whose first pass cancelled w below reorth_eta of
      // its norm; the others get zero second projections)
      SDD_CUDA(dots(G.hcol, j + 1, G.active));
      SDD_CUDA(sub_norm(G.hcol, j + 1, G.active, &G, j));
      SDD_CUDA(dots(G.h2, j + 1, G.reo));
      SDD_CUDA(sub_norm(G.h2, j + 1, G.reo, nullptr, j));
      SDD_CUDA(krylov_arnoldi_finish(G, p->kv_nrm2, j, B, s));
      if (j + 1 < m) SDD_CUDA(to_basis(p->kv_w, j + 1));
      // the flags after column j go to slot j; the host reads those of column j - kFlagLag
      const int slot = j % (kFlagLag + 1);
      SDD_CUDA(cudaMemcpyAsync(p->h_int + (size_t)slot * B, G.active, B * sizeof(int), cudaMemcpyDeviceToHost, s));
      SDD_CUDA(cudaEventRecord(p->flag_ev[slot], s));
      if (j >= kFlagLag) {
        const int old = (j - kFlagLag) % (kFlagLag + 1);
        SDD_CUDA(cudaEventSynchronize(p->flag_ev[old]));
        bool act = false;
        for (int b = 0; b < B; ++b) act = act || p->h_int[(size_t)old * B + b];
        if (!act) {                // every shell stopped after column j - kFlagLag: the later columns were void
          *matvecs -= kFlagLag;
          break;
        }
      }
    }
    SDD_CUDA(krylov_solve_y(G, B, s));
    if (basis32) SDD_CUDA(krylov_add_combination(V32, vs, x, G.y, m, G.kb, nu, ld, B, s));
    else SDD_CUDA(krylov_add_combination(p->kv_V, vs, x, G.y, m, G.kb, nu, ld, B, s));
    SDD_CUDA(cudaMemcpyAsync(p->h_dbl, G.resid, B * sizeof(double), cudaMemcpyDeviceToHost, s));
    if ((st = solver_wait(p, s))) return st;
    bool more = false;
    for (int b = 0; b < B; ++b) {
      if (again[b]) resid[b] = p->h_dbl[b];
      again[b] = again[b] && p->h_dbl[b] > target[b];
      more = more || again[b];
    }
    if (!more) break;
    SDD_CUDA(cudaMemcpyAsync(G.solve, again.data(), B * sizeof(int), cudaMemcpyHostToDevice, s));
  }
  return SDD_OK;
}

// |v_b|^2 over nu doubles at stride ld -> host h_dbl[0..B)
static int host_norms2(sdd_plan* p, const double* v, int nu, int ld, int B, cudaStream_t s) {
  SDD_CUDA(krylov_dots(v, 0, v, nu, ld, 1, B, p->kv_part, p->kv_nrm2, 1, 0, s, nullptr, p->kv_ticket));
  SDD_CUDA(cudaMemcpyAsync(p->h_dbl, p->kv_nrm2, B * sizeof(double), cudaMemcpyDeviceToHost, s));
  return solver_wait(p, s);
}

extern "C" int sdd_newton_gmres(sdd_plan* p, int B, const double* Ra, const double* Ras, double* X,
                                const sdd_newton_opts* o, sdd_newton_result* res, void* stream) {
  int st = check_plan(p, B);
  if (st) return st;
  if (!Ra || !Ras || !X || !o || !res) return SDD_ERR_ARG;
  const int m = o->restart;
  if (m < 1 || m > 64 || o->max_newton < 0 || o->max_restarts < 1 || !(o->tol >= 0.0)) return SDD_ERR_ARG;
  if (o->mixed_matvec < 0 || o->mixed_matvec > 3) return SDD_ERR_ARG;
  if (o->mixed_matvec && p->prec != SDD_PREC_MIXED) return SDD_ERR_ARG;
  if ((st = solver_reserve(p, B, m))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int n = (int)shell_elems(p), ld = n + 1;
  const int mv_prec = o->mixed_matvec ? SDD_PREC_MIXED : SDD_PREC_FP64;
  void* base_mv = o->mixed_matvec ? (void*)p->sv_base32 : (void*)p->sv_base64;
  std::vector<double> resF(B, 0.0), target(B, 0.0), resid;
  std::vector<int> nmask(B, 0), iters(B, 0);
  int matvecs = 0;
  // the parameters in the plan's own buffers: the captured products read them there whatever the caller passes
  double* Ra_d = p->sv_dev + 6 * (size_t)B;
  double* Ras_d = p->sv_dev + 7 * (size_t)B;
  SDD_CUDA(cudaMemcpyAsync(Ra_d, Ra, B * sizeof(double), cudaMemcpyDeviceToDevice, s));
  SDD_CUDA(cudaMemcpyAsync(Ras_d, Ras, B * sizeof(double), cudaMemcpyDeviceToDevice, s));
  // the Jacobian of PFX about the cached base state, on vectors of stride ld
  const bool fp32_rhs = o->mixed_matvec >= 2;
  const bool basis32 = o->mixed_matvec == 3;
  MatVec J = [&](const double* v, double* out, const int* active, const float* v32, cudaStream_t sm) {
    return apply_step_ld(p, B, Ra_d, Ras_d, v, ld, out, ld, v, ld, 1, base_mv, mv_prec, sm, nullptr, nullptr, nullptr,
                         active, 0, 0, o->mixed_matvec ? v32 : nullptr, fp32_rhs);
  };
  const MvSpec Jspec{1 + (fp32_rhs ? 2 : o->mixed_matvec), Ra_d, Ras_d, base_mv};
  for (int it = 0;; ++it) {
    if ((st = apply_step_ld(p, B, Ra_d, Ras_d, X, n, p->sv_F, ld, X, n, 0, p->sv_base64, SDD_PREC_FP64, s)))
      return st;                                                         // F = PFX(X), base cached
    if ((st = host_norms2(p, p->sv_F, n, ld, B, s))) return st;
    bool any = false;
    for (int b = 0; b < B; ++b) {
      resF[b] = std::sqrt(p->h_dbl[b]);
      if (it == 0) res[b].residual0 = resF[b];
      // a non-finite residual (a NaN/Inf state or a diverged update) stops that shell at once: it is
      // reported as not converged instead of iterating to the caps
      nmask[b] = (std::isfinite(resF[b]) && resF[b] > o->tol) ? 1 : 0;
      any = any || nmask[b];
    }
    if (!any || it >= o->max_newton) break;
    if (o->mixed_matvec) {
      FxArgs ga = fx_args(p, SDD_PREC_MIXED, X, p->sv_base32, p->out4);
      SDD_CUDA(launch_fx(ga, B, 2, SDD_PREC_MIXED, s));
    }
    for (int b = 0; b < B; ++b) target[b] = o->gmres_rtol * resF[b];
    if ((st = gmres_solve(p, J, Jspec, p->sv_F, p->sv_x, B, n, ld, m, o->max_restarts, target, nmask, s, &matvecs,
                          resid, basis32)))
      return st;
    int* mask_dev = p->kv_ismall + 3 * B;
    SDD_CUDA(cudaMemcpyAsync(mask_dev, nmask.data(), B * sizeof(int), cudaMemcpyHostToDevice, s));
    SDD_CUDA(krylov_masked_sub(X, p->sv_x, mask_dev, n, n, ld, B, s));
    for (int b = 0; b < B; ++b) iters[b] += nmask[b];
  }
  bool all = true;
  for (int b = 0; b < B; ++b) {
    res[b].residual = resF[b];
    res[b].newton_iters = iters[b];
    res[b].matvecs = matvecs;
    res[b].converged = resF[b] <= o->tol ? 1 : 0;
    res[b].pad = 0;
    all = all && res[b].converged;
  }
  return all ? SDD_OK : SDD_ERR_NOT_CONVERGED;
}

// PDFmu(X) = [A4 solve of dt Pr gr_k T; 0; 0] (Main.py:829-837) into p->sv_Jmu (stride n)
static int pdfmu(sdd_plan* p, int B, const double* X, int ldx, cudaStream_t s) {
  const int n = (int)shell_elems(p);
  SDD_CUDA(contin_grk_T(X, ldx, p->sv_g, p->M, p->nr, p->gr, p->dt * p->Pr, p->sym, B, s));
  SDD_CUDA(cudaMemsetAsync(p->sv_Jmu, 0, (size_t)B * n * sizeof(double), s));
  ChainArgs ca = chain_args(p, p->sv_g, p->sv_Jmu, nullptr);
  SDD_CUDA(launch_chain(ca, B, 1, s));
  return SDD_OK;
}

extern "C" int sdd_contin_step(sdd_plan* p, int B, double* X, double* Ra, const double* Ras, double* X_dot,
                               const double* sign, const double* ds_in, const sdd_contin_opts* o,
                               sdd_contin_result* res, void* stream) {
  int st = check_plan(p, B);
  if (st) return st;
  if (!X || !Ra || !Ras || !X_dot || !sign || !ds_in || !o || !res) return SDD_ERR_ARG;
  const int m = o->restart;
  if (m < 1 || m > 64 || o->max_restarts < 1 || o->max_corrector < 1 || o->max_halvings < 0 || !(o->tol > 0.0))
    return SDD_ERR_ARG;
  if (o->mixed_matvec < 0 || o->mixed_matvec > 3) return SDD_ERR_ARG;
  if (o->mixed_matvec && p->prec != SDD_PREC_MIXED) return SDD_ERR_ARG;
  if ((st = solver_reserve(p, B, m))) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int n = (int)shell_elems(p), ld = n + 1, Npsi = p->M * p->nr;
  const bool fp32_rhs = o->mixed_matvec >= 2;   // FP32 right-hand sides and h matvecs in the products too
  const bool basis32 = o->mixed_matvec == 3;    // and an FP32 Krylov basis
  const double delta = 1.0 / n;                         // 1/(3N), Main.py:771
  const int mv_prec = o->mixed_matvec ? SDD_PREC_MIXED : SDD_PREC_FP64;
  void* base_mv = o->mixed_matvec ? (void*)p->sv_base32 : (void*)p->sv_base64;
  double* mu_dev = p->sv_dev;            // current parameter Ra (per shell)
  double* mudot_dev = p->sv_dev + B;
  double* c_dev = p->sv_dev + 2 * B;     // per-shell scalars
  double* last_dev = p->sv_dev + 3 * B;
  double* Ras_d = p->sv_dev + 7 * (size_t)B;   // Ra_s in the plan's own buffer (read by the captured products)
  std::vector<double> mu0(B), mu(B), mudot(B), ds(ds_in, ds_in + B), resF(B, 0.0), gl(B, 0.0), c(B), tgt(B), resid;
  std::vector<int> it(B, 0), halv(B, 0), conv(B, 0), fail(B, 0), solve(B, 0);
  int matvecs = 0;
  SDD_CUDA(cudaMemcpyAsync(Ras_d, Ras, B * sizeof(double), cudaMemcpyDeviceToDevice, s));
  SDD_CUDA(cudaMemcpyAsync(mu0.data(), Ra, B * sizeof(double), cudaMemcpyDeviceToHost, s));
  if ((st = solver_wait(p, s))) return st;
  mu = mu0;
  auto upload = [&](double* dst, const std::vector<double>& v) {
    return cudaMemcpyAsync(dst, v.data(), B * sizeof(double), cudaMemcpyHostToDevice, s);
  };
  auto base_at = [&](const double* Xs) -> int {        // F = PFX(Xs, mu) into sv_F (stride ld), base cached
    int r = apply_step_ld(p, B, mu_dev, Ras, Xs, n, p->sv_F, ld, Xs, n, 0, p->sv_base64, SDD_PREC_FP64, s);
    if (r) return r;
    if (o->mixed_matvec) {
      FxArgs ga = fx_args(p, SDD_PREC_MIXED, Xs, p->sv_base32, p->out4);
      SDD_CUDA(launch_fx(ga, B, 2, SDD_PREC_MIXED, s));
    }
    return pdfmu(p, B, Xs, n, s);
  };
  MatVec J = [&](const double* v, double* out, const int* active, const float* v32, cudaStream_t sm) {
    return apply_step_ld(p, B, mu_dev, Ras_d, v, ld, out, ld, v, ld, 1, base_mv, mv_prec, sm, nullptr, nullptr,
                         nullptr, active, 0, 0, o->mixed_matvec ? v32 : nullptr, fp32_rhs);
  };
  // bordered operator DG = [[DF_X, DF_mu], [delta X_dot^T, (1-delta) mu_dot]]  (Main.py:914-915)
  MatVec DG = [&](const double* v, double* out, const int* active, const float* v32, cudaStream_t sm) -> int {
    int r = apply_step_ld(p, B, mu_dev, Ras_d, v, ld, out, ld, v, ld, 1, base_mv, mv_prec, sm, nullptr, nullptr,
                          nullptr, active, 0, 0, o->mixed_matvec ? v32 : nullptr, fp32_rhs);
    if (r) return r;
    SDD_CUDA(krylov_dots(p->sv_Xd, 0, v, n, ld, 1, B, p->kv_part, p->kv_dot, 1, 0, sm, nullptr, p->kv_ticket));
    SDD_CUDA(contin_border(v, out, n, ld, p->sv_Jmu, n, Npsi, p->kv_dot, mudot_dev, delta, B, sm));
    return SDD_OK;
  };
  const int mv_kind = fp32_rhs ? 2 : o->mixed_matvec;   // the products of modes 2 and 3 are the same
  const MvSpec Jspec{4 + mv_kind, mu_dev, Ras_d, base_mv};
  const MvSpec DGspec{8 + mv_kind, mu_dev, Ras_d, base_mv};

  // ---- predictor (Main.py:839-876; with dt < 10 the tangent is always recomputed) ----
  SDD_CUDA(upload(mu_dev, mu));
  if ((st = base_at(X))) return st;
  SDD_CUDA(krylov_copy_scaled(p->sv_Jmu, n, p->sv_G, ld, n, -1.0, nullptr, B, s));   // rhs = -DF_mu
  if ((st = host_norms2(p, p->sv_G, n, ld, B, s))) return st;
  for (int b = 0; b < B; ++b) {
    const double nj = std::sqrt(p->h_dbl[b]);
    tgt[b] = o->tangent_rtol * nj;
    solve[b] = nj > 0.0;
  }
  if ((st = gmres_solve(p, J, Jspec, p->sv_G, p->sv_x, B, n, ld, m, o->max_restarts, tgt, solve, s, &matvecs, resid,
                        basis32)))
    return st;
  if ((st = host_norms2(p, p->sv_x, n, ld, B, s))) return st;
  for (int b = 0; b < B; ++b) {
    const double nxi = std::sqrt(p->h_dbl[b]);
    mudot[b] = sign[b] / std::sqrt(1.0 + delta * (nxi - 1.0));    // Main.py:861
    c[b] = mudot[b];
  }
  SDD_CUDA(upload(mudot_dev, mudot));
  SDD_CUDA(upload(c_dev, c));
  SDD_CUDA(krylov_scale(p->sv_x, c_dev, p->sv_Xd, n, ld, B, s));                     // X_dot = mu_dot xi
  SDD_CUDA(cudaMemcpyAsync(p->sv_X0, X, (size_t)B * n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  auto predict = [&](int b) -> int {                     // X_b = X0_b + ds_b X_dot_b, mu_b = mu0_b + ds_b mu_dot_b
    c[b] = ds[b];
    SDD_CUDA(cudaMemcpyAsync(c_dev + b, &c[b], sizeof(double), cudaMemcpyHostToDevice, s));
    SDD_CUDA(krylov_axpy_shell(p->sv_X0 + (size_t)b * n, n, p->sv_Xd + (size_t)b * ld, ld, c_dev + b,
                               X + (size_t)b * n, n, n, 1, s));
    mu[b] = mu0[b] + ds[b] * mudot[b];
    return SDD_OK;
  };
  for (int b = 0; b < B; ++b)
    if ((st = predict(b))) return st;

  // ---- corrector (Main.py:885-930), stopping on absolute residuals ----
  const int max_rounds = (o->max_halvings + 1) * (o->max_corrector + 1) + 1;
  for (int round = 0; round < max_rounds; ++round) {
    SDD_CUDA(upload(mu_dev, mu));
    if ((st = base_at(X))) return st;
    // arclength residual p = delta X_dot.(X - X0) + (1 - delta) mu_dot (mu - mu0) - ds   (Main.py:910)
    SDD_CUDA(krylov_copy_scaled(X, n, p->sv_t, ld, n, 1.0, nullptr, B, s));
    for (int b = 0; b < B; ++b) c[b] = -1.0;
    SDD_CUDA(upload(c_dev, c));
    SDD_CUDA(krylov_axpy_shell(p->sv_t, ld, p->sv_X0, n, c_dev, p->sv_t, ld, n, B, s));
    SDD_CUDA(krylov_dots(p->sv_Xd, 0, p->sv_t, n, ld, 1, B, p->kv_part, p->kv_dot, 1, 0, s, nullptr, p->kv_ticket));
    SDD_CUDA(cudaMemcpyAsync(p->h_dbl + B, p->kv_dot, B * sizeof(double), cudaMemcpyDeviceToHost, s));
    if ((st = host_norms2(p, p->sv_F, n, ld, B, s))) return st;
    bool pending = false;
    for (int b = 0; b < B; ++b) {
      resF[b] = std::sqrt(p->h_dbl[b]);
      gl[b] = delta * p->h_dbl[B + b] + (1.0 - delta) * mudot[b] * (mu[b] - mu0[b]) - ds[b];
      solve[b] = 0;
      if (conv[b] || fail[b]) continue;
      if (!std::isfinite(resF[b]) || !std::isfinite(gl[b]) || !std::isfinite(mu[b])) {   // NaN/Inf: give up
        fail[b] = 1;
        continue;
      }
      if (resF[b] <= o->tol && std::fabs(gl[b]) <= o->tol) {
        conv[b] = 1;
        continue;
      }
      if (it[b] >= o->max_corrector) {                    // halve ds and predict again (Main.py:888-899)
        ds[b] *= 0.5;
        ++halv[b];
        it[b] = 0;
        if (halv[b] > o->max_halvings || ds[b] < o->tol) {
          fail[b] = 1;
          continue;
        }
        if ((st = predict(b))) return st;
        pending = true;
        continue;
      }
      solve[b] = 1;
      pending = true;
    }
    if (!pending) break;
    bool any = false;
    for (int b = 0; b < B; ++b) any = any || solve[b];
    if (!any) continue;                                   // only re-predicted shells this round
    SDD_CUDA(upload(last_dev, gl));
    SDD_CUDA(krylov_copy_scaled(p->sv_F, ld, p->sv_G, ld, n, 1.0, last_dev, B, s));     // G = [F; p]
    for (int b = 0; b < B; ++b)
      tgt[b] = o->gmres_rtol * std::sqrt(delta * resF[b] * resF[b] + (1.0 - delta) * gl[b] * gl[b]);  // :919
    if ((st = gmres_solve(p, DG, DGspec, p->sv_G, p->sv_x, B, n + 1, ld, m, o->max_restarts, tgt, solve, s, &matvecs,
                          resid, basis32)))
      return st;
    int* mask_dev = p->kv_ismall + 3 * B;
    SDD_CUDA(cudaMemcpyAsync(mask_dev, solve.data(), B * sizeof(int), cudaMemcpyHostToDevice, s));
    SDD_CUDA(krylov_masked_sub(X, p->sv_x, mask_dev, n, n, ld, B, s));                   // Y -= dY
    SDD_CUDA(cudaMemcpy2DAsync(p->h_dbl, sizeof(double), p->sv_x + n, ld * sizeof(double), sizeof(double), B,
                               cudaMemcpyDeviceToHost, s));
    if ((st = solver_wait(p, s))) return st;
    for (int b = 0; b < B; ++b)
      if (solve[b]) {
        mu[b] -= p->h_dbl[b];
        ++it[b];
      }
  }

  // ---- new tangent: DG y = e_last at the converged point, normalised (Main.py:944-953) ----
  SDD_CUDA(cudaMemsetAsync(p->sv_G, 0, (size_t)B * ld * sizeof(double), s));
  for (int b = 0; b < B; ++b) c[b] = 1.0;
  SDD_CUDA(upload(last_dev, c));
  SDD_CUDA(krylov_copy_scaled(p->sv_G, ld, p->sv_G, ld, n, 1.0, last_dev, B, s));   // G = e_last (G[n] = 1)
  for (int b = 0; b < B; ++b) {
    tgt[b] = o->tangent_rtol;
    solve[b] = conv[b];
  }
  if ((st = gmres_solve(p, DG, DGspec, p->sv_G, p->sv_x, B, n + 1, ld, m, o->max_restarts, tgt, solve, s, &matvecs,
                        resid, basis32)))
    return st;
  if ((st = host_norms2(p, p->sv_x, n, ld, B, s))) return st;
  std::vector<double> yx2(p->h_dbl, p->h_dbl + B);
  SDD_CUDA(cudaMemcpy2DAsync(p->h_dbl, sizeof(double), p->sv_x + n, ld * sizeof(double), sizeof(double), B,
                             cudaMemcpyDeviceToHost, s));
  if ((st = solver_wait(p, s))) return st;
  for (int b = 0; b < B; ++b) {
    const double yl = p->h_dbl[b];
    const double nrm = std::sqrt(delta * yx2[b] + (1.0 - delta) * yl * yl);
    c[b] = (conv[b] && nrm > 0.0) ? 1.0 / nrm : 0.0;
    res[b].Ra_dot = c[b] * yl;
  }
  SDD_CUDA(upload(c_dev, c));
  SDD_CUDA(krylov_scale(p->sv_x, c_dev, p->sv_t, n, ld, B, s));
  SDD_CUDA(krylov_copy_scaled(p->sv_t, ld, X_dot, n, n, 1.0, nullptr, B, s));
  SDD_CUDA(upload(Ra, mu));
  if ((st = solver_wait(p, s))) return st;
  bool all = true;
  for (int b = 0; b < B; ++b) {
    res[b].residual = resF[b];
    res[b].arclength = std::fabs(gl[b]);
    res[b].ds = (conv[b] && it[b] <= 4) ? 2.0 * ds[b] : ds[b];        // Main.py:933-935
    res[b].corrector_iters = it[b];
    res[b].halvings = halv[b];
    res[b].matvecs = matvecs;
    res[b].converged = conv[b];
    all = all && conv[b];
  }
  return all ? SDD_OK : SDD_ERR_NOT_CONVERGED;
}

// ---- instrumentation ------------------------------------------------------------------------------
extern "C" int sdd_step_profile(sdd_plan* p, int B, const double* Ra, const double* Ras, const double* X_in,
                                double* X_out, int nsteps, double* ms, void* stream) {
  int st = check_plan(p, B);
  if (st) return st;
  if (!Ra || !Ras || !X_in || !X_out || !ms || nsteps < 1 || X_in == X_out) return SDD_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t ev[4];
  for (auto& e : ev) SDD_CUDA(cudaEventCreate(&e));
  const double* cur = X_in;
  int rc = SDD_OK;
  for (int it = 0; it < nsteps && rc == SDD_OK; ++it) {
    const int left = nsteps - it;
    double* dst = (left % 2 == 1) ? X_out : p->xtmp;
    const size_t n = shell_elems(p);
    rc = apply_step_ld(p, B, Ra, Ras, cur, n, dst, n, nullptr, n, 0, nullptr, p->prec, s, ev);
    if (rc != SDD_OK) break;
    cudaError_t e = cudaEventSynchronize(ev[3]);
    float t = 0.f;
    for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
      e = cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
      ms[k] += t;
    }
    if (e != cudaSuccess) {
      set_cuda_error(e);
      rc = SDD_ERR_CUDA;
    }
    cur = dst;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return rc;
}

static DiagArgs diag_args(const sdd_plan* p, const double* X, double* out) {
  DiagArgs a;
  std::memset(&a, 0, sizeof(a));
  a.M = p->M; a.nr = p->nr; a.sym = p->sym; a.L = p->dfft->L;
  a.st = stage_args(p->dfft);
  a.w = p->dfft->w64; a.e = p->dfft->e64;
  a.Dr = p->Dr; a.ir = p->dg_ir; a.tw = p->dg_tw; a.wr = p->dg_wr; a.nuw = p->dg_nuw;
  a.ke_scale = p->ke_scale;
  a.X = X; a.x_stride = shell_elems(p);
  a.part = p->dg_part; a.out = out;
  return a;
}

extern "C" int sdd_diagnostics(sdd_plan* p, int batch, const double* X, double* out, void* stream) {
  int st = check_plan(p, batch);
  if (st) return st;
  if (!X || !out) return SDD_ERR_ARG;
  if (!p->dfft) return SDD_ERR_UNSUPPORTED;
  SDD_CUDA(launch_diag(diag_args(p, X, out), batch, (cudaStream_t)stream));
  return SDD_OK;
}

extern "C" int sdd_step_diag(sdd_plan* p, int batch, const double* Ra, const double* Ras, const double* X_in,
                             double* X_out, int nsteps, int linear, double* diag, void* stream) {
  int st = check_plan(p, batch);
  if (st) return st;
  if (!Ra || !Ras || !X_in || !X_out || !diag || nsteps < 0) return SDD_ERR_ARG;
  if (!p->dfft) return SDD_ERR_UNSUPPORTED;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = (size_t)batch * shell_elems(p) * sizeof(double);
  const double* cur = X_in;
  for (int it = 0; it < nsteps; ++it) {
    const int left = nsteps - it;
    double* dst = (left % 2 == 1) ? X_out : p->xtmp;
    if (dst == cur) dst = (dst == X_out) ? p->xtmp : X_out;
    if ((st = apply_step(p, batch, Ra, Ras, cur, dst, nullptr, linear ? 2 : 0, nullptr, p->prec, s))) return st;
    SDD_CUDA(launch_diag(diag_args(p, dst, diag + (size_t)it * batch * 4), batch, s));
    cur = dst;
  }
  if (cur != X_out) SDD_CUDA(cudaMemcpyAsync(X_out, cur, bytes, cudaMemcpyDeviceToDevice, s));
  return SDD_OK;
}

extern "C" const char* sdd_kernel_name(int id) {
  static const char* names[SDD_NUM_KERNELS] = {"k_fx_rows", "k_fx_deriv", "k_fx_grid", "k_fx_prod", "k_rhs",
                                               "k_mode_mv(h)", "k_chain", "k_chain_carry", "k_mode_mv(fix)",
                                               "k_deriv_tc"};
  return (id >= 0 && id < SDD_NUM_KERNELS) ? names[id] : "unknown";
}

extern "C" int sdd_step_kernel_profile(sdd_plan* p, int B, const double* Ra, const double* Ras, const double* X_in,
                                       double* X_out, int nsteps, double* ms, int* launches, void* stream) {
  int st = check_plan(p, B);
  if (st) return st;
  if (!Ra || !Ras || !X_in || !X_out || !ms || !launches || nsteps < 1 || X_in == X_out) return SDD_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  KernelTimer t;
  t.n = 0;
  cudaEvent_t start;
  SDD_CUDA(cudaEventCreate(&start));
  int made = 0;
  cudaError_t e = cudaSuccess;
  for (; made < KernelTimer::kMax && e == cudaSuccess; ++made) e = cudaEventCreate(&t.ev[made]);
  if (e != cudaSuccess) --made;
  const double* cur = X_in;
  int rc = e == cudaSuccess ? SDD_OK : SDD_ERR_CUDA;
  if (rc) set_cuda_error(e);
  const int dfix = step_defers_fix(p, B, 0) ? 1 : 0;   // the sequencing of sdd_step
  for (int it = 0; it < nsteps && rc == SDD_OK; ++it) {
    double* dst = ((nsteps - it) % 2 == 1) ? X_out : p->xtmp;
    t.n = 0;
    if ((e = cudaEventRecord(start, s)) != cudaSuccess) {
      set_cuda_error(e);
      rc = SDD_ERR_CUDA;
      break;
    }
    g_ktimer = &t;
    const size_t n = shell_elems(p);
    rc = apply_step_ld(p, B, Ra, Ras, cur, n, dst, n, nullptr, n, 0, nullptr, p->prec, s, nullptr, nullptr, nullptr,
                       nullptr, dfix, dfix && it > 0);
    if (rc == SDD_OK && dfix && it + 1 == nsteps) rc = finish_fix(p, B, dst, nullptr, s);
    g_ktimer = nullptr;
    if (rc != SDD_OK) break;
    if (t.n > 0 && (e = cudaEventSynchronize(t.ev[t.n - 1])) != cudaSuccess) {
      set_cuda_error(e);
      rc = SDD_ERR_CUDA;
      break;
    }
    cudaEvent_t prev = start;
    for (int k = 0; k < t.n; ++k) {
      float ms_k = 0.f;
      if (cudaEventElapsedTime(&ms_k, prev, t.ev[k]) == cudaSuccess && t.id[k] >= 0 && t.id[k] < SDD_NUM_KERNELS) {
        ms[t.id[k]] += ms_k;
        launches[t.id[k]] += 1;
      }
      prev = t.ev[k];
    }
    cur = dst;
  }
  g_ktimer = nullptr;
  for (int k = 0; k < made; ++k) cudaEventDestroy(t.ev[k]);
  cudaEventDestroy(start);
  return rc;
}

namespace sdd {
__global__ void k_fp64_fma_loop(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace sdd

extern "C" int sdd_deriv_tc(sdd_plan* p, int batch, const float* X32, float* out, void* stream) {
  if (!p || batch < 1 || !X32 || !out) return SDD_ERR_ARG;
  if (!p->tcB) return SDD_ERR_UNSUPPORTED;
  int dev = 0;
  SDD_CUDA(cudaGetDevice(&dev));
  if (dev != p->device) return SDD_ERR_ARG;
  TcArgs t;
  std::memset(&t, 0, sizeof(t));
  t.M = p->M; t.nr = p->nr; t.sym = p->sym; t.KP = p->tcKP; t.NP = p->tcNP;
  t.rows = batch * 3 * p->M;
  t.X32 = X32;
  t.x32_stride = shell_elems(p);
  t.B = p->tcB;
  t.out = out;
  t.out_stride = (size_t)4 * p->M * p->nr;
  t.err = p->tc_err;
  SDD_CUDA(launch_deriv_tc(t, (cudaStream_t)stream));
  return SDD_OK;
}

extern "C" int sdd_debug_fail_allocations(long long after) {
  g_alloc_left.store(after < 0 ? -1 : after);
  return SDD_OK;
}

extern "C" int sdd_measure_fp64_peak(double* gflops, void* stream) {
  if (!gflops) return SDD_ERR_ARG;
  int dev = 0, sms = 0;
  SDD_CUDA(cudaGetDevice(&dev));
  SDD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256, iters = 2000;
  cudaStream_t s = (cudaStream_t)stream;
  double* out = nullptr;
  SDD_CUDA(cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  cudaError_t e = cudaSuccess;
  for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) {
    cudaEventRecord(e0, s);
    k_fp64_fma_loop<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, s);
    e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    if (t > 0.f && t < best) best = t;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) {
    set_cuda_error(e);
    return SDD_ERR_CUDA;
  }
  *gflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e9;
  return SDD_OK;
}

// ---- NLIN_FX with a fixed, library-owned scratch (no allocation on the call) ------------------------
// The scratch lives in a file-scope __device__ array.  In host code its name is only a host-side
// stand-in, so its device address is looked up with cudaGetSymbolAddress once per device (with that
// device current) and that address is what the kernels receive.
static __device__ __align__(256) double g_noalloc_scratch[SDD_NOALLOC_SCRATCH_DOUBLES];
static std::mutex g_noalloc_mu;
static double* g_noalloc_ptr[64] = {nullptr};

static int noalloc_scratch(int dev, double** out) {
  if (dev < 0 || dev >= 64) return SDD_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || ptr == nullptr) {
      set_cuda_error(e);
      return SDD_ERR_CUDA;
    }
    g_noalloc_ptr[dev] = static_cast<double*>(ptr);
  }
  *out = g_noalloc_ptr[dev];
  return SDD_OK;
}

extern "C" int sdd_nlin_fx_noalloc(sdd_plan* p, int batch, const double* X, double* F, void* stream) {
  if (!p || batch < 1 || !X || !F) return SDD_ERR_ARG;
  int dev = 0;
  SDD_CUDA(cudaGetDevice(&dev));
  if (dev != p->device) return SDD_ERR_ARG;
  const size_t need = (size_t)batch * 4 * p->M * p->nr;
  if (need > (size_t)SDD_NOALLOC_SCRATCH_DOUBLES) return SDD_ERR_UNSUPPORTED;
  double* scratch = nullptr;
  const int st = noalloc_scratch(dev, &scratch);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  // the row kernel writes every element of the batch's 4*N_fm*nr outputs before k_fx_finish reads them
  FxArgs fa = fx_args(p, SDD_PREC_FP64, X, nullptr, scratch);
  fa.grid = nullptr;   // the fused row kernel: no grid scratch (the plan's may be smaller than the batch)
  fa.deriv = nullptr;
  SDD_CUDA(launch_fx(fa, batch, 0, SDD_PREC_FP64, s));
  SDD_CUDA(launch_fx_finish(p->M, p->nr, p->Dr, scratch, (size_t)4 * p->M * p->nr, F, shell_elems(p), batch, s));
  return SDD_OK;
}
