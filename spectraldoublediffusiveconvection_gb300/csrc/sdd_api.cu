// C ABI of libsdd_gb300: plans (device-resident operators), FFT tables, workspaces, entry points.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "sdd_internal.cuh"
#include "sdd_krylov.cuh"

namespace sdd {
cudaError_t launch_fx_finish(int M, int nr, const double* Dr, const double* out4, size_t out_stride,
                             double* F, size_t f_stride, int batch, cudaStream_t s);

static thread_local int g_last_cuda = 0;
void set_cuda_error(cudaError_t e) { g_last_cuda = (int)e; }

#define SDD_CUDA(call)                         \
  do {                                         \
    cudaError_t e_ = (call);                   \
    if (e_ != cudaSuccess) {                   \
      set_cuda_error(e_);                      \
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
struct sdd_plan {
  int M, nr, P, ldl, sym, prec, device;
  int chain_layout;
  double dt, Pr, Tau;
  const FftPlan* fft;
  // FP64 operators
  double *Dr, *D2r2, *ir4r2, *D2s, *ir2s, *D2A4, *ir2A4, *ir4A4, *rsq, *dT0, *gr;
  double *LinvA4, *LinvT, *LinvS;
  double *ABA4;                     // transposed [A_j B_j] of the psi chain
  double *coefA4, *coefT, *coefS;   // per-step scalars of the chains
  // FP32 copies used by the mixed-precision nonlinear term
  float *Dr32, *D2r232, *ir4r232;
  // workspace
  int ws_batch;
  double* out4;     // [B][4][M][nr]
  double* rhs;      // [B][3][M][nr]
  double* xtmp;     // [B][3][M][nr]
  double* hbuf;     // [B][3][M][nr] h = Linv g of the chains
  void* base_tmp;   // [B][nr][9][P] (T precision), for DFX without a caller cache
  // Newton-GMRES workspace
  int nw_B, nw_m;
  double *nw_V, *nw_F, *nw_x, *nw_w, *nw_r, *nw_part, *nw_nrm2, *nw_base64;
  float* nw_base32;
  double *nw_small;   // H, hcol, h2, cs, sn, g, y, beta, inv, resid, target
  int* nw_ismall;     // active, solve, kb, newton mask
  double* h_dbl;      // pinned host: nrm2 / resid
  int* h_int;         // pinned host: active flags
};

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

static void free_plan(sdd_plan* p) {
  if (!p) return;
  double* d[] = {p->Dr, p->D2r2, p->ir4r2, p->D2s, p->ir2s, p->D2A4, p->ir2A4, p->ir4A4, p->rsq, p->dT0,
                 p->gr, p->LinvA4, p->LinvT, p->LinvS, p->out4, p->rhs, p->xtmp, p->coefA4, p->coefT, p->coefS, p->ABA4, p->hbuf};
  for (double* x : d) cudaFree(x);
  cudaFree(p->Dr32); cudaFree(p->D2r232); cudaFree(p->ir4r232);
  cudaFree(p->base_tmp);
  double* nw[] = {p->nw_V, p->nw_F, p->nw_x, p->nw_w, p->nw_r, p->nw_part, p->nw_nrm2, p->nw_base64, p->nw_small};
  for (double* x : nw) cudaFree(x);
  cudaFree(p->nw_base32);
  cudaFree(p->nw_ismall);
  cudaFreeHost(p->h_dbl);
  cudaFreeHost(p->h_int);
  delete p;
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
  int smem_optin = 0;
  SDD_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  if (fx_smem_bytes(M, P, d->precision) > (size_t)smem_optin) return SDD_ERR_UNSUPPORTED;
  // the FP64 nonlinear term is also needed by the mixed plan's Newton residual
  if (fx_smem_bytes(M, P, SDD_PREC_FP64) > (size_t)smem_optin) return SDD_ERR_UNSUPPORTED;
  const FftPlan* fp = get_fft_plan(P);
  if (!fp) return SDD_ERR_UNSUPPORTED;
  sdd_plan* p = new sdd_plan();
  std::memset(p, 0, sizeof(*p));
  p->M = M; p->nr = nr; p->P = P; p->ldl = nr + (nr & 1); p->sym = d->symmetric ? 1 : 0;
  p->prec = d->precision; p->device = dev;
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
  (void)nm;
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
    if ((st = upload(&p->ABA4, AB.data(), AB.size()))) {
      free_plan(p);
      return st;
    }
  }
  *out = p;
  return SDD_OK;
}

int sdd_plan_destroy(sdd_plan* p) {
  if (!p) return SDD_ERR_ARG;
  free_plan(p);
  return SDD_OK;
}

int sdd_plan_set_chain_layout(sdd_plan* p, int layout) {
  if (!p || (layout != 0 && layout != 1 && layout != 4)) return SDD_ERR_ARG;
  p->chain_layout = layout;
  return SDD_OK;
}

size_t sdd_plan_base_cache_elems(const sdd_plan* p) { return p ? (size_t)9 * p->nr * p->P : 0; }

static size_t shell_elems(const sdd_plan* p) { return (size_t)3 * p->M * p->nr; }

int sdd_plan_reserve(sdd_plan* p, int max_batch) {
  if (!p || max_batch < 1) return SDD_ERR_ARG;
  if (max_batch <= p->ws_batch) return SDD_OK;
  cudaFree(p->out4); cudaFree(p->rhs); cudaFree(p->xtmp); cudaFree(p->base_tmp); cudaFree(p->hbuf);
  p->out4 = p->rhs = p->xtmp = p->hbuf = nullptr;
  p->base_tmp = nullptr;
  p->ws_batch = 0;
  const size_t se = shell_elems(p);
  const size_t be = sdd_plan_base_cache_elems(p);
  SDD_CUDA(cudaMalloc(&p->out4, (size_t)max_batch * 4 * p->M * p->nr * sizeof(double)));
  SDD_CUDA(cudaMalloc(&p->rhs, (size_t)max_batch * se * sizeof(double)));
  SDD_CUDA(cudaMalloc(&p->xtmp, (size_t)max_batch * se * sizeof(double)));
  SDD_CUDA(cudaMalloc(&p->hbuf, (size_t)max_batch * se * sizeof(double)));
  SDD_CUDA(cudaMalloc(&p->base_tmp, (size_t)max_batch * be * sizeof(double)));
  p->ws_batch = max_batch;
  return SDD_OK;
}

}  // extern "C"

// ---- internal launch helpers ---------------------------------------------------------------------
static FxArgs fx_args(const sdd_plan* p, int prec, const double* X, void* base, double* out4) {
  FxArgs a;
  std::memset(&a, 0, sizeof(a));
  a.M = p->M; a.nr = p->nr; a.P = p->P; a.sym = p->sym;
  a.st.L = p->fft->L; a.st.nst = p->fft->nst;
  for (int i = 0; i < kMaxStages; ++i) a.st.rad[i] = p->fft->rad[i];
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
  return a;
}

static RhsArgs rhs_args(const sdd_plan* p, const double* X, const double* out4, const double* Ra,
                        const double* Ras, double* rhs, int linear) {
  RhsArgs a;
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
  a.M = p->M; a.nr = p->nr; a.ldl = p->ldl; a.sym = p->sym; a.field0 = 0; a.layout = p->chain_layout;
  a.field_off = (size_t)p->M * p->nr;
  a.g = g; a.g_stride = shell_elems(p);
  a.f = f; a.f_stride = shell_elems(p);
  a.sub = sub; a.sub_stride = shell_elems(p);
  a.LinvA4 = p->LinvA4; a.LinvT = p->LinvT; a.LinvS = p->LinvS;
  a.ABA4 = p->ABA4; a.ir2A4 = p->ir2A4; a.ir4A4 = p->ir4A4;
  a.h = p->hbuf;
  a.coefA4 = p->coefA4; a.coefT = p->coefT; a.coefS = p->coefS;
  a.dtA4 = p->Pr * p->dt; a.dtT = p->dt; a.dtS = p->Tau * p->dt;
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
static int apply_step(sdd_plan* p, int batch, const double* Ra, const double* Ras, const double* X,
                      double* out, const double* sub, int mode, void* base, int prec, cudaStream_t s) {
  cudaError_t e;
  if (mode != 2) {
    FxArgs fa = fx_args(p, prec, X, base, p->out4);
    e = launch_fx(fa, batch, mode == 1 ? 1 : 0, prec, s);
    SDD_CUDA(e);
  }
  RhsArgs ra = rhs_args(p, X, p->out4, Ra, Ras, p->rhs, mode == 2);
  SDD_CUDA(launch_rhs(ra, batch, s));
  ChainArgs ca = chain_args(p, p->rhs, out, sub);
  SDD_CUDA(launch_chain(ca, batch, 3, s));
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
  // ping-pong so that the last step lands in X_out
  const double* cur = X_in;
  for (int it = 0; it < nsteps; ++it) {
    const int left = nsteps - it;  // steps remaining including this one
    double* dst = (left % 2 == 1) ? X_out : p->xtmp;
    if (dst == cur) dst = (dst == X_out) ? p->xtmp : X_out;  // never write the input in place
    st = apply_step(p, batch, Ra, Ras, cur, dst, nullptr, linear ? 2 : 0, nullptr, p->prec, s);
    if (st) return st;
    cur = dst;
  }
  if (cur != X_out) SDD_CUDA(cudaMemcpyAsync(X_out, cur, bytes, cudaMemcpyDeviceToDevice, s));
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

// ---- Newton-GMRES --------------------------------------------------------------------------------
static int newton_reserve(sdd_plan* p, int B, int m) {
  if (p->nw_B >= B && p->nw_m >= m) return SDD_OK;
  double* nw[] = {p->nw_V, p->nw_F, p->nw_x, p->nw_w, p->nw_r, p->nw_part, p->nw_nrm2, p->nw_base64, p->nw_small};
  for (double* x : nw) cudaFree(x);
  cudaFree(p->nw_base32); cudaFree(p->nw_ismall); cudaFreeHost(p->h_dbl); cudaFreeHost(p->h_int);
  p->nw_V = p->nw_F = p->nw_x = p->nw_w = p->nw_r = p->nw_part = p->nw_nrm2 = p->nw_base64 = p->nw_small = nullptr;
  p->nw_base32 = nullptr; p->nw_ismall = nullptr; p->h_dbl = nullptr; p->h_int = nullptr;
  p->nw_B = p->nw_m = 0;
  const size_t n = shell_elems(p), be = sdd_plan_base_cache_elems(p);
  const int nchunk = (int)((n + kDotChunk - 1) / kDotChunk);
  SDD_CUDA(cudaMalloc(&p->nw_V, (size_t)(m + 1) * B * n * sizeof(double)));
  SDD_CUDA(cudaMalloc(&p->nw_F, (size_t)B * n * sizeof(double)));
  SDD_CUDA(cudaMalloc(&p->nw_x, (size_t)B * n * sizeof(double)));
  SDD_CUDA(cudaMalloc(&p->nw_w, (size_t)B * n * sizeof(double)));
  SDD_CUDA(cudaMalloc(&p->nw_r, (size_t)B * n * sizeof(double)));
  SDD_CUDA(cudaMalloc(&p->nw_part, (size_t)B * (m + 1) * nchunk * sizeof(double)));
  SDD_CUDA(cudaMalloc(&p->nw_nrm2, (size_t)B * sizeof(double)));
  SDD_CUDA(cudaMalloc(&p->nw_base64, (size_t)B * be * sizeof(double)));
  SDD_CUDA(cudaMalloc(&p->nw_base32, (size_t)B * be * sizeof(float)));
  const size_t small = (size_t)B * ((size_t)(m + 1) * m + 3 * (m + 1) + 3 * m + 4);
  SDD_CUDA(cudaMalloc(&p->nw_small, small * sizeof(double)));
  SDD_CUDA(cudaMalloc(&p->nw_ismall, (size_t)4 * B * sizeof(int)));
  SDD_CUDA(cudaMallocHost(&p->h_dbl, (size_t)B * sizeof(double)));
  SDD_CUDA(cudaMallocHost(&p->h_int, (size_t)B * sizeof(int)));
  p->nw_B = B;
  p->nw_m = m;
  return SDD_OK;
}

static GmresState gmres_state(sdd_plan* p, int B, int m) {
  GmresState s;
  s.m = m;
  double* q = p->nw_small;
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
  int* iq = p->nw_ismall;
  s.active = iq; iq += B;
  s.solve = iq; iq += B;
  s.kb = iq; iq += B;
  return s;
}

extern "C" int sdd_newton_gmres(sdd_plan* p, int B, const double* Ra, const double* Ras, double* X,
                                const sdd_newton_opts* o, sdd_newton_result* res, void* stream) {
  int st = check_plan(p, B);
  if (st) return st;
  if (!Ra || !Ras || !X || !o || !res) return SDD_ERR_ARG;
  const int m = o->restart;
  if (m < 1 || m > 64 || o->max_newton < 0 || o->max_restarts < 1 || !(o->tol >= 0.0)) return SDD_ERR_ARG;
  if (o->mixed_matvec && p->prec != SDD_PREC_MIXED) return SDD_ERR_ARG;
  st = newton_reserve(p, B, m);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int n = (int)shell_elems(p);
  const size_t vs = (size_t)B * n;            // stride between Krylov vectors
  GmresState G = gmres_state(p, B, m);
  int* newton_mask = p->nw_ismall + 3 * B;
  const int mv_prec = o->mixed_matvec ? SDD_PREC_MIXED : SDD_PREC_FP64;
  void* base_mv = o->mixed_matvec ? (void*)p->nw_base32 : (void*)p->nw_base64;
  std::vector<double> resF(B, 0.0), target(B, 0.0);
  std::vector<int> nmask(B, 0), iters(B, 0);
  int matvecs = 0;

  auto norms = [&](const double* v) -> int {   // ||v_b||^2 -> p->h_dbl
    SDD_CUDA(krylov_dots(v, 0, v, n, 1, B, p->nw_part, p->nw_nrm2, 1, 0, s));
    SDD_CUDA(cudaMemcpyAsync(p->h_dbl, p->nw_nrm2, B * sizeof(double), cudaMemcpyDeviceToHost, s));
    SDD_CUDA(cudaStreamSynchronize(s));
    return SDD_OK;
  };
  auto jac = [&](const double* v, double* out) -> int {   // out = PDFX(v) about the cached base
    ++matvecs;
    return apply_step(p, B, Ra, Ras, v, out, v, 1, base_mv, mv_prec, s);
  };

  for (int it = 0;; ++it) {
    st = apply_step(p, B, Ra, Ras, X, p->nw_F, X, 0, p->nw_base64, SDD_PREC_FP64, s);   // F = PFX(X)
    if (st) return st;
    if ((st = norms(p->nw_F))) return st;
    bool any = false;
    for (int b = 0; b < B; ++b) {
      resF[b] = std::sqrt(p->h_dbl[b]);
      if (it == 0) res[b].residual0 = resF[b];
      nmask[b] = (resF[b] > o->tol) ? 1 : 0;
      any = any || nmask[b];
    }
    if (!any || it >= o->max_newton) break;
    if (o->mixed_matvec) {
      FxArgs ga = fx_args(p, SDD_PREC_MIXED, X, p->nw_base32, p->out4);
      SDD_CUDA(launch_fx(ga, B, 2, SDD_PREC_MIXED, s));
    }
    for (int b = 0; b < B; ++b) target[b] = o->gmres_rtol * resF[b];
    SDD_CUDA(cudaMemcpyAsync(G.target, target.data(), B * sizeof(double), cudaMemcpyHostToDevice, s));
    SDD_CUDA(cudaMemcpyAsync(G.solve, nmask.data(), B * sizeof(int), cudaMemcpyHostToDevice, s));
    SDD_CUDA(cudaMemcpyAsync(newton_mask, nmask.data(), B * sizeof(int), cudaMemcpyHostToDevice, s));
    SDD_CUDA(cudaMemsetAsync(p->nw_x, 0, (size_t)B * n * sizeof(double), s));
    for (int cyc = 0; cyc < o->max_restarts; ++cyc) {
      const double* r = p->nw_F;
      if (cyc > 0) {                                  // r = F - J x
        if ((st = jac(p->nw_x, p->nw_w))) return st;
        SDD_CUDA(krylov_sub(p->nw_F, p->nw_w, p->nw_r, (size_t)B * n, s));
        r = p->nw_r;
      }
      SDD_CUDA(krylov_dots(r, 0, r, n, 1, B, p->nw_part, p->nw_nrm2, 1, 0, s));
      SDD_CUDA(krylov_cycle_start(G, p->nw_nrm2, B, s));
      SDD_CUDA(krylov_scale(r, G.inv, p->nw_V, n, B, s));
      for (int j = 0; j < m; ++j) {
        double* Vj = p->nw_V + (size_t)j * vs;
        if ((st = jac(Vj, p->nw_w))) return st;
        SDD_CUDA(krylov_dots(p->nw_V, vs, p->nw_w, n, j + 1, B, p->nw_part, G.hcol, m + 1, 0, s));
        SDD_CUDA(krylov_sub_combination(p->nw_V, vs, p->nw_w, G.hcol, m + 1, n, j + 1, B, s));
        SDD_CUDA(krylov_dots(p->nw_V, vs, p->nw_w, n, j + 1, B, p->nw_part, G.h2, m + 1, 0, s));
        SDD_CUDA(krylov_sub_combination(p->nw_V, vs, p->nw_w, G.h2, m + 1, n, j + 1, B, s));
        SDD_CUDA(krylov_dots(p->nw_w, 0, p->nw_w, n, 1, B, p->nw_part, p->nw_nrm2, 1, 0, s));
        SDD_CUDA(krylov_arnoldi_finish(G, p->nw_nrm2, j, B, s));
        if (j + 1 < m) SDD_CUDA(krylov_scale(p->nw_w, G.inv, p->nw_V + (size_t)(j + 1) * vs, n, B, s));
        SDD_CUDA(cudaMemcpyAsync(p->h_int, G.active, B * sizeof(int), cudaMemcpyDeviceToHost, s));
        SDD_CUDA(cudaStreamSynchronize(s));
        bool act = false;
        for (int b = 0; b < B; ++b) act = act || p->h_int[b];
        if (!act) break;
      }
      SDD_CUDA(krylov_solve_y(G, B, s));
      SDD_CUDA(krylov_add_combination(p->nw_V, vs, p->nw_x, G.y, m, G.kb, n, B, s));
      SDD_CUDA(cudaMemcpyAsync(p->h_dbl, G.resid, B * sizeof(double), cudaMemcpyDeviceToHost, s));
      SDD_CUDA(cudaStreamSynchronize(s));
      std::vector<int> again(B, 0);
      bool more = false;
      for (int b = 0; b < B; ++b) {
        again[b] = nmask[b] && p->h_dbl[b] > target[b];
        more = more || again[b];
      }
      if (!more) break;
      SDD_CUDA(cudaMemcpyAsync(G.solve, again.data(), B * sizeof(int), cudaMemcpyHostToDevice, s));
    }
    SDD_CUDA(krylov_masked_sub(X, p->nw_x, newton_mask, n, B, s));
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
    cudaError_t e = cudaEventRecord(ev[0], s);
    FxArgs fa = fx_args(p, p->prec, cur, nullptr, p->out4);
    if (e == cudaSuccess) e = launch_fx(fa, B, 0, p->prec, s);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], s);
    RhsArgs ra = rhs_args(p, cur, p->out4, Ra, Ras, p->rhs, 0);
    if (e == cudaSuccess) e = launch_rhs(ra, B, s);
    if (e == cudaSuccess) e = cudaEventRecord(ev[2], s);
    ChainArgs ca = chain_args(p, p->rhs, dst, nullptr);
    if (e == cudaSuccess) e = launch_chain(ca, B, 3, s);
    if (e == cudaSuccess) e = cudaEventRecord(ev[3], s);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[3]);
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
  SDD_CUDA(launch_fx(fa, batch, 0, SDD_PREC_FP64, s));
  SDD_CUDA(launch_fx_finish(p->M, p->nr, p->Dr, scratch, (size_t)4 * p->M * p->nr, F, shell_elems(p), batch, s));
  return SDD_OK;
}
