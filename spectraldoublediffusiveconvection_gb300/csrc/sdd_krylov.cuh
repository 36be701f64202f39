// Krylov (GMRES) device state and kernel wrappers, see sdd_krylov.cu.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace sdd {

constexpr int kDotChunk = 2048;   // elements per CTA in the two-level dot products
constexpr int kSubChunk = 512;    // elements per CTA of the fused Gram-Schmidt update and norm
constexpr int kMaxRestart = 64;   // GMRES restart length limit (Newton and continuation check it)

struct GmresState {
  int m;            // restart length
  double* H;        // [B][m+1][m] Hessenberg, rotated in place to R
  double* hcol;     // [B][m+1] first Gram-Schmidt pass projections of the current column
  double* h2;       // [B][m+1] second pass projections
  double* cs;       // [B][m]
  double* sn;       // [B][m]
  double* g;        // [B][m+1] rotated right-hand side beta e1
  double* y;        // [B][m]
  double* beta;     // [B]
  double* inv;      // [B] 1/beta or 1/h_{j+1,j} (0 when the shell is inactive)
  double* resid;    // [B] current GMRES residual estimate |g_{j+1}|
  double* target;   // [B] inner tolerance (absolute)
  int* active;      // [B] still iterating in the current cycle
  int* solve;       // [B] shell takes part in this solve
  int* kb;          // [B] columns used
  int* reo;         // [B] shell repeats the Gram-Schmidt pass for the current column
};

// The second Gram-Schmidt pass of a column runs only where the first one left less than this fraction of
// w's norm (|w'| < eta |w|), the criterion of Daniel, Gragg, Kaufman and Stewart with Kahan's 1/sqrt(2)
// ("twice is enough").  A looser threshold skips more second passes, but classical Gram-Schmidt then
// compounds the loss column by column: with 1e-2 a 50-column cycle was measured to lose orthogonality
// entirely (|V^T V - I| = 1), with 1/sqrt(2) it stays at 2e-15.
constexpr double kReorthEta = 0.70710678118654752440;

// n: used doubles per shell, ld: stride between shells (n <= ld); active (device, nullable): shells whose
// flag is 0 are skipped (dots: zero results; combinations: w left as it was)
// ticket (nullable): B zeroed counters; with it the partials are reduced by each shell's last CTA (one launch)
cudaError_t krylov_dots(const double* V, size_t vstride_i, const double* w, int n, int ld, int nv, int B,
                        double* part, double* h, int ldh, int accumulate, cudaStream_t st,
                        const int* active = nullptr, int* ticket = nullptr);
// The FP32-basis forms (V stored in FP32, the products in FP32 arithmetic, see sdd_krylov.cu) of krylov_dots,
// krylov_sub_norm, krylov_add_combination and krylov_scale (out rounded to FP32; out2 = the FP32 values).
cudaError_t krylov_dots(const float* V, size_t vstride_i, const double* w, int n, int ld, int nv, int B,
                        double* part, double* h, int ldh, int accumulate, cudaStream_t st,
                        const int* active = nullptr, int* ticket = nullptr);
cudaError_t krylov_sub_norm(const float* V, size_t vstride_i, double* w, const double* coef, int ldc, int n, int ld,
                            int nv, int B, const int* sub_mask, const int* norm_mask, double* part, int* ticket,
                            double* nrm2, const GmresState* reo_of, int j, double eta, cudaStream_t st);
cudaError_t krylov_add_combination(const float* V, size_t vstride_i, double* x, const double* y, int ldy,
                                   const int* kb, int n, int ld, int B, cudaStream_t st);
cudaError_t krylov_scale(const double* a, const double* scale, float* out, int n, int ld, int B, cudaStream_t st,
                         float* out32 = nullptr, double* out2 = nullptr);
// One launch for a Gram-Schmidt pass's update and the new norm: w -= V coef where sub_mask (nullable: all),
// nrm2 = |w|^2 where norm_mask (nullable: all; 0 elsewhere), with the sums of krylov_dots; reo_of
// (nullable): also set reo_of->reo for column j (active and |w'|^2 < eta^2 (|w'|^2 + |h|^2), the shells
// whose first pass cancelled w below eta of its norm).  ticket: B zeroed counters.
cudaError_t krylov_sub_norm(const double* V, size_t vstride_i, double* w, const double* coef, int ldc, int n, int ld,
                            int nv, int B, const int* sub_mask, const int* norm_mask, double* part, int* ticket,
                            double* nrm2, const GmresState* reo_of, int j, double eta, cudaStream_t st);
cudaError_t krylov_add_combination(const double* V, size_t vstride_i, double* x, const double* y, int ldy,
                                   const int* kb, int n, int ld, int B, cudaStream_t st);
// out = a * scale[b]; out32 / out2 (nullable, same strides): the result also rounded to FP32 / copied
cudaError_t krylov_scale(const double* a, const double* scale, double* out, int n, int ld, int B, cudaStream_t st,
                         float* out32 = nullptr, double* out2 = nullptr);
cudaError_t krylov_sub(const double* a, const double* b, double* out, size_t n, cudaStream_t st);
cudaError_t krylov_widen(const float* in, double* out, size_t n, cudaStream_t st);   // out = (double)in
cudaError_t krylov_masked_sub(double* X, const double* dx, const int* mask, int n, int ldx, int ld, int B,
                              cudaStream_t st);
cudaError_t krylov_cycle_start(const GmresState& s, const double* nrm2, int B, cudaStream_t st);
cudaError_t krylov_arnoldi_finish(const GmresState& s, const double* nrm2, int j, int B, cudaStream_t st);
cudaError_t krylov_solve_y(const GmresState& s, int B, cudaStream_t st);
cudaError_t krylov_copy_scaled(const double* src, int lds, double* dst, int ldd, int n, double a, const double* last,
                               int B, cudaStream_t st);
cudaError_t krylov_axpy_shell(const double* x0, int ldx0, const double* d, int ldd, const double* c, double* y,
                              int ldy, int n, int B, cudaStream_t st);
cudaError_t contin_grk_T(const double* X, int ldx, double* g, int M, int nr, const double* gr, double dtPr, int sym,
                         int B, cudaStream_t st);
cudaError_t contin_border(const double* v, double* out, int n, int ld, const double* Jmu, int ldj, int Npsi,
                          const double* dot, const double* mudot, double delta, int B, cudaStream_t st);

}  // namespace sdd
