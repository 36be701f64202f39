/*
 * sdd_gb300.h -- C ABI of the GB300 (sm_103a) pseudospectral time-step / Newton hot path of
 * mannixp/SpectralDoubleDiffusiveConvection (axisymmetric double-diffusive convection in a spherical
 * shell, Chebyshev in r x sine/cosine in theta).
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream (as void*), returns an int
 * status (SDD_OK = 0, negative on error) and is stream-ordered.  No entry point synchronises the
 * stream except sdd_newton_gmres (it reads its convergence history back to the host).
 *
 * State layout (the reference's, Matrix_Operators.py:530-575): one shell's state X has 3*N_fm*nr
 * doubles; field f (0 psi, 1 T, 2 S) starts at f*N_fm*nr and mode k occupies [k*nr, (k+1)*nr).
 * psi slot k holds the coefficient of sin((k+1) theta); T/S slot k the coefficient of cos(k theta).
 * A batch of B shells sharing one plan is B such states back to back.
 */
#ifndef SDD_GB300_H
#define SDD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------------- */
#define SDD_OK 0
#define SDD_ERR_ARG (-1)            /* bad pointer / size / enum                                     */
#define SDD_ERR_ODD_NFM (-2)        /* N_fm not even: Matrix_Operators.py:758-759 raises ValueError   */
#define SDD_ERR_UNSUPPORTED (-3)    /* size the kernels do not support (shared memory / FFT radix)   */
#define SDD_ERR_CUDA (-4)           /* a CUDA runtime call failed; sdd_last_cuda_error() has the code */
#define SDD_ERR_NOMEM (-5)          /* device allocation failed                                       */
#define SDD_ERR_NOT_CONVERGED (-6)  /* Newton/GMRES hit its iteration cap (Main.py:541-544)           */

/* precision of the nonlinear term (transforms, products, derivative contractions) */
#define SDD_PREC_FP64 0             /* plain: FP64 throughout                                         */
#define SDD_PREC_MIXED 1            /* FP32 nonlinear term; rhs, chains, residuals stay FP64          */

/* transform kinds (Transforms.py) */
#define SDD_IDCT 0                  /* Transforms.py:116 IDCT(f_hat, n)                               */
#define SDD_IDST 1                  /* Transforms.py:87  IDST(g_hat, n)                               */
#define SDD_DCT 2                   /* Transforms.py:102 DCT(f)[..., :n_out]                          */
#define SDD_DST 3                   /* Transforms.py:73  DST(g)[..., :n_out]                          */

const char* sdd_error_string(int status);
/* the cudaError_t of the last failing CUDA call made by this library (0 if none) */
int sdd_last_cuda_error(void);
/* library version as major*10000 + minor*100 + patch */
int sdd_version(void);

/* ---- theta transforms ------------------------------------------------------------------------ */
/* Batched rows.  Replaces Transforms.py:73-129 (DCT, DST, IDCT, IDST).
 * Inverse kinds (IDCT/IDST): in = rows x n_in sinusoid amplitudes, out = rows x n_out grid values on
 *   grid(n_out) (Transforms.py:8); n_out >= n_in zero-pads exactly as IDCT(f_hat, n=n_out) does.
 * Forward kinds (DCT/DST): in = rows x n_in grid values, out = rows x n_out leading sinusoid
 *   amplitudes (n_out <= n_in), i.e. DCT(f)[..., :n_out].
 * fp64 arithmetic; in and out may not alias. */
int sdd_transform(int kind, int rows, int n_in, int n_out, const double* in, double* out,
                  void* stream);

/* ---- plan: device-resident operators for one (N_fm, N_r, d, dt, Pr, Tau, symmetric) ------------ */
/* All host arrays are FP64, row-major, built by the caller with the reference's formulas
 * (Main.py:179-225 Build_Matrix_Operators and the operator builders it calls). */
typedef struct sdd_plan_desc {
  int32_t N_fm;            /* theta modes M (even)                                                 */
  int32_t nr;              /* interior radial points N_r - 1                                       */
  int32_t symmetric;       /* 1: equatorially symmetric subspace (Main.py:137-176)                  */
  int32_t precision;       /* SDD_PREC_FP64 or SDD_PREC_MIXED                                      */
  double dt, Pr, Tau;      /* step of this operator set (dt=1 for Newton, Main.py:430)             */
  const double* Dr;        /* nr*nr  D[1:-1,1:-1]                         (Matrix_Operators.py:764)*/
  const double* D2_r2;     /* nr*nr  (diag(1/R^2) D@D)[1:-1,1:-1]         (A2_SINE_R2 :498)        */
  const double* ir4_r2;    /* nr     1/R^4                                (A2_SINE_R2 :496)        */
  const double* D2_sine;   /* nr*nr  (D@D)[1:-1,1:-1]                     (A2_SINE :217)           */
  const double* ir2_sine;  /* nr     1/R^2                                (A2_SINE :216)           */
  const double* D2_A4;     /* nr*nr  args_A4 D2                           (Main.py:212)            */
  const double* ir2_A4;    /* nr     diag of args_A4 IR2                  (Main.py:213)            */
  const double* ir4_A4;    /* nr     diag of args_A4 IR4                  (Main.py:214)            */
  const double* rsq;       /* nr     R^2 (R2 block diagonal)              (Matrix_Operators.py:85) */
  const double* dT0;       /* nr     A_T/R^2                              (Main.py:201-202)        */
  const double* gr;        /* nr     R_1^2/R^2 (kGR_RT diagonal)          (Matrix_Operators.py:113)*/
  const double* Linv_A4;   /* N_fm*nr*nr  A4_TSTEP_MATS(Pr*dt)            (Matrix_Operators.py:1089)*/
  const double* Linv_T;    /* N_fm*nr*nr  NAB2_TSTEP_MATS(dt)             (Matrix_Operators.py:1014)*/
  const double* Linv_S;    /* N_fm*nr*nr  NAB2_TSTEP_MATS(Tau*dt)                                  */
  /* diagnostics (sdd_diagnostics / sdd_step_diag); nullable: without them those entry points return
   * SDD_ERR_UNSUPPORTED                                                                             */
  const double* nu_w;      /* nr     (R[0]^2/A_T) D[0][1..nr]: Nusselt weights (Main.py:41-68)         */
  const double* r_int;     /* nr     interior radii R[1:-1] (Kinetic_Energy trapezoid, Main.py:124-131) */
  double r_i, r_o;         /* R[0], R[-1] (Kinetic_Energy volume, Main.py:132)                      */
} sdd_plan_desc;

typedef struct sdd_plan sdd_plan;

/* Uploads the operators to the current device.  Replaces Main.py:179-225 (the returned tuple).  Sizes:
 * nr <= 64 (N_r <= 65); N_fm even, with P = 3 N_fm / 2 a product of the radices 2, 3, 4, 5, 7 and the fused
 * FP64 row kernel's 34 P doubles beside its static shared memory within a CTA's limit (N_fm <= 540 on
 * GB300); otherwise SDD_ERR_UNSUPPORTED before anything is allocated (odd N_fm: SDD_ERR_ODD_NFM). */
int sdd_plan_create(const sdd_plan_desc* desc, sdd_plan** plan);
int sdd_plan_destroy(sdd_plan* plan);
/* Pre-allocates the plan's workspace for up to max_batch shells (otherwise grown on first use). */
int sdd_plan_reserve(sdd_plan* plan, int max_batch);
/* Chain-kernel layout of the implicit solves: 0 automatic (chunked while its CTAs fit the GPU at two per
 * SM, layout 3 before 2, else split rows over 4 warps when the launch leaves SMs idle, else layout 8 (6 for
 * launches of fewer than three fields or where its shared memory does not fit, 5 where the right-hand side
 * is fused or FP32)),
 * 1 one lane per row, 2 chunked (each chain cut into chunks that run concurrently, joined by a short
 * sequential carried-state recurrence), 3 chunked with shorter chunks joined by a parallel carry
 * (precomputed products of the chunk maps, all applied at once), 4 split rows over 4 warps, 5 split rows
 * over 2 lanes in 2 warps (nr <= 32; 4 otherwise), 6 / 7 the chains in the reference's own order of
 * operations (Matrix_Operators.py:1139-1164, 1056-1083: per step D2 f_e, then Linv_j (g_j + b)), without the
 * h = Linv g pre-pass of the other layouts: 4 nr^2 multiply-adds per mode instead of 7, rows over 2 / 4
 * lanes; they need the full FP64 right-hand side, so launches with the fused or the FP32 right-hand side run
 * layout 5.  8: the same order of operations with the three chains of one (parity, shell) in one CTA, psi
 * rows over 2 lanes, T and S one lane per row, so every warp carries about the same work per step (launches
 * of fewer than three fields run layout 6).  9: the h pre-pass form (any right-hand side: fused, FP32) with
 * the three chains of one (parity, shell) in one CTA, psi rows over 2 lanes, T and S one lane per row
 * (launches of fewer than three fields, or whose three rings exceed a CTA's shared memory, run layout 5).
 * 10 / 11: the chunks of layouts 2 / 3 with each chunk in the reference's order of operations (no h
 * pre-pass; with the right-hand side fused into the split nonlinear term each chunk forms its own; FP32
 * right-hand sides run layouts 2 / 3).  The automatic choice runs its chunked layout as 10 / 11 where the
 * full FP64 right-hand side is there, and as 2 / 3 where it is fused (one shell: the pre-pass form is
 * faster there).  Set by the batch autotuner; no counterpart in the reference. */
int sdd_plan_set_chain_layout(sdd_plan* plan, int layout);
/* Chunk length (steps per chunk) of chunk set 0 (layouts 2 / 10, sequential carry) or 1 (layouts 3 / 11,
 * parallel carry): the set's tables are rebuilt for kc and the carry workspace regrown; kc = 0 restores the
 * plan's rule (round(sqrt(2 S)) / round(sqrt(S / 2)) steps, S = N_fm / 2).  2 <= kc <= S, at most 64 chunks
 * (32 for set 1, whose products grow as the square); otherwise SDD_ERR_ARG.  Synchronises the device.  Set
 * by the batch autotuner; no counterpart in the reference. */
int sdd_plan_set_chunk_length(sdd_plan* plan, int set, int kc);
/* The layout (1-11) a step of `batch` shells runs under the current setting, with its chunk length and
 * chunks per chain (0 and 1 when not chunked). */
int sdd_plan_chain_choice(const sdd_plan* plan, int batch, int* layout, int* kc, int* nch);
/* Mixed plans: the FP32 radial contractions of the nonlinear term (Derivatives, Matrix_Operators.py:698-729)
 * on the tensor cores (1, the default: 3xTF32 split products with tcgen05.mma, FP32-level accuracy) or as FP32
 * multiply-adds on the CUDA cores (0).  SDD_ERR_UNSUPPORTED for FP64 plans.  No counterpart in the
 * reference. */
int sdd_plan_set_tensor_cores(sdd_plan* plan, int on);
/* 1 in *timed_out if a tensor-core kernel of this plan gave up waiting for its matrix products (its outputs
 * were then NaN); 0 otherwise.  Synchronous. */
int sdd_plan_tensor_core_status(const sdd_plan* plan, int* timed_out);
/* Phase-boundary probe (no plan): `nphase` phases of `work` dependent FP64 multiply-adds per thread over
 * ctas x threads threads, once as a captured CUDA graph of nphase kernel launches and once as one
 * cooperative (persistent) kernel with nphase - 1 grid-wide barriers of its own (bounded spins: a barrier
 * that runs out sets *barrier_timed_out and the kernel returns).  Best of `reps` timed runs of each, in
 * microseconds.  SDD_ERR_UNSUPPORTED if the CTAs cannot all be resident at once.  Measures what a persistent
 * step kernel could save over the captured step graphs; no counterpart in the reference. */
int sdd_probe_phase_boundaries(int ctas, int threads, int nphase, int work, int reps, double* graph_us,
                               double* persistent_us, int* barrier_timed_out, void* stream);
/* How the Newton / continuation GMRES products of this plan ran so far: captured into a CUDA graph (and
 * launched), replayed from a captured graph, or launched kernel by kernel (a product that could not be
 * captured).  The products of every Arnoldi column read one fixed vector, so a solve captures a product
 * once per batch size and kind and replays it for the other columns and later solves.  No counterpart in
 * the reference. */
int sdd_plan_product_graph_stats(const sdd_plan* plan, long long* captured, long long* replayed, long long* direct);
/* 1 (the default): the GMRES products run as captured CUDA graphs; 0: kernel by kernel (the same kernels
 * and arguments, so the same results).  No counterpart in the reference. */
int sdd_plan_set_product_graphs(sdd_plan* plan, int on);
/* Nonlinear-term kernel choice: 0 automatic (split while the fused kernel's nr*batch CTAs would fill
 * under half the SMs), 1 the fused row kernel (one CTA per radial row), 2 split (7 CTAs per radial row:
 * five paired inverse transforms, then two paired forward transforms).  Results are identical bit for
 * bit.  Set by the batch autotuner; no counterpart in the reference. */
int sdd_plan_set_fx_split(sdd_plan* plan, int mode);
/* FP64 elements of one shell's base-state grid cache used by sdd_nlin_dfx (9 * nr * 3N_fm/2). */
size_t sdd_plan_base_cache_elems(const sdd_plan* plan);

/* ---- Matrix_Operators.py drop-ins (batched over shells sharing the plan) ----------------------- */
/* F(X,X), Matrix_Operators.py:743-804 NLIN_FX.  X, F: batch x 3*N_fm*nr.
 * base_cache (nullable, batch x sdd_plan_base_cache_elems): receives X's nine padded grid fields. */
int sdd_nlin_fx(sdd_plan* plan, int batch, const double* X, double* F, double* base_cache,
                void* stream);
/* DF(X) dv = F(X,dv)+F(dv,X), Matrix_Operators.py:807-898 NLIN_DFX.  base_cache (nullable) must hold
 * X's grid fields from sdd_nlin_fx; when NULL they are recomputed from X. */
int sdd_nlin_dfx(sdd_plan* plan, int batch, const double* dv, const double* X,
                 const double* base_cache, double* out, void* stream);
/* psi solve, Matrix_Operators.py:1115-1194 A4_BSub_TSTEP_V2 with the plan's Linv_A4 and dt*Pr.
 * g, f: batch x N_fm*nr. */
int sdd_a4_bsub(sdd_plan* plan, int batch, const double* g, double* f, void* stream);
/* T (field=1, dt) or S (field=2, Tau*dt) solve, Matrix_Operators.py:1033-1086 NAB2_BSub_TSTEP_V2. */
int sdd_nab2_bsub(sdd_plan* plan, int field, int batch, const double* g, double* f, void* stream);
/* theta-coupling recurrences (batch x N_fm*nr in and out):
 * op 0 J_theta_RT (Matrix_Operators.py:436), 1 A2_SINE_R2 (:475), 2 A2_SINE (:192), 3 DT0_theta (:131) */
int sdd_theta_op(sdd_plan* plan, int op, int batch, const double* g, double* f, void* stream);

/* ---- Main.py drivers ------------------------------------------------------------------------- */
/* nsteps IMEX ("CNAB1") steps, Main.py:255-283 Step_Python inside the loop of _Time_Step :286-324
 * (X <- X_SYM * X_new).  Ra, Ra_s: per-shell device arrays (batch).  X_in and X_out may alias.
 * linear != 0 drops the nonlinear term (Main.py:261-264). */
int sdd_step(sdd_plan* plan, int batch, const double* Ra, const double* Ra_s, const double* X_in,
             double* X_out, int nsteps, int linear, void* stream);
/* One group of a batched call: `batch` shells of one plan (device arrays as in sdd_step). */
typedef struct sdd_batch_group {
  sdd_plan* plan;
  int32_t batch;
  int32_t pad;
  const double* Ra;
  const double* Ra_s;
  const double* X_in;
  double* X_out;
} sdd_batch_group;
/* sdd_step for several plans at once (shells of different shapes, one plan per shape group; no counterpart
 * in the reference, which steps one shell per process): every group runs on its plan's own branch stream,
 * forked from and joined back into `stream` by events, so the groups run concurrently and the call is
 * ordered on `stream` like one sdd_step.  Captured on `stream`, it becomes one graph with a branch per group.
 * Each plan may appear once per call (SDD_ERR_ARG otherwise); a group's result equals its sdd_step alone. */
int sdd_batch_step(const sdd_batch_group* groups, int ngroups, int nsteps, int linear, void* stream);
/* One Crank-Nicolson / Adams-Bashforth-2 step (an opt-in scheme; the reference and sdd_step are IMEX Euler,
 * "CNAB1", Main.py:255-283).  The plan is built with HALF the step, dt_plan = dt/2 (its blocks invert
 * A^2 - (dt/2) Pr A^4 and r^2 - (dt/2) r^2 Lap, Matrix_Operators.py:1014-1112): composed of the reference's
 * own operations, psi' = A4_BSub(2 A2_SINE(psi) + dt E~_psi) - psi and T' = NAB2_BSub(2 r^2 T + dt E~_T) - T
 * (S alike with Tau), where E are the explicit terms per unit time (psi: -NLIN_FX_psi + Pr gr_k(Ra T - Ra_s S);
 * T/S: -NLIN_FX_T/S - DT0_theta(psi)) and E~ = 3/2 E - 1/2 E_prev.  hist (device, batch x 3*N_fm*nr) holds
 * E_prev on entry when hist_valid (else E~ = E: the first step), and this step's E on exit.  X_in, X_out
 * and hist must not alias. */
int sdd_step_cnab2(sdd_plan* plan, int batch, const double* Ra, const double* Ra_s, const double* X_in,
                   double* X_out, double* hist, int hist_valid, void* stream);
/* Newton residual F(X) = Phi_dt(X) - X, Main.py:473-496 PFX.  base_cache as in sdd_nlin_fx. */
int sdd_pfx(sdd_plan* plan, int batch, const double* Ra, const double* Ra_s, const double* X,
            double* F, double* base_cache, void* stream);
/* Jacobian-vector product, Main.py:498-521 PDFX. */
int sdd_pdfx(sdd_plan* plan, int batch, const double* Ra, const double* Ra_s, const double* dv,
             const double* X, const double* base_cache, double* out, void* stream);

/* ---- matrix-free Newton-GMRES steady states (Main.py:430-554 _Newton) -------------------------- */
/* The reference solves DF(X) dv = F(X) with scipy lgmres and stops on the relative step
 * |dv|/|X| < tol (Main.py:523-536), which cannot be met when the solution is X = 0.  Here the stop is
 * the absolute FP64 residual |F(X)|_2 <= tol; the inner solve is restarted GMRES(restart) with CGS2
 * orthogonalisation and inner tolerance gmres_rtol*|F| (the reference's atol = tol_gmres*|F|). */
typedef struct sdd_newton_opts {
  double tol;              /* absolute |F(X)|_2 target                                              */
  double gmres_rtol;       /* inner tolerance relative to |F(X)|                                     */
  int32_t restart;         /* GMRES restart length (<= 64)                                          */
  int32_t max_restarts;    /* GMRES cycles per Newton iteration                                     */
  int32_t max_newton;      /* Newton iteration cap                                                  */
  int32_t mixed_matvec;    /* 1: FP32 nonlinear term inside the Jacobian products (plan must be mixed);
                              2: also FP32 right-hand sides and h = Linv g matvecs (chains stay FP64);
                              3: as 2 with the GMRES basis stored and orthogonalised in FP32 (the
                              residual, its norm and the update stay FP64)                          */
} sdd_newton_opts;

typedef struct sdd_newton_result {
  double residual0;        /* |F(X0)|_2                                                             */
  double residual;         /* |F(X)|_2 at exit (FP64)                                               */
  int32_t newton_iters;    /* Newton updates applied                                                */
  int32_t matvecs;         /* Jacobian-vector products (batch-wide)                                 */
  int32_t converged;       /* residual <= tol                                                       */
  int32_t pad;
} sdd_newton_result;

/* In place: X (batch x 3*N_fm*nr, device) is replaced by the Newton iterate.  results: host array of
 * batch entries.  Uses the plan's dt (1 for Newton, Main.py:430).  Synchronises the stream (it reads
 * residuals back to decide convergence).  Returns SDD_ERR_NOT_CONVERGED if a shell misses tol. */
int sdd_newton_gmres(sdd_plan* plan, int batch, const double* Ra, const double* Ra_s, double* X,
                     const sdd_newton_opts* opts, sdd_newton_result* results, void* stream);

/* The classical Gram-Schmidt pass of a GMRES column is repeated where the first pass left less than eta of
 * the column's norm (|w'| < eta |w|); default 1/sqrt(2); eta >= 1 repeats it on every column, 0 never.
 * Thresholds well below the default lose the basis' orthogonality over long cycles.  No counterpart in
 * the reference (scipy's lgmres). */
int sdd_plan_set_reorth_eta(sdd_plan* plan, double eta);
/* Copies the Krylov basis vectors V_0 .. V_{k-1} of the last GMRES cycle of the last solve of this plan
 * (sdd_newton_gmres / sdd_contin_step) for one shell into out (device, max_cols x 3*N_fm*nr doubles);
 * *ncols = k (at most max_cols).  Synchronous.  For checking the basis' orthogonality. */
int sdd_krylov_basis(const sdd_plan* plan, int shell, int max_cols, double* out, int* ncols, void* stream);

/* ---- pseudo-arclength continuation step (Main.py:742-955 _ContinC) ------------------------------ */
/* One step along the branch of steady states in Ra_T.  Predictor: with dt = 1 the reference always
 * recomputes the tangent from DF_X xi = -DF_mu (Main.py:845-862): mu_dot = sign/sqrt(1 + delta(|xi|-1)),
 * X_dot = mu_dot xi, delta = 1/(3 N_fm nr); prediction Y = Y0 + ds Y_dot.  Corrector: Newton on the
 * bordered system [[DF_X, DF_mu], [delta X_dot^T, (1-delta) mu_dot]] (Main.py:914-920) solved by GMRES; ds is
 * halved after max_corrector iterations (Main.py:888-899).  The stop is absolute: |F(X,Ra)|_2 <= tol and
 * |arclength residual| <= tol.  New tangent: DG y = e_last, normalised (Main.py:944-953).
 * X (batch x 3 N_fm nr) and Ra (batch) are device arrays updated in place; X_dot (device, batch x n)
 * receives the new tangent's state part; sign and ds are host arrays (batch). */
typedef struct sdd_contin_opts {
  double tol;              /* absolute corrector tolerance                                          */
  double gmres_rtol;       /* corrector inner tolerance relative to the bordered residual (:919)    */
  double tangent_rtol;     /* predictor/tangent inner tolerance (the reference uses tol_newton)    */
  int32_t restart, max_restarts;
  int32_t max_corrector;   /* corrector iterations before ds is halved (5)                         */
  int32_t max_halvings;
  int32_t mixed_matvec;    /* as in sdd_newton_opts: 0 FP64 products, 1 FP32 nonlinear term, 2 also FP32
                              right-hand sides and h matvecs, 3 also an FP32 Krylov basis (mixed plans) */
  int32_t pad;
} sdd_contin_opts;

typedef struct sdd_contin_result {
  double residual;         /* |F(X,Ra)|_2 at exit                                                  */
  double arclength;        /* |arclength residual| at exit                                          */
  double ds;               /* step for the next call (doubled after <= 4 corrector iterations)     */
  double Ra_dot;           /* parameter component of the new normalised tangent                    */
  int32_t corrector_iters, halvings, matvecs, converged;
} sdd_contin_result;

int sdd_contin_step(sdd_plan* plan, int batch, double* X, double* Ra, const double* Ra_s, double* X_dot,
                    const double* sign, const double* ds, const sdd_contin_opts* opts,
                    sdd_contin_result* results, void* stream);

/* ---- nonlinear term without any allocation (no counterpart in the reference) --------------------- */
/* NLIN_FX like sdd_nlin_fx, for callers that must not allocate device memory when they call it: hosts
 * whose device memory is owned by another allocator (a framework's caching allocator, a serving runtime
 * that reserves the whole budget up front) and latency-critical paths where cudaMalloc/cudaFree, which can
 * synchronise the device, are not allowed.  The plan (created earlier) supplies the operators; X and F are
 * the caller's.  The intermediate spectral outputs (4*N_fm*nr doubles per shell) go to a fixed scratch
 * array of SDD_NOALLOC_SCRATCH_DOUBLES doubles (8 MiB) that the library keeps in device memory on every
 * GPU it is loaded on until the process exits; batch*4*N_fm*nr above that limit returns
 * SDD_ERR_UNSUPPORTED.  The first call on a device looks up the array's device address, so make that first
 * call before any stream capture.  Every call on a device shares the one array (each call overwrites all
 * of it that it reads, so stale contents never leak into a result): calls that overlap on the GPU race. */
#define SDD_NOALLOC_SCRATCH_DOUBLES (1 << 20)
int sdd_nlin_fx_noalloc(sdd_plan* plan, int batch, const double* X, double* F, void* stream);

/* ---- radial contractions on the tensor cores ------------------------------------------------- */
/* The four radial contractions of Derivatives (Matrix_Operators.py:698-729: Dr psi_k, (D^2/r^2) psi_k
 * (A2_SINE_R2 :498), Dr T_k, Dr S_k) of every mode of every shell, as the mixed plans' nonlinear term forms
 * them: 3xTF32 products on the tensor cores (tcgen05.mma, TMEM accumulators), FP32-level accuracy.
 * X32: batch x 3*N_fm*nr floats (the state in FP32, reference layout); out: batch x 4*nr*N_fm floats,
 * out[shell][op][n][k] (op 0..3 in the order above, radial row n, mode k contiguous).  Rows outside the
 * symmetric subspace give zeros.  Mixed plans only (SDD_ERR_UNSUPPORTED otherwise). */
int sdd_deriv_tc(sdd_plan* plan, int batch, const float* X32, float* out, void* stream);

/* ---- instrumentation (no counterpart in the reference) ---------------------------------------- */
/* Runs nsteps steps like sdd_step (launched one by one, not from graphs) with CUDA events between the
 * three stages of each step and adds the elapsed milliseconds to ms[0] (nonlinear term), ms[1]
 * (right-hand sides; ~0 when fused into the other two) and ms[2] (implicit solves).  Synchronises the
 * stream. */
int sdd_step_profile(sdd_plan* plan, int batch, const double* Ra, const double* Ra_s, const double* X_in,
                     double* X_out, int nsteps, double* ms, void* stream);
/* Per-shell diagnostics of the state X (device, batch x 3*N_fm*nr) into out (device, batch x 4):
 * |X|_2, Kinetic_Energy (Main.py:71-134), Nusselt of T and of S (Main.py:41-68, without the check).
 * Replaces the per-step scalar records of _Time_Step (Main.py:285-296). */
int sdd_diagnostics(sdd_plan* plan, int batch, const double* X, double* out, void* stream);
/* nsteps steps like sdd_step (launched one by one), with the diagnostics of the state after every step
 * written to diag (device, nsteps x batch x 4). */
int sdd_step_diag(sdd_plan* plan, int batch, const double* Ra, const double* Ra_s, const double* X_in,
                  double* X_out, int nsteps, int linear, double* diag, void* stream);
/* Kernel ids of sdd_step_kernel_profile and their names (sdd_kernel_name). */
#define SDD_K_FX_ROWS 0      /* fused nonlinear-term row kernel */
#define SDD_K_FX_DERIV 1     /* split path: radial derivatives per mode */
#define SDD_K_FX_GRID 2      /* split path: paired inverse transforms to the grid */
#define SDD_K_FX_PROD 3      /* split path: grid products and paired forward transforms */
#define SDD_K_RHS 4          /* right-hand sides */
#define SDD_K_MODE_H 5       /* h = Linv g per mode */
#define SDD_K_CHAIN 6        /* the chains (whole, or the concurrent chunks) */
#define SDD_K_CHAIN_CARRY 7  /* chunked chains: carried states */
#define SDD_K_MODE_FIX 8     /* chunked chains: correction per mode */
#define SDD_K_DERIV_TC 9     /* mixed plans: radial contractions on the tensor cores (3xTF32) */
#define SDD_NUM_KERNELS 10
const char* sdd_kernel_name(int id);
/* Like sdd_step_profile, but with an event after every kernel launch: adds the elapsed milliseconds of
 * each kernel to ms[id] and counts its launches in launches[id] (arrays of SDD_NUM_KERNELS). */
int sdd_step_kernel_profile(sdd_plan* plan, int batch, const double* Ra, const double* Ra_s,
                            const double* X_in, double* X_out, int nsteps, double* ms, int* launches,
                            void* stream);
/* Test hook (no counterpart in the reference): the next `after` workspace allocations (sdd_plan_reserve, and
 * the Krylov workspace of sdd_newton_gmres / sdd_contin_step) succeed and every later one fails on the host,
 * before cudaMalloc is called, as if the device were out of memory, so that a caller can check how
 * SDD_ERR_NOMEM reaches it.  after < 0 removes the limit.  Process-wide. */
int sdd_debug_fail_allocations(long long after);
/* Measured FP64 FMA throughput of the current device in GFLOP/s (a register-resident FMA loop over
 * all SMs, a few milliseconds).  The roofline denominator of the FP64-bound kernels. */
int sdd_measure_fp64_peak(double* gflops, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SDD_GB300_H */
