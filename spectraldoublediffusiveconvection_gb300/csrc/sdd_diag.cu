// Per-step diagnostics of _Time_Step (Main.py:285-296): the 2-norm of the state, the volume-averaged
// kinetic energy (Kinetic_Energy, Main.py:71-134) and the Nusselt numbers of T and S (Nusselt,
// Main.py:41-68), on the device.
//
// Kinetic energy.  With JPSI = J_theta_RT(psi) (Matrix_Operators.py:437), the reference forms for every
// interior radius r_n the cosine row JPSI_k(r_n)/r_n and the sine row (Dr psi_k)(r_n) (shifted to the
// sinusoid convention), transforms both to the 3 N_fm midpoint grid (IDCT / IDST with n = 3 N_fm) and
// integrates |.|^2 by the trapezoidal rule over r (x = R interior) and then over theta with sin(theta).
// Both rules are weighted sums, so KE = (1/2V) sum_n wr_n sum_i wt_i sin(theta_i) (J^2 + D^2)(r_n, theta_i):
// k_diag_rows computes the inner sum of one radius (the two transforms ride in one complex FFT of length
// 3 N_fm, power-of-two balanced as in the other transforms) and k_diag_final the outer sums.
//
// Nusselt.  Nu - 1 at r = R[0] is (R[0]^2/A_T) sum_{k even} (D TT_k)[0]/(1 - k^2), TT_k the zero-padded
// radial profile of mode k: a fixed weighted sum of the even-mode coefficients (weights from the plan).
#include <cuda_runtime.h>

#include "sdd_fft.cuh"
#include "sdd_rowops.cuh"
#include "sdd_internal.cuh"

namespace sdd {

template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int t = 0; t < K; ++t) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v[t] += __shfl_xor_sync(0xffffffffu, v[t], off);
    if (lane == 0) red[t * 32 + warp] = v[t];
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += red[threadIdx.x * 32 + w];
    red[32 * K + threadIdx.x] = s;
  }
  __syncthreads();
#pragma unroll
  for (int t = 0; t < K; ++t) v[t] = red[32 * K + t];
}

size_t diag_rows_smem_bytes(int M, int L) { return (4 * (size_t)L * 2 + 5 * (size_t)M + 8) * sizeof(double) + 4 * 32 * 8; }

// One CTA per (interior radius n, shell).
__global__ void __launch_bounds__(256) k_diag_rows(DiagArgs a) {
  using C = double2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int M = a.M, nr = a.nr, L = a.L;
  const int n = blockIdx.x, b = blockIdx.y;
  const int tid = threadIdx.x, bd = blockDim.x;
  C* RA = reinterpret_cast<C*>(smem_raw);
  C* RB = RA + L;
  C* Wt = RB + L;
  C* Et = Wt + L;
  double* pv = reinterpret_cast<double*>(Et + L);
  double* Sc = pv + M;
  double* dp = Sc + M;
  double* Ar = dp + M;        // cosine row: J_theta_RT(psi)_k(r_n) / r_n
  double* Br = Ar + M;        // sine row: (Dr psi)_{k-1}(r_n), [0] = 0
  double* scl = Br + M;       // 2 scales + 2 inverses
  unsigned long long* red = reinterpret_cast<unsigned long long*>(scl + 8);
  for (int i = tid; i < L; i += bd) {
    Wt[i] = a.w[i];
    Et[i] = a.e[i];
  }
  const double* ps = a.X + (size_t)b * a.x_stride;
  const double* drn = a.Dr + (size_t)n * nr;
  for (int k = tid; k < M; k += bd) {
    const double* pk = ps + (size_t)k * nr;
    double acc = 0.0;
    for (int m = 0; m < nr; ++m) acc = fma(drn[m], pk[m], acc);
    dp[k] = acc;
    pv[k] = (a.sym && (k % 2 == 0)) ? 0.0 : pk[n];
  }
  __syncthreads();
  parity_suffix<double>(pv, Sc, M);   // as J_theta_RT
  __syncthreads();
  const double irn = a.ir[n];
  unsigned long long mb[2] = {0, 0};
  for (int k = tid; k < M; k += bd) {
    const double s1 = (k + 1 < M) ? Sc[k + 1] : 0.0;
    double jp = (k == 0) ? 1.0 * s1 : (k + 1.0) * pv[k - 1] + 2.0 * s1;
    if (a.sym && (k % 2 == 1)) jp = 0.0;
    const double av = irn * jp;
    const double bv = k >= 1 ? dp[k - 1] : 0.0;
    Ar[k] = av;
    Br[k] = bv;
    const unsigned long long ua = Bits<double>::absbits(av), ub = Bits<double>::absbits(bv);
    mb[0] = ua > mb[0] ? ua : mb[0];
    mb[1] = ub > mb[1] ? ub : mb[1];
  }
  block_max_scales<double, 2>(mb, red, scl);   // ends with a barrier
  const double sa = scl[0], sb = scl[1];
  // DCT3 inputs with n_in = M on length L (see k_transform): cosine x_k = A_k; sine x_k = B_{L-k}
  for (int k = tid; k < L; k += bd) {
    const double xa = (k < M) ? Ar[k] : 0.0;
    const double xb = (L - k <= M - 1 && k > 0) ? Br[L - k] : 0.0;
    if (k == 0) {
      RA[k] = make_double2(sa * xa, sb * xb);
    } else {
      const double xar = (L - k < M) ? Ar[L - k] : 0.0;
      const double xbr = (k <= M - 1) ? Br[k] : 0.0;
      const C e = Et[k];
      const double a1 = fma(e.x, xa, e.y * xar), a2 = fma(e.y, xa, -(e.x * xar));
      const double b1 = fma(e.x, xb, e.y * xbr), b2 = fma(e.y, xb, -(e.x * xbr));
      RA[k] = make_double2(fma(sa, a1, -(sb * b2)), fma(sa, a2, sb * b1));
    }
  }
  __syncthreads();
  C* res = fft_rows<double, true>(RA, RB, 1, a.st, Wt);
  double s[1] = {0.0};
  for (int i = tid; i < L; i += bd) {
    const int src = (i & 1) ? (L - 1 - (i >> 1)) : (i >> 1);
    const C v = res[src];
    const double ja = v.x * scl[2];
    double db = v.y * scl[3];
    if (i & 1) db = -db;
    s[0] = fma(a.tw[i], fma(ja, ja, db * db), s[0]);
  }
  block_sum<1>(s, reinterpret_cast<double*>(red));
  if (tid == 0) a.part[(size_t)b * nr + n] = s[0];
}

// One CTA per shell: |X|_2, KE from the per-radius sums, Nu_T and Nu_S.
__global__ void __launch_bounds__(256) k_diag_final(DiagArgs a) {
  __shared__ double red[32 * 4 + 4];
  const int M = a.M, nr = a.nr, b = blockIdx.x;
  const size_t N = (size_t)M * nr;
  const double* X = a.X + (size_t)b * a.x_stride;
  double v[4] = {0.0, 0.0, 0.0, 0.0};   // |X|^2, KE, NuT, NuS
  for (size_t e = threadIdx.x; e < 3 * N; e += blockDim.x) v[0] = fma(X[e], X[e], v[0]);
  for (int n = threadIdx.x; n < nr; n += blockDim.x) v[1] = fma(a.wr[n], a.part[(size_t)b * nr + n], v[1]);
  const int ne = (M + 1) / 2;
  for (int e = threadIdx.x; e < ne * nr; e += blockDim.x) {
    const int kk = e / nr, m = e - kk * nr;
    const size_t o = (size_t)(2 * kk) * nr + m;
    v[2] = fma(a.nuw[e], X[N + o], v[2]);
    v[3] = fma(a.nuw[e], X[2 * N + o], v[3]);
  }
  block_sum<4>(v, red);
  if (threadIdx.x == 0) {
    double* o = a.out + (size_t)b * 4;
    o[0] = sqrt(v[0]);
    o[1] = a.ke_scale * v[1];
    o[2] = v[2];
    o[3] = v[3];
  }
}

cudaError_t launch_diag(const DiagArgs& a, int batch, cudaStream_t s) {
  static unsigned long long done = 0;
  cudaError_t e = ensure_smem_attr(k_diag_rows, &done);
  if (e != cudaSuccess) return e;
  if ((e = launch_kernel(k_diag_rows, dim3(a.nr, batch), dim3(256), diag_rows_smem_bytes(a.M, a.L), s, a)) !=
      cudaSuccess)
    return e;
  return launch_kernel(k_diag_final, dim3(batch), dim3(256), 0, s, a);
}

}  // namespace sdd
