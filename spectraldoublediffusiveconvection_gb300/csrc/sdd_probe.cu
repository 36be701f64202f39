// Phase-boundary probe: what a boundary between two dependent phases of a step costs as a kernel boundary
// inside a captured CUDA graph (the form every batched and single-shell step here runs in) against a
// grid-wide barrier inside one persistent kernel (the form a persistent step kernel would take).
//
// Both forms run `nphase` phases of the same work: every thread of `ctas` CTAs applies `work` dependent
// FP64 multiply-adds to its own element (work = 0: the boundary alone).  The persistent kernel is launched
// cooperatively (all CTAs resident, or the launch fails) and separates its phases with a barrier of its
// own: one arrival counter per phase, a bounded spin (about half a second at most; a barrier that runs out
// sets *err and the kernel returns, so the GPU is never held), and fences on both sides.
#include <cuda_runtime.h>

#include "sdd_internal.cuh"

namespace sdd {

__device__ __forceinline__ double probe_work(double x, int work) {
  for (int i = 0; i < work; ++i) x = fma(x, 0.999999999, 1e-9);
  return x;
}

__global__ void k_probe_phase(double* buf, int work) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  buf[e] = probe_work(buf[e], work);
}

// bar[p]: CTAs arrived at the end of phase p (zeroed by the host before the launch)
__global__ void k_probe_persistent(double* buf, int work, int nphase, unsigned* bar, int* err) {
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  __shared__ int s_fail;
  for (int p = 0; p < nphase; ++p) {
    buf[e] = probe_work(buf[e], work);
    if (p + 1 == nphase) break;
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(bar + p, 1u);
      int fail = 1;
      for (long it = 0; it < (1L << 22); ++it) {
        if (*reinterpret_cast<volatile unsigned*>(bar + p) >= gridDim.x) {
          fail = 0;
          break;
        }
        __nanosleep(32);
      }
      __threadfence();
      if (fail) atomicExch(err, 1);
      s_fail = fail;
    }
    __syncthreads();
    if (s_fail) return;
  }
}

}  // namespace sdd

using namespace sdd;

extern "C" int sdd_probe_phase_boundaries(int ctas, int threads, int nphase, int work, int reps, double* graph_us,
                                          double* persistent_us, int* barrier_timed_out, void* stream) {
  if (ctas < 1 || threads < 32 || threads > 1024 || threads % 32 || nphase < 1 || nphase > 4096 || work < 0 ||
      reps < 1 || !graph_us || !persistent_us || !barrier_timed_out)
    return SDD_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, per_sm = 0, sms = 0;
  cudaError_t q = cudaGetDevice(&dev);
  if (q == cudaSuccess) q = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (q == cudaSuccess) q = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_probe_persistent, threads, 0);
  if (q != cudaSuccess) {
    set_cuda_error(q);
    cudaGetLastError();
    return SDD_ERR_CUDA;
  }
  if ((long)per_sm * sms < ctas) return SDD_ERR_UNSUPPORTED;   // not all CTAs resident at once
  double* buf = nullptr;
  unsigned* bar = nullptr;
  int* err = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaStream_t cs = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int st = SDD_OK;
  const size_t n = (size_t)ctas * threads;
  auto fail = [&](cudaError_t ce) {
    set_cuda_error(ce);
    cudaGetLastError();
    st = ce == cudaErrorMemoryAllocation ? SDD_ERR_NOMEM : SDD_ERR_CUDA;
  };
  do {
    cudaError_t ce;
    if ((ce = cudaMalloc(&buf, n * sizeof(double))) != cudaSuccess) { fail(ce); break; }
    if ((ce = cudaMalloc(&bar, (size_t)nphase * sizeof(unsigned))) != cudaSuccess) { fail(ce); break; }
    if ((ce = cudaMalloc(&err, sizeof(int))) != cudaSuccess) { fail(ce); break; }
    if ((ce = cudaMemsetAsync(buf, 0, n * sizeof(double), s)) != cudaSuccess) { fail(ce); break; }
    if ((ce = cudaMemsetAsync(err, 0, sizeof(int), s)) != cudaSuccess) { fail(ce); break; }
    if ((ce = cudaEventCreate(&e0)) != cudaSuccess || (ce = cudaEventCreate(&e1)) != cudaSuccess) { fail(ce); break; }
    // the graph form: nphase launches captured once on a private stream
    if ((ce = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) { fail(ce); break; }
    if ((ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) { fail(ce); break; }
    for (int p = 0; p < nphase; ++p) k_probe_phase<<<ctas, threads, 0, cs>>>(buf, work);
    if ((ce = cudaStreamEndCapture(cs, &graph)) != cudaSuccess) { fail(ce); break; }
    if ((ce = cudaGraphInstantiate(&exec, graph, 0)) != cudaSuccess) { fail(ce); break; }
    float ms = 0.f;
    double best = 1e30;
    for (int r = 0; r < reps + 1; ++r) {                // the first run is a warm-up
      cudaEventRecord(e0, s);
      cudaGraphLaunch(exec, s);
      cudaEventRecord(e1, s);
      if ((ce = cudaEventSynchronize(e1)) != cudaSuccess) { fail(ce); break; }
      cudaEventElapsedTime(&ms, e0, e1);
      if (r > 0 && ms < best) best = ms;
    }
    if (st) break;
    *graph_us = best * 1e3;
    // the persistent form: one cooperative launch, nphase - 1 grid barriers
    best = 1e30;
    for (int r = 0; r < reps + 1; ++r) {
      if ((ce = cudaMemsetAsync(bar, 0, (size_t)nphase * sizeof(unsigned), s)) != cudaSuccess) { fail(ce); break; }
      void* args[] = {&buf, &work, &nphase, &bar, &err};
      cudaEventRecord(e0, s);
      if ((ce = cudaLaunchCooperativeKernel((void*)k_probe_persistent, dim3(ctas), dim3(threads), args, 0, s)) !=
          cudaSuccess) { fail(ce); break; }
      cudaEventRecord(e1, s);
      if ((ce = cudaEventSynchronize(e1)) != cudaSuccess) { fail(ce); break; }
      cudaEventElapsedTime(&ms, e0, e1);
      if (r > 0 && ms < best) best = ms;
    }
    if (st) break;
    *persistent_us = best * 1e3;
    int h_err = 0;
    if ((ce = cudaMemcpy(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess) { fail(ce); break; }
    *barrier_timed_out = h_err;
  } while (false);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cs) cudaStreamDestroy(cs);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(buf);
  cudaFree(bar);
  cudaFree(err);
  return st;
}
