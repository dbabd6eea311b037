// Cost of a pass boundary on one GPU, two ways (test infrastructure, run by
// tests/test_gpu_pass_boundary.py):
//  * a grid-wide barrier inside a cooperative persistent kernel (flat: one arrival counter;
//    tree: 16 group counters, then one root counter), every spin capped at `cap` polls, after
//    which the CTA records a timeout in g_err and returns;
//  * the boundary between two kernels on one stream: empty kernels launched back to back,
//    directly or from a CUDA graph, with and without programmatic stream serialization (each
//    kernel waits with griddepcontrol.wait, as the solver's pass kernels do).
// It also checks the capped wait: with cap = 0 the barrier kernel must return with g_err set, and
// a following launch with the normal cap must complete with g_err clear.
// Output: one line per measurement, "barrier <flat|tree> <ctas> <threads> <us> <err>" and
// "kernel <pdl 0|1> <direct|graph> <ctas> <us>", then "timeout_status <err>" and "after <err>".
#include <cstdio>
#include <cuda_runtime.h>

constexpr int kGroups = 16;

// Arrival counters, one per 128-byte line; root at index kGroups.
__device__ unsigned g_count[(kGroups + 1) * 32];
__device__ unsigned g_gen;
__device__ int g_err;

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Thread 0 of each CTA arrives; the last arriver of the barrier resets the counters it passed
// and publishes generation gen + 1; the others poll the generation at most cap times.
template <bool TREE>
__device__ __forceinline__ bool grid_barrier(unsigned& gen, unsigned cap) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned nb = gridDim.x;
    __threadfence();
    bool last;
    if (TREE) {
      const unsigned g = blockIdx.x % kGroups;
      const unsigned gsize = nb / kGroups + (g < nb % kGroups ? 1u : 0u);
      const unsigned ng = nb < (unsigned)kGroups ? nb : (unsigned)kGroups;
      last = false;
      if (atomicAdd(&g_count[g * 32], 1u) == gsize - 1) {
        atomicExch(&g_count[g * 32], 0u);
        __threadfence();  // the group's reset is ordered before its arrival at the root
        last = atomicAdd(&g_count[kGroups * 32], 1u) == ng - 1;
        if (last) atomicExch(&g_count[kGroups * 32], 0u);
      }
    } else {
      last = atomicAdd(&g_count[0], 1u) == nb - 1;
      if (last) atomicExch(&g_count[0], 0u);
    }
    if (last) {
      __threadfence();
      atomicExch(&g_gen, gen + 1);
    } else {
      unsigned it = 0;
      while (ld_acquire(&g_gen) == gen) {
        if (++it > cap) {
          atomicExch(&g_err, 1);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    gen += 1;
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

template <bool TREE>
__global__ void k_barriers(int iters, unsigned cap, float* sink) {
  unsigned gen = 0;
  if (threadIdx.x == 0) gen = ld_acquire(&g_gen);
  float acc = 0.f;
  for (int i = 0; i < iters; ++i) {
    acc += threadIdx.x * 1e-9f;
    if (!grid_barrier<TREE>(gen, cap)) break;
  }
  if (acc < -1.f) sink[blockIdx.x] = acc;
}

__global__ void k_empty(float* sink) {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (threadIdx.x == 1u << 30) sink[0] = 1.f;
}

#define CK(x)                                                                     \
  do {                                                                            \
    cudaError_t e_ = (x);                                                         \
    if (e_ != cudaSuccess) {                                                      \
      std::printf("error %s: %s\n", #x, cudaGetErrorString(e_));                  \
      return 1;                                                                   \
    }                                                                             \
  } while (0)

static int reset_barrier_state() {
  static unsigned zeros[(kGroups + 1) * 32] = {};
  const unsigned z = 0;
  const int zi = 0;
  CK(cudaMemcpyToSymbol(g_count, zeros, sizeof(zeros)));
  CK(cudaMemcpyToSymbol(g_gen, &z, sizeof(z)));
  CK(cudaMemcpyToSymbol(g_err, &zi, sizeof(zi)));
  return 0;
}

template <bool TREE>
static int run_barriers(cudaStream_t s, int grid, int threads, int iters, unsigned cap, float* sink,
                        float* ms, int* err) {
  cudaEvent_t a, b;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  void* args[3] = {&iters, &cap, &sink};
  CK(cudaEventRecord(a, s));
  CK(cudaLaunchCooperativeKernel((void*)k_barriers<TREE>, dim3(grid), dim3(threads), args, 0, s));
  CK(cudaEventRecord(b, s));
  CK(cudaStreamSynchronize(s));
  CK(cudaEventElapsedTime(ms, a, b));
  CK(cudaMemcpyFromSymbol(err, g_err, sizeof(int)));
  CK(cudaEventDestroy(a));
  CK(cudaEventDestroy(b));
  return 0;
}

int main() {
  CK(cudaSetDevice(0));
  cudaDeviceProp pr;
  CK(cudaGetDeviceProperties(&pr, 0));
  const int sms = pr.multiProcessorCount;
  float* sink;
  CK(cudaMalloc(&sink, 1 << 20));
  cudaStream_t s;
  CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  const int iters = 2000;
  const unsigned cap = 1u << 22;  // polls; far above any barrier of a healthy grid
  if (reset_barrier_state()) return 1;

  const int threads_list[2] = {64, 256};
  const int per_sm_list[3] = {1, 2, 4};
  for (int tree = 0; tree < 2; ++tree)
    for (int threads : threads_list)
      for (int per_sm : per_sm_list) {
        int maxb = 0;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &maxb, tree ? (const void*)k_barriers<true> : (const void*)k_barriers<false>, threads, 0));
        if (maxb < per_sm) continue;
        const int grid = sms * per_sm;
        float ms = 0.f;
        int err = 0;
        for (int rep = 0; rep < 2; ++rep) {  // the first launch warms up
          const int rc = tree ? run_barriers<true>(s, grid, threads, iters, cap, sink, &ms, &err)
                              : run_barriers<false>(s, grid, threads, iters, cap, sink, &ms, &err);
          if (rc) return 1;
        }
        std::printf("barrier %s %d %d %.3f %d\n", tree ? "tree" : "flat", grid, threads,
                    1e3 * ms / iters, err);
        if (err) return 1;
      }

  for (int pdl = 0; pdl < 2; ++pdl)
    for (int per_sm : per_sm_list) {
      const int grid = sms * per_sm;
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(grid);
      cfg.blockDim = dim3(64);
      cfg.stream = s;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
      at[0].val.programmaticStreamSerializationAllowed = 1;
      cfg.attrs = at;
      cfg.numAttrs = pdl ? 1 : 0;
      cudaEvent_t a, b;
      CK(cudaEventCreate(&a));
      CK(cudaEventCreate(&b));
      for (int graph = 0; graph < 2; ++graph) {
        cudaGraph_t gr = nullptr;
        cudaGraphExec_t ge = nullptr;
        if (graph) {
          CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
          for (int i = 0; i < iters; ++i) CK(cudaLaunchKernelEx(&cfg, k_empty, sink));
          CK(cudaStreamEndCapture(s, &gr));
          CK(cudaGraphInstantiate(&ge, gr, 0));
        }
        float ms = 0.f;
        for (int rep = 0; rep < 2; ++rep) {
          CK(cudaEventRecord(a, s));
          if (graph) {
            CK(cudaGraphLaunch(ge, s));
          } else {
            for (int i = 0; i < iters; ++i) CK(cudaLaunchKernelEx(&cfg, k_empty, sink));
          }
          CK(cudaEventRecord(b, s));
          CK(cudaStreamSynchronize(s));
          CK(cudaEventElapsedTime(&ms, a, b));
        }
        std::printf("kernel %d %s %d %.3f\n", pdl, graph ? "graph" : "direct", grid, 1e3 * ms / iters);
        if (graph) {
          CK(cudaGraphExecDestroy(ge));
          CK(cudaGraphDestroy(gr));
        }
      }
      CK(cudaEventDestroy(a));
      CK(cudaEventDestroy(b));
    }

  // The capped wait: cap = 0 makes every CTA that is not the last to arrive give up at once.
  {
    float ms = 0.f;
    int err = 0;
    if (run_barriers<false>(s, sms, 64, 4, 0u, sink, &ms, &err)) return 1;
    std::printf("timeout_status %d\n", err);
    if (reset_barrier_state()) return 1;
    if (run_barriers<false>(s, sms, 64, 4, cap, sink, &ms, &err)) return 1;
    std::printf("after %d\n", err);
  }
  CK(cudaFree(sink));
  return 0;
}
