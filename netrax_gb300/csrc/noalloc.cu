// Allocation-free mixing of displayed-tree site log-likelihoods.
//
// Who needs this: callers that must not allocate device memory themselves or
// have it allocated on their behalf - programs whose device memory is fully
// handed to another allocator or a fixed budget, and latency-critical loops
// where cudaMalloc/cudaFree would synchronise the device. They still pass every input and output buffer; the only working
// memory this entry point needs - the per-(tree, partition) sums between its
// two kernels - lives in the fixed array below, which is part of the loaded
// library image on every GPU that loads it and stays there until exit.
//
// This is a variant of the context path's tree_reduce_kernel + mix_kernel
// (kernels.cu) without a context: the caller supplies per-site (or per-block)
// log-likelihood contributions of each displayed tree instead of the
// library's own forward sweep.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/netlk.h"

namespace netlk {
void set_global_error(const std::string &msg);
}

// Working memory shared by every call on a device: NETLK_NOALLOC_MAX_TREE_PARTITIONS
// doubles (512 KiB). Calls whose work overlaps on the GPU (different streams,
// or host threads) race on it; each call's first kernel writes every entry its
// second kernel reads, so nothing has to start at zero.
static __device__ __align__(256) double g_tree_partition_sum[NETLK_NOALLOC_MAX_TREE_PARTITIONS];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double *g_scratch_ptr[kMaxDevices] = {nullptr};
unsigned long long g_scratch_ctx[kMaxDevices] = {0};

typedef CUresult(CUDAAPI *CtxGetCurrentFn)(CUcontext *);
typedef CUresult(CUDAAPI *CtxGetIdFn)(CUcontext, unsigned long long *);

// Process-unique id of the current CUDA context (0 if it cannot be read).
// The driver functions are fetched through the runtime, so the library does
// not link libcuda itself.
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    looked_up = true;
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, &id) == CUDA_SUCCESS)
    return id;
  return 0;
}

// Device address of the array on the current device, looked up at the first
// call on a device, and again whenever the device's context has changed
// since (after cudaDeviceReset the library image is loaded anew and the old
// address is gone). In host code the symbol name is only a stand-in and must
// never be handed to a kernel.
cudaError_t scratch_address(int device, double **out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  const unsigned long long ctx = current_context_id();
  if (!g_scratch_ptr[device] || ctx == 0 || ctx != g_scratch_ctx[device]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_tree_partition_sum);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[device] = static_cast<double *>(p);
    g_scratch_ctx[device] = ctx;
  }
  *out = g_scratch_ptr[device];
  return cudaSuccess;
}

// sum[tree][part] = sum of site_logl[tree][s] over the partition's sites
// (compensated FP64 per thread, fixed-order block reduction).
__global__ void noalloc_reduce_kernel(const double *__restrict__ site_logl, int64_t n_sites,
                                      const int64_t *__restrict__ part_begin, int n_parts,
                                      double *__restrict__ sum) {
  const int tree = blockIdx.x, part = blockIdx.y;
  // a range outside [0, n_sites] is clipped to it: a bad caller range gives
  // a wrong sum, never an out-of-bounds read
  const int64_t b = min(max(part_begin[part], (int64_t)0), n_sites);
  const int64_t e = min(max(part_begin[part + 1], b), n_sites);
  const double *src = site_logl + (size_t)tree * n_sites;
  double s = 0.0, c = 0.0;
  for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
    const double y = src[i] - c;
    const double t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) sum[(size_t)tree * n_parts + part] = red[0];
}

// Per partition: AVERAGE = log sum_T exp(logprob_T + sum_T,p) (max-shifted),
// BEST = max_T; trees with logprob below min_logprob are skipped (the
// reference's min_interesting_tree_logprob). out[0] = sum over partitions.
__global__ void noalloc_mix_kernel(const double *__restrict__ sum, int n_trees, int n_parts,
                                   const double *__restrict__ logprob, int variant, double min_logprob,
                                   double *__restrict__ out) {
  __shared__ double red[256];
  const int tid = threadIdx.x;
  double total = 0.0;
  for (int part = 0; part < n_parts; ++part) {
    double mx = -INFINITY;
    for (int t = tid; t < n_trees; t += blockDim.x)
      if (logprob[t] >= min_logprob) mx = fmax(mx, logprob[t] + sum[(size_t)t * n_parts + part]);
    red[tid] = mx;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if (tid < o) red[tid] = fmax(red[tid], red[tid + o]);
      __syncthreads();
    }
    mx = red[0];
    __syncthreads();
    double lp = mx;
    if (variant == NETLK_AVERAGE && mx > -INFINITY) {
      double acc = 0.0;
      for (int t = tid; t < n_trees; t += blockDim.x)
        if (logprob[t] >= min_logprob) acc += exp(logprob[t] + sum[(size_t)t * n_parts + part] - mx);
      red[tid] = acc;
      __syncthreads();
      for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (tid < o) red[tid] += red[tid + o];
        __syncthreads();
      }
      lp = mx + log(red[0]);
      __syncthreads();
    }
    if (tid == 0) out[1 + part] = lp;
    total += lp;
  }
  if (tid == 0) out[0] = total;
}

int fail(int status, const std::string &msg) {
  netlk::set_global_error(msg);
  return status;
}

}  // namespace

extern "C" int netlk_mix_site_loglikelihoods_noalloc(const double *d_site_logl, int32_t n_trees, int64_t n_sites,
                                                     const int64_t *d_part_site_begin, int32_t n_parts,
                                                     const double *d_tree_logprob, int32_t variant,
                                                     double min_interesting_tree_logprob, double *d_out,
                                                     void *stream) {
  if (!d_site_logl || !d_part_site_begin || !d_tree_logprob || !d_out)
    return fail(NETLK_ERR_INVALID_ARGUMENT, "netlk_mix_site_loglikelihoods_noalloc: null buffer");
  if (n_trees < 1 || n_parts < 1 || n_sites < 1 || n_parts > 65535)
    return fail(NETLK_ERR_INVALID_ARGUMENT, "netlk_mix_site_loglikelihoods_noalloc: bad sizes");
  if ((int64_t)n_trees * n_parts > NETLK_NOALLOC_MAX_TREE_PARTITIONS)
    return fail(NETLK_ERR_INVALID_ARGUMENT,
                "netlk_mix_site_loglikelihoods_noalloc: n_trees * n_partitions = " +
                    std::to_string((int64_t)n_trees * n_parts) + " exceeds the fixed working array of " +
                    std::to_string(NETLK_NOALLOC_MAX_TREE_PARTITIONS) + " entries");
  if (variant != NETLK_AVERAGE && variant != NETLK_BEST)
    return fail(NETLK_ERR_INVALID_ARGUMENT, "netlk_mix_site_loglikelihoods_noalloc: variant");
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return fail(NETLK_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (device < 0 || device >= kMaxDevices) return fail(NETLK_ERR_NO_DEVICE, "device ordinal out of range");
  double *scratch = nullptr;
  e = scratch_address(device, &scratch);
  if (e != cudaSuccess)
    return fail(NETLK_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  noalloc_reduce_kernel<<<dim3(n_trees, n_parts), 256, 0, s>>>(d_site_logl, n_sites, d_part_site_begin, n_parts,
                                                                scratch);
  noalloc_mix_kernel<<<1, 256, 0, s>>>(scratch, n_trees, n_parts, d_tree_logprob, variant,
                                       min_interesting_tree_logprob, d_out);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(NETLK_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return NETLK_OK;
}
