// Hierarchy construction for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: code running inside a framework that
// owns the device heap (a caching allocator or a memory pool it must not
// bypass), or a plugin loaded into a process whose allocations are audited.
// They still hand in device memory they already own for the outputs.  The
// regular path (heomgb_qme_set_param) uploads its binomial-coefficient table
// into a fresh cudaMalloc'd buffer; this entry point keeps that table in a
// file-scope __device__ array instead and allocates nothing.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "heomgb.h"
#include "heomgb_impl.cuh"

namespace heomgb {
void set_error_message(const std::string& msg);
}

namespace {

// Largest binomial-table dimension K + max_depth + 2 the fixed scratch holds.
constexpr int kMaxBinomDim = HEOMGB_NOALLOC_MAX_BINOM_DIM;

// Shared scratch: one table per device, held by every GPU that loads the
// library until the process exits.  Each call rewrites the part it reads.
__device__ __align__(256) long long g_binom_scratch[kMaxBinomDim * kMaxBinomDim];

// C(a, b) for a, b < dim by Pascal's rule, saturated like the host table.
__global__ void k_binom_fill(long long* t, int dim) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const long long cap = 0x7fffffffffffffffLL / 4;
  for (int a = 0; a < dim; ++a) {
    for (int b = 0; b < dim; ++b) {
      long long v;
      if (b > a)
        v = 0;
      else if (b == 0 || b == a)
        v = 1;
      else {
        const long long x = t[static_cast<size_t>(a - 1) * dim + b - 1], y = t[static_cast<size_t>(a - 1) * dim + b];
        v = (x >= cap || y >= cap || x + y >= cap) ? cap : x + y;
      }
      t[static_cast<size_t>(a) * dim + b] = v;
    }
  }
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
long long* g_scratch_ptr[kMaxDevices] = {};

}  // namespace

extern "C" heomgb_status heomgb_hrchy_build_noalloc(int n_dim, int max_depth, int* n_dev, int* ptr_p1_dev,
                                                    int* ptr_m1_dev, int* n_hrchy, void* cuda_stream) {
  using heomgb::set_error_message;
  if (n_dim < 1 || max_depth < 0 || !n_dev || !ptr_p1_dev || !ptr_m1_dev || !n_hrchy) {
    set_error_message("heomgb_hrchy_build_noalloc: n_dim >= 1, max_depth >= 0 and non-null pointers required");
    return HEOMGB_ERR_INVALID_ARGUMENT;
  }
  // the sum is formed in 64 bits: n_dim and max_depth near INT_MAX must not wrap
  // to a small value that passes the capacity check
  const long long dim_ll = static_cast<long long>(n_dim) + max_depth + 2;
  if (dim_ll > kMaxBinomDim) {
    set_error_message("heomgb_hrchy_build_noalloc: n_dim + max_depth + 2 = " + std::to_string(dim_ll) +
                      " exceeds the fixed scratch maximum of " + std::to_string(kMaxBinomDim));
    return HEOMGB_ERR_CAPACITY;
  }
  const int dim = static_cast<int>(dim_ll);
  // ADO count C(n_dim + max_depth, max_depth), checked against int range on the host.
  long double c = 1;
  for (int i = 1; i <= max_depth; ++i) c = c * (n_dim + i) / i;
  if (c > 2147483646.0L) {
    set_error_message("heomgb_hrchy_build_noalloc: more than 2^31-2 ADOs");
    return HEOMGB_ERR_INVALID_ARGUMENT;
  }
  const int count = static_cast<int>(c + 0.5L);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_error_message(std::string("heomgb_hrchy_build_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return HEOMGB_ERR_CUDA;
  }
  long long* table = nullptr;
  {
    // First call on a device: look up the device address of the scratch array
    // (its host-side name is only a stand-in, not a device address).
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_binom_scratch);
      if (e != cudaSuccess || !p) {
        set_error_message(std::string("heomgb_hrchy_build_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return HEOMGB_ERR_CUDA;
      }
      g_scratch_ptr[dev] = static_cast<long long*>(p);
    }
    table = g_scratch_ptr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  k_binom_fill<<<1, 1, 0, s>>>(table, dim);
  ++heomgb::g_launches;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = heomgb::launch_hrchy_build(n_dim, max_depth, count, table, dim, n_dev, ptr_p1_dev,
                                                       ptr_m1_dev, s);
  if (e != cudaSuccess) {
    set_error_message(std::string("heomgb_hrchy_build_noalloc: launch: ") + cudaGetErrorString(e));
    return HEOMGB_ERR_CUDA;
  }
  *n_hrchy = count;
  return HEOMGB_OK;
}
