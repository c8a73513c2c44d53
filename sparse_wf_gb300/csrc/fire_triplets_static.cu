// fire_triplets_static.cu -- the triplet index builder without a caller workspace.
//
// fire_triplets needs a device workspace for the intermediate neighbour structure (degrees, row
// pointers, neighbour and reverse-pair lists).  Some callers cannot hand one over:
//   * a custom-call handler running inside another runtime's executable (an XLA FFI handler, a
//     TensorRT plugin) whose device memory belongs to that runtime's allocator, which may already have
//     reserved most of HBM, and where a cudaMalloc/cudaFree would synchronise the device in the middle
//     of asynchronous execution;
//   * a plain C host program or a serving loop that keeps no memory pool of its own and must not pay
//     for an allocation (and its implicit synchronisation) on every request.
// fire_triplets_static takes its scratch from a file-scope device array instead, so it allocates
// nothing.  The array has a fixed maximum size; larger requests are rejected.
//
// Set-up: the first call on each device (with that device current) looks the array's device address
// up with cudaGetSymbolAddress and caches it with the unique id of the current CUDA context; a call in a
// different context (after cudaDeviceReset, or once the primary context has been created again) looks it up
// afresh.  A call that does the look-up should come before any stream capture.
// Nothing in the scratch needs to start at zero: k_neighbors writes deg, rowptr (n + 1 entries), and
// -- when the walker's pair list fits -- nbr and rev for every pair, before k_triplets reads them, and
// k_triplets skips a walker whose pair list overflowed.  There is one scratch array per device, so two
// calls that may run at the same time on one device (different streams, or different host threads)
// race on it; calls ordered on one stream do not.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "fire.h"
#include "fire_common.cuh"
#include "fire_kernels.cuh"

using namespace fire;

namespace {

// The scratch: int32 words, laid out per call as deg [B, n] | rowptr [B, n + 1] | nbr [B, cap_pairs] |
// rev [B, cap_pairs].
static __device__ __align__(256) int g_triplet_scratch[FIRE_TRIPLETS_STATIC_MAX_WORDS];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
int* g_scratch_ptr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};  // unique id of the context the cached address belongs to

// Unique id of the current CUDA context (cuCtxGetId, never reused within a process), 0 if there is none or the
// driver cannot tell; the driver entry points come through the runtime, so the library needs no -lcuda.
unsigned long long current_context_id() {
  typedef CUresult (*GetCurrent)(CUcontext*);
  typedef CUresult (*GetId)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
    cudaGetLastError();
    looked_up = true;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, &id) == CUDA_SUCCESS)
    return id;
  return 0;
}

// Device address of the current device's scratch array (looked up once per device and context).
fire_status current_scratch(int** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return FIRE_ERR_CUDA;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  const unsigned long long ctx = current_context_id();
  if (!g_scratch_ptr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_triplet_scratch);
    if (e != cudaSuccess || p == nullptr) {
      if (std::getenv("FIRE_DEBUG"))
        std::fprintf(stderr, "[fire] fire_triplets_static: cudaGetSymbolAddress failed on device %d: %s\n", dev,
                     cudaGetErrorString(e));
      cudaGetLastError();
      return FIRE_ERR_CUDA;
    }
    g_scratch_ptr[dev] = static_cast<int*>(p);
    g_scratch_ctx[dev] = current_context_id();  // the look-up made the context current if there was none
  }
  *out = g_scratch_ptr[dev];
  return FIRE_OK;
}

}  // namespace

extern "C" fire_status fire_triplets_static(void* stream, const fire_problem* prob, const void* r,
                                            int32_t cap_triplets, int32_t* trip_in, int32_t* trip_k,
                                            int32_t* trip_kn, int32_t* trip_i, int32_t* status) {
  // the problem checks of the other entry points
  if (!prob || prob->n_el < 2 || prob->n_el > MAX_EL || prob->n_up < 0 || prob->n_up > prob->n_el ||
      prob->n_nuc < 1 || prob->n_walkers < 1 || !(prob->cutoff > 0) || !(prob->cutoff_1el > 0) ||
      prob->cap_pairs < 1 || prob->cap_nuc < 1 || prob->precision < 0 || prob->precision > 2)
    return FIRE_ERR_INVALID;
  if (!r || !trip_in || !trip_k || !trip_kn || !trip_i || cap_triplets < 1) return FIRE_ERR_INVALID;
  const int n = prob->n_el, B = prob->n_walkers;
  const unsigned long long words =
      (unsigned long long)B * ((unsigned long long)n + (n + 1) + 2ULL * (unsigned long long)prob->cap_pairs);
  if (words > FIRE_TRIPLETS_STATIC_MAX_WORDS) return FIRE_ERR_UNSUPPORTED;  // checked before any CUDA call

  int* w = nullptr;
  const fire_status st = current_scratch(&w);
  if (st != FIRE_OK) return st;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  Nbr nb;
  nb.W = B; nb.n = n; nb.n_up = prob->n_up; nb.N = 0; nb.cap_p = prob->cap_pairs; nb.cap_nuc = prob->cap_nuc;
  nb.deg = w; w += (size_t)B * n;
  nb.rowptr = w; w += (size_t)B * (n + 1);
  nb.nbr = w; w += (size_t)B * prob->cap_pairs;
  nb.rev = w;
  nb.en_cnt = nullptr;  // the e-n lists are not part of the triplet structure
  nb.en_idx = nullptr;
  nb.counts = nullptr;
  fire_neighbor_out ext;
  std::memset(&ext, 0, sizeof(ext));
  if (prob->precision == FIRE_PREC_FP64) {
    const size_t smem = 3 * n * sizeof(double) + (5 * n + 2) * sizeof(int);
    cudaFuncSetAttribute(k_neighbors<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_neighbors<double><<<B, 512, smem, s>>>(reinterpret_cast<const double*>(r), nullptr, (double)prob->cutoff,
                                            (double)prob->cutoff_1el, nb, ext, status);
  } else {
    const size_t smem = 3 * n * sizeof(float) + (5 * n + 2) * sizeof(int);
    cudaFuncSetAttribute(k_neighbors<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_neighbors<float><<<B, 512, smem, s>>>(reinterpret_cast<const float*>(r), nullptr, prob->cutoff,
                                           prob->cutoff_1el, nb, ext, status);
  }
  k_triplets<<<B, 256, 0, s>>>(nb, cap_triplets, trip_in, trip_k, trip_kn, trip_i, status);
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return FIRE_OK;
  if (std::getenv("FIRE_DEBUG")) std::fprintf(stderr, "[fire] fire_triplets_static: %s\n", cudaGetErrorString(e));
  return FIRE_ERR_CUDA;
}
