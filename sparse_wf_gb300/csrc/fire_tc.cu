// fire_tc.cu -- instantiations and host launchers of the tcgen05 contraction (fire_tc.cuh), and the
// weight splitter that prepares its BF16 hi/lo, K-contiguous operands.
#include <cstdint>

#include "fire_tc.cuh"

namespace fire {

// hi/lo split of W[K][N] (row-major float) into transposed BF16 planes [N][K]
__global__ void k_split_transpose(const float* __restrict__ W, int K, int N, __nv_bfloat16* __restrict__ hi,
                                  __nv_bfloat16* __restrict__ lo) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;  // over (n, k)
  if (idx >= (long)N * K) return;
  const int n = (int)(idx / K), k = (int)(idx % K);
  const float w = W[(long)k * N + n];
  const __nv_bfloat16 h = __float2bfloat16_rn(w);
  hi[idx] = h;
  lo[idx] = __float2bfloat16_rn(w - __bfloat162float(h));
}

// hi/lo split of W[K][N] into tiles of 128 columns x 64 K: tile (j, kb) at block j * ceil(K / 64) + kb holds the
// hi plane then the lo plane, each [8 k-groups][128 columns][8 k] (zero padding beyond N and K).  With cs: every
// column scaled and split on the grid of its largest magnitude in FP16 (hi parts of at most 2^(hb + 1), hb =
// grid_hb(K)), its scale in cs[n]; else an elementwise BF16 split.
__global__ void k_split_tiles(const float* __restrict__ W, int K, int N, __nv_bfloat16* __restrict__ Bt,
                              float* __restrict__ cs, int hb) {
  const int nkt = (K + 63) / 64, nnt = (N + 127) / 128;
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;  // over (block, g, r, e)
  if (idx >= (long)nnt * nkt * 8192) return;
  const long blk = idx >> 13;
  const int w = (int)(idx & 8191), g = w >> 10, r = (w >> 3) & 127, e = w & 7;
  const int j = (int)(blk / nkt), kb = (int)(blk % nkt);
  const int n = j * 128 + r, k = kb * 64 + g * 8 + e;
  const float v = (n < N && k < K) ? W[(long)k * N + n] : 0.f;
  __nv_bfloat16* base = Bt + blk * 16384;
  if (cs) {
    float inv = 0.f, sc = 0.f;
    if (n < N) {
      float mx = 0.f;
      for (int q = 0; q < K; ++q) mx = fmaxf(mx, fabsf(W[(long)q * N + n]));
      grid_scales(grid_code(mx), inv, sc, hb);
      if (kb == 0 && g == 0 && e == 0) cs[n] = sc;
    }
    const float x = v * inv, h = rintf(x);
    __half* hb = reinterpret_cast<__half*>(base);
    hb[w] = __float2half_rn(h);
    hb[8192 + w] = __float2half_rn(x - h);
    return;
  }
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  base[w] = h;
  base[8192 + w] = __float2bfloat16_rn(v - __bfloat162float(h));
}

__global__ void k_tile_mask(GemmP<float> p, int* mask) {
  const int m_tile = blockIdx.x;
  int rows = p.M;
  if (p.M_dev) rows = min(rows, p.M_scale * (*p.M_dev));
  const int row = m_tile * TC_BM + threadIdx.x;
  int up = 0, dn = 0;
  if (row < rows) {
    const int node = gemm_node(p, row);
    if ((node % p.n_el) < p.n_up) up = 1; else dn = 1;
  }
  up = __syncthreads_or(up);
  dn = __syncthreads_or(dn);
  if (threadIdx.x == 0) mask[m_tile] = up | (dn << 1);
}

cudaError_t split_tiles(const float* W, int K, int N, __nv_bfloat16* Bt, cudaStream_t s, float* cs) {
  const long tot = (long)((N + 127) / 128) * ((K + 63) / 64) * 8192;
  k_split_tiles<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(W, K, N, Bt, cs, grid_hb(K));
  return cudaPeekAtLastError();
}

cudaError_t split_transpose(const float* W, int K, int N, __nv_bfloat16* hi, __nv_bfloat16* lo, cudaStream_t s) {
  const long tot = (long)N * K;
  k_split_transpose<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(W, K, N, hi, lo);
  return cudaPeekAtLastError();
}

namespace {
// cuTensorMapEncodeTiled, looked up through the runtime (no link-time dependency on the driver library)
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(ptr);
    else
      cudaGetLastError();
  }
  return fn;
}
}  // namespace

bool tc_c_map(const GemmP<float>& p, CUtensorMap* map) {
  const EncodeTiledFn fn = encode_tiled();
  if (!fn || !p.C || p.M < 1 || p.N < 16 || (p.ldc * sizeof(float)) % 16 != 0 ||
      (reinterpret_cast<uintptr_t>(p.C) & 15) != 0)
    return false;
  const cuuint64_t dims[2] = {(cuuint64_t)p.N, (cuuint64_t)p.M};
  const cuuint64_t strides[1] = {(cuuint64_t)p.ldc * sizeof(float)};
  const cuuint32_t box[2] = {16, 32};
  const cuuint32_t elem[2] = {1, 1};
  // 64-byte swizzle: 16-byte chunk c of box row r sits at chunk c ^ ((r >> 1) & 3) in shared memory, so that a
  // warp writing one chunk of each of its 32 rows hits every bank once per 8 rows (tc_epilogue_tile)
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, p.C, dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
         CUDA_SUCCESS;
}

cudaError_t gemm_tc(int mode, int bn, const GemmP<float>& p, const TcWeights& wt, int* mask_buf, int32_t* status,
                    cudaStream_t s) {
  if (p.K % 8 != 0 || p.lda % 4 != 0 || p.ldc % 4 != 0 || (p.ld_aux % 4 != 0 && mode != EPI_PLAIN))
    return cudaErrorInvalidValue;
  // float4 operand loads and stores: A, C and every vector-accessed buffer 16-byte aligned
  auto mis = [](const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15) != 0; };
  if (mis(p.A) || mis(p.aux0) || mis(p.aux1) || mis(p.aux2) || mis(p.aux3) || mis(p.C))
    return cudaErrorInvalidValue;
  static int num_sms = 0;
  if (num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (num_sms <= 0) num_sms = 1;
  }
  (void)bn;
#define FIRE_TC_CASE(M) \
  case M:               \
    return launch_gemm_tc<M>(p, wt, mask_buf, status, s, num_sms);
  switch (mode) {
    FIRE_TC_CASE(EPI_PLAIN)
    FIRE_TC_CASE(EPI_SILU_J)
    FIRE_TC_CASE(EPI_SILU_L)
    FIRE_TC_CASE(EPI_ORB_J)
    FIRE_TC_CASE(EPI_ORB_L)
    default:
      return cudaErrorInvalidValue;
  }
#undef FIRE_TC_CASE
}

}  // namespace fire
