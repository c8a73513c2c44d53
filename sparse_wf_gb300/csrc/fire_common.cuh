// fire_common.cuh -- shared constants, device math and helpers for the FiRE hot-path kernels.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "fire.h"

namespace fire {

// Architecture of config/default.yaml (model section): feature_dim 256, 4 determinants,
// pair_mlp_widths (16, 8), pair_n_envelopes 32 (e-n), filter_dims[0] = 16 e-e envelopes,
// 8 isotropic orbital envelopes, Jastrow width 256 / depth 2, 16 heads x 16 dims.
constexpr int F = 256;
constexpr int NDET = 4;
constexpr int F0 = 16;
constexpr int F1 = 8;
constexpr int NENV_EN = 32;
constexpr int NENV_EE = 16;
constexpr int NENV_ORB = 8;
constexpr int HEADS = 16;
constexpr int HDIM = 16;
constexpr int MAX_EL = 1024;  // electrons per walker supported by the neighbour kernels

// Slots of the prepared-parameter buffer: first the blob slots converted to the compute type,
// then derived weights.
enum PrepSlot {
  PR_BLOB_END = FIRE_P_COUNT,
  PR_UPD1_W_S0 = FIRE_P_COUNT,  // scales[0] * upd1_W
  PR_ORB_UP_W_S1,               // scales[1] * orb_up_W
  PR_ORB_DN_W_S1,
  PR_JMLP1_W_S1,                // scales[1] * jmlp1_W
  PR_QK_W_S1,                   // [F, HEADS]: scales[1] * sum_d Q_W[:, h*16+d] * keys[h, d]
  PR_QK_B,                      // [HEADS]
  PR_V_W_S1,                    // scales[1] * V_W
  PR_EN_INVSCALE,               // [N, 32]   1 / softplus(en_scales)
  PR_EESAME_INVSCALE,           // [16]
  PR_EEDIFF_INVSCALE,           // [16]
  PR_ENV_UP_SP,                 // [N, D, 8] softplus(sigma)
  PR_ENV_DN_SP,
  PR_ENV_UP_PI,                 // [D, N*8, n] pi re-laid out per determinant
  PR_ENV_DN_PI,
  PR_SCALARS,                   // [8]: cutoff_eff, ...
  PR_COUNT
};

template <typename T>
struct Weights {
  const T* w[PR_COUNT];
};

// ------------------------------------------------------------------------------------- math
template <typename T> __device__ __forceinline__ T dexp(T x);
template <> __device__ __forceinline__ float dexp<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double dexp<double>(double x) { return exp(x); }
template <typename T> __device__ __forceinline__ T dlog(T x);
template <> __device__ __forceinline__ float dlog<float>(float x) { return logf(x); }
template <> __device__ __forceinline__ double dlog<double>(double x) { return log(x); }
template <typename T> __device__ __forceinline__ T dlog1p(T x);
template <> __device__ __forceinline__ float dlog1p<float>(float x) { return log1pf(x); }
template <> __device__ __forceinline__ double dlog1p<double>(double x) { return log1p(x); }
template <typename T> __device__ __forceinline__ T dsqrt(T x);
template <> __device__ __forceinline__ float dsqrt<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double dsqrt<double>(double x) { return sqrt(x); }

template <typename T>
__device__ __forceinline__ T sigm(T x) {
  return T(1) / (T(1) + dexp<T>(-x));
}
// silu(x) = x s(x); silu' = s (1 + x (1 - s)); silu'' = s (1 - s) (2 + x (1 - 2 s))
template <typename T>
__device__ __forceinline__ void silu3(T x, T& y, T& d1, T& d2) {
  T s = sigm(x);
  y = x * s;
  d1 = s * (T(1) + x * (T(1) - s));
  d2 = s * (T(1) - s) * (T(2) + x * (T(1) - T(2) * s));
}
template <typename T>
__device__ __forceinline__ T silu(T x) {
  return x * sigm(x);
}
template <typename T>
__device__ __forceinline__ T softplus(T x) {
  return x > T(20) ? x : dlog1p<T>(dexp<T>(x));
}
// cutoff_function (model/utils.py:103-112) with p = 4 and its first two derivatives in u
template <typename T>
__device__ __forceinline__ void cutoff3(T u, T& c, T& c1, T& c2) {
  if (u < T(1)) {
    T u2 = u * u, u3 = u2 * u, u4 = u2 * u2;
    c = T(1) + T(-15) * u4 + T(24) * u4 * u + T(-10) * u4 * u2;
    c1 = T(-60) * u3 + T(120) * u4 + T(-60) * u4 * u;
    c2 = T(-180) * u2 + T(480) * u3 + T(-300) * u4;
  } else {
    c = T(0); c1 = T(0); c2 = T(0);
  }
}
template <typename T>
__device__ __forceinline__ T cutoff_val(T u) {
  if (u < T(1)) {
    T u2 = u * u, u4 = u2 * u2;
    return T(1) + T(-15) * u4 + T(24) * u4 * u + T(-10) * u4 * u2;
  }
  return T(0);
}

// ------------------------------------------------------------------------------------- reductions
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// Sum of NV values per thread over the whole block (blockDim.x multiple of 32, <= 1024).
// `red` must hold 32 * NV elements of shared memory.  Every thread gets the totals.
template <typename T, int NV>
__device__ __forceinline__ void block_sum(T (&v)[NV], T* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) red[wid * NV + k] = v[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    T s = T(0);
    for (int w = 0; w < nw; ++w) s += red[w * NV + k];
    v[k] = s;
  }
  __syncthreads();
}

__device__ __forceinline__ void set_flag(int32_t* status, int flag) {
  if (status) atomicOr(reinterpret_cast<int*>(status), flag);
}
__device__ __forceinline__ void max_word(int32_t* status, int word, int v) {
  if (status) atomicMax(reinterpret_cast<int*>(status) + word, v);
}

// Squared distance with the rounding the neighbour lists rely on: ((dx^2 + dy^2) + dz^2), each
// product and sum rounded (no fused multiply-add), then a correctly rounded square root.
__device__ __forceinline__ float exact_dist(float ax, float ay, float az, float bx, float by, float bz) {
  float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
  float s = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
  s = __fadd_rn(s, __fmul_rn(dz, dz));
  return __fsqrt_rn(s);
}
__device__ __forceinline__ double exact_dist(double ax, double ay, double az, double bx, double by,
                                             double bz) {
  double dx = __dsub_rn(ax, bx), dy = __dsub_rn(ay, by), dz = __dsub_rn(az, bz);
  double s = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
  s = __dadd_rn(s, __dmul_rn(dz, dz));
  return __dsqrt_rn(s);
}

template <typename T>
__device__ __forceinline__ void atomic_add(T* p, T v) {
  atomicAdd(p, v);
}

}  // namespace fire

#define FIRE_CUDA_OK(x)                     \
  do {                                      \
    if ((x) != cudaSuccess) return FIRE_ERR_CUDA; \
  } while (0)
