// fire_tc.cuh -- tcgen05 (5th-generation tensor core) contraction for the mixed-precision path.
//
// C[M, N] = A[M, K] * W[K, N] for the Jacobian and Laplacian planes of the sparse forward Laplacian,
// with the same epilogues as the CUDA-core GEMM (fire_gemm.cuh).  A is an FP32 plane; while it is
// staged into shared memory every element is split into two 16-bit numbers, a = a_hi + a_lo.  The
// weights are pre-split the same way and stored transposed (K contiguous).
//   - k_gemm_tca (K <= 256) splits on a power-of-two grid per row of A and per column of W into FP16 hi + lo
//     and issues four FP16 MMAs per 16-deep K step: the exact hi x hi sums into one TMEM accumulator, the three
//     cross terms into a second (the splitting comment before k_gemm_tca has the details);
//   - k_gemm_tcs (K > 256) splits elementwise into BF16, a_hi = bf16(a), a_lo = bf16(a - a_hi), and issues
//     three BF16 MMAs into one FP32 accumulator:  a_hi b_hi + a_hi b_lo + a_lo b_hi  (relative error ~2^-17
//     per product instead of BF16's 2^-9).
//
// Two kernels share the epilogues: k_gemm_tca (K <= 256; the A tile stays in shared memory, the pre-tiled
// weights stream in by bulk copies) and k_gemm_tcs (K > 256; A and weight k-tiles stream together).  Tiles
// are 128 rows (TMEM lanes) x 128 columns, K staged 64 deep, in the canonical K-major layout without
// swizzle (8-row x 16-byte core matrices; A: K-adjacent core matrices 128 bytes apart, 8-row groups 1024
// bytes apart; pre-tiled weights: 2048 and 128 bytes).  One thread issues the MMAs and commits them to
// mbarriers; every wait is bounded and reports FIRE_FLAG_TIMEOUT.
#pragma once
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstring>

#include "fire_gemm.cuh"
#include "fire_internal.cuh"

namespace fire {

constexpr int TC_BM = 128, TC_BK = 64;
constexpr uint32_t TC_LBO = 128, TC_SBO = 1024;
constexpr long TC_SPIN_LIMIT = 1L << 22;
constexpr int TCP_THREADS = 416, TCP_BN = 128, TCP_KMAX = 256, TCP_STAGES = 3;


__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((TC_LBO >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((TC_SBO >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for sm_100-family tensor cores
  // base offset 0, relative LBO mode, swizzle none (bits 61-63 = 0)
  return d;
}

// K-major no-swizzle descriptor with explicit byte strides between core matrices along K (lbo) and along
// M / N (sbo)
__device__ __forceinline__ uint64_t tc_desc_s(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// FP16 A and B (the scaled-grid split of the A-resident kernel)
template <int BN>
__device__ __forceinline__ uint32_t tc_idesc_f16() {
  uint32_t d = 0;
  d |= 1u << 4;                       // D format F32; A and B format F16 (0)
  d |= (uint32_t)(BN >> 3) << 17;     // N / 8
  d |= (uint32_t)(TC_BM >> 4) << 24;  // M / 16
  return d;
}

template <int BN>
__device__ __forceinline__ uint32_t tc_idesc() {
  uint32_t d = 0;
  d |= 1u << 4;                   // D format F32
  d |= 1u << 7;                   // A format BF16
  d |= 1u << 10;                  // B format BF16
  d |= (uint32_t)(BN >> 3) << 17;  // N / 8
  d |= (uint32_t)(TC_BM >> 4) << 24;  // M / 16
  return d;                       // A and B K-major, no negation, dense
}

__device__ __forceinline__ void mbar_init(uint32_t addr, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count));
}
__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// TMA store of a box of C (tensor map in kernel-parameter space) from shared memory; bulk async-groups
// belong to the issuing thread
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, uint32_t src, int x, int y) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(src), "r"(x), "r"(y)
               : "memory");
}
__device__ __forceinline__ void tma_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void tma_wait_read1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void tma_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// one contiguous global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16) completing on an
// mbarrier that expects its bytes
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

// byte offset of element (row, k) in a canonical no-swizzle K-major tile (BF16)
__device__ __forceinline__ uint32_t tc_off(int row, int k) {
  return (uint32_t)((row & 7) * 16 + (row >> 3) * TC_SBO + (k & 7) * 2 + (k >> 3) * TC_LBO);
}

// 16-byte global -> shared asynchronous copy (zero fill when !ok), commit and wait (n copies groups may stay
// in flight, n <= 3)
__device__ __forceinline__ void cp_async16_tc(void* dst, const void* src, bool ok) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(ok ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit_tc() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_tc(int n) {
  if (n <= 0) asm volatile("cp.async.wait_group 0;" ::: "memory");
  else if (n == 1) asm volatile("cp.async.wait_group 1;" ::: "memory");
  else if (n == 2) asm volatile("cp.async.wait_group 2;" ::: "memory");
  else asm volatile("cp.async.wait_group 3;" ::: "memory");
}
// Scaled-grid split (the A-resident kernel, K <= 256).  A row of A (or a column of W) whose largest magnitude is in
// [2^e, 2^(e+1)) is scaled by 2^(7 - e) (exactly), so its values lie in (-256, 256); each scaled value x is split
// into hi = rint(x), an integer of magnitude <= 256, and lo = x - hi (exact in FP32, |lo| <= 1/2), both stored in
// FP16 (hi exactly; lo to 2^-12 of itself, i.e. to 2^-20 of the row's largest value).  Products of two hi parts are
// integers below 2^16, so up to 256 of them sum exactly in an FP32 accumulator, whatever order and rounding the
// tensor core's accumulation uses; the epilogue multiplies by the row's and the column's scale 2^(e - 7).
// Exponent code of a row: ilogb of its largest magnitude clamped to >= -120, GRID_ZERO for an all-zero row,
// GRID_NAN when the row holds an infinity or a NaN.
constexpr int GRID_ZERO = -32768, GRID_NAN = 32767;
__device__ __forceinline__ int grid_code(float mx) {
  if (mx == 0.f) return GRID_ZERO;
  if (!(mx <= 3.4e38f)) return GRID_NAN;
  return max(ilogbf(mx), -120);
}
// (inverse scale applied to the values, scale the epilogue applies) of an exponent code, for hi parts of at most
// 2^(hb + 1) in magnitude (hb = 7 for K <= 256; grid_hb gives hb for longer sums)
__device__ __forceinline__ void grid_scales(int code, float& inv, float& sc, int hb = 7) {
  if (code == GRID_ZERO) {
    inv = 0.f;
    sc = 0.f;
  } else if (code == GRID_NAN) {
    inv = 0.f;
    sc = __int_as_float(0x7fc00000);
  } else {
    inv = ldexpf(1.f, hb - code);
    sc = ldexpf(1.f, code - hb);
  }
}
// the largest hb for which K products of two hi parts (each <= 2^(hb + 1)) sum exactly in FP32:
// K 2^(2 hb + 2) <= 2^24
__host__ __device__ inline int grid_hb(int K) {
  int l = 0;
  while ((1 << l) < K) ++l;
  return (22 - l) / 2;
}
__device__ __forceinline__ void split_grid_f16x2(float a, float b, float inv, uint32_t& hi, uint32_t& lo) {
  const float xa = a * inv, xb = b * inv;
  const float ha = rintf(xa), hb = rintf(xb);
  const __half2 h = __floats2half2_rn(ha, hb);
  const __half2 l = __floats2half2_rn(xa - ha, xb - hb);
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}
// a = hi + lo for two values: BF16 pairs (first value in the low half)
__device__ __forceinline__ void split_bf16x2(float a, float b, uint32_t& hi, uint32_t& lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}

// ----------------------------------------------------------------------------- vectorised epilogues
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }

// Epilogue values of columns col..col+3 of one row (col % 4 == 0, col + 3 < N): everything but the store
// of C (the orbital Jacobian epilogue stores its side output itself).
template <int MODE>
__device__ __forceinline__ float4 tc_val4(const GemmP<float>& p, int row, int node, int col, const float* a,
                                          int spin) {
  if (MODE == EPI_PLAIN) {
    float4 v = make_float4(a[0], a[1], a[2], a[3]);
    if (p.bias && p.bias_period > 0 && (row % p.bias_period) == 0) {
      const float4 b = ld4(p.bias + col);
      v.x += b.x; v.y += b.y; v.z += b.z; v.w += b.w;
    }
    return v;
  } else if (MODE == EPI_SILU_J) {  // aux1: silu' plane (per center)
    const float4 d = ld4(p.aux1 + (long)node * p.ld_aux + col);
    return make_float4(a[0] * d.x, a[1] * d.y, a[2] * d.z, a[3] * d.w);
  } else if (MODE == EPI_SILU_L) {  // aux1: silu', aux0: silu'', aux3: sum of squared Jacobian rows
    const long o = (long)row * p.ld_aux + col;
    const float4 d1 = ld4(p.aux1 + o), d2 = ld4(p.aux0 + o), q = ld4(p.aux3 + o);
    return make_float4(a[0] * d1.x + q.x * d2.x, a[1] * d1.y + q.y * d2.y, a[2] * d1.z + q.z * d2.z,
                       a[3] * d1.w + q.w * d2.w);
  } else if (MODE == EPI_ORB_J) {
    const int pos = row / 3, t = row - 3 * pos;
    const float* env = p.aux1 + (long)node * 5 * p.ld_aux;
    const float4 ex = ld4(env + col);
    if (p.dep_map[pos] == node) {
      const float4 raw = ld4(p.aux3 + (long)node * p.ld_aux + col);
      const float4 ej = ld4(env + (1 + t) * p.ld_aux + col);
      st4(p.aux2 + ((long)node * 3 + t) * p.ld_aux + col, make_float4(a[0], a[1], a[2], a[3]));
      return make_float4(raw.x * ej.x + ex.x * a[0], raw.y * ej.y + ex.y * a[1], raw.z * ej.z + ex.z * a[2],
                         raw.w * ej.w + ex.w * a[3]);
    }
    return make_float4(ex.x * a[0], ex.y * a[1], ex.z * a[2], ex.w * a[3]);
  } else {  // EPI_ORB_L
    const float* env = p.aux1 + (long)row * 5 * p.ld_aux;
    const float* rjs = p.aux2 + (long)row * 3 * p.ld_aux;
    const float4 ex = ld4(env + col), el = ld4(env + 4 * p.ld_aux + col), raw = ld4(p.aux3 + (long)row * p.ld_aux + col);
    float4 v = make_float4(a[0] * ex.x + el.x * raw.x, a[1] * ex.y + el.y * raw.y, a[2] * ex.z + el.z * raw.z,
                           a[3] * ex.w + el.w * raw.w);
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      const float4 r = ld4(rjs + t * p.ld_aux + col), e = ld4(env + (1 + t) * p.ld_aux + col);
      v.x += 2.f * r.x * e.x; v.y += 2.f * r.y * e.y; v.z += 2.f * r.z * e.z; v.w += 2.f * r.w * e.w;
    }
    return v;
  }
}

// Applies the epilogue of MODE to columns col..col+3 of one row and stores C.
template <int MODE>
__device__ __forceinline__ void tc_store4(const GemmP<float>& p, int row, int node, int col, const float* a,
                                          int spin) {
  st4(p.C + (long)row * p.ldc + col, tc_val4<MODE>(p, row, node, col, a, spin));
}

// Epilogue values of 16 consecutive columns (col0 + 15 < N) of one row, into o: all operand loads are
// issued before the first store so that their latencies overlap.
template <int MODE>
__device__ __forceinline__ void tc_val16(const GemmP<float>& p, int row, int node, int col0, const float (&v)[16],
                                         int spin, float4 (&o)[4]) {
  if (MODE == EPI_SILU_J) {
    const float* d = p.aux1 + (long)node * p.ld_aux + col0;
    float4 dd[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) dd[u] = ld4(d + 4 * u);
#pragma unroll
    for (int u = 0; u < 4; ++u)
      o[u] = make_float4(v[4 * u] * dd[u].x, v[4 * u + 1] * dd[u].y, v[4 * u + 2] * dd[u].z, v[4 * u + 3] * dd[u].w);
  } else if (MODE == EPI_SILU_L) {
    const long of = (long)row * p.ld_aux + col0;
    float4 d1[4], d2[4], q[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      d1[u] = ld4(p.aux1 + of + 4 * u);
      d2[u] = ld4(p.aux0 + of + 4 * u);
      q[u] = ld4(p.aux3 + of + 4 * u);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      o[u] = make_float4(v[4 * u] * d1[u].x + q[u].x * d2[u].x, v[4 * u + 1] * d1[u].y + q[u].y * d2[u].y,
                         v[4 * u + 2] * d1[u].z + q[u].z * d2[u].z, v[4 * u + 3] * d1[u].w + q[u].w * d2[u].w);
  } else if (MODE == EPI_ORB_J) {
    const int pos = row / 3, t = row - 3 * pos;
    const float* env = p.aux1 + (long)node * 5 * p.ld_aux + col0;
    const bool self = p.dep_map[pos] == node;
    float4 ex[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) ex[u] = ld4(env + 4 * u);
    if (self) {
      float4 raw[4], ej[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        raw[u] = ld4(p.aux3 + (long)node * p.ld_aux + col0 + 4 * u);
        ej[u] = ld4(env + (1 + t) * p.ld_aux + 4 * u);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        o[u] = make_float4(raw[u].x * ej[u].x + ex[u].x * v[4 * u], raw[u].y * ej[u].y + ex[u].y * v[4 * u + 1],
                           raw[u].z * ej[u].z + ex[u].z * v[4 * u + 2], raw[u].w * ej[u].w + ex[u].w * v[4 * u + 3]);
        st4(p.aux2 + ((long)node * 3 + t) * p.ld_aux + col0 + 4 * u,
            make_float4(v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]));
      }
    } else {
#pragma unroll
      for (int u = 0; u < 4; ++u)
        o[u] = make_float4(ex[u].x * v[4 * u], ex[u].y * v[4 * u + 1], ex[u].z * v[4 * u + 2], ex[u].w * v[4 * u + 3]);
    }
  } else {
#pragma unroll
    for (int u = 0; u < 4; ++u) o[u] = tc_val4<MODE>(p, row, node, col0 + 4 * u, v + 4 * u, spin);
  }
}

// Epilogue of one 128-row x 128-column accumulator tile (rows [m0, m0 + 128), columns [n0, n0 + 128)) held
// in tensor memory at column tacc.  Called by the 8 epilogue warps: warp w reads TMEM lane quadrant w % 4
// (rows m0 + 32 (w % 4) + lane) and column half w / 4.  Whole-warp full 16-column chunks go out through the
// shared staging buffers stg with TMA (tma != 0), the rest with vector / scalar stores; in SILU_J mode every
// chunk first passes its squared values through the same buffer for the per-center sums.  nst counts this
// warp's TMA stores (lane 0 owns their bulk groups).
template <int MODE>
__device__ __forceinline__ void tc_epilogue_tile(const GemmP<float>& p, int rows, int m0, int n0, uint32_t tacc,
                                                 int spin_filter, int tma, const CUtensorMap* tmC, float* stg,
                                                 int& nst, int warp, int lane, bool two_acc = false,
                                                 float row_sc = 1.f, const float* col_sc = nullptr) {
  const int quad = warp & 3, half = warp >> 2;
  const int row = m0 + quad * 32 + lane;
  const bool valid = row < rows;
  const int node = valid ? gemm_node(p, row) : -1;
  bool mine = valid && !(p.row_skip > 0 && row % p.row_skip == 0);
  if (mine && spin_filter >= 0) mine = ((((node % p.n_el) < p.n_up) ? 0 : 1) == spin_filter);
  const bool tma_warp = tma != 0 && __all_sync(0xffffffffu, mine);
  // per-center sums of squared Jacobian rows: lanes 0-15 sum the even rows of column lane % 16 of a chunk,
  // lanes 16-31 the odd rows; the centers of those rows are fetched once per tile
  int nodes_h[16];
  if (MODE == EPI_SILU_J) {
#pragma unroll
    for (int i = 0; i < 16; ++i) nodes_h[i] = __shfl_sync(0xffffffffu, valid ? node : -1, 2 * i + (lane >> 4));
  }
  const uint32_t base = tacc + ((uint32_t)(quad * 32) << 16);
  for (int c0 = half * (TCP_BN / 2); c0 < (half + 1) * (TCP_BN / 2); c0 += 16) {
    float v[16];
    tmem_ld16(base + (uint32_t)c0, v);
    if (two_acc) {  // the exact hi x hi sums plus the cross terms, TCP_BN columns further on
      float v2[16];
      tmem_ld16(base + (uint32_t)(TCP_BN + c0), v2);
#pragma unroll
      for (int k = 0; k < 16; ++k) v[k] += v2[k];
    }
    if (col_sc) {  // undo the scaled-grid split: row scale times column scale (powers of two: exact)
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const int col = n0 + c0 + k;
        v[k] *= row_sc * (col < p.N ? col_sc[col] : 0.f);
      }
    }
    const int spin = spin_filter < 0 ? 0 : spin_filter;
    const bool full = n0 + c0 + 15 < p.N;
    const bool use_tma = tma_warp && full;
    float* sb = stg + (size_t)(warp * 2 + (nst & 1)) * 32 * 16;  // this chunk's staging buffer
    if (use_tma || MODE == EPI_SILU_J) {
      if (lane == 0 && nst >= 2) tma_wait_read1();  // the store from this buffer two chunks ago has read it
      __syncwarp();
    }
    if (MODE == EPI_SILU_J) {
      // squared pre-activation values through the staging buffer (row-major, 16-column rows, column index
      // XOR-swizzled by row / 2: conflict-free both ways), then segmented column sums, one atomic per center
      // run; the last runs of the two half-warps merge when they belong to the same center
#pragma unroll
      for (int c = 0; c < 16; ++c) sb[lane * 16 + (c ^ ((lane >> 1) & 15))] = valid ? v[c] * v[c] : 0.f;
      __syncwarp();
      const int c = lane & 15, h = lane >> 4, col = n0 + c0 + c;
      float s2 = 0.f;
      int cur = nodes_h[0];
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        if (nodes_h[i] != cur) {
          if (cur >= 0 && col < p.N) atomicAdd(&p.aux2[(long)cur * p.ld_aux + col], s2);
          s2 = 0.f;
          cur = nodes_h[i];
        }
        s2 += sb[(2 * i + h) * 16 + (c ^ i)];
      }
      const int other = __shfl_xor_sync(0xffffffffu, cur, 16);
      const float s2o = __shfl_xor_sync(0xffffffffu, s2, 16);
      if (other == cur) s2 = h ? 0.f : s2 + s2o;
      if (cur >= 0 && col < p.N && !(other == cur && h)) atomicAdd(&p.aux2[(long)cur * p.ld_aux + col], s2);
      __syncwarp();
    }
    if (use_tma) {
      float4 o[4];
      tc_val16<MODE>(p, row, node, n0 + c0, v, spin, o);
#pragma unroll
      for (int u = 0; u < 4; ++u)  // the tensor map's 64-byte swizzle (staging buffers are 512-byte aligned)
        *reinterpret_cast<float4*>(sb + lane * 16 + 4 * (u ^ ((lane >> 1) & 3))) = o[u];
      proxy_fence();
      __syncwarp();
      if (lane == 0) {
        tma_store_2d(tmC, smem_u32(sb), n0 + c0, m0 + quad * 32);
        tma_commit();
      }
      ++nst;
    } else if (mine) {
      if (full) {
        float4 o[4];
        tc_val16<MODE>(p, row, node, n0 + c0, v, spin, o);
#pragma unroll
        for (int u = 0; u < 4; ++u) st4(p.C + (long)row * p.ldc + n0 + c0 + 4 * u, o[u]);
      } else {
#pragma unroll
        for (int j = 0; j < 16; j += 4) {
          const int col = n0 + c0 + j;
          if (col + 3 < p.N) tc_store4<MODE>(p, row, node, col, v + j, spin);
          else
            for (int e = 0; e < 4; ++e)
              if (col + e < p.N) gemm_store<float, MODE>(p, row, col + e, v[j + e], spin);
        }
      }
    }
  }
}

// ----------------------------------------------------------------------------- streamed-weight kernel
// For K > 256 (the envelope contraction, K = 8 n_nuc): each CTA owns one 128-column slice of the output
// (n_tile = blockIdx.x % nt) and walks the 128-row tiles m = blockIdx.x / nt, + gridDim.x / nt, ...; every
// stage of a 3-stage ring carries one 64-deep k-tile of A (converted from FP32 to BF16 hi/lo by the loader
// warps) and of the split weights (copied by the same warps).  Warp roles: warps 0-7 epilogue (TMEM lane
// quadrant = warp % 4, column half = warp / 4), warps 8-11 loaders, warp 12 lane 0 issues the MMAs; TMEM
// holds two 128-column accumulators so the epilogue of one tile overlaps the MMAs of the next.
struct TcCfg {
  static constexpr int A_BYTES = TC_BM * TC_BK * 2;              // one BF16 plane of an A stage
  static constexpr int A_STAGE = 2 * A_BYTES;                    // hi + lo
  static constexpr int BK_BYTES = TCP_BN * TC_BK * 2;            // one BF16 plane of a weight k-tile
  // epilogue staging for the TMA stores of C: [warp][2 buffers][32 rows][16 columns] float
  static constexpr int STG_BYTES = 8 * 2 * 32 * 16 * 4;
  static constexpr int SB_STAGE = A_STAGE + 2 * BK_BYTES;        // A and weight k-tiles
  static constexpr int STAGES_SB = 3;
  static constexpr int TOTAL_SB = STAGES_SB * SB_STAGE + STG_BYTES + 256;
};

struct TcBar {
  uint64_t full[TCP_STAGES], empty[TCP_STAGES], tfull[2], tempty[2];
  uint32_t tmem;
  int abort;
};

__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity, volatile int* abort) {
  const uint32_t a = smem_u32(bar);
  for (long i = 0; i < TC_SPIN_LIMIT; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if ((i & 63) == 63 && *abort) return false;
  }
  *abort = 1;
  return false;
}
__device__ __forceinline__ void tc_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// tma != 0: warps whose 32 rows all belong to the launch store full 16-column chunks of C through shared
// memory with TMA (tensor map tmC over C, box 16 columns x 32 rows); other chunks use vector stores.
template <int MODE>
__global__ void __launch_bounds__(TCP_THREADS, 1) k_gemm_tcs(GemmP<float> p, const __nv_bfloat16* Bhi,
                                                            const __nv_bfloat16* Blo, int32_t* status,
                                                            const __grid_constant__ CUtensorMap tmC, int tma) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  constexpr int STAGE = TcCfg::SB_STAGE;
  constexpr int NS = TcCfg::STAGES_SB;
  constexpr int spin_filter = -1;
  const int* tile_mask = nullptr;
  unsigned char* astage = tc_smem;                               // [stage][A hi, A lo, B hi, B lo]
  float* stg = reinterpret_cast<float*>(astage + NS * STAGE);    // epilogue staging
  TcBar* bars = reinterpret_cast<TcBar*>(astage + NS * STAGE + TcCfg::STG_BYTES);
  volatile int* abort = &bars->abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  int rows = p.M;
  if (p.M_dev) rows = min(rows, p.M_scale * (*p.M_dev));
  const int mt = (rows + TC_BM - 1) / TC_BM, nt = (p.N + TCP_BN - 1) / TCP_BN;
  const int groups = gridDim.x / nt;  // CTAs per n-tile
  const int n_tile = blockIdx.x % nt, m_first = blockIdx.x / nt;
  if (m_first >= mt || n_tile >= nt) return;
  const int n0 = n_tile * TCP_BN;
  const int nk = (p.K + TC_BK - 1) / TC_BK;

  if (tid == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(smem_u32(&bars->full[s]), 128);
      mbar_init(smem_u32(&bars->empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&bars->tfull[b]), 1);
      mbar_init(smem_u32(&bars->tempty[b]), 256);
    }
    bars->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 12) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&bars->tmem)),
                 "r"(2 * TCP_BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  proxy_fence();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = bars->tmem;
  auto skip = [&](int m) -> bool {
    return spin_filter >= 0 && !((tile_mask[m] >> spin_filter) & 1);
  };

  if (warp >= 8 && warp < 12) {
    // ------------------------------------------------------------------ loaders (128 threads)
    const int lt = tid - 256;
    long kc = 0;
    for (int m = m_first; m < mt && !*abort; m += groups) {
      if (skip(m)) continue;
      const int m0 = m * TC_BM;
      for (int kt = 0; kt < nk; ++kt, ++kc) {
        const int s = (int)(kc % NS);
        const long use = kc / NS;
        if (use > 0 && !tc_wait(&bars->empty[s], (uint32_t)((use - 1) & 1), abort)) break;
        unsigned char* a_hi = astage + s * STAGE;
        unsigned char* a_lo = a_hi + TcCfg::A_BYTES;
        const int k0 = kt * TC_BK;
        // warp lw converts 8-row x 16-column blocks blk = lw + 4 u (u < 16) of the 128 x 64 tile: lane
        // (r8, kq) = (lane % 8, lane / 8) owns 4 K-consecutive elements, so a warp's loads cover 8 rows x
        // 64 contiguous bytes and its 8-byte stores fill whole 128-byte core-matrix rows (no bank conflicts)
        const int lw = lt >> 5, r8 = lane & 7, kq = lane >> 3;
        float4 v[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int blk = lw + 4 * u;
          const int r = (blk >> 2) * 8 + r8, kk = (blk & 3) * 16 + kq * 4;
          const int gr = m0 + r, gk = k0 + kk;
          v[u] = (gr < rows && gk < p.K) ? ld4(p.A + (long)gr * p.lda + gk) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int blk = lw + 4 * u;
          const int r = (blk >> 2) * 8 + r8, kk = (blk & 3) * 16 + kq * 4;
          const float f[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
          uint32_t hw[2], lw2[2];
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const __nv_bfloat16 h0 = __float2bfloat16_rn(f[2 * e]), h1 = __float2bfloat16_rn(f[2 * e + 1]);
            const __nv_bfloat16 l0 = __float2bfloat16_rn(f[2 * e] - __bfloat162float(h0));
            const __nv_bfloat16 l1 = __float2bfloat16_rn(f[2 * e + 1] - __bfloat162float(h1));
            hw[e] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
            lw2[e] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
          }
          const uint32_t off = tc_off(r, kk);
          *reinterpret_cast<uint2*>(a_hi + off) = make_uint2(hw[0], hw[1]);
          *reinterpret_cast<uint2*>(a_lo + off) = make_uint2(lw2[0], lw2[1]);
        }
        {  // this k-tile of the weights: 128 rows x 64 K of the hi and the lo plane
          unsigned char* b_hi = a_hi + TcCfg::A_STAGE;
#pragma unroll 4
          for (int u = 0; u < 16; ++u) {
            const int idx = lt + 128 * u;
            const int pl = idx >> 10, rq = idx & 1023, r = rq >> 3, c8 = rq & 7;
            const int gn = n0 + r, gk = k0 + c8 * 8;
            uint4 v4 = make_uint4(0, 0, 0, 0);
            if (gn < p.N && gk < p.K) v4 = *reinterpret_cast<const uint4*>((pl ? Blo : Bhi) + (long)gn * p.K + gk);
            *reinterpret_cast<uint4*>(b_hi + pl * TcCfg::BK_BYTES + tc_off(r, c8 * 8)) = v4;
          }
        }
        proxy_fence();
        tc_arrive(&bars->full[s]);
      }
    }
  } else if (warp == 12) {
    // ------------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      const uint32_t idesc = tc_idesc<TCP_BN>();
      const uint32_t a0 = smem_u32(astage);
      long kc = 0, uc = 0;
      for (int m = m_first; m < mt && !*abort; m += groups) {
        if (skip(m)) continue;
        const int b = (int)(uc & 1);
        const long ub = uc >> 1;
        if (ub > 0 && !tc_wait(&bars->tempty[b], (uint32_t)((ub - 1) & 1), abort)) break;
        tc_fence_after();
        const uint32_t acc_t = tmem + (uint32_t)(b * TCP_BN);
        for (int kt = 0; kt < nk; ++kt, ++kc) {
          const int s = (int)(kc % NS);
          if (!tc_wait(&bars->full[s], (uint32_t)((kc / NS) & 1), abort)) break;
          tc_fence_after();
          const uint32_t ah = a0 + s * STAGE, al = ah + TcCfg::A_BYTES;
          const uint32_t bh = ah + TcCfg::A_STAGE, bl = bh + TcCfg::BK_BYTES;
#pragma unroll
          for (int kk = 0; kk < TC_BK / 16; ++kk) {
            const uint32_t step = kk * 2 * TC_LBO;
            tc_mma(acc_t, tc_desc(ah + step), tc_desc(bh + step), idesc, (kt > 0 || kk > 0) ? 1u : 0u);
            tc_mma(acc_t, tc_desc(ah + step), tc_desc(bl + step), idesc, 1u);
            tc_mma(acc_t, tc_desc(al + step), tc_desc(bh + step), idesc, 1u);
          }
          tc_commit(smem_u32(&bars->empty[s]));
        }
        if (*abort) break;
        tc_commit(smem_u32(&bars->tfull[b]));
        ++uc;
      }
    }
  } else {
    // ------------------------------------------------------------------ epilogue (warps 0-7, 256 threads)
    long uc = 0;
    int nst = 0;  // TMA stores issued by this warp (lane 0 owns the bulk groups)
    for (int m = m_first; m < mt && !*abort; m += groups) {
      if (skip(m)) continue;
      const int m0 = m * TC_BM;
      const int b = (int)(uc & 1);
      if (!tc_wait(&bars->tfull[b], (uint32_t)((uc >> 1) & 1), abort)) break;
      tc_fence_after();
      tc_epilogue_tile<MODE>(p, rows, m0, n0, tmem + (uint32_t)(b * TCP_BN), spin_filter, tma, &tmC, stg, nst, warp,
                             lane);
      tc_fence_before();
      tc_arrive(&bars->tempty[b]);
      ++uc;
    }
    if (lane == 0 && nst > 0) tma_wait_all();  // C written and the staging buffers read
  }
  __syncthreads();
  if (*abort && tid == 0) set_flag(status, FIRE_FLAG_TIMEOUT);
  if (*abort && warp == 12 && lane == 0) {
    // bounded drain: an MMA still in flight must finish before tensor memory is released
    for (int s = 0; s < NS; ++s) {
      const uint32_t a = smem_u32(&bars->empty[s]);
      for (int i = 0; i < (1 << 16); ++i) {
        uint32_t d0, d1;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(d0)
            : "r"(a)
            : "memory");
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], 1;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(d1)
            : "r"(a)
            : "memory");
        if (d0 || d1) break;
      }
    }
  }
  __syncthreads();
  tc_fence_after();
  if (warp == 12) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TCP_BN));
  }
}

// ----------------------------------------------------------------------------- A-resident kernel (K <= 256)
// Each CTA walks its 128-row tiles m = blockIdx.x, + gridDim.x, ... and, for each, every 128-column tile of
// the output: the split A tile (hi, lo, all of K) stays in shared memory and is converted once per row tile,
// while the split weights stream through a 2-stage ring by bulk copies of pre-tiled 32 KB blocks (one
// 128-column x 64-deep tile, hi and lo planes, already in the canonical K-major layout: k-groups 2048 bytes
// apart, 8-row groups 128 bytes apart).  A is a ring of 64-deep blocks: block kb is released once the MMAs of
// the last column tile have read it, so the next row tile's conversion overlaps the current tile's tail.
// Warp roles: 0-7 epilogue, 8-11 A converters, 12 (lane 0) MMA issuer, 13 (lane 0) weight loader.
// Splitting: every row of A (and, at preparation, every column of the weights) is scaled and split on the grid of
// its own largest magnitude (split_grid_f16x2, FP16 operands), so that the hi x hi products of a row and a column are
// integers and their sum over K <= 256 is exact in FP32 whatever order and rounding the tensor core's accumulation
// uses; they accumulate in one TMEM accumulator and the terms a_hi w_lo + a_lo w_hi + a_lo w_lo in a second one (~2^-8
// of the result, so their accumulation rounding is ~2^-32 of it); the epilogue adds the two and applies the row and
// column scales.  (a_lo w_lo is kept: on the grid lo reaches half a step, 2^-8 of the row's largest value, so the
// term is ~2^-16 of a product.)  The per-element error is ~2^-20 of the row's (column's) largest value.
constexpr int TCA_THREADS = 448, TCA_KB = 4, TCA_BSTAGES = 2;
struct TcaCfg {
  static constexpr int A_BYTES = TC_BM * TC_BK * 2;  // one BF16 plane of a 128 x 64 block
  static constexpr int A_BLOCK = 2 * A_BYTES;        // hi + lo
  static constexpr int B_BLOCK = 2 * TCP_BN * TC_BK * 2;  // one tiled weight block (hi + lo)
  static constexpr int STG_BYTES = TcCfg::STG_BYTES;
  // row exponent codes (int16): the converters' halves [row tile parity][k half][128 rows], then the rows' codes for
  // the epilogue [row tile mod 4][128 rows]
  static constexpr int RMAX_BYTES = 2 * 2 * TC_BM * 2 + 4 * TC_BM * 2;
  static constexpr int TOTAL = TCA_KB * A_BLOCK + TCA_BSTAGES * B_BLOCK + STG_BYTES + RMAX_BYTES + 256;
};
struct TcaBar {
  uint64_t afull[TCA_KB], aempty[TCA_KB], bfull[TCA_BSTAGES], bempty[TCA_BSTAGES], tfull[2], tempty[2];
  uint64_t rmax;      // the converters' row maxima of a row tile are complete
  uint64_t rsfull[4];  // the row codes of row tile t (slot t mod 4) are written
  uint32_t tmem;
  int abort;
};

// Bt: tiled weights [ceil(N / 128)][ceil(K / 64)] blocks of TcaCfg::B_BLOCK bytes
template <int MODE>
__global__ void __launch_bounds__(TCA_THREADS, 1) k_gemm_tca(GemmP<float> p, const __nv_bfloat16* Bt, const float* col_sc,
                                                            int spin_filter, const int* tile_mask, int32_t* status,
                                                            const __grid_constant__ CUtensorMap tmC, int tma) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  unsigned char* ares = tc_smem;                                   // [kb][hi, lo][128 x 64], LBO 128, SBO 1024
  unsigned char* bst = tc_smem + TCA_KB * TcaCfg::A_BLOCK;         // [stage][hi, lo][8 k-groups][128 rows][16 B]
  float* stg = reinterpret_cast<float*>(bst + TCA_BSTAGES * TcaCfg::B_BLOCK);
  int16_t* rpart = reinterpret_cast<int16_t*>(bst + TCA_BSTAGES * TcaCfg::B_BLOCK + TcaCfg::STG_BYTES);
  int16_t* rcode = rpart + 2 * 2 * TC_BM;
  TcaBar* bars = reinterpret_cast<TcaBar*>(bst + TCA_BSTAGES * TcaCfg::B_BLOCK + TcaCfg::STG_BYTES +
                                           TcaCfg::RMAX_BYTES);
  volatile int* abort = &bars->abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  int rows = p.M;
  if (p.M_dev) rows = min(rows, p.M_scale * (*p.M_dev));
  const int mt = (rows + TC_BM - 1) / TC_BM, nt = (p.N + TCP_BN - 1) / TCP_BN;
  const int nk = (p.K + TC_BK - 1) / TC_BK;  // <= TCA_KB
  if ((int)blockIdx.x >= mt) return;
  auto skip = [&](int m) -> bool { return spin_filter >= 0 && !((tile_mask[m] >> spin_filter) & 1); };

  if (tid == 0) {
    for (int k = 0; k < TCA_KB; ++k) {
      mbar_init(smem_u32(&bars->afull[k]), 128);
      mbar_init(smem_u32(&bars->aempty[k]), 1);
    }
    for (int s2 = 0; s2 < TCA_BSTAGES; ++s2) {
      mbar_init(smem_u32(&bars->bfull[s2]), 1);
      mbar_init(smem_u32(&bars->bempty[s2]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&bars->tfull[b]), 1);
      mbar_init(smem_u32(&bars->tempty[b]), 256);
    }
    mbar_init(smem_u32(&bars->rmax), 128);
    for (int q = 0; q < 4; ++q) mbar_init(smem_u32(&bars->rsfull[q]), 128);
    bars->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 12) {  // two accumulator pairs (exact hi x hi sums, cross terms): all 512 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&bars->tmem)),
                 "r"(4 * TCP_BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  proxy_fence();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = bars->tmem;
  long bc_issued = 0;  // weight blocks issued (loader lane)

  if (warp >= 8 && warp < 12) {
    // ------------------------------------------------------------------ A converters (128 threads)
    // Each thread owns 8 (row, 8-deep k-group) items of every 64-deep block: one 16-byte core-matrix row in the hi
    // plane and the same row in the lo plane.  The FP32 values of an item (32 bytes) are copied asynchronously
    // straight into those two rows (first 4 into the hi row, last 4 into the lo row) as soon as the block's slot
    // is free, then split in place by the same thread: no other thread touches these bytes, so the thread's own
    // cp.async wait is the only synchronisation.  A row tile's copies are all issued before its first block is
    // split, so its HBM latency is paid about once per row tile, not once per block.
    const int lt = tid - 256, lw = lt >> 5, r8 = lane & 7, kq8 = lane >> 3;
    long ua = 0;
    for (int m = blockIdx.x; m < mt && !*abort; m += gridDim.x) {
      if (skip(m)) continue;
      const int m0 = m * TC_BM;
      int issued = 0;
      for (int kb = 0; kb < nk; ++kb) {
        if (ua > 0 && !tc_wait(&bars->aempty[kb], (uint32_t)((ua - 1) & 1), abort)) break;
        unsigned char* a_hi = ares + kb * TcaCfg::A_BLOCK;
        unsigned char* a_lo = a_hi + TcaCfg::A_BYTES;
        const int k0 = kb * TC_BK;
#pragma unroll
        for (int it = 0; it < 8; ++it) {
          const int blk = lw + 4 * it;  // (8-row group, k half)
          const int r = (blk >> 1) * 8 + r8, kk = (blk & 1) * 32 + kq8 * 8;
          const int gr = m0 + r, gk = k0 + kk;
          const bool ok = gr < rows && gk < p.K;  // K % 8 == 0: the whole k-group is inside
          const float* src = ok ? p.A + (long)gr * p.lda + gk : p.A;
          const uint32_t off = tc_off(r, kk);
          cp_async16_tc(a_hi + off, src, ok);
          cp_async16_tc(a_lo + off, src + 4, ok);
        }
        cp_async_commit_tc();
        ++issued;
      }
      if (issued < nk) break;  // aborted
      // the grid of every row: the exponent of its largest magnitude over K.  A row's k-groups belong to lanes r8,
      // r8 + 8, r8 + 16, r8 + 24 of two warps (k halves lw & 1); each warp writes its half's code, and the converters
      // meet on an mbarrier (bounded wait) before reading the other half's.  The buffer alternates between row tiles:
      // a warp writing row tile t + 2 has passed the barrier of t + 1, so every reader of t is done.
      cp_async_wait_tc(0);
      float mx[8];
#pragma unroll
      for (int it = 0; it < 8; ++it) mx[it] = 0.f;
      for (int kb = 0; kb < nk; ++kb) {
        const unsigned char* a_hi = ares + kb * TcaCfg::A_BLOCK;
        const unsigned char* a_lo = a_hi + TcaCfg::A_BYTES;
#pragma unroll
        for (int it = 0; it < 8; ++it) {
          const int blk = lw + 4 * it;
          const uint32_t off = tc_off((blk >> 1) * 8 + r8, (blk & 1) * 32 + kq8 * 8);
          const float4 x = *reinterpret_cast<const float4*>(a_hi + off);
          const float4 y = *reinterpret_cast<const float4*>(a_lo + off);
          mx[it] = fmaxf(mx[it], fmaxf(fmaxf(fmaxf(fabsf(x.x), fabsf(x.y)), fmaxf(fabsf(x.z), fabsf(x.w))),
                                       fmaxf(fmaxf(fabsf(y.x), fabsf(y.y)), fmaxf(fabsf(y.z), fabsf(y.w)))));
        }
      }
      int16_t* part = rpart + (ua & 1) * 2 * TC_BM;
#pragma unroll
      for (int it = 0; it < 8; ++it) {
        mx[it] = fmaxf(mx[it], __shfl_xor_sync(0xffffffffu, mx[it], 8));
        mx[it] = fmaxf(mx[it], __shfl_xor_sync(0xffffffffu, mx[it], 16));
        if (kq8 == 0) part[(lw & 1) * TC_BM + ((lw + 4 * it) >> 1) * 8 + r8] = (int16_t)grid_code(mx[it]);
      }
      tc_arrive(&bars->rmax);
      if (!tc_wait(&bars->rmax, (uint32_t)(ua & 1), abort)) break;
      // the rows' codes for the epilogue (slot ua mod 4; the epilogue of row tile ua - 4 finished before the MMAs of
      // row tile ua - 1, whose completion released these A blocks), published by an mbarrier of their own
      int16_t* codes = rcode + (ua & 3) * TC_BM;
      float inv[8];
#pragma unroll
      for (int it = 0; it < 8; ++it) {
        const int r = ((lw + 4 * it) >> 1) * 8 + r8;
        const int code = max((int)part[r], (int)part[TC_BM + r]);
        float sc;
        grid_scales(code, inv[it], sc);
        if (kq8 == 0 && (lw & 1) == 0) codes[r] = (int16_t)code;
      }
      tc_arrive(&bars->rsfull[ua & 3]);
      for (int kb = 0; kb < nk; ++kb) {
        unsigned char* a_hi = ares + kb * TcaCfg::A_BLOCK;
        unsigned char* a_lo = a_hi + TcaCfg::A_BYTES;
#pragma unroll
        for (int it = 0; it < 8; ++it) {
          const int blk = lw + 4 * it;
          const int r = (blk >> 1) * 8 + r8, kk = (blk & 1) * 32 + kq8 * 8;
          const uint32_t off = tc_off(r, kk);
          const float4 x = *reinterpret_cast<const float4*>(a_hi + off);
          const float4 y = *reinterpret_cast<const float4*>(a_lo + off);
          uint4 hi, lo;
          split_grid_f16x2(x.x, x.y, inv[it], hi.x, lo.x);
          split_grid_f16x2(x.z, x.w, inv[it], hi.y, lo.y);
          split_grid_f16x2(y.x, y.y, inv[it], hi.z, lo.z);
          split_grid_f16x2(y.z, y.w, inv[it], hi.w, lo.w);
          *reinterpret_cast<uint4*>(a_hi + off) = hi;
          *reinterpret_cast<uint4*>(a_lo + off) = lo;
        }
        proxy_fence();
        tc_arrive(&bars->afull[kb]);
      }
      ++ua;
    }
    cp_async_wait_tc(0);
  } else if (warp == 13) {
    // ------------------------------------------------------------------ weight loader
    if (lane == 0) {
      long bc = 0;
      for (int m = blockIdx.x; m < mt && !*abort; m += gridDim.x) {
        if (skip(m)) continue;
        for (int j = 0; j < nt && !*abort; ++j)
          for (int kb = 0; kb < nk; ++kb, ++bc) {
            const int s2 = (int)(bc % TCA_BSTAGES);
            const long use = bc / TCA_BSTAGES;
            if (use > 0 && !tc_wait(&bars->bempty[s2], (uint32_t)((use - 1) & 1), abort)) break;
            const unsigned char* src = reinterpret_cast<const unsigned char*>(Bt) +
                                       ((size_t)j * nk + kb) * (size_t)TcaCfg::B_BLOCK;
            bulk_load(smem_u32(bst + s2 * TcaCfg::B_BLOCK), src, TcaCfg::B_BLOCK, smem_u32(&bars->bfull[s2]));
            bc_issued = bc + 1;
          }
      }
    }
  } else if (warp == 12) {
    // ------------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      const uint32_t idesc = tc_idesc_f16<TCP_BN>();
      const uint32_t a0 = smem_u32(ares), b0 = smem_u32(bst);
      long ua = 0, bc = 0, uc = 0;
      for (int m = blockIdx.x; m < mt && !*abort; m += gridDim.x) {
        if (skip(m)) continue;
        for (int j = 0; j < nt && !*abort; ++j) {
          const int b = (int)(uc & 1);
          const long ub = uc >> 1;
          if (ub > 0 && !tc_wait(&bars->tempty[b], (uint32_t)((ub - 1) & 1), abort)) break;
          tc_fence_after();
          const uint32_t acc_t = tmem + (uint32_t)(b * 2 * TCP_BN);  // hi x hi sums; cross terms TCP_BN further
          for (int kb = 0; kb < nk; ++kb, ++bc) {
            if (j == 0 && !tc_wait(&bars->afull[kb], (uint32_t)(ua & 1), abort)) break;
            const int s2 = (int)(bc % TCA_BSTAGES);
            if (!tc_wait(&bars->bfull[s2], (uint32_t)((bc / TCA_BSTAGES) & 1), abort)) break;
            tc_fence_after();
            const uint32_t ah = a0 + kb * TcaCfg::A_BLOCK, al = ah + TcaCfg::A_BYTES;
            const uint32_t bh = b0 + s2 * TcaCfg::B_BLOCK, bl = bh + TcaCfg::B_BLOCK / 2;
#pragma unroll
            for (int kk = 0; kk < TC_BK / 16; ++kk) {
              const uint32_t sa = kk * 2 * TC_LBO, sb = kk * 2 * 2048;
              const uint64_t dah = tc_desc(ah + sa), dal = tc_desc(al + sa);
              const uint64_t dbh = tc_desc_s(bh + sb, 2048, 128), dbl = tc_desc_s(bl + sb, 2048, 128);
              tc_mma(acc_t, dah, dbh, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
              tc_mma(acc_t + TCP_BN, dah, dbl, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
              tc_mma(acc_t + TCP_BN, dal, dbh, idesc, 1u);
              tc_mma(acc_t + TCP_BN, dal, dbl, idesc, 1u);
            }
            tc_commit(smem_u32(&bars->bempty[s2]));
            if (j == nt - 1) tc_commit(smem_u32(&bars->aempty[kb]));
          }
          if (*abort) break;
          tc_commit(smem_u32(&bars->tfull[b]));
          ++uc;
        }
        ++ua;
      }
    }
  } else {
    // ------------------------------------------------------------------ epilogue (warps 0-7, 256 threads)
    long uc = 0, ue = 0;
    int nst = 0;
    for (int m = blockIdx.x; m < mt && !*abort; m += gridDim.x) {
      if (skip(m)) continue;
      const int m0 = m * TC_BM;
      // this thread's row scale (the converters' code of row m0 + 32 (warp % 4) + lane)
      if (!tc_wait(&bars->rsfull[ue & 3], (uint32_t)((ue >> 2) & 1), abort)) break;
      float inv_unused, row_sc;
      grid_scales((int)rcode[(ue & 3) * TC_BM + (warp & 3) * 32 + lane], inv_unused, row_sc);
      ++ue;
      for (int j = 0; j < nt && !*abort; ++j) {
        const int b = (int)(uc & 1);
        if (!tc_wait(&bars->tfull[b], (uint32_t)((uc >> 1) & 1), abort)) break;
        tc_fence_after();
        tc_epilogue_tile<MODE>(p, rows, m0, j * TCP_BN, tmem + (uint32_t)(b * 2 * TCP_BN), spin_filter, tma, &tmC,
                               stg, nst, warp, lane, true, row_sc, col_sc);
        tc_fence_before();
        tc_arrive(&bars->tempty[b]);
        ++uc;
      }
    }
    if (lane == 0 && nst > 0) tma_wait_all();
  }
  __syncthreads();
  if (*abort && tid == 0) set_flag(status, FIRE_FLAG_TIMEOUT);
  if (*abort && warp == 13 && lane == 0) {
    // bounded drain: weight copies still in flight must land before the CTA's shared memory goes away
    for (long q = bc_issued > TCA_BSTAGES ? bc_issued - TCA_BSTAGES : 0; q < bc_issued; ++q) {
      const uint32_t a = smem_u32(&bars->bfull[q % TCA_BSTAGES]);
      const uint32_t par = (uint32_t)((q / TCA_BSTAGES) & 1);
      for (int i = 0; i < (1 << 16); ++i) {
        uint32_t d0;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(d0)
            : "r"(a), "r"(par)
            : "memory");
        if (d0) break;
      }
    }
  }
  if (*abort && warp == 12 && lane == 0) {
    // bounded drain: an MMA still in flight must finish before tensor memory is released
    for (int s2 = 0; s2 < TCA_BSTAGES; ++s2) {
      const uint32_t a = smem_u32(&bars->bempty[s2]);
      for (int i = 0; i < (1 << 16); ++i) {
        uint32_t d0, d1;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(d0)
            : "r"(a)
            : "memory");
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], 1;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(d1)
            : "r"(a)
            : "memory");
        if (d0 || d1) break;
      }
    }
  }
  __syncthreads();
  tc_fence_after();
  if (warp == 12) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(4 * TCP_BN));
  }
}

// per 128-row tile: bit 0 if it holds a spin-up electron's row, bit 1 if a spin-down one (fire_tc.cu)
__global__ void k_tile_mask(GemmP<float> p, int* mask);

// Tensor map over C for the TMA-store epilogue (box 16 columns x 32 rows); false if unavailable.
bool tc_c_map(const GemmP<float>& p, CUtensorMap* map);

template <int MODE>
inline cudaError_t launch_gemm_tc(const GemmP<float>& p, const TcWeights& wt, int* mask_buf, int32_t* status,
                                  cudaStream_t s, int num_sms) {
  CUtensorMap tmC;
  std::memset(&tmC, 0, sizeof(tmC));
  const int tma = tc_c_map(p, &tmC) ? 1 : 0;
  if (p.K <= TCP_KMAX) {  // A-resident kernel with pre-tiled, column-scaled weights
    if (!wt.tiles || !wt.cs || (wt.tiles2 && !wt.cs2)) return cudaErrorInvalidValue;
    constexpr int smem = TcaCfg::TOTAL;
    cudaError_t e = cudaFuncSetAttribute(k_gemm_tca<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const long mt = (p.M + TC_BM - 1) / TC_BM;
    if (mt == 0 || p.N == 0) return cudaSuccess;
    const unsigned grid = (unsigned)std::min<long>(mt, num_sms);
    if (wt.tiles2) {
      if (!mask_buf) return cudaErrorInvalidValue;
      k_tile_mask<<<(unsigned)mt, TC_BM, 0, s>>>(p, mask_buf);
      k_gemm_tca<MODE><<<grid, TCA_THREADS, smem, s>>>(p, wt.tiles, wt.cs, 0, mask_buf, status, tmC, tma);
      k_gemm_tca<MODE><<<grid, TCA_THREADS, smem, s>>>(p, wt.tiles2, wt.cs2, 1, mask_buf, status, tmC, tma);
    } else {
      k_gemm_tca<MODE><<<grid, TCA_THREADS, smem, s>>>(p, wt.tiles, wt.cs, -1, nullptr, status, tmC, tma);
    }
    return cudaPeekAtLastError();
  }
  // K > 256: streamed weights
  if (!wt.hi) return cudaErrorInvalidValue;
  constexpr int smem = TcCfg::TOTAL_SB;
  cudaError_t e = cudaFuncSetAttribute(k_gemm_tcs<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const long mt = (p.M + TC_BM - 1) / TC_BM, nt = (p.N + TCP_BN - 1) / TCP_BN;
  if (mt == 0 || nt == 0) return cudaSuccess;
  const long groups = std::max<long>(1, std::min<long>(mt, num_sms / nt));
  k_gemm_tcs<MODE><<<(unsigned)(groups * nt), TCP_THREADS, smem, s>>>(p, wt.hi, wt.lo, status, tmC, tma);
  return cudaPeekAtLastError();
}

}  // namespace fire
