// fire_tc.cuh -- tcgen05 (5th-generation tensor core) contraction for the mixed-precision path.
//
// C[M, N] = A[M, K] * W[K, N] for the Jacobian and Laplacian planes of the sparse forward Laplacian,
// with the same epilogues as the CUDA-core GEMM (fire_gemm.cuh).  A is an FP32 plane; while it is
// staged into shared memory every element is split into two BF16 numbers, a = a_hi + a_lo
// (a_hi = bf16(a), a_lo = bf16(a - a_hi)).  The weights are pre-split the same way and stored
// transposed (K contiguous).  Each 16-deep K step issues three BF16 MMAs into one FP32 accumulator in
// tensor memory:  a_hi b_hi + a_hi b_lo + a_lo b_hi  (relative error ~2^-17 per product instead of
// BF16's 2^-9).
//
// Tile: 128 rows (TMEM lanes) x BN columns, K staged 64 deep, two shared-memory stages.  Shared memory
// uses the canonical K-major layout without swizzle: 8-row x 16-byte core matrices, K-adjacent core
// matrices LBO = 128 bytes apart, 8-row groups SBO = 1024 bytes apart.  One thread issues the MMAs and
// commits them to an mbarrier per stage; all waits are bounded and report FIRE_FLAG_TIMEOUT.
#pragma once
#include "fire_gemm.cuh"

namespace fire {

constexpr int TC_BM = 128, TC_BK = 64, TC_THREADS = 256;
constexpr uint32_t TC_LBO = 128, TC_SBO = 1024;
constexpr long TC_SPIN_LIMIT = 1L << 22;

struct TcWeights {
  const __nv_bfloat16* hi;   // [N][K] (K contiguous)
  const __nv_bfloat16* lo;
  const __nv_bfloat16* hi2;  // second weight set (spin down) or nullptr
  const __nv_bfloat16* lo2;
};

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
__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
  for (long i = 0; i < TC_SPIN_LIMIT; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
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

template <int BN>
struct TcSmem {
  static constexpr int A_BYTES = TC_BM * TC_BK * 2;  // 16 KB per BF16 plane
  static constexpr int B_BYTES = BN * TC_BK * 2;
  static constexpr int STAGE = 2 * A_BYTES + 2 * B_BYTES;  // a_hi, a_lo, b_hi, b_lo
  static constexpr int TOTAL = 2 * STAGE + 1024;           // + barriers / tmem holder / row ids
};

template <int MODE, int BN>
__global__ void __launch_bounds__(TC_THREADS, 1) k_gemm_tc(GemmP<float> p, TcWeights wt, int32_t* status) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  using SM = TcSmem<BN>;
  unsigned char* stage_base = tc_smem;
  unsigned char* misc = tc_smem + 2 * SM::STAGE;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(misc);       // [2]
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(misc + 64);
  int* row_node = reinterpret_cast<int*>(misc + 128);       // [128] (SILU_J)

  int rows = p.M;
  if (p.M_dev) rows = min(rows, p.M_scale * (*p.M_dev));
  const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * BN;
  if (m0 >= rows) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  int passes = 1, first_spin = 0;
  if (wt.hi2) {
    int up = 0, dn = 0;
    if (tid < TC_BM && m0 + tid < rows) {
      const int node = gemm_node(p, m0 + tid);
      if ((node % p.n_el) < p.n_up) up = 1; else dn = 1;
    }
    up = __syncthreads_or(up);
    dn = __syncthreads_or(dn);
    first_spin = up ? 0 : 1;
    passes = up + dn;
  }
  if (MODE == EPI_SILU_J && tid < TC_BM) row_node[tid] = (m0 + tid < rows) ? gemm_node(p, m0 + tid) : -1;
  if (tid == 0) {
    mbar_init(smem_u32(&mbar[0]), 1);
    mbar_init(smem_u32(&mbar[1]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                 "r"(BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  const uint32_t idesc = tc_idesc<BN>();
  const int nk = (p.K + TC_BK - 1) / TC_BK;
  uint32_t commits[2] = {0, 0};  // completed-commit counters per stage (tracked identically by all threads)
  bool ok = true;

  for (int pass = 0; pass < passes && ok; ++pass) {
    const int spin = first_spin + pass;
    const __nv_bfloat16* Bhi = spin == 0 ? wt.hi : wt.hi2;
    const __nv_bfloat16* Blo = spin == 0 ? wt.lo : wt.lo2;
    for (int kt = 0; kt < nk && ok; ++kt) {
      const int s = kt & 1;
      unsigned char* st = stage_base + s * SM::STAGE;
      if (commits[s] > 0) {
        // the MMAs that last read this stage must be complete before it is overwritten; the decision
        // is made uniform across the CTA so every thread takes the same path
        const bool w = mbar_wait(smem_u32(&mbar[s]), (commits[s] - 1) & 1);
        ok = __syncthreads_and(w) != 0;
      }
      if (!ok) break;
      const int k0 = kt * TC_BK;
      // ---- stage A (FP32 -> BF16 hi/lo), 128 x 64: 2048 float4, 8 per thread
      unsigned char* a_hi = st;
      unsigned char* a_lo = st + SM::A_BYTES;
#pragma unroll 4
      for (int q = tid; q < TC_BM * TC_BK / 4; q += TC_THREADS) {
        const int r = q / (TC_BK / 4), kq = (q % (TC_BK / 4)) * 4;
        const int gr = m0 + r, gk = k0 + kq;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gr < rows) {
          const float* src = p.A + (long)gr * p.lda + gk;
          if (gk + 3 < p.K) v = *reinterpret_cast<const float4*>(src);
          else {
            if (gk < p.K) v.x = src[0];
            if (gk + 1 < p.K) v.y = src[1];
            if (gk + 2 < p.K) v.z = src[2];
          }
        }
        const __nv_bfloat16 h0 = __float2bfloat16_rn(v.x), h1 = __float2bfloat16_rn(v.y),
                            h2 = __float2bfloat16_rn(v.z), h3 = __float2bfloat16_rn(v.w);
        const __nv_bfloat16 l0 = __float2bfloat16_rn(v.x - __bfloat162float(h0)),
                            l1 = __float2bfloat16_rn(v.y - __bfloat162float(h1)),
                            l2 = __float2bfloat16_rn(v.z - __bfloat162float(h2)),
                            l3 = __float2bfloat16_rn(v.w - __bfloat162float(h3));
        const uint32_t off = tc_off(r, kq);
        uint2 hv, lv;
        hv.x = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
        hv.y = (uint32_t)__bfloat16_as_ushort(h2) | ((uint32_t)__bfloat16_as_ushort(h3) << 16);
        lv.x = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
        lv.y = (uint32_t)__bfloat16_as_ushort(l2) | ((uint32_t)__bfloat16_as_ushort(l3) << 16);
        *reinterpret_cast<uint2*>(a_hi + off) = hv;
        *reinterpret_cast<uint2*>(a_lo + off) = lv;
      }
      // ---- stage B (pre-split BF16, [N][K]), BN x 64: 16-byte chunks of 8 elements
      unsigned char* b_hi = st + 2 * SM::A_BYTES;
      unsigned char* b_lo = b_hi + SM::B_BYTES;
      for (int q = tid; q < BN * (TC_BK / 8); q += TC_THREADS) {
        const int r = q / (TC_BK / 8), c = q % (TC_BK / 8);
        const int gn = n0 + r, gk = k0 + c * 8;
        uint4 h = make_uint4(0, 0, 0, 0), l = make_uint4(0, 0, 0, 0);
        if (gn < p.N && gk < p.K) {
          h = *reinterpret_cast<const uint4*>(Bhi + (long)gn * p.K + gk);
          l = *reinterpret_cast<const uint4*>(Blo + (long)gn * p.K + gk);
        }
        const uint32_t off = tc_off(r, c * 8);
        *reinterpret_cast<uint4*>(b_hi + off) = h;
        *reinterpret_cast<uint4*>(b_lo + off) = l;
      }
      proxy_fence();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const uint32_t ah = smem_u32(a_hi), al = smem_u32(a_lo), bh = smem_u32(b_hi), bl = smem_u32(b_lo);
#pragma unroll
        for (int kk = 0; kk < TC_BK / 16; ++kk) {
          const uint32_t step = kk * 2 * TC_LBO;
          tc_mma(tmem, tc_desc(ah + step), tc_desc(bh + step), idesc, (kt > 0 || kk > 0) ? 1u : 0u);
          tc_mma(tmem, tc_desc(ah + step), tc_desc(bl + step), idesc, 1u);
          tc_mma(tmem, tc_desc(al + step), tc_desc(bh + step), idesc, 1u);
        }
        tc_commit(smem_u32(&mbar[s]));
      }
      commits[s] += 1;
    }
    // ---- wait for the last commit, then the epilogue from TMEM
    if (ok) {
      const int s_last = (nk - 1) & 1;
      const bool w = mbar_wait(smem_u32(&mbar[s_last]), (commits[s_last] - 1) & 1);
      ok = __syncthreads_and(w) != 0;
      // the other stage's last commit precedes it in issue order and is therefore complete too
    }
    tc_fence_after();
    if (ok) {
      const int wq = warp & 3, half = warp >> 2;
      const int row_l = wq * 32 + lane;
      const int row = m0 + row_l;
      bool row_ok = row < rows;
      if (row_ok && wt.hi2) {
        const int node = gemm_node(p, row);
        row_ok = (((node % p.n_el) < p.n_up) ? 0 : 1) == spin;
      }
      float* sq = reinterpret_cast<float*>(stage_base);  // SILU_J squares [128][BN + 1] (reuses stage memory)
      for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(wq * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = n0 + c0 + j;
          if (row_ok && col < p.N) gemm_store<float, MODE>(p, row, col, v[j], spin);
          if (MODE == EPI_SILU_J) sq[row_l * (BN + 1) + c0 + j] = (row < rows) ? v[j] * v[j] : 0.f;
        }
      }
      if (MODE == EPI_SILU_J) {
        __syncthreads();
        for (int lc = tid; lc < BN; lc += TC_THREADS) {
          const int col = n0 + lc;
          if (col >= p.N) continue;
          int cur = -1;
          float acc = 0.f;
          for (int lr = 0; lr < TC_BM; ++lr) {
            const int nd = row_node[lr];
            if (nd != cur) {
              if (cur >= 0) atomicAdd(&p.aux2[(long)cur * p.ld_aux + col], acc);
              cur = nd;
              acc = 0.f;
            }
            if (nd >= 0) acc += sq[lr * (BN + 1) + lc];
          }
          if (cur >= 0) atomicAdd(&p.aux2[(long)cur * p.ld_aux + col], acc);
        }
      }
    }
    tc_fence_before();
    __syncthreads();  // TMEM reads of this pass are done before the next pass's MMAs overwrite it
    tc_fence_after();
  }
  if (!ok && tid == 0) set_flag(status, FIRE_FLAG_TIMEOUT);
  if (!ok) {
    // drain: wait (bounded) for any MMA still in flight before releasing tensor memory
    for (int s = 0; s < 2; ++s)
      if (commits[s] > 0) mbar_wait(smem_u32(&mbar[s]), (commits[s] - 1) & 1);
  }
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN));
  }
}

template <int MODE, int BN>
inline cudaError_t launch_gemm_tc(const GemmP<float>& p, const TcWeights& wt, int32_t* status, cudaStream_t s) {
  const int smem = TcSmem<BN>::TOTAL;
  cudaError_t e = cudaFuncSetAttribute(k_gemm_tc<MODE, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  dim3 grid((p.N + BN - 1) / BN, (p.M + TC_BM - 1) / TC_BM);
  if (grid.x == 0 || grid.y == 0) return cudaSuccess;
  k_gemm_tc<MODE, BN><<<grid, TC_THREADS, smem, s>>>(p, wt, status);
  return cudaPeekAtLastError();
}

}  // namespace fire
