// fire_env_tc.cu -- envelope contraction of the mixed path with its coefficients generated on chip.
//
// For electron g of one spin block and determinant d, the derivative rows of the envelope carrier are
//   env[g][v][d n + o] = sum_{I, k} c_v(g, I, k) pi_d[8 I + k][o],   v = jac x, y, z and lap,
// with the forward-Laplacian coefficients of exp(-a |r_g - R_I|), a = softplus(sigma)[I][d][k]
// (EfficientIsotropicEnvelopes, envelopes.py:55-82; the same expressions as k_env_coef):
//   jac: -a e (r_g - R_I) / rho,   lap: e (a^2 - 2 a / rho),   e = exp(-a rho), rho = |r_g - R_I|.
// The coefficient matrix (8 N columns for each of 4 rows per electron) is never written to memory.  Four
// producer warps compute every 128 x 64 A block -- 32 electrons x 4 planes (plane-major: tile row
// v * 32 + electron) by 8 nuclei x 8 envelopes -- directly into shared memory: one thread per (electron,
// nucleus) evaluates rho once and the 8 exponentials and writes whole 16-byte core-matrix rows.
// The split is the scaled grid of k_gemm_tca (fire_tc.cuh) with hi parts narrowed to 2^(grid_hb(8 N) + 1), so that
// the hi x hi sums over all 8 N stay exact in FP32: a first sweep over the tile's nuclei gives every row's largest
// coefficient (the four producer warps meet on an mbarrier), then each block is written as FP16 hi + lo of the
// scaled coefficients.  The determinant's pre-tiled weights (split the same way, column scales beside them) stream
// in by bulk copies; four FP16 MMAs per 16-deep step, hi x hi into one TMEM accumulator and the other three products
// into a second, two accumulator pairs so that the epilogue of one tile overlaps the MMAs of the next; the epilogue
// adds the pair and applies the row and column scales.  Every wait is bounded.  The value row (coefficient e) stays
// on the compensated CUDA-core contraction.
#include "fire_tc.cuh"

namespace fire {

constexpr int ENV_THREADS = 448, ENV_STAGES = 3;
struct EnvCfg {
  static constexpr int A_BYTES = TC_BM * TC_BK * 2;       // one FP16 plane of a 128 x 64 A block
  static constexpr int A_BLOCK = 2 * A_BYTES;             // hi + lo
  static constexpr int B_BLOCK = 2 * TCP_BN * TC_BK * 2;  // one pre-tiled weight block (hi + lo)
  static constexpr int STAGE = A_BLOCK + B_BLOCK;
  // row exponent codes (int16): the producer warps' maxima [tile parity][warp][plane][electron], then the rows'
  // codes for the epilogue [tile mod 8][128 rows]: the producers run at most 3 blocks ahead of the MMAs and those
  // at most 2 tiles ahead of the epilogue, i.e. at most 5 tiles ahead of its reads with one block per tile
  static constexpr int CODE_SLOTS = 8;
  static constexpr int CODE_BYTES = 2 * 4 * 4 * 32 * 2 + CODE_SLOTS * TC_BM * 2;
  static constexpr int TOTAL = ENV_STAGES * STAGE + CODE_BYTES + 256;
};
struct EnvBar {
  uint64_t afull[ENV_STAGES], bfull[ENV_STAGES], empty[ENV_STAGES], tfull[2], tempty[2];
  uint64_t rmax;       // the producers' row maxima of a tile are complete
  uint64_t rsfull[EnvCfg::CODE_SLOTS];  // the row codes of tile t (slot t mod 8) are written
  uint32_t tmem;
  int abort;
};

// the 4 derivative coefficients of the 8 envelopes of nucleus I for an electron at (rx, ry, rz) (zero when !ok)
// Rn: nuclear positions [N][3]; spd: this determinant's exponents of nucleus I at spd + I * sps (shared memory,
// sps = NENV_ORB, when staged; else the global table, sps = NDET * NENV_ORB)
__device__ __forceinline__ void env_coef_vals(const float* Rn, const float* spd, int sps, bool ok, float rx, float ry,
                                              float rz, int I, float (&c)[4][NENV_ORB]) {
  if (ok) {
    const float dx = rx - Rn[3 * I], dy = ry - Rn[3 * I + 1], dz = rz - Rn[3 * I + 2];
    const float rho = sqrtf(dx * dx + dy * dy + dz * dz);
    const float irho = 1.f / rho;
    const float* a = spd + (long)I * sps;
#pragma unroll
    for (int k = 0; k < NENV_ORB; ++k) {
      const float ak = a[k];
      const float e = expf(-ak * rho);
      const float gj = -ak * e * irho;
      c[0][k] = gj * dx;
      c[1][k] = gj * dy;
      c[2][k] = gj * dz;
      c[3][k] = e * (ak * ak - 2.f * ak * irho);
    }
  } else {
#pragma unroll
    for (int v = 0; v < 4; ++v)
#pragma unroll
      for (int k = 0; k < NENV_ORB; ++k) c[v][k] = 0.f;
  }
}

// the value coefficients exp(-a rho) of the 8 envelopes of nucleus I (zero when !ok)
__device__ __forceinline__ void env_value_vals(const float* Rn, const float* spd, int sps, bool ok, float rx, float ry,
                                               float rz, int I, float (&c)[NENV_ORB]) {
  if (ok) {
    const float dx = rx - Rn[3 * I], dy = ry - Rn[3 * I + 1], dz = rz - Rn[3 * I + 2];
    const float rho = sqrtf(dx * dx + dy * dy + dz * dz);
    const float* a = spd + (long)I * sps;
#pragma unroll
    for (int k = 0; k < NENV_ORB; ++k) c[k] = expf(-a[k] * rho);
  } else {
#pragma unroll
    for (int k = 0; k < NENV_ORB; ++k) c[k] = 0.f;
  }
}

// Bt: the determinant's tiled split weights [ceil(n / 128)][ceil(8 N / 64)] blocks of EnvCfg::B_BLOCK bytes.
// Each CTA owns one 128-column slice of the output (blockIdx.x % nt) and walks the tiles of 32 electrons (4
// derivative planes), or with VAL of 128 electrons (the value plane only: the Metropolis blocks' value path, whose
// plain FP32 contraction it replaces at the same ~2^-19 accuracy; each producer thread then owns a whole row).
template <bool VAL>
__global__ void __launch_bounds__(ENV_THREADS, 1) k_env_tc(EnvTcP p, const __nv_bfloat16* Bt, int32_t* status,
                                                           int stage_params) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];  // [stage][A hi, A lo, B hi, B lo]
  int16_t* rpart = reinterpret_cast<int16_t*>(tc_smem + ENV_STAGES * EnvCfg::STAGE);  // [2][4 warps][4][32]
  int16_t* rcode = rpart + 2 * 4 * 4 * 32;                                            // [8][128]
  EnvBar* bars = reinterpret_cast<EnvBar*>(tc_smem + ENV_STAGES * EnvCfg::STAGE + EnvCfg::CODE_BYTES);
  // the nuclear positions and this determinant's exponents, staged once (stage_params) after the barriers
  float* Rsm = reinterpret_cast<float*>(tc_smem + EnvCfg::TOTAL);
  float* spsm = Rsm + 3 * p.N;
  volatile int* abort = &bars->abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n_e = p.Wc * p.ns;
  constexpr int ET = VAL ? 128 : 32;  // electrons per tile
  const int mt = (n_e + ET - 1) / ET, nt = (p.n + TCP_BN - 1) / TCP_BN;
  const int nk = (NENV_ORB * p.N + TC_BK - 1) / TC_BK;
  const int hb = grid_hb(NENV_ORB * p.N);  // hi parts of at most 2^(hb + 1): the 8 N-long hi x hi sums are exact
  const int groups = gridDim.x / nt;
  const int j = blockIdx.x % nt, m_first = blockIdx.x / nt;
  if (m_first >= mt) return;
  const int n0 = j * TCP_BN;

  if (tid == 0) {
    for (int s = 0; s < ENV_STAGES; ++s) {
      mbar_init(smem_u32(&bars->afull[s]), 128);
      mbar_init(smem_u32(&bars->bfull[s]), 1);
      mbar_init(smem_u32(&bars->empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&bars->tfull[b]), 1);
      mbar_init(smem_u32(&bars->tempty[b]), 256);
    }
    mbar_init(smem_u32(&bars->rmax), 128);
    for (int q = 0; q < EnvCfg::CODE_SLOTS; ++q) mbar_init(smem_u32(&bars->rsfull[q]), 128);
    bars->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 12) {  // two accumulator pairs (exact hi x hi sums, the other products): all 512 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&bars->tmem)),
                 "r"(4 * TCP_BN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (stage_params) {
    for (int e = tid; e < 3 * p.N; e += blockDim.x) Rsm[e] = p.R[e];
    for (int e = tid; e < NENV_ORB * p.N; e += blockDim.x)
      spsm[e] = p.sp[((long)(e / NENV_ORB) * NDET + p.d) * NENV_ORB + e % NENV_ORB];
  }
  proxy_fence();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = bars->tmem;
  long b_issued = 0;  // weight blocks issued (loader lane)
  const float* Rn = stage_params ? Rsm : p.R;
  const float* spd = stage_params ? spsm : p.sp + (long)p.d * NENV_ORB;
  const int sps = stage_params ? NENV_ORB : NDET * NENV_ORB;

  if (warp >= 8 && warp < 12) {
    // ------------------------------------------------------------------ A producers (128 threads)
    // thread (lw, lane): electron lane of the tile, nuclei 2 lw and 2 lw + 1 of every 8-nucleus block
    const int lw = warp - 8;
    long kc = 0, ut = 0;
    for (int m = m_first; m < mt && !*abort; m += groups, ++ut) {
      if constexpr (VAL) {
        // one row (electron m * 128 + 32 lw + lane) per thread: its own maximum gives its grid, no exchange
        const int row = lw * 32 + lane, ev = m * 128 + row;
        const bool vv = ev < n_e;
        float vx = 0.f, vy = 0.f, vz = 0.f;
        if (vv) {
          const long g = (long)(ev / p.ns) * p.n + p.soff + ev % p.ns;
          vx = p.r[3 * g];
          vy = p.r[3 * g + 1];
          vz = p.r[3 * g + 2];
        }
        float mxv = 0.f;
        for (int I = 0; I < p.N; ++I) {
          float c[NENV_ORB];
          env_value_vals(Rn, spd, sps, vv, vx, vy, vz, I, c);
#pragma unroll
          for (int k = 0; k < NENV_ORB; ++k) mxv = fmaxf(mxv, c[k]);
        }
        const int code = grid_code(mxv);
        float inv, sc;
        grid_scales(code, inv, sc, hb);
        rcode[(ut % EnvCfg::CODE_SLOTS) * TC_BM + row] = (int16_t)code;
        tc_arrive(&bars->rsfull[ut % EnvCfg::CODE_SLOTS]);
        for (int kb = 0; kb < nk; ++kb, ++kc) {
          const int st = (int)(kc % ENV_STAGES);
          const long use = kc / ENV_STAGES;
          if (use > 0 && !tc_wait(&bars->empty[st], (uint32_t)((use - 1) & 1), abort)) break;
          unsigned char* a_hi = tc_smem + st * EnvCfg::STAGE;
          unsigned char* a_lo = a_hi + EnvCfg::A_BYTES;
#pragma unroll 2
          for (int il = 0; il < 8; ++il) {
            const int I = kb * 8 + il;
            float c[NENV_ORB];
            env_value_vals(Rn, spd, sps, vv && I < p.N, vx, vy, vz, I, c);
            uint4 hi, lo;
            split_grid_f16x2(c[0], c[1], inv, hi.x, lo.x);
            split_grid_f16x2(c[2], c[3], inv, hi.y, lo.y);
            split_grid_f16x2(c[4], c[5], inv, hi.z, lo.z);
            split_grid_f16x2(c[6], c[7], inv, hi.w, lo.w);
            const uint32_t off = tc_off(row, il * 8);
            *reinterpret_cast<uint4*>(a_hi + off) = hi;
            *reinterpret_cast<uint4*>(a_lo + off) = lo;
          }
          proxy_fence();
          tc_arrive(&bars->afull[st]);
        }
        continue;
      }
      const int e = m * 32 + lane;
      const bool ve = e < n_e;
      float rx = 0.f, ry = 0.f, rz = 0.f;
      if (ve) {
        const long g = (long)(e / p.ns) * p.n + p.soff + e % p.ns;
        rx = p.r[3 * g];
        ry = p.r[3 * g + 1];
        rz = p.r[3 * g + 2];
      }
      // first sweep: this thread's largest coefficient of every plane over its nuclei; the four warps' maxima meet
      // in shared memory (the buffer alternates between tiles: a warp writing tile t + 2 has passed the barrier of
      // tile t + 1, so every reader of tile t is done)
      float mx[4] = {0.f, 0.f, 0.f, 0.f};
      for (int kb = 0; kb < nk; ++kb)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int I = kb * 8 + 2 * lw + q;
          float c[4][NENV_ORB];
          env_coef_vals(Rn, spd, sps, ve && I < p.N, rx, ry, rz, I, c);
#pragma unroll
          for (int v = 0; v < 4; ++v)
#pragma unroll
            for (int k = 0; k < NENV_ORB; ++k) mx[v] = fmaxf(mx[v], fabsf(c[v][k]));
        }
      int16_t* part = rpart + (ut & 1) * 4 * 4 * 32;
#pragma unroll
      for (int v = 0; v < 4; ++v) part[(lw * 4 + v) * 32 + lane] = (int16_t)grid_code(mx[v]);
      tc_arrive(&bars->rmax);
      if (!tc_wait(&bars->rmax, (uint32_t)(ut & 1), abort)) break;
      float inv[4];
      int16_t* codes = rcode + (ut % EnvCfg::CODE_SLOTS) * TC_BM;  // the epilogue has read tile ut - 8's codes
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        int code = part[v * 32 + lane];
#pragma unroll
        for (int w2 = 1; w2 < 4; ++w2) code = max(code, (int)part[(w2 * 4 + v) * 32 + lane]);
        float sc;
        grid_scales(code, inv[v], sc, hb);
        if (lw == 0) codes[v * 32 + lane] = (int16_t)code;
      }
      tc_arrive(&bars->rsfull[ut % EnvCfg::CODE_SLOTS]);
      for (int kb = 0; kb < nk; ++kb, ++kc) {
        const int st = (int)(kc % ENV_STAGES);
        const long use = kc / ENV_STAGES;
        if (use > 0 && !tc_wait(&bars->empty[st], (uint32_t)((use - 1) & 1), abort)) break;
        unsigned char* a_hi = tc_smem + st * EnvCfg::STAGE;
        unsigned char* a_lo = a_hi + EnvCfg::A_BYTES;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int il = 2 * lw + q, I = kb * 8 + il;
          float c[4][NENV_ORB];
          env_coef_vals(Rn, spd, sps, ve && I < p.N, rx, ry, rz, I, c);
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            uint4 hi, lo;
            split_grid_f16x2(c[v][0], c[v][1], inv[v], hi.x, lo.x);
            split_grid_f16x2(c[v][2], c[v][3], inv[v], hi.y, lo.y);
            split_grid_f16x2(c[v][4], c[v][5], inv[v], hi.z, lo.z);
            split_grid_f16x2(c[v][6], c[v][7], inv[v], hi.w, lo.w);
            const uint32_t off = tc_off(v * 32 + lane, il * 8);
            *reinterpret_cast<uint4*>(a_hi + off) = hi;
            *reinterpret_cast<uint4*>(a_lo + off) = lo;
          }
        }
        proxy_fence();
        tc_arrive(&bars->afull[st]);
      }
    }
  } else if (warp == 13) {
    // ------------------------------------------------------------------ weight loader
    if (lane == 0) {
      long kc = 0;
      for (int m = m_first; m < mt && !*abort; m += groups)
        for (int kb = 0; kb < nk; ++kb, ++kc) {
          const int s = (int)(kc % ENV_STAGES);
          const long use = kc / ENV_STAGES;
          if (use > 0 && !tc_wait(&bars->empty[s], (uint32_t)((use - 1) & 1), abort)) break;
          const unsigned char* src =
              reinterpret_cast<const unsigned char*>(Bt) + ((size_t)j * nk + kb) * (size_t)EnvCfg::B_BLOCK;
          bulk_load(smem_u32(tc_smem + s * EnvCfg::STAGE + EnvCfg::A_BLOCK), src, EnvCfg::B_BLOCK,
                    smem_u32(&bars->bfull[s]));
          b_issued = kc + 1;
        }
    }
  } else if (warp == 12) {
    // ------------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      const uint32_t idesc = tc_idesc_f16<TCP_BN>();
      long kc = 0, uc = 0;
      for (int m = m_first; m < mt && !*abort; m += groups) {
        const int b = (int)(uc & 1);
        const long ub = uc >> 1;
        if (ub > 0 && !tc_wait(&bars->tempty[b], (uint32_t)((ub - 1) & 1), abort)) break;
        tc_fence_after();
        const uint32_t acc_t = tmem + (uint32_t)(b * 2 * TCP_BN);  // hi x hi sums; the rest TCP_BN further
        for (int kb = 0; kb < nk; ++kb, ++kc) {
          const int s = (int)(kc % ENV_STAGES);
          const uint32_t par = (uint32_t)((kc / ENV_STAGES) & 1);
          if (!tc_wait(&bars->afull[s], par, abort) || !tc_wait(&bars->bfull[s], par, abort)) break;
          tc_fence_after();
          const uint32_t ah = smem_u32(tc_smem + s * EnvCfg::STAGE), al = ah + EnvCfg::A_BYTES;
          const uint32_t bh = ah + EnvCfg::A_BLOCK, bl = bh + EnvCfg::B_BLOCK / 2;
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
          tc_commit(smem_u32(&bars->empty[s]));
        }
        if (*abort) break;
        tc_commit(smem_u32(&bars->tfull[b]));
        ++uc;
      }
    }
  } else {
    // ------------------------------------------------------------------ epilogue (warps 0-7, 256 threads)
    // warp w: TMEM lane quadrant w % 4 = plane v (jac x, y, z, lap), lane = electron, column half w / 4
    const int quad = warp & 3, half = warp >> 2;
    long uc = 0;
    for (int m = m_first; m < mt && !*abort; m += groups) {
      const int b = (int)(uc & 1);
      // this row's scale (plane quad, electron lane), published by the producers for tile uc
      const int slot = (int)(uc % EnvCfg::CODE_SLOTS);
      if (!tc_wait(&bars->rsfull[slot], (uint32_t)((uc / EnvCfg::CODE_SLOTS) & 1), abort)) break;
      float inv_unused, row_sc;
      grid_scales((int)rcode[slot * TC_BM + quad * 32 + lane], inv_unused, row_sc, hb);
      if (!tc_wait(&bars->tfull[b], (uint32_t)((uc >> 1) & 1), abort)) break;
      tc_fence_after();
      // derivative tiles: plane quad of electron m * 32 + lane (carrier row quad + 1); value tiles: electron
      // m * 128 + 32 quad + lane (carrier row 0)
      const int e = VAL ? m * 128 + quad * 32 + lane : m * 32 + lane;
      float* out = nullptr;
      if (e < n_e) {
        const long g = (long)(e / p.ns) * p.n + p.soff + e % p.ns;
        out = p.C + (g * p.nv + (VAL ? 0 : quad + 1)) * p.ldc;
      }
      const uint32_t base = tmem + (uint32_t)(b * 2 * TCP_BN) + ((uint32_t)(quad * 32) << 16);
      for (int c0 = half * (TCP_BN / 2); c0 < (half + 1) * (TCP_BN / 2); c0 += 16) {
        const int col = n0 + c0;
        if (col >= p.n) break;  // warp-uniform
        float v[16], v2[16];
        tmem_ld16(base + (uint32_t)c0, v);
        tmem_ld16(base + (uint32_t)(TCP_BN + c0), v2);
#pragma unroll
        for (int k = 0; k < 16; ++k) v[k] = (v[k] + v2[k]) * row_sc * (col + k < p.n ? p.cs[col + k] : 0.f);
        if (!out) continue;
        if (p.vec == 4 && col + 15 < p.n) {
#pragma unroll
          for (int u = 0; u < 4; ++u) st4(out + col + 4 * u, make_float4(v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]));
        } else if (p.vec == 2 && col + 15 < p.n) {
#pragma unroll
          for (int u = 0; u < 8; ++u) *reinterpret_cast<float2*>(out + col + 2 * u) = make_float2(v[2 * u], v[2 * u + 1]);
        } else {
#pragma unroll
          for (int k = 0; k < 16; ++k)
            if (col + k < p.n) out[col + k] = v[k];
        }
      }
      tc_fence_before();
      tc_arrive(&bars->tempty[b]);
      ++uc;
    }
  }
  __syncthreads();
  if (*abort && tid == 0) set_flag(status, FIRE_FLAG_TIMEOUT);
  if (*abort && warp == 13 && lane == 0) {
    // bounded drain: weight copies still in flight must land before the CTA's shared memory goes away
    for (long q = b_issued > ENV_STAGES ? b_issued - ENV_STAGES : 0; q < b_issued; ++q) {
      const uint32_t a = smem_u32(&bars->bfull[q % ENV_STAGES]);
      const uint32_t par = (uint32_t)((q / ENV_STAGES) & 1);
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
    for (int s = 0; s < ENV_STAGES; ++s) {
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
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(4 * TCP_BN));
  }
}

cudaError_t env_tc(const EnvTcP& p, const __nv_bfloat16* Bt, int32_t* status, cudaStream_t s, bool value_rows) {
  static int num_sms = 0;
  if (num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (num_sms <= 0) num_sms = 1;
  }
  if (!Bt || !p.cs || (reinterpret_cast<uintptr_t>(Bt) & 15) != 0 || NENV_ORB * p.N > ENV_TC_KMAX)
    return cudaErrorInvalidValue;
  const long n_e = (long)p.Wc * p.ns;
  if (n_e <= 0 || p.n <= 0) return cudaSuccess;
  const long mt = (n_e + (value_rows ? 127 : 31)) / (value_rows ? 128 : 32), nt = (p.n + TCP_BN - 1) / TCP_BN;
  const long groups = std::max<long>(1, std::min<long>(mt, num_sms / nt));
  // the nuclear positions and this determinant's exponents go to shared memory when they fit
  static int smem_max = 0;
  if (smem_max == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  const size_t staged = (size_t)EnvCfg::TOTAL + sizeof(float) * (3 + NENV_ORB) * (size_t)p.N;
  const int stage_params = staged <= (size_t)smem_max ? 1 : 0;
  const int smem = stage_params ? (int)staged : EnvCfg::TOTAL;
  auto kern = value_rows ? k_env_tc<true> : k_env_tc<false>;
  const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  kern<<<(unsigned)(groups * nt), ENV_THREADS, smem, s>>>(p, Bt, status, stage_params);
  return cudaPeekAtLastError();
}

}  // namespace fire
