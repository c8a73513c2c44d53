// fire_gemm.cuh -- CUDA-core GEMM C = A[M,K] * B[K,N] with fused forward-Laplacian epilogues.
//
// This is the contraction engine of the FP32 and FP64 paths.  Every dense layer of the sparse
// forward Laplacian (sparse_fwd_lap.py:160-225) is applied to three "planes" of one node:
//   X plane  [nodes, K]        values            (bias added)
//   J plane  [3 * positions, K] Jacobian rows    (sorted by center)
//   L plane  [nodes, K]        Laplacians
// and the ElementWise rule (sparse_fwd_lap.py:196-206) is fused into the epilogues:
//   X:  z = acc + b;  store z and silu(z)
//   J:  out = acc * silu'(z[center]);  jsq[center] += acc^2  (segmented over the tile's rows)
//   L:  out = acc * silu'(z) + jsq * silu''(z)
// The orbital layer (orbitals.py:148-174 + multiply_with_1el_fn, sparse_fwd_lap.py:322-335) uses
// per-spin weights (rows of spin-up centers use B, spin-down centers B2) and multiplies by the
// envelope carrier in its epilogues.
#pragma once
#include "fire_common.cuh"

namespace fire {

enum EpiMode { EPI_PLAIN = 0, EPI_SILU_X, EPI_SILU_J, EPI_SILU_L, EPI_ORB_X, EPI_ORB_J, EPI_ORB_L, EPI_ENV };

template <typename T>
struct GemmP {
  const T* A;
  long lda;
  const T* B;
  long ldb;
  const T* B2;  // spin-down weights (or nullptr)
  const T* bias;
  const T* bias2;
  int bias_period;  // bias added on rows with row % bias_period == 0 (0: no bias)
  T* C;
  long ldc;
  int M;             // row capacity
  const int* M_dev;  // optional device row count: rows = min(M, M_scale * *M_dev)
  int M_scale;
  int N, K;
  const int* node_map;  // node of a row = node_map ? node_map[row / node_div] : row / node_div
  int node_div;
  int n_el, n_up;       // spin of node g: (g % n_el) < n_up
  T* aux0;
  const T* aux1;
  T* aux2;
  const T* aux3;
  long ld_aux;
  const int* dep_map;  // ORB_J: a position is "self" when dep_map[pos] == node
  int env_ns, env_soff;  // ENV: rows are (w * env_ns + i) * env_nv + v  ->  electron w * n_el + env_soff + i
  int env_nv;            // rows per electron of the envelope carrier (5: x, jac xyz, lap; 1: value)
  int row_skip;          // tensor-core path: rows with row % row_skip == 0 are not stored (0: none)
};

constexpr int GBM = 128, GBN = 128, GBK = 8, GTHREADS = 256;

template <typename T>
__device__ __forceinline__ int gemm_node(const GemmP<T>& p, int row) {
  return p.node_map ? p.node_map[row / p.node_div] : row / p.node_div;
}

template <typename T, int MODE>
__device__ __forceinline__ void gemm_store(const GemmP<T>& p, int row, int col, T acc, int pass_spin) {
  if (MODE == EPI_PLAIN) {
    T v = acc;
    if (p.bias && p.bias_period > 0 && (row % p.bias_period) == 0) v += p.bias[col];
    p.C[(long)row * p.ldc + col] = v;
  } else if (MODE == EPI_SILU_X) {
    // value plane; with aux0 set it also writes silu'(z) (aux0) and silu''(z) (aux2), which the
    // Jacobian and Laplacian epilogues of the same layer read instead of re-evaluating them per row
    T z = acc + (p.bias ? p.bias[col] : T(0));
    p.C[(long)row * p.ldc + col] = silu(z);
    if (p.aux0) {
      T y, d1, d2;
      silu3(z, y, d1, d2);
      p.aux0[(long)row * p.ld_aux + col] = d1;
      p.aux2[(long)row * p.ld_aux + col] = d2;
    }
  } else if (MODE == EPI_SILU_J) {  // aux1: silu' plane
    const int node = gemm_node(p, row);
    p.C[(long)row * p.ldc + col] = acc * p.aux1[(long)node * p.ld_aux + col];
  } else if (MODE == EPI_SILU_L) {  // aux1: silu', aux0: silu'', aux3: sum of squared Jacobian rows
    const long o = (long)row * p.ld_aux + col;
    p.C[(long)row * p.ldc + col] = acc * p.aux1[o] + p.aux3[o] * p.aux0[o];
  } else if (MODE == EPI_ORB_X) {
    const T* b = pass_spin == 0 ? p.bias : p.bias2;
    const T raw = acc + b[col];
    p.aux0[(long)row * p.ld_aux + col] = raw;
    p.C[(long)row * p.ldc + col] = raw * p.aux1[(long)row * p.env_nv * p.ld_aux + col];
  } else if (MODE == EPI_ORB_J) {
    const int pos = row / 3, t = row - 3 * (row / 3);
    const int node = p.node_map[pos];
    const T* env = p.aux1 + (long)node * 5 * p.ld_aux;
    const T ex = env[col];
    if (p.dep_map[pos] == node) {
      const T raw = p.aux3[(long)node * p.ld_aux + col];
      p.C[(long)row * p.ldc + col] = raw * env[(1 + t) * p.ld_aux + col] + ex * acc;
      p.aux2[((long)node * 3 + t) * p.ld_aux + col] = acc;
    } else {
      p.C[(long)row * p.ldc + col] = ex * acc;
    }
  } else if (MODE == EPI_ORB_L) {
    const T* env = p.aux1 + (long)row * 5 * p.ld_aux;
    const T* rjs = p.aux2 + (long)row * 3 * p.ld_aux;
    T v = acc * env[col] + env[4 * p.ld_aux + col] * p.aux3[(long)row * p.ld_aux + col];
    v += T(2) * (rjs[col] * env[p.ld_aux + col] + rjs[p.ld_aux + col] * env[2 * p.ld_aux + col] +
                 rjs[2 * p.ld_aux + col] * env[3 * p.ld_aux + col]);
    p.C[(long)row * p.ldc + col] = v;
  } else if (MODE == EPI_ENV) {
    const int rr = row / p.env_nv, v = row - p.env_nv * rr;
    const int g = (rr / p.env_ns) * p.n_el + p.env_soff + rr % p.env_ns;
    p.C[((long)g * p.env_nv + v) * p.ldc + col] = acc;
  }
}

template <typename T, int MODE>
__global__ void __launch_bounds__(GTHREADS) k_gemm(GemmP<T> p) {
  __shared__ __align__(16) T As[2][GBK][GBM];
  __shared__ __align__(16) T Bs[2][GBK][GBN];
  extern __shared__ __align__(16) unsigned char gemm_dyn[];  // SILU_J: [GBM][GBN + 1] squares
  __shared__ int row_node[GBM];

  int rows = p.M;
  if (p.M_dev) rows = min(rows, p.M_scale * (*p.M_dev));
  const int m0 = blockIdx.y * GBM, n0 = blockIdx.x * GBN;
  if (m0 >= rows) return;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;

  // spin composition of the tile (per-spin weights)
  int passes = 1, first_spin = 0;
  if (p.B2) {
    int up = 0, dn = 0;
    if (tid < GBM && m0 + tid < rows) {
      const int node = gemm_node(p, m0 + tid);
      if ((node % p.n_el) < p.n_up) up = 1; else dn = 1;
    }
    up = __syncthreads_or(up);
    dn = __syncthreads_or(dn);
    first_spin = up ? 0 : 1;
    passes = up + dn;
  }
  if (MODE == EPI_SILU_J) {
    if (tid < GBM) row_node[tid] = (m0 + tid < rows) ? gemm_node(p, m0 + tid) : -1;
  }

  for (int pass = 0; pass < passes; ++pass) {
    const int spin = first_spin + pass;
    const T* Bp = spin == 0 ? p.B : p.B2;
    T acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = T(0);

    // global -> register staging: A: row a_r, k a_k..a_k+3; B: k b_k, cols b_c..b_c+3
    const int a_r = tid >> 1, a_k = (tid & 1) * 4;
    const int b_k = tid >> 5, b_c = (tid & 31) * 4;
    T ra[4], rb[4];
    // FP32 with 16-byte aligned rows: one vector load per operand whenever the 4 elements are in range
    const bool va = sizeof(T) == 4 && p.lda % 4 == 0 && (reinterpret_cast<uintptr_t>(p.A) & 15) == 0;
    const bool vb = sizeof(T) == 4 && p.ldb % 4 == 0 && (reinterpret_cast<uintptr_t>(Bp) & 15) == 0;
    auto load_tile = [&](int k0) {
      const int gr = m0 + a_r;
      if (va && gr < rows && k0 + a_k + 3 < p.K) {
        const float4 q = *reinterpret_cast<const float4*>(p.A + (long)gr * p.lda + k0 + a_k);
        ra[0] = q.x; ra[1] = q.y; ra[2] = q.z; ra[3] = q.w;
      } else {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int gk = k0 + a_k + u;
          ra[u] = (gr < rows && gk < p.K) ? p.A[(long)gr * p.lda + gk] : T(0);
        }
      }
      const int gk = k0 + b_k;
      if (vb && gk < p.K && n0 + b_c + 3 < p.N) {
        const float4 q = *reinterpret_cast<const float4*>(Bp + (long)gk * p.ldb + n0 + b_c);
        rb[0] = q.x; rb[1] = q.y; rb[2] = q.z; rb[3] = q.w;
      } else {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int gc = n0 + b_c + u;
          rb[u] = (gk < p.K && gc < p.N) ? Bp[(long)gk * p.ldb + gc] : T(0);
        }
      }
    };
    auto store_tile = [&](int buf) {
#pragma unroll
      for (int u = 0; u < 4; ++u) As[buf][a_k + u][a_r] = ra[u];
#pragma unroll
      for (int u = 0; u < 4; ++u) Bs[buf][b_k][b_c + u] = rb[u];
    };
    load_tile(0);
    store_tile(0);
    __syncthreads();
    int buf = 0;
    for (int k0 = 0; k0 < p.K; k0 += GBK) {
      const bool more = k0 + GBK < p.K;
      if (more) load_tile(k0 + GBK);
#pragma unroll
      for (int kk = 0; kk < GBK; ++kk) {
        T a[8], b[8];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          a[i] = As[buf][kk][ty * 4 + i];
          a[4 + i] = As[buf][kk][64 + ty * 4 + i];
          b[i] = Bs[buf][kk][tx * 4 + i];
          b[4 + i] = Bs[buf][kk][64 + tx * 4 + i];
        }
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
          for (int j = 0; j < 8; ++j) acc[i][j] += a[i] * b[j];
      }
      if (more) {
        store_tile(buf ^ 1);
        __syncthreads();
        buf ^= 1;
      }
    }

    // ---- epilogue
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int lr = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
      const int row = m0 + lr;
      if (row >= rows) continue;
      if (p.B2) {
        const int node = gemm_node(p, row);
        const int s = ((node % p.n_el) < p.n_up) ? 0 : 1;
        if (s != spin) continue;
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int col = n0 + ((j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4));
        if (col < p.N) gemm_store<T, MODE>(p, row, col, acc[i][j], spin);
      }
    }
    if (MODE == EPI_SILU_J) {
      // segmented sum of acc^2 over rows of the same center, one atomic per (segment, column)
      T* sq = reinterpret_cast<T*>(gemm_dyn);
      __syncthreads();
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int lr = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int lc = (j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4);
          sq[lr * (GBN + 1) + lc] = acc[i][j] * acc[i][j];
        }
      }
      __syncthreads();
      // 256 threads: column lc = tid & 127, rows half (tid >> 7)
      const int lc = tid & (GBN - 1), half = tid >> 7;
      const int col = n0 + lc;
      if (col < p.N) {
        int cur = -1;
        T s = T(0);
        for (int lr = half * 64; lr < half * 64 + 64; ++lr) {
          const int nd = row_node[lr];
          if (nd != cur) {
            if (cur >= 0) atomic_add(&p.aux2[(long)cur * p.ld_aux + col], s);
            cur = nd;
            s = T(0);
          }
          if (nd >= 0) s += sq[lr * (GBN + 1) + lc];
        }
        if (cur >= 0) atomic_add(&p.aux2[(long)cur * p.ld_aux + col], s);
      }
    }
    if (pass + 1 < passes) __syncthreads();
  }
}

template <typename T, int MODE>
inline cudaError_t launch_gemm(const GemmP<T>& p, cudaStream_t s) {
  dim3 grid((p.N + GBN - 1) / GBN, (p.M + GBM - 1) / GBM);
  size_t dyn = (MODE == EPI_SILU_J) ? sizeof(T) * GBM * (GBN + 1) : 0;
  if (dyn > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_gemm<T, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
  }
  if (grid.y == 0 || grid.x == 0) return cudaSuccess;
  k_gemm<T, MODE><<<grid, GTHREADS, dyn, s>>>(p);
  return cudaPeekAtLastError();
}


// ----------------------------------------------------------------------------- compensated value contraction
// FP32 and mixed paths: the value planes (one row per node) feed the orbital matrices, whose inverse amplifies
// their rounding by the condition number in the derivatives of log det.  k_gemm_comp computes them as compensated
// dot products, as if in twice the working precision and then rounded once: the error is ~2^-24 of the result even
// where the terms cancel (the orbital values are small differences of large products), which a shorter FMA chain
// per partial sum does not give.
// The exact part of every product is summed on a power-of-two grid instead of by a TwoSum per product (Ogita, Rump
// and Oishi's Dot2), in the spirit of Rump's error-free extraction against a fixed power of two:
//   - each column of B is bounded over the whole K by |b| < 2^eb, and each row of a staged 16-k tile of A is
//     scaled by a power of two so that |a'| < 1 (the row's scale 2^ea kept beside the tile);
//   - t = fma(a', b, 3 * 2^eb) then lies in [2^(eb+1), 2^(eb+2)], where floats are evenly spaced by G = 2^(eb-22),
//     so bits(t) - bits(3 * 2^eb) is the product rounded to that grid, counted in steps and summed exactly in a
//     32-bit integer (at most 16 * 2^22 per tile);
//   - fma(a', b, 3 * 2^eb - t) is the exact remainder below G / 2, summed in FP32;
//   - after each tile the step count leaves as xh + xl (xh its FP32 rounding, |xl| <= 2), and (xh G, xl G + rest),
//     scaled back by 2^ea, join a hi + lo pair by one TwoSum.
// That is five FP32/integer operations per product where Dot2 takes ten, with the same worst-case error on
// envelope- and orbital-like operands (~2^-42 of sum |a b|; measured against exact sums in a CPU restatement).
// The orbital-matrix values and the envelope values they are made of also leave the kernel as unevaluated hi + lo
// float pairs, so that the double-FP32 elimination sees them to ~2^-48.
//   COMP_PLAIN  C = a.b + bias (bias on rows with row % bias_period == 0)
//   COMP_SILU   C = silu(z), z = a.b + bias; with aux0 set also silu'(z) (aux0) and silu''(z) (aux2)
//   COMP_ENV    envelope value rows (EPI_ENV's row map, env_nv = 1): hi into C, lo into C_lo [g][ld_lo]
//   COMP_ORB    orbital values (EPI_ORB_X): raw = a.b + bias (per-spin weights and bias), rawx (aux0) = raw,
//               C + C_lo = raw (env + env_lo) with env = aux1 [row * env_nv * ld_aux], env_lo [row * ld_lo]
enum CompMode { COMP_PLAIN = 0, COMP_SILU, COMP_ENV, COMP_ORB };
constexpr int CBM = 64, CBN = 64, CBK = 16, CTHREADS = 256;

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Grid of a column whose values are bounded by m >= 0: |b| < 2^eb (eb in [-100, 119]); sg = 3 * 2^eb, g = 2^(eb-22)
// (the spacing of the floats in [2^(eb+1), 2^(eb+2)]), sb16 = 16 bits(sg) (the offset of 16 summed products).
// A non-finite or huge bound gives NaN, which every output of the column then carries.
__device__ __forceinline__ void comp_grid_col(float m, float& sg, float& g, unsigned& sb16) {
  const int field = (__float_as_int(m) >> 23) & 0xff;
  int eb = field - 126;  // m < 2^(field - 126)
  if (eb < -100) eb = -100;
  if (field == 255 || eb > 119) {
    sg = g = __int_as_float(0x7fc00000);
    sb16 = 0u;
    return;
  }
  sg = 3.f * __int_as_float((eb + 127) << 23);
  g = __int_as_float((eb + 105) << 23);
  sb16 = 16u * (unsigned)__float_as_int(sg);
}

// Scale of a row tile whose values are bounded by m >= 0: inv = 2^-ea (|a| inv < 1), sc = 2^ea; a non-finite or
// huge bound gives NaN.
__device__ __forceinline__ void comp_grid_row(float m, float& inv, float& sc) {
  if (m == 0.f) {
    inv = sc = 1.f;
    return;
  }
  const int field = (__float_as_int(m) >> 23) & 0xff;
  int ea = field - 126;  // m < 2^ea
  if (ea < -125) ea = -125;
  if (field == 255 || ea > 126) {
    inv = sc = __int_as_float(0x7fc00000);
    return;
  }
  inv = __int_as_float((127 - ea) << 23);
  sc = __int_as_float((127 + ea) << 23);
}

// 64 x 64 outputs per CTA, 4 x 4 per thread (rows 4 ty.., columns 4 tx..); A and B tiles of 16 k staged in shared
// memory (A transposed and scaled per row), the next tile prefetched into registers while the current one is
// summed.  Before the first tile every pass bounds its 64 columns of B over the whole K.
template <int MODE>
__global__ void __launch_bounds__(CTHREADS, 2) k_gemm_comp(GemmP<float> p, float* __restrict__ C_lo,
                                                           const float* __restrict__ env_lo, long ld_lo) {
  __shared__ __align__(16) float As[2][CBK][CBM];
  __shared__ __align__(16) float Bs[2][CBK][CBN];
  __shared__ __align__(16) float Asc[2][CBM];     // 2^ea of every row of the staged A tile
  __shared__ float Bmx[CTHREADS / 32][CBN];       // per-warp column maxima of |B|
  __shared__ __align__(16) float Csg[CBN];        // per column: 3 * 2^eb, the grid spacing 2^(eb-22), 16 bits(3 * 2^eb)
  __shared__ __align__(16) float Cg[CBN];
  __shared__ __align__(16) unsigned Cs16[CBN];
  const int rows = p.M;
  const int m0 = blockIdx.y * CBM, n0 = blockIdx.x * CBN;
  if (m0 >= rows) return;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  int passes = 1, first_spin = 0;
  if (p.B2) {  // per-spin weights: a pass per spin present in the tile
    int up = 0, dn = 0;
    if (tid < CBM && m0 + tid < rows) {
      if (((m0 + tid) % p.n_el) < p.n_up) up = 1; else dn = 1;
    }
    up = __syncthreads_or(up);
    dn = __syncthreads_or(dn);
    first_spin = up ? 0 : 1;
    passes = up + dn;
  }
  const int ar = tid >> 2, aq = (tid & 3) * 4;   // A: row ar, k aq..aq+3 of the tile
  const int bk = tid >> 4, bc = (tid & 15) * 4;  // B: k bk, columns bc..bc+3
  const bool va = p.lda % 4 == 0 && (reinterpret_cast<uintptr_t>(p.A) & 15) == 0;
  for (int pass = 0; pass < passes; ++pass) {
    const int spin = first_spin + pass;
    const float* Bp = spin == 0 ? p.B : p.B2;
    const bool vb = p.ldb % 4 == 0 && (reinterpret_cast<uintptr_t>(Bp) & 15) == 0;
    // the bounds of this CTA's columns over the whole K: 16 threads per k row (4 columns each), k strided by 16
    {
      const int c4 = (tid & 15) * 4, gc = n0 + c4;
      float m[4] = {0.f, 0.f, 0.f, 0.f};
      if (vb && gc + 3 < p.N) {
#pragma unroll 4
        for (int k = tid >> 4; k < p.K; k += 16) {
          const float4 q = *reinterpret_cast<const float4*>(Bp + (long)k * p.ldb + gc);
          m[0] = fmaxf(m[0], fabsf(q.x));
          m[1] = fmaxf(m[1], fabsf(q.y));
          m[2] = fmaxf(m[2], fabsf(q.z));
          m[3] = fmaxf(m[3], fabsf(q.w));
        }
      } else {
        for (int k = tid >> 4; k < p.K; k += 16) {
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (gc + u < p.N) m[u] = fmaxf(m[u], fabsf(Bp[(long)k * p.ldb + gc + u]));
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        m[u] = fmaxf(m[u], __shfl_xor_sync(0xffffffffu, m[u], 16));  // the warp's two k rows
        if ((tid & 16) == 0) Bmx[tid >> 5][c4 + u] = m[u];
      }
    }
    __syncthreads();
    if (tid < CBN) {  // one column each; read after the barrier that follows the first tile's staging
      float m = 0.f;
#pragma unroll
      for (int w = 0; w < CTHREADS / 32; ++w) m = fmaxf(m, Bmx[w][tid]);
      comp_grid_col(m, Csg[tid], Cg[tid], Cs16[tid]);
    }
    float ra[4], rb[4];
    auto load = [&](int k0) {
      const int gr = m0 + ar, gk = k0 + aq;
      if (va && gr < rows && gk + 3 < p.K) {
        const float4 q = *reinterpret_cast<const float4*>(p.A + (long)gr * p.lda + gk);
        ra[0] = q.x; ra[1] = q.y; ra[2] = q.z; ra[3] = q.w;
      } else {
#pragma unroll
        for (int u = 0; u < 4; ++u) ra[u] = (gr < rows && gk + u < p.K) ? p.A[(long)gr * p.lda + gk + u] : 0.f;
      }
      const int gk2 = k0 + bk, gc = n0 + bc;
      if (vb && gk2 < p.K && gc + 3 < p.N) {
        const float4 q = *reinterpret_cast<const float4*>(Bp + (long)gk2 * p.ldb + gc);
        rb[0] = q.x; rb[1] = q.y; rb[2] = q.z; rb[3] = q.w;
      } else {
#pragma unroll
        for (int u = 0; u < 4; ++u) rb[u] = (gk2 < p.K && gc + u < p.N) ? Bp[(long)gk2 * p.ldb + gc + u] : 0.f;
      }
    };
    // A's 16 values of row ar are held by the 4 lanes tid ^ {0, 1, 2, 3}: their maximum scales the row
    auto store = [&](int buf) {
      float m = fmaxf(fmaxf(fabsf(ra[0]), fabsf(ra[1])), fmaxf(fabsf(ra[2]), fabsf(ra[3])));
      m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
      m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 2));
      float inv, sc;
      comp_grid_row(m, inv, sc);
#pragma unroll
      for (int u = 0; u < 4; ++u) As[buf][aq + u][ar] = ra[u] * inv;
      if ((tid & 3) == 0) Asc[buf][ar] = sc;
      *reinterpret_cast<float4*>(&Bs[buf][bk][bc]) = make_float4(rb[0], rb[1], rb[2], rb[3]);
    };
    float hi[4][4], lo[4][4], rh[4][4];
    unsigned ti[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        hi[i][j] = lo[i][j] = rh[i][j] = 0.f;
        ti[i][j] = 0u;
      }
    load(0);
    store(0);
    __syncthreads();
    float sg[4];
    {
      const float4 s4 = *reinterpret_cast<const float4*>(&Csg[tx * 4]);
      sg[0] = s4.x; sg[1] = s4.y; sg[2] = s4.z; sg[3] = s4.w;
    }
    int buf = 0;
    for (int k0 = 0; k0 < p.K; k0 += CBK) {
      const bool more = k0 + CBK < p.K;
      if (more) load(k0 + CBK);
#pragma unroll 4
      for (int kk = 0; kk < CBK; ++kk) {
        const float4 a = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4]);
        const float4 b = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
        const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float t = fmaf(av[i], bv[j], sg[j]);  // the product on the grid, offset by 3 * 2^eb
            ti[i][j] += (unsigned)__float_as_int(t);
            rh[i][j] += fmaf(av[i], bv[j], sg[j] - t);  // its exact remainder
          }
      }
      // the tile's sums into the hi + lo pairs: the step count (< 2^26) as its FP32 rounding xh plus xl (|xl| <= 2)
      {
        const float4 s4 = *reinterpret_cast<const float4*>(&Asc[buf][ty * 4]);
        const float4 g4 = *reinterpret_cast<const float4*>(&Cg[tx * 4]);
        const uint4 o4 = *reinterpret_cast<const uint4*>(&Cs16[tx * 4]);
        const float sv[4] = {s4.x, s4.y, s4.z, s4.w}, gg[4] = {g4.x, g4.y, g4.z, g4.w};
        const unsigned sb16[4] = {o4.x, o4.y, o4.z, o4.w};
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int d = (int)(ti[i][j] - sb16[j]);
            const float xh = __int2float_rn(d);
            const float xl = __int2float_rn(d - __float2int_rn(xh));
            const float uh = xh * gg[j] * sv[i];
            const float ul = fmaf(xl, gg[j], rh[i][j]) * sv[i];
            float s2, e;
            two_sum(hi[i][j], uh, s2, e);
            hi[i][j] = s2;
            lo[i][j] += e + ul;
            ti[i][j] = 0u;
            rh[i][j] = 0.f;
          }
      }
      if (more) {
        store(buf ^ 1);
        __syncthreads();
        buf ^= 1;
      }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int row = m0 + ty * 4 + i;
      if (row >= rows) continue;
      if (p.B2 && (((row % p.n_el) < p.n_up) ? 0 : 1) != spin) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int col = n0 + tx * 4 + j;
        if (col >= p.N) continue;
        float h = hi[i][j], l = lo[i][j];
        if (MODE == COMP_PLAIN || MODE == COMP_SILU || MODE == COMP_ORB) {
          const float* bias = (MODE == COMP_ORB && spin == 1) ? p.bias2 : p.bias;
          const bool has_b = bias && (MODE != COMP_PLAIN || (p.bias_period > 0 && row % p.bias_period == 0));
          if (has_b) {
            float s2, e;
            two_sum(h, bias[col], s2, e);
            h = s2;
            l += e;
          }
        }
        float s2, e;  // normalised pair: s2 = fl(h + l)
        two_sum(h, l, s2, e);
        if (MODE == COMP_PLAIN) {
          p.C[(long)row * p.ldc + col] = s2;
        } else if (MODE == COMP_SILU) {
          p.C[(long)row * p.ldc + col] = silu(s2);
          if (p.aux0) {
            float y, d1, d2;
            silu3(s2, y, d1, d2);
            p.aux0[(long)row * p.ld_aux + col] = d1;
            p.aux2[(long)row * p.ld_aux + col] = d2;
          }
        } else if (MODE == COMP_ENV) {
          const int g = (row / p.env_ns) * p.n_el + p.env_soff + row % p.env_ns;
          p.C[(long)g * p.ldc + col] = s2;
          C_lo[(long)g * ld_lo + col] = e;
        } else {  // COMP_ORB
          p.aux0[(long)row * p.ld_aux + col] = s2;
          const float eh = p.aux1[(long)row * p.env_nv * p.ld_aux + col], el = env_lo[(long)row * ld_lo + col];
          const float ph = s2 * eh;
          const float pl = fmaf(s2, eh, -ph) + (s2 * el + e * eh);
          float oh, ol;
          two_sum(ph, pl, oh, ol);
          p.C[(long)row * p.ldc + col] = oh;
          C_lo[(long)row * ld_lo + col] = ol;
        }
      }
    }
    if (pass + 1 < passes) __syncthreads();
  }
}

// Envelope value rows of the refinement pass (EPI_ENV's row map, env_nv = 1) on the FP32 pipes: A holds FP64
// coefficients, B weights whose values are exact in FP32 (the float32 parameter blob's), C is FP64.  Each a is split
// into a_hi + a_lo floats; a_hi b by Dot2 (as in k_gemm_comp), a_lo b by FP32 FMAs into the low accumulator, and the
// result hi + lo leaves as a double: ~2^-44 of the terms' magnitude, where the FP64 pipe (~1/64 of the FP32 rate)
// would spend most of the pass.
template <int V = 0>  // a template so that every translation unit that includes this header may hold it
__global__ void __launch_bounds__(CTHREADS) k_gemm_env_df(GemmP<double> p) {
  __shared__ __align__(16) float Ah[2][CBK][CBM];
  __shared__ __align__(16) float Al[2][CBK][CBM];
  __shared__ __align__(16) float Bs[2][CBK][CBN];
  const int rows = p.M;
  const int m0 = blockIdx.y * CBM, n0 = blockIdx.x * CBN;
  if (m0 >= rows) return;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int ar = tid >> 2, aq = (tid & 3) * 4;   // A: row ar, k aq..aq+3 of the tile
  const int bk = tid >> 4, bc = (tid & 15) * 4;  // B: k bk, columns bc..bc+3
  double ra[4];
  float rb[4];
  auto load = [&](int k0) {
    const int gr = m0 + ar, gk = k0 + aq;
#pragma unroll
    for (int u = 0; u < 4; ++u) ra[u] = (gr < rows && gk + u < p.K) ? p.A[(long)gr * p.lda + gk + u] : 0.0;
    const int gk2 = k0 + bk, gc = n0 + bc;
#pragma unroll
    for (int u = 0; u < 4; ++u) rb[u] = (gk2 < p.K && gc + u < p.N) ? (float)p.B[(long)gk2 * p.ldb + gc + u] : 0.f;
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float h = __double2float_rn(ra[u]);
      Ah[buf][aq + u][ar] = h;
      Al[buf][aq + u][ar] = __double2float_rn(ra[u] - (double)h);
    }
    *reinterpret_cast<float4*>(&Bs[buf][bk][bc]) = make_float4(rb[0], rb[1], rb[2], rb[3]);
  };
  float hi[4][4], lo[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) hi[i][j] = lo[i][j] = 0.f;
  load(0);
  store(0);
  __syncthreads();
  int buf = 0;
  for (int k0 = 0; k0 < p.K; k0 += CBK) {
    const bool more = k0 + CBK < p.K;
    if (more) load(k0 + CBK);
#pragma unroll 4
    for (int kk = 0; kk < CBK; ++kk) {
      const float4 a = *reinterpret_cast<const float4*>(&Ah[buf][kk][ty * 4]);
      const float4 al = *reinterpret_cast<const float4*>(&Al[buf][kk][ty * 4]);
      const float4 b = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
      const float av[4] = {a.x, a.y, a.z, a.w}, alv[4] = {al.x, al.y, al.z, al.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float pr = av[i] * bv[j];
          const float pe = fmaf(av[i], bv[j], -pr);
          float s2, e;
          two_sum(hi[i][j], pr, s2, e);
          hi[i][j] = s2;
          lo[i][j] = fmaf(alv[i], bv[j], lo[i][j] + (e + pe));
        }
    }
    if (more) {
      store(buf ^ 1);
      __syncthreads();
      buf ^= 1;
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int row = m0 + ty * 4 + i;
    if (row >= rows) continue;
    const int g = (row / p.env_ns) * p.n_el + p.env_soff + row % p.env_ns;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int col = n0 + tx * 4 + j;
      if (col < p.N) p.C[(long)g * p.ldc + col] = (double)hi[i][j] + (double)lo[i][j];
    }
  }
}

inline cudaError_t launch_gemm_env_df(const GemmP<double>& p, cudaStream_t s) {
  dim3 grid((p.N + CBN - 1) / CBN, (p.M + CBM - 1) / CBM);
  if (grid.y == 0 || grid.x == 0) return cudaSuccess;
  k_gemm_env_df<0><<<grid, CTHREADS, 0, s>>>(p);
  return cudaPeekAtLastError();
}

template <int MODE>
inline cudaError_t launch_gemm_comp(const GemmP<float>& p, float* C_lo, const float* env_lo, long ld_lo,
                                    cudaStream_t s) {
  dim3 grid((p.N + CBN - 1) / CBN, (p.M + CBM - 1) / CBM);
  if (grid.y == 0 || grid.x == 0) return cudaSuccess;
  k_gemm_comp<MODE><<<grid, CTHREADS, 0, s>>>(p, C_lo, env_lo, ld_lo);
  return cudaPeekAtLastError();
}

}  // namespace fire
