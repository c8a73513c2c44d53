// fire_det.cu -- orbital envelopes, slogdet/inverse of the orbital matrices and the sparse
// determinant Laplacian.
//
//  k_env_coef   forward-Laplacian coefficients of exp(-softplus(sigma) |r - R|) per electron,
//               nucleus, determinant and envelope (EfficientIsotropicEnvelopes, envelopes.py:55-82);
//               a GEMM with pi then gives the envelope carrier [x, jac(3), lap] per orbital.
//  k_gj_global  sign/log|det| and (optionally) the inverse of every orbital matrix, computed in
//               double precision (native FP64 in the FP64 build, double-FP32 "df64" with a 48-bit
//               significand in the FP32 and mixed paths, fire_df64.cuh; the value-only path's LU in
//               FP32), one CTA per matrix with the working matrix in the workspace, eliminated in
//               panels.  Partial pivoting like jax.lax.linalg.lu, sign/log|det| as slogdet_from_lu
//               (model/utils.py:153-161), inverse as get_inverse_from_lu (144-150).
//  k_detlap     sparse_slogdet_with_fwd_lap (model/sparse_fwd_lap.py:294-319) restricted to the
//               triplets: for every dependency m, B = J[(i, m) rows] @ A^-1[:, k] for i, k in {m} + N(m)
//               gives d log det / d r_m = sum_i B[(i,m)][i] and the triplet term
//               -sum_xyz sum_{i,k} B[(i,m)][k] B[(k,m)][i]; the first Laplacian term tr(lap A A^-1) is
//               accumulated row by row.
#include "fire_df64.cuh"
#include "fire_internal.cuh"

namespace fire {

// coef layout: [det][rows = (w * n_s + i) * NV + v][N * 8]
template <typename T, int NV>
__global__ void k_env_coef(const T* __restrict__ r, const float* __restrict__ R, const T* __restrict__ sp,
                           int n, int n_s, int s_off, int N, int Wn, T* __restrict__ coef) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;  // over (w * n_s + i, I, k)
  const long total = (long)Wn * n_s * N * NENV_ORB;
  if (idx >= total) return;
  const int k = (int)(idx % NENV_ORB);
  const int I = (int)((idx / NENV_ORB) % N);
  const long rr = idx / ((long)NENV_ORB * N);
  const int w = (int)(rr / n_s), i = (int)(rr % n_s);
  const long g = (long)w * n + s_off + i;
  const T dx = r[3 * g] - (T)R[3 * I], dy = r[3 * g + 1] - (T)R[3 * I + 1], dz = r[3 * g + 2] - (T)R[3 * I + 2];
  const T rho = dsqrt(dx * dx + dy * dy + dz * dz);
  const T irho = T(1) / rho;
  const long rows = (long)Wn * n_s * NV;
  const int K8 = N * NENV_ORB;
#pragma unroll
  for (int d = 0; d < NDET; ++d) {
    const T a = sp[(I * NDET + d) * NENV_ORB + k];
    const T e = dexp(-a * rho);
    T* out = coef + (long)d * rows * K8 + (rr * NV) * K8 + I * NENV_ORB + k;
    out[0] = e;
    if (NV > 1) {
      const T gj = -a * e * irho;
      out[K8] = gj * dx;
      out[2 * K8] = gj * dy;
      out[3 * K8] = gj * dz;
      out[4 * K8] = e * (a * a - T(2) * a * irho);
    }
  }
}

// two adjacent elements with one 16-byte (double, df64) or 8-byte (float) shared-memory load; p is aligned to
// twice the element size
__device__ __forceinline__ void ld_pair(const float* p, float& a, float& b) {
  const float2 v = *reinterpret_cast<const float2*>(p);
  a = v.x;
  b = v.y;
}
__device__ __forceinline__ void ld_pair(const double* p, double& a, double& b) {
  const double2 v = *reinterpret_cast<const double2*>(p);
  a = v.x;
  b = v.y;
}
__device__ __forceinline__ void ld_pair(const df64* p, df64& a, df64& b) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  a = df64(v.x, v.y);
  b = df64(v.z, v.w);
}

__device__ __forceinline__ uint32_t smem_u32_det(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

constexpr int GJG_BW = 16, GJG_THREADS = 512;

// Gauss-Jordan inversion / LU with partial pivoting, one matrix per CTA, the working matrix in global
// memory (the caller's workspace, row-major [n][n] in the elimination type S) instead of shared memory, so
// that every matrix of the batch is in flight at once (two CTAs per SM) and the kernel is bound by
// arithmetic, not by the latency of n dependent steps.  Columns are eliminated in panels of GJG_BW:
//  1. the panel is loaded into shared memory and factored there, recording the pivot row p_t of every
//     step and the step's transform x <- x - w_t x[k_t] of any other column x (w_t kept in the final row
//     order of the panel: later interchanges are applied to it as well);
//  2. W~ = W L^-1 with L[t][s] = w_s[k_t] (unit lower triangular), so that the whole panel acts on another
//     column as: interchange rows k_t <-> p_t, then x <- x - W~ x[k_0 .. k_{b-1}];
//  3. every other column (LU: every column right of the panel) is streamed through shared memory in chunks
//     of GJG_BW columns and updated with that rank-b product.
// A: element (i, o) of matrix (w, d) at A[((w * n + i) * NDET + d) * n + o]  (the orbital plane [G][D * n]);
// A_lo (double-FP32 elimination only, may be null): the low parts of the same elements.
// Outputs: logdet[w * NDET + d], sign[...] (double); if INV the inverse, transposed and aligned for
// k_detlap: Ainv[((w * NDET + d) * n + i) * ainv_ld(n) + sh + o] = (A^-1)[o][i] with sh = (d n) mod 4 and zeros
// in the other entries of the row, written after undoing the column permutation; if INV and cond is not null,
// cond[w * NDET + d] = ||A||_F ||A^-1||_F (the Frobenius condition number, >= the 2-norm one).
template <typename S, typename TI, typename TO, bool INV>
__global__ void __launch_bounds__(GJG_THREADS, 2) k_gj_global(const TI* __restrict__ A, const TI* __restrict__ A_lo,
                                                             int n, S* __restrict__ work,
                                                             double* __restrict__ logdet, double* __restrict__ sign,
                                                             double* __restrict__ cond, TO* __restrict__ Ainv,
                                                             int32_t* status) {
  extern __shared__ __align__(16) unsigned char gj_smem[];
  constexpr int BW = GJG_BW, LD = GJG_BW + 1;  // shared rows padded: column walks spread over the banks
  const int mat = blockIdx.x;
  const int w = mat / NDET, d = mat - w * NDET;
  // two working copies per matrix: every panel reads one and writes the other
  S* Mb[2] = {work + (size_t)mat * n * n, work + ((size_t)gridDim.x + mat) * n * n};
  S* pan = reinterpret_cast<S*>(gj_smem);  // [n][LD] the panel, then each chunk of other columns
  S* W = pan + (size_t)n * LD;             // [n][LD] panel transforms (then W~)
  S* Li = W + (size_t)n * LD;              // [BW][BW] L^-1
  S* colk = Li + BW * BW;                  // [n] pivot column before the step (interchanged order)
  S* rk = colk + n;                        // [BW] row k of the panel before the step
  S* rp = rk + BW;                         // [BW] row p
  S* rj = rp + BW;                         // [BW] row p scaled by the inverse pivot
  int* perm = reinterpret_cast<int*>(rj + BW);  // [n]
  int* piv = perm + n;                     // [BW]
  int* rowmap = piv + BW;                  // [n] source row of every row after the panel's interchanges
  static_assert(sizeof(S) == 8, "redv doubles as the double reduction buffer");
  __shared__ __align__(8) S redv[32];
  __shared__ int redi[32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nwarp = blockDim.x >> 5;
  double sq = 0.0;  // ||A||_F^2, then ||A^-1||_F^2 (condition number output)
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e / n, o = e - i * n;
    const long ia = ((long)(w * n + i) * NDET + d) * n + o;
    const TI a = A[ia];
    if constexpr (std::is_same<S, df64>::value && std::is_same<TI, float>::value)
      Mb[0][e] = A_lo ? df64(a, A_lo[ia]) : S(a);  // the compensated orbital values: a normalised hi + lo pair
    else
      Mb[0][e] = (S)a;
    sq += (double)a * (double)a;
  }
  // the block sums of the condition number go through redv (8-byte elements; no static shared memory is added,
  // so that the largest matrix still fits): thread 0 keeps ||A||_F^2
  double* redd = reinterpret_cast<double*>(redv);
  double a2 = 0.0;
  if (INV && cond) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if (lane == 0) redd[wid] = sq;
    sq = 0.0;
  }
  __syncthreads();
  if (INV && cond && tid == 0)  // before the first panel's barrier, after which redv is written again
    for (int q = 0; q < nwarp; ++q) a2 += redd[q];
  double ld = 0.0;
  int neg = 0, sing = 0;
  const int npan = (n + BW - 1) / BW;
  const int cj = tid % BW, rg = tid / BW, rn = blockDim.x / BW;  // chunk update: column, row group
  for (int P = 0; P < npan; ++P) {
    const int k0 = P * BW, bw = min(BW, n - k0);
    const S* src = Mb[P & 1];
    S* dst = Mb[(P + 1) & 1];
    if (cj < bw)
      for (int i = rg; i < n; i += rn) pan[i * LD + cj] = src[(size_t)i * n + k0 + cj];
    __syncthreads();
    // ---- factor the panel
    for (int t = 0; t < bw; ++t) {
      const int k = k0 + t;
      S best = S(-1);
      int bi = n;
      for (int i = k + tid; i < n; i += blockDim.x) {
        const S v = absv(pan[i * LD + t]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const S ov = shfl_xor_any(best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (lane == 0) {
        redv[wid] = best;
        redi[wid] = bi;
      }
      __syncthreads();
      S bv = lane < nwarp ? redv[lane] : S(-1);
      int p = lane < nwarp ? redi[lane] : n;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const S ov = shfl_xor_any(bv, o);
        const int oi = __shfl_xor_sync(0xffffffffu, p, o);
        if (ov > bv || (ov == bv && oi < p)) {
          bv = ov;
          p = oi;
        }
      }
      if (p >= n) p = k;
      const S pv = pan[p * LD + t];
      const S ipv = pv != S(0) ? S(1) / pv : S(0);
      if (tid == 0) {
        piv[t] = p;
        perm[k] = p;
        if (pv == S(0)) sing = 1;
        ld += ::log(::fabs((double)pv));
        if (pv < S(0)) neg ^= 1;
        if (p != k) neg ^= 1;
      }
      for (int i = (INV ? 0 : k) + tid; i < n; i += blockDim.x) colk[i] = pan[(i == k ? p : (i == p ? k : i)) * LD + t];
      for (int j = tid; j < bw; j += blockDim.x) {
        rk[j] = pan[k * LD + j];
        rp[j] = pan[p * LD + j];
        rj[j] = rp[j] * ipv;
      }
      if (p != k)  // earlier transforms follow the interchange
        for (int s2 = tid; s2 < t; s2 += blockDim.x) {
          const S tk = W[k * LD + s2];
          W[k * LD + s2] = W[p * LD + s2];
          W[p * LD + s2] = tk;
        }
      __syncthreads();
      if (INV) {  // Gauss-Jordan: every row of the panel columns not yet eliminated (the eliminated ones are
                  // rebuilt from W~ after the panel)
        const int nc = bw - t - 1;
        if (nc > 0) {
          const float inc = 1.f / (float)nc;
          for (int e = tid; e < n * nc; e += blockDim.x) {
            int i = (int)((float)e * inc);
            if (i * nc > e) --i;
            else if ((i + 1) * nc <= e) ++i;
            const int j = t + 1 + (e - i * nc);
            S* el = pan + i * LD + j;
            *el = i == k ? rj[j] : df_sub_mul(i == p ? rk[j] : *el, colk[i], rj[j]);
          }
        }
      } else {  // LU: rows k.. of the panel columns right of the pivot (rows above k do not change)
        const int nc = bw - t - 1, nr = n - k;
        for (int e = tid; e < nr * nc; e += blockDim.x) {
          const int ii = e / nc, i = k + ii, j = t + 1 + (e - ii * nc);
          S* el = pan + i * LD + j;
          const S old = i == k ? rp[j] : (i == p ? rk[j] : *el);
          *el = i > k ? df_sub_mul(old, colk[i] * ipv, rp[j]) : old;
        }
      }
      for (int i = tid; i < n; i += blockDim.x)
        W[i * LD + t] = INV ? (i == k ? S(1) - ipv : colk[i] * ipv) : (i > k ? colk[i] * ipv : S(0));
      __syncthreads();
    }
    // ---- L^-1 (one lane per column s: Li[t][s] = -sum_{u=s}^{t-1} L[t][u] Li[u][s]) and W~ = W L^-1
    if (tid < bw) {
      for (int t = 0; t < bw; ++t) {
        SubDot<S> acc;
        for (int u = tid; u < t; ++u) acc.add(W[(k0 + t) * LD + u], Li[u * BW + tid]);
        Li[t * BW + tid] = acc.finish(t == tid ? S(1) : S(0));
      }
    }
    if (tid == 0) {  // the panel's row interchanges as one permutation
      for (int i = 0; i < n; ++i) rowmap[i] = i;
      for (int t = 0; t < bw; ++t) {
        const int q = piv[t];
        const int tmp = rowmap[k0 + t];
        rowmap[k0 + t] = rowmap[q];
        rowmap[q] = tmp;
      }
    }
    __syncthreads();
    for (int i = tid; i < n; i += blockDim.x) {
      S wr[BW];
#pragma unroll
      for (int q = 0; q < BW; ++q) wr[q] = q < bw ? W[i * LD + q] : S(0);
#pragma unroll
      for (int t = 0; t < BW; ++t) {
        if (t >= bw) break;
        SubDot<S> acc;
#pragma unroll
        for (int q = 0; q < BW; ++q)
          if (q >= t && q < bw) acc.add(wr[q], Li[q * BW + t]);
        W[i * LD + t] = acc.sum();
      }
    }
    __syncthreads();
    if (INV && cj < bw)  // the panel's final columns, e_{k0+s} - W~[:, s] (the LU never reads finished panels)
      for (int i = rg; i < n; i += rn) dst[(size_t)i * n + k0 + cj] = (i == k0 + cj ? S(1) : S(0)) - W[i * LD + cj];
    // ---- apply the panel to the other columns (LU: the columns right of the panel, rows from k0):
    // x <- x - W~ y with y the panel's pivot rows of x.  Y (the bw pivot rows of every column, interchanged
    // order, rows padded to an even length) is staged over the panel buffer, which is free now; each thread
    // owns a pair of adjacent columns and walks its rows two at a time (2 x 2 tiles: three shared loads per
    // four products), reading the interchanged rows of src and writing dst (no in-place hazard).
    S* Y = pan;
    const int ldy = n + (n & 1);
    for (int t = 0; t < bw; ++t) {
      const S* yr = src + (size_t)rowmap[k0 + t] * n;
      for (int c = (INV ? 0 : k0 + bw) + tid; c < n; c += blockDim.x) Y[t * ldy + c] = yr[c];
    }
    __syncthreads();
    {
      const int cp = tid & 15, rg = tid >> 4, rn2 = blockDim.x >> 4;  // column pair, row group
      const int i0 = INV ? 0 : k0;
      for (int c = (INV ? 0 : k0 + bw) + 2 * cp; c < n; c += 32) {
        if (INV && c >= k0 && c < k0 + bw) continue;  // the panel's own columns (pairs never straddle it)
        const bool c1 = c + 1 < n;
        int i = i0 + rg;
        for (; i + rn2 < n; i += 2 * rn2) {
          const S* s0 = src + (size_t)rowmap[i] * n + c;
          const S* s1 = src + (size_t)rowmap[i + rn2] * n + c;
          const S a00 = s0[0], a10 = s1[0];
          const S a01 = c1 ? s0[1] : S(0), a11 = c1 ? s1[1] : S(0);
          const S *w0 = W + i * LD, *w1 = W + (i + rn2) * LD;
          SubDot<S> d00, d01, d10, d11;
          if (bw == BW) {
#pragma unroll
            for (int t = 0; t < BW; ++t) {
              S y0, y1;
              ld_pair(Y + t * ldy + c, y0, y1);
              const S wa = w0[t], wb = w1[t];
              d00.add(wa, y0);
              d01.add(wa, y1);
              d10.add(wb, y0);
              d11.add(wb, y1);
            }
          } else {
            for (int t = 0; t < bw; ++t) {
              S y0, y1;
              ld_pair(Y + t * ldy + c, y0, y1);
              const S wa = w0[t], wb = w1[t];
              d00.add(wa, y0);
              d01.add(wa, y1);
              d10.add(wb, y0);
              d11.add(wb, y1);
            }
          }
          S* o0 = dst + (size_t)i * n + c;
          S* o1 = dst + (size_t)(i + rn2) * n + c;
          o0[0] = d00.finish(a00);
          o1[0] = d10.finish(a10);
          if (c1) {
            o0[1] = d01.finish(a01);
            o1[1] = d11.finish(a11);
          }
        }
        if (i < n) {
          const S* s0 = src + (size_t)rowmap[i] * n + c;
          const S a00 = s0[0], a01 = c1 ? s0[1] : S(0);
          const S* w0 = W + i * LD;
          SubDot<S> d00, d01;
          for (int t = 0; t < bw; ++t) {
            S y0, y1;
            ld_pair(Y + t * ldy + c, y0, y1);
            d00.add(w0[t], y0);
            d01.add(w0[t], y1);
          }
          S* o0 = dst + (size_t)i * n + c;
          o0[0] = d00.finish(a00);
          if (c1) o0[1] = d01.finish(a01);
        }
      }
    }
    __syncthreads();  // dst complete before the next panel reads it
  }
  if (tid == 0) {
    logdet[mat] = ld;
    sign[mat] = neg ? -1.0 : 1.0;
    if (sing) set_flag(status, FIRE_FLAG_SINGULAR);
  }
  if (INV) {
    // undo the row interchanges on the columns: final column jc holds working column src(jc)
    int* srcc = reinterpret_cast<int*>(colk);
    if (tid == 0) {
      for (int q = 0; q < n; ++q) srcc[q] = q;
      for (int k = n - 1; k >= 0; --k) {
        const int p = perm[k];
        if (p != k) {
          const int t = srcc[k];
          srcc[k] = srcc[p];
          srcc[p] = t;
        }
      }
    }
    __syncthreads();
    // transposed output, row i = column i of the inverse, shifted by the determinant's offset sh within the
    // orbital plane and zero-padded (see ainv_ld): 32 rows of the working matrix at a time are staged in
    // shared memory (the panel buffers are free) so that both the reads and the writes are row-contiguous
    const int nA = ainv_ld(n), sh = (d * n) & 3;
    TO* out = Ainv + (size_t)mat * n * nA;
    const S* M = Mb[npan & 1];
    S* tile = pan;  // [32][n]
    for (int o0 = 0; o0 < n; o0 += 32) {
      const int ro = min(32, n - o0);
      for (int e = tid; e < ro * n; e += blockDim.x) {
        const S v = M[(size_t)o0 * n + e];
        tile[e] = v;
        sq += (double)v * (double)v;
      }
      __syncthreads();
      for (int e = tid; e < n * 32; e += blockDim.x) {
        const int i = e >> 5, r = e & 31;
        if (r < ro) out[(size_t)i * nA + sh + o0 + r] = (TO)tile[r * n + srcc[i]];
      }
      __syncthreads();
    }
    const int npad = nA - n;
    for (int e = tid; e < n * npad; e += blockDim.x) {
      const int i = e / npad, q = e - i * npad;
      out[(size_t)i * nA + (q < sh ? q : n + q)] = TO(0);
    }
    if (cond) {  // kappa_F = ||A||_F ||A^-1||_F
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
      if (lane == 0) redd[wid] = sq;
      __syncthreads();
      if (tid == 0) {
        double b2 = 0.0;
        for (int q = 0; q < nwarp; ++q) b2 += redd[q];
        cond[mat] = sqrt(a2 * b2);
      }
    }
  }
}

// Determinant Laplacian for one (walker, det, dependency m).  Jp: orbital Jacobian plane
// [3 * positions][NDET * n]; AinvT: the transposed, shifted inverse written by k_gj_global; lapA [G][NDET * n].
// Outputs: grad [W][NDET][n][3], lap [W * NDET] (double, +=).
// B = J[(i, m) rows] (3c x n) @ A^-1[:, {i}] (n x c): both operands are read along the contraction index o
// (J rows and rows of the transposed inverse), in 16-byte quads of x = o + sh where sh = (d n) mod 4 makes the
// J rows of determinant d 16-byte aligned; the inverse rows carry the same shift and zeros outside o in [0, n),
// which cancel the neighbouring columns the J quads pick up.  Chunks of DL_OC x are copied asynchronously
// (cp.async) into a ring of DL_STAGES shared-memory buffers, rows of DL_LD elements; each thread accumulates 4 x 4 tiles
// whose rows (r, r + TR, r + 2 TR, r + 3 TR) and columns (k, k + TC, ...) are strided, so that a warp's 16-byte
// loads hit consecutive rows: 8 shared loads per 64 FMAs, no bank conflicts.  The result tile reuses the
// staging memory.
static_assert(3 * DL_CMAX * (DL_CMAX + 1) <= dl_smem_elems(DL_CMAX), "result tile inside the staging buffers");
static_assert(3 * DL_CSPLIT * (DL_CSPLIT + 1) <= dl_smem_elems(DL_CSPLIT), "result tile inside the staging buffers");
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool ok) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32_det(dst)), "l"(src), "r"(ok ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// four consecutive elements of a 16-byte aligned row
__device__ __forceinline__ void ld_quad(const float* p, float (&v)[4]) {
  const float4 q = *reinterpret_cast<const float4*>(p);
  v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
__device__ __forceinline__ void ld_quad(const double* p, double (&v)[4]) {
  const double2 a = *reinterpret_cast<const double2*>(p), b = *reinterpret_cast<const double2*>(p + 2);
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
// NT threads; jobs with CLO < cnt <= CHI (the others are left to the other instance; cnt > DL_CMAX reports a
// pair overflow)
template <typename T, int NT, int CLO, int CHI>
__global__ void __launch_bounds__(NT) k_detlap(Nbr nb, Layout L, const T* __restrict__ Jp,
                                               const T* __restrict__ AinvT, const T* __restrict__ lapA,
                                               double* __restrict__ grad, double* __restrict__ lap, int32_t* status) {
  constexpr int JROWS = dl_jrows(CHI), STAGE = dl_stage_elems(CHI), BLD = CHI + 1;
  constexpr int MAXT = ((3 * CHI + 3) / 4 * ((CHI + 3) / 4) + NT - 1) / NT;  // 4 x 4 tiles per thread
  constexpr int RPT = (4 * CHI + NT - 1) / NT;                              // staged rows per thread
  extern __shared__ __align__(16) unsigned char dl_smem[];
  const int n = nb.n, nA = ainv_ld(n);
  const int m = blockIdx.x, d = blockIdx.y, w = blockIdx.z;
  const int* rp = nb.rowptr + (size_t)w * (n + 1);
  if (rp[n] > nb.cap_p) return;
  const int cnt = rp[m + 1] - rp[m] + 1;
  if (cnt <= CLO) return;
  if (cnt > CHI) {
    if (CHI == DL_CMAX && threadIdx.x == 0) set_flag(status, FIRE_FLAG_PAIR_OVERFLOW);
    return;
  }
  T* stg = reinterpret_cast<T*>(dl_smem);  // [DL_STAGES][J rows JROWS, inverse rows CHI + 4][DL_LD]
  T* Bm = reinterpret_cast<T*>(dl_smem);   // [3 * CHI][BLD] after the main loop
  __shared__ long qrow[3 * CHI];           // element index of x = 0 of J row rr
  __shared__ int is[CHI];
  const int tid = threadIdx.x;
  const int off = L.pos_off[w];
  const int s0 = off + rp[m] + m;
  const long ldj = (long)NDET * n;
  const int sh = (d * n) & 3, XN = (sh + n + 3) & ~3;
  for (int k = tid; k < cnt; k += blockDim.x) {
    const int q = L.dep_pos[s0 + k];
    is[k] = L.pos_ctr[q] - w * n;
    for (int t = 0; t < 3; ++t) qrow[3 * k + t] = (3L * q + t) * ldj + (long)d * n - sh;
  }
  __syncthreads();
  const int R = 3 * cnt;
  const T* Ab = AinvT + ((size_t)w * NDET + d) * n * nA;
  constexpr int QPR = DL_OC / 4;           // quads per row and chunk
  constexpr int CPQ = 4 * sizeof(T) / 16;  // 16-byte copies per quad
  constexpr int EPC = 16 / sizeof(T);      // elements per copy
  // staging: thread tid owns rows tid, tid + NT, ... of the R J rows followed by the cnt inverse rows is[k],
  // for the whole job
  const T* srow[RPT];
  int drow[RPT];
#pragma unroll
  for (int q = 0; q < RPT; ++q) {
    const int row = tid + q * NT;
    srow[q] = Ab;
    drow[q] = -1;
    if (row < R) {
      srow[q] = Jp + qrow[row];
      drow[q] = row * DL_LD;
    } else if (row < R + cnt) {
      srow[q] = Ab + (size_t)is[row - R] * nA;
      drow[q] = (JROWS + row - R) * DL_LD;
    }
  }
  auto stage = [&](int buf, int x0) {
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      if (drow[q] < 0) continue;
      T* dst = stg + (size_t)buf * STAGE + drow[q];
#pragma unroll
      for (int qx = 0; qx < QPR; ++qx) {
        const int x = x0 + 4 * qx;
        const bool ok = x < XN;
#pragma unroll
        for (int h = 0; h < CPQ; ++h) cp_async16(dst + 4 * qx + h * EPC, ok ? srow[q] + x + h * EPC : Ab, ok);
      }
    }
  };
  const int TR = (R + 3) / 4, TC = (cnt + 3) / 4, ntile = TR * TC;
  T acc[MAXT][16];
#pragma unroll
  for (int u = 0; u < MAXT; ++u)
#pragma unroll
    for (int e = 0; e < 16; ++e) acc[u][e] = T(0);
  // DL_STAGES - 1 chunks ahead; one commit group per chunk (empty past the end), one barrier per chunk: the
  // buffer restaged after the barrier of chunk ch held chunk ch - 1, which every thread has finished
  const int nch = (XN + DL_OC - 1) / DL_OC;
#pragma unroll
  for (int c = 0; c < DL_STAGES - 1; ++c) {
    if (c < nch) stage(c, c * DL_OC);
    cp_async_commit();
  }
  for (int ch = 0; ch < nch; ++ch) {
    cp_async_wait<DL_STAGES - 2>();
    __syncthreads();
    {
      const int nx = ch + DL_STAGES - 1;
      if (nx < nch) stage(nx % DL_STAGES, nx * DL_OC);
      cp_async_commit();
    }
    const T* Jb = stg + (size_t)(ch % DL_STAGES) * STAGE;
    const T* Ac = Jb + JROWS * DL_LD;
#pragma unroll
    for (int u = 0; u < MAXT; ++u) {
      const int t = tid + u * NT;
      if (t < ntile) {
        const int r0 = t / TC, k0 = t - r0 * TC;
#pragma unroll 2
        for (int qx = 0; qx < QPR; ++qx) {
          T a[4][4], b[4][4];
#pragma unroll
          for (int j = 0; j < 4; ++j) ld_quad(Jb + (r0 + TR * j) * DL_LD + 4 * qx, a[j]);
#pragma unroll
          for (int y = 0; y < 4; ++y) ld_quad(Ac + (k0 + TC * y) * DL_LD + 4 * qx, b[y]);
#pragma unroll
          for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int y = 0; y < 4; ++y)
#pragma unroll
              for (int o = 0; o < 4; ++o) acc[u][4 * j + y] += a[j][o] * b[y][o];
        }
      }
    }
  }
  cp_async_wait<0>();
  __syncthreads();  // every chunk consumed: the result tile overwrites the staging buffers
#pragma unroll
  for (int u = 0; u < MAXT; ++u) {
    const int t = tid + u * NT;
    if (t < ntile) {
      const int r0 = t / TC, k0 = t - r0 * TC;
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int y = 0; y < 4; ++y) {
          const int r = r0 + TR * j, k = k0 + TC * y;
          if (r < R && k < cnt) Bm[r * BLD + k] = acc[u][4 * j + y];
        }
    }
  }
  __syncthreads();
  // triplet term: sum_t sum_{k, k2} B[(k, t)][k2] * B[(k2, t)][k];  gradient: sum_k B[(k, t)][k]
  double tl = 0.0;
  const int nel = R * cnt;
  for (int e = tid; e < nel; e += blockDim.x) {
    const int rr = e / cnt, k2 = e - rr * cnt;
    const int k = rr / 3, t = rr - 3 * k;
    tl += (double)Bm[rr * BLD + k2] * (double)Bm[(3 * k2 + t) * BLD + k];
  }
  // tr(lap A A^-1) row m: sum_o lapA[m][o] Ainv[o][m]
  double tr = 0.0;
  for (int o = tid; o < n; o += blockDim.x)
    tr += (double)lapA[((size_t)w * n + m) * ldj + (long)d * n + o] * (double)Ab[(size_t)m * nA + sh + o];
  double v = tr - tl;
  v = warp_sum(v);
  __shared__ double rs[NT / 32];
  if ((tid & 31) == 0) rs[tid >> 5] = v;
  __syncthreads();
  if (tid == 0) {
    double sum = 0.0;
    for (int q = 0; q < NT / 32; ++q) sum += rs[q];
    atomicAdd(&lap[w * NDET + d], sum);
  }
  if (tid < 3) {
    double gsum = 0.0;  // kept in double: near a node |grad log psi|^2 is ~1e4 |E_loc|
    for (int k = 0; k < cnt; ++k) gsum += (double)Bm[(3 * k + tid) * BLD + k];
    grad[(((size_t)w * NDET + d) * n + m) * 3 + tid] = gsum;
  }
}

// One thread per 4 consecutive orbital columns of one electron (DN % 4 == 0, every plane 16-byte aligned).  env: the
// envelope carrier [G][5][DN] (value, Jacobian xyz, Laplacian), raw [G][DN], rjs: the raw orbitals' self Jacobian
// rows [G][3][DN] (written by the Jacobian contraction's epilogue).
__global__ void k_orb_lap(float* __restrict__ lapA, const float* __restrict__ env, const float* __restrict__ raw,
                          const float* __restrict__ rjs, long G, int DN) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x, nq = (long)DN / 4;
  if (q >= G * nq) return;
  const long g = q / nq;
  const int c = (int)(q - g * nq) * 4;
  const float* e = env + g * 5 * DN + c;
  const float* rj = rjs + g * 3 * DN + c;
  float4* out = reinterpret_cast<float4*>(lapA + g * DN + c);
  const float4 a = *out, ex = *reinterpret_cast<const float4*>(e), el = *reinterpret_cast<const float4*>(e + 4 * DN),
               rw = *reinterpret_cast<const float4*>(raw + g * DN + c);
  float4 v = make_float4(a.x * ex.x + el.x * rw.x, a.y * ex.y + el.y * rw.y, a.z * ex.z + el.z * rw.z,
                         a.w * ex.w + el.w * rw.w);
#pragma unroll
  for (int t = 0; t < 3; ++t) {
    const float4 r = *reinterpret_cast<const float4*>(rj + t * DN), ej = *reinterpret_cast<const float4*>(e + (1 + t) * DN);
    v.x += 2.f * r.x * ej.x; v.y += 2.f * r.y * ej.y; v.z += 2.f * r.z * ej.z; v.w += 2.f * r.w * ej.w;
  }
  *out = v;
}

template __global__ void k_env_coef<float, 1>(const float*, const float*, const float*, int, int, int, int, int,
                                              float*);
template __global__ void k_env_coef<float, 5>(const float*, const float*, const float*, int, int, int, int, int,
                                              float*);
template __global__ void k_env_coef<double, 1>(const double*, const float*, const double*, int, int, int, int,
                                               int, double*);
template __global__ void k_env_coef<double, 5>(const double*, const float*, const double*, int, int, int, int,
                                               int, double*);
template __global__ void k_gj_global<df64, float, float, false>(const float*, const float*, int, df64*, double*, double*, double*,
                                                                 float*, int32_t*);
template __global__ void k_gj_global<df64, float, float, true>(const float*, const float*, int, df64*, double*, double*, double*,
                                                                float*, int32_t*);
// FP64 elimination of FP64 orbital matrices with the inverse in FP32 (the refinement pass of the FP32 / mixed local
// energy, whose determinant Laplacian reads an FP32 inverse)
template __global__ void k_gj_global<double, double, float, true>(const double*, const double*, int, double*, double*, double*,
                                                                   double*, float*, int32_t*);
template __global__ void k_gj_global<double, double, double, true>(const double*, const double*, int, double*, double*, double*,
                                                                    double*, double*, int32_t*);
template __global__ void k_gj_global<double, double, double, false>(const double*, const double*, int, double*, double*, double*,
                                                                     double*, double*, int32_t*);
template __global__ void k_detlap<float, 128, 0, DL_CSPLIT>(Nbr, Layout, const float*, const float*, const float*,
                                                            double*, double*, int32_t*);
template __global__ void k_detlap<float, 256, DL_CSPLIT, DL_CMAX>(Nbr, Layout, const float*, const float*,
                                                                  const float*, double*, double*, int32_t*);
template __global__ void k_detlap<double, 256, 0, DL_CMAX>(Nbr, Layout, const double*, const double*,
                                                            const double*, double*, double*, int32_t*);

}  // namespace fire
