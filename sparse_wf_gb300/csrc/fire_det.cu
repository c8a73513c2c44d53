// fire_det.cu -- orbital envelopes, slogdet/inverse of the orbital matrices and the sparse
// determinant Laplacian.
//
//  k_env_coef   forward-Laplacian coefficients of exp(-softplus(sigma) |r - R|) per electron,
//               nucleus, determinant and envelope (EfficientIsotropicEnvelopes, envelopes.py:55-82);
//               a GEMM with pi then gives the envelope carrier [x, jac(3), lap] per orbital.
//  k_gauss_jordan  sign/log|det| and (optionally) the inverse of every orbital matrix, computed
//               in FP64 by a thread-block cluster: the n x n matrix is split by columns over the
//               cluster's CTAs and stays in their shared memory; the pivot column is read through
//               distributed shared memory.  Partial pivoting like jax.lax.linalg.lu, sign/log|det|
//               as slogdet_from_lu (model/utils.py:153-161), inverse as get_inverse_from_lu (144-150).
//  k_detlap     sparse_slogdet_with_fwd_lap (model/sparse_fwd_lap.py:294-319) restricted to the
//               triplets: for every dependency m, B = J[(i, m) rows] @ A^-1[:, k] for i, k in {m} + N(m)
//               gives d log det / d r_m = sum_i B[(i,m)][i] and the triplet term
//               -sum_xyz sum_{i,k} B[(i,m)][k] B[(k,m)][i]; the first Laplacian term tr(lap A A^-1) is
//               accumulated row by row.
#include <cooperative_groups.h>

#include "fire_internal.cuh"

namespace cg = cooperative_groups;

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

// Gauss-Jordan inversion / LU with partial pivoting.  grid = (CL, matrices), cluster = (CL, 1, 1).
// A: [matrices][lda-strided rows] with element (i, o) of matrix (w, d) at
//    A[((w * n + i) * NDET + d) * n + o]  (the orbital plane [G][D * n]).
// Outputs: logdet[w * NDET + d], sign[...] (double); Ainv[(w * NDET + d) * n * n + o * n + i] (if INV).
template <typename S, typename TI, typename TO, bool INV>
__global__ void __launch_bounds__(256) k_gauss_jordan(const TI* __restrict__ A, int n, int CL,
                                                      double* __restrict__ logdet, double* __restrict__ sign,
                                                      TO* __restrict__ Ainv, int32_t* status) {
  extern __shared__ __align__(16) unsigned char gj_smem[];
  cg::cluster_group cluster = cg::this_cluster();
  const int c = (int)cluster.block_rank();
  const int mat = blockIdx.y;
  const int w = mat / NDET, d = mat - w * NDET;
  const int wc = (n + CL - 1) / CL;
  const int j0 = c * wc, jn = max(0, min(wc, n - j0));
  S* a = reinterpret_cast<S*>(gj_smem);  // [n][wc]
  S* col = a + (size_t)n * wc;           // [n]
  S* rowk = col + n;                     // [wc]
  int* perm = reinterpret_cast<int*>(rowk + wc);  // [n]
  __shared__ S redv[8];
  __shared__ int redi[8];
  __shared__ int piv_s;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int e = tid; e < n * wc; e += blockDim.x) {
    const int i = e / wc, jl = e - i * wc;
    a[e] = jl < jn ? (S)A[((long)(w * n + i) * NDET + d) * n + j0 + jl] : S(0);
  }
  double ld = 0.0;
  int neg = 0;
  bool singular = false;
  for (int k = 0; k < n; ++k) {
    const int owner = k / wc, kl = k - owner * wc;
    cluster.sync();  // previous updates complete everywhere
    const S* ra = cluster.map_shared_rank(a, owner);
    for (int i = tid; i < n; i += blockDim.x) col[i] = ra[(size_t)i * wc + kl];
    __syncthreads();
    // pivot: first index of the max |col[i]|, i >= k
    S best = S(-1);
    int bi = n;
    for (int i = k + tid; i < n; i += blockDim.x) {
      const S v = fabs(col[i]);
      if (v > best) {
        best = v;
        bi = i;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const S ov = __shfl_xor_sync(0xffffffffu, best, o);
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
    if (tid == 0) {
      S bv = redv[0];
      int b = redi[0];
      for (int q = 1; q < (int)(blockDim.x >> 5); ++q)
        if (redv[q] > bv || (redv[q] == bv && redi[q] < b)) {
          bv = redv[q];
          b = redi[q];
        }
      piv_s = b < n ? b : k;
    }
    __syncthreads();
    const int p = piv_s;
    cluster.sync();  // everyone has read column k before the owner overwrites it
    const S pv = col[p];
    if (tid == 0) perm[k] = p;
    if (pv == S(0)) singular = true;
    ld += log(fabs((double)pv));
    if (pv < S(0)) neg ^= 1;
    if (p != k) neg ^= 1;
    // swap rows k, p (own columns) and entries of col
    if (p != k) {
      for (int jl = tid; jl < wc; jl += blockDim.x) {
        const S t = a[(size_t)k * wc + jl];
        a[(size_t)k * wc + jl] = a[(size_t)p * wc + jl];
        a[(size_t)p * wc + jl] = t;
      }
    }
    __syncthreads();
    if (tid == 0 && p != k) {
      const S t = col[k];
      col[k] = col[p];
      col[p] = t;
    }
    __syncthreads();
    const S ipv = pv != S(0) ? S(1) / pv : S(0);
    if (INV) {
      for (int jl = tid; jl < wc; jl += blockDim.x) rowk[jl] = a[(size_t)k * wc + jl] * ipv;
      __syncthreads();
      for (int e = tid; e < n * wc; e += blockDim.x) {
        const int i = e / wc, jl = e - i * wc;
        const bool is_k_col = (owner == c && jl == kl);
        if (i == k) {
          a[e] = is_k_col ? ipv : rowk[jl];
        } else {
          a[e] = is_k_col ? -col[i] * ipv : a[e] - col[i] * rowk[jl];
        }
      }
    } else {
      // LU only: trailing update of rows > k, global columns > k
      for (int e = tid; e < n * wc; e += blockDim.x) {
        const int i = e / wc, jl = e - i * wc;
        if (i > k && j0 + jl > k) a[e] -= col[i] * ipv * a[(size_t)k * wc + jl];
      }
    }
    __syncthreads();
  }
  if (c == 0 && tid == 0) {
    logdet[mat] = ld;
    sign[mat] = neg ? -1.0 : 1.0;
    if (singular) set_flag(status, FIRE_FLAG_SINGULAR);
  }
  if (INV) {
    // undo the row interchanges on the columns: final column jc holds working column src(jc)
    int* src = perm + n;  // [n] scratch after perm (allocated by the launcher)
    if (tid == 0) {
      for (int q = 0; q < n; ++q) src[q] = q;
      for (int k = n - 1; k >= 0; --k) {
        const int p = perm[k];
        if (p != k) {
          const int t = src[k];
          src[k] = src[p];
          src[p] = t;
        }
      }
    }
    cluster.sync();
    __syncthreads();
    TO* out = Ainv + (size_t)mat * n * n;
    for (int e = tid; e < n * jn; e += blockDim.x) {
      const int i = e / jn, jl = e - i * jn;
      const int jc = j0 + jl;
      const int sc = src[jc];
      const int ow = sc / wc;
      const S* rs = cluster.map_shared_rank(a, ow);
      out[(size_t)i * n + jc] = (TO)rs[(size_t)i * wc + (sc - ow * wc)];
    }
    cluster.sync();  // keep shared memory alive until all remote reads are done
  } else {
    cluster.sync();
  }
}

// Determinant Laplacian for one (walker, det, dependency m).  Jp: orbital Jacobian plane
// [3 * positions][NDET * n]; Ainv [W][NDET][n][n]; lapA [G][NDET * n].
// Outputs: grad [W][NDET][n][3] (+=), lap [W * NDET] (double, +=).
constexpr int DL_CMAX = 64;
template <typename T>
__global__ void __launch_bounds__(256) k_detlap(Nbr nb, Layout L, const T* __restrict__ Jp,
                                                const T* __restrict__ Ainv, const T* __restrict__ lapA,
                                                T* __restrict__ grad, double* __restrict__ lap, int32_t* status) {
  extern __shared__ __align__(16) unsigned char dl_smem[];
  const int n = nb.n;
  const int m = blockIdx.x, d = blockIdx.y, w = blockIdx.z;
  const int* rp = nb.rowptr + (size_t)w * (n + 1);
  if (rp[n] > nb.cap_p) return;
  const int cnt = rp[m + 1] - rp[m] + 1;
  if (cnt > DL_CMAX) {
    if (threadIdx.x == 0) set_flag(status, FIRE_FLAG_PAIR_OVERFLOW);
    return;
  }
  constexpr int OC = 32;
  T* Bm = reinterpret_cast<T*>(dl_smem);        // [3 * cnt][cnt + 1]
  T* Jt = Bm + 3 * DL_CMAX * (DL_CMAX + 1);      // [3 * cnt][OC + 1]
  T* At = Jt + 3 * DL_CMAX * (OC + 1);           // [OC][cnt + 1]
  __shared__ int qs[DL_CMAX], is[DL_CMAX];
  const int tid = threadIdx.x;
  const int off = L.pos_off[w];
  const int s0 = off + rp[m] + m;
  for (int k = tid; k < cnt; k += blockDim.x) {
    const int q = L.dep_pos[s0 + k];
    qs[k] = q;
    is[k] = L.pos_ctr[q] - w * n;
  }
  __syncthreads();
  const int nel = 3 * cnt * cnt;
  constexpr int MAXE = 3 * DL_CMAX * DL_CMAX / 256;
  T acc[MAXE];
#pragma unroll
  for (int u = 0; u < MAXE; ++u) acc[u] = T(0);
  const T* Ai = Ainv + ((size_t)w * NDET + d) * n * n;
  const long ldj = (long)NDET * n;
  for (int o0 = 0; o0 < n; o0 += OC) {
    const int oc = min(OC, n - o0);
    for (int e = tid; e < 3 * cnt * OC; e += blockDim.x) {
      const int rr = e / OC, o = e - rr * OC;
      const int k = rr / 3, t = rr - 3 * k;
      Jt[rr * (OC + 1) + o] = o < oc ? Jp[(3L * qs[k] + t) * ldj + (long)d * n + o0 + o] : T(0);
    }
    for (int e = tid; e < OC * cnt; e += blockDim.x) {
      const int o = e / cnt, k = e - o * cnt;
      At[o * (DL_CMAX + 1) + k] = o < oc ? Ai[(size_t)(o0 + o) * n + is[k]] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < MAXE; ++u) {
      const int e = tid + u * 256;
      if (e < nel) {
        const int rr = e / cnt, k2 = e - rr * cnt;
        T s = T(0);
#pragma unroll 8
        for (int o = 0; o < OC; ++o) s += Jt[rr * (OC + 1) + o] * At[o * (DL_CMAX + 1) + k2];
        acc[u] += s;
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < MAXE; ++u) {
    const int e = tid + u * 256;
    if (e < nel) {
      const int rr = e / cnt, k2 = e - rr * cnt;
      Bm[rr * (DL_CMAX + 1) + k2] = acc[u];
    }
  }
  __syncthreads();
  // gradient: sum_k B[(k, t)][k];  triplet term: sum_t sum_{k, k2} B[(k,t)][k2] * B[(k2,t)][k]
  double tl = 0.0;
  for (int e = tid; e < nel; e += blockDim.x) {
    const int rr = e / cnt, k2 = e - rr * cnt;
    const int k = rr / 3, t = rr - 3 * k;
    tl += (double)Bm[rr * (DL_CMAX + 1) + k2] * (double)Bm[(3 * k2 + t) * (DL_CMAX + 1) + k];
  }
  // tr(lap A A^-1) row m: sum_o lapA[m][o] Ainv[o][m]
  double tr = 0.0;
  for (int o = tid; o < n; o += blockDim.x)
    tr += (double)lapA[((size_t)w * n + m) * ldj + (long)d * n + o] * (double)Ai[(size_t)o * n + m];
  double v = tr - tl;
  v = warp_sum(v);
  __shared__ double rs[8];
  if ((tid & 31) == 0) rs[tid >> 5] = v;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int q = 0; q < 8; ++q) s += rs[q];
    atomicAdd(&lap[w * NDET + d], s);
  }
  if (tid < 3) {
    T gsum = T(0);
    for (int k = 0; k < cnt; ++k) gsum += Bm[(3 * k + tid) * (DL_CMAX + 1) + k];
    grad[(((size_t)w * NDET + d) * n + m) * 3 + tid] = gsum;
  }
}

template __global__ void k_env_coef<float, 1>(const float*, const float*, const float*, int, int, int, int, int,
                                              float*);
template __global__ void k_env_coef<float, 5>(const float*, const float*, const float*, int, int, int, int, int,
                                              float*);
template __global__ void k_env_coef<double, 1>(const double*, const float*, const double*, int, int, int, int,
                                               int, double*);
template __global__ void k_env_coef<double, 5>(const double*, const float*, const double*, int, int, int, int,
                                               int, double*);
template __global__ void k_gauss_jordan<double, float, float, true>(const float*, int, int, double*, double*,
                                                                    float*, int32_t*);
template __global__ void k_gauss_jordan<double, float, float, false>(const float*, int, int, double*, double*,
                                                                     float*, int32_t*);
template __global__ void k_gauss_jordan<float, float, float, false>(const float*, int, int, double*, double*,
                                                                    float*, int32_t*);
template __global__ void k_gauss_jordan<double, double, double, true>(const double*, int, int, double*,
                                                                      double*, double*, int32_t*);
template __global__ void k_gauss_jordan<double, double, double, false>(const double*, int, int, double*,
                                                                       double*, double*, int32_t*);
template __global__ void k_detlap<float>(Nbr, Layout, const float*, const float*, const float*, float*, double*,
                                         int32_t*);
template __global__ void k_detlap<double>(Nbr, Layout, const double*, const double*, const double*, double*,
                                          double*, int32_t*);

}  // namespace fire
