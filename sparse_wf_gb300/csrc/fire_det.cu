// fire_det.cu -- orbital envelopes, slogdet/inverse of the orbital matrices and the sparse
// determinant Laplacian.
//
//  k_env_coef   forward-Laplacian coefficients of exp(-softplus(sigma) |r - R|) per electron,
//               nucleus, determinant and envelope (EfficientIsotropicEnvelopes, envelopes.py:55-82);
//               a GEMM with pi then gives the envelope carrier [x, jac(3), lap] per orbital.
//  k_gauss_jordan  sign/log|det| and (optionally) the inverse of every orbital matrix, computed
//               in double precision (native FP64 in the FP64 build, double-FP32 "df64" with a 48-bit
//               significand in the FP32 and mixed paths, fire_df64.cuh) by a thread-block cluster: the n x n matrix is split by columns over the
//               cluster's CTAs and stays in their shared memory; the pivot column is read through
//               distributed shared memory.  Partial pivoting like jax.lax.linalg.lu, sign/log|det|
//               as slogdet_from_lu (model/utils.py:153-161), inverse as get_inverse_from_lu (144-150).
//  k_detlap     sparse_slogdet_with_fwd_lap (model/sparse_fwd_lap.py:294-319) restricted to the
//               triplets: for every dependency m, B = J[(i, m) rows] @ A^-1[:, k] for i, k in {m} + N(m)
//               gives d log det / d r_m = sum_i B[(i,m)][i] and the triplet term
//               -sum_xyz sum_{i,k} B[(i,m)][k] B[(k,m)][i]; the first Laplacian term tr(lap A A^-1) is
//               accumulated row by row.
#include <cooperative_groups.h>

#include "fire_df64.cuh"
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

// Gauss-Jordan inversion / LU with partial pivoting.  grid = (CL, matrices), cluster = (CL, 1, 1),
// 1024 threads (many warps hide the dependent double-FP32 operation chains); thread (tx, ty) = (tid % wc, tid / wc) owns column tx of this CTA's slice and rows
// ty, ty + ty_n, ...
// Look-ahead: during step k the CTA that owns column k + 1 computes that column's post-step values first
// and writes them into every CTA's colbuf[(k + 1) % 3] (distributed shared memory), then all threads
// arrive on the cluster barrier; step k + 1 starts with the matching wait, so each step has a single
// split cluster barrier and the pivot column is read from local shared memory.  Three buffers: the one
// rewritten during step k was last read during step k - 2, which every CTA finished before arriving in
// step k - 1 (the arrival the writer waited for).
// A: element (i, o) of matrix (w, d) at A[((w * n + i) * NDET + d) * n + o]  (the orbital plane [G][D * n]).
// Outputs: logdet[w * NDET + d], sign[...] (double); Ainv[(w * NDET + d) * n * n + o * n + i] (if INV).
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

constexpr int GJ_THREADS = 1024;
template <typename S, typename TI, typename TO, bool INV>
__global__ void __launch_bounds__(GJ_THREADS, 1) k_gauss_jordan(const TI* __restrict__ A, int n, int CL,
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
  S* colbuf = a + (size_t)n * wc;        // [3][n] pivot columns (published by their owner)
  S* rowk = colbuf + 3 * n;              // [wc]
  int* perm = reinterpret_cast<int*>(rowk + wc);  // [n] (+ [n] scratch)
  __shared__ S redv[32];
  __shared__ int redi[32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nwarp = blockDim.x >> 5;
  const int ty_n = max(1, (int)blockDim.x / wc);
  const int tx = tid % wc, ty = tid / wc;
  const bool upd = ty < ty_n && tx < jn;
  for (int e = tid; e < n * wc; e += blockDim.x) {
    const int i = e / wc, jl = e - i * wc;
    a[e] = jl < jn ? (S)A[((long)(w * n + i) * NDET + d) * n + j0 + jl] : S(0);
  }
  cluster.sync();  // every CTA of the cluster is running and has its slice
  if (c == 0) {     // publish column 0
    for (int i = tid; i < n; i += blockDim.x) {
      const S v = a[(size_t)i * wc];
      for (int r = 0; r < CL; ++r) cluster.map_shared_rank(colbuf, r)[i] = v;
    }
  }
  __syncthreads();
  cluster_arrive();
  double ld = 0.0;
  int neg = 0;
  bool singular = false;
  // Rows k and p of step k are not written in place during step k: their new values wait in registers
  // (one designated thread per column, and the look-ahead threads for column k + 1) and are stored at the
  // start of step k + 1.  Every read of those rows in step k happens before the thread's cluster arrive,
  // and the stores come after the next cluster wait, so one cluster barrier and one CTA barrier per step
  // order all shared-memory traffic.
  int pk = -1, pp = -1;                 // pending rows (designated update thread, column tx)
  S uk = S(0), up = S(0);
  int la_row = -1, la_col = 0;          // pending look-ahead element
  S la_val = S(0);
  for (int k = 0; k < n; ++k) {
    const int owner = k / wc, kl = k - owner * wc;
    cluster_wait();  // column k has been published into colbuf[k % 3]
    const S* col = colbuf + (k % 3) * n;
    S best = S(-1);
    int bi = n;
    for (int i = k + tid; i < n; i += blockDim.x) {
      const S v = absv(col[i]);
      if (v > best) {
        best = v;
        bi = i;
      }
    }
    if (pk >= 0) {  // rows k - 1 and p(k - 1) of the previous step
      a[(size_t)pk * wc + tx] = uk;
      if (pp != pk) a[(size_t)pp * wc + tx] = up;
      pk = -1;
    }
    if (la_row >= 0) {
      a[(size_t)la_row * wc + la_col] = la_val;
      la_row = -1;
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
    // every warp reduces the per-warp candidates itself (no second barrier)
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
    const S pv = col[p];
    const S ipv = pv != S(0) ? S(1) / pv : S(0);
    const S ck = col[k], cp = col[p];  // pivot-column entries; rows k and p are interchanged
    // look-ahead: the owner of column k + 1 computes and publishes its post-step-k values (and keeps them)
    const int owner1 = (k + 1) / wc, kl1 = (k + 1) - owner1 * wc;
    const bool la = k + 1 < n && owner1 == c;
    if (la) {
      const S rk = (INV ? a[(size_t)p * wc + kl1] * ipv : a[(size_t)p * wc + kl1]);
      S* nb = colbuf + ((k + 1) % 3) * n;
      for (int i = tid; i < n; i += blockDim.x) {
        S v;
        const int src = i == k ? p : (i == p ? k : i);
        const S ci = i == k ? cp : (i == p ? ck : col[i]);
        if (INV) v = i == k ? rk : a[(size_t)src * wc + kl1] - ci * rk;
        else v = i > k ? a[(size_t)src * wc + kl1] - ci * ipv * rk : a[(size_t)src * wc + kl1];
        for (int r = 0; r < CL; ++r) cluster.map_shared_rank(nb, r)[i] = v;
        if (i == k || i == p) {
          la_row = i;
          la_col = kl1;
          la_val = v;
        } else {
          a[(size_t)i * wc + kl1] = v;
        }
      }
    }
    // rows p and k of this thread's column, read before the arrive
    const bool mycol = upd && !(la && tx == kl1);
    const S vp = mycol ? a[(size_t)p * wc + tx] : S(0);
    const S vk = (mycol && ty == 0) ? a[(size_t)k * wc + tx] : S(0);
    if (k + 1 < n) cluster_arrive();  // releases the published column
    if (tid == 0) {  // one thread keeps the permutation, sign and log|det|
      perm[k] = p;
      if (pv == S(0)) singular = true;
      ld += ::log(::fabs((double)pv));
      if (pv < S(0)) neg ^= 1;
      if (p != k) neg ^= 1;
    }
    if (mycol) {
      if (INV) {
        const bool kcol = owner == c && tx == kl;
        const S rj = vp * ipv;
        for (int i = ty; i < n; i += ty_n) {
          if (i == k || i == p) continue;
          const S ci = col[i];
          S* e = a + (size_t)i * wc + tx;
          *e = kcol ? -ci * ipv : *e - ci * rj;
        }
        if (ty == 0) {
          uk = kcol ? ipv : rj;
          up = kcol ? -ck * ipv : vk - ck * rj;
          pk = k;
          pp = p;
        }
      } else {
        if (j0 + tx > k) {
          const S rj = vp;
          for (int i = k + 1 + ty; i < n; i += ty_n) {
            if (i == p) continue;
            a[(size_t)i * wc + tx] -= col[i] * ipv * rj;
          }
          if (ty == 0) {
            uk = vp;
            up = vk - ck * ipv * vp;
            pk = k;
            pp = p;
          }
        } else if (ty == 0) {  // columns left of the pivot: rows k and p are only interchanged
          uk = vp;
          up = vk;
          pk = k;
          pp = p;
        }
      }
    }
  }
  if (pk >= 0) {
    a[(size_t)pk * wc + tx] = uk;
    if (pp != pk) a[(size_t)pp * wc + tx] = up;
  }
  if (la_row >= 0) a[(size_t)la_row * wc + la_col] = la_val;
  __syncthreads();
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
// Outputs: grad [W][NDET][n][3], lap [W * NDET] (double, +=).
// B = J[(i, m) rows] (3c x n) @ Ainv[:, {i}] (n x c) is computed with 2 x 4 register tiles from K-chunks
// staged (J transposed) in shared memory; the next chunk is prefetched into registers while the current
// one is multiplied.  The result tile reuses the staging memory.
constexpr int DL_CMAX = 64, DL_RP = 196, DL_OC = 32;
constexpr int DL_JPT = 3 * DL_CMAX * DL_OC / 256;  // J chunk elements per thread (24)
constexpr int DL_APT = DL_OC * DL_CMAX / 256;      // Ainv chunk elements per thread (8)
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
  T* Jt = reinterpret_cast<T*>(dl_smem);  // [DL_OC][DL_RP]   J chunk, transposed
  T* At = Jt + DL_OC * DL_RP;             // [DL_OC][DL_CMAX] Ainv chunk
  T* Bm = reinterpret_cast<T*>(dl_smem);  // [3 * DL_CMAX][DL_CMAX + 1] after the main loop
  __shared__ long qrow[3 * DL_CMAX];      // J plane row of local row rr
  __shared__ int is[DL_CMAX];
  const int tid = threadIdx.x;
  const int off = L.pos_off[w];
  const int s0 = off + rp[m] + m;
  const long ldj = (long)NDET * n;
  for (int k = tid; k < cnt; k += blockDim.x) {
    const int q = L.dep_pos[s0 + k];
    is[k] = L.pos_ctr[q] - w * n;
    for (int t = 0; t < 3; ++t) qrow[3 * k + t] = (3L * q + t) * ldj + (long)d * n;
  }
  __syncthreads();
  const int R = 3 * cnt;
  const int rt = (R + 1) / 2, ct = (cnt + 3) / 4, ntile = rt * ct;
  constexpr int MAXT = (3 * DL_CMAX / 2) * (DL_CMAX / 4) / 256;  // 6
  T acc[MAXT][8];
#pragma unroll
  for (int u = 0; u < MAXT; ++u)
#pragma unroll
    for (int e = 0; e < 8; ++e) acc[u][e] = T(0);
  const T* Ai = Ainv + ((size_t)w * NDET + d) * n * n;
  T jr[DL_JPT], ar[DL_APT];
  auto fetch = [&](int o0) {
#pragma unroll
    for (int u = 0; u < DL_JPT; ++u) {
      const int e = tid + 256 * u;
      const int rr = e / DL_OC, o = e - rr * DL_OC;
      jr[u] = (rr < R && o0 + o < n) ? Jp[qrow[rr] + o0 + o] : T(0);
    }
#pragma unroll
    for (int u = 0; u < DL_APT; ++u) {
      const int e = tid + 256 * u;
      const int o = e / DL_CMAX, k = e - o * DL_CMAX;
      ar[u] = (k < cnt && o0 + o < n) ? Ai[(size_t)(o0 + o) * n + is[k]] : T(0);
    }
  };
  fetch(0);
  for (int o0 = 0; o0 < n; o0 += DL_OC) {
#pragma unroll
    for (int u = 0; u < DL_JPT; ++u) {
      const int e = tid + 256 * u;
      const int rr = e / DL_OC, o = e - rr * DL_OC;
      Jt[o * DL_RP + rr] = jr[u];
    }
#pragma unroll
    for (int u = 0; u < DL_APT; ++u) At[tid + 256 * u] = ar[u];
    __syncthreads();
    if (o0 + DL_OC < n) fetch(o0 + DL_OC);
#pragma unroll
    for (int u = 0; u < MAXT; ++u) {
      const int tile = tid + u * 256;
      if (tile < ntile) {
        const int r0 = (tile / ct) * 2, c0 = (tile % ct) * 4;
#pragma unroll 8
        for (int o = 0; o < DL_OC; ++o) {
          const T a0 = Jt[o * DL_RP + r0], a1 = Jt[o * DL_RP + r0 + 1];
          T b[4];
#pragma unroll
          for (int y = 0; y < 4; ++y) b[y] = At[o * DL_CMAX + c0 + y];
#pragma unroll
          for (int y = 0; y < 4; ++y) {
            acc[u][y] += a0 * b[y];
            acc[u][4 + y] += a1 * b[y];
          }
        }
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < MAXT; ++u) {
    const int tile = tid + u * 256;
    if (tile < ntile) {
      const int r0 = (tile / ct) * 2, c0 = (tile % ct) * 4;
#pragma unroll
      for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y)
          if (r0 + x < R && c0 + y < cnt) Bm[(r0 + x) * (DL_CMAX + 1) + c0 + y] = acc[u][4 * x + y];
    }
  }
  __syncthreads();
  // triplet term: sum_t sum_{k, k2} B[(k, t)][k2] * B[(k2, t)][k];  gradient: sum_k B[(k, t)][k]
  double tl = 0.0;
  const int nel = R * cnt;
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
    double sum = 0.0;
    for (int q = 0; q < 8; ++q) sum += rs[q];
    atomicAdd(&lap[w * NDET + d], sum);
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
template __global__ void k_gauss_jordan<df64, float, float, true>(const float*, int, int, double*, double*, float*,
                                                                  int32_t*);
template __global__ void k_gauss_jordan<df64, float, float, false>(const float*, int, int, double*, double*, float*,
                                                                   int32_t*);
template __global__ void k_gauss_jordan<double, double, double, true>(const double*, int, int, double*,
                                                                      double*, double*, int32_t*);
template __global__ void k_gauss_jordan<double, double, double, false>(const double*, int, int, double*,
                                                                       double*, double*, int32_t*);
template __global__ void k_detlap<float>(Nbr, Layout, const float*, const float*, const float*, float*, double*,
                                         int32_t*);
template __global__ void k_detlap<double>(Nbr, Layout, const double*, const double*, const double*, double*,
                                          double*, int32_t*);

}  // namespace fire
