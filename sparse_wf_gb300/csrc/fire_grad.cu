// fire_grad.cu -- per-walker gradient of log|psi| with respect to every parameter: reverse mode through the value
// path (MoonLikeWaveFunction.signed, model/wave_function.py:183-198).  Its rows are the Jacobian that the dense
// SPRING preconditioner contracts: jax.grad of log_p vmapped over the walkers (preconditioner.py:185-191),
// called from the optimisation step (update.py:177-191).
//
// The forward pass runs again here and keeps in the workspace what the reverse pass needs: the filter rows of every
// e-n edge and e-e pair, the pre-activations of every SiLU, the orbital rows, envelopes and matrices with their
// inverses.  The reverse pass then walks the stages backwards:
//   head         logsumexp weights of the determinants, Jastrow scalars (scales, biases, cusp);
//   readout      attention readout MLP 512 -> 256 -> 256 -> 2 and the spin sums of the attention values;
//   Jastrow      attention queries / values and the MLP Jastrow rows;
//   determinant  d log|det A_d| / d A_d = A_d^-T (the Gauss-Jordan inverse), through the orbital rows and the
//                isotropic envelopes (model/envelopes.py:55-82) to their weights, pi and sigma;
//   update MLP   two SiLU layers between the normalisation scales;
//   messages     the e-e pairs' Gamma * silu(e + m_ct + m_nb) (new_sparse_model.py:83-131), their filters and
//                the cutoff parameter;
//   ElecInit     Dense 1280, SiLU, GLU, LayerNorm and the e-n edges with the per-nucleus filter parameters.
// Dense layers are row-major GEMMs on the CUDA cores (gk_mm).  Every weight gradient is a per-walker reduction over
// that walker's rows (gk_wgrad: X^T Y and the column sums of Y for a bias), written straight into the walker's
// gradient row, which has the layout of the parameter blob (fire_param_layout).
//
// Rows: "electron order" g = w n + i; "spin-major" order puts every walker's spin-up electrons first,
// sm(w, i) = w n_up + i (i < n_up) and W n_up + w n_dn + i - n_up (i >= n_up), so that the spin-resolved layers
// (orbitals, envelopes) are single GEMMs per spin.
#include <algorithm>
#include <cstring>
#include <type_traits>

#include "fire_df64.cuh"
#include "fire_internal.cuh"
#include "fire_kernels.cuh"

namespace fire {
namespace {

constexpr int ENW = 80;  // e-n edge row: feat 0-4 | pre 4-20 | envv 20-52 | dirf 52-60 | ew 60-68 | scaled 68-72 | beta 72-80
constexpr int PRW = 84;  // e-e pair row: feat 0-4 | pre 4-20 | envv 20-36 | dirf 36-44 | ew 44-52 | tag 52 |
                         // beta (same) 56-64 | beta (diff) 64-72 | [scaled, 1] (same) 72-77 | [scaled, 1] (diff) 77-82
constexpr int PX = 74, PY = 49;  // pair small-filter reduction rows: X = per tag [s 16 | envv 16 | feat 4 | 1], Y below
constexpr int EX = 49, EY = 16;  // e-n shared-filter reduction rows: X = [s 16 | envv 32 | 1], Y = [ddirf 8 | dew 8]
constexpr int EN2 = 48;          // e-n per-nucleus rows: dpre 16 | dscale 32

inline unsigned nb_(long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

__host__ __device__ inline long sm_row(int w, int i, int Wc, int nu, int nd) {
  return i < nu ? (long)w * nu + i : (long)Wc * nu + (long)w * nd + (i - nu);
}

// ------------------------------------------------------------------------------------------ GEMMs
// C[M, N] (ldc) = A[M, K] (lda) op(B) (+ bias) (+ C when acc); op(B) = B [K, N] (ldb), or with BT the transpose of
// B [N, K] (ldb).  64 x 64 tiles, 16-deep k steps, 256 threads with 4 x 4 outputs each; every load bounds-checked.
template <typename T, bool BT>
__global__ void __launch_bounds__(256) gk_mm(long M, int N, int K, const T* __restrict__ A, long lda,
                                             const T* __restrict__ B, long ldb, const T* __restrict__ bias,
                                             T* __restrict__ C, long ldc, int acc) {
  __shared__ T sA[16][65];
  __shared__ T sB[16][65];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long m0 = (long)blockIdx.x * 64;
  const int n0 = blockIdx.y * 64;
  T c[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) c[a][b] = T(0);
  for (int k0 = 0; k0 < K; k0 += 16) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = threadIdx.x + 256 * q, rr = idx >> 4, kk = idx & 15;
      const long m = m0 + rr;
      const int k = k0 + kk;
      sA[kk][rr] = (m < M && k < K) ? A[m * lda + k] : T(0);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int idx = threadIdx.x + 256 * q;
      if (!BT) {
        const int kk = idx >> 6, nn = idx & 63, k = k0 + kk, nc = n0 + nn;
        sB[kk][nn] = (k < K && nc < N) ? B[(long)k * ldb + nc] : T(0);
      } else {
        const int nn = idx >> 4, kk = idx & 15, k = k0 + kk, nc = n0 + nn;
        sB[kk][nn] = (k < K && nc < N) ? B[(long)nc * ldb + k] : T(0);
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        a[t] = sA[kk][ty + 16 * t];
        b[t] = sB[kk][tx + 16 * t];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) c[u][v] += a[u] * b[v];
    }
    __syncthreads();
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const long m = m0 + ty + 16 * u;
    if (m >= M) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int nc = n0 + tx + 16 * v;
      if (nc >= N) continue;
      T val = c[u][v];
      if (bias) val += bias[nc];
      if (acc) val += C[m * ldc + nc];
      C[m * ldc + nc] = val;
    }
  }
}

// Rows of walker w: base + w * wstride + [0, rows).
struct Seg {
  long base, wstride;
  int rows;
};
template <typename T>
struct WgP {
  const T* X;
  long ldx;
  const T* Y;
  long ldy;
  Seg s[2];  // second segment: rows = 0 when unused
  int K, N;
  T* out;    // walker w's gradient row: out + w * ldw; element (k, n) at (k / grp) * grp_stride + (k % grp) * ldo + n
  long ldw, ldo, grp_stride;
  int grp;
  T* bias;   // optional: column sums of Y at bias + w * ldw + n
};

// Per-walker X^T Y (K x N) over the walker's rows, with the column sums of Y as an extra row when bias is set.
// Grid (N tiles, K tiles, walkers); each output element is written by one thread (deterministic).
template <typename T>
__global__ void __launch_bounds__(256) gk_wgrad(WgP<T> p) {
  __shared__ T sX[16][65];
  __shared__ T sY[16][65];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int n0 = blockIdx.x * 64, k0 = blockIdx.y * 64, w = blockIdx.z;
  const int Ke = p.K + (p.bias ? 1 : 0);
  T c[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) c[a][b] = T(0);
#pragma unroll
  for (int sg = 0; sg < 2; ++sg) {
    const int rows = p.s[sg].rows;
    const long rb = p.s[sg].base + (long)w * p.s[sg].wstride;
    for (int r0 = 0; r0 < rows; r0 += 16) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int idx = threadIdx.x + 256 * q, rr = idx >> 6, cc = idx & 63;
        const int r = r0 + rr, k = k0 + cc, nc = n0 + cc;
        T xv = T(0), yv = T(0);
        if (r < rows) {
          if (k < p.K) xv = p.X[(rb + r) * p.ldx + k];
          else if (k == p.K && p.bias) xv = T(1);
          if (nc < p.N) yv = p.Y[(rb + r) * p.ldy + nc];
        }
        sX[rr][cc] = xv;
        sY[rr][cc] = yv;
      }
      __syncthreads();
#pragma unroll
      for (int rr = 0; rr < 16; ++rr) {
        T a[4], b[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          a[t] = sX[rr][ty + 16 * t];
          b[t] = sY[rr][tx + 16 * t];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) c[u][v] += a[u] * b[v];
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int k = k0 + ty + 16 * u;
    if (k >= Ke) continue;
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int nc = n0 + tx + 16 * v;
      if (nc >= p.N) continue;
      if (k < p.K)
        p.out[(long)w * p.ldw + (long)(k / p.grp) * p.grp_stride + (long)(k % p.grp) * p.ldo + nc] = c[u][v];
      else
        p.bias[(long)w * p.ldw + nc] = c[u][v];
    }
  }
}

// The same reduction for K + (bias ? 1 : 0) <= 16 over many rows (the edge and pair filters' 4- to 16-row weights):
// one CTA per 64 columns and walker, 4 row groups of 64 threads; each thread keeps its column's K sums in registers
// (the X row is a broadcast load, the Y row a coalesced one) and the row groups are summed through shared memory.
template <typename T>
__global__ void __launch_bounds__(256) gk_wgrad_skinny(WgP<T> p) {
  constexpr int KS = 16;
  __shared__ T red[3][KS][64];
  const int c = threadIdx.x & 63, rg = threadIdx.x >> 6;
  const int n0 = blockIdx.x * 64, w = blockIdx.z, nc = n0 + c;
  T acc[KS];
#pragma unroll
  for (int k = 0; k < KS; ++k) acc[k] = T(0);
  if (nc < p.N) {
#pragma unroll
    for (int sg = 0; sg < 2; ++sg) {
      const long rb = p.s[sg].base + (long)w * p.s[sg].wstride;
      for (int r = rg; r < p.s[sg].rows; r += 4) {
        const T* x = p.X + (rb + r) * p.ldx;
        const T y = p.Y[(rb + r) * p.ldy + nc];
#pragma unroll
        for (int k = 0; k < KS; ++k) {
          const T xv = k < p.K ? x[k] : (k == p.K && p.bias ? T(1) : T(0));
          acc[k] += xv * y;
        }
      }
    }
  }
  if (rg > 0) {
#pragma unroll
    for (int k = 0; k < KS; ++k) red[rg - 1][k][c] = acc[k];
  }
  __syncthreads();
  if (rg > 0 || nc >= p.N) return;
#pragma unroll
  for (int k = 0; k < KS; ++k) {
    const T v = acc[k] + red[0][k][c] + red[1][k][c] + red[2][k][c];
    if (k < p.K)
      p.out[(long)w * p.ldw + (long)(k / p.grp) * p.grp_stride + (long)(k % p.grp) * p.ldo + nc] = v;
    else if (k == p.K && p.bias)
      p.bias[(long)w * p.ldw + nc] = v;
  }
}

// ------------------------------------------------------------------------------------------ elementwise
template <typename T>
__global__ void gk_silu_fwd(const T* __restrict__ z, T* __restrict__ a, long cnt) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cnt) a[i] = silu(z[i]);
}
// dz = da * silu'(z) (in place allowed)
template <typename T>
__global__ void gk_dsilu(const T* da, const T* __restrict__ z, T* dz, long cnt) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  T y, d1, d2;
  silu3(z[i], y, d1, d2);
  dz[i] = da[i] * d1;
}
template <typename T>
__global__ void gk_scale(const T* __restrict__ x, const T* __restrict__ s, T* __restrict__ y, long cnt) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cnt) y[i] = x[i] * s[0];
}

// ------------------------------------------------------------------------------------------ ElecInit forward
// One thread per e-n edge row (g, k), k < en_cnt[g]: the PairwiseFilter (model/utils.py:393-433) with the nucleus's
// own kernel, bias and scales (ElecNucEdge, new_sparse_model.py:139-158), the log-scaled features; inv[g][J] = k.
template <typename T>
__global__ void gk_en_fwd(const T* __restrict__ r, const float* __restrict__ R, Nbr nb, Weights<T> W, T inv_c1,
                          T* __restrict__ enr, int* __restrict__ inv) {
  const long row = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int E = nb.cap_nuc;
  if (row >= (long)nb.W * nb.n * E) return;
  const long g = row / E;
  const int k = (int)(row - g * E);
  if (k >= nb.en_cnt[g]) return;
  const int J = nb.en_idx[g * E + k];
  inv[g * nb.N + J] = k;
  const T diff[3] = {r[3 * g] - (T)R[3 * J], r[3 * g + 1] - (T)R[3 * J + 1], r[3 * g + 2] - (T)R[3 * J + 2]};
  const T d = dsqrt(diff[0] * diff[0] + diff[1] * diff[1] + diff[2] * diff[2]);
  const T feat[4] = {d, diff[0], diff[1], diff[2]};
  T* o = enr + row * ENW;
  const T* Kj = W.w[FIRE_P_EN_KERNEL] + (long)J * 4 * F0;
  const T* bj = W.w[FIRE_P_EN_BIAS] + (long)J * F0;
  T s[F0];
#pragma unroll
  for (int l = 0; l < F0; ++l) {
    T pre = bj[l];
#pragma unroll
    for (int q = 0; q < 4; ++q) pre += feat[q] * Kj[q * F0 + l];
    o[4 + l] = pre;
    s[l] = silu(pre);
  }
  const T* dW = W.w[FIRE_P_EI_DIR_W];
  const T* db = W.w[FIRE_P_EI_DIR_B];
  const T* eW = W.w[FIRE_P_EI_ENV_W];
  const T* isc = W.w[PR_EN_INVSCALE] + (long)J * NENV_EN;
  const T cut = cutoff_val(d * inv_c1);
  T ew[F1];
#pragma unroll
  for (int c = 0; c < F1; ++c) ew[c] = T(0);
  for (int m = 0; m < NENV_EN; ++m) {
    const T u = d * isc[m];
    const T ev = dexp(-u * u) * cut;
    o[20 + m] = ev;
#pragma unroll
    for (int c = 0; c < F1; ++c) ew[c] += ev * eW[m * F1 + c];
  }
#pragma unroll
  for (int c = 0; c < F1; ++c) {
    T df = db[c];
#pragma unroll
    for (int l = 0; l < F0; ++l) df += s[l] * dW[l * F1 + c];
    o[52 + c] = df;
    o[60 + c] = ew[c];
    o[72 + c] = df * ew[c];
  }
  const T lp = dlog1p(d);
  o[68] = lp;
#pragma unroll
  for (int q = 0; q < 3; ++q) o[69 + q] = diff[q] / d * lp;
#pragma unroll
  for (int q = 0; q < 4; ++q) o[q] = feat[q];
}

// One CTA (thread = feature) per electron: h = sum_J Gamma_J * e_J, then LayerNorm (eps 1e-6); keeps x-hat and 1/sigma.
template <typename T>
__global__ void __launch_bounds__(256) gk_en_sum(Nbr nb, Weights<T> W, const T* __restrict__ enr, T* __restrict__ h1,
                                                 T* __restrict__ xhat, T* __restrict__ rstd) {
  __shared__ T red[32];
  const long g = blockIdx.x;
  const int f = threadIdx.x, E = nb.cap_nuc;
  const int ne = nb.en_cnt[g];
  T wg[F1], we[4];
#pragma unroll
  for (int c = 0; c < F1; ++c) wg[c] = W.w[FIRE_P_EI_GAMMA_W][c * F + f];
#pragma unroll
  for (int q = 0; q < 4; ++q) we[q] = W.w[FIRE_P_EI_EDGE_W][q * F + f];
  const T* ne_emb = W.w[FIRE_P_EN_NUC_EMB];
  T hs = T(0);
  for (int k = 0; k < ne; ++k) {
    const T* e = enr + (g * E + k) * ENW;
    const int J = nb.en_idx[g * E + k];
    T gm = T(0), ed = ne_emb[(long)J * F + f];
#pragma unroll
    for (int c = 0; c < F1; ++c) gm += e[72 + c] * wg[c];
#pragma unroll
    for (int q = 0; q < 4; ++q) ed += e[68 + q] * we[q];
    hs += gm * ed;
  }
  T v1[1] = {hs};
  block_sum<T, 1>(v1, red);
  const T c = hs - v1[0] / T(F);
  T v2[1] = {c * c};
  block_sum<T, 1>(v2, red);
  const T rs = T(1) / dsqrt(v2[0] / T(F) + T(1e-6));
  const T xh = c * rs;
  xhat[g * F + f] = xh;
  h1[g * F + f] = xh * W.w[FIRE_P_EI_LN_SCALE][f] + W.w[FIRE_P_EI_LN_BIAS][f];
  if (f == 0) rstd[g] = rs;
}

template <typename T>
__global__ void gk_glu_fwd(const T* __restrict__ gb, T* __restrict__ h2, long G) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= G * F) return;
  const long g = i / F;
  const int f = (int)(i - g * F);
  h2[i] = gb[g * 2 * F + f] * silu(gb[g * 2 * F + F + f]);
}

// ------------------------------------------------------------------------------------------ e-e pairs forward
__device__ __forceinline__ int pair_center(const int* rp, int n, int p) {
  int lo = 0, hi = n;  // last i with rp[i] <= p
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (rp[mid] <= p) lo = mid; else hi = mid;
  }
  return lo;
}

// One thread per pair slot (w, p), p < P_w: the ElecElecEdges filter (new_sparse_model.py:161-187) of the pair's tag
// (same / different spin) with the cutoff cutoff * sigmoid(cutoff_param).
template <typename T>
__global__ void gk_pair_fwd(const T* __restrict__ r, Nbr nb, Weights<T> W, T* __restrict__ prr) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int cp = nb.cap_p, n = nb.n;
  if (idx >= (long)nb.W * cp) return;
  const int w = (int)(idx / cp), p = (int)(idx - (long)w * cp);
  const int* rp = nb.rowptr + (long)w * (n + 1);
  const int P = rp[n];
  if (P > cp || p >= P) return;
  const int i = pair_center(rp, n, p);
  const int j = nb.nbr[(long)w * cp + p];
  const int tag = ((i < nb.n_up) == (j < nb.n_up)) ? 0 : 1;
  const T* Kt = W.w[tag == 0 ? FIRE_P_EESAME_KERNEL : FIRE_P_EEDIFF_KERNEL];
  const T* bt = W.w[tag == 0 ? FIRE_P_EESAME_BIAS : FIRE_P_EEDIFF_BIAS];
  const T* dW = W.w[tag == 0 ? FIRE_P_EESAME_DIR_W : FIRE_P_EEDIFF_DIR_W];
  const T* db = W.w[tag == 0 ? FIRE_P_EESAME_DIR_B : FIRE_P_EEDIFF_DIR_B];
  const T* eW = W.w[tag == 0 ? FIRE_P_EESAME_ENV_W : FIRE_P_EEDIFF_ENV_W];
  const T* isc = W.w[tag == 0 ? PR_EESAME_INVSCALE : PR_EEDIFF_INVSCALE];
  const T inv_c = T(1) / W.w[PR_SCALARS][0];
  const long gi = (long)w * n + i, gj = (long)w * n + j;
  const T diff[3] = {r[3 * gi] - r[3 * gj], r[3 * gi + 1] - r[3 * gj + 1], r[3 * gi + 2] - r[3 * gj + 2]};
  const T d = dsqrt(diff[0] * diff[0] + diff[1] * diff[1] + diff[2] * diff[2]);
  const T feat[4] = {d, diff[0], diff[1], diff[2]};
  T* o = prr + idx * PRW;
  T s[F0];
#pragma unroll
  for (int l = 0; l < F0; ++l) {
    T pre = bt[l];
#pragma unroll
    for (int q = 0; q < 4; ++q) pre += feat[q] * Kt[q * F0 + l];
    o[4 + l] = pre;
    s[l] = silu(pre);
  }
  const T cut = cutoff_val(d * inv_c);
  T ew[F1];
#pragma unroll
  for (int c = 0; c < F1; ++c) ew[c] = T(0);
#pragma unroll
  for (int m = 0; m < NENV_EE; ++m) {
    const T u = d * isc[m];
    const T ev = dexp(-u * u) * cut;
    o[20 + m] = ev;
#pragma unroll
    for (int c = 0; c < F1; ++c) ew[c] += ev * eW[m * F1 + c];
  }
  const int bo = tag == 0 ? 56 : 64, so = tag == 0 ? 72 : 77;
#pragma unroll
  for (int c = 0; c < F1; ++c) {
    T df = db[c];
#pragma unroll
    for (int l = 0; l < F0; ++l) df += s[l] * dW[l * F1 + c];
    o[36 + c] = df;
    o[44 + c] = ew[c];
    o[bo + c] = df * ew[c];
  }
  const T lp = dlog1p(d);
  o[so] = lp;
#pragma unroll
  for (int q = 0; q < 3; ++q) o[so + 1 + q] = diff[q] / d * lp;
  o[so + 4] = T(1);
  o[52] = (T)tag;
#pragma unroll
  for (int q = 0; q < 4; ++q) o[q] = feat[q];
}

// One CTA (thread = feature) per center electron: h = h0 + sum over the pairs of Gamma * silu(e + m_ct[i] + m_nb[j])
// (contract_pair, new_sparse_model.py:83-93; ElecInit output ei = h0 | ct_same | ct_diff | nb_same | nb_diff).
template <typename T>
__global__ void __launch_bounds__(256) gk_contract_fwd(Nbr nb, Weights<T> W, const T* __restrict__ prr,
                                                       const T* __restrict__ ei, T* __restrict__ hc) {
  const long g = blockIdx.x;
  const int f = threadIdx.x, n = nb.n, cp = nb.cap_p;
  const int w = (int)(g / n), i = (int)(g - (long)w * n);
  const int* rp = nb.rowptr + (long)w * (n + 1);
  T h = ei[g * 5 * F + f];
  if (rp[n] <= cp) {
    T wg[2][F1], we[2][4], be[2];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const T* Wg = W.w[t == 0 ? FIRE_P_EESAME_GAMMA_W : FIRE_P_EEDIFF_GAMMA_W];
      const T* We = W.w[t == 0 ? FIRE_P_EESAME_EDGE_W : FIRE_P_EEDIFF_EDGE_W];
#pragma unroll
      for (int c = 0; c < F1; ++c) wg[t][c] = Wg[c * F + f];
#pragma unroll
      for (int q = 0; q < 4; ++q) we[t][q] = We[q * F + f];
      be[t] = W.w[t == 0 ? FIRE_P_EESAME_EDGE_B : FIRE_P_EEDIFF_EDGE_B][f];
    }
    const T mct[2] = {ei[g * 5 * F + F + f], ei[g * 5 * F + 2 * F + f]};
    for (int p = rp[i]; p < rp[i + 1]; ++p) {
      const long pr = (long)w * cp + p;
      const T* o = prr + pr * PRW;
      const int t = o[52] != T(0) ? 1 : 0;
      const int j = nb.nbr[pr];
      const T* be8 = o + (t == 0 ? 56 : 64);
      const T* sc = o + (t == 0 ? 72 : 77);
      T gm = T(0), ed = be[t];
#pragma unroll
      for (int c = 0; c < F1; ++c) gm += be8[c] * wg[t][c];
#pragma unroll
      for (int q = 0; q < 4; ++q) ed += sc[q] * we[t][q];
      const T u = ed + mct[t] + ei[((long)w * n + j) * 5 * F + (3 + t) * F + f];
      h += gm * silu(u);
    }
  }
  hc[g * F + f] = h;
}

// hf (spin-major) = a2 * scales[1]
template <typename T>
__global__ void gk_hf(const T* __restrict__ a2, const T* __restrict__ s1, T* __restrict__ hf, int Wc, int n, int nu) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)Wc * n * F) return;
  const long g = idx / F;
  const int f = (int)(idx - g * F), w = (int)(g / n), i = (int)(g - (long)w * n);
  hf[sm_row(w, i, Wc, nu, n - nu) * F + f] = a2[idx] * s1[0];
}

// ------------------------------------------------------------------------------------------ orbitals forward
// ex[d][row][I * 8 + k] = exp(-|r - R_I| softplus(sigma_s[I, d, k])) for spin-major rows
template <typename T>
__global__ void gk_ex(const T* __restrict__ r, const float* __restrict__ R, Weights<T> W, int Wc, int n, int nu,
                      int N, T* __restrict__ ex) {
  const long N8 = (long)N * NENV_ORB, G = (long)Wc * n;
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= NDET * G * N8) return;
  const int Ik = (int)(idx % N8);
  const long row = (idx / N8) % G;
  const int d = (int)(idx / (N8 * G));
  int w, i, s;
  if (row < (long)Wc * nu) { w = (int)(row / nu); i = (int)(row % nu); s = 0; }
  else { const long t = row - (long)Wc * nu; w = (int)(t / (n - nu)); i = nu + (int)(t % (n - nu)); s = 1; }
  const int I = Ik / NENV_ORB, k = Ik % NENV_ORB;
  const long g = (long)w * n + i;
  const T dx = r[3 * g] - (T)R[3 * I], dy = r[3 * g + 1] - (T)R[3 * I + 1], dz = r[3 * g + 2] - (T)R[3 * I + 2];
  const T dist = dsqrt(dx * dx + dy * dy + dz * dz);
  const T sp = W.w[s == 0 ? PR_ENV_UP_SP : PR_ENV_DN_SP][((long)I * NDET + d) * NENV_ORB + k];
  ex[idx] = dexp(-dist * sp);
}

// A[((w n + i) D + d) n + o] = raw * env of the spin-major row of (w, i) (the layout k_gj_global reads)
template <typename T>
__global__ void gk_amat(const T* __restrict__ raw, const T* __restrict__ env, T* __restrict__ A, int Wc, int n,
                        int nu) {
  const long DN = (long)NDET * n;
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)Wc * n * DN) return;
  const long g = idx / DN, c = idx - g * DN;
  const int w = (int)(g / n), i = (int)(g - (long)w * n);
  const long rs = sm_row(w, i, Wc, nu, n - nu);
  A[idx] = raw[rs * DN + c] * env[rs * DN + c];
}

// ------------------------------------------------------------------------------------------ Jastrow forward
// att[row][h] = exp(-(q[row, h, :] . keys[h, :]) / 4)  (GlobalAttentionJastrow, jastrow.py:85-100)
template <typename T>
__global__ void gk_att(const T* __restrict__ q, const T* __restrict__ keys, T* __restrict__ att, long G) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= G * HEADS) return;
  const long row = idx / HEADS;
  const int h = (int)(idx - row * HEADS);
  T s = T(0);
#pragma unroll
  for (int a = 0; a < HDIM; ++a) s += q[row * F + h * HDIM + a] * keys[h * HDIM + a];
  att[idx] = dexp(-s * T(0.25));
}

// One CTA (thread = h * 16 + a) per walker: per spin the attention normaliser and weighted value sums, and the
// readout input X[w][s * 256 + h * 16 + a] = V_s / norm_s (jastrow.py:139-151).
template <typename T>
__global__ void __launch_bounds__(256) gk_readout_in(const T* __restrict__ att, const T* __restrict__ v, int Wc, int n,
                                                     int nu, T* __restrict__ nrm, T* __restrict__ Vs,
                                                     T* __restrict__ X) {
  const int w = blockIdx.x, f = threadIdx.x, h = f / HDIM;
  for (int s = 0; s < 2; ++s) {
    const int ns = s == 0 ? nu : n - nu;
    const long base = s == 0 ? (long)w * nu : (long)Wc * nu + (long)w * (n - nu);
    T a = T(0), b = T(0);
    for (int k = 0; k < ns; ++k) {
      const T at = att[(base + k) * HEADS + h];
      a += at;
      b += at * v[(base + k) * F + f];
    }
    if ((f & (HDIM - 1)) == 0) nrm[((long)w * 2 + s) * HEADS + h] = a;
    Vs[((long)w * 2 + s) * F + f] = b;
    X[(long)w * 2 * F + s * F + f] = b / a;
  }
}

// ------------------------------------------------------------------------------------------ head
// One CTA per walker: logsumexp over the determinants (wave_function.py:178, signed_logpsi_from_orbitals,
// model/utils.py:196-213), the psiformer cusp (jastrow.py:48-64) and the Jastrow readout sums; log|psi| and sign;
// the seeds of the reverse pass (seed[w] = c_0..c_3, dJ0, dJ1 with c_d = d log|sum| / d logdet_d) and the
// gradients of the scalar Jastrow parameters.
template <typename T>
__global__ void __launch_bounds__(256) gk_head(const T* __restrict__ r, Weights<T> W, int Wc, int n, int nu,
                                               const double* __restrict__ ld, const double* __restrict__ sd,
                                               const T* __restrict__ m3, const T* __restrict__ x3, int w0,
                                               T* __restrict__ logpsi, T* __restrict__ sign, T* __restrict__ seed,
                                               T* __restrict__ grad, long ldg, const int64_t* __restrict__ off,
                                               int32_t* status) {
  __shared__ T red[32 * 8];
  const int w = blockIdx.x, t = threadIdx.x;
  const T* cusp = W.w[FIRE_P_CUSP];
  const T as = cusp[0], ad = cusp[1], fs = cusp[2], fd = cusp[3];
  const T* rw = r + (long)w * n * 3;
  T v[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = T(0);
  // pairs i < j
  const long npair = (long)n * (n - 1) / 2;
  for (long q = t; q < npair; q += blockDim.x) {
    // invert q = i (2n - i - 1) / 2 + (j - i - 1)
    int i = (int)((2.0 * n - 1.0 - sqrt((2.0 * n - 1.0) * (2.0 * n - 1.0) - 8.0 * (double)q)) / 2.0);
    if (i < 0) i = 0;
    while ((long)(i + 1) * (2 * n - i - 2) / 2 <= q) ++i;
    while (i > 0 && (long)i * (2 * n - i - 1) / 2 > q) --i;
    const int j = (int)(q - (long)i * (2 * n - i - 1) / 2) + i + 1;
    const T dx = rw[3 * i] - rw[3 * j], dy = rw[3 * i + 1] - rw[3 * j + 1], dz = rw[3 * i + 2] - rw[3 * j + 2];
    const T dd = dsqrt(dx * dx + dy * dy + dz * dz);
    const bool same = (i < nu) == (j < nu);
    const T a = same ? as : ad;
    const T ia = T(1) / (a + dd);
    const T term = a * a * ia;                      // a^2 / (a + d)
    const T dterm = a * (a + T(2) * dd) * ia * ia;  // d term / d a
    if (same) { v[0] += term; v[1] += dterm; }
    else { v[2] += term; v[3] += dterm; }
  }
  // MLP Jastrow rows of this walker (spin-major: its up rows, then its down rows)
  for (int k = t; k < n; k += blockDim.x) {
    const long row = k < nu ? (long)w * nu + k : (long)Wc * nu + (long)w * (n - nu) + (k - nu);
    v[4] += m3[row * 2];
    v[5] += m3[row * 2 + 1];
  }
  block_sum<T, 8>(v, red);
  if (t == 0) {
    const T* ms = W.w[FIRE_P_MLP_SCALE];
    const T* asc = W.w[FIRE_P_ATT_SCALE];
    const T J0 = x3[w * 2] * asc[0] + v[4] * ms[0];
    const T J1 = x3[w * 2 + 1] * asc[1] + W.w[FIRE_P_ATT_BIAS][0] + v[5] * ms[1] + (T)n * W.w[FIRE_P_LOG_BIAS][0];
    const T lc = fs * v[0] + fd * v[2];
    double m = -1e300;
    for (int d = 0; d < NDET; ++d) m = fmax(m, ld[w * NDET + d]);
    double S = 0.0;
    for (int d = 0; d < NDET; ++d) S += sd[w * NDET + d] * exp(ld[w * NDET + d] - m);
    const double ldet = m + log(fabs(S));
    const T lp = (T)ldet + lc + J0 + dlog(J1 < T(0) ? -J1 : J1);
    const T sg = (T)((S < 0.0) != (J1 < T(0)) ? -1 : 1);
    logpsi[w0 + w] = lp;
    sign[w0 + w] = sg;
    if (!(lp == lp) || lp - lp != T(0)) set_flag(status, FIRE_FLAG_NONFINITE);
    T* sw = seed + (long)w * 8;
    for (int d = 0; d < NDET; ++d) sw[d] = (T)(sd[w * NDET + d] * exp(ld[w * NDET + d] - m) / S);
    const T dJ0 = T(1), dJ1 = T(1) / J1;
    sw[4] = dJ0;
    sw[5] = dJ1;
    T* gw = grad + (long)(w0 + w) * ldg;
    gw[off[FIRE_P_MLP_SCALE]] = v[4] * dJ0;
    gw[off[FIRE_P_MLP_SCALE] + 1] = v[5] * dJ1;
    gw[off[FIRE_P_LOG_BIAS]] = (T)n * dJ1;
    gw[off[FIRE_P_ATT_SCALE]] = x3[w * 2] * dJ0;
    gw[off[FIRE_P_ATT_SCALE] + 1] = x3[w * 2 + 1] * dJ1;
    gw[off[FIRE_P_ATT_BIAS]] = dJ1;
    gw[off[FIRE_P_CUSP]] = fs * v[1];
    gw[off[FIRE_P_CUSP] + 1] = fd * v[3];
    gw[off[FIRE_P_CUSP] + 2] = v[0];
    gw[off[FIRE_P_CUSP] + 3] = v[2];
  }
}

// dx3[w][k] = att_scale[k] dJ_k (readout output), dzm3[row][k] = mlp_scale[k] dJ_k silu'(zm3) (MLP Jastrow rows)
template <typename T>
__global__ void gk_jseed(Weights<T> W, const T* __restrict__ seed, const T* __restrict__ zm3, int Wc, int n, int nu,
                         T* __restrict__ dx3, T* __restrict__ dzm3) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long G = (long)Wc * n;
  if (idx < (long)Wc * 2) {
    const int w = (int)(idx / 2), k = (int)(idx & 1);
    dx3[idx] = W.w[FIRE_P_ATT_SCALE][k] * seed[w * 8 + 4 + k];
  }
  if (idx >= G * 2) return;
  const long row = idx / 2;
  const int k = (int)(idx & 1);
  const int w = row < (long)Wc * nu ? (int)(row / nu) : (int)((row - (long)Wc * nu) / (n - nu));
  T y, d1, d2;
  silu3(zm3[idx], y, d1, d2);
  dzm3[idx] = W.w[FIRE_P_MLP_SCALE][k] * seed[w * 8 + 4 + k] * d1;
}

// ------------------------------------------------------------------------------------------ Jastrow backward
// One CTA (thread = h * 16 + a) per walker: from dX (readout input) to d att, d v and d q of every row, and the
// gradient of the attention keys.
template <typename T>
__global__ void __launch_bounds__(256) gk_att_bwd(Weights<T> W, const T* __restrict__ dX, const T* __restrict__ nrm,
                                                  const T* __restrict__ Vs, const T* __restrict__ att,
                                                  const T* __restrict__ v, const T* __restrict__ q, int Wc, int n,
                                                  int nu, T* __restrict__ dq, T* __restrict__ dv, T* __restrict__ grad,
                                                  long ldg, int w0, int64_t off_keys) {
  const int w = blockIdx.x, f = threadIdx.x, h = f / HDIM;
  const T key = W.w[FIRE_P_ATT_KEYS][f];
  T kacc = T(0);
  for (int s = 0; s < 2; ++s) {
    const int ns = s == 0 ? nu : n - nu;
    const long base = s == 0 ? (long)w * nu : (long)Wc * nu + (long)w * (n - nu);
    const T nm = nrm[((long)w * 2 + s) * HEADS + h];
    const T dXv = dX[(long)w * 2 * F + s * F + f];
    const T dV = dXv / nm;
    T dn = -dXv * Vs[((long)w * 2 + s) * F + f] / (nm * nm);
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) dn += __shfl_xor_sync(0xffffffffu, dn, o);
    for (int k = 0; k < ns; ++k) {
      const long row = base + k;
      const T at = att[row * HEADS + h];
      T da = dV * v[row * F + f];
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) da += __shfl_xor_sync(0xffffffffu, da, o);
      da += dn;
      dv[row * F + f] = at * dV;
      const T dl = da * at * T(-0.25);  // d (q . key) of this row and head
      dq[row * F + f] = dl * key;
      kacc += dl * q[row * F + f];
    }
  }
  grad[(long)(w0 + w) * ldg + off_keys + f] = kacc;
}

// ------------------------------------------------------------------------------------------ determinant backward
// draw = G env, denv = G raw with G_d[i][o] = c_d (A_d^-1)[o][i] (the transposed inverse written by k_gj_global)
template <typename T>
__global__ void gk_dA(const T* __restrict__ Ainv, const T* __restrict__ seed, const T* __restrict__ raw,
                      const T* __restrict__ env, int Wc, int n, int nu, T* __restrict__ draw, T* __restrict__ denv) {
  const long DN = (long)NDET * n;
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)Wc * n * DN) return;
  const long g = idx / DN, c = idx - g * DN;
  const int w = (int)(g / n), i = (int)(g - (long)w * n), d = (int)(c / n), o = (int)(c - (long)d * n);
  const int lda = ainv_ld(n), sh = (d * n) & 3;
  const T G = seed[w * 8 + d] * Ainv[(((long)w * NDET + d) * n + i) * lda + sh + o];
  const long rs = sm_row(w, i, Wc, nu, n - nu);
  draw[rs * DN + c] = G * env[rs * DN + c];
  denv[rs * DN + c] = G * raw[rs * DN + c];
}

// One CTA per (walker, spin): d sigma_s[I, d, k] = sum_rows dex ex (-|r - R_I|) sigmoid(sigma)
template <typename T>
__global__ void __launch_bounds__(256) gk_dsigma(const T* __restrict__ r, const float* __restrict__ R, Weights<T> W,
                                                 const T* __restrict__ ex, const T* __restrict__ dex, int Wc, int n,
                                                 int nu, int N, T* __restrict__ grad, long ldg, int w0,
                                                 int64_t off_up, int64_t off_dn) {
  const int w = blockIdx.x, s = blockIdx.y;
  const int ns = s == 0 ? nu : n - nu;
  const long base = s == 0 ? (long)w * nu : (long)Wc * nu + (long)w * (n - nu);
  const long N8 = (long)N * NENV_ORB, G = (long)Wc * n;
  const T* sig = W.w[s == 0 ? FIRE_P_ENV_UP_SIGMA : FIRE_P_ENV_DN_SIGMA];
  for (long e = threadIdx.x; e < NDET * N8; e += blockDim.x) {
    const int d = (int)(e / N8), Ik = (int)(e - d * N8), I = Ik / NENV_ORB, k = Ik % NENV_ORB;
    T acc = T(0);
    for (int q = 0; q < ns; ++q) {
      const long row = base + q;
      const int i = s == 0 ? q : nu + q;
      const long g = (long)w * n + i;
      const T dx = r[3 * g] - (T)R[3 * I], dy = r[3 * g + 1] - (T)R[3 * I + 1], dz = r[3 * g + 2] - (T)R[3 * I + 2];
      const T dist = dsqrt(dx * dx + dy * dy + dz * dz);
      const long a = ((long)d * G + row) * N8 + Ik;
      acc -= dex[a] * ex[a] * dist;
    }
    const long pi = ((long)I * NDET + d) * NENV_ORB + k;
    grad[(long)(w0 + w) * ldg + (s == 0 ? off_up : off_dn) + pi] = acc * sigm(sig[pi]);
  }
}

// ------------------------------------------------------------------------------------------ embedding backward
// One CTA per walker: da2 = dhf * scales[1] (electron order) and d scales[1] = sum dhf a2
template <typename T>
__global__ void __launch_bounds__(256) gk_hf_bwd(const T* __restrict__ dhf, const T* __restrict__ a2,
                                                 const T* __restrict__ s1, int Wc, int n, int nu, T* __restrict__ da2,
                                                 T* __restrict__ grad, long ldg, int w0, int64_t off_s1) {
  __shared__ T red[32];
  const int w = blockIdx.x;
  T acc = T(0);
  for (long e = threadIdx.x; e < (long)n * F; e += blockDim.x) {
    const int i = (int)(e / F), f = (int)(e - (long)i * F);
    const long g = (long)w * n + i;
    const T dy = dhf[sm_row(w, i, Wc, nu, n - nu) * F + f];
    acc += dy * a2[g * F + f];
    da2[g * F + f] = dy * s1[0];
  }
  T v[1] = {acc};
  block_sum<T, 1>(v, red);
  if (threadIdx.x == 0) grad[(long)(w0 + w) * ldg + off_s1] = v[0];
}
// One CTA per walker: dh = dxs * scales[0] and d scales[0] = sum dxs hc
template <typename T>
__global__ void __launch_bounds__(256) gk_s0_bwd(const T* __restrict__ dxs, const T* __restrict__ hc,
                                                 const T* __restrict__ s0, int n, T* __restrict__ dh,
                                                 T* __restrict__ grad, long ldg, int w0, int64_t off_s0) {
  __shared__ T red[32];
  const int w = blockIdx.x;
  T acc = T(0);
  for (long e = threadIdx.x; e < (long)n * F; e += blockDim.x) {
    const long a = (long)w * n * F + e;
    acc += dxs[a] * hc[a];
    dh[a] = dxs[a] * s0[0];
  }
  T v[1] = {acc};
  block_sum<T, 1>(v, red);
  if (threadIdx.x == 0) grad[(long)(w0 + w) * ldg + off_s0] = v[0];
}

// One CTA (thread = feature) per center: d Gamma and d u of every pair of the center (the message
// Gamma * silu(u), u = e + m_ct[i] + m_nb[j]); dgp, dup [pair rows][F].
template <typename T>
__global__ void __launch_bounds__(256) gk_pair_bwd(Nbr nb, Weights<T> W, const T* __restrict__ prr,
                                                   const T* __restrict__ ei, const T* __restrict__ dh,
                                                   T* __restrict__ dgp, T* __restrict__ dup) {
  const long g = blockIdx.x;
  const int f = threadIdx.x, n = nb.n, cp = nb.cap_p;
  const int w = (int)(g / n), i = (int)(g - (long)w * n);
  const int* rp = nb.rowptr + (long)w * (n + 1);
  if (rp[n] > cp) return;
  T wg[2][F1], we[2][4], be[2];
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const T* Wg = W.w[t == 0 ? FIRE_P_EESAME_GAMMA_W : FIRE_P_EEDIFF_GAMMA_W];
    const T* We = W.w[t == 0 ? FIRE_P_EESAME_EDGE_W : FIRE_P_EEDIFF_EDGE_W];
#pragma unroll
    for (int c = 0; c < F1; ++c) wg[t][c] = Wg[c * F + f];
#pragma unroll
    for (int q = 0; q < 4; ++q) we[t][q] = We[q * F + f];
    be[t] = W.w[t == 0 ? FIRE_P_EESAME_EDGE_B : FIRE_P_EEDIFF_EDGE_B][f];
  }
  const T mct[2] = {ei[g * 5 * F + F + f], ei[g * 5 * F + 2 * F + f]};
  const T dy = dh[g * F + f];
  for (int p = rp[i]; p < rp[i + 1]; ++p) {
    const long pr = (long)w * cp + p;
    const T* o = prr + pr * PRW;
    const int t = o[52] != T(0) ? 1 : 0;
    const int j = nb.nbr[pr];
    const T* be8 = o + (t == 0 ? 56 : 64);
    const T* sc = o + (t == 0 ? 72 : 77);
    T gm = T(0), ed = be[t];
#pragma unroll
    for (int c = 0; c < F1; ++c) gm += be8[c] * wg[t][c];
#pragma unroll
    for (int q = 0; q < 4; ++q) ed += sc[q] * we[t][q];
    const T u = ed + mct[t] + ei[((long)w * n + j) * 5 * F + (3 + t) * F + f];
    T y, d1, d2;
    silu3(u, y, d1, d2);
    dgp[pr * F + f] = dy * y;
    dup[pr * F + f] = dy * gm * d1;
  }
}

// One CTA per electron: d ei = [dh, sum_own pairs du (same, diff), sum_pairs where it is the neighbour du (same, diff)]
template <typename T>
__global__ void __launch_bounds__(256) gk_dei(Nbr nb, const T* __restrict__ prr, const T* __restrict__ dh,
                                              const T* __restrict__ dup, T* __restrict__ dei) {
  const long g = blockIdx.x;
  const int f = threadIdx.x, n = nb.n, cp = nb.cap_p;
  const int w = (int)(g / n), i = (int)(g - (long)w * n);
  const int* rp = nb.rowptr + (long)w * (n + 1);
  T ct[2] = {T(0), T(0)}, nbv[2] = {T(0), T(0)};
  if (rp[n] <= cp) {
    for (int p = rp[i]; p < rp[i + 1]; ++p) {
      const long pr = (long)w * cp + p;
      const int t = prr[pr * PRW + 52] != T(0) ? 1 : 0;
      ct[t] += dup[pr * F + f];
      const long qr = (long)w * cp + nb.rev[pr];
      nbv[t] += dup[qr * F + f];
    }
  }
  T* o = dei + g * 5 * F;
  o[f] = dh[g * F + f];
  o[F + f] = ct[0];
  o[2 * F + f] = ct[1];
  o[3 * F + f] = nbv[0];
  o[4 * F + f] = nbv[1];
}

// Small filter of one pair / edge backwards from d beta: the per-edge rows of the parameter reductions.
// Pair rows (X per tag): [s 16 | envv 16 | feat 4 | 1] at tag * 37; Y: [ddirf 8 | dew 8 | dpre 16 | dscale 16 | dcp 1].
template <typename T>
__global__ void gk_pair_small_bwd(Nbr nb, Weights<T> W, const T* __restrict__ prr, const T* __restrict__ dbs,
                                  const T* __restrict__ dbd, T* __restrict__ px, T* __restrict__ py) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int cp = nb.cap_p, n = nb.n;
  if (idx >= (long)nb.W * cp) return;
  const int w = (int)(idx / cp), p = (int)(idx - (long)w * cp);
  const int* rp = nb.rowptr + (long)w * (n + 1);
  const int P = rp[n];
  if (P > cp || p >= P) return;
  const T* o = prr + idx * PRW;
  const int t = o[52] != T(0) ? 1 : 0;
  const T* db = (t == 0 ? dbs : dbd) + idx * F1;
  const T* dW = W.w[t == 0 ? FIRE_P_EESAME_DIR_W : FIRE_P_EEDIFF_DIR_W];
  const T* eW = W.w[t == 0 ? FIRE_P_EESAME_ENV_W : FIRE_P_EEDIFF_ENV_W];
  const T* isc = W.w[t == 0 ? PR_EESAME_INVSCALE : PR_EEDIFF_INVSCALE];
  const T* sraw = W.w[t == 0 ? FIRE_P_EESAME_SCALE : FIRE_P_EEDIFF_SCALE];
  const T c_eff = W.w[PR_SCALARS][0];
  const T cpar = W.w[FIRE_P_CUTOFF_PARAM][0];
  const T d = o[0];
  T* X = px + idx * PX + t * 37;
  T* Y = py + idx * PY;
  T ddirf[F1], dew[F1];
#pragma unroll
  for (int c = 0; c < F1; ++c) {
    ddirf[c] = db[c] * o[44 + c];
    dew[c] = db[c] * o[36 + c];
    Y[c] = ddirf[c];
    Y[8 + c] = dew[c];
  }
#pragma unroll
  for (int l = 0; l < F0; ++l) {
    const T pre = o[4 + l];
    T y, d1, d2;
    silu3(pre, y, d1, d2);
    T ds = T(0);
#pragma unroll
    for (int c = 0; c < F1; ++c) ds += ddirf[c] * dW[l * F1 + c];
    X[l] = y;
    Y[16 + l] = ds * d1;
  }
  const T x = d / c_eff;
  T cu, cu1, cu2;
  cutoff3(x, cu, cu1, cu2);
  T dcp = T(0);
#pragma unroll
  for (int m = 0; m < NENV_EE; ++m) {
    T de = T(0);
#pragma unroll
    for (int c = 0; c < F1; ++c) de += dew[c] * eW[m * F1 + c];
    const T ev = o[20 + m];
    X[16 + m] = ev;
    const T a = isc[m];                 // 1 / softplus(raw)
    const T u = d * a;
    const T gq = dexp(-u * u);
    // d envv / d sc = gq cut 2 d^2 / sc^3; d sc / d raw = sigmoid(raw)
    Y[32 + m] = de * ev * T(2) * u * u * a * sigm(sraw[m]);
    dcp += de * gq * cu1 * (-x);
  }
  const T sg = sigm(cpar);
  Y[48] = dcp * (T(1) - sg);
#pragma unroll
  for (int q = 0; q < 4; ++q) X[32 + q] = o[q];
  X[36] = T(1);
}

// Scatter of the per-walker pair reduction out[PX][PY] into the filter parameter slots of both tags.
template <typename T>
__global__ void gk_pair_small_scatter(const T* __restrict__ red, int Wc, T* __restrict__ grad, long ldg, int w0,
                                      const int64_t* __restrict__ off) {
  const int w = blockIdx.x;
  const T* R0 = red + (long)w * PX * PY;
  T* gw = grad + (long)(w0 + w) * ldg;
  for (int e = threadIdx.x; e < 2 * 360 + 1; e += blockDim.x) {
    if (e == 720) {
      gw[off[FIRE_P_CUTOFF_PARAM]] = R0[36 * PY + 48] + R0[(37 + 36) * PY + 48];
      continue;
    }
    const int t = e / 360, k = e - t * 360;
    const T* R = R0 + t * 37 * PY;
    const int base = t == 0 ? FIRE_P_EESAME_SCALE : FIRE_P_EEDIFF_SCALE;  // slot order: scale kernel bias dir_W dir_b env_W
    if (k < 128) {  // dir_W [16][8] = s^T ddirf
      const int l = k / 8, c = k % 8;
      gw[off[base + 3] + k] = R[l * PY + c];
    } else if (k < 136) {  // dir_b
      gw[off[base + 4] + (k - 128)] = R[36 * PY + (k - 128)];
    } else if (k < 264) {  // env_W [16][8] = envv^T dew
      const int m = (k - 136) / 8, c = (k - 136) % 8;
      gw[off[base + 5] + (k - 136)] = R[(16 + m) * PY + 8 + c];
    } else if (k < 328) {  // kernel [4][16] = feat^T dpre
      const int q = (k - 264) / 16, l = (k - 264) % 16;
      gw[off[base + 1] + (k - 264)] = R[(32 + q) * PY + 16 + l];
    } else if (k < 344) {  // bias
      gw[off[base + 2] + (k - 328)] = R[36 * PY + 16 + (k - 328)];
    } else {  // scale
      gw[off[base] + (k - 344)] = R[36 * PY + 32 + (k - 344)];
    }
  }
}

template <typename T>
__global__ void gk_glu_bwd(const T* __restrict__ gb, const T* __restrict__ dh2, T* __restrict__ dg, long G) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= G * F) return;
  const long g = i / F;
  const int f = (int)(i - g * F);
  const T a = gb[g * 2 * F + f], b = gb[g * 2 * F + F + f];
  T y, d1, d2;
  silu3(b, y, d1, d2);
  dg[g * 2 * F + f] = dh2[i] * y;
  dg[g * 2 * F + F + f] = dh2[i] * a * d1;
}

// One CTA per electron: LayerNorm backwards, d h = (dxh - mean(dxh) - xh mean(dxh xh)) / sigma, dxh = dh1 scale
template <typename T>
__global__ void __launch_bounds__(256) gk_ln_bwd(Weights<T> W, const T* __restrict__ dh1, const T* __restrict__ xhat,
                                                 const T* __restrict__ rstd, T* __restrict__ dhs) {
  __shared__ T red[64];
  const long g = blockIdx.x;
  const int f = threadIdx.x;
  const T xh = xhat[g * F + f];
  const T dx = dh1[g * F + f] * W.w[FIRE_P_EI_LN_SCALE][f];
  T v[2] = {dx, dx * xh};
  block_sum<T, 2>(v, red);
  dhs[g * F + f] = rstd[g] * (dx - v[0] / T(F) - xh * v[1] / T(F));
}
// One CTA (thread = feature) per walker: d ln_scale = sum dh1 xh, d ln_bias = sum dh1
template <typename T>
__global__ void __launch_bounds__(256) gk_ln_params(const T* __restrict__ dh1, const T* __restrict__ xhat, int n,
                                                    T* __restrict__ grad, long ldg, int w0, int64_t off_s,
                                                    int64_t off_b) {
  const int w = blockIdx.x, f = threadIdx.x;
  T a = T(0), b = T(0);
  for (int i = 0; i < n; ++i) {
    const long e = ((long)w * n + i) * F + f;
    a += dh1[e] * xhat[e];
    b += dh1[e];
  }
  grad[(long)(w0 + w) * ldg + off_s + f] = a;
  grad[(long)(w0 + w) * ldg + off_b + f] = b;
}

// One CTA (thread = feature) per electron: d Gamma and d e of its e-n edges (h = sum Gamma * e)
template <typename T>
__global__ void __launch_bounds__(256) gk_en_bwd_rows(Nbr nb, Weights<T> W, const T* __restrict__ enr,
                                                      const T* __restrict__ dhs, T* __restrict__ dge,
                                                      T* __restrict__ dee) {
  const long g = blockIdx.x;
  const int f = threadIdx.x, E = nb.cap_nuc;
  const int ne = nb.en_cnt[g];
  T wg[F1], we[4];
#pragma unroll
  for (int c = 0; c < F1; ++c) wg[c] = W.w[FIRE_P_EI_GAMMA_W][c * F + f];
#pragma unroll
  for (int q = 0; q < 4; ++q) we[q] = W.w[FIRE_P_EI_EDGE_W][q * F + f];
  const T dy = dhs[g * F + f];
  for (int k = 0; k < ne; ++k) {
    const long row = g * E + k;
    const T* e = enr + row * ENW;
    const int J = nb.en_idx[row];
    T gm = T(0), ed = W.w[FIRE_P_EN_NUC_EMB][(long)J * F + f];
#pragma unroll
    for (int c = 0; c < F1; ++c) gm += e[72 + c] * wg[c];
#pragma unroll
    for (int q = 0; q < 4; ++q) ed += e[68 + q] * we[q];
    dge[row * F + f] = dy * ed;
    dee[row * F + f] = dy * gm;
  }
}

// One thread per e-n edge row: the small filter backwards from d beta.  Shared rows X [s 16 | envv 32 | 1],
// Y [ddirf 8 | dew 8]; per-nucleus rows [dpre 16 | dscale 32].
template <typename T>
__global__ void gk_en_small_bwd(Nbr nb, Weights<T> W, const T* __restrict__ enr, const T* __restrict__ dbe,
                                T* __restrict__ ex_, T* __restrict__ ey_, T* __restrict__ e2_) {
  const long row = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int E = nb.cap_nuc;
  if (row >= (long)nb.W * nb.n * E) return;
  const long g = row / E;
  const int k = (int)(row - g * E);
  if (k >= nb.en_cnt[g]) return;
  const int J = nb.en_idx[row];
  const T* o = enr + row * ENW;
  const T* db = dbe + row * F1;
  const T* dW = W.w[FIRE_P_EI_DIR_W];
  const T* eW = W.w[FIRE_P_EI_ENV_W];
  const T* isc = W.w[PR_EN_INVSCALE] + (long)J * NENV_EN;
  const T* sraw = W.w[FIRE_P_EN_SCALES] + (long)J * NENV_EN;
  T* X = ex_ + row * EX;
  T* Y = ey_ + row * EY;
  T* Z = e2_ + row * EN2;
  const T d = o[0];
  T ddirf[F1], dew[F1];
#pragma unroll
  for (int c = 0; c < F1; ++c) {
    ddirf[c] = db[c] * o[60 + c];
    dew[c] = db[c] * o[52 + c];
    Y[c] = ddirf[c];
    Y[8 + c] = dew[c];
  }
#pragma unroll
  for (int l = 0; l < F0; ++l) {
    T y, d1, d2;
    silu3(o[4 + l], y, d1, d2);
    T ds = T(0);
#pragma unroll
    for (int c = 0; c < F1; ++c) ds += ddirf[c] * dW[l * F1 + c];
    X[l] = y;
    Z[l] = ds * d1;
  }
  for (int m = 0; m < NENV_EN; ++m) {
    T de = T(0);
#pragma unroll
    for (int c = 0; c < F1; ++c) de += dew[c] * eW[m * F1 + c];
    const T ev = o[20 + m];
    X[16 + m] = ev;
    const T a = isc[m], u = d * a;
    Z[16 + m] = de * ev * T(2) * u * u * a * sigm(sraw[m]);
  }
  X[48] = T(1);
}

// Scatter of the per-walker e-n reduction out[EX][EY] into dir_W, dir_b and env_W of ElecInit's filter.
template <typename T>
__global__ void gk_en_small_scatter(const T* __restrict__ red, T* __restrict__ grad, long ldg, int w0,
                                    const int64_t* __restrict__ off) {
  const int w = blockIdx.x;
  const T* R = red + (long)w * EX * EY;
  T* gw = grad + (long)(w0 + w) * ldg;
  for (int k = threadIdx.x; k < 128 + 8 + 256; k += blockDim.x) {
    if (k < 128) gw[off[FIRE_P_EI_DIR_W] + k] = R[(k / 8) * EY + k % 8];
    else if (k < 136) gw[off[FIRE_P_EI_DIR_B] + k - 128] = R[48 * EY + (k - 128)];
    else {
      const int m = (k - 136) / 8, c = (k - 136) % 8;
      gw[off[FIRE_P_EI_ENV_W] + k - 136] = R[(16 + m) * EY + 8 + c];
    }
  }
}

// One CTA per (walker, nucleus J): the per-nucleus parameters, summed over the electrons with J in their e-n list:
// nuc_emb[J] (d e), kernel[J] (feat^T dpre), bias[J] (dpre), scales[J] (dscale).
template <typename T>
__global__ void __launch_bounds__(256) gk_en_nuc(Nbr nb, const T* __restrict__ enr, const T* __restrict__ dee,
                                                 const T* __restrict__ e2, const int* __restrict__ inv,
                                                 T* __restrict__ grad, long ldg, int w0,
                                                 const int64_t* __restrict__ off) {
  const int J = blockIdx.x, w = blockIdx.y, t = threadIdx.x, n = nb.n, N = nb.N, E = nb.cap_nuc;
  T a = T(0), b = T(0);
  for (int i = 0; i < n; ++i) {
    const long g = (long)w * n + i;
    const int k = inv[g * N + J];
    if (k < 0) continue;
    const long row = g * E + k;
    a += dee[row * F + t];
    if (t < 64) b += enr[row * ENW + t / 16] * e2[row * EN2 + t % 16];
    else if (t < 80) b += e2[row * EN2 + (t - 64)];
    else if (t < 112) b += e2[row * EN2 + 16 + (t - 80)];
  }
  T* gw = grad + (long)(w0 + w) * ldg;
  gw[off[FIRE_P_EN_NUC_EMB] + (long)J * F + t] = a;
  if (t < 64) gw[off[FIRE_P_EN_KERNEL] + (long)J * 64 + t] = b;
  else if (t < 80) gw[off[FIRE_P_EN_BIAS] + (long)J * F0 + (t - 64)] = b;
  else if (t < 112) gw[off[FIRE_P_EN_SCALES] + (long)J * NENV_EN + (t - 80)] = b;
}

// ------------------------------------------------------------------------------------------ host
struct GPlan {
  size_t deg, rowptr, nbr, rev, en_cnt, en_idx, counts, inv;
  size_t enr, h1, xhat, rstd, gb, h2, z3, a3, ei, prr, hc, xs, z1, a1, z2, a2, hf, ex, env, raw, A, Ainv, gjw, ld, sd;
  size_t q, v, att, zm1, am1, zm2, am2, zm3, m3, nrm, Vs, Xr, zo1, ao1, zo2, ao2, x3, seed;
  size_t dhf, draw, denv, dex, dq, dv, d1, d2, dh, dei, dgp, dup, dbs, dbd, px, py, pred, dx3, dzm3, dXr, dzo1,
      dzo2, dg, dh1, dhs, dge, dee, dbe, enx, eny, en2, ered;
  size_t total;
};

GPlan make_gplan(const fire_problem* p, int Wc) {
  GPlan P;
  std::memset(&P, 0, sizeof(P));
  const size_t es = p->precision == FIRE_PREC_FP64 ? 8 : 4;
  const size_t n = p->n_el, N = p->n_nuc, E = p->cap_nuc, cp = p->cap_pairs, W = Wc, G = W * n, DN = NDET * n,
               N8 = N * NENV_ORB, GE = G * E, PC = W * cp;
  size_t o = 0;
  auto take = [&](size_t& field, size_t count, size_t bytes_per) {
    o = (o + 255) / 256 * 256;
    field = o;
    o += count * bytes_per;
  };
  take(P.deg, G, 4);
  take(P.rowptr, W * (n + 1), 4);
  take(P.nbr, PC, 4);
  take(P.rev, PC, 4);
  take(P.en_cnt, G, 4);
  take(P.en_idx, GE, 4);
  take(P.counts, W * 4, 4);
  take(P.inv, G * N, 4);
  take(P.enr, GE * ENW, es);
  take(P.h1, G * F, es);
  take(P.xhat, G * F, es);
  take(P.rstd, G, es);
  take(P.gb, G * 2 * F, es);
  take(P.h2, G * F, es);
  take(P.z3, G * F, es);
  take(P.a3, G * F, es);
  take(P.ei, G * 5 * F, es);
  take(P.prr, PC * PRW, es);
  take(P.hc, G * F, es);
  take(P.xs, G * F, es);
  take(P.z1, G * F, es);
  take(P.a1, G * F, es);
  take(P.z2, G * F, es);
  take(P.a2, G * F, es);
  take(P.hf, G * F, es);
  take(P.ex, NDET * G * N8, es);
  take(P.env, G * DN, es);
  take(P.raw, G * DN, es);
  take(P.A, G * DN, es);
  take(P.Ainv, W * NDET * n * (size_t)ainv_ld((int)n), es);
  take(P.gjw, 2 * W * NDET * n * n, 8);
  take(P.ld, W * NDET, 8);
  take(P.sd, W * NDET, 8);
  take(P.q, G * F, es);
  take(P.v, G * F, es);
  take(P.att, G * HEADS, es);
  take(P.zm1, G * F, es);
  take(P.am1, G * F, es);
  take(P.zm2, G * F, es);
  take(P.am2, G * F, es);
  take(P.zm3, G * 2, es);
  take(P.m3, G * 2, es);
  take(P.nrm, W * 2 * HEADS, es);
  take(P.Vs, W * 2 * F, es);
  take(P.Xr, W * 2 * F, es);
  take(P.zo1, W * F, es);
  take(P.ao1, W * F, es);
  take(P.zo2, W * F, es);
  take(P.ao2, W * F, es);
  take(P.x3, W * 2, es);
  take(P.seed, W * 8, es);
  take(P.dhf, G * F, es);
  take(P.draw, G * DN, es);
  take(P.denv, G * DN, es);
  take(P.dex, NDET * G * N8, es);
  take(P.dq, G * F, es);
  take(P.dv, G * F, es);
  take(P.d1, G * F, es);
  take(P.d2, G * F, es);
  take(P.dh, G * F, es);
  take(P.dei, G * 5 * F, es);
  take(P.dgp, PC * F, es);
  take(P.dup, PC * F, es);
  take(P.dbs, PC * F1, es);
  take(P.dbd, PC * F1, es);
  take(P.px, PC * PX, es);
  take(P.py, PC * PY, es);
  take(P.pred, W * PX * PY, es);
  take(P.dx3, W * 2, es);
  take(P.dzm3, G * 2, es);
  take(P.dXr, W * 2 * F, es);
  take(P.dzo1, W * F, es);
  take(P.dzo2, W * F, es);
  take(P.dg, G * 2 * F, es);
  take(P.dh1, G * F, es);
  take(P.dhs, G * F, es);
  take(P.dge, GE * F, es);
  take(P.dee, GE * F, es);
  take(P.dbe, GE * F1, es);
  take(P.enx, GE * EX, es);
  take(P.eny, GE * EY, es);
  take(P.en2, GE * EN2, es);
  take(P.ered, W * EX * EY, es);
  P.total = (o + 255) / 256 * 256;
  return P;
}

// Walkers per pass: prob->chunk_walkers when its plan fits the workspace (0 when it does not), else the most that fit.
int grad_chunk(const fire_problem* p, size_t ws_bytes) {
  const int B = p->n_walkers;
  if (p->chunk_walkers > 0) {
    const int c = std::min(p->chunk_walkers, B);
    return make_gplan(p, c).total <= ws_bytes ? c : 0;
  }
  int lo = 1, hi = B;
  if (make_gplan(p, 1).total > ws_bytes) return 0;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (make_gplan(p, mid).total <= ws_bytes) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <typename T>
struct G {
  cudaStream_t s;
  unsigned char* ws;
  GPlan P;
  template <typename U>
  U* b(size_t off) const {
    return reinterpret_cast<U*>(ws + off);
  }
};

template <typename T, bool BT = false>
void mm(cudaStream_t s, long M, int N, int K, const T* A, long lda, const T* B, long ldb, const T* bias, T* C,
        long ldc, int acc = 0) {
  if (M <= 0 || N <= 0) return;
  dim3 grid((unsigned)((M + 63) / 64), (unsigned)((N + 63) / 64));
  gk_mm<T, BT><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, bias, C, ldc, acc);
}
// dX = dY W^T for a layer Y = X W with W [K, N] row-major
template <typename T>
void mm_bt(cudaStream_t s, long M, int Kin, int Nout, const T* dY, long ldy, const T* Wt, T* dX, long ldx,
           int acc = 0) {
  mm<T, true>(s, M, Kin, Nout, dY, ldy, Wt, (long)Nout, nullptr, dX, ldx, acc);
}
template <typename T>
void wgrad(cudaStream_t s, int Wc, WgP<T> p) {
  const int Ke = p.K + (p.bias ? 1 : 0);
  if (p.grp <= 0) p.grp = p.K > 0 ? p.K : 1;
  if (Ke <= 16) {
    gk_wgrad_skinny<T><<<dim3((unsigned)((p.N + 63) / 64), 1, (unsigned)Wc), 256, 0, s>>>(p);
    return;
  }
  dim3 grid((unsigned)((p.N + 63) / 64), (unsigned)((Ke + 63) / 64), (unsigned)Wc);
  gk_wgrad<T><<<grid, 256, 0, s>>>(p);
}
// a dense layer's weight (K x N, blob slot wslot) and bias (bslot, or < 0) gradient of walker rows Seg(s)
template <typename T>
WgP<T> wg_layer(const T* X, long ldx, const T* Y, long ldy, Seg s0, Seg s1, int K, int N, T* gbase, long ldg,
                const int64_t* off, int wslot, int bslot) {
  WgP<T> p;
  std::memset(&p, 0, sizeof(p));
  p.X = X; p.ldx = ldx; p.Y = Y; p.ldy = ldy; p.s[0] = s0; p.s[1] = s1; p.K = K; p.N = N;
  p.out = gbase + off[wslot]; p.ldw = ldg; p.ldo = N; p.grp = K; p.grp_stride = (long)K * N;
  p.bias = bslot >= 0 ? gbase + off[bslot] : nullptr;
  return p;
}

template <typename T>
fire_status grad_chunk_run(const fire_problem* p, cudaStream_t s, const float* R, const Weights<T>& W, const T* r,
                           int Wc, int w0, T* sign, T* logpsi, T* grad, long ldg, const int64_t* off_host,
                           const int64_t* off_dev, unsigned char* ws, const GPlan& P, int32_t* status) {
  const int n = p->n_el, nu = p->n_up, nd = n - nu, N = p->n_nuc, E = p->cap_nuc, cp = p->cap_pairs;
  const long G = (long)Wc * n, DN = (long)NDET * n, N8 = (long)N * NENV_ORB, GE = G * E, PC = (long)Wc * cp;
  auto B = [&](size_t o) { return reinterpret_cast<T*>(ws + o); };
  auto I = [&](size_t o) { return reinterpret_cast<int*>(ws + o); };
  T* gb0 = grad + (long)w0 * ldg;  // gradient row of the chunk's first walker
  cudaMemsetAsync(gb0, 0, sizeof(T) * (size_t)Wc * ldg, s);
  // rows that the reductions read must be zero where no edge / pair exists
  cudaMemsetAsync(B(P.enr), 0, sizeof(T) * GE * ENW, s);
  cudaMemsetAsync(B(P.prr), 0, sizeof(T) * PC * PRW, s);
  cudaMemsetAsync(B(P.dgp), 0, sizeof(T) * PC * F, s);
  cudaMemsetAsync(B(P.dup), 0, sizeof(T) * PC * F, s);
  cudaMemsetAsync(B(P.px), 0, sizeof(T) * PC * PX, s);
  cudaMemsetAsync(B(P.py), 0, sizeof(T) * PC * PY, s);
  cudaMemsetAsync(B(P.dge), 0, sizeof(T) * GE * F, s);
  cudaMemsetAsync(B(P.dee), 0, sizeof(T) * GE * F, s);
  cudaMemsetAsync(B(P.enx), 0, sizeof(T) * GE * EX, s);
  cudaMemsetAsync(B(P.eny), 0, sizeof(T) * GE * EY, s);
  cudaMemsetAsync(B(P.en2), 0, sizeof(T) * GE * EN2, s);
  cudaMemsetAsync(I(P.inv), 0xff, sizeof(int) * G * N, s);

  // ---- neighbour lists
  Nbr nb;
  nb.W = Wc; nb.n = n; nb.n_up = nu; nb.N = N; nb.cap_p = cp; nb.cap_nuc = E;
  nb.deg = I(P.deg); nb.rowptr = I(P.rowptr); nb.nbr = I(P.nbr); nb.rev = I(P.rev); nb.en_cnt = I(P.en_cnt);
  nb.en_idx = I(P.en_idx); nb.counts = I(P.counts);
  {
    const size_t smem = 3 * n * sizeof(T) + (5 * n + 2) * sizeof(int);
    cudaFuncSetAttribute(k_neighbors<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    fire_neighbor_out ext;
    std::memset(&ext, 0, sizeof(ext));
    k_neighbors<T><<<Wc, 512, smem, s>>>(r, R, (T)p->cutoff, (T)p->cutoff_1el, nb, ext, status);
  }
  const Seg none{0, 0, 0};
  const Seg el{0, n, n};                         // electron-order rows of a walker
  const Seg up{0, nu, nu}, dn{(long)Wc * nu, nd, nd};  // spin-major rows
  const Seg one{0, 1, 1};
  const T* s0 = W.w[FIRE_P_SCALES];
  const T* s1 = W.w[FIRE_P_SCALES] + 1;

  // ---- forward: ElecInit
  gk_en_fwd<T><<<nb_(GE), 256, 0, s>>>(r, R, nb, W, T(1) / (T)p->cutoff_1el, B(P.enr), I(P.inv));
  gk_en_sum<T><<<(unsigned)G, 256, 0, s>>>(nb, W, B(P.enr), B(P.h1), B(P.xhat), B(P.rstd));
  mm<T>(s, G, 2 * F, F, B(P.h1), F, W.w[FIRE_P_EI_GLU_W], 2 * F, nullptr, B(P.gb), 2 * F);
  gk_glu_fwd<T><<<nb_(G * F), 256, 0, s>>>(B(P.gb), B(P.h2), G);
  mm<T>(s, G, F, F, B(P.h2), F, W.w[FIRE_P_EI_DENSE_W], F, W.w[FIRE_P_EI_DENSE_B], B(P.z3), F);
  gk_silu_fwd<T><<<nb_(G * F), 256, 0, s>>>(B(P.z3), B(P.a3), G * F);
  mm<T>(s, G, 5 * F, F, B(P.a3), F, W.w[FIRE_P_EI_OUT_W], 5 * F, W.w[FIRE_P_EI_OUT_B], B(P.ei), 5 * F);
  // ---- forward: messages and update MLP
  gk_pair_fwd<T><<<nb_(PC), 256, 0, s>>>(r, nb, W, B(P.prr));
  gk_contract_fwd<T><<<(unsigned)G, 256, 0, s>>>(nb, W, B(P.prr), B(P.ei), B(P.hc));
  gk_scale<T><<<nb_(G * F), 256, 0, s>>>(B(P.hc), s0, B(P.xs), G * F);
  mm<T>(s, G, F, F, B(P.xs), F, W.w[FIRE_P_UPD1_W], F, W.w[FIRE_P_UPD1_B], B(P.z1), F);
  gk_silu_fwd<T><<<nb_(G * F), 256, 0, s>>>(B(P.z1), B(P.a1), G * F);
  mm<T>(s, G, F, F, B(P.a1), F, W.w[FIRE_P_UPD2_W], F, W.w[FIRE_P_UPD2_B], B(P.z2), F);
  gk_silu_fwd<T><<<nb_(G * F), 256, 0, s>>>(B(P.z2), B(P.a2), G * F);
  gk_hf<T><<<nb_(G * F), 256, 0, s>>>(B(P.a2), s1, B(P.hf), Wc, n, nu);
  // ---- forward: envelopes, orbital rows and matrices, their inverses
  gk_ex<T><<<nb_(NDET * G * N8), 256, 0, s>>>(r, R, W, Wc, n, nu, N, B(P.ex));
  for (int sp = 0; sp < 2; ++sp) {
    const long ns = sp == 0 ? nu : nd, base = sp == 0 ? 0 : (long)Wc * nu;
    if (ns == 0) continue;
    for (int d = 0; d < NDET; ++d)
      mm<T>(s, Wc * ns, n, (int)N8, B(P.ex) + ((long)d * G + base) * N8, N8,
            W.w[sp == 0 ? PR_ENV_UP_PI : PR_ENV_DN_PI] + (long)d * N8 * n, n, nullptr, B(P.env) + base * DN + d * n,
            DN);
    mm<T>(s, Wc * ns, (int)DN, F, B(P.hf) + base * F, F, W.w[sp == 0 ? FIRE_P_ORB_UP_W : FIRE_P_ORB_DN_W], DN,
          W.w[sp == 0 ? FIRE_P_ORB_UP_B : FIRE_P_ORB_DN_B], B(P.raw) + base * DN, DN);
  }
  gk_amat<T><<<nb_(G * DN), 256, 0, s>>>(B(P.raw), B(P.env), B(P.A), Wc, n, nu);
  {
    using S = typename std::conditional<sizeof(T) == 8, double, df64>::type;
    constexpr int BW = GJG_BW_DECL;
    const size_t smem =
        sizeof(S) * (2 * (size_t)n * (BW + 1) + BW * BW + n + 3 * BW) + sizeof(int) * (2 * (size_t)n + BW);
    auto kern = k_gj_global<S, T, T, true>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return FIRE_ERR_CUDA;
    kern<<<Wc * NDET, GJG_THREADS_DECL, smem, s>>>(B(P.A), (const T*)nullptr, n, reinterpret_cast<S*>(ws + P.gjw),
                                                    reinterpret_cast<double*>(ws + P.ld),
                                                    reinterpret_cast<double*>(ws + P.sd), nullptr, B(P.Ainv), status);
  }
  // ---- forward: Jastrow
  mm<T>(s, G, F, F, B(P.hf), F, W.w[FIRE_P_ATT_Q_W], F, W.w[FIRE_P_ATT_Q_B], B(P.q), F);
  mm<T>(s, G, F, F, B(P.hf), F, W.w[FIRE_P_ATT_V_W], F, W.w[FIRE_P_ATT_V_B], B(P.v), F);
  gk_att<T><<<nb_(G * HEADS), 256, 0, s>>>(B(P.q), W.w[FIRE_P_ATT_KEYS], B(P.att), G);
  mm<T>(s, G, F, F, B(P.hf), F, W.w[FIRE_P_JMLP1_W], F, W.w[FIRE_P_JMLP1_B], B(P.zm1), F);
  gk_silu_fwd<T><<<nb_(G * F), 256, 0, s>>>(B(P.zm1), B(P.am1), G * F);
  mm<T>(s, G, F, F, B(P.am1), F, W.w[FIRE_P_JMLP2_W], F, W.w[FIRE_P_JMLP2_B], B(P.zm2), F);
  gk_silu_fwd<T><<<nb_(G * F), 256, 0, s>>>(B(P.zm2), B(P.am2), G * F);
  mm<T>(s, G, 2, F, B(P.am2), F, W.w[FIRE_P_JMLP3_W], 2, W.w[FIRE_P_JMLP3_B], B(P.zm3), 2);
  gk_silu_fwd<T><<<nb_(G * 2), 256, 0, s>>>(B(P.zm3), B(P.m3), G * 2);
  gk_readout_in<T><<<Wc, 256, 0, s>>>(B(P.att), B(P.v), Wc, n, nu, B(P.nrm), B(P.Vs), B(P.Xr));
  mm<T>(s, Wc, F, 2 * F, B(P.Xr), 2 * F, W.w[FIRE_P_ATT_OUT1_W], F, W.w[FIRE_P_ATT_OUT1_B], B(P.zo1), F);
  gk_silu_fwd<T><<<nb_((long)Wc * F), 256, 0, s>>>(B(P.zo1), B(P.ao1), (long)Wc * F);
  mm<T>(s, Wc, F, F, B(P.ao1), F, W.w[FIRE_P_ATT_OUT2_W], F, W.w[FIRE_P_ATT_OUT2_B], B(P.zo2), F);
  gk_silu_fwd<T><<<nb_((long)Wc * F), 256, 0, s>>>(B(P.zo2), B(P.ao2), (long)Wc * F);
  mm<T>(s, Wc, 2, F, B(P.ao2), F, W.w[FIRE_P_ATT_OUT3_W], 2, W.w[FIRE_P_ATT_OUT3_B], B(P.x3), 2);
  // ---- head
  gk_head<T><<<Wc, 256, 0, s>>>(r, W, Wc, n, nu, reinterpret_cast<double*>(ws + P.ld),
                                reinterpret_cast<double*>(ws + P.sd), B(P.m3), B(P.x3), w0, logpsi, sign, B(P.seed),
                                grad, ldg, off_dev, status);
  gk_jseed<T><<<nb_(G * 2), 256, 0, s>>>(W, B(P.seed), B(P.zm3), Wc, n, nu, B(P.dx3), B(P.dzm3));

  // ---- reverse: readout MLP
  wgrad<T>(s, Wc, wg_layer<T>(B(P.ao2), F, B(P.dx3), 2, one, none, F, 2, gb0, ldg, off_host, FIRE_P_ATT_OUT3_W,
                              FIRE_P_ATT_OUT3_B));
  mm_bt<T>(s, Wc, F, 2, B(P.dx3), 2, W.w[FIRE_P_ATT_OUT3_W], B(P.dzo2), F);
  gk_dsilu<T><<<nb_((long)Wc * F), 256, 0, s>>>(B(P.dzo2), B(P.zo2), B(P.dzo2), (long)Wc * F);
  wgrad<T>(s, Wc, wg_layer<T>(B(P.ao1), F, B(P.dzo2), F, one, none, F, F, gb0, ldg, off_host, FIRE_P_ATT_OUT2_W,
                              FIRE_P_ATT_OUT2_B));
  mm_bt<T>(s, Wc, F, F, B(P.dzo2), F, W.w[FIRE_P_ATT_OUT2_W], B(P.dzo1), F);
  gk_dsilu<T><<<nb_((long)Wc * F), 256, 0, s>>>(B(P.dzo1), B(P.zo1), B(P.dzo1), (long)Wc * F);
  wgrad<T>(s, Wc, wg_layer<T>(B(P.Xr), 2 * F, B(P.dzo1), F, one, none, 2 * F, F, gb0, ldg, off_host,
                              FIRE_P_ATT_OUT1_W, FIRE_P_ATT_OUT1_B));
  mm_bt<T>(s, Wc, 2 * F, F, B(P.dzo1), F, W.w[FIRE_P_ATT_OUT1_W], B(P.dXr), 2 * F);
  // ---- reverse: attention queries and values
  gk_att_bwd<T><<<Wc, 256, 0, s>>>(W, B(P.dXr), B(P.nrm), B(P.Vs), B(P.att), B(P.v), B(P.q), Wc, n, nu, B(P.dq),
                                   B(P.dv), grad, ldg, w0, off_host[FIRE_P_ATT_KEYS]);
  wgrad<T>(s, Wc, wg_layer<T>(B(P.hf), F, B(P.dq), F, up, dn, F, F, gb0, ldg, off_host, FIRE_P_ATT_Q_W,
                              FIRE_P_ATT_Q_B));
  wgrad<T>(s, Wc, wg_layer<T>(B(P.hf), F, B(P.dv), F, up, dn, F, F, gb0, ldg, off_host, FIRE_P_ATT_V_W,
                              FIRE_P_ATT_V_B));
  mm_bt<T>(s, G, F, F, B(P.dq), F, W.w[FIRE_P_ATT_Q_W], B(P.dhf), F);
  mm_bt<T>(s, G, F, F, B(P.dv), F, W.w[FIRE_P_ATT_V_W], B(P.dhf), F, 1);
  // ---- reverse: MLP Jastrow
  wgrad<T>(s, Wc, wg_layer<T>(B(P.am2), F, B(P.dzm3), 2, up, dn, F, 2, gb0, ldg, off_host, FIRE_P_JMLP3_W,
                              FIRE_P_JMLP3_B));
  mm_bt<T>(s, G, F, 2, B(P.dzm3), 2, W.w[FIRE_P_JMLP3_W], B(P.d1), F);
  gk_dsilu<T><<<nb_(G * F), 256, 0, s>>>(B(P.d1), B(P.zm2), B(P.d1), G * F);
  wgrad<T>(s, Wc, wg_layer<T>(B(P.am1), F, B(P.d1), F, up, dn, F, F, gb0, ldg, off_host, FIRE_P_JMLP2_W,
                              FIRE_P_JMLP2_B));
  mm_bt<T>(s, G, F, F, B(P.d1), F, W.w[FIRE_P_JMLP2_W], B(P.d2), F);
  gk_dsilu<T><<<nb_(G * F), 256, 0, s>>>(B(P.d2), B(P.zm1), B(P.d2), G * F);
  wgrad<T>(s, Wc, wg_layer<T>(B(P.hf), F, B(P.d2), F, up, dn, F, F, gb0, ldg, off_host, FIRE_P_JMLP1_W,
                              FIRE_P_JMLP1_B));
  mm_bt<T>(s, G, F, F, B(P.d2), F, W.w[FIRE_P_JMLP1_W], B(P.dhf), F, 1);
  // ---- reverse: determinants -> orbital rows and envelopes
  gk_dA<T><<<nb_(G * DN), 256, 0, s>>>(B(P.Ainv), B(P.seed), B(P.raw), B(P.env), Wc, n, nu, B(P.draw), B(P.denv));
  for (int sp = 0; sp < 2; ++sp) {
    const long ns = sp == 0 ? nu : nd, base = sp == 0 ? 0 : (long)Wc * nu;
    if (ns == 0) continue;
    const Seg sg{base, ns, (int)ns};
    wgrad<T>(s, Wc, wg_layer<T>(B(P.hf), F, B(P.draw), DN, sg, none, F, (int)DN, gb0, ldg, off_host,
                                sp == 0 ? FIRE_P_ORB_UP_W : FIRE_P_ORB_DN_W, sp == 0 ? FIRE_P_ORB_UP_B : FIRE_P_ORB_DN_B));
    mm_bt<T>(s, Wc * ns, F, (int)DN, B(P.draw) + base * DN, DN, W.w[sp == 0 ? FIRE_P_ORB_UP_W : FIRE_P_ORB_DN_W],
             B(P.dhf) + base * F, F, 1);
    const T* pi = W.w[sp == 0 ? PR_ENV_UP_PI : PR_ENV_DN_PI];
    for (int d = 0; d < NDET; ++d) {
      // d ex = d env . pi^T (pi per determinant [N8, n]);  d pi = ex^T d env, into the blob layout [N, D, 8, n]
      mm<T, true>(s, Wc * ns, (int)N8, n, B(P.denv) + base * DN + d * n, DN, pi + (long)d * N8 * n, n, nullptr,
                  B(P.dex) + ((long)d * G + base) * N8, N8);
      WgP<T> q;
      std::memset(&q, 0, sizeof(q));
      q.X = B(P.ex) + (long)d * G * N8; q.ldx = N8; q.Y = B(P.denv) + d * n; q.ldy = DN;
      q.s[0] = sg; q.s[1] = none; q.K = (int)N8; q.N = n;
      q.out = gb0 + off_host[sp == 0 ? FIRE_P_ENV_UP_PI : FIRE_P_ENV_DN_PI] + (long)d * NENV_ORB * n;
      q.ldw = ldg; q.ldo = n; q.grp = NENV_ORB; q.grp_stride = (long)NDET * NENV_ORB * n;
      wgrad<T>(s, Wc, q);
    }
  }
  gk_dsigma<T><<<dim3(Wc, 2), 256, 0, s>>>(r, R, W, B(P.ex), B(P.dex), Wc, n, nu, N, grad, ldg, w0,
                                           off_host[FIRE_P_ENV_UP_SIGMA], off_host[FIRE_P_ENV_DN_SIGMA]);
  // ---- reverse: update MLP and the normalisation scales
  gk_hf_bwd<T><<<Wc, 256, 0, s>>>(B(P.dhf), B(P.a2), s1, Wc, n, nu, B(P.d1), grad, ldg, w0,
                                  off_host[FIRE_P_SCALES] + 1);
  gk_dsilu<T><<<nb_(G * F), 256, 0, s>>>(B(P.d1), B(P.z2), B(P.d1), G * F);
  wgrad<T>(s, Wc, wg_layer<T>(B(P.a1), F, B(P.d1), F, el, none, F, F, gb0, ldg, off_host, FIRE_P_UPD2_W,
                              FIRE_P_UPD2_B));
  mm_bt<T>(s, G, F, F, B(P.d1), F, W.w[FIRE_P_UPD2_W], B(P.d2), F);
  gk_dsilu<T><<<nb_(G * F), 256, 0, s>>>(B(P.d2), B(P.z1), B(P.d2), G * F);
  wgrad<T>(s, Wc, wg_layer<T>(B(P.xs), F, B(P.d2), F, el, none, F, F, gb0, ldg, off_host, FIRE_P_UPD1_W,
                              FIRE_P_UPD1_B));
  mm_bt<T>(s, G, F, F, B(P.d2), F, W.w[FIRE_P_UPD1_W], B(P.d1), F);
  gk_s0_bwd<T><<<Wc, 256, 0, s>>>(B(P.d1), B(P.hc), s0, n, B(P.dh), grad, ldg, w0, off_host[FIRE_P_SCALES]);
  // ---- reverse: messages of the e-e pairs
  gk_pair_bwd<T><<<(unsigned)G, 256, 0, s>>>(nb, W, B(P.prr), B(P.ei), B(P.dh), B(P.dgp), B(P.dup));
  gk_dei<T><<<(unsigned)G, 256, 0, s>>>(nb, B(P.prr), B(P.dh), B(P.dup), B(P.dei));
  {
    const Seg pr{0, cp, cp};
    WgP<T> q;
    std::memset(&q, 0, sizeof(q));
    // gamma_W of both tags: X = [beta (same) | beta (diff)] (16 columns), rows 0-7 -> same, 8-15 -> diff
    q.X = B(P.prr) + 56; q.ldx = PRW; q.Y = B(P.dgp); q.ldy = F; q.s[0] = pr; q.s[1] = none; q.K = 2 * F1; q.N = F;
    q.out = gb0 + off_host[FIRE_P_EESAME_GAMMA_W]; q.ldw = ldg; q.ldo = F; q.grp = F1;
    q.grp_stride = off_host[FIRE_P_EEDIFF_GAMMA_W] - off_host[FIRE_P_EESAME_GAMMA_W];
    wgrad<T>(s, Wc, q);
    // edge_W and edge_b of both tags: X = [scaled, 1] per tag (10 columns); edge_b follows edge_W in the blob
    q.X = B(P.prr) + 72; q.Y = B(P.dup); q.K = 10; q.grp = 5;
    q.out = gb0 + off_host[FIRE_P_EESAME_EDGE_W];
    q.grp_stride = off_host[FIRE_P_EEDIFF_EDGE_W] - off_host[FIRE_P_EESAME_EDGE_W];
    wgrad<T>(s, Wc, q);
    mm_bt<T>(s, PC, F1, F, B(P.dgp), F, W.w[FIRE_P_EESAME_GAMMA_W], B(P.dbs), F1);
    mm_bt<T>(s, PC, F1, F, B(P.dgp), F, W.w[FIRE_P_EEDIFF_GAMMA_W], B(P.dbd), F1);
    gk_pair_small_bwd<T><<<nb_(PC), 256, 0, s>>>(nb, W, B(P.prr), B(P.dbs), B(P.dbd), B(P.px), B(P.py));
    std::memset(&q, 0, sizeof(q));
    q.X = B(P.px); q.ldx = PX; q.Y = B(P.py); q.ldy = PY; q.s[0] = pr; q.s[1] = none; q.K = PX; q.N = PY;
    q.out = B(P.pred); q.ldw = (long)PX * PY; q.ldo = PY; q.grp = PX; q.grp_stride = (long)PX * PY;
    wgrad<T>(s, Wc, q);
    gk_pair_small_scatter<T><<<Wc, 256, 0, s>>>(B(P.pred), Wc, grad, ldg, w0, off_dev);
  }
  // ---- reverse: ElecInit
  wgrad<T>(s, Wc, wg_layer<T>(B(P.a3), F, B(P.dei), 5 * F, el, none, F, 5 * F, gb0, ldg, off_host, FIRE_P_EI_OUT_W,
                              FIRE_P_EI_OUT_B));
  mm_bt<T>(s, G, F, 5 * F, B(P.dei), 5 * F, W.w[FIRE_P_EI_OUT_W], B(P.d1), F);
  gk_dsilu<T><<<nb_(G * F), 256, 0, s>>>(B(P.d1), B(P.z3), B(P.d1), G * F);
  wgrad<T>(s, Wc, wg_layer<T>(B(P.h2), F, B(P.d1), F, el, none, F, F, gb0, ldg, off_host, FIRE_P_EI_DENSE_W,
                              FIRE_P_EI_DENSE_B));
  mm_bt<T>(s, G, F, F, B(P.d1), F, W.w[FIRE_P_EI_DENSE_W], B(P.d2), F);
  gk_glu_bwd<T><<<nb_(G * F), 256, 0, s>>>(B(P.gb), B(P.d2), B(P.dg), G);
  wgrad<T>(s, Wc, wg_layer<T>(B(P.h1), F, B(P.dg), 2 * F, el, none, F, 2 * F, gb0, ldg, off_host, FIRE_P_EI_GLU_W,
                              -1));
  mm_bt<T>(s, G, F, 2 * F, B(P.dg), 2 * F, W.w[FIRE_P_EI_GLU_W], B(P.dh1), F);
  gk_ln_bwd<T><<<(unsigned)G, 256, 0, s>>>(W, B(P.dh1), B(P.xhat), B(P.rstd), B(P.dhs));
  gk_ln_params<T><<<Wc, 256, 0, s>>>(B(P.dh1), B(P.xhat), n, grad, ldg, w0, off_host[FIRE_P_EI_LN_SCALE],
                                     off_host[FIRE_P_EI_LN_BIAS]);
  gk_en_bwd_rows<T><<<(unsigned)G, 256, 0, s>>>(nb, W, B(P.enr), B(P.dhs), B(P.dge), B(P.dee));
  {
    const Seg er{0, (long)n * E, n * E};
    WgP<T> q;
    std::memset(&q, 0, sizeof(q));
    q.X = B(P.enr) + 72; q.ldx = ENW; q.Y = B(P.dge); q.ldy = F; q.s[0] = er; q.s[1] = none; q.K = F1; q.N = F;
    q.out = gb0 + off_host[FIRE_P_EI_GAMMA_W]; q.ldw = ldg; q.ldo = F; q.grp = F1; q.grp_stride = (long)F1 * F;
    wgrad<T>(s, Wc, q);
    q.X = B(P.enr) + 68; q.Y = B(P.dee); q.K = 4; q.grp = 4; q.grp_stride = 4L * F;
    q.out = gb0 + off_host[FIRE_P_EI_EDGE_W];
    wgrad<T>(s, Wc, q);
    mm_bt<T>(s, GE, F1, F, B(P.dge), F, W.w[FIRE_P_EI_GAMMA_W], B(P.dbe), F1);
    gk_en_small_bwd<T><<<nb_(GE), 256, 0, s>>>(nb, W, B(P.enr), B(P.dbe), B(P.enx), B(P.eny), B(P.en2));
    std::memset(&q, 0, sizeof(q));
    q.X = B(P.enx); q.ldx = EX; q.Y = B(P.eny); q.ldy = EY; q.s[0] = er; q.s[1] = none; q.K = EX; q.N = EY;
    q.out = B(P.ered); q.ldw = (long)EX * EY; q.ldo = EY; q.grp = EX; q.grp_stride = (long)EX * EY;
    wgrad<T>(s, Wc, q);
    gk_en_small_scatter<T><<<Wc, 256, 0, s>>>(B(P.ered), grad, ldg, w0, off_dev);
    gk_en_nuc<T><<<dim3(N, Wc), 256, 0, s>>>(nb, B(P.enr), B(P.dee), B(P.en2), I(P.inv), grad, ldg, w0, off_dev);
  }
  return cudaPeekAtLastError() == cudaSuccess ? FIRE_OK : FIRE_ERR_CUDA;
}

template <typename T>
fire_status run_grad(const fire_problem* p, cudaStream_t s, const float* R, const void* prepared, const void* r,
                     void* sign, void* logpsi, void* grad, void* ws, size_t ws_bytes, int32_t* status) {
  const int Wc = grad_chunk(p, ws_bytes);
  if (Wc <= 0) return FIRE_ERR_WORKSPACE;
  const GPlan P = make_gplan(p, Wc);
  int64_t off[PR_COUNT + 1];
  prep_offsets_host(p, off);
  Weights<T> W;
  const T* base = reinterpret_cast<const T*>(prepared);
  for (int k = 0; k < PR_COUNT; ++k) W.w[k] = base + off[k];
  const long ldg = off[FIRE_P_COUNT];
  // the blob offsets the scatter kernels read on the device live at the end of the workspace plan
  unsigned char* wsb = reinterpret_cast<unsigned char*>(ws);
  int64_t* off_dev = reinterpret_cast<int64_t*>(wsb + P.total);
  cudaMemcpyAsync(off_dev, off, sizeof(int64_t) * (FIRE_P_COUNT + 1), cudaMemcpyHostToDevice, s);
  for (int w0 = 0; w0 < p->n_walkers; w0 += Wc) {
    const int Wn = std::min(Wc, p->n_walkers - w0);
    const fire_status e = grad_chunk_run<T>(p, s, R, W, reinterpret_cast<const T*>(r) + (long)w0 * p->n_el * 3, Wn,
                                            w0, reinterpret_cast<T*>(sign), reinterpret_cast<T*>(logpsi),
                                            reinterpret_cast<T*>(grad), ldg, off, off_dev, wsb, P, status);
    if (e != FIRE_OK) return e;
  }
  return FIRE_OK;
}

}  // namespace

// bytes of the gradient workspace (plan plus the device copy of the blob offsets)
size_t grad_workspace_bytes(const fire_problem* p, int chunk) {
  const int Wc = chunk > 0 ? std::min(chunk, p->n_walkers) : p->n_walkers;
  return make_gplan(p, Wc).total + 256 * ((sizeof(int64_t) * (FIRE_P_COUNT + 1) + 255) / 256);
}

fire_status grad_dispatch(const fire_problem* p, cudaStream_t s, const float* R, const void* prepared, const void* r,
                          void* sign, void* logpsi, void* grad, void* ws, size_t ws_bytes, int32_t* status) {
  const size_t tail = 256 * ((sizeof(int64_t) * (FIRE_P_COUNT + 1) + 255) / 256);
  if (ws_bytes < tail) return FIRE_ERR_WORKSPACE;
  if (p->precision == FIRE_PREC_FP64)
    return run_grad<double>(p, s, R, prepared, r, sign, logpsi, grad, ws, ws_bytes - tail, status);
  return run_grad<float>(p, s, R, prepared, r, sign, logpsi, grad, ws, ws_bytes - tail, status);
}

}  // namespace fire
