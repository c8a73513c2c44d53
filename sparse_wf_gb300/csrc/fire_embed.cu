// fire_embed.cu -- the new_sparse embedding up to the update MLP.
//
//  k_elec_init   ElecInit (model/new_sparse_model.py:190-215): per electron, the e-n edges
//                (ElecNucEdge 139-158 with PairwiseFilter, model/utils.py:393-433) are reduced to
//                h = sum_J Gamma_J * e_J and layer-normalised.  With NT = 3 every value carries its
//                forward-Laplacian tangents w.r.t. the electron's own position (the jax.vmap(fwd_lap)
//                of new_sparse_model.py:648-650); NT = 0 is the value path (new_sparse_model.py:507-519).
//  k_glu / k_silu5  the GatedLinearUnit and Dense+SiLU of ElecInit on the [x, jac(3), lap] rows.
//  k_edge_contract  ElecElecEdges (161-187) + contract_with_fwd_lap (95-131): per center i the
//                messages Gamma_ij * silu(e_ij + h_ct[i] + h_nb[j]) with 6 tangents (center and
//                neighbour coordinates) are summed into h[i]; d msg / d r_j becomes the Jacobian row of
//                the pair (i, j) and d msg / d r_i accumulates into the self row.
#include "fire_internal.cuh"

namespace fire {

template <typename T, int NT>
struct FLv {
  T x, l;
  T j[NT > 0 ? NT : 1];
};

template <typename T, int NT>
__device__ __forceinline__ void fl_zero(FLv<T, NT>& a) {
  a.x = T(0);
  a.l = T(0);
#pragma unroll
  for (int t = 0; t < NT; ++t) a.j[t] = T(0);
}
template <typename T, int NT>
__device__ __forceinline__ FLv<T, NT> fl_apply(const FLv<T, NT>& a, T f, T f1, T f2) {
  FLv<T, NT> r;
  r.x = f;
  T sq = T(0);
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    r.j[t] = f1 * a.j[t];
    sq += a.j[t] * a.j[t];
  }
  r.l = f1 * a.l + f2 * sq;
  return r;
}
template <typename T, int NT>
__device__ __forceinline__ FLv<T, NT> fl_mul(const FLv<T, NT>& a, const FLv<T, NT>& b) {
  FLv<T, NT> r;
  r.x = a.x * b.x;
  T c = T(0);
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    r.j[t] = a.j[t] * b.x + a.x * b.j[t];
    c += a.j[t] * b.j[t];
  }
  r.l = a.l * b.x + a.x * b.l + T(2) * c;
  return r;
}
template <typename T, int NT>
__device__ __forceinline__ void fl_axpy(FLv<T, NT>& acc, T c, const FLv<T, NT>& a) {
  acc.x += c * a.x;
  acc.l += c * a.l;
#pragma unroll
  for (int t = 0; t < NT; ++t) acc.j[t] += c * a.j[t];
}
template <typename T, int NT>
__device__ __forceinline__ FLv<T, NT> fl_silu(const FLv<T, NT>& a) {
  T y, d1, d2;
  silu3(a.x, y, d1, d2);
  return fl_apply(a, y, d1, d2);
}
// number of stored rows of a carrier: x, j[NT], l (value path: x only)
template <int NT>
struct NVr {
  static constexpr int v = NT > 0 ? NT + 2 : 1;
};
template <typename T, int NT>
__device__ __forceinline__ void fl_store(T* dst, int stride, const FLv<T, NT>& a) {
  dst[0] = a.x;
  if (NT > 0) {
#pragma unroll
    for (int t = 0; t < NT; ++t) dst[(1 + t) * stride] = a.j[t];
    dst[(NT + 1) * stride] = a.l;
  }
}
template <typename T, int NT>
__device__ __forceinline__ FLv<T, NT> fl_load(const T* src, int stride) {
  FLv<T, NT> a;
  a.x = src[0];
  a.l = T(0);
  if (NT > 0) {
#pragma unroll
    for (int t = 0; t < NT; ++t) a.j[t] = src[(1 + t) * stride];
    a.l = src[(NT + 1) * stride];
  }
  return a;
}

// Edge features and the filter of one edge, computed by one warp.  NT = 3: e-n edge (tangents =
// electron coordinates); NT = 6: e-e edge (tangents 0..2 center, 3..5 neighbour).  Writes
// beta[8] to sB[v * 8 + c] and the log-scaled features to sS[v * 4 + k], v over the stored rows.
template <typename T, int NT, int NENV>
__device__ __forceinline__ void edge_filter_warp(const T diff[3], const T* K /*[4][16]*/, const T* bias /*[16]*/,
                                                 const T* inv_scale /*[NENV]*/, const T* dir_W /*[16][8]*/,
                                                 const T* dir_b /*[8]*/, const T* env_W /*[NENV][8]*/,
                                                 T inv_cutoff, FLv<T, NT>* wS /*[16]*/, FLv<T, NT>* wE /*[32]*/,
                                                 T* sB, T* sS) {
  constexpr int NV = NVr<NT>::v;
  const int lane = threadIdx.x & 31;
  // distance carrier
  const T s2 = diff[0] * diff[0] + diff[1] * diff[1] + diff[2] * diff[2];
  const T d = dsqrt(s2);
  FLv<T, NT> fd;
  fd.x = d;
  fl_zero(fd);
  fd.x = d;
  if (NT > 0) {
    const T id = T(1) / d;
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      fd.j[t] = diff[t] * id;
      if (NT == 6) fd.j[3 + t] = -diff[t] * id;
    }
    fd.l = (NT == 6 ? T(4) : T(2)) * id;
  }
  auto feat = [&](int k) -> FLv<T, NT> {
    if (k == 0) return fd;
    FLv<T, NT> f;
    fl_zero(f);
    f.x = diff[k - 1];
    if (NT > 0) {
      f.j[k - 1] = T(1);
      if (NT == 6) f.j[k + 2] = T(-1);
    }
    return f;
  };
  if (lane < F0) {
    FLv<T, NT> pre;
    fl_zero(pre);
    pre.x = bias[lane];
#pragma unroll
    for (int k = 0; k < 4; ++k) fl_axpy(pre, K[k * F0 + lane], feat(k));
    wS[lane] = fl_silu(pre);
  }
  if (lane < NENV) {
    const T a = inv_scale[lane];
    const T u = d * a;
    const T g = dexp(-u * u);
    const T g1 = T(-2) * u * a * g;
    const T g2 = (T(4) * u * u * a * a - T(2) * a * a) * g;
    T c, c1, c2;
    cutoff3(d * inv_cutoff, c, c1, c2);
    c1 *= inv_cutoff;
    c2 *= inv_cutoff * inv_cutoff;
    wE[lane] = fl_apply(fd, g * c, g1 * c + g * c1, g2 * c + T(2) * g1 * c1 + g * c2);
  }
  __syncwarp();
  if (lane < F1) {
    FLv<T, NT> dirv, env8;
    fl_zero(dirv);
    fl_zero(env8);
    dirv.x = dir_b[lane];
#pragma unroll
    for (int l = 0; l < F0; ++l) fl_axpy(dirv, dir_W[l * F1 + lane], wS[l]);
#pragma unroll 8
    for (int k = 0; k < NENV; ++k) fl_axpy(env8, env_W[k * F1 + lane], wE[k]);
    const FLv<T, NT> beta = fl_mul(dirv, env8);
    fl_store(sB + lane, F1, beta);
  } else if (lane < F1 + 4) {
    const int k = lane - F1;
    const T lp = dlog1p(d);
    FLv<T, NT> sf;
    if (k == 0) {
      const T q = T(1) / (T(1) + d);
      sf = fl_apply(fd, lp, q, -q * q);
    } else {
      const T id = T(1) / d;
      const T L1 = T(1) / (T(1) + d), L2 = -L1 * L1;
      const T psi = lp * id;
      const T psi1 = L1 * id - lp * id * id;
      const T psi2 = L2 * id - T(2) * L1 * id * id + T(2) * lp * id * id * id;
      sf = fl_mul(feat(k), fl_apply(fd, psi, psi1, psi2));
    }
    fl_store(sS + k, 4, sf);
  }
  __syncwarp();
  (void)NV;
}

constexpr int EB = 32;  // edges staged per batch

// One CTA (256 threads, thread = feature) per electron.  Output E5 [G][NV][F] (x, jac xyz, lap).
template <typename T, int NT>
__global__ void __launch_bounds__(256) k_elec_init(const T* __restrict__ r, const float* __restrict__ R,
                                                   Nbr nb, Weights<T> W, T inv_cutoff1, T* __restrict__ E5) {
  constexpr int NV = NVr<NT>::v;
  __shared__ T sB[EB][NV * F1];
  __shared__ T sS[EB][NV * 4];
  __shared__ int sJ[EB];
  __shared__ FLv<T, NT> wS[8][F0];
  __shared__ FLv<T, NT> wE[8][NENV_EN];
  __shared__ T red[32 * 6];
  const int g = blockIdx.x, f = threadIdx.x, lane = f & 31, wid = f >> 5;
  const int ne = nb.en_cnt[g];
  const int* eidx = nb.en_idx + (size_t)g * nb.cap_nuc;
  const T rx = r[3 * g], ry = r[3 * g + 1], rz = r[3 * g + 2];
  const T* Wg = W.w[FIRE_P_EI_GAMMA_W];
  const T* We = W.w[FIRE_P_EI_EDGE_W];
  T wg[F1], we[4];
#pragma unroll
  for (int c = 0; c < F1; ++c) wg[c] = Wg[c * F + f];
#pragma unroll
  for (int k = 0; k < 4; ++k) we[k] = We[k * F + f];
  FLv<T, NT> h;
  fl_zero(h);
  for (int e0 = 0; e0 < ne; e0 += EB) {
    const int nbe = min(EB, ne - e0);
    for (int e = wid; e < nbe; e += 8) {
      const int J = eidx[e0 + e];
      const T diff[3] = {rx - (T)R[3 * J], ry - (T)R[3 * J + 1], rz - (T)R[3 * J + 2]};
      edge_filter_warp<T, NT, NENV_EN>(diff, W.w[FIRE_P_EN_KERNEL] + J * 4 * F0, W.w[FIRE_P_EN_BIAS] + J * F0,
                                       W.w[PR_EN_INVSCALE] + J * NENV_EN, W.w[FIRE_P_EI_DIR_W],
                                       W.w[FIRE_P_EI_DIR_B], W.w[FIRE_P_EI_ENV_W], inv_cutoff1, wS[wid], wE[wid],
                                       sB[e], sS[e]);
      if (lane == 0) sJ[e] = J;
    }
    __syncthreads();
    const T* hn = W.w[FIRE_P_EN_NUC_EMB];
    for (int e = 0; e < nbe; ++e) {
      FLv<T, NT> G, E;
      fl_zero(G);
      fl_zero(E);
#pragma unroll
      for (int c = 0; c < F1; ++c) {
        const FLv<T, NT> b = fl_load<T, NT>(&sB[e][c], F1);
        fl_axpy(G, wg[c], b);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const FLv<T, NT> s = fl_load<T, NT>(&sS[e][k], 4);
        fl_axpy(E, we[k], s);
      }
      E.x += hn[sJ[e] * F + f];
      const FLv<T, NT> m = fl_mul(G, E);
      h.x += m.x;
      h.l += m.l;
#pragma unroll
      for (int t = 0; t < NT; ++t) h.j[t] += m.j[t];
    }
    __syncthreads();
  }
  // LayerNorm (flax, eps = 1e-6) with forward-Laplacian propagation
  const T invF = T(1) / T(F);
  const T gam = W.w[FIRE_P_EI_LN_SCALE][f], bet = W.w[FIRE_P_EI_LN_BIAS][f];
  FLv<T, NT> y;
  if (NT == 0) {
    T v1[1] = {h.x};
    block_sum<T, 1>(v1, red);
    const T c = h.x - v1[0] * invF;
    T v2[1] = {c * c};
    block_sum<T, 1>(v2, red);
    const T s = T(1) / dsqrt(v2[0] * invF + T(1e-6));
    fl_zero(y);
    y.x = gam * c * s + bet;
  } else {
    T v1[5];
    v1[0] = h.x;
#pragma unroll
    for (int t = 0; t < 3; ++t) v1[1 + t] = h.j[t];
    v1[4] = h.l;
    block_sum<T, 5>(v1, red);
    const T c = h.x - v1[0] * invF;
    T cj[3];
#pragma unroll
    for (int t = 0; t < 3; ++t) cj[t] = h.j[t] - v1[1 + t] * invF;
    const T cl = h.l - v1[4] * invF;
    T v2[6];
    v2[0] = c * c;
#pragma unroll
    for (int t = 0; t < 3; ++t) v2[1 + t] = c * cj[t];
    v2[4] = cj[0] * cj[0] + cj[1] * cj[1] + cj[2] * cj[2];
    v2[5] = c * cl;
    block_sum<T, 6>(v2, red);
    const T var = v2[0] * invF;
    const T s = T(1) / dsqrt(var + T(1e-6));
    const T s3 = s * s * s, s5 = s3 * s * s;
    T vj[3], sj[3], vjsq = T(0);
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      vj[t] = T(2) * v2[1 + t] * invF;
      sj[t] = T(-0.5) * s3 * vj[t];
      vjsq += vj[t] * vj[t];
    }
    const T vtt = T(2) * (v2[4] + v2[5]) * invF;
    const T stt = T(0.75) * s5 * vjsq - T(0.5) * s3 * vtt;
    y.x = gam * c * s + bet;
    T cross = T(0);
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      y.j[t] = gam * (cj[t] * s + c * sj[t]);
      cross += cj[t] * sj[t];
    }
    y.l = gam * (cl * s + T(2) * cross + c * stt);
  }
  fl_store(E5 + (size_t)g * NV * F + f, F, y);
}

// out[g][v][f] = a * silu(gate) with a = Z[g][v][f], gate = Z[g][v][F + f]   (GatedLinearUnit)
template <typename T, int NT>
__global__ void k_glu(const T* __restrict__ Z, T* __restrict__ out, int G) {
  constexpr int NV = NVr<NT>::v;
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)G * F) return;
  const long g = idx / F;
  const int f = (int)(idx - g * F);
  const FLv<T, NT> a = fl_load<T, NT>(Z + g * NV * 2 * F + f, 2 * F);
  const FLv<T, NT> b = fl_load<T, NT>(Z + g * NV * 2 * F + F + f, 2 * F);
  fl_store(out + g * NV * F + f, F, fl_mul(a, fl_silu(b)));
}

// in-place silu on carriers [G][NV][F]
template <typename T, int NT>
__global__ void k_silu5(T* __restrict__ Z, int G) {
  constexpr int NV = NVr<NT>::v;
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)G * F) return;
  const long g = idx / F;
  const int f = (int)(idx - g * F);
  const FLv<T, NT> a = fl_load<T, NT>(Z + g * NV * F + f, F);
  fl_store(Z + g * NV * F + f, F, fl_silu(a));
}

// One CTA (256 threads) per center electron g.  E5o: [G][NV][5F] = h0 | ct_same | ct_diff | nb_same | nb_diff.
// Outputs X [G][F], Lp [G][F] (if NT) and the Jacobian plane Jp [3 * positions][F] (if NT).
template <typename T, int NT>
__global__ void __launch_bounds__(256) k_edge_contract(const T* __restrict__ r, Nbr nb, Layout L, Weights<T> W,
                                                       const T* __restrict__ E5o, T* __restrict__ X,
                                                       T* __restrict__ Lp, T* __restrict__ Jp) {
  constexpr int NV = NVr<NT>::v;       // rows of the electron carriers (NT_e = 3 tangents)
  constexpr int NT6 = NT > 0 ? 6 : 0;  // pair carriers
  constexpr int NV6 = NVr<NT6>::v;
  __shared__ T sB[EB][NV6 * F1];
  __shared__ T sS[EB][NV6 * 4];
  __shared__ int sj[EB];
  __shared__ FLv<T, NT6> wS[8][F0];
  __shared__ FLv<T, NT6> wE[8][NENV_EE];
  const int g = blockIdx.x, f = threadIdx.x, lane = f & 31, wid = f >> 5;
  const int n = nb.n, w = g / n, i = g - w * n;
  const int* rp = nb.rowptr + (size_t)w * (n + 1);
  const int P = rp[n];
  if (P > nb.cap_p) return;
  const int deg = rp[i + 1] - rp[i];
  const int* nbl = nb.nbr + (size_t)w * nb.cap_p + rp[i];
  const bool si = i < nb.n_up;
  const T cutoff_eff = W.w[PR_SCALARS][0];
  const T inv_c = T(1) / cutoff_eff;
  const T rx = r[3 * g], ry = r[3 * g + 1], rz = r[3 * g + 2];
  T wg[2][F1], we[2][4], be[2];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const T* Wg = W.w[s == 0 ? FIRE_P_EESAME_GAMMA_W : FIRE_P_EEDIFF_GAMMA_W];
    const T* We = W.w[s == 0 ? FIRE_P_EESAME_EDGE_W : FIRE_P_EEDIFF_EDGE_W];
#pragma unroll
    for (int c = 0; c < F1; ++c) wg[s][c] = Wg[c * F + f];
#pragma unroll
    for (int k = 0; k < 4; ++k) we[s][k] = We[k * F + f];
    be[s] = W.w[s == 0 ? FIRE_P_EESAME_EDGE_B : FIRE_P_EEDIFF_EDGE_B][f];
  }
  const T* eg = E5o + (size_t)g * NV * 5 * F;
  const FLv<T, NT> h0 = fl_load<T, NT>(eg + f, 5 * F);
  const FLv<T, NT> cts = fl_load<T, NT>(eg + F + f, 5 * F);
  const FLv<T, NT> ctd = fl_load<T, NT>(eg + 2 * F + f, 5 * F);
  T ax = T(0), al = T(0), aj[3] = {T(0), T(0), T(0)};
  const long q0 = NT > 0 ? (long)L.pos_off[w] + rp[i] + i : 0;
  for (int k0 = 0; k0 < deg; k0 += EB) {
    const int nbe = min(EB, deg - k0);
    for (int e = wid; e < nbe; e += 8) {
      const int j = nbl[k0 + e];
      const int gj = w * n + j;
      const T diff[3] = {rx - r[3 * gj], ry - r[3 * gj + 1], rz - r[3 * gj + 2]};
      const bool same = (j < nb.n_up) == si;
      if (same)
        edge_filter_warp<T, NT6, NENV_EE>(diff, W.w[FIRE_P_EESAME_KERNEL], W.w[FIRE_P_EESAME_BIAS],
                                          W.w[PR_EESAME_INVSCALE], W.w[FIRE_P_EESAME_DIR_W],
                                          W.w[FIRE_P_EESAME_DIR_B], W.w[FIRE_P_EESAME_ENV_W], inv_c, wS[wid],
                                          wE[wid], sB[e], sS[e]);
      else
        edge_filter_warp<T, NT6, NENV_EE>(diff, W.w[FIRE_P_EEDIFF_KERNEL], W.w[FIRE_P_EEDIFF_BIAS],
                                          W.w[PR_EEDIFF_INVSCALE], W.w[FIRE_P_EEDIFF_DIR_W],
                                          W.w[FIRE_P_EEDIFF_DIR_B], W.w[FIRE_P_EEDIFF_ENV_W], inv_c, wS[wid],
                                          wE[wid], sB[e], sS[e]);
      if (lane == 0) sj[e] = same ? j : -1 - j;
    }
    __syncthreads();
    for (int e = 0; e < nbe; ++e) {
      const int code = sj[e];
      const bool same = code >= 0;
      const int j = same ? code : -1 - code;
      const int s = same ? 0 : 1;
      FLv<T, NT6> G, E;
      fl_zero(G);
      fl_zero(E);
#pragma unroll
      for (int c = 0; c < F1; ++c) fl_axpy(G, wg[s][c], fl_load<T, NT6>(&sB[e][c], F1));
#pragma unroll
      for (int k = 0; k < 4; ++k) fl_axpy(E, we[s][k], fl_load<T, NT6>(&sS[e][k], 4));
      E.x += be[s];
      // u = e + h_ct[i] (tangents 0..2) + h_nb[j] (tangents 3..5)
      const FLv<T, NT>& ct = same ? cts : ctd;
      const FLv<T, NT> hn = fl_load<T, NT>(E5o + (size_t)(w * n + j) * NV * 5 * F + (same ? 3 : 4) * F + f, 5 * F);
      FLv<T, NT6> u = E;
      u.x += ct.x + hn.x;
      if (NT > 0) {
        u.l += ct.l + hn.l;
#pragma unroll
        for (int t = 0; t < 3; ++t) {
          u.j[t] += ct.j[t];
          u.j[3 + t] += hn.j[t];
        }
      }
      const FLv<T, NT6> msg = fl_mul(G, fl_silu(u));
      ax += msg.x;
      if (NT > 0) {
        al += msg.l;
#pragma unroll
        for (int t = 0; t < 3; ++t) aj[t] += msg.j[t];
        const long q = q0 + 1 + k0 + e;
#pragma unroll
        for (int t = 0; t < 3; ++t) Jp[(3 * q + t) * F + f] = msg.j[3 + t];
      }
    }
    __syncthreads();
  }
  X[(size_t)g * F + f] = h0.x + ax;
  if (NT > 0) {
    Lp[(size_t)g * F + f] = h0.l + al;
#pragma unroll
    for (int t = 0; t < 3; ++t) Jp[(3 * q0 + t) * F + f] = h0.j[t] + aj[t];
  }
}

// Low-rank step, value path (NewSparseEmbedding.low_rank_update, new_sparse_model.py:553-629): one CTA (256
// threads, thread = feature) per changed center c = S[w][slot] of walker w.  Its neighbours are taken in the proposed
// configuration rn, ascending like the pair list, and the messages are those of k_edge_contract; the ElecInit rows
// (h0 | ct_same | ct_diff | nb_same | nb_diff) come from the state E5 [W][n][5F] except for the moved electrons
// moved[w][0..KM), whose rows are E5p [W][KM][5F].  Output HS [W][KS][F] = h0[c] + sum of the messages (before the update MLP).
template <typename T>
__global__ void __launch_bounds__(256) k_lr_contract(const T* __restrict__ rn, int n, int n_up, T cutoff,
                                                     const int* __restrict__ moved, int KM, const int* __restrict__ S,
                                                     const int* __restrict__ S_cnt, int KS,
                                                     Weights<T> W, const T* __restrict__ E5, const T* __restrict__ E5p,
                                                     T* __restrict__ HS) {
  __shared__ T sB[EB][F1];
  __shared__ T sS[EB][4];
  __shared__ int sj[EB];
  __shared__ FLv<T, 0> wS[8][F0];
  __shared__ FLv<T, 0> wE[8][NENV_EE];
  __shared__ int snb[ELOC_MAX_EL];
  __shared__ int wcnt[8];
  const int slot = blockIdx.x, w = blockIdx.y, f = threadIdx.x, lane = f & 31, wid = f >> 5;
  if (slot >= min(S_cnt[w], KS)) return;
  const int c = S[(size_t)w * KS + slot];
  __shared__ int sm[CLUSTER_KMAX];
  if (f < KM) sm[f] = moved[(size_t)w * KM + f];
  __syncthreads();
  auto e5row = [&](int j) -> const T* {
    for (int t = 0; t < KM; ++t)
      if (sm[t] == j) return E5p + ((size_t)w * KM + t) * 5 * F;
    return E5 + ((size_t)w * n + j) * 5 * F;
  };
  const T* rw = rn + (size_t)w * n * 3;
  const T rx = rw[3 * c], ry = rw[3 * c + 1], rz = rw[3 * c + 2];
  // neighbours of c after the move, ascending: 256 candidates per pass, compacted across the block
  const unsigned lt = (1u << lane) - 1u;
  int deg = 0;
  for (int j0 = 0; j0 < n; j0 += 256) {
    const int j = j0 + f;
    bool in = false;
    if (j < n && j != c) in = exact_dist(rx, ry, rz, rw[3 * j], rw[3 * j + 1], rw[3 * j + 2]) < cutoff;
    const unsigned m = __ballot_sync(0xffffffffu, in);
    if (lane == 0) wcnt[wid] = __popc(m);
    __syncthreads();
    int off = deg, tot = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      off += q < wid ? wcnt[q] : 0;
      tot += wcnt[q];
    }
    if (in) snb[off + __popc(m & lt)] = j;
    deg += tot;
    __syncthreads();
  }
  const bool si = c < n_up;
  const T inv_c = T(1) / W.w[PR_SCALARS][0];
  T wg[2][F1], we[2][4], be[2];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    const T* Wg = W.w[s == 0 ? FIRE_P_EESAME_GAMMA_W : FIRE_P_EEDIFF_GAMMA_W];
    const T* We = W.w[s == 0 ? FIRE_P_EESAME_EDGE_W : FIRE_P_EEDIFF_EDGE_W];
#pragma unroll
    for (int q = 0; q < F1; ++q) wg[s][q] = Wg[q * F + f];
#pragma unroll
    for (int q = 0; q < 4; ++q) we[s][q] = We[q * F + f];
    be[s] = W.w[s == 0 ? FIRE_P_EESAME_EDGE_B : FIRE_P_EEDIFF_EDGE_B][f];
  }
  const T* ec = e5row(c);
  const T h0 = ec[f], cts = ec[F + f], ctd = ec[2 * F + f];
  T ax = T(0);
  for (int k0 = 0; k0 < deg; k0 += EB) {
    const int nbe = min(EB, deg - k0);
    for (int q = wid; q < nbe; q += 8) {
      const int j = snb[k0 + q];
      const T diff[3] = {rx - rw[3 * j], ry - rw[3 * j + 1], rz - rw[3 * j + 2]};
      const bool same = (j < n_up) == si;
      if (same)
        edge_filter_warp<T, 0, NENV_EE>(diff, W.w[FIRE_P_EESAME_KERNEL], W.w[FIRE_P_EESAME_BIAS],
                                        W.w[PR_EESAME_INVSCALE], W.w[FIRE_P_EESAME_DIR_W], W.w[FIRE_P_EESAME_DIR_B],
                                        W.w[FIRE_P_EESAME_ENV_W], inv_c, wS[wid], wE[wid], sB[q], sS[q]);
      else
        edge_filter_warp<T, 0, NENV_EE>(diff, W.w[FIRE_P_EEDIFF_KERNEL], W.w[FIRE_P_EEDIFF_BIAS],
                                        W.w[PR_EEDIFF_INVSCALE], W.w[FIRE_P_EEDIFF_DIR_W], W.w[FIRE_P_EEDIFF_DIR_B],
                                        W.w[FIRE_P_EEDIFF_ENV_W], inv_c, wS[wid], wE[wid], sB[q], sS[q]);
      if (lane == 0) sj[q] = same ? j : -1 - j;
    }
    __syncthreads();
    for (int q = 0; q < nbe; ++q) {
      const int code = sj[q];
      const bool same = code >= 0;
      const int j = same ? code : -1 - code;
      const int s = same ? 0 : 1;
      T G = T(0), E = T(0);
#pragma unroll
      for (int u = 0; u < F1; ++u) G += wg[s][u] * sB[q][u];
#pragma unroll
      for (int u = 0; u < 4; ++u) E += we[s][u] * sS[q][u];
      E += be[s];
      const T* ej = e5row(j);
      const T u = E + ((same ? cts : ctd) + ej[(same ? 3 : 4) * F + f]);
      T y, d1, d2;
      silu3(u, y, d1, d2);
      ax += G * y;
    }
    __syncthreads();
  }
  HS[((size_t)w * KS + slot) * F + f] = h0 + ax;
}

template __global__ void k_lr_contract<float>(const float*, int, int, float, const int*, int, const int*, const int*,
                                              int, Weights<float>, const float*, const float*, float*);
template __global__ void k_lr_contract<double>(const double*, int, int, double, const int*, int, const int*,
                                               const int*, int, Weights<double>, const double*, const double*, double*);

#define FIRE_INST_EMBED(T, NT)                                                                              \
  template __global__ void k_elec_init<T, NT>(const T*, const float*, Nbr, Weights<T>, T, T*);            \
  template __global__ void k_glu<T, NT>(const T*, T*, int);                                                 \
  template __global__ void k_silu5<T, NT>(T*, int);                                                         \
  template __global__ void k_edge_contract<T, NT>(const T*, Nbr, Layout, Weights<T>, const T*, T*, T*, T*);
FIRE_INST_EMBED(float, 0)
FIRE_INST_EMBED(float, 3)
FIRE_INST_EMBED(double, 0)
FIRE_INST_EMBED(double, 3)

}  // namespace fire
