// fire_jastrow.cu -- Jastrow factor, log-sum-exp over determinants and the local-energy assembly.
//
//  k_narrow      a node-local Linear(F -> NC) + ElementWise on the sparse forward-Laplacian node, one
//                CTA per center (its value row, its 3 * (deg + 1) Jacobian rows and its Laplacian row):
//                the attention logits with the query weights pre-contracted with the register keys
//                (GlobalAttentionJastrow.attention_and_values, jastrow.py:85-91, activation
//                exp(-x / sqrt(16))) and the last layer of the MLP Jastrow (SparseMLP [256, 256, 2]
//                with its final SiLU, jastrow.py:213-216, times mlp_scale plus [0, log_bias], 363-364).
//  k_mlp_sum     sum_over_nodes (sparse_fwd_lap.py:38-45) of the MLP Jastrow.
//  k_att_sums    attention[..., None] * values and sum_from_to over each spin (jastrow.py:91, 132-137):
//                dense Jacobians over all 3n coordinates, one CTA per dependency.
//  k_readout_in  values / normalizer (jastrow.py:98) with forward-Laplacian quotient rule.
//  k_assemble    log-sum-exp of the determinants with signs (wave_function.py:178), the Jastrow
//                log|J1| + J0 (_mlp_to_logpsi, jastrow.py:372-382), the e-e cusp (ElElCusp 48-64,
//                analytic), the kinetic energy -1/2 (lap + |grad|^2) (wave_function.py:215-221) and the
//                Coulomb potential (hamiltonian.py:15-26).
#include "fire_internal.cuh"

namespace fire {

constexpr int NARROW_MAXROWS = 3 * 64 + 2;

template <typename T, int ACT>
__device__ __forceinline__ void act3(T z, T& f, T& f1, T& f2) {
  if (ACT == 0) {
    silu3(z, f, f1, f2);
  } else {
    const T s = T(0.25);  // 1 / sqrt(attention_dim = 16)
    f = dexp(-z * s);
    f1 = -s * f;
    f2 = s * s * f;
  }
}

// FLM: forward-Laplacian mode (X, J, L planes) or value mode (X only).
template <typename T, int NC, int ACT, bool FLM>
__global__ void __launch_bounds__(256) k_narrow(const T* __restrict__ X, const T* __restrict__ Jp,
                                                const T* __restrict__ Lp, Nbr nb, Layout L, const T* __restrict__ Wn,
                                                const T* __restrict__ bn, const T* __restrict__ post_scale,
                                                const T* __restrict__ post_shift, T* __restrict__ Xo,
                                                T* __restrict__ Jo, T* __restrict__ Lo, int32_t* status,
                                                T* __restrict__ D1o, T* __restrict__ D2o) {
  // weights staged in shared memory (the FP64 validation build reads them through L1 instead, to stay
  // within the static shared-memory limit)
  constexpr bool kSmemW = sizeof(T) == 4;
  __shared__ T Ws_s[kSmemW ? F * NC : 1];
  __shared__ T zr[NARROW_MAXROWS][NC];
  const T* Ws = kSmemW ? Ws_s : Wn;
  const int g = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int n = nb.n, w = g / n, i = g - w * n;
  int cnt = 0;
  long q0 = 0;
  if (FLM) {
    const int* rp = nb.rowptr + (size_t)w * (n + 1);
    if (rp[n] > nb.cap_p) return;
    cnt = rp[i + 1] - rp[i] + 1;
    if (3 * cnt + 2 > NARROW_MAXROWS) {
      if (tid == 0) set_flag(status, FIRE_FLAG_PAIR_OVERFLOW);
      return;
    }
    q0 = (long)L.pos_off[w] + rp[i] + i;
  }
  if (kSmemW)
    for (int e = tid; e < F * NC; e += blockDim.x) Ws_s[e] = Wn[e];
  __syncthreads();
  const int nrows = FLM ? 3 * cnt + 2 : 1;
  for (int rr = wid; rr < nrows; rr += 8) {
    const T* src;
    if (rr == 0) src = X + (size_t)g * F;
    else if (rr == nrows - 1) src = Lp + (size_t)g * F;
    else src = Jp + (size_t)(3 * q0 + rr - 1) * F;
    T acc[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] = T(0);
#pragma unroll
    for (int u = 0; u < F / 32; ++u) {
      const int f = lane + 32 * u;
      const T v = src[f];
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[c] += v * Ws[f * NC + c];
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const T s = warp_sum(acc[c]);
      if (lane == 0) zr[rr][c] = s;
    }
  }
  __syncthreads();
  if (tid < NC) {
    const int c = tid;
    const T zx = zr[0][c] + bn[c];
    T f, f1, f2;
    act3<T, ACT>(zx, f, f1, f2);
    const T ps = post_scale ? post_scale[c] : T(1);
    const T sh = post_shift ? post_shift[c] : T(0);
    Xo[(size_t)g * NC + c] = f * ps + sh;
    if (!FLM && D1o) {  // value mode: derivative planes for separately computed Jacobian / Laplacian rows
      D1o[(size_t)g * NC + c] = f1 * ps;
      D2o[(size_t)g * NC + c] = f2 * ps;
    }
    if (FLM) {
      T jsq = T(0);
      for (int rr = 1; rr < nrows - 1; ++rr) {
        const T z = zr[rr][c];
        jsq += z * z;
        Jo[(size_t)(3 * q0 + rr - 1) * NC + c] = z * f1 * ps;
      }
      Lo[(size_t)g * NC + c] = (zr[nrows - 1][c] * f1 + jsq * f2) * ps;
    }
  }
}

// MLP-Jastrow sum over nodes: out_x [W][2], out_l [W][2], out_j [W][3n][2] (dense, tangent 3 m + t).
template <typename T, bool FLM>
__global__ void k_mlp_sum(Nbr nb, Layout L, const T* __restrict__ Xo, const T* __restrict__ Jo,
                          const T* __restrict__ Lo, T* __restrict__ ox, T* __restrict__ ol, T* __restrict__ oj) {
  const int w = blockIdx.x, n = nb.n, tid = threadIdx.x;
  const int* rp = nb.rowptr + (size_t)w * (n + 1);
  if (rp[n] > nb.cap_p) return;
  __shared__ T red[32 * 4];
  T v[4] = {T(0), T(0), T(0), T(0)};
  for (int i = tid; i < n; i += blockDim.x) {
    const size_t g = (size_t)w * n + i;
    v[0] += Xo[g * 2];
    v[1] += Xo[g * 2 + 1];
    if (FLM) {
      v[2] += Lo[g * 2];
      v[3] += Lo[g * 2 + 1];
    }
  }
  block_sum<T, 4>(v, red);
  if (tid == 0) {
    ox[w * 2] = v[0];
    ox[w * 2 + 1] = v[1];
    if (FLM) {
      ol[w * 2] = v[2];
      ol[w * 2 + 1] = v[3];
    }
  }
  if (!FLM) return;
  const int off = L.pos_off[w];
  for (int mt = tid; mt < 3 * n; mt += blockDim.x) {
    const int m = mt / 3, t = mt - 3 * m;
    const int s0 = off + rp[m] + m, cnt = rp[m + 1] - rp[m] + 1;
    T a0 = T(0), a1 = T(0);
    for (int k = 0; k < cnt; ++k) {
      const long q = L.dep_pos[s0 + k];
      a0 += Jo[(3 * q + t) * 2];
      a1 += Jo[(3 * q + t) * 2 + 1];
    }
    oj[((size_t)w * 3 * n + mt) * 2] = a0;
    oj[((size_t)w * 3 * n + mt) * 2 + 1] = a1;
  }
}

// Attention sums.  a: (aX [G][16], aJ [3 pos][16], aL [G][16]); V: (VX [G][256], VJ, VL).
// Ax, Al: [W][2][272] accumulators (256 values then 16 norms), zeroed by the caller.
// AJ: [W][3n][2][272] dense Jacobians.  One CTA (256 threads, thread = r * 16 + d) per (dep m, walker).
template <typename T, bool FLM>
__global__ void __launch_bounds__(256) k_att_sums(Nbr nb, Layout L, const T* __restrict__ aX,
                                                  const T* __restrict__ aJ, const T* __restrict__ aL,
                                                  const T* __restrict__ VX, const T* __restrict__ VJ,
                                                  const T* __restrict__ VL, T* __restrict__ Ax, T* __restrict__ Al,
                                                  T* __restrict__ AJ) {
  const int m = blockIdx.x, w = blockIdx.y, n = nb.n, tid = threadIdx.x;
  const int r = tid >> 4;
  const size_t gm = (size_t)w * n + m;
  const int sm = m < nb.n_up ? 0 : 1;
  T* ax = Ax + ((size_t)w * 2 + sm) * 272;
  const T amx = aX[gm * HEADS + r];
  const T vmx = VX[gm * F + tid];
  atomicAdd(&ax[tid], amx * vmx);
  if (tid < HEADS) atomicAdd(&ax[256 + tid], aX[gm * HEADS + tid]);
  if (!FLM) return;
  const int* rp = nb.rowptr + (size_t)w * (n + 1);
  if (rp[n] > nb.cap_p) return;
  T* al = Al + ((size_t)w * 2 + sm) * 272;
  atomicAdd(&al[tid], aL[gm * HEADS + r] * vmx + amx * VL[gm * F + tid]);
  if (tid < HEADS) atomicAdd(&al[256 + tid], aL[gm * HEADS + tid]);
  T jv[2][3], jn[2][3], lc[2];
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    lc[s] = T(0);
#pragma unroll
    for (int t = 0; t < 3; ++t) jv[s][t] = jn[s][t] = T(0);
  }
  const int off = L.pos_off[w];
  const int s0 = off + rp[m] + m, cnt = rp[m + 1] - rp[m] + 1;
  for (int k = 0; k < cnt; ++k) {
    const long q = L.dep_pos[s0 + k];
    const int gi = L.pos_ctr[q];
    const int s = (gi - w * n) < nb.n_up ? 0 : 1;
    const T aix = aX[(size_t)gi * HEADS + r];
    const T vix = VX[(size_t)gi * F + tid];
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      const T aj = aJ[(3 * q + t) * HEADS + r];
      const T vj = VJ[(3 * q + t) * F + tid];
      const T add = aj * vix + aix * vj;
      const T lcx = T(2) * aj * vj;
      if (s == 0) {
        jv[0][t] += add;
        lc[0] += lcx;
      } else {
        jv[1][t] += add;
        lc[1] += lcx;
      }
      if (tid < HEADS) {
        const T an = aJ[(3 * q + t) * HEADS + tid];
        if (s == 0) jn[0][t] += an; else jn[1][t] += an;
      }
    }
  }
#pragma unroll
  for (int s = 0; s < 2; ++s) {
    atomicAdd(&Al[((size_t)w * 2 + s) * 272 + tid], lc[s]);
#pragma unroll
    for (int t = 0; t < 3; ++t) {
      T* dst = AJ + (((size_t)w * 3 * n + 3 * m + t) * 2 + s) * 272;
      dst[tid] = jv[s][t];
      if (tid < HEADS) dst[256 + tid] = jn[s][t];
    }
  }
}

// Readout input x = values / normalizer, flattened [2][16][16] -> 512 (jastrow.py:98).
// Planes RX [W][512], RJ [W * 3n][512], RL [W][512].  One CTA (512 threads) per walker.
template <typename T, bool FLM>
__global__ void __launch_bounds__(512) k_readout_in(int n, const T* __restrict__ Ax, const T* __restrict__ Al,
                                                    const T* __restrict__ AJ, T* __restrict__ RX,
                                                    T* __restrict__ RJ, T* __restrict__ RL) {
  const int w = blockIdx.x, slot = threadIdx.x;  // slot = s * 256 + r * 16 + d
  const int s = slot >> 8, rd = slot & 255, r = rd >> 4;
  const T* ax = Ax + ((size_t)w * 2 + s) * 272;
  const T N = ax[256 + r], V = ax[rd];
  const T iN = T(1) / N;
  RX[(size_t)w * 512 + slot] = V * iN;
  if (!FLM) return;
  const T* al = Al + ((size_t)w * 2 + s) * 272;
  T nj2 = T(0), vn = T(0);
  const int T3 = 3 * n;
  for (int tt = 0; tt < T3; ++tt) {
    const T* a = AJ + (((size_t)w * T3 + tt) * 2 + s) * 272;
    const T Nj = a[256 + r], Vj = a[rd];
    nj2 += Nj * Nj;
    vn += Vj * Nj;
    RJ[((size_t)w * T3 + tt) * 512 + slot] = Vj * iN - V * Nj * iN * iN;
  }
  RL[(size_t)w * 512 + slot] = al[rd] * iN - V * al[256 + r] * iN * iN + T(2) * V * nj2 * iN * iN * iN -
                               T(2) * vn * iN * iN;
}

// e-e cusp (value, gradient per electron, Laplacian) and electronic Coulomb potential of one walker (the
// nucleus-nucleus term enn is added once); used by k_assemble.  grad_s: shared [n][3] (double).  In FP32 the
// per-pair terms are FP32 and every per-thread sum is compensated (Kahan), then reduced in FP64 across the CTA;
// the FP64 build stays in double.
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}
template <typename T>
__device__ void cusp_and_potential(const T* r, const float* R, const float* Z, int n, int n_up, int N,
                                   const T* cusp, double enn, double* grad_s, double& cval, double& clap,
                                   double& pot, double* red) {
  const int tid = threadIdx.x;
  double v = 0.0, l = 0.0, p = tid == 0 ? enn : 0.0;
  if constexpr (sizeof(T) == 4) {
    const float as = cusp[0], ad = cusp[1], fs = cusp[2], fd = cusp[3];
    float sv = 0.f, cv = 0.f, sl = 0.f, cl = 0.f, sp = 0.f, cp = 0.f;
    for (int e = tid; e < n; e += blockDim.x) {
      const float xe = r[3 * e], ye = r[3 * e + 1], ze = r[3 * e + 2];
      float gx = 0.f, gy = 0.f, gz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
      const bool se = e < n_up;
      for (int j = 0; j < n; ++j) {
        if (j == e) continue;
        const float dx = xe - r[3 * j], dy = ye - r[3 * j + 1], dz = ze - r[3 * j + 2];
        const float d = sqrtf(dx * dx + dy * dy + dz * dz), id = 1.f / d;
        const bool same = (j < n_up) == se;
        const float a = same ? as : ad, fac = same ? fs : fd;
        const float ia = 1.f / (a + d);
        const float u = a * a * ia, u1 = -u * ia, u2 = -2.f * u1 * ia;
        kahan_add(sv, cv, 0.5f * fac * u);
        kahan_add(sl, cl, fac * (u2 + 2.f * u1 * id));
        const float gd = fac * u1 * id;
        kahan_add(gx, cx, gd * dx);
        kahan_add(gy, cy, gd * dy);
        kahan_add(gz, cz, gd * dz);
        if (j > e) kahan_add(sp, cp, id);
      }
      for (int I = 0; I < N; ++I) {
        const float dx = xe - R[3 * I], dy = ye - R[3 * I + 1], dz = ze - R[3 * I + 2];
        kahan_add(sp, cp, -Z[I] / sqrtf(dx * dx + dy * dy + dz * dz));
      }
      grad_s[3 * e] = (double)gx - (double)cx;
      grad_s[3 * e + 1] = (double)gy - (double)cy;
      grad_s[3 * e + 2] = (double)gz - (double)cz;
    }
    v += (double)sv - (double)cv;
    l += (double)sl - (double)cl;
    p += (double)sp - (double)cp;
  } else {
    const double as = (double)cusp[0], ad = (double)cusp[1], fs = (double)cusp[2], fd = (double)cusp[3];
    for (int e = tid; e < n; e += blockDim.x) {
      const T xe = r[3 * e], ye = r[3 * e + 1], ze = r[3 * e + 2];
      double gx = 0.0, gy = 0.0, gz = 0.0;
      const bool se = e < n_up;
      for (int j = 0; j < n; ++j) {
        if (j == e) continue;
        const T dx = xe - r[3 * j], dy = ye - r[3 * j + 1], dz = ze - r[3 * j + 2];
        const double d = (double)dsqrt(dx * dx + dy * dy + dz * dz);
        const bool same = (j < n_up) == se;
        const double a = same ? as : ad, fac = same ? fs : fd;
        const double ia = 1.0 / (a + d);
        const double u = a * a * ia, u1 = -a * a * ia * ia, u2 = 2.0 * a * a * ia * ia * ia;
        v += 0.5 * fac * u;
        l += fac * (u2 + 2.0 * u1 / d);
        const double gd = fac * u1 / d;
        gx += gd * (double)dx;
        gy += gd * (double)dy;
        gz += gd * (double)dz;
        if (j > e) p += 1.0 / d;
      }
      for (int I = 0; I < N; ++I) {
        const T dx = xe - (T)R[3 * I], dy = ye - (T)R[3 * I + 1], dz = ze - (T)R[3 * I + 2];
        p -= (double)Z[I] / (double)dsqrt(dx * dx + dy * dy + dz * dz);
      }
      grad_s[3 * e] = gx;
      grad_s[3 * e + 1] = gy;
      grad_s[3 * e + 2] = gz;
    }
  }
  double vv[3] = {v, l, p};
  block_sum<double, 3>(vv, red);
  cval = vv[0];
  clap = vv[1];
  pot = vv[2];
}

// One CTA (256 threads) per walker.  FLM = false: value path (logpsi/sign only).
template <typename T, bool FLM>
__global__ void __launch_bounds__(256) k_assemble(int n, int n_up, int N, int w0, const T* __restrict__ r,
                                                  const float* __restrict__ R, const float* __restrict__ Z,
                                                  Weights<T> W, const double* __restrict__ ld,
                                                  const double* __restrict__ sd, const double* __restrict__ dgrad,
                                                  const double* __restrict__ dlap, const T* __restrict__ JAx,
                                                  const T* __restrict__ JAj, const T* __restrict__ JAl,
                                                  const T* __restrict__ JMx, const T* __restrict__ JMj,
                                                  const T* __restrict__ JMl, AssembleOut out, int32_t* status) {
  extern __shared__ __align__(16) unsigned char as_smem[];
  double* grad_s = reinterpret_cast<double*>(as_smem);  // [3n]
  __shared__ double red[32 * 6];
  const int w = blockIdx.x, tid = threadIdx.x;
  if (out.wmap && w >= *out.wcnt) return;
  const long row = out.wmap ? (long)out.wmap[w] : (long)w0 + w;  // output row of this walker
  const T* rw = r + (size_t)w * n * 3;
  double cval, clap, pot;
  cusp_and_potential<T>(rw, R, Z, n, n_up, N, W.w[FIRE_P_CUSP], out.enn ? *out.enn : 0.0, grad_s, cval, clap, pot,
                        red);
  __syncthreads();
  // determinants
  double mx = -1e300;
  for (int d = 0; d < NDET; ++d) mx = fmax(mx, ld[w * NDET + d]);
  double wd[NDET], S = 0.0;
  for (int d = 0; d < NDET; ++d) {
    wd[d] = sd[w * NDET + d] * exp(ld[w * NDET + d] - mx);
    S += wd[d];
  }
  const T* as_ = W.w[FIRE_P_ATT_SCALE];
  const double sc0 = (double)as_[0], sc1 = (double)as_[1];
  const double abias = (double)W.w[FIRE_P_ATT_BIAS][0];
  const double J0 = (double)JAx[w * 2] * sc0 + (double)JMx[w * 2];
  const double J1 = (double)JAx[w * 2 + 1] * sc1 + abias + (double)JMx[w * 2 + 1];
  const double logpsi = mx + log(fabs(S)) + J0 + log(fabs(J1)) + cval;
  const double sgn = ((S < 0) != (J1 < 0)) ? -1.0 : 1.0;
  if (!FLM) {
    if (tid == 0) {
      reinterpret_cast<T*>(out.logpsi)[row] = (T)logpsi;
      if (out.sign) reinterpret_cast<T*>(out.sign)[row] = (T)sgn;
      if (!isfinite(logpsi)) set_flag(status, FIRE_FLAG_NONFINITE);
    }
    return;
  }
  const int T3 = 3 * n;
  double a_tot2 = 0.0, a_lse2 = 0.0, a_dj2 = 0.0, a_J1j2 = 0.0;
  const double iS = 1.0 / S, iJ1 = 1.0 / J1;
  for (int tt = tid; tt < T3; tt += blockDim.x) {
    double lse_j = 0.0, dj2 = 0.0;
    for (int d = 0; d < NDET; ++d) {
      const double gj = dgrad[(((size_t)w * NDET + d) * n) * 3 + tt];
      lse_j += wd[d] * gj;
      dj2 += wd[d] * gj * gj;
    }
    lse_j *= iS;
    const double J0j = (double)JAj[((size_t)w * T3 + tt) * 2] * sc0 + (double)JMj[((size_t)w * T3 + tt) * 2];
    const double J1j =
        (double)JAj[((size_t)w * T3 + tt) * 2 + 1] * sc1 + (double)JMj[((size_t)w * T3 + tt) * 2 + 1];
    const double tot = lse_j + J0j + J1j * iJ1 + grad_s[tt];
    a_tot2 += tot * tot;
    a_lse2 += lse_j * lse_j;
    a_dj2 += dj2;
    a_J1j2 += J1j * J1j;
    if (out.dbg.grad) reinterpret_cast<T*>(out.dbg.grad)[(size_t)row * T3 + tt] = (T)tot;
  }
  double vv[4] = {a_tot2, a_lse2, a_dj2, a_J1j2};
  block_sum<double, 4>(vv, red);
  if (tid == 0) {
    double dl = 0.0;
    for (int d = 0; d < NDET; ++d) dl += wd[d] * dlap[w * NDET + d];
    const double lse_l = (dl + vv[2]) * iS - vv[1];
    const double J0l = (double)JAl[w * 2] * sc0 + (double)JMl[w * 2];
    const double J1l = (double)JAl[w * 2 + 1] * sc1 + (double)JMl[w * 2 + 1];
    const double lj_l = J0l + J1l * iJ1 - vv[3] * iJ1 * iJ1;
    const double lap = lse_l + lj_l + clap;
    const double ekin = -0.5 * (lap + vv[0]);
    const double eloc = ekin + pot;
    reinterpret_cast<T*>(out.eloc)[row] = (T)eloc;
    if (out.logpsi) reinterpret_cast<T*>(out.logpsi)[row] = (T)logpsi;
    if (out.sign) reinterpret_cast<T*>(out.sign)[row] = (T)sgn;
    if (out.dbg.kinetic) reinterpret_cast<T*>(out.dbg.kinetic)[row] = (T)ekin;
    if (out.dbg.potential) reinterpret_cast<T*>(out.dbg.potential)[row] = (T)pot;
    if (out.dbg.lap) reinterpret_cast<T*>(out.dbg.lap)[row] = (T)lap;
    if (out.dbg.jastrow) reinterpret_cast<T*>(out.dbg.jastrow)[row] = (T)(J0 + log(fabs(J1)) + cval);
    if (out.dbg.logdet)
      for (int d = 0; d < NDET; ++d) out.dbg.logdet[(size_t)row * NDET + d] = ld[w * NDET + d];
    if (out.dbg.sign_det)
      for (int d = 0; d < NDET; ++d) out.dbg.sign_det[(size_t)row * NDET + d] = sd[w * NDET + d];
    if (out.dbg.refined) out.dbg.refined[row] = out.wmap ? 1 : 0;
    // determinant-weighted condition number of the orbital matrices: the factor by which their rounding enters
    // the derivatives of log sum_d w_d det A_d
    double cw = 0.0;
    if (out.cond) {
      for (int d = 0; d < NDET; ++d) cw += fabs(wd[d]) * out.cond[w * NDET + d];
      cw /= fabs(S);
    }
    if (out.dbg.cond && !out.wmap) out.dbg.cond[row] = cw;
    const double ks = 0.5 * (fabs(lap) + vv[0]);
    if (out.ref_idx &&
        !(ks <= out.ref_ratio * fabs(eloc) && ks <= out.ref_ks && cw <= out.ref_kappa && ks * cw <= out.ref_kscond)) {
      const int slot = atomicAdd(out.ref_cnt, 1);
      if (slot < out.ref_cap) out.ref_idx[slot] = (int32_t)row;
    }
    if (!isfinite(eloc) || !isfinite(logpsi)) set_flag(status, FIRE_FLAG_NONFINITE);
  }
}

// Nucleus-nucleus repulsion sum_{I<J} Z_I Z_J / |R_I - R_J| (hamiltonian.py:15-26), once per call.
__global__ void __launch_bounds__(256) k_nn_energy(const float* __restrict__ R, const float* __restrict__ Z, int N,
                                                   double* __restrict__ out) {
  __shared__ double red[32];
  double p = 0.0;
  for (int k = threadIdx.x; k < N * N; k += blockDim.x) {
    const int I = k / N, J = k - I * N;
    if (J > I) {
      const double dx = (double)R[3 * I] - R[3 * J], dy = (double)R[3 * I + 1] - R[3 * J + 1],
                   dz = (double)R[3 * I + 2] - R[3 * J + 2];
      p += (double)Z[I] * Z[J] / sqrt(dx * dx + dy * dy + dz * dz);
    }
  }
  double v[1] = {p};
  block_sum<double, 1>(v, red);
  if (threadIdx.x == 0) out[0] = v[0];
}

// Coulomb potential only (fire_potential_energy).
template <typename T>
__global__ void __launch_bounds__(256) k_potential(int n, int N, const T* __restrict__ r, const float* __restrict__ R,
                                                   const float* __restrict__ Z, T* __restrict__ out) {
  __shared__ double red[32];
  const int w = blockIdx.x, tid = threadIdx.x;
  const T* rw = r + (size_t)w * n * 3;
  double p = 0.0;
  for (int e = tid; e < n; e += blockDim.x) {
    const T xe = rw[3 * e], ye = rw[3 * e + 1], ze = rw[3 * e + 2];
    for (int j = e + 1; j < n; ++j) {
      const T dx = xe - rw[3 * j], dy = ye - rw[3 * j + 1], dz = ze - rw[3 * j + 2];
      p += 1.0 / (double)dsqrt(dx * dx + dy * dy + dz * dz);
    }
    for (int I = 0; I < N; ++I) {
      const T dx = xe - (T)R[3 * I], dy = ye - (T)R[3 * I + 1], dz = ze - (T)R[3 * I + 2];
      p -= (double)Z[I] / (double)dsqrt(dx * dx + dy * dy + dz * dz);
    }
  }
  for (int k = tid; k < N * N; k += blockDim.x) {
    const int I = k / N, J = k - I * N;
    if (J > I) {
      const double dx = (double)R[3 * I] - R[3 * J], dy = (double)R[3 * I + 1] - R[3 * J + 1],
                   dz = (double)R[3 * I + 2] - R[3 * J + 2];
      p += (double)Z[I] * Z[J] / sqrt(dx * dx + dy * dy + dz * dz);
    }
  }
  double v[1] = {p};
  block_sum<double, 1>(v, red);
  if (tid == 0) out[w] = (T)v[0];
}

// Batch mean and standard deviation of E_loc in FP64 (update.py:130-134).
template <typename T>
__global__ void k_stats(const T* __restrict__ e, int B, double* __restrict__ out) {
  __shared__ double red[64];
  double s = 0.0;
  for (int k = threadIdx.x; k < B; k += blockDim.x) s += (double)e[k];
  double v[1] = {s};
  block_sum<double, 1>(v, red);
  const double mean = v[0] / B;
  double q = 0.0;
  for (int k = threadIdx.x; k < B; k += blockDim.x) {
    const double d = (double)e[k] - mean;
    q += d * d;
  }
  double v2[1] = {q};
  block_sum<double, 1>(v2, red);
  if (threadIdx.x == 0) {
    out[0] = mean;
    out[1] = sqrt(v2[0] / B);
  }
}

#define FIRE_INST_JAS(T)                                                                                         \
  template __global__ void k_narrow<T, 16, 1, true>(const T*, const T*, const T*, Nbr, Layout, const T*, const T*, \
                                                    const T*, const T*, T*, T*, T*, int32_t*, T*, T*);                   \
  template __global__ void k_narrow<T, 16, 1, false>(const T*, const T*, const T*, Nbr, Layout, const T*,         \
                                                     const T*, const T*, const T*, T*, T*, T*, int32_t*, T*, T*);        \
  template __global__ void k_narrow<T, 2, 0, true>(const T*, const T*, const T*, Nbr, Layout, const T*, const T*,  \
                                                   const T*, const T*, T*, T*, T*, int32_t*, T*, T*);                    \
  template __global__ void k_narrow<T, 2, 0, false>(const T*, const T*, const T*, Nbr, Layout, const T*, const T*, \
                                                    const T*, const T*, T*, T*, T*, int32_t*, T*, T*);                   \
  template __global__ void k_mlp_sum<T, true>(Nbr, Layout, const T*, const T*, const T*, T*, T*, T*);             \
  template __global__ void k_mlp_sum<T, false>(Nbr, Layout, const T*, const T*, const T*, T*, T*, T*);            \
  template __global__ void k_att_sums<T, true>(Nbr, Layout, const T*, const T*, const T*, const T*, const T*,     \
                                               const T*, T*, T*, T*);                                            \
  template __global__ void k_att_sums<T, false>(Nbr, Layout, const T*, const T*, const T*, const T*, const T*,    \
                                                const T*, T*, T*, T*);                                           \
  template __global__ void k_readout_in<T, true>(int, const T*, const T*, const T*, T*, T*, T*);                  \
  template __global__ void k_readout_in<T, false>(int, const T*, const T*, const T*, T*, T*, T*);                 \
  template __global__ void k_assemble<T, true>(int, int, int, int, const T*, const float*, const float*,          \
                                               Weights<T>, const double*, const double*, const double*,          \
                                               const double*, const T*, const T*, const T*, const T*, const T*,   \
                                               const T*, AssembleOut, int32_t*);                                 \
  template __global__ void k_assemble<T, false>(int, int, int, int, const T*, const float*, const float*,         \
                                                Weights<T>, const double*, const double*, const double*,         \
                                                const double*, const T*, const T*, const T*, const T*, const T*,  \
                                                const T*, AssembleOut, int32_t*);                                \
  template __global__ void k_potential<T>(int, int, const T*, const float*, const float*, T*);                    \
  template __global__ void k_stats<T>(const T*, int, double*);
FIRE_INST_JAS(float)
FIRE_INST_JAS(double)

}  // namespace fire
