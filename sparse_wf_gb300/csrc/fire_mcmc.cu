// fire_mcmc.cu -- Metropolis proposals (all-electron, mcmc.py:38-97; single-electron, mcmc.py:100-111; jump to a
// nucleus, mcmc.py:164-193; cluster update, mcmc.py:119-161) and accept/reject.
//
// Random numbers: Philox4x32-10 (Salmon et al., "Parallel random numbers: as easy as 1, 2, 3",
// SC'11), counter = (step, walker, electron, stream counter), key = seed; normals by Box-Muller.
// jax.random (threefry) cannot be reproduced here, so bit-level parity of the chain is checked in
// replay mode, where the caller supplies the normal draws and log-uniforms.
#include "fire_internal.cuh"
#include "fire_philox.cuh"

namespace fire {

// r_new = r + width * eps for every electron of every walker of the chunk.
template <typename T>
__global__ void k_propose(const T* __restrict__ r, T* __restrict__ rn, int n, int Wc, int w0, int B, int step,
                          T width, uint64_t seed, uint64_t counter, const T* __restrict__ replay) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;  // (w, e)
  if (idx >= (long)Wc * n) return;
  const int w = (int)(idx / n), e = (int)(idx - (long)w * n);
  const long gw = w0 + w;
  T eps[3];
  if (replay) {
    const T* src = replay + (((long)step * B + gw) * n + e) * 3;
    eps[0] = src[0]; eps[1] = src[1]; eps[2] = src[2];
  } else {
    uint32_t ctr[4] = {(uint32_t)step, (uint32_t)gw, (uint32_t)e, (uint32_t)counter};
    philox10(ctr, seed ^ (counter >> 32) * 0x9E3779B97F4A7C15ull);
    const double r1 = sqrt(-2.0 * log(u01(ctr[0]))), t1 = 6.283185307179586 * u01(ctr[1]);
    const double r2 = sqrt(-2.0 * log(u01(ctr[2]))), t2 = 6.283185307179586 * u01(ctr[3]);
    eps[0] = (T)(r1 * cos(t1));
    eps[1] = (T)(r1 * sin(t1));
    eps[2] = (T)(r2 * cos(t2));
  }
  const long base = idx * 3;
#pragma unroll
  for (int c = 0; c < 3; ++c) rn[base + c] = r[base + c] + width * eps[c];
}

// Single-electron proposal (proposal_single_electron, mcmc.py:100-111): r_new = r with electron
// (offset + step) mod n moved by width * eps, eps [3] per walker and step; one CTA per walker of the chunk.
// replay [steps, B, 3]; moved (may be null) receives the moved electron of every walker of the chunk.
template <typename T>
__global__ void k_propose_single(const T* __restrict__ r, T* __restrict__ rn, int n, int w0, int B, int step,
                                 int offset, T width, uint64_t seed, uint64_t counter, const T* __restrict__ replay,
                                 int* __restrict__ moved) {
  const int w = blockIdx.x;
  const long gw = w0 + w;
  const T* src = r + (long)w * 3 * n;
  T* dst = rn + (long)w * 3 * n;
  for (int k = threadIdx.x; k < 3 * n; k += blockDim.x) dst[k] = src[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    const int e = (int)(((long)offset + step) % n);
    if (moved) moved[w] = e;
    T eps[3];
    if (replay) {
      const T* q = replay + ((long)step * B + gw) * 3;
      eps[0] = q[0]; eps[1] = q[1]; eps[2] = q[2];
    } else {
      uint32_t ctr[4] = {(uint32_t)step, (uint32_t)gw, 0xFFFFFFFEu, (uint32_t)counter};
      philox10(ctr, seed ^ (counter >> 32) * 0x9E3779B97F4A7C15ull);
      const double r1 = sqrt(-2.0 * log(u01(ctr[0]))), t1 = 6.283185307179586 * u01(ctr[1]);
      const double r2 = sqrt(-2.0 * log(u01(ctr[2]))), t2 = 6.283185307179586 * u01(ctr[3]);
      eps[0] = (T)(r1 * cos(t1));
      eps[1] = (T)(r1 * sin(t1));
      eps[2] = (T)(r2 * cos(t2));
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) dst[3 * e + c] = src[3 * e + c] + width * eps[c];
  }
}

// Jump proposal (proposal_jump_to_atom, mcmc.py:164-193): a random electron of every walker is moved to
// R_I + sigma * eps around a nucleus I drawn with probability Z_I / sum Z; plr[w] receives the proposal's
// log ratio log(q(r_old) / q(r_new)), q(x) = sum_J Z_J exp(-|x - R_J|^2 / (2 sigma^2)).  Draws per walker
// and step: d = (u_electron, u_nucleus, eps_x, eps_y, eps_z); electron = min(floor(u_e n), n - 1), nucleus =
// the first J with cumulative charge > u_n sum Z.  replay [steps, B, 5]; moved (may be null) receives the jumped
// electron of every walker of the chunk; one CTA per walker of the chunk.
template <typename T>
__global__ void k_propose_jump(const T* __restrict__ r, T* __restrict__ rn, T* __restrict__ plr, int n, int w0,
                               int B, int step, const float* __restrict__ R, const float* __restrict__ Z, int N,
                               T sigma, uint64_t seed, uint64_t counter, const T* __restrict__ replay,
                               int* __restrict__ moved) {
  const int w = blockIdx.x;
  const long gw = w0 + w;
  const T* src = r + (long)w * 3 * n;
  T* dst = rn + (long)w * 3 * n;
  for (int k = threadIdx.x; k < 3 * n; k += blockDim.x) dst[k] = src[k];
  __shared__ double dr[5];
  __shared__ int sel[2];
  if (threadIdx.x == 0) {
    if (replay) {
      const T* q = replay + ((long)step * B + gw) * 5;
      for (int k = 0; k < 5; ++k) dr[k] = (double)q[k];
    } else {
      uint32_t c0[4] = {(uint32_t)step, (uint32_t)gw, 0xFFFFFFFDu, (uint32_t)counter};
      uint32_t c1[4] = {(uint32_t)step, (uint32_t)gw, 0xFFFFFFFCu, (uint32_t)counter};
      philox10(c0, seed ^ (counter >> 32) * 0x9E3779B97F4A7C15ull);
      philox10(c1, seed ^ (counter >> 32) * 0x9E3779B97F4A7C15ull);
      dr[0] = u01(c0[0]);
      dr[1] = u01(c0[1]);
      const double r1 = sqrt(-2.0 * log(u01(c1[0]))), t1 = 6.283185307179586 * u01(c1[1]);
      const double r2 = sqrt(-2.0 * log(u01(c1[2]))), t2 = 6.283185307179586 * u01(c1[3]);
      dr[2] = r1 * cos(t1);
      dr[3] = r1 * sin(t1);
      dr[4] = r2 * cos(t2);
    }
    const int e = min((int)(dr[0] * n), n - 1);
    double zs = 0.0;
    for (int J = 0; J < N; ++J) zs += (double)Z[J];
    const double tz = dr[1] * zs;
    int I = N - 1;
    double cz = 0.0;
    for (int J = 0; J < N; ++J) {
      cz += (double)Z[J];
      if (cz > tz) {
        I = J;
        break;
      }
    }
    sel[0] = e;
    sel[1] = I;
    if (moved) moved[w] = e;
  }
  __syncthreads();
  const int e = sel[0], I = sel[1];
  // new position (written after every thread has read the old one below)
  const T xn = (T)R[3 * I] + sigma * (T)dr[2], yn = (T)R[3 * I + 1] + sigma * (T)dr[3],
          zn = (T)R[3 * I + 2] + sigma * (T)dr[4];
  const T xo = src[3 * e], yo = src[3 * e + 1], zo = src[3 * e + 2];
  // q(old) and q(new) over the nuclei (block reduction in double)
  const double inv2s2 = 0.5 / ((double)sigma * (double)sigma);
  double qo = 0.0, qn = 0.0;
  for (int J = threadIdx.x; J < N; J += blockDim.x) {
    const double ax = (double)xo - R[3 * J], ay = (double)yo - R[3 * J + 1], az = (double)zo - R[3 * J + 2];
    const double bx = (double)xn - R[3 * J], by = (double)yn - R[3 * J + 1], bz = (double)zn - R[3 * J + 2];
    qo += (double)Z[J] * exp(-inv2s2 * (ax * ax + ay * ay + az * az));
    qn += (double)Z[J] * exp(-inv2s2 * (bx * bx + by * by + bz * bz));
  }
  __shared__ double red[2][32];
  for (int o = 16; o > 0; o >>= 1) {
    qo += __shfl_xor_sync(0xffffffffu, qo, o);
    qn += __shfl_xor_sync(0xffffffffu, qn, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = qo;
    red[1][threadIdx.x >> 5] = qn;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double so = 0.0, sn = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      so += red[0][k];
      sn += red[1][k];
    }
    plr[w] = (T)(log(so) - log(sn));
    dst[3 * e] = xn;
    dst[3 * e + 1] = yn;
    dst[3 * e + 2] = zn;
  }
}

// The k electrons closest to position c (distance ascending, ties: lower index first, like jax.lax.top_k of
// -dist) whose distance is at most radius; pos(j) gives electron j's position.  Returns how many qualify.
template <typename T, typename PosFn>
__device__ int closest_k(PosFn pos, int n, const T (&c)[3], int k, T radius, int (&idx)[CLUSTER_KMAX]) {
  T best[CLUSTER_KMAX];
  int m = 0;
  for (int j = 0; j < n; ++j) {
    T q[3];
    pos(j, q);
    const T dx = q[0] - c[0], dy = q[1] - c[1], dz = q[2] - c[2];
    const T d = sqrt(dx * dx + dy * dy + dz * dz);
    if (m == k && !(d < best[k - 1])) continue;
    int i = m < k ? m++ : k - 1;
    while (i > 0 && d < best[i - 1]) {
      best[i] = best[i - 1];
      idx[i] = idx[i - 1];
      --i;
    }
    best[i] = d;
    idx[i] = j;
  }
  int cnt = 0;
  while (cnt < m && best[cnt] <= radius) ++cnt;
  return cnt;
}

// Cluster proposal (proposal_cluster_update, mcmc.py:119-161): center (offset + step) mod n (sequential) or a
// uniform draw (random); the k closest electrons within radius move by width * eps (noise row i to the i-th
// closest); of CLUSTER_TRIALS draws the first whose moved center has the same k-closest set is used, plr = 0, else
// the first draw with plr = -inf (always rejected).  Draws per walker and step: u_center, then eps
// [CLUSTER_TRIALS][k][3]; replay [steps, B, 1 + 3 CLUSTER_TRIALS k].  One CTA per walker of the chunk.
template <typename T>
__global__ void k_propose_cluster(const T* __restrict__ r, T* __restrict__ rn, T* __restrict__ plr, int n, int w0,
                                  int B, int step, int offset, int k, T radius, T width, int random_sweep,
                                  uint64_t seed, uint64_t counter, const T* __restrict__ replay,
                                  int* __restrict__ moved_idx) {
  const int w = blockIdx.x;
  const long gw = w0 + w;
  const T* src = r + (long)w * 3 * n;
  T* dst = rn + (long)w * 3 * n;
  for (int q = threadIdx.x; q < 3 * n; q += blockDim.x) dst[q] = src[q];
  __syncthreads();
  if (threadIdx.x != 0) return;
  const int nd = 1 + 3 * CLUSTER_TRIALS * k;
  const T* rep = replay ? replay + ((long)step * B + gw) * nd : nullptr;
  // draw m of this walker and step: uniform (m = 0) or standard normal (m >= 1)
  double nbuf[4];
  int nbase = -4;
  auto draw = [&](int m) -> double {
    if (rep) return (double)rep[m];
    if (m == 0) {
      uint32_t c0[4] = {(uint32_t)step, (uint32_t)gw, 0xFFFFFFFBu, (uint32_t)counter};
      philox10(c0, seed ^ (counter >> 32) * 0x9E3779B97F4A7C15ull);
      return u01(c0[0]);
    }
    const int q = (m - 1) >> 2;
    if (q * 4 != nbase) {
      uint32_t c1[4] = {(uint32_t)step, (uint32_t)gw, 0x80000000u | (uint32_t)q, (uint32_t)counter};
      philox10(c1, seed ^ (counter >> 32) * 0x9E3779B97F4A7C15ull);
      const double r1 = sqrt(-2.0 * log(u01(c1[0]))), t1 = 6.283185307179586 * u01(c1[1]);
      const double r2 = sqrt(-2.0 * log(u01(c1[2]))), t2 = 6.283185307179586 * u01(c1[3]);
      nbuf[0] = r1 * cos(t1);
      nbuf[1] = r1 * sin(t1);
      nbuf[2] = r2 * cos(t2);
      nbuf[3] = r2 * sin(t2);
      nbase = q * 4;
    }
    return nbuf[(m - 1) & 3];
  };
  const int center = random_sweep ? min((int)(draw(0) * n), n - 1) : (int)(((long)offset + step) % n);
  T cpos[3] = {src[3 * center], src[3 * center + 1], src[3 * center + 2]};
  int sel[CLUSTER_KMAX];
  const int cnt = closest_k<T>([&](int j, T (&q)[3]) { q[0] = src[3 * j]; q[1] = src[3 * j + 1]; q[2] = src[3 * j + 2]; },
                               n, cpos, k, radius, sel);
  int sorted_sel[CLUSTER_KMAX];
  for (int i = 0; i < cnt; ++i) sorted_sel[i] = sel[i];
  for (int i = 1; i < cnt; ++i)
    for (int a = i; a > 0 && sorted_sel[a] < sorted_sel[a - 1]; --a) {
      const int t = sorted_sel[a];
      sorted_sel[a] = sorted_sel[a - 1];
      sorted_sel[a - 1] = t;
    }
  int chosen = -1;
  T moved[CLUSTER_KMAX][3], first[CLUSTER_KMAX][3];
  for (int t = 0; t < CLUSTER_TRIALS && chosen < 0; ++t) {
    for (int i = 0; i < cnt; ++i)
      for (int c = 0; c < 3; ++c)
        moved[i][c] = src[3 * sel[i] + c] + width * (T)draw(1 + (t * k + i) * 3 + c);
    if (t == 0)
      for (int i = 0; i < cnt; ++i)
        for (int c = 0; c < 3; ++c) first[i][c] = moved[i][c];
    // the moved center (always in its own cluster, at distance 0)
    T c2[3] = {cpos[0], cpos[1], cpos[2]};
    for (int i = 0; i < cnt; ++i)
      if (sel[i] == center) {
        c2[0] = moved[i][0]; c2[1] = moved[i][1]; c2[2] = moved[i][2];
      }
    int rev[CLUSTER_KMAX];
    const int cr = closest_k<T>(
        [&](int j, T (&q)[3]) {
          for (int i = 0; i < cnt; ++i)
            if (sel[i] == j) {
              q[0] = moved[i][0]; q[1] = moved[i][1]; q[2] = moved[i][2];
              return;
            }
          q[0] = src[3 * j]; q[1] = src[3 * j + 1]; q[2] = src[3 * j + 2];
        },
        n, c2, k, radius, rev);
    bool same = cr == cnt;
    if (same) {
      for (int i = 1; i < cr; ++i)
        for (int a = i; a > 0 && rev[a] < rev[a - 1]; --a) {
          const int tt = rev[a];
          rev[a] = rev[a - 1];
          rev[a - 1] = tt;
        }
      for (int i = 0; i < cr; ++i) same = same && rev[i] == sorted_sel[i];
    }
    if (same) chosen = t;
  }
  for (int i = 0; i < cnt; ++i)
    for (int c = 0; c < 3; ++c) dst[3 * sel[i] + c] = chosen >= 0 ? moved[i][c] : first[i][c];
  plr[w] = chosen >= 0 ? T(0) : T(-INFINITY);
  if (moved_idx)  // the cluster's index list, closest first, FIRE_NO_NEIGHBOUR beyond the radius (mcmc.py:141-143)
    for (int i = 0; i < k; ++i) moved_idx[(long)w * k + i] = i < cnt ? sel[i] : FIRE_NO_NEIGHBOUR;
}

// Accept if 2 (logpsi_new - logpsi_old) > log u (mcmc.py:68-73); one CTA per walker.
// r, logpsi: whole batch (global walker index); rn, logpsi_new, counts: this chunk (local index).
// plr (may be null): the proposals' log ratios log(q(r_old) / q(r_new)), added to the test (mcmc.py:238).
// acc_out (may be null): the decision per walker of the chunk (1 accepted, 0 rejected).
template <typename T>
__global__ void k_accept(T* __restrict__ r, const T* __restrict__ rn, T* __restrict__ logpsi,
                         const T* __restrict__ logpsi_new, int n, int w0, int B, int step, uint64_t seed,
                         uint64_t counter, const T* __restrict__ replay_log_u, int32_t* __restrict__ n_accept,
                         const int* __restrict__ counts, int32_t* __restrict__ static_max, const T* __restrict__ plr,
                         int32_t* __restrict__ acc_out) {
  const int w = blockIdx.x;
  const long gw = w0 + w;
  __shared__ int acc_s;
  if (threadIdx.x == 0) {
    double logu;
    if (replay_log_u) {
      logu = (double)replay_log_u[(long)step * B + gw];
    } else {
      uint32_t ctr[4] = {(uint32_t)step, (uint32_t)gw, 0xFFFFFFFFu, (uint32_t)counter};
      philox10(ctr, seed ^ (counter >> 32) * 0x9E3779B97F4A7C15ull);
      logu = log(u01(ctr[0]));
    }
    const double ratio = 2.0 * ((double)logpsi_new[w] - (double)logpsi[gw]) + (plr ? (double)plr[w] : 0.0);
    const int a = ratio > logu ? 1 : 0;
    acc_s = a;
    if (acc_out) acc_out[w] = a;
    if (a) logpsi[gw] = logpsi_new[w];
    if (n_accept) n_accept[gw] += a;
    if (static_max && counts) {
      atomicMax(&static_max[0], counts[w * 4 + 0]);
      atomicMax(&static_max[1], counts[w * 4 + 1]);
      atomicMax(&static_max[3], counts[w * 4 + 3]);
    }
  }
  __syncthreads();
  if (acc_s) {
    for (int k = threadIdx.x; k < 3 * n; k += blockDim.x) r[gw * 3 * n + k] = rn[(long)w * 3 * n + k];
  }
}

template __global__ void k_propose<float>(const float*, float*, int, int, int, int, int, float, uint64_t, uint64_t,
                                          const float*);
template __global__ void k_propose<double>(const double*, double*, int, int, int, int, int, double, uint64_t,
                                           uint64_t, const double*);
template __global__ void k_propose_single<float>(const float*, float*, int, int, int, int, int, float, uint64_t,
                                                 uint64_t, const float*, int*);
template __global__ void k_propose_single<double>(const double*, double*, int, int, int, int, int, double,
                                                  uint64_t, uint64_t, const double*, int*);
template __global__ void k_propose_jump<float>(const float*, float*, float*, int, int, int, int, const float*,
                                               const float*, int, float, uint64_t, uint64_t, const float*, int*);
template __global__ void k_propose_jump<double>(const double*, double*, double*, int, int, int, int, const float*,
                                                const float*, int, double, uint64_t, uint64_t, const double*, int*);
template __global__ void k_propose_cluster<float>(const float*, float*, float*, int, int, int, int, int, int, float,
                                                  float, int, uint64_t, uint64_t, const float*, int*);
template __global__ void k_propose_cluster<double>(const double*, double*, double*, int, int, int, int, int, int,
                                                   double, double, int, uint64_t, uint64_t, const double*, int*);
template __global__ void k_accept<float>(float*, const float*, float*, const float*, int, int, int, int, uint64_t,
                                         uint64_t, const float*, int32_t*, const int*, int32_t*, const float*, int32_t*);
template __global__ void k_accept<double>(double*, const double*, double*, const double*, int, int, int, int,
                                          uint64_t, uint64_t, const double*, int32_t*, const int*, int32_t*,
                                          const double*, int32_t*);

}  // namespace fire
