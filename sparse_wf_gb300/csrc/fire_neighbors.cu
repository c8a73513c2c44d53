// fire_neighbors.cu -- cutoff neighbour lists, triplet indices and the sparse Jacobian layout.
//
// One CTA per walker builds, bit-exactly like get_pair_indices (model/new_sparse_model.py:238-263)
// and get_neighbouring_nuclei (:476-481), the row-major sorted directed e-e pair list with its
// same-spin / opposite-spin sub-lists and their positions in the combined list, the e-n lists and
// the static counts of get_static_input (:399-437).  Distances are computed in the walkers' dtype
// with every operation rounded separately (exact_dist), so "d < cutoff" decides the same way as
// the float32 reference arithmetic on the same inputs.
#include "fire_internal.cuh"

namespace fire {

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <typename T>
__global__ void __launch_bounds__(512) k_neighbors(const T* __restrict__ r, const float* __restrict__ R,
                                                   T cutoff, T cutoff_1el, Nbr nb, fire_neighbor_out ext,
                                                   int32_t* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int w = blockIdx.x;
  const int n = nb.n, n_up = nb.n_up, N = nb.N;
  T* sr = reinterpret_cast<T*>(smem_raw);
  int* sdeg = reinterpret_cast<int*>(sr + 3 * n);
  int* sdegs = sdeg + n;
  int* sptr = sdegs + n;    // [n + 1]
  int* ssptr = sptr + n + 1;  // [n + 1]
  int* sen = ssptr + n + 1;   // [n]
  __shared__ int red[64];

  const T* rw = r + (size_t)w * n * 3;
  for (int k = threadIdx.x; k < 3 * n; k += blockDim.x) sr[k] = rw[k];
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const unsigned lt = lanemask_lt();

  // ---- pass 1: counts and e-n lists
  for (int i = wid; i < n; i += nw) {
    const T xi = sr[3 * i], yi = sr[3 * i + 1], zi = sr[3 * i + 2];
    const bool si = i < n_up;
    int c = 0, cs = 0;
    for (int j0 = 0; j0 < n; j0 += 32) {
      const int j = j0 + lane;
      bool in = false;
      if (j < n && j != i) in = exact_dist(xi, yi, zi, sr[3 * j], sr[3 * j + 1], sr[3 * j + 2]) < cutoff;
      const unsigned m = __ballot_sync(0xffffffffu, in);
      const unsigned ms = __ballot_sync(0xffffffffu, in && ((j < n_up) == si));
      c += __popc(m);
      cs += __popc(ms);
    }
    int ce = 0;
    for (int I0 = 0; I0 < N; I0 += 32) {
      const int I = I0 + lane;
      bool in = false;
      if (I < N) in = exact_dist(xi, yi, zi, (T)R[3 * I], (T)R[3 * I + 1], (T)R[3 * I + 2]) < cutoff_1el;
      const unsigned m = __ballot_sync(0xffffffffu, in);
      if (in) {
        const int pos = ce + __popc(m & lt);
        if (pos < nb.cap_nuc) {
          if (nb.en_idx) nb.en_idx[((size_t)w * n + i) * nb.cap_nuc + pos] = I;
          if (ext.en_idx) ext.en_idx[((size_t)w * n + i) * nb.cap_nuc + pos] = I;
        }
      }
      ce += __popc(m);
    }
    if (ext.en_idx) {
      for (int pos = ce + lane; pos < nb.cap_nuc; pos += 32)
        ext.en_idx[((size_t)w * n + i) * nb.cap_nuc + pos] = FIRE_NO_NEIGHBOUR;
    }
    if (lane == 0) {
      sdeg[i] = c;
      sdegs[i] = cs;
      sen[i] = ce;
    }
  }
  __syncthreads();

  // ---- exclusive scans of the row counts (warp 0)
  if (wid == 0) {
    int carry = 0, carrys = 0;
    for (int i0 = 0; i0 < n; i0 += 32) {
      const int i = i0 + lane;
      const int v = i < n ? sdeg[i] : 0, vs = i < n ? sdegs[i] : 0;
      int x = v, xs = vs;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o), ys = __shfl_up_sync(0xffffffffu, xs, o);
        if (lane >= o) {
          x += y;
          xs += ys;
        }
      }
      if (i < n) {
        sptr[i] = carry + x - v;
        ssptr[i] = carrys + xs - vs;
      }
      carry += __shfl_sync(0xffffffffu, x, 31);
      carrys += __shfl_sync(0xffffffffu, xs, 31);
    }
    if (lane == 0) {
      sptr[n] = carry;
      ssptr[n] = carrys;
    }
  }
  __syncthreads();
  const int P = sptr[n], Ps = ssptr[n], Pd = P - Ps;
  const bool fits = P <= nb.cap_p;
  const int capS = ext.cap_same, capD = ext.cap_diff, capC = capS + capD;

  // ---- pass 2: write the lists
  for (int i = wid; i < n; i += nw) {
    const T xi = sr[3 * i], yi = sr[3 * i + 1], zi = sr[3 * i + 2];
    const bool si = i < n_up;
    int c = 0, cs = 0, cd = 0;
    const int base = sptr[i], bases = ssptr[i], based = sptr[i] - ssptr[i];
    for (int j0 = 0; j0 < n; j0 += 32) {
      const int j = j0 + lane;
      bool in = false;
      if (j < n && j != i) in = exact_dist(xi, yi, zi, sr[3 * j], sr[3 * j + 1], sr[3 * j + 2]) < cutoff;
      const bool same = (j < n_up) == si;
      const unsigned m = __ballot_sync(0xffffffffu, in);
      const unsigned ms = __ballot_sync(0xffffffffu, in && same);
      const unsigned md = m & ~ms;
      if (in) {
        const int p = base + c + __popc(m & lt);
        if (p < nb.cap_p && nb.nbr) nb.nbr[(size_t)w * nb.cap_p + p] = j;
        if (ext.jac_ctr && n + p < n + capC) {
          ext.jac_ctr[(size_t)w * (n + capC) + n + p] = i;
          ext.jac_dep[(size_t)w * (n + capC) + n + p] = j;
        }
        if (same) {
          const int k = bases + cs + __popc(ms & lt);
          if (ext.ct_same && k < capS) {
            ext.ct_same[(size_t)w * capS + k] = i;
            ext.nb_same[(size_t)w * capS + k] = j;
            ext.jac_same[(size_t)w * capS + k] = n + p;
          }
        } else {
          const int k = based + cd + __popc(md & lt);
          if (ext.ct_diff && k < capD) {
            ext.ct_diff[(size_t)w * capD + k] = i;
            ext.nb_diff[(size_t)w * capD + k] = j;
            ext.jac_diff[(size_t)w * capD + k] = n + p;
          }
        }
      }
      c += __popc(m);
      cs += __popc(ms);
      cd += __popc(md);
    }
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    if (nb.deg) nb.deg[(size_t)w * n + i] = sdeg[i];
    if (nb.en_cnt) nb.en_cnt[(size_t)w * n + i] = min(sen[i], nb.cap_nuc);
    if (ext.jac_ctr) {
      ext.jac_ctr[(size_t)w * (n + capC) + i] = i;
      ext.jac_dep[(size_t)w * (n + capC) + i] = i;
    }
  }
  for (int i = threadIdx.x; i <= n; i += blockDim.x)
    if (nb.rowptr) nb.rowptr[(size_t)w * (n + 1) + i] = sptr[i];
  // padding of the reference-format lists
  if (ext.ct_same)
    for (int k = Ps + threadIdx.x; k < capS; k += blockDim.x) {
      ext.ct_same[(size_t)w * capS + k] = FIRE_NO_NEIGHBOUR;
      ext.nb_same[(size_t)w * capS + k] = FIRE_NO_NEIGHBOUR;
      ext.jac_same[(size_t)w * capS + k] = n + P;
    }
  if (ext.ct_diff)
    for (int k = Pd + threadIdx.x; k < capD; k += blockDim.x) {
      ext.ct_diff[(size_t)w * capD + k] = FIRE_NO_NEIGHBOUR;
      ext.nb_diff[(size_t)w * capD + k] = FIRE_NO_NEIGHBOUR;
      ext.jac_diff[(size_t)w * capD + k] = n + P;
    }
  if (ext.jac_ctr)
    for (int k = P + threadIdx.x; k < capC; k += blockDim.x) {
      ext.jac_ctr[(size_t)w * (n + capC) + n + k] = FIRE_NO_NEIGHBOUR;
      ext.jac_dep[(size_t)w * (n + capC) + n + k] = FIRE_NO_NEIGHBOUR;
    }
  __syncthreads();

  // ---- reverse-pair index (needs the complete list)
  if (fits && nb.rev && nb.nbr) {
    const int* nbw = nb.nbr + (size_t)w * nb.cap_p;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
      int lo = 0, hi = n;  // center: last i with sptr[i] <= p
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (sptr[mid] <= p) lo = mid; else hi = mid;
      }
      const int i = lo, j = nbw[p];
      int a = sptr[j], b = sptr[j] + sdeg[j];  // lower_bound of i in j's list
      while (a < b) {
        const int mid = (a + b) >> 1;
        if (nbw[mid] < i) a = mid + 1; else b = mid;
      }
      nb.rev[(size_t)w * nb.cap_p + p] = a;
    }
  }

  // ---- static counts
  int t = 0, e = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    t += sdeg[i] * sdeg[i];
    e = max(e, sen[i]);
  }
  t = warp_sum(t);
  e = warp_max(e);
  if (lane == 0) {
    red[wid] = t;
    red[32 + wid] = e;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int tt = 0, ee = 0;
    for (int k = 0; k < nw; ++k) {
      tt += red[k];
      ee = max(ee, red[32 + k]);
    }
    if (nb.counts) {
      nb.counts[w * 4 + 0] = Ps;
      nb.counts[w * 4 + 1] = Pd;
      nb.counts[w * 4 + 2] = tt;
      nb.counts[w * 4 + 3] = ee;
    }
    if (ext.counts) {
      ext.counts[w * 4 + 0] = Ps;
      ext.counts[w * 4 + 1] = Pd;
      ext.counts[w * 4 + 2] = tt;
      ext.counts[w * 4 + 3] = ee;
    }
    max_word(status, 1, P);
    max_word(status, 2, ee);
    max_word(status, 3, tt);
    if (!fits) set_flag(status, FIRE_FLAG_PAIR_OVERFLOW);
    if (ee > nb.cap_nuc) set_flag(status, FIRE_FLAG_NUC_OVERFLOW);
    if (ext.ct_same && (Ps > capS || Pd > capD)) set_flag(status, FIRE_FLAG_PAIR_OVERFLOW);
  }
}

// Triplet quadruples in _get_triplet_indices order (model/sparse_fwd_lap.py:252-291).
__global__ void __launch_bounds__(256) k_triplets(Nbr nb, int cap_t, int32_t* __restrict__ t_in,
                                                  int32_t* __restrict__ t_k, int32_t* __restrict__ t_kn,
                                                  int32_t* __restrict__ t_i, int32_t* status) {
  const int w = blockIdx.x, n = nb.n;
  const int* rp = nb.rowptr + (size_t)w * (n + 1);
  const int* nbw = nb.nbr + (size_t)w * nb.cap_p;
  const int* rv = nb.rev + (size_t)w * nb.cap_p;
  const int* dg = nb.deg + (size_t)w * n;
  const int P = rp[n];
  int32_t *oin = t_in + (size_t)w * cap_t, *ok = t_k + (size_t)w * cap_t, *okn = t_kn + (size_t)w * cap_t,
          *oi = t_i + (size_t)w * cap_t;
  if (P > nb.cap_p) return;
  auto put = [&](long long q, int a, int b, int c, int d) {
    if (q < cap_t) {
      oin[q] = a; ok[q] = b; okn[q] = c; oi[q] = d;
    }
  };
  for (int i = threadIdx.x; i < n; i += blockDim.x) put(i, i, i, i, i);
  for (int p = threadIdx.x; p < P; p += blockDim.x) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (rp[mid] <= p) lo = mid; else hi = mid;
    }
    const int i = lo, m = nbw[p];
    put(n + p, n + p, m, m, i);
    put(n + P + p, m, i, n + p, m);
  }
  // distinct triplets: block p occupies sum_{p' < p} deg(nb(p')) .. + deg(nb(p))
  __shared__ long long carry_s;
  __shared__ long long wsum[8];
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  const long long base0 = (long long)n + 2LL * P;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int p0 = 0; p0 < P; p0 += blockDim.x) {
    const int p = p0 + threadIdx.x;
    const int v = p < P ? dg[nbw[p]] : 0;
    long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    long long off = carry_s;
    for (int k = 0; k < wid; ++k) off += wsum[k];
    const long long excl = off + x - v;
    if (p < P) {
      int lo = 0, hi = n;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (rp[mid] <= p) lo = mid; else hi = mid;
      }
      const int i = lo, m = nbw[p];
      for (int t = 0; t < v; ++t) {
        const int q = rp[m] + t;  // (m, k): k = nbw[q]; (k, m) has index rv[q]
        put(base0 + excl + t, n + p, nbw[q], n + rv[q], i);
      }
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry_s = excl + v;
    __syncthreads();
  }
  const long long total = base0 + carry_s;
  for (long long q = total + threadIdx.x; q < cap_t; q += blockDim.x) {
    oin[q] = FIRE_NO_NEIGHBOUR; ok[q] = FIRE_NO_NEIGHBOUR; okn[q] = FIRE_NO_NEIGHBOUR; oi[q] = FIRE_NO_NEIGHBOUR;
  }
  if (threadIdx.x == 0 && total > cap_t) set_flag(status, FIRE_FLAG_TRIPLET_OVERFLOW);
}

// pos_off[w] = sum_{w' < w} (n + P_w') (single CTA)
__global__ void k_pos_scan(Nbr nb, int* __restrict__ pos_off) {
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int n = nb.n;
  for (int w0 = 0; w0 < nb.W; w0 += blockDim.x) {
    const int w = w0 + threadIdx.x;
    int v = 0;
    if (w < nb.W) v = n + min(nb.rowptr[(size_t)w * (n + 1) + n], nb.cap_p);
    // block inclusive scan (blockDim = 1024)
    __shared__ int buf[1024];
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < blockDim.x; o <<= 1) {
      const int y = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
      __syncthreads();
      buf[threadIdx.x] += y;
      __syncthreads();
    }
    if (w < nb.W) pos_off[w] = carry + buf[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry += buf[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) pos_off[nb.W] = carry;
}

// Fills pos_ctr / pos_dep / dep_pos (one CTA per walker).
__global__ void __launch_bounds__(256) k_layout(Nbr nb, Layout L) {
  const int w = blockIdx.x, n = nb.n;
  const int* rp = nb.rowptr + (size_t)w * (n + 1);
  const int P = rp[n];
  if (P > nb.cap_p) return;
  const int* nbw = nb.nbr + (size_t)w * nb.cap_p;
  const int* rv = nb.rev + (size_t)w * nb.cap_p;
  const int off = L.pos_off[w];
  const int g0 = w * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const int q0 = off + rp[i] + i;
    L.pos_ctr[q0] = g0 + i;
    L.pos_dep[q0] = g0 + i;
    L.dep_pos[q0] = q0;  // (m, m) first in m's dependency group
  }
  for (int p = threadIdx.x; p < P; p += blockDim.x) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (rp[mid] <= p) lo = mid; else hi = mid;
    }
    const int i = lo, j = nbw[p];
    const int q = off + p + i + 1;  // position of pair p (center i)
    L.pos_ctr[q] = g0 + i;
    L.pos_dep[q] = g0 + j;
    // dependency group of m = i: slot k >= 1 holds (nbw[rp[i] + k - 1], i) whose index is rv[p]
    const int jj = j;  // the pair (j, i) = reverse of p, lives in j's rows
    const int rq = rv[p];
    L.dep_pos[off + p + i + 1] = off + rq + jj + 1;
  }
}

template __global__ void k_neighbors<float>(const float*, const float*, float, float, Nbr, fire_neighbor_out,
                                            int32_t*);
template __global__ void k_neighbors<double>(const double*, const float*, double, double, Nbr,
                                             fire_neighbor_out, int32_t*);

}  // namespace fire
