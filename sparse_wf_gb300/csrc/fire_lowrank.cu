// fire_lowrank.cu -- low-rank single-electron Metropolis steps: log|psi| of a proposal that moved one electron, from
// a state cached per walker instead of a full evaluation (log_psi_low_rank_update, model/wave_function.py:249-287,
// driven by mcmc_steps_low_rank, mcmc.py:196-275).  The state is the value path's own buffers of the chunk (ElecInit
// rows, embeddings, envelope / raw orbital / orbital-matrix rows, attention and MLP Jastrow rows, slogdets, e-n lists
// and statics) plus the transposed inverse B = A^-T of every orbital matrix.  Per step, with e = moved[w] the electron
// walker w moved:
//
//  k_lr_select  the changed set S (ascending): e and every electron within the cutoff of e before or after the move
//               (get_low_rank_pair_indices, model/new_sparse_model.py:439-474); the proposal's statics
//               (get_static_input, :399-437: the pair counts corrected by e's old and new neighbours, the e-n
//               maximum, and the move statics n_changed_hout / n_changed_pair_same / n_changed_pair_diff, :414-424)
//               and e's e-n list at its new position.
//  k_lr_orb     the raw orbital rows of S, each from its spin's contraction (Orbitals.low_rank_update,
//               orbitals.py:121-146).
//  k_lr_env_coef, k_lr_env_add
//               the envelope row of the moved electron at its new position, with its spin's envelope.
//  k_lr_det     per walker and determinant: V = A'[S] - A[S], M = I + V A^-1[:, S], log|det M| and M^-1 by
//               Gauss-Jordan with partial pivoting in FP64 (the determinant lemma of woodburry_update,
//               model/utils.py:216-245).
//  k_lr_jsums   the Jastrow sums over all electrons with the rows of S replaced (Jastrow.low_rank_update,
//               jastrow.py:309-361): attention numerators and normalisers per spin, and the MLP rows.
//  k_lr_commit  on acceptance, the proposal's rows into the state.
//  k_lr_wb_z, k_lr_wb_q, k_lr_wb_apply
//               on acceptance, the Woodbury update of the transposed inverse: B' = B - (B V^T)(M^-T B[S, :]).
#include <type_traits>

#include "fire_df64.cuh"
#include "fire_internal.cuh"

namespace fire {

namespace {
constexpr unsigned kFull = 0xffffffffu;
constexpr int kAcc = LR_KMAX / 8;  // accumulators per thread of the Woodbury products (8 warps share the k columns)
}  // namespace

// One CTA (256 threads) per walker of the chunk.  r: the chunk's current positions; rn: the proposal, in which walker
// w moved the electrons moved[w][0..KM) (entries >= n are padding: NO_NEIGHBOUR of a cluster's index list).  nb: the
// state's e-n counts [W][n] and statics [W][4].  Outputs S [W][KS] (the first KS members of the changed set), S_cnt
// [W] (its true size), per moved slot t the new position re_p [W][KM][3] and e-n list en_cnt_p [W][KM], en_idx_p
// [W][KM][cap_nuc], the proposal's statics counts_p [W][4] (triplets 0); static_max [7] entries 4..6 take the move
// statics.  The changed set holds the moved electrons and every electron within the cutoff of a gathered moved entry
// before or after the move, a padded entry gathering electron n - 1 as an out-of-range JAX gather clamps
// (get_low_rank_pair_indices, model/new_sparse_model.py:439-474).
template <typename T>
__global__ void __launch_bounds__(256) k_lr_select(const T* __restrict__ r, const T* __restrict__ rn, int n, int n_up,
                                                   const int* __restrict__ moved, int KM, const float* __restrict__ R,
                                                   int N, T cutoff, T cutoff_1el, Nbr nb, int KS, int* __restrict__ S,
                                                   int* __restrict__ S_cnt, T* __restrict__ re_p,
                                                   int* __restrict__ en_cnt_p, int* __restrict__ en_idx_p,
                                                   int* __restrict__ counts_p, int32_t* __restrict__ static_max,
                                                   int32_t* status) {
  __shared__ int wcnt[8];
  __shared__ int emx[8];
  __shared__ int red[32 * 4];
  __shared__ int sS[LR_KMAX];
  __shared__ int sm[CLUSTER_KMAX];
  __shared__ int ce_max;
  const int w = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const T* ro = r + (size_t)w * n * 3;
  const T* rp = rn + (size_t)w * n * 3;
  if (tid < KM) sm[tid] = moved[(size_t)w * KM + tid];
  if (tid == 0) ce_max = 0;
  __syncthreads();
  // S in ascending order, 256 candidates per pass; dv: the change of the directed pair counts (same, diff spin), each
  // pair (m, j) of a moved m counted twice when j stays and once when j moves too (its own term counts the other)
  int cnt = 0;
  int dv[2] = {0, 0};
  for (int j0 = 0; j0 < n; j0 += 256) {
    const int j = j0 + tid;
    bool aff = false;
    if (j < n) {
      bool isM = false;
      for (int t = 0; t < KM; ++t) isM |= sm[t] == j;
      aff = isM;
      const bool sj = j < n_up;
      for (int t = 0; t < KM; ++t) {
        const int m = min(sm[t], n - 1);
        if (m == j) continue;
        const bool io = exact_dist(ro[3 * m], ro[3 * m + 1], ro[3 * m + 2], ro[3 * j], ro[3 * j + 1], ro[3 * j + 2]) <
                        cutoff;
        const bool in = exact_dist(rp[3 * m], rp[3 * m + 1], rp[3 * m + 2], rp[3 * j], rp[3 * j + 1], rp[3 * j + 2]) <
                        cutoff;
        aff |= io || in;
        if (sm[t] < n) {
          const int d = (isM ? 1 : 2) * ((int)in - (int)io);
          dv[((m < n_up) == sj) ? 0 : 1] += d;
        }
      }
    }
    const unsigned mk = __ballot_sync(kFull, aff);
    if (lane == 0) wcnt[wid] = __popc(mk);
    __syncthreads();
    int off = cnt, tot = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      off += q < wid ? wcnt[q] : 0;
      tot += wcnt[q];
    }
    const int pos = off + __popc(mk & lt);
    if (aff && pos < KS) {
      S[(size_t)w * KS + pos] = j;
      sS[pos] = j;
    }
    cnt += tot;
    __syncthreads();
  }
  block_sum<int, 2>(dv, red);
  // neighbours of the changed centers after the move, by spin (one warp per center; lane 0 keeps the counts)
  const int k = min(cnt, KS);
  int pc[2] = {0, 0};
  for (int a = wid; a < k; a += 8) {
    const int c = sS[a];
    const T xc = rp[3 * c], yc = rp[3 * c + 1], zc = rp[3 * c + 2];
    const bool sc = c < n_up;
    for (int j0 = 0; j0 < n; j0 += 32) {
      const int j = j0 + lane;
      bool in = false;
      if (j < n && j != c) in = exact_dist(xc, yc, zc, rp[3 * j], rp[3 * j + 1], rp[3 * j + 2]) < cutoff;
      const bool same = (j < n_up) == sc;
      pc[0] += __popc(__ballot_sync(kFull, in && same));
      pc[1] += __popc(__ballot_sync(kFull, in && !same));
    }
  }
  if (lane != 0) pc[0] = pc[1] = 0;
  // e-n maximum of the electrons that stay (the state's lists); the moved electrons' lists at their new positions
  // (one warp per moved slot; padded slots get an empty list)
  int em = 0;
  for (int i = tid; i < n; i += blockDim.x) {
    bool isM = false;
    for (int t = 0; t < KM; ++t) isM |= sm[t] == i;
    if (!isM) em = max(em, nb.en_cnt[(size_t)w * n + i]);
  }
  em = warp_max(em);
  if (lane == 0) emx[wid] = em;
  for (int t = wid; t < KM; t += 8) {
    const int m = sm[t];
    const size_t slot = (size_t)w * KM + t;
    if (m >= n) {
      if (lane == 0) {
        en_cnt_p[slot] = 0;
        re_p[3 * slot] = re_p[3 * slot + 1] = re_p[3 * slot + 2] = T(0);
      }
      continue;
    }
    const T xn = rp[3 * m], yn = rp[3 * m + 1], zn = rp[3 * m + 2];
    int ce = 0;
    for (int I0 = 0; I0 < N; I0 += 32) {
      const int I = I0 + lane;
      bool in = false;
      if (I < N) in = exact_dist(xn, yn, zn, (T)R[3 * I], (T)R[3 * I + 1], (T)R[3 * I + 2]) < cutoff_1el;
      const unsigned mk = __ballot_sync(kFull, in);
      const int pos = ce + __popc(mk & lt);
      if (in && pos < nb.cap_nuc) en_idx_p[slot * nb.cap_nuc + pos] = I;
      ce += __popc(mk);
    }
    if (lane == 0) {
      en_cnt_p[slot] = min(ce, nb.cap_nuc);
      re_p[3 * slot] = xn;
      re_p[3 * slot + 1] = yn;
      re_p[3 * slot + 2] = zn;
      atomicMax(&ce_max, ce);
    }
  }
  block_sum<int, 2>(pc, red);
  if (tid == 0) {
    int ee = ce_max;
    for (int q = 0; q < 8; ++q) ee = max(ee, emx[q]);
    counts_p[w * 4 + 0] = nb.counts[w * 4 + 0] + dv[0];
    counts_p[w * 4 + 1] = nb.counts[w * 4 + 1] + dv[1];
    counts_p[w * 4 + 2] = 0;
    counts_p[w * 4 + 3] = ee;
    S_cnt[w] = cnt;
    if (static_max) {
      atomicMax(&static_max[4], cnt);
      atomicMax(&static_max[5], pc[0]);
      atomicMax(&static_max[6], pc[1]);
    }
    if (cnt > KS) {
      set_flag(status, FIRE_FLAG_CHANGED_OVERFLOW);
      max_word(status, 4, cnt);
    }
    if (ce_max > nb.cap_nuc) {
      set_flag(status, FIRE_FLAG_NUC_OVERFLOW);
      max_word(status, 2, ce_max);
    }
  }
}

// rawU [W][KS][DN] holds the spin-up contraction of every changed row and rawD the spin-down one; the rows of
// spin-down centers are copied over, so that rawU ends with each row contracted with its own spin's weights.
// One CTA per (slot, walker).
template <typename T>
__global__ void __launch_bounds__(256) k_lr_orb(const int* __restrict__ S, const int* __restrict__ S_cnt, int KS,
                                                int n_up, int DN, T* __restrict__ rawU, const T* __restrict__ rawD) {
  const int slot = blockIdx.x, w = blockIdx.y;
  if (slot >= min(S_cnt[w], KS) || S[(size_t)w * KS + slot] < n_up) return;
  const size_t row = ((size_t)w * KS + slot) * DN;
  for (int q = threadIdx.x; q < DN; q += blockDim.x) rawU[row + q] = rawD[row + q];
}

// Envelope coefficients of the moved electrons at their new positions, one row per moved slot (walker w, slot t,
// electron e = moved[w][t]), with the softplus scales of e's spin: coefU / coefD [NDET][W KM][N * 8] hold
// exp(-|r_e - R_I| sp[I][d][k]) in the set of e's spin and zeros in the other (both zero for a padded slot), so that
// the two spins' contractions with their own envelope weights add up to e's row.  One thread per (row, nucleus, k).
template <typename T>
__global__ void k_lr_env_coef(const T* __restrict__ rn, const float* __restrict__ R, const T* __restrict__ sp_up,
                              const T* __restrict__ sp_dn, const int* __restrict__ moved, int KM, int n, int n_up,
                              int N, int Wc, T* __restrict__ coefU, T* __restrict__ coefD) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long rows = (long)Wc * KM;
  if (idx >= rows * N * NENV_ORB) return;
  const int k = (int)(idx % NENV_ORB), I = (int)((idx / NENV_ORB) % N);
  const long row = idx / ((long)NENV_ORB * N);
  const int w = (int)(row / KM), e = moved[row];
  const int K8 = N * NENV_ORB;
  if (e >= n) {
#pragma unroll
    for (int d = 0; d < NDET; ++d) {
      coefU[((long)d * rows + row) * K8 + I * NENV_ORB + k] = T(0);
      coefD[((long)d * rows + row) * K8 + I * NENV_ORB + k] = T(0);
    }
    return;
  }
  const bool up = e < n_up;
  const T* x = rn + ((size_t)w * n + e) * 3;
  const T dx = x[0] - (T)R[3 * I], dy = x[1] - (T)R[3 * I + 1], dz = x[2] - (T)R[3 * I + 2];
  const T rho = dsqrt(dx * dx + dy * dy + dz * dz);
  const T* sp = up ? sp_up : sp_dn;
#pragma unroll
  for (int d = 0; d < NDET; ++d) {
    const long o = ((long)d * rows + row) * K8 + I * NENV_ORB + k;
    const T v = dexp(-sp[(I * NDET + d) * NENV_ORB + k] * rho);
    coefU[o] = up ? v : T(0);
    coefD[o] = up ? T(0) : v;
  }
}

// env_p [W KM][DN] += env_d [W KM][DN]: the spin-down contraction added to the spin-up one (one of the two is zero).
template <typename T>
__global__ void k_lr_env_add(long total, T* __restrict__ env_p, const T* __restrict__ env_d) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < total) env_p[i] += env_d[i];
}

// One CTA (256 threads) per (determinant d, walker w).  rawS [W][KS][DN]: raw orbital rows of S; env, Apl
// [W][n][DN]: the state's envelope and orbital-matrix rows; env_p [W][KM][DN]: the envelope rows of the moved
// electrons moved[w][0..KM) after the move.  B: the
// transposed inverse, B[((w NDET + d) n + i) nA + sh + o] = (A^-1)[o][i] with nA = ainv_ld(n), sh = (d n) mod 4.
// Writes V [W][NDET][KS][n] (A'[S] - A[S]), Minv [W][NDET][KS][KS] (double) and the proposal's slogdet
// (ld_p, sd_p) = (ld + log|det M|, sd sign(det M)).  A set larger than KS (flagged by k_lr_select) gives sign 0:
// the proposal is rejected.  Dynamic shared memory: KS * KS doubles (M, inverted in place) + 2 * KS * 33 elements
// of T (the staged V and B[S] columns).
template <typename T>
__global__ void __launch_bounds__(256) k_lr_det(const int* __restrict__ S, const int* __restrict__ S_cnt, int KS,
                                                int n, const int* __restrict__ moved, int KM, const T* __restrict__ rawS,
                                                const T* __restrict__ env,
                                                const T* __restrict__ env_p, const T* __restrict__ Apl,
                                                const T* __restrict__ B, const double* __restrict__ ld,
                                                const double* __restrict__ sd, T* __restrict__ V,
                                                double* __restrict__ Minv, double* __restrict__ ld_p,
                                                double* __restrict__ sd_p) {
  // the k x k elimination in double precision: FP64 in the FP64 build, double-FP32 otherwise (the FP32 pipes run it
  // several times faster than GB300's FP64 pipe)
  using SE = typename std::conditional<sizeof(T) == 8, double, df64>::type;
  extern __shared__ __align__(16) unsigned char lr_smem[];
  SE* Ms = reinterpret_cast<SE*>(lr_smem);                      // [k][k], row stride k
  T* Vt = reinterpret_cast<T*>(Ms + (size_t)KS * KS);          // [KS][33]
  T* Bt = Vt + (size_t)KS * 33;                                // [KS][33]
  __shared__ int sS[LR_KMAX];
  __shared__ int perm[LR_KMAX];
  __shared__ SE fac[LR_KMAX];
  __shared__ int piv_row;
  const int d = blockIdx.x, w = blockIdx.y, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int cnt = S_cnt[w];
  const size_t md = (size_t)w * NDET + d;
  if (cnt > KS) {
    if (tid == 0) {
      ld_p[md] = ld[md];
      sd_p[md] = 0.0;
    }
    return;
  }
  const int k = cnt;
  const int DN = NDET * n, nA = ainv_ld(n), sh = (d * n) & 3;
  for (int a = tid; a < k; a += blockDim.x) sS[a] = S[(size_t)w * KS + a];
  for (int q = tid; q < k * k; q += blockDim.x) Ms[q] = (q / k == q % k) ? SE(1.0) : SE(0.0);
  __syncthreads();
  // V rows: A'[S] - A[S] (the orbital-matrix rows are raw * envelope, as in the value path)
  T* Vw = V + md * KS * n;
  for (long q = tid; q < (long)k * n; q += blockDim.x) {
    const int a = (int)(q / n), o = (int)(q - (long)a * n), c = sS[a];
    const T* er = env + ((size_t)w * n + c) * DN;
    for (int t = 0; t < KM; ++t)
      if (moved[(size_t)w * KM + t] == c) er = env_p + ((size_t)w * KM + t) * DN;
    const T an = rawS[((size_t)w * KS + a) * DN + (size_t)d * n + o] * er[(size_t)d * n + o];
    Vw[(size_t)a * n + o] = an - Apl[((size_t)w * n + c) * DN + (size_t)d * n + o];
  }
  __syncthreads();
  // M = I + V A^-1[:, S]: (A^-1)[o][S_b] = B[S_b][o]; 32 orbitals per pass
  const T* Bw = B + md * n * nA + sh;
  for (int o0 = 0; o0 < n; o0 += 32) {
    for (int q = tid; q < k * 32; q += blockDim.x) {
      const int a = q >> 5, oo = q & 31, o = o0 + oo;
      Vt[a * 33 + oo] = o < n ? Vw[(size_t)a * n + o] : T(0);
      Bt[a * 33 + oo] = o < n ? Bw[(size_t)sS[a] * nA + o] : T(0);
    }
    __syncthreads();
    for (int q = tid; q < k * k; q += blockDim.x) {
      const int a = q / k, b = q - a * k;
      T s = T(0);
#pragma unroll 8
      for (int oo = 0; oo < 32; ++oo) s += Vt[a * 33 + oo] * Bt[b * 33 + oo];
      Ms[q] += SE(s);
    }
    __syncthreads();
  }
  // in-place Gauss-Jordan with row pivoting: after step t row t holds the pivot row of the inverse; the row swaps
  // are undone on the columns at the end.  det M = (-1)^swaps prod(pivots).
  double ldet = 0.0;
  int neg = 0;
  bool singular = false;
  for (int t = 0; t < k; ++t) {
    if (wid == 0) {
      double best = -1.0;
      int bi = t;
      for (int i = t + lane; i < k; i += 32) {
        const double v = fabs((double)Ms[i * k + t]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(kFull, best, o);
        const int oi = __shfl_xor_sync(kFull, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
          best = ob;
          bi = oi;
        }
      }
      if (lane == 0) {
        piv_row = bi;
        perm[t] = bi;
      }
    }
    __syncthreads();
    const int p = piv_row;
    if (p != t) {
      for (int q = tid; q < k; q += blockDim.x) {
        const SE x = Ms[t * k + q];
        Ms[t * k + q] = Ms[p * k + q];
        Ms[p * k + q] = x;
      }
      neg ^= 1;
    }
    __syncthreads();
    const SE pv = Ms[t * k + t];
    const double pvd = (double)pv;
    if (pvd == 0.0) {
      singular = true;
      break;
    }
    ldet += log(fabs(pvd));
    if (pvd < 0.0) neg ^= 1;
    const SE ip = SE(1.0) / pv;
    __syncthreads();
    for (int q = tid; q < k; q += blockDim.x) {
      Ms[t * k + q] = q == t ? ip : Ms[t * k + q] * ip;
      fac[q] = q == t ? SE(0.0) : Ms[q * k + t];
    }
    __syncthreads();
    for (int q = tid; q < k * k; q += blockDim.x) {
      const int i = q / k, c = q - i * k;
      if (i == t) continue;
      Ms[q] = c == t ? -(fac[i] * Ms[t * k + t]) : df_sub_mul(Ms[q], fac[i], Ms[t * k + c]);
    }
    __syncthreads();
  }
  if (!singular) {
    for (int t = k - 1; t >= 0; --t) {
      const int p = perm[t];
      if (p != t)
        for (int i = tid; i < k; i += blockDim.x) {
          const SE x = Ms[i * k + t];
          Ms[i * k + t] = Ms[i * k + p];
          Ms[i * k + p] = x;
        }
      __syncthreads();
    }
  }
  double* Mo = Minv + md * KS * KS;
  for (int q = tid; q < k * k; q += blockDim.x) {
    const int a = q / k, b = q - a * k;
    Mo[(size_t)a * KS + b] = singular ? 0.0 : (double)Ms[q];
  }
  if (tid == 0) {
    ld_p[md] = ld[md] + (singular ? 0.0 : ldet);
    sd_p[md] = singular ? 0.0 : (neg ? -sd[md] : sd[md]);
  }
}

// Jastrow sums of the proposal, one CTA (256 threads) per walker.  Ax [W][2][272]: per spin the attention
// numerators sum_i a_i[h] v_i[h * 16 + dd] (thread h * 16 + dd) then the 16 normalisers sum_i a_i[h], the layout of
// the value path's sums; JM [W][2]: the sum of the MLP rows.  Rows of S come from the proposal (aS [W][KS][16],
// vS [W][KS][256], oS [W][KS][2]), all others from the state (aX [W][n][16], vals [W][n][256], Xo [W][n][2]).
template <typename T>
__global__ void __launch_bounds__(256) k_lr_jsums(int n, int n_up, const int* __restrict__ S,
                                                  const int* __restrict__ S_cnt, int KS, const T* __restrict__ aX,
                                                  const T* __restrict__ vals, const T* __restrict__ Xo,
                                                  const T* __restrict__ aS, const T* __restrict__ vS,
                                                  const T* __restrict__ oS, T* __restrict__ Ax, T* __restrict__ JM) {
  __shared__ int slot_of[ELOC_MAX_EL];
  __shared__ T red[32 * 2];
  const int w = blockIdx.x, tid = threadIdx.x, h = tid >> 4;
  const int k = min(S_cnt[w], KS);
  for (int i = tid; i < n; i += blockDim.x) slot_of[i] = -1;
  __syncthreads();
  for (int a = tid; a < k; a += blockDim.x) slot_of[S[(size_t)w * KS + a]] = a;
  __syncthreads();
  T num0 = T(0), num1 = T(0), nrm0 = T(0), nrm1 = T(0);
  for (int i = 0; i < n; ++i) {
    const int sl = slot_of[i];
    const T* ar = sl >= 0 ? aS + ((size_t)w * KS + sl) * HEADS : aX + ((size_t)w * n + i) * HEADS;
    const T* vr = sl >= 0 ? vS + ((size_t)w * KS + sl) * F : vals + ((size_t)w * n + i) * F;
    const T x = ar[h] * vr[tid];
    const T a = tid < HEADS ? ar[tid] : T(0);
    if (i < n_up) {
      num0 += x;
      nrm0 += a;
    } else {
      num1 += x;
      nrm1 += a;
    }
  }
  T m[2] = {T(0), T(0)};
  for (int i = tid; i < n; i += blockDim.x) {
    const int sl = slot_of[i];
    const T* orow = sl >= 0 ? oS + ((size_t)w * KS + sl) * 2 : Xo + ((size_t)w * n + i) * 2;
    m[0] += orow[0];
    m[1] += orow[1];
  }
  block_sum<T, 2>(m, red);
  T* a0 = Ax + (size_t)w * 2 * 272;
  a0[tid] = num0;
  a0[272 + tid] = num1;
  if (tid < HEADS) {
    a0[256 + tid] = nrm0;
    a0[272 + 256 + tid] = nrm1;
  }
  if (tid == 0) {
    JM[w * 2] = m[0];
    JM[w * 2 + 1] = m[1];
  }
}

// On acceptance (accf[w] != 0) the proposal's rows go into the state.  Blocks 0..KS-1: the rows of that slot's
// changed center (embedding h, raw orbital and orbital-matrix rows, attention weight / value rows, MLP rows);
// blocks KS..KS+KM-1: a moved electron's ElecInit and envelope rows and its e-n list, block KS also the statics and
// the slogdets.
template <typename T>
__global__ void __launch_bounds__(256) k_lr_commit(const int* __restrict__ accf, const int* __restrict__ S,
                                                   const int* __restrict__ S_cnt, int KS, int n,
                                                   const int* __restrict__ moved, int KM,
                                                   const T* __restrict__ hS, const T* __restrict__ rawS,
                                                   const T* __restrict__ env_p, const T* __restrict__ aS,
                                                   const T* __restrict__ vS, const T* __restrict__ oS,
                                                   const T* __restrict__ E5p, const int* __restrict__ en_cnt_p,
                                                   const int* __restrict__ en_idx_p, const int* __restrict__ counts_p,
                                                   const double* __restrict__ ld_p, const double* __restrict__ sd_p,
                                                   T* __restrict__ h, T* __restrict__ rawx, T* __restrict__ env,
                                                   T* __restrict__ Apl, T* __restrict__ aX, T* __restrict__ vals,
                                                   T* __restrict__ Xo, T* __restrict__ E5o, Nbr nb,
                                                   double* __restrict__ ld, double* __restrict__ sd) {
  const int slot = blockIdx.x, w = blockIdx.y, tid = threadIdx.x;
  if (!accf[w]) return;
  const int DN = NDET * n;
  if (slot >= KS) {
    const int t = slot - KS;
    const size_t ms = (size_t)w * KM + t;
    if (t == 0) {
      if (tid < 4) nb.counts[w * 4 + tid] = counts_p[w * 4 + tid];
      if (tid < NDET) {
        ld[(size_t)w * NDET + tid] = ld_p[(size_t)w * NDET + tid];
        sd[(size_t)w * NDET + tid] = sd_p[(size_t)w * NDET + tid];
      }
    }
    const int e = moved[ms];
    if (e >= n) return;
    const size_t g = (size_t)w * n + e;
    for (int q = tid; q < 5 * F; q += blockDim.x) E5o[g * 5 * F + q] = E5p[ms * 5 * F + q];
    for (int q = tid; q < DN; q += blockDim.x) env[g * DN + q] = env_p[ms * DN + q];
    const int ce = en_cnt_p[ms];
    for (int q = tid; q < ce; q += blockDim.x) nb.en_idx[g * nb.cap_nuc + q] = en_idx_p[ms * nb.cap_nuc + q];
    if (tid == 0) nb.en_cnt[g] = ce;
    return;
  }
  if (slot >= min(S_cnt[w], KS)) return;
  const int c = S[(size_t)w * KS + slot];
  const size_t g = (size_t)w * n + c, row = (size_t)w * KS + slot;
  // a moved electron's envelope row is read from the proposal (the blocks from KS on overwrite the state's row)
  const T* er = env + g * DN;
  for (int t = 0; t < KM; ++t)
    if (moved[(size_t)w * KM + t] == c) er = env_p + ((size_t)w * KM + t) * DN;
  for (int q = tid; q < F; q += blockDim.x) {
    h[g * F + q] = hS[row * F + q];
    vals[g * F + q] = vS[row * F + q];
  }
  for (int q = tid; q < DN; q += blockDim.x) {
    const T x = rawS[row * DN + q];
    rawx[g * DN + q] = x;
    Apl[g * DN + q] = x * er[q];
  }
  if (tid < HEADS) aX[g * HEADS + tid] = aS[row * HEADS + tid];
  if (tid < 2) Xo[g * 2 + tid] = oS[row * 2 + tid];
}

// Woodbury, part 1: Z = B V^T for 32 rows of B per CTA, Z [W][NDET][n][KS].  grid (ceil(n / 32), NDET, W), 256
// threads: thread (ii, g) accumulates rows i0 + ii against columns a = g + 8 t.
template <typename T>
__global__ void __launch_bounds__(256) k_lr_wb_z(const int* __restrict__ accf, const int* __restrict__ S_cnt, int KS,
                                                 int n, const T* __restrict__ B, const T* __restrict__ V,
                                                 T* __restrict__ Zb) {
  __shared__ T Bt[32][33];
  __shared__ T Vt[LR_KMAX][33];
  const int w = blockIdx.z, d = blockIdx.y, i0 = blockIdx.x * 32, tid = threadIdx.x, ii = tid & 31, g = tid >> 5;
  if (!accf[w]) return;
  const int k = min(S_cnt[w], KS);
  const int nA = ainv_ld(n), sh = (d * n) & 3;
  const size_t md = (size_t)w * NDET + d;
  const T* Bw = B + md * n * nA + sh;
  const T* Vw = V + md * KS * n;
  T acc[kAcc];
#pragma unroll
  for (int t = 0; t < kAcc; ++t) acc[t] = T(0);
  for (int o0 = 0; o0 < n; o0 += 32) {
    for (int q = tid; q < 32 * 32; q += blockDim.x) {
      const int rr = q >> 5, oo = q & 31;
      Bt[rr][oo] = (i0 + rr < n && o0 + oo < n) ? Bw[(size_t)(i0 + rr) * nA + o0 + oo] : T(0);
    }
    for (int q = tid; q < k * 32; q += blockDim.x) {
      const int a = q >> 5, oo = q & 31;
      Vt[a][oo] = o0 + oo < n ? Vw[(size_t)a * n + o0 + oo] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < kAcc; ++t) {
      const int a = g + 8 * t;
      if (a < k) {
        T s = acc[t];
#pragma unroll 8
        for (int oo = 0; oo < 32; ++oo) s += Bt[ii][oo] * Vt[a][oo];
        acc[t] = s;
      }
    }
    __syncthreads();
  }
  if (i0 + ii < n) {
#pragma unroll
    for (int t = 0; t < kAcc; ++t) {
      const int a = g + 8 * t;
      if (a < k) Zb[(md * n + i0 + ii) * KS + a] = acc[t];
    }
  }
}

// Woodbury, part 2: Q = M^-T B[S, :] for 32 columns per CTA, Q [W][NDET][KS][n]: Q[a][j] = sum_b M^-1[b][a]
// B[S_b][j].  grid (ceil(n / 32), NDET, W), 256 threads: thread (jj, g) accumulates column j0 + jj for a = g + 8 t.
template <typename T>
__global__ void __launch_bounds__(256) k_lr_wb_q(const int* __restrict__ accf, const int* __restrict__ S,
                                                 const int* __restrict__ S_cnt, int KS, int n, const T* __restrict__ B,
                                                 const double* __restrict__ Minv, T* __restrict__ Qb) {
  __shared__ T Ms[32][LR_KMAX + 1];
  __shared__ T Bs[32][33];
  const int w = blockIdx.z, d = blockIdx.y, j0 = blockIdx.x * 32, tid = threadIdx.x, jj = tid & 31, g = tid >> 5;
  if (!accf[w]) return;
  const int k = min(S_cnt[w], KS);
  const int nA = ainv_ld(n), sh = (d * n) & 3;
  const size_t md = (size_t)w * NDET + d;
  const T* Bw = B + md * n * nA + sh;
  const double* Mo = Minv + md * KS * KS;
  T acc[kAcc];
#pragma unroll
  for (int t = 0; t < kAcc; ++t) acc[t] = T(0);
  for (int b0 = 0; b0 < k; b0 += 32) {
    for (int q = tid; q < 32 * k; q += blockDim.x) {
      const int bb = q / k, a = q - bb * k;
      Ms[bb][a] = b0 + bb < k ? (T)Mo[(size_t)(b0 + bb) * KS + a] : T(0);
    }
    for (int q = tid; q < 32 * 32; q += blockDim.x) {
      const int bb = q >> 5, cc = q & 31;
      Bs[bb][cc] = (b0 + bb < k && j0 + cc < n) ? Bw[(size_t)S[(size_t)w * KS + b0 + bb] * nA + j0 + cc] : T(0);
    }
    __syncthreads();
    for (int bb = 0; bb < 32; ++bb) {
      const T bv = Bs[bb][jj];
#pragma unroll
      for (int t = 0; t < kAcc; ++t) {
        const int a = g + 8 * t;
        if (a < k) acc[t] += Ms[bb][a] * bv;
      }
    }
    __syncthreads();
  }
  if (j0 + jj < n) {
#pragma unroll
    for (int t = 0; t < kAcc; ++t) {
      const int a = g + 8 * t;
      if (a < k) Qb[(md * KS + a) * n + j0 + jj] = acc[t];
    }
  }
}

// Woodbury, part 3: B -= Z Q for 32 rows of B per CTA, all columns.  grid (ceil(n / 32), NDET, W), 256 threads:
// thread (jj, g) updates rows i0 + g + 8 t (t < 4) of column j0 + jj.
template <typename T>
__global__ void __launch_bounds__(256) k_lr_wb_apply(const int* __restrict__ accf, const int* __restrict__ S_cnt,
                                                     int KS, int n, T* __restrict__ B, const T* __restrict__ Zb,
                                                     const T* __restrict__ Qb) {
  __shared__ T Zs[32][33];
  __shared__ T Qs[32][33];
  const int w = blockIdx.z, d = blockIdx.y, i0 = blockIdx.x * 32, tid = threadIdx.x, jj = tid & 31, g = tid >> 5;
  if (!accf[w]) return;
  const int k = min(S_cnt[w], KS);
  const int nA = ainv_ld(n), sh = (d * n) & 3;
  const size_t md = (size_t)w * NDET + d;
  T* Bw = B + md * n * nA + sh;
  const T* Zw = Zb + md * n * KS;
  const T* Qw = Qb + md * KS * n;
  for (int j0 = 0; j0 < n; j0 += 32) {
    T acc[4] = {T(0), T(0), T(0), T(0)};
    for (int a0 = 0; a0 < k; a0 += 32) {
      for (int q = tid; q < 32 * 32; q += blockDim.x) {
        const int rr = q >> 5, cc = q & 31;
        Zs[rr][cc] = (i0 + rr < n && a0 + cc < k) ? Zw[(size_t)(i0 + rr) * KS + a0 + cc] : T(0);
        Qs[rr][cc] = (a0 + rr < k && j0 + cc < n) ? Qw[(size_t)(a0 + rr) * n + j0 + cc] : T(0);
      }
      __syncthreads();
#pragma unroll 8
      for (int aa = 0; aa < 32; ++aa) {
        const T qv = Qs[aa][jj];
#pragma unroll
        for (int t = 0; t < 4; ++t) acc[t] += Zs[g + 8 * t][aa] * qv;
      }
      __syncthreads();
    }
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int i = i0 + g + 8 * t, j = j0 + jj;
      if (i < n && j < n) Bw[(size_t)i * nA + j] -= acc[t];
    }
  }
}

#define FIRE_INST_LR(T)                                                                                             \
  template __global__ void k_lr_select<T>(const T*, const T*, int, int, const int*, int, const float*, int, T, T, Nbr, \
                                          int, int*, int*, T*, int*, int*, int*, int32_t*, int32_t*);                \
  template __global__ void k_lr_env_coef<T>(const T*, const float*, const T*, const T*, const int*, int, int, int, int,  \
                                            int, T*, T*);                                                             \
  template __global__ void k_lr_env_add<T>(long, T*, const T*);                                                      \
  template __global__ void k_lr_orb<T>(const int*, const int*, int, int, int, T*, const T*);                         \
  template __global__ void k_lr_det<T>(const int*, const int*, int, int, const int*, int, const T*, const T*, const T*, \
                                       const T*, const T*, const double*, const double*, T*, double*, double*,       \
                                       double*);                                                                      \
  template __global__ void k_lr_jsums<T>(int, int, const int*, const int*, int, const T*, const T*, const T*,        \
                                         const T*, const T*, const T*, T*, T*);                                       \
  template __global__ void k_lr_commit<T>(const int*, const int*, const int*, int, int, const int*, int, const T*,     \
                                          const T*,                                                                  \
                                          const T*, const T*, const T*, const T*, const T*, const int*, const int*,   \
                                          const int*, const double*, const double*, T*, T*, T*, T*, T*, T*, T*, T*, \
                                          Nbr, double*, double*);                                                     \
  template __global__ void k_lr_wb_z<T>(const int*, const int*, int, int, const T*, const T*, T*);                   \
  template __global__ void k_lr_wb_q<T>(const int*, const int*, const int*, int, int, const T*, const double*, T*); \
  template __global__ void k_lr_wb_apply<T>(const int*, const int*, int, int, T*, const T*, const T*);
FIRE_INST_LR(float)
FIRE_INST_LR(double)

}  // namespace fire
