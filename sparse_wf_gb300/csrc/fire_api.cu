// fire_api.cu -- the C ABI (include/fire.h): layouts, workspace planning and the chunked pipelines.
//
// Stage order of one chunk of walkers for the local energy (the forward-Laplacian path,
// wave_function.py:165-181 + hamiltonian.py:69-81):
//   neighbours -> layout -> ElecInit (edges, LayerNorm) -> GLU/Dense/Dense GEMMs on [x, jac, lap]
//   -> e-e edges + messages -> update MLP (2 x silu layers) -> envelopes -> orbitals
//   -> FP64 Gauss-Jordan -> determinant Laplacian -> attention Jastrow -> MLP Jastrow -> assembly.
// The value path (log|psi|, the MCMC building block) runs the same stages without tangents.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fire_gemm.cuh"
#include "fire_kernels.cuh"

using namespace fire;

namespace {

// Converts the last launch error into a status; with FIRE_DEBUG set in the environment the CUDA error
// string is printed to stderr.
fire_status launch_status(const char* where) {
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return FIRE_OK;
  if (std::getenv("FIRE_DEBUG")) std::fprintf(stderr, "[fire] %s: %s\n", where, cudaGetErrorString(e));
  return FIRE_ERR_CUDA;
}

// ------------------------------------------------------------------------------ stage profiling
struct ProfRec {
  const char* name;
  cudaEvent_t a, b;
};
bool g_prof = false;
long long g_nlaunch = 0;  // kernels launched by this library since the last fire_profile_enable
std::vector<ProfRec> g_recs;
std::vector<cudaEvent_t> g_pool;
cudaEvent_t prof_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}
struct Prof {
  const char* name;
  cudaStream_t s;
  cudaEvent_t a = nullptr;
  Prof(const char* n, cudaStream_t st) : name(n), s(st) {
    if (g_prof) {
      a = prof_event();
      cudaEventRecord(a, s);
    }
  }
  ~Prof() {
    if (g_prof && a) {
      cudaEvent_t b = prof_event();
      cudaEventRecord(b, s);
      g_recs.push_back({name, a, b});
    }
  }
};

// ------------------------------------------------------------------------------ parameter layout
void slot_sizes(const fire_problem* p, int64_t* sz) {
  const int64_t n = p->n_el, N = p->n_nuc, D = NDET, Fl = F;
  const int64_t s[FIRE_P_COUNT] = {
      N * NENV_EN, N * 4 * F0, N * F0, N * Fl,                      // en
      F0 * F1, F1, NENV_EN * F1, F1 * Fl, 4 * Fl,                   // ei filter, gamma, edge
      Fl, Fl, Fl * 2 * Fl, Fl * Fl, Fl, Fl * 5 * Fl, 5 * Fl,        // ln, glu, dense, out
      F0, 4 * F0, F0, F0 * F1, F1, NENV_EE * F1, F1 * Fl, 4 * Fl, Fl,  // ee same
      F0, 4 * F0, F0, F0 * F1, F1, NENV_EE * F1, F1 * Fl, 4 * Fl, Fl,  // ee diff
      Fl * Fl, Fl, Fl * Fl, Fl, 2, 1,                               // updates, scales, cutoff_param
      Fl * D * n, D * n, Fl * D * n, D * n,                         // orbitals
      N * D * NENV_ORB, N * D * NENV_ORB * n, N * D * NENV_ORB, N * D * NENV_ORB * n,  // envelopes
      4,                                                            // cusp
      Fl * Fl, Fl, Fl * Fl, Fl, Fl * 2, 2, 2, 1,                    // MLP Jastrow
      HEADS * HDIM, Fl * Fl, Fl, Fl * Fl, Fl,                       // attention keys, Q, V
      2 * Fl * Fl, Fl, Fl * Fl, Fl, Fl * 2, 2, 2, 1};               // readout, scale, bias
  for (int k = 0; k < FIRE_P_COUNT; ++k) sz[k] = s[k];
}
int64_t align64(int64_t x) { return (x + 63) / 64 * 64; }
void blob_offsets(const fire_problem* p, int64_t* off) {
  int64_t sz[FIRE_P_COUNT];
  slot_sizes(p, sz);
  int64_t o = 0;
  for (int k = 0; k < FIRE_P_COUNT; ++k) {
    off[k] = o;
    o += align64(sz[k]);
  }
  off[FIRE_P_COUNT] = o;
}
// prepared slots (elements of the compute type)
void prep_offsets(const fire_problem* p, int64_t* off) {
  blob_offsets(p, off);
  const int64_t n = p->n_el, N = p->n_nuc, D = NDET;
  int64_t o = off[FIRE_P_COUNT];
  const int64_t ds[PR_COUNT - PR_UPD1_W_S0] = {
      F * F, F * D * n, F * D * n, F * F, F * HEADS, HEADS, F * F, N * NENV_EN, NENV_EE, NENV_EE,
      N * D * NENV_ORB, N * D * NENV_ORB, D * N * NENV_ORB * n, D * N * NENV_ORB * n, 8};
  for (int k = PR_UPD1_W_S0; k < PR_COUNT; ++k) {
    off[k] = o;
    o += align64(ds[k - PR_UPD1_W_S0]);
  }
  off[PR_COUNT] = o;
}
size_t elem_size(const fire_problem* p) { return p->precision == FIRE_PREC_FP64 ? 8 : 4; }

// Split BF16 copies of the contraction weights used on tensor cores (mixed precision only), stored
// after the float slots of the prepared buffer: for each, hi [N][K] then lo [N][K].
enum TcSlot {
  TC_UPD1, TC_UPD2, TC_ORB_UP, TC_ORB_DN, TC_V, TC_JMLP1, TC_JMLP2, TC_EI_GLU, TC_EI_DENSE, TC_EI_OUT,
  TC_ENV_UP, TC_ENV_DN, TC_QK, TC_COUNT
};
struct TcSrc {
  int slot;  // prepared slot (already scaled), row-major [K][N] per matrix
  int kind;  // > 0: K = F, N = kind * F;  0: K = F, N = NDET * n_el (orbitals);
             // -1: NDET matrices with K = 8 n_nuc, N = n_el (envelope weights per determinant);
             // -2: K = F, N = HEADS (attention logits)
};
const TcSrc kTcSrc[TC_COUNT] = {{PR_UPD1_W_S0, 1},   {FIRE_P_UPD2_W, 1},    {PR_ORB_UP_W_S1, 0},
                                {PR_ORB_DN_W_S1, 0}, {PR_V_W_S1, 1},        {PR_JMLP1_W_S1, 1},
                                {FIRE_P_JMLP2_W, 1}, {FIRE_P_EI_GLU_W, 2},  {FIRE_P_EI_DENSE_W, 1},
                                {FIRE_P_EI_OUT_W, 5}, {PR_ENV_UP_PI, -1},   {PR_ENV_DN_PI, -1},
                                {PR_QK_W_S1, -2}};
// K, N and the number of matrices of a slot.  Its BF16 copy: the pre-tiled split of every matrix
// (tc_tiles_bytes each) for the A-resident kernel (K <= 256) and the envelope kernel, else hi [cnt][N][K]
// followed by lo [cnt][N][K] (for the streamed-weight kernel).
void tc_shape(int k, const fire_problem* p, size_t* K, size_t* N, int* cnt) {
  const int kind = kTcSrc[k].kind;
  *K = kind == -1 ? (size_t)NENV_ORB * p->n_nuc : (size_t)F;
  *N = kind > 0 ? (size_t)kind * F
                : (kind == 0 ? (size_t)NDET * p->n_el : (kind == -1 ? (size_t)p->n_el : (size_t)HEADS));
  *cnt = kind == -1 ? NDET : 1;
}
bool tc_tiled(int k, size_t K) { return K <= 256 || kTcSrc[k].kind == -1; }
// FP16 scaled-grid tiles followed by the column scales (cnt x N floats): the A-resident kernel's slots (K <= 256) and
// the envelope kernel's (K = 8 N <= ENV_TC_KMAX, hi parts narrowed by grid_hb so that the K-long sums stay exact)
bool tc_grid(int k, size_t K) { return K <= 256 || (kTcSrc[k].kind == -1 && K <= (size_t)ENV_TC_KMAX); }
// byte offset of a grid slot's column scales from its tiles
size_t tc_cs_offset(size_t K, size_t N, int cnt) { return (size_t)cnt * tc_tiles_bytes(K, N); }
// byte offsets of the BF16 region (tc_off[TC_COUNT] = end)
void tc_offsets(const fire_problem* p, size_t float_bytes, size_t* off) {
  size_t o = (float_bytes + 255) / 256 * 256;
  for (int k = 0; k < TC_COUNT; ++k) {
    off[k] = o;
    size_t K, N;
    int cnt;
    tc_shape(k, p, &K, &N, &cnt);
    o += tc_tiled(k, K) ? (size_t)cnt * tc_tiles_bytes(K, N) : 2 * (size_t)cnt * N * K * sizeof(__nv_bfloat16);
    if (tc_grid(k, K)) o += (size_t)cnt * N * sizeof(float);
    o = (o + 255) / 256 * 256;
  }
  off[TC_COUNT] = o;
}

// Byte offset of the FP64 prepared weights (the refinement pass's) in an FP32 / mixed prepared buffer: after the
// float slots and, in the mixed path, the BF16 tensor-core weights.
size_t prep64_offset(const fire_problem* p) {
  int64_t off[PR_COUNT + 1];
  prep_offsets(p, off);
  size_t end = (size_t)off[PR_COUNT] * 4;
  if (p->precision == FIRE_PREC_MIXED) {
    size_t to[TC_COUNT + 1];
    tc_offsets(p, end, to);
    end = to[TC_COUNT];
  }
  return (end + 255) / 256 * 256;
}

bool valid(const fire_problem* p) {
  return p && p->n_el >= 2 && p->n_el <= MAX_EL && p->n_up >= 0 && p->n_up <= p->n_el && p->n_nuc >= 1 &&
         p->n_walkers >= 1 && p->cutoff > 0 && p->cutoff_1el > 0 && p->cap_pairs >= 1 && p->cap_nuc >= 1 &&
         p->precision >= 0 && p->precision <= 2 && p->refine_cap >= 0;
}

// ------------------------------------------------------------------------------ workspace plan
struct Plan {
  // int
  size_t deg, rowptr, nbr, rev, en_cnt, en_idx, counts, pos_off, pos_ctr, pos_dep, dep_pos;
  // T
  size_t E5a, Z1, E5o, HX, HL, HJ, B1X, B1L, B1J, B2X, B2L, B2J, Zx, Zx2, jsq;
  size_t env, rawx, rjs, Apl, lapA, Jorb, coef_up, coef_dn, Ainv, dgrad, env_lo, Apl_lo;
  size_t aX, aJ, aL, Ax, Al, AJ, RX, RJ, RL, R1X, R1J, R1L, R2X, R2J, R2L, Zr, Zr2, jsqr;
  size_t JAx, JAj, JAl, Xo2, Jo2, Lo2, JMx, JMl, JMj, rn, lpn, plr, tile_mask, aD1, aD2, ajsq;
  // double
  size_t ld, sd, dlap, cond, gjw, enn;
  size_t total;
};

Plan make_plan(const fire_problem* p, int Wc, bool fl) {
  Plan P;
  std::memset(&P, 0, sizeof(P));
  const size_t es = elem_size(p);
  const size_t n = p->n_el, nu = p->n_up, nd = p->n_el - p->n_up, N = p->n_nuc, cp = p->cap_pairs,
               cn = p->cap_nuc, W = Wc;
  const size_t G = W * n, Pc = W * (n + cp), Jr = 3 * Pc, DN = NDET * n, NV = fl ? 5 : 1;
  size_t o = 0;
  auto take = [&](size_t& field, size_t count, size_t bytes_per) {
    o = (o + 255) / 256 * 256;
    field = o;
    o += count * bytes_per;
  };
  take(P.deg, G, 4);
  take(P.rowptr, W * (n + 1), 4);
  take(P.nbr, W * cp, 4);
  take(P.rev, W * cp, 4);
  take(P.en_cnt, G, 4);
  take(P.en_idx, G * cn, 4);
  take(P.counts, W * 4, 4);
  if (fl) {
    take(P.pos_off, W + 1, 4);
    take(P.pos_ctr, Pc, 4);
    take(P.pos_dep, Pc, 4);
    take(P.dep_pos, Pc, 4);
  }
  take(P.E5a, G * NV * F, es);
  take(P.Z1, G * NV * 2 * F, es);
  take(P.E5o, G * NV * 5 * F, es);
  take(P.HX, G * F, es);
  take(P.B1X, G * F, es);
  take(P.B2X, G * F, es);
  take(P.Zx, G * F, es);
  if (fl) {
    take(P.HL, G * F, es);
    take(P.HJ, Jr * F, es);
    take(P.B1L, G * F, es);
    take(P.B1J, Jr * F, es);
    take(P.B2L, G * F, es);
    take(P.B2J, Jr * F, es);
    take(P.jsq, G * F, es);
    take(P.Zx2, G * F, es);
  }
  take(P.env, G * NV * DN, es);
  take(P.rawx, G * DN, es);
  take(P.Apl, G * DN, es);
  if (es == 4) {  // FP32 / mixed: the low parts of the compensated envelope values and orbital matrices
    take(P.env_lo, G * DN, 4);
    take(P.Apl_lo, G * DN, 4);
  }
  take(P.coef_up, NDET * W * nu * NV * N * NENV_ORB, es);
  take(P.coef_dn, NDET * W * nd * NV * N * NENV_ORB, es);
  if (fl) {
    take(P.rjs, G * 3 * DN, es);
    take(P.lapA, G * DN, es);
    take(P.Jorb, Jr * DN, es);
    take(P.Ainv, W * NDET * n * (size_t)ainv_ld((int)n), es);
    take(P.dgrad, W * NDET * n * 3, 8);
  }
  take(P.aX, G * HEADS, es);
  take(P.Ax, W * 2 * 272, es);
  take(P.RX, W * 512, es);
  take(P.R1X, W * F, es);
  take(P.R2X, W * F, es);
  take(P.Zr, W * F, es);
  take(P.JAx, W * 2, es);
  take(P.Xo2, G * 2, es);
  take(P.JMx, W * 2, es);
  if (fl) {
    take(P.aJ, Jr * HEADS, es);
    take(P.aD1, G * HEADS, es);
    take(P.aD2, G * HEADS, es);
    take(P.ajsq, G * HEADS, es);
    take(P.aL, G * HEADS, es);
    take(P.Al, W * 2 * 272, es);
    take(P.AJ, W * 3 * n * 2 * 272, es);
    take(P.RJ, W * 3 * n * 512, es);
    take(P.RL, W * 512, es);
    take(P.R1J, W * 3 * n * F, es);
    take(P.R1L, W * F, es);
    take(P.R2J, W * 3 * n * F, es);
    take(P.R2L, W * F, es);
    take(P.jsqr, W * F, es);
    take(P.Zr2, W * F, es);
    take(P.JAj, W * 3 * n * 2, es);
    take(P.JAl, W * 2, es);
    take(P.Jo2, Jr * 2, es);
    take(P.Lo2, G * 2, es);
    take(P.JMl, W * 2, es);
    take(P.JMj, W * 3 * n * 2, es);
  }
  take(P.gjw, 2 * W * NDET * n * n, 8);  // two working copies per matrix for the Gauss-Jordan / LU kernel
  take(P.enn, 1, 8);
  take(P.tile_mask, (fl ? 3 * Pc : G) / 128 + 2, 4);
  take(P.rn, G * 3, es);
  take(P.lpn, W, es);
  take(P.plr, W, es);
  take(P.ld, W * NDET, 8);
  take(P.sd, W * NDET, 8);
  take(P.dlap, W * NDET, 8);
  if (fl) take(P.cond, W * NDET, 8);
  P.total = (o + 255) / 256 * 256;
  return P;
}

// ---- refinement pass of the FP32 / mixed local energy (see fire_local_energy in fire.h)
// Walkers refined per call: refine_cap, at most the batch; none in the FP64 build.
int refine_walkers(const fire_problem* p) {
  return p->precision == FIRE_PREC_FP64 ? 0 : std::min(p->refine_cap, p->n_walkers);
}
// The FP64 value path's problem for KF walkers.
fire_problem refine_problem64(const fire_problem* p, int KF) {
  fire_problem q = *p;
  q.precision = FIRE_PREC_FP64;
  q.n_walkers = KF;
  q.chunk_walkers = KF;
  q.refine_cap = 0;
  return q;
}
// Workspace of one pass over KC refined walkers, at offset 0 once the batch's chunks are done: the chunk plan of
// the KC walkers, the FP64 value-path plan of the same walkers, their positions in the walkers' dtype and in FP64.
struct RefineLayout {
  size_t c64, r_ref, r64, total;
};
RefineLayout refine_layout(const fire_problem* p, int KC) {
  RefineLayout L;
  fire_problem pr = *p;
  pr.n_walkers = KC;
  const fire_problem p64 = refine_problem64(p, KC);
  const size_t n3 = (size_t)KC * p->n_el * 3;
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  L.c64 = up(make_plan(&pr, KC, true).total);
  L.r_ref = up(L.c64 + make_plan(&p64, KC, false).total);
  L.r64 = up(L.r_ref + n3 * elem_size(p));
  L.total = up(L.r64 + n3 * 8);
  return L;
}
// Total workspace of the local energy with chunks of Wc walkers: the larger of the chunk plan and the refinement
// pass (in passes of at most Wc walkers), then the list of ill-conditioned walkers (KF indices, their count and
// one count per pass), which lives through both.
size_t eloc_ws_bytes(const fire_problem* p, int Wc, size_t* list_off) {
  const int KF = refine_walkers(p);
  size_t t = make_plan(p, Wc, true).total;
  if (KF > 0) t = std::max(t, refine_layout(p, std::min(KF, Wc)).total);
  if (list_off) *list_off = t;
  return KF > 0 ? t + ((size_t)(2 * KF + 1) * 4 + 255) / 256 * 256 : t;
}

int choose_chunk(const fire_problem* p, size_t ws_bytes, bool fl) {
  int B = p->n_walkers;
  auto need = [&](int c) { return fl ? eloc_ws_bytes(p, c, nullptr) : make_plan(p, c, fl).total; };
  if (p->chunk_walkers > 0) {
    int c = std::min(B, p->chunk_walkers);
    // a fixed pass is reduced to what the CUDA-core contraction of the Jacobian planes can launch: 65535 row tiles
    // of 128 in the grid's y dimension
    if (fl) c = (int)std::min<long>(c, std::max<long>(1, 65535L * 128 / (3L * (p->n_el + p->cap_pairs))));
    return need(c) <= ws_bytes ? c : 0;
  }
  // the rows of a pass's largest contraction (the Jacobian planes; the electron rows of the value path) stay within
  // the 65535 row tiles of 64 that a launch grid's y dimension holds
  const long rows_per_walker = fl ? 3L * (p->n_el + p->cap_pairs) : (long)p->n_el;
  B = (int)std::min<long>(B, std::max<long>(1, 65535L * 64 / rows_per_walker));
  int lo = 0, hi = B;
  while (lo < hi) {  // largest c with plan(c) <= ws
    const int mid = (lo + hi + 1) / 2;
    if (need(mid) <= ws_bytes) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ------------------------------------------------------------------------------ prepare kernels
template <typename T>
__global__ void k_convert(const float* __restrict__ in, T* __restrict__ out, long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (T)in[i];
}
template <typename T>
__global__ void k_scale_copy(const float* __restrict__ in, T* __restrict__ out, long n, const float* __restrict__ sc) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (T)((double)in[i] * (double)sc[0]);
}
template <typename T>
__global__ void k_qk(const float* __restrict__ QW, const float* __restrict__ Qb, const float* __restrict__ K,
                     const float* __restrict__ s1, T* __restrict__ W, T* __restrict__ b) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;  // f * 16 + h
  if (idx < F * HEADS) {
    const int f = idx / HEADS, h = idx % HEADS;
    double s = 0.0;
    for (int d = 0; d < HDIM; ++d) s += (double)QW[f * F + h * HDIM + d] * K[h * HDIM + d];
    W[idx] = (T)(s * s1[0]);
  }
  if (idx < HEADS) {
    double s = 0.0;
    for (int d = 0; d < HDIM; ++d) s += (double)Qb[idx * HDIM + d] * K[idx * HDIM + d];
    b[idx] = (T)s;
  }
}
template <typename T>
__global__ void k_softplus(const float* __restrict__ in, T* __restrict__ out, long n, int invert) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double x = in[i];
    const double sp = x > 30.0 ? x : log1p(exp(x));
    out[i] = (T)(invert ? 1.0 / sp : sp);
  }
}
template <typename T>
__global__ void k_pi_perdet(const float* __restrict__ pi, T* __restrict__ out, int N, int n) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;  // over (d, I, k, o)
  const long total = (long)NDET * N * NENV_ORB * n;
  if (idx >= total) return;
  const int o = (int)(idx % n);
  const int k = (int)((idx / n) % NENV_ORB);
  const int I = (int)((idx / ((long)n * NENV_ORB)) % N);
  const int d = (int)(idx / ((long)n * NENV_ORB * N));
  out[idx] = (T)pi[(((long)I * NDET + d) * NENV_ORB + k) * n + o];
}
template <typename T>
__global__ void k_scalars(const float* __restrict__ cutoff_param, const float* __restrict__ log_bias, float cutoff,
                          T* __restrict__ out) {
  if (threadIdx.x == 0) {
    const double cp = cutoff_param[0];
    out[0] = (T)((double)cutoff / (1.0 + exp(-cp)));
    out[1] = T(0);
    out[2] = (T)log_bias[0];
    for (int k = 3; k < 8; ++k) out[k] = T(0);
  }
}

inline unsigned nblk(long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

template <typename T>
fire_status prepare_impl(cudaStream_t s, const fire_problem* p, const float* blob, const int64_t* boff,
                         void* prepared) {
  int64_t off[PR_COUNT + 1];
  prep_offsets(p, off);
  T* out = reinterpret_cast<T*>(prepared);
  const long nb = (long)off[FIRE_P_COUNT];
  g_nlaunch++;
  k_convert<T><<<nblk(nb), 256, 0, s>>>(blob, out, nb);
  const float* s0 = blob + boff[FIRE_P_SCALES];
  const float* s1 = blob + boff[FIRE_P_SCALES] + 1;
  const long n = p->n_el, N = p->n_nuc;
  auto scl = [&](int src, int dst, long cnt, const float* sc) {
    g_nlaunch++;
    k_scale_copy<T><<<nblk(cnt), 256, 0, s>>>(blob + boff[src], out + off[dst], cnt, sc);
  };
  scl(FIRE_P_UPD1_W, PR_UPD1_W_S0, (long)F * F, s0);
  scl(FIRE_P_ORB_UP_W, PR_ORB_UP_W_S1, (long)F * NDET * n, s1);
  scl(FIRE_P_ORB_DN_W, PR_ORB_DN_W_S1, (long)F * NDET * n, s1);
  scl(FIRE_P_JMLP1_W, PR_JMLP1_W_S1, (long)F * F, s1);
  scl(FIRE_P_ATT_V_W, PR_V_W_S1, (long)F * F, s1);
  g_nlaunch++;
  k_qk<T><<<nblk(F * HEADS), 256, 0, s>>>(blob + boff[FIRE_P_ATT_Q_W], blob + boff[FIRE_P_ATT_Q_B],
                                          blob + boff[FIRE_P_ATT_KEYS], s1, out + off[PR_QK_W_S1],
                                          out + off[PR_QK_B]);
  g_nlaunch++;
  k_softplus<T><<<nblk(N * NENV_EN), 256, 0, s>>>(blob + boff[FIRE_P_EN_SCALES], out + off[PR_EN_INVSCALE],
                                                  N * NENV_EN, 1);
  g_nlaunch++;
  k_softplus<T><<<1, 256, 0, s>>>(blob + boff[FIRE_P_EESAME_SCALE], out + off[PR_EESAME_INVSCALE], NENV_EE, 1);
  g_nlaunch++;
  k_softplus<T><<<1, 256, 0, s>>>(blob + boff[FIRE_P_EEDIFF_SCALE], out + off[PR_EEDIFF_INVSCALE], NENV_EE, 1);
  g_nlaunch++;
  k_softplus<T><<<nblk(N * NDET * NENV_ORB), 256, 0, s>>>(blob + boff[FIRE_P_ENV_UP_SIGMA], out + off[PR_ENV_UP_SP],
                                                          N * NDET * NENV_ORB, 0);
  g_nlaunch++;
  k_softplus<T><<<nblk(N * NDET * NENV_ORB), 256, 0, s>>>(blob + boff[FIRE_P_ENV_DN_SIGMA], out + off[PR_ENV_DN_SP],
                                                          N * NDET * NENV_ORB, 0);
  g_nlaunch++;
  k_pi_perdet<T><<<nblk((long)NDET * N * NENV_ORB * n), 256, 0, s>>>(blob + boff[FIRE_P_ENV_UP_PI],
                                                                      out + off[PR_ENV_UP_PI], (int)N, (int)n);
  g_nlaunch++;
  k_pi_perdet<T><<<nblk((long)NDET * N * NENV_ORB * n), 256, 0, s>>>(blob + boff[FIRE_P_ENV_DN_PI],
                                                                      out + off[PR_ENV_DN_PI], (int)N, (int)n);
  g_nlaunch++;
  k_scalars<T><<<1, 32, 0, s>>>(blob + boff[FIRE_P_CUTOFF_PARAM], blob + boff[FIRE_P_LOG_BIAS], p->cutoff,
                                out + off[PR_SCALARS]);
  return launch_status(__func__);
}

template <typename T>
Weights<T> make_weights(const fire_problem* p, const void* prepared) {
  int64_t off[PR_COUNT + 1];
  prep_offsets(p, off);
  Weights<T> W;
  const T* base = reinterpret_cast<const T*>(prepared);
  for (int k = 0; k < PR_COUNT; ++k) W.w[k] = base + off[k];
  return W;
}

// ------------------------------------------------------------------------------ chunk context
template <typename T>
struct Ctx {
  const fire_problem* p;
  cudaStream_t s;
  int Wc;     // walkers in this chunk
  int Wmax;   // planned chunk size
  int w0;
  int B;
  const T* r;  // chunk base
  const float* R;
  const float* Z;
  Weights<T> W;
  int32_t* status;
  unsigned char* ws;
  Plan P;
  Nbr nb;
  Layout L;
  bool mixed = false;
  // FP32 / mixed: value planes by the compensated contraction and the orbital matrices as hi + lo pairs (the local
  // energy, log|psi| and the low-rank state); the Metropolis blocks' proposals, which only compare log|psi| values,
  // take the plain contraction
  bool comp = true;
  // the refinement pass's FP64 value path: its envelope value rows by the double-FP32 compensated contraction
  bool env_df = false;
  TcWeights tcw[TC_COUNT];
  template <typename U>
  U* buf(size_t off) const {
    return reinterpret_cast<U*>(ws + off);
  }
};

template <typename T>
void setup_ctx(Ctx<T>& c, bool fl) {
  const fire_problem* p = c.p;
  c.nb.W = c.Wc;
  c.nb.n = p->n_el;
  c.nb.n_up = p->n_up;
  c.nb.N = p->n_nuc;
  c.nb.cap_p = p->cap_pairs;
  c.nb.cap_nuc = p->cap_nuc;
  c.nb.deg = c.template buf<int>(c.P.deg);
  c.nb.rowptr = c.template buf<int>(c.P.rowptr);
  c.nb.nbr = c.template buf<int>(c.P.nbr);
  c.nb.rev = c.template buf<int>(c.P.rev);
  c.nb.en_cnt = c.template buf<int>(c.P.en_cnt);
  c.nb.en_idx = c.template buf<int>(c.P.en_idx);
  c.nb.counts = c.template buf<int>(c.P.counts);
  if (fl) {
    c.L.pos_off = c.template buf<int>(c.P.pos_off);
    c.L.pos_ctr = c.template buf<int>(c.P.pos_ctr);
    c.L.pos_dep = c.template buf<int>(c.P.pos_dep);
    c.L.dep_pos = c.template buf<int>(c.P.dep_pos);
    c.L.cap_pos = c.Wc * (p->n_el + p->cap_pairs);
  } else {
    std::memset(&c.L, 0, sizeof(c.L));
  }
}

template <typename T>
GemmP<T> gp0() {
  GemmP<T> g;
  std::memset(&g, 0, sizeof(g));
  g.node_div = 1;
  g.M_scale = 1;
  g.env_nv = 1;
  return g;
}

template <typename T, int MODE>
cudaError_t gemm(const Ctx<T>& c, GemmP<T> g, int tc_id = -1) {
  // profile stages: "gemm_tc" the tensor-core contractions, "gemm" the CUDA-core ones
  const bool tc = sizeof(T) == 4 && c.mixed && tc_id >= 0;
  Prof pr(tc ? "gemm_tc" : "gemm", c.s);
  g_nlaunch++;
  if constexpr (sizeof(T) == 4) {
    if (tc) {
      const int bn = g.N > 256 ? 128 : 256;
      return gemm_tc(MODE, bn, g, c.tcw[tc_id], c.template buf<int>(c.P.tile_mask), c.status, c.s);
    }
  }
  return launch_gemm<T, MODE>(g, c.s);
}

// compensated value contraction (FP32 and mixed paths): low parts into C_lo / read from env_lo, row stride ld_lo
template <int MODE>
cudaError_t gemm_comp(const Ctx<float>& c, const GemmP<float>& g, float* C_lo, const float* env_lo, long ld_lo) {
  Prof pr("gemm_comp", c.s);
  g_nlaunch++;
  return launch_gemm_comp<MODE>(g, C_lo, env_lo, ld_lo, c.s);
}

// Value-plane contraction of a dense layer (EPI_PLAIN or EPI_SILU_X): compensated in the FP32 and mixed paths.
template <typename T, int MODE>
cudaError_t value_gemm(const Ctx<T>& c, const GemmP<T>& g) {
  if constexpr (sizeof(T) == 4) {
    static_assert(MODE == EPI_PLAIN || MODE == EPI_SILU_X, "value_gemm: plain or SiLU layers");
    if (!c.comp) return gemm<T, MODE>(c, g);
    return gemm_comp<MODE == EPI_PLAIN ? COMP_PLAIN : COMP_SILU>(c, g, nullptr, nullptr, 0);
  } else {
    return gemm<T, MODE>(c, g);
  }
}

// neighbour lists (+ layout for the forward-Laplacian path)
template <typename T>
cudaError_t stage_neighbors(Ctx<T>& c, bool fl) {
  Prof pr("neighbors", c.s);
  const int n = c.p->n_el;
  const size_t smem = 3 * n * sizeof(T) + (5 * n + 2) * sizeof(int);
  fire_neighbor_out ext;
  std::memset(&ext, 0, sizeof(ext));
  // always opt in: the kernel's static shared memory adds to the dynamic size
  cudaFuncSetAttribute(k_neighbors<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  g_nlaunch++;
  k_neighbors<T><<<c.Wc, 512, smem, c.s>>>(c.r, c.R, (T)c.p->cutoff, (T)c.p->cutoff_1el, c.nb, ext, c.status);
  if (fl) {
    g_nlaunch++;
    k_pos_scan<<<1, 1024, 0, c.s>>>(c.nb, c.L.pos_off);
    g_nlaunch++;
    k_layout<<<c.Wc, 256, 0, c.s>>>(c.nb, c.L);
  }
  return cudaPeekAtLastError();
}

// ElecInit + GLU/Dense/Dense on the electron carriers, then edges + messages -> H
// ElecInit contraction over the interleaved [x, jac(3), lap] rows of every electron.  In the mixed path
// the tensor cores take the derivative rows (the value rows they also compute are not stored) and the
// CUDA cores the value rows, read with a stride of NV rows: the value plane stays FP32.
template <typename T>
cudaError_t ei_gemm(Ctx<T>& c, const GemmP<T>& g, int NV, int tc_id) {
  if (NV == 1) return value_gemm<T, EPI_PLAIN>(c, g);
  GemmP<T> gv = g;  // the value rows (every NV-th row), compensated in the FP32 and mixed paths
  gv.lda = g.lda * NV;
  gv.ldc = g.ldc * NV;
  gv.M = g.M / NV;
  gv.bias_period = g.bias ? 1 : 0;
  if (!c.mixed) {
    // FP32 (and FP64): all rows by the CUDA-core contraction; in FP32 the value rows once more, compensated
    cudaError_t e = gemm<T, EPI_PLAIN>(c, g);
    if (e != cudaSuccess || sizeof(T) == 8) return e;
    return value_gemm<T, EPI_PLAIN>(c, gv);
  }
  GemmP<T> gt = g;
  gt.bias = nullptr;
  gt.bias_period = 0;
  gt.row_skip = NV;
  cudaError_t e = gemm<T, EPI_PLAIN>(c, gt, tc_id);
  if (e != cudaSuccess) return e;
  return value_gemm<T, EPI_PLAIN>(c, gv);
}

template <typename T, int NT>
cudaError_t stage_embedding(Ctx<T>& c) {
  constexpr int NV = NT > 0 ? NT + 2 : 1;
  const int n = c.p->n_el, G = c.Wc * n;
  T* E5a = c.template buf<T>(c.P.E5a);
  T* Z1 = c.template buf<T>(c.P.Z1);
  T* E5o = c.template buf<T>(c.P.E5o);
  {
    Prof pr("elec_init", c.s);
    g_nlaunch++;
    k_elec_init<T, NT><<<G, 256, 0, c.s>>>(c.r, c.R, c.nb, c.W, (T)(1.0 / c.p->cutoff_1el), E5a);
  }
  Prof pr_e5("elec_mlp", c.s);
  GemmP<T> g = gp0<T>();
  g.A = E5a; g.lda = F; g.B = c.W.w[FIRE_P_EI_GLU_W]; g.ldb = 2 * F; g.C = Z1; g.ldc = 2 * F;
  g.M = G * NV; g.N = 2 * F; g.K = F;
  ei_gemm<T>(c, g, NV, TC_EI_GLU);
  g_nlaunch++;
  k_glu<T, NT><<<nblk((long)G * F), 256, 0, c.s>>>(Z1, E5a, G);
  g = gp0<T>();
  g.A = E5a; g.lda = F; g.B = c.W.w[FIRE_P_EI_DENSE_W]; g.ldb = F; g.C = Z1; g.ldc = F;
  g.bias = c.W.w[FIRE_P_EI_DENSE_B]; g.bias_period = NV;
  g.M = G * NV; g.N = F; g.K = F;
  ei_gemm<T>(c, g, NV, TC_EI_DENSE);
  g_nlaunch++;
  k_silu5<T, NT><<<nblk((long)G * F), 256, 0, c.s>>>(Z1, G);
  g = gp0<T>();
  g.A = Z1; g.lda = F; g.B = c.W.w[FIRE_P_EI_OUT_W]; g.ldb = 5 * F; g.C = E5o; g.ldc = 5 * F;
  g.bias = c.W.w[FIRE_P_EI_OUT_B]; g.bias_period = NV;
  g.M = G * NV; g.N = 5 * F; g.K = F;
  ei_gemm<T>(c, g, NV, TC_EI_OUT);
  Prof pr("edge_contract", c.s);
  k_edge_contract<T, NT><<<G, 256, 0, c.s>>>(c.r, c.nb, c.L, c.W, E5o, c.template buf<T>(c.P.HX),
                                             NT ? c.template buf<T>(c.P.HL) : nullptr,
                                             NT ? c.template buf<T>(c.P.HJ) : nullptr);
  return cudaPeekAtLastError();
}

struct Planes {
  size_t X, J, L;
};

// Linear(F -> N) + SiLU on a sparse node (value path: X plane only)
template <typename T>
cudaError_t silu_layer(Ctx<T>& c, bool fl, Planes in, Planes out, const T* Wt, const T* b, int K, int N,
                       int rowsX, int rowsJcap, const int* rowsJdev, const int* node_map, int node_div, size_t zx,
                       size_t jsq, int tc_id = -1) {
  GemmP<T> g = gp0<T>();
  g.A = c.template buf<T>(in.X); g.lda = K; g.B = Wt; g.ldb = N; g.bias = b; g.C = c.template buf<T>(out.X);
  g.ldc = N; g.M = rowsX; g.N = N; g.K = K; g.ld_aux = N;
  if (fl) {  // silu' and silu'' planes for the Jacobian / Laplacian epilogues
    g.aux0 = c.template buf<T>(zx);
    g.aux2 = c.template buf<T>(c.P.Zx2);
  }
  value_gemm<T, EPI_SILU_X>(c, g);
  if (!fl) return cudaPeekAtLastError();
  cudaMemsetAsync(c.template buf<T>(jsq), 0, sizeof(T) * (size_t)rowsX * N, c.s);
  g = gp0<T>();
  g.A = c.template buf<T>(in.J); g.lda = K; g.B = Wt; g.ldb = N; g.C = c.template buf<T>(out.J); g.ldc = N;
  g.M = rowsJcap; g.M_dev = rowsJdev; g.M_scale = 3; g.N = N; g.K = K; g.node_map = node_map;
  g.node_div = node_div; g.aux1 = c.template buf<T>(zx); g.aux2 = c.template buf<T>(jsq); g.ld_aux = N;
  gemm<T, EPI_SILU_J>(c, g, tc_id);
  g = gp0<T>();
  g.A = c.template buf<T>(in.L); g.lda = K; g.B = Wt; g.ldb = N; g.C = c.template buf<T>(out.L); g.ldc = N;
  g.M = rowsX; g.N = N; g.K = K; g.aux1 = c.template buf<T>(zx); g.aux0 = c.template buf<T>(c.P.Zx2);
  g.aux3 = c.template buf<T>(jsq); g.ld_aux = N;
  gemm<T, EPI_SILU_L>(c, g, tc_id);
  return cudaPeekAtLastError();
}

// Linear(F -> N) without activation on a node (bias on X only)
template <typename T>
cudaError_t linear_layer(Ctx<T>& c, bool fl, Planes in, Planes out, const T* Wt, const T* b, int K, int N,
                         int rowsX, int rowsJcap, const int* rowsJdev, int tc_id = -1) {
  GemmP<T> g = gp0<T>();
  g.A = c.template buf<T>(in.X); g.lda = K; g.B = Wt; g.ldb = N; g.bias = b; g.bias_period = 1;
  g.C = c.template buf<T>(out.X); g.ldc = N; g.M = rowsX; g.N = N; g.K = K;
  value_gemm<T, EPI_PLAIN>(c, g);
  if (!fl) return cudaPeekAtLastError();
  g.A = c.template buf<T>(in.J); g.bias = nullptr; g.C = c.template buf<T>(out.J); g.M = rowsJcap;
  g.M_dev = rowsJdev; g.M_scale = rowsJdev ? 3 : 1;
  gemm<T, EPI_PLAIN>(c, g, tc_id);
  g.A = c.template buf<T>(in.L); g.C = c.template buf<T>(out.L); g.M = rowsX; g.M_dev = nullptr; g.M_scale = 1;
  gemm<T, EPI_PLAIN>(c, g, tc_id);
  return cudaPeekAtLastError();
}

// envelopes + orbital matrices (+ their Jacobian/Laplacian planes)
template <typename T, int NT>
cudaError_t stage_orbitals(Ctx<T>& c) {
  constexpr int NV = NT > 0 ? NT + 2 : 1;
  const bool fl = NT > 0;
  const int n = c.p->n_el, nu = c.p->n_up, N = c.p->n_nuc, G = c.Wc * n, DN = NDET * n;
  T* env = c.template buf<T>(c.P.env);
  Prof pr("orbitals", c.s);
  for (int s = 0; s < 2; ++s) {
    const int ns = s == 0 ? nu : n - nu;
    if (ns == 0) continue;
    T* coef = c.template buf<T>(s == 0 ? c.P.coef_up : c.P.coef_dn);
    const T* sp = c.W.w[s == 0 ? PR_ENV_UP_SP : PR_ENV_DN_SP];
    const long tot = (long)c.Wc * ns * N * NENV_ORB, K8 = (long)N * NENV_ORB;
    // mixed path: the derivative rows come from k_env_tc (coefficients generated on chip, tensor cores), so
    // only the value coefficients are materialised, for the compensated FP32 contraction of the value rows; the
    // Metropolis blocks' plain value rows come from k_env_tc as well (value tiles), with no coefficients in memory
    const bool tc_ok = sizeof(T) == 4 && c.mixed && NENV_ORB * N <= ENV_TC_KMAX;
    const bool tc_env = tc_ok && NV > 1;
    const bool tc_val = tc_ok && NV == 1 && !c.comp;
    const int nvc = tc_env ? 1 : NV;  // coefficient rows per electron
    if (!tc_val) {
      g_nlaunch++;
      if (tc_env)
        k_env_coef<T, 1><<<nblk(tot), 256, 0, c.s>>>(c.r, c.R, sp, n, ns, s == 0 ? 0 : nu, N, c.Wc, coef);
      else
        k_env_coef<T, NV><<<nblk(tot), 256, 0, c.s>>>(c.r, c.R, sp, n, ns, s == 0 ? 0 : nu, N, c.Wc, coef);
    }
    const long rows = (long)c.Wc * ns * nvc;
    for (int d = 0; d < NDET; ++d) {
      if constexpr (sizeof(T) == 4) {
        if (tc_env || tc_val) {
          const int slot = s == 0 ? TC_ENV_UP : TC_ENV_DN;
          float* C = env + (long)d * n;
          const long ldc = (long)DN;
          const uintptr_t a = reinterpret_cast<uintptr_t>(C);
          const int vec = (a % 16 == 0 && ldc % 4 == 0) ? 4 : ((a % 8 == 0 && ldc % 2 == 0) ? 2 : 1);
          const EnvTcP ep{c.r, c.R, sp, C, ldc, n, ns, s == 0 ? 0 : nu, N, c.Wc, d, NV, vec, c.tcw[slot].cs + (size_t)d * n};
          Prof pg("gemm_tc", c.s);
          g_nlaunch++;
          const cudaError_t e = env_tc(ep, c.tcw[slot].tiles + (size_t)d * tc_tiles_bytes((size_t)K8, (size_t)n) / 2,
                                       c.status, c.s, tc_val);
          if (e != cudaSuccess) return e;
          if (tc_val) continue;
        }
      }
      GemmP<T> g = gp0<T>();
      g.A = coef + d * rows * K8; g.lda = K8;
      g.B = c.W.w[s == 0 ? PR_ENV_UP_PI : PR_ENV_DN_PI] + (long)d * K8 * n; g.ldb = n;
      g.C = env + (long)d * n; g.ldc = (long)DN * (NV / nvc); g.M = (int)rows; g.N = n; g.K = (int)K8;
      g.n_el = n; g.env_ns = ns; g.env_soff = s == 0 ? 0 : nu; g.env_nv = nvc;
      if constexpr (sizeof(T) == 8) {
        if (c.env_df && nvc == 1) {
          Prof pg("gemm", c.s);
          g_nlaunch++;
          const cudaError_t e = launch_gemm_env_df(g, c.s);
          if (e != cudaSuccess) return e;
          continue;
        }
      }
      if (sizeof(T) == 8 || !c.comp) {
        gemm<T, EPI_ENV>(c, g);
      } else if constexpr (sizeof(T) == 4) {
        // the value rows by the compensated contraction (hi into the carrier, lo into env_lo); with derivative
        // rows in the same coefficient block (FP32 forward Laplacian) the plain contraction takes those first
        if (nvc > 1) gemm<T, EPI_ENV>(c, g);
        GemmP<float> gv = g;
        gv.lda = (long)nvc * K8; gv.M = c.Wc * ns; gv.ldc = (long)NV * DN; gv.env_nv = 1;
        gemm_comp<COMP_ENV>(c, gv, c.template buf<float>(c.P.env_lo) + (long)d * n, nullptr, DN);
      }
    }
  }
  GemmP<T> g = gp0<T>();
  g.A = c.template buf<T>(c.P.B2X); g.lda = F; g.B = c.W.w[PR_ORB_UP_W_S1]; g.B2 = c.W.w[PR_ORB_DN_W_S1];
  g.ldb = DN; g.bias = c.W.w[FIRE_P_ORB_UP_B]; g.bias2 = c.W.w[FIRE_P_ORB_DN_B];
  g.C = c.template buf<T>(c.P.Apl); g.ldc = DN; g.M = G; g.N = DN; g.K = F; g.n_el = n; g.n_up = nu;
  g.aux0 = c.template buf<T>(c.P.rawx); g.aux1 = env; g.ld_aux = DN; g.env_nv = NV;
  if constexpr (sizeof(T) == 4) {
    if (c.comp)
      gemm_comp<COMP_ORB>(c, g, c.template buf<float>(c.P.Apl_lo), c.template buf<float>(c.P.env_lo), DN);
    else
      gemm<T, EPI_ORB_X>(c, g);
  } else {
    gemm<T, EPI_ORB_X>(c, g);
  }
  if (!fl) return cudaPeekAtLastError();
  g = gp0<T>();
  g.A = c.template buf<T>(c.P.B2J); g.lda = F; g.B = c.W.w[PR_ORB_UP_W_S1]; g.B2 = c.W.w[PR_ORB_DN_W_S1];
  g.ldb = DN; g.C = c.template buf<T>(c.P.Jorb); g.ldc = DN; g.M = 3 * c.L.cap_pos;
  g.M_dev = c.L.pos_off + c.Wc; g.M_scale = 3; g.N = DN; g.K = F; g.n_el = n; g.n_up = nu;
  g.node_map = c.L.pos_ctr; g.node_div = 3; g.dep_map = c.L.pos_dep; g.aux1 = env;
  g.aux2 = c.template buf<T>(c.P.rjs); g.aux3 = c.template buf<T>(c.P.rawx); g.ld_aux = DN; g.env_nv = 5;
  gemm<T, EPI_ORB_J>(c, g, TC_ORB_UP);
  g = gp0<T>();
  g.A = c.template buf<T>(c.P.B2L); g.lda = F; g.B = c.W.w[PR_ORB_UP_W_S1]; g.B2 = c.W.w[PR_ORB_DN_W_S1];
  g.ldb = DN; g.C = c.template buf<T>(c.P.lapA); g.ldc = DN; g.M = G; g.N = DN; g.K = F; g.n_el = n; g.n_up = nu;
  g.aux1 = env; g.aux2 = c.template buf<T>(c.P.rjs); g.aux3 = c.template buf<T>(c.P.rawx); g.ld_aux = DN;
  g.env_nv = 5;
  if constexpr (sizeof(T) == 4) {
    if (c.mixed) {
      // the Laplacian rows' product rule reads nine planes per output; as the tensor-core epilogue it left the MMAs
      // idle (one CTA of 8 epilogue warps per SM), so the contraction stores plain values and a streaming kernel
      // at full occupancy applies the rule in place
      GemmP<T> gp = g;
      gp.aux0 = nullptr; gp.aux1 = nullptr; gp.aux2 = nullptr; gp.aux3 = nullptr; gp.env_nv = 1;
      const cudaError_t e = gemm<T, EPI_PLAIN>(c, gp, TC_ORB_UP);
      if (e != cudaSuccess) return e;
      const long q = (long)G * (DN / 4);
      g_nlaunch++;
      k_orb_lap<<<nblk(q), 256, 0, c.s>>>(c.template buf<float>(c.P.lapA), env, c.template buf<float>(c.P.rawx),
                                          c.template buf<float>(c.P.rjs), G, DN);
      return cudaPeekAtLastError();
    }
  }
  gemm<T, EPI_ORB_L>(c, g, TC_ORB_UP);
  return cudaPeekAtLastError();
}

// Gauss-Jordan inversion (INV) or LU of every orbital matrix of the chunk, one CTA per matrix with the
// working matrix in the workspace (k_gj_global).  Its shared memory (two panel buffers of n x 17 eight-byte
// elements plus ~2.5 KB) limits the inverse, and so the local energy, to ELOC_MAX_EL electrons.
template <typename S, typename TI, typename TO, bool INV>
cudaError_t launch_gjg(const Ctx<TI>& c, const TI* A, const TI* A_lo, TO* Ainv, double* cond = nullptr) {
  const int n = c.p->n_el;
  constexpr int BW = GJG_BW_DECL;
  const size_t smem =
      sizeof(S) * (2 * (size_t)n * (BW + 1) + BW * BW + n + 3 * BW) + sizeof(int) * (2 * (size_t)n + BW);
  auto kern = k_gj_global<S, TI, TO, INV>;
  // always opt in: the kernel's static shared memory adds to the dynamic size
  const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  g_nlaunch++;
  kern<<<c.Wc * NDET, GJG_THREADS_DECL, smem, c.s>>>(A, A_lo, n, c.template buf<S>(c.P.gjw),
                                                      c.template buf<double>(c.P.ld), c.template buf<double>(c.P.sd),
                                                      cond, Ainv, c.status);
  return cudaPeekAtLastError();
}

// Jastrow: attention (Q.keys narrow + V + sums + readout MLP) and MLP Jastrow; H and B1 are scratch.
template <typename T, int NT>
cudaError_t stage_jastrow(Ctx<T>& c) {
  constexpr bool FLM = NT > 0;
  const int n = c.p->n_el, G = c.Wc * n, Wc = c.Wc;
  const int Jcap = 3 * c.L.cap_pos;
  const int* Jdev = FLM ? c.L.pos_off + c.Wc : nullptr;
  const Planes B2{c.P.B2X, c.P.B2J, c.P.B2L}, B1{c.P.B1X, c.P.B1J, c.P.B1L}, H{c.P.HX, c.P.HJ, c.P.HL};
  Prof pr("jastrow", c.s);
  // attention logits exp(-(h W_Qk + b_Qk) / 4)
  if (FLM && c.mixed) {
    // mixed path: value rows and the activation derivatives on the CUDA cores, Jacobian and Laplacian rows
    // as tensor-core contractions with the derivative-plane epilogues
    g_nlaunch++;
    k_narrow<T, HEADS, 1, false><<<G, 256, 0, c.s>>>(
        c.template buf<T>(B2.X), nullptr, nullptr, c.nb, c.L, c.W.w[PR_QK_W_S1], c.W.w[PR_QK_B], nullptr, nullptr,
        c.template buf<T>(c.P.aX), nullptr, nullptr, c.status, c.template buf<T>(c.P.aD1),
        c.template buf<T>(c.P.aD2));
    cudaMemsetAsync(c.template buf<T>(c.P.ajsq), 0, sizeof(T) * (size_t)G * HEADS, c.s);
    GemmP<T> g = gp0<T>();
    g.A = c.template buf<T>(B2.J); g.lda = F; g.B = c.W.w[PR_QK_W_S1]; g.ldb = HEADS;
    g.C = c.template buf<T>(c.P.aJ); g.ldc = HEADS; g.M = Jcap; g.M_dev = Jdev; g.M_scale = 3; g.N = HEADS;
    g.K = F; g.node_map = c.L.pos_ctr; g.node_div = 3; g.aux1 = c.template buf<T>(c.P.aD1);
    g.aux2 = c.template buf<T>(c.P.ajsq); g.ld_aux = HEADS;
    gemm<T, EPI_SILU_J>(c, g, TC_QK);
    g = gp0<T>();
    g.A = c.template buf<T>(B2.L); g.lda = F; g.B = c.W.w[PR_QK_W_S1]; g.ldb = HEADS;
    g.C = c.template buf<T>(c.P.aL); g.ldc = HEADS; g.M = G; g.N = HEADS; g.K = F;
    g.aux1 = c.template buf<T>(c.P.aD1); g.aux0 = c.template buf<T>(c.P.aD2);
    g.aux3 = c.template buf<T>(c.P.ajsq); g.ld_aux = HEADS;
    gemm<T, EPI_SILU_L>(c, g, TC_QK);
  } else {
    g_nlaunch++;
    k_narrow<T, HEADS, 1, FLM><<<G, 256, 0, c.s>>>(
        c.template buf<T>(B2.X), FLM ? c.template buf<T>(B2.J) : nullptr, FLM ? c.template buf<T>(B2.L) : nullptr,
        c.nb, c.L, c.W.w[PR_QK_W_S1], c.W.w[PR_QK_B], nullptr, nullptr, c.template buf<T>(c.P.aX),
        FLM ? c.template buf<T>(c.P.aJ) : nullptr, FLM ? c.template buf<T>(c.P.aL) : nullptr, c.status, nullptr,
        nullptr);
  }
  linear_layer<T>(c, FLM, B2, B1, c.W.w[PR_V_W_S1], c.W.w[FIRE_P_ATT_V_B], F, F, G, Jcap, Jdev, TC_V);
  cudaMemsetAsync(c.template buf<T>(c.P.Ax), 0, sizeof(T) * Wc * 2 * 272, c.s);
  if (FLM) cudaMemsetAsync(c.template buf<T>(c.P.Al), 0, sizeof(T) * Wc * 2 * 272, c.s);
  g_nlaunch++;
  k_att_sums<T, FLM><<<dim3(n, Wc), 256, 0, c.s>>>(
      c.nb, c.L, c.template buf<T>(c.P.aX), FLM ? c.template buf<T>(c.P.aJ) : nullptr,
      FLM ? c.template buf<T>(c.P.aL) : nullptr, c.template buf<T>(B1.X), FLM ? c.template buf<T>(B1.J) : nullptr,
      FLM ? c.template buf<T>(B1.L) : nullptr, c.template buf<T>(c.P.Ax), FLM ? c.template buf<T>(c.P.Al) : nullptr,
      FLM ? c.template buf<T>(c.P.AJ) : nullptr);
  k_readout_in<T, FLM><<<Wc, 512, 0, c.s>>>(n, c.template buf<T>(c.P.Ax), FLM ? c.template buf<T>(c.P.Al) : nullptr,
                                            FLM ? c.template buf<T>(c.P.AJ) : nullptr, c.template buf<T>(c.P.RX),
                                            FLM ? c.template buf<T>(c.P.RJ) : nullptr,
                                            FLM ? c.template buf<T>(c.P.RL) : nullptr);
  // readout MLP 512 -> 256 -> 256 -> 2 on the dense carrier (node = walker, tangents 3n)
  const Planes RI{c.P.RX, c.P.RJ, c.P.RL}, R1{c.P.R1X, c.P.R1J, c.P.R1L}, R2{c.P.R2X, c.P.R2J, c.P.R2L};
  {
    GemmP<T> g = gp0<T>();
    // layer 1/2 with dense Jacobian rows: node of a J row = row / (3n)
    auto dense_silu = [&](Planes in, Planes out, const T* Wt, const T* b, int K) {
      GemmP<T> q = gp0<T>();
      q.A = c.template buf<T>(in.X); q.lda = K; q.B = Wt; q.ldb = F; q.bias = b; q.C = c.template buf<T>(out.X);
      q.ldc = F; q.M = Wc; q.N = F; q.K = K; q.ld_aux = F;
      if (FLM) {
        q.aux0 = c.template buf<T>(c.P.Zr);
        q.aux2 = c.template buf<T>(c.P.Zr2);
      }
      gemm<T, EPI_SILU_X>(c, q);
      if (!FLM) return;
      cudaMemsetAsync(c.template buf<T>(c.P.jsqr), 0, sizeof(T) * Wc * F, c.s);
      q = gp0<T>();
      q.A = c.template buf<T>(in.J); q.lda = K; q.B = Wt; q.ldb = F; q.C = c.template buf<T>(out.J); q.ldc = F;
      q.M = Wc * 3 * n; q.N = F; q.K = K; q.node_div = 3 * n; q.aux1 = c.template buf<T>(c.P.Zr);
      q.aux2 = c.template buf<T>(c.P.jsqr); q.ld_aux = F;
      gemm<T, EPI_SILU_J>(c, q);
      q = gp0<T>();
      q.A = c.template buf<T>(in.L); q.lda = K; q.B = Wt; q.ldb = F; q.C = c.template buf<T>(out.L); q.ldc = F;
      q.M = Wc; q.N = F; q.K = K; q.aux1 = c.template buf<T>(c.P.Zr); q.aux0 = c.template buf<T>(c.P.Zr2);
      q.aux3 = c.template buf<T>(c.P.jsqr); q.ld_aux = F;
      gemm<T, EPI_SILU_L>(c, q);
    };
    dense_silu(RI, R1, c.W.w[FIRE_P_ATT_OUT1_W], c.W.w[FIRE_P_ATT_OUT1_B], 2 * F);
    dense_silu(R1, R2, c.W.w[FIRE_P_ATT_OUT2_W], c.W.w[FIRE_P_ATT_OUT2_B], F);
    g.A = c.template buf<T>(R2.X); g.lda = F; g.B = c.W.w[FIRE_P_ATT_OUT3_W]; g.ldb = 2; g.bias = c.W.w[FIRE_P_ATT_OUT3_B];
    g.bias_period = 1; g.C = c.template buf<T>(c.P.JAx); g.ldc = 2; g.M = Wc; g.N = 2; g.K = F;
    gemm<T, EPI_PLAIN>(c, g);
    if (FLM) {
      g.A = c.template buf<T>(R2.J); g.bias = nullptr; g.C = c.template buf<T>(c.P.JAj); g.M = Wc * 3 * n;
      gemm<T, EPI_PLAIN>(c, g);
      g.A = c.template buf<T>(R2.L); g.C = c.template buf<T>(c.P.JAl); g.M = Wc;
      gemm<T, EPI_PLAIN>(c, g);
    }
  }
  // MLP Jastrow: SparseMLP [256, 256, 2] (silu on every layer), * mlp_scale + [0, log_bias], sum over nodes
  silu_layer<T>(c, FLM, B2, B1, c.W.w[PR_JMLP1_W_S1], c.W.w[FIRE_P_JMLP1_B], F, F, G, Jcap, Jdev, c.L.pos_ctr, 3,
                c.P.Zx, c.P.jsq, TC_JMLP1);
  silu_layer<T>(c, FLM, B1, H, c.W.w[FIRE_P_JMLP2_W], c.W.w[FIRE_P_JMLP2_B], F, F, G, Jcap, Jdev, c.L.pos_ctr, 3,
                c.P.Zx, c.P.jsq, TC_JMLP2);
  g_nlaunch++;
  k_narrow<T, 2, 0, FLM><<<G, 256, 0, c.s>>>(
      c.template buf<T>(H.X), FLM ? c.template buf<T>(H.J) : nullptr, FLM ? c.template buf<T>(H.L) : nullptr, c.nb,
      c.L, c.W.w[FIRE_P_JMLP3_W], c.W.w[FIRE_P_JMLP3_B], c.W.w[FIRE_P_MLP_SCALE], c.W.w[PR_SCALARS] + 1,
      c.template buf<T>(c.P.Xo2), FLM ? c.template buf<T>(c.P.Jo2) : nullptr,
      FLM ? c.template buf<T>(c.P.Lo2) : nullptr, c.status, nullptr, nullptr);
  k_mlp_sum<T, FLM><<<Wc, 256, 0, c.s>>>(c.nb, c.L, c.template buf<T>(c.P.Xo2),
                                         FLM ? c.template buf<T>(c.P.Jo2) : nullptr,
                                         FLM ? c.template buf<T>(c.P.Lo2) : nullptr, c.template buf<T>(c.P.JMx),
                                         FLM ? c.template buf<T>(c.P.JMl) : nullptr,
                                         FLM ? c.template buf<T>(c.P.JMj) : nullptr);
  return cudaPeekAtLastError();
}

// update MLP: H -> B1 -> B2 (scales[0] folded into the first weight, scales[1] into the consumers)
template <typename T, int NT>
cudaError_t stage_update(Ctx<T>& c) {
  constexpr bool FLM = NT > 0;
  const int G = c.Wc * c.p->n_el;
  const int Jcap = 3 * c.L.cap_pos;
  const int* Jdev = FLM ? c.L.pos_off + c.Wc : nullptr;
  const Planes H{c.P.HX, c.P.HJ, c.P.HL}, B1{c.P.B1X, c.P.B1J, c.P.B1L}, B2{c.P.B2X, c.P.B2J, c.P.B2L};
  Prof pr("update_mlp", c.s);
  silu_layer<T>(c, FLM, H, B1, c.W.w[PR_UPD1_W_S0], c.W.w[FIRE_P_UPD1_B], F, F, G, Jcap, Jdev, c.L.pos_ctr, 3, c.P.Zx,
                c.P.jsq, TC_UPD1);
  silu_layer<T>(c, FLM, B1, B2, c.W.w[FIRE_P_UPD2_W], c.W.w[FIRE_P_UPD2_B], F, F, G, Jcap, Jdev, c.L.pos_ctr, 3, c.P.Zx,
                c.P.jsq, TC_UPD2);
  return cudaPeekAtLastError();
}

// value path for one chunk: writes logpsi/sign via the assembly (indices w0 + w)
template <typename T>
cudaError_t chunk_logpsi(Ctx<T>& c, void* logpsi, void* sign, int w0_out) {
  setup_ctx(c, false);
  stage_neighbors(c, false);
  stage_embedding<T, 0>(c);
  stage_update<T, 0>(c);
  stage_orbitals<T, 0>(c);
  // slogdet only: double-FP32 LU in the FP32 and mixed paths (FP64-class, like the inverse of the local
  // energy), native FP64 in the FP64 build
  Prof pr_lu("lu", c.s);
  if constexpr (sizeof(T) == 8)
    launch_gjg<double, T, T, false>(c, c.template buf<T>(c.P.Apl), (const T*)nullptr, (T*)nullptr);
  else
    launch_gjg<df64, T, T, false>(c, c.template buf<T>(c.P.Apl), c.comp ? c.template buf<T>(c.P.Apl_lo) : nullptr,
                                  (T*)nullptr);
  stage_jastrow<T, 0>(c);
  AssembleOut o;
  std::memset(&o, 0, sizeof(o));
  g_nlaunch++;
  k_nn_energy<<<1, 256, 0, c.s>>>(c.R, c.Z, c.p->n_nuc, c.template buf<double>(c.P.enn));
  o.enn = c.template buf<double>(c.P.enn);
  o.logpsi = logpsi;
  o.sign = sign;
  g_nlaunch++;
  k_assemble<T, false><<<c.Wc, 256, 3 * c.p->n_el * sizeof(double), c.s>>>(
      c.p->n_el, c.p->n_up, c.p->n_nuc, w0_out, c.r, c.R, c.Z, c.W, c.template buf<double>(c.P.ld),
      c.template buf<double>(c.P.sd), nullptr, nullptr, c.template buf<T>(c.P.JAx), nullptr, nullptr,
      c.template buf<T>(c.P.JMx), nullptr, nullptr, o, c.status);
  return cudaPeekAtLastError();
}

// Ill-conditioned walkers of a local-energy call: the first pass appends them to idx (count cnt, capacity cap);
// the refinement pass evaluates the chunk of their positions with the orbital matrices of c64 (FP64 values of the
// same walkers) and writes its results to their rows.
struct Refine {
  int32_t* idx = nullptr;
  int32_t* cnt = nullptr;
  int cap = 0;
  const Ctx<double>* c64 = nullptr;
};

template <typename T>
cudaError_t chunk_eloc(Ctx<T>& c, void* logpsi, void* sign, void* eloc, const fire_eloc_debug* dbg,
                       const Refine& rf = Refine()) {
  setup_ctx(c, true);
  stage_neighbors(c, true);
  stage_embedding<T, 3>(c);
  stage_update<T, 3>(c);
  stage_orbitals<T, 3>(c);
  {
    // orbital-matrix inverse: native FP64 in the FP64 build, double-FP32 (48-bit significand) otherwise; the
    // refinement pass eliminates the FP64 orbital matrices of its walkers in FP64
    Prof pr("gauss_jordan", c.s);
    if constexpr (sizeof(T) == 8) {
      launch_gjg<double, T, T, true>(c, c.template buf<T>(c.P.Apl), (const T*)nullptr, c.template buf<T>(c.P.Ainv));
    } else if (rf.c64) {
      const Ctx<double>& c64 = *rf.c64;
      launch_gjg<double, double, T, true>(c64, c64.template buf<double>(c64.P.Apl), (const double*)nullptr,
                                          c.template buf<T>(c.P.Ainv));
      const size_t nb = sizeof(double) * (size_t)c.Wc * NDET;
      cudaMemcpyAsync(c.template buf<double>(c.P.ld), c64.template buf<double>(c64.P.ld), nb,
                      cudaMemcpyDeviceToDevice, c.s);
      cudaMemcpyAsync(c.template buf<double>(c.P.sd), c64.template buf<double>(c64.P.sd), nb,
                      cudaMemcpyDeviceToDevice, c.s);
    } else {
      // the condition numbers of the orbital matrices feed the ill-conditioned test of the assembly
      launch_gjg<df64, T, T, true>(c, c.template buf<T>(c.P.Apl), c.template buf<T>(c.P.Apl_lo),
                                   c.template buf<T>(c.P.Ainv),
                                   rf.idx ? c.template buf<double>(c.P.cond) : nullptr);
    }
  }
  cudaMemsetAsync(c.template buf<double>(c.P.dlap), 0, sizeof(double) * c.Wc * NDET, c.s);
  {
    // FP32: dependencies with at most DL_CSPLIT positions in 128-thread CTAs (4 per SM), the rest in 256-thread
    // CTAs; each launch leaves the other's dependencies alone.  FP64: one 256-thread launch.
    Prof pr("detlap", c.s);
    const dim3 grid(c.p->n_el, NDET, c.Wc);
    auto go = [&](auto kern, int threads, int chi) {
      const size_t smem = sizeof(T) * (size_t)dl_smem_elems(chi);
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      g_nlaunch++;
      kern<<<grid, threads, smem, c.s>>>(c.nb, c.L, c.template buf<T>(c.P.Jorb), c.template buf<T>(c.P.Ainv),
                                         c.template buf<T>(c.P.lapA), c.template buf<double>(c.P.dgrad),
                                         c.template buf<double>(c.P.dlap), c.status);
    };
    if constexpr (sizeof(T) == 4) {
      go(k_detlap<T, 128, 0, DL_CSPLIT>, 128, DL_CSPLIT);
      go(k_detlap<T, 256, DL_CSPLIT, DL_CMAX>, 256, DL_CMAX);
    } else {
      go(k_detlap<T, 256, 0, DL_CMAX>, 256, DL_CMAX);
    }
  }
  stage_jastrow<T, 3>(c);
  AssembleOut o;
  std::memset(&o, 0, sizeof(o));
  g_nlaunch++;
  k_nn_energy<<<1, 256, 0, c.s>>>(c.R, c.Z, c.p->n_nuc, c.template buf<double>(c.P.enn));
  o.enn = c.template buf<double>(c.P.enn);
  o.logpsi = logpsi;
  o.sign = sign;
  o.eloc = eloc;
  if (dbg) o.dbg = *dbg;
  if (rf.c64) {  // refinement pass: walker w of the chunk is batch walker idx[w]
    o.wmap = rf.idx;
    o.wcnt = rf.cnt;
  } else if (rf.idx) {
    o.ref_idx = rf.idx;
    o.ref_cnt = rf.cnt;
    o.ref_cap = rf.cap;
    o.ref_ratio = c.p->refine_ratio > 0.f ? (double)c.p->refine_ratio : (double)FIRE_REFINE_RATIO;
    o.ref_kappa = c.p->refine_kappa > 0.f ? (double)c.p->refine_kappa : (double)FIRE_REFINE_KAPPA;
    o.ref_ks = c.p->refine_ks > 0.f ? (double)c.p->refine_ks : (double)FIRE_REFINE_KS;
    o.ref_kscond = c.p->refine_kscond > 0.f ? (double)c.p->refine_kscond : (double)FIRE_REFINE_KSCOND;
    o.cond = c.template buf<double>(c.P.cond);
  }
  Prof pr("assemble", c.s);
  g_nlaunch++;
  k_assemble<T, true><<<c.Wc, 256, 3 * c.p->n_el * sizeof(double), c.s>>>(
      c.p->n_el, c.p->n_up, c.p->n_nuc, c.w0, c.r, c.R, c.Z, c.W, c.template buf<double>(c.P.ld),
      c.template buf<double>(c.P.sd), c.template buf<double>(c.P.dgrad), c.template buf<double>(c.P.dlap),
      c.template buf<T>(c.P.JAx), c.template buf<T>(c.P.JAj), c.template buf<T>(c.P.JAl), c.template buf<T>(c.P.JMx),
      c.template buf<T>(c.P.JMj), c.template buf<T>(c.P.JMl), o, c.status);
  return cudaPeekAtLastError();
}

template <typename T>
Ctx<T> make_ctx(const fire_problem* p, cudaStream_t s, const float* R, const float* Z, const void* prepared,
                int32_t* status, void* ws, int Wmax, bool fl) {
  Ctx<T> c;
  c.p = p;
  c.s = s;
  c.Wmax = Wmax;
  c.B = p->n_walkers;
  c.R = R;
  c.Z = Z;
  c.W = make_weights<T>(p, prepared);
  c.status = status;
  c.ws = reinterpret_cast<unsigned char*>(ws);
  c.P = make_plan(p, Wmax, fl);
  c.mixed = p->precision == FIRE_PREC_MIXED;
  if (c.mixed) {
    int64_t off[PR_COUNT + 1];
    prep_offsets(p, off);
    size_t to[TC_COUNT + 1];
    tc_offsets(p, (size_t)off[PR_COUNT] * 4, to);
    const unsigned char* base = reinterpret_cast<const unsigned char*>(prepared);
    for (int k = 0; k < TC_COUNT; ++k) {
      size_t K, N;
      int cnt;
      tc_shape(k, p, &K, &N, &cnt);
      const __nv_bfloat16* hi = reinterpret_cast<const __nv_bfloat16*>(base + to[k]);
      if (tc_grid(k, K) && tc_tiled(k, K))
        c.tcw[k] = TcWeights{nullptr, nullptr, hi, nullptr,
                             reinterpret_cast<const float*>(base + to[k] + tc_cs_offset(K, N, cnt)), nullptr};
      else if (tc_tiled(k, K)) c.tcw[k] = TcWeights{nullptr, nullptr, hi, nullptr, nullptr, nullptr};
      else c.tcw[k] = TcWeights{hi, hi + (size_t)cnt * N * K, nullptr, nullptr, nullptr, nullptr};
    }
    c.tcw[TC_ORB_UP].tiles2 = c.tcw[TC_ORB_DN].tiles;
    c.tcw[TC_ORB_UP].cs2 = c.tcw[TC_ORB_DN].cs;
  }
  return c;
}

// Positions of the walkers of one refinement pass: entries k0 .. k0 + KC - 1 of the list.  r_ref [k] (walkers'
// dtype) and r64 [k] (FP64) = walker idx[k0 + k] of the batch while k0 + k < min(cnt, KF) (a copy of the first
// entry, or of walker 0, beyond); sub_cnt = the pass's number of listed walkers.  The first pass reports the count
// in status[5] and an overflow of the capacity KF.
template <typename T>
__global__ void k_refine_gather(const T* __restrict__ r, int n, const int32_t* __restrict__ idx,
                                const int32_t* __restrict__ cnt, int KF, int k0, int KC, T* __restrict__ r_ref,
                                double* __restrict__ r64, int32_t* __restrict__ sub_cnt, int32_t* status) {
  const int k = blockIdx.x, c = min(*cnt, KF);
  const int src = k0 + k < c ? idx[k0 + k] : (c > 0 ? idx[0] : 0);
  for (int q = threadIdx.x; q < 3 * n; q += blockDim.x) {
    const T v = r[(size_t)src * 3 * n + q];
    r_ref[(size_t)k * 3 * n + q] = v;
    r64[(size_t)k * 3 * n + q] = (double)v;
  }
  if (k == 0 && threadIdx.x == 0) {
    *sub_cnt = max(0, min(KC, c - k0));
    if (k0 == 0) {
      max_word(status, 5, *cnt);
      if (*cnt > KF) set_flag(status, FIRE_FLAG_REFINE_OVERFLOW);
    }
  }
}

// The refinement pass over the ill-conditioned walkers of the batch (rf.idx, rf.cnt): the FP64 value path
// (embedding, update, envelopes, orbitals) of their positions, then the chunk evaluation of the same positions with
// those orbital matrices eliminated in FP64 and the derivative planes on the FP32 CUDA cores; the results go to the
// walkers' rows.  The list is evaluated in passes of KC <= Wc walkers (the batch's chunk size, so that they fit
// the workspace); a pass whose walkers are all beyond the count exits in its assembly.
template <typename T>
cudaError_t refine_pass(const fire_problem* p, int Wc, cudaStream_t s, const float* R, const float* Z,
                        const void* prepared, const T* r, void* logpsi, void* sign, void* eloc,
                        const fire_eloc_debug* dbg, unsigned char* ws, int32_t* status, Refine rf) {
  const int KF = rf.cap, KC = std::min(KF, Wc), n = p->n_el;
  const RefineLayout L = refine_layout(p, KC);
  T* r_ref = reinterpret_cast<T*>(ws + L.r_ref);
  double* r64 = reinterpret_cast<double*>(ws + L.r64);
  int32_t* sub_cnt = rf.cnt + 1;  // one count per pass
  const fire_problem p64 = refine_problem64(p, KC);
  fire_problem pr_ = *p;
  pr_.n_walkers = KC;
  pr_.chunk_walkers = KC;
  pr_.precision = FIRE_PREC_FP32;  // derivative planes on the CUDA cores in FP32 (the float slots are shared)
  Prof pr("refine", s);
  for (int k0 = 0, j = 0; k0 < KF; k0 += KC, ++j) {
    g_nlaunch++;
    k_refine_gather<T><<<KC, 128, 0, s>>>(r, n, rf.idx, rf.cnt, KF, k0, KC, r_ref, r64, sub_cnt + j, status);
    Ctx<double> c64 = make_ctx<double>(&p64, s, R, Z,
                                       reinterpret_cast<const unsigned char*>(prepared) + prep64_offset(p), status,
                                       ws + L.c64, KC, false);
    c64.w0 = 0;
    c64.Wc = KC;
    c64.env_df = true;
    c64.r = r64;
    setup_ctx(c64, false);
    stage_neighbors(c64, false);
    stage_embedding<double, 0>(c64);
    stage_update<double, 0>(c64);
    stage_orbitals<double, 0>(c64);
    Ctx<T> c = make_ctx<T>(&pr_, s, R, Z, prepared, status, ws, KC, true);
    c.w0 = 0;
    c.Wc = KC;
    c.r = r_ref;
    Refine sub = rf;
    sub.idx = rf.idx + k0;
    sub.cnt = sub_cnt + j;
    sub.c64 = &c64;
    const cudaError_t e = chunk_eloc<T>(c, logpsi, sign, eloc, dbg, sub);
    if (e != cudaSuccess) return e;
  }
  return cudaPeekAtLastError();
}

template <typename T>
fire_status run_eloc(const fire_problem* p, cudaStream_t s, const float* R, const float* Z, const void* prepared,
                     const void* r, void* logpsi, void* sign, void* eloc, double* stats, const fire_eloc_debug* dbg,
                     void* ws, size_t wsb, int32_t* status) {
  const int Wc = choose_chunk(p, wsb, true);
  if (Wc <= 0) return FIRE_ERR_WORKSPACE;
  Ctx<T> c = make_ctx<T>(p, s, R, Z, prepared, status, ws, Wc, true);
  const T* rr = reinterpret_cast<const T*>(r);
  Refine rf;
  if constexpr (sizeof(T) == 4) {
    rf.cap = refine_walkers(p);
    if (rf.cap > 0) {
      size_t list_off = 0;
      eloc_ws_bytes(p, Wc, &list_off);
      rf.idx = reinterpret_cast<int32_t*>(reinterpret_cast<unsigned char*>(ws) + list_off);
      rf.cnt = rf.idx + rf.cap;
      cudaMemsetAsync(rf.cnt, 0, sizeof(int32_t), s);
    }
  }
  for (int w0 = 0; w0 < p->n_walkers; w0 += Wc) {
    c.w0 = w0;
    c.Wc = std::min(Wc, p->n_walkers - w0);
    c.r = rr + (size_t)w0 * p->n_el * 3;
    if (chunk_eloc<T>(c, logpsi, sign, eloc, dbg, rf) != cudaSuccess) return launch_status("local_energy chunk");
  }
  if constexpr (sizeof(T) == 4) {
    if (rf.cap > 0 && refine_pass<T>(p, Wc, s, R, Z, prepared, rr, logpsi, sign, eloc, dbg,
                                     reinterpret_cast<unsigned char*>(ws), status, rf) != cudaSuccess)
      return launch_status("local_energy refinement");
  }
  g_nlaunch++;
  if (stats) k_stats<T><<<1, 1024, 0, s>>>(reinterpret_cast<const T*>(eloc), p->n_walkers, stats);
  return launch_status(__func__);
}

template <typename T>
fire_status run_logpsi(const fire_problem* p, cudaStream_t s, const float* R, const float* Z, const void* prepared,
                       const void* r, void* sign, void* logpsi, void* ws, size_t wsb, int32_t* status) {
  const int Wc = choose_chunk(p, wsb, false);
  if (Wc <= 0) return FIRE_ERR_WORKSPACE;
  Ctx<T> c = make_ctx<T>(p, s, R, Z, prepared, status, ws, Wc, false);
  const T* rr = reinterpret_cast<const T*>(r);
  for (int w0 = 0; w0 < p->n_walkers; w0 += Wc) {
    c.w0 = w0;
    c.Wc = std::min(Wc, p->n_walkers - w0);
    c.r = rr + (size_t)w0 * p->n_el * 3;
    if (chunk_logpsi<T>(c, logpsi, sign, w0) != cudaSuccess) return launch_status("logpsi chunk");
  }
  return FIRE_OK;
}

template <typename T>
fire_status run_embedding(const fire_problem* p, cudaStream_t s, const float* R, const void* prepared,
                          const void* r, void* hc, void* hu, void* ws, size_t wsb, int32_t* status) {
  const int Wc = choose_chunk(p, wsb, false);
  if (Wc <= 0) return FIRE_ERR_WORKSPACE;
  Ctx<T> c = make_ctx<T>(p, s, R, nullptr, prepared, status, ws, Wc, false);
  const T* rr = reinterpret_cast<const T*>(r);
  for (int w0 = 0; w0 < p->n_walkers; w0 += Wc) {
    c.w0 = w0;
    c.Wc = std::min(Wc, p->n_walkers - w0);
    c.r = rr + (size_t)w0 * p->n_el * 3;
    setup_ctx(c, false);
    stage_neighbors(c, false);
    stage_embedding<T, 0>(c);
    stage_update<T, 0>(c);
    const size_t cnt = (size_t)c.Wc * p->n_el * F;
    if (hc)
      cudaMemcpyAsync(reinterpret_cast<T*>(hc) + (size_t)w0 * p->n_el * F, c.template buf<T>(c.P.HX),
                      cnt * sizeof(T), cudaMemcpyDeviceToDevice, s);
    if (hu)
      cudaMemcpyAsync(reinterpret_cast<T*>(hu) + (size_t)w0 * p->n_el * F, c.template buf<T>(c.P.B2X),
                      cnt * sizeof(T), cudaMemcpyDeviceToDevice, s);
    if (launch_status("embedding chunk") != FIRE_OK) return FIRE_ERR_CUDA;
  }
  return FIRE_OK;
}

// Metropolis block.  Proposals: all electrons moved (MC_ALL), one electron per step, (offset + step) mod n
// (MC_SINGLE), or one random electron jumping next to a nucleus with the proposal's log ratio in the test
// (MC_JUMP, width = the jump's sigma).  Every proposal is evaluated by the full value path.
// MC_CLUSTER: the cluster update (ck electrons at most within cradius of the center, sequential or random
// centers) with its validity in the test.
enum McKind { MC_ALL = 0, MC_SINGLE = 1, MC_JUMP = 2, MC_CLUSTER = 3 };
template <typename T>
fire_status run_mcmc(const fire_problem* p, cudaStream_t s, const float* R, const float* Z, const void* prepared,
                     void* r, void* logpsi, int steps, float width, uint64_t seed, uint64_t counter,
                     const void* noise, const void* logu, int32_t* n_accept, int32_t* static_max, void* ws,
                     size_t wsb, int32_t* status, int kind = MC_ALL, int offset = 0, int ck = 0, float cradius = 0.f,
                     int crandom = 0) {
  const int Wc = choose_chunk(p, wsb, false);
  if (Wc <= 0) return FIRE_ERR_WORKSPACE;
  Ctx<T> c = make_ctx<T>(p, s, R, Z, prepared, status, ws, Wc, false);
  c.comp = false;  // proposals are only compared by their log|psi|: plain value contractions
  T* rr = reinterpret_cast<T*>(r);
  const int n = p->n_el;
  for (int w0 = 0; w0 < p->n_walkers; w0 += Wc) {
    c.w0 = w0;
    c.Wc = std::min(Wc, p->n_walkers - w0);
    T* rn = c.template buf<T>(c.P.rn);
    T* lpn = c.template buf<T>(c.P.lpn);
    T* plr = (kind == MC_JUMP || kind == MC_CLUSTER) ? c.template buf<T>(c.P.plr) : nullptr;
    for (int st = 0; st < steps; ++st) {
      g_nlaunch++;
      if (kind == MC_SINGLE)
        k_propose_single<T><<<c.Wc, 128, 0, s>>>(rr + (size_t)w0 * n * 3, rn, n, w0, p->n_walkers, st, offset,
                                                 (T)width, seed, counter, reinterpret_cast<const T*>(noise), nullptr);
      else if (kind == MC_CLUSTER)
        k_propose_cluster<T><<<c.Wc, 32, 0, s>>>(rr + (size_t)w0 * n * 3, rn, plr, n, w0, p->n_walkers, st, offset, ck,
                                                 (T)cradius, (T)width, crandom, seed, counter,
                                                 reinterpret_cast<const T*>(noise), nullptr);
      else if (kind == MC_JUMP)
        k_propose_jump<T><<<c.Wc, 128, 0, s>>>(rr + (size_t)w0 * n * 3, rn, plr, n, w0, p->n_walkers, st, R, Z,
                                               p->n_nuc, (T)width, seed, counter, reinterpret_cast<const T*>(noise),
                                               nullptr);
      else
        k_propose<T><<<nblk((long)c.Wc * n), 256, 0, s>>>(rr + (size_t)w0 * n * 3, rn, n, c.Wc, w0, p->n_walkers,
                                                          st, (T)width, seed, counter,
                                                          reinterpret_cast<const T*>(noise));
      c.r = rn;
      if (chunk_logpsi<T>(c, lpn, nullptr, 0) != cudaSuccess) return launch_status("mcmc chunk");
      g_nlaunch++;
      k_accept<T><<<c.Wc, 128, 0, s>>>(rr, rn, reinterpret_cast<T*>(logpsi), lpn, n, w0, p->n_walkers, st, seed,
                                      counter, reinterpret_cast<const T*>(logu), n_accept, c.nb.counts, static_max,
                                      plr, nullptr);
    }
  }
  return launch_status(__func__);
}

// ------------------------------------------------------------------------------ low-rank single-electron block
// Buffers of the low-rank block beyond the value path's plan of the same chunk (byte offsets into the workspace).
// The state of a chunk is the value path's own buffers (E5o, B2X, rawx, env, Apl, aX, Xo2, ld, sd and the e-n
// lists / statics of Nbr) plus `vals` (the attention value rows) and `B` (the transposed inverse of every orbital
// matrix); the rest is per-step scratch of the proposal.
struct LrPlan {
  size_t vals, B;                                        // state
  size_t S, S_cnt, en_cnt_p, en_idx_p, counts_p, acc, moved;  // int
  size_t re_p, E5p, HS, B1S, hS, rawU, rawD, coefE, coefD, env_p, env_pD, aS, vS, oS, V, Zb, Qb;  // T
  size_t Minv, ld_p, sd_p;                               // double
  size_t lp0, sgn0, sgn_p, ecp_acc, ecp_pt;              // pseudopotential energy: T x 3, double x 2
  size_t total;
};

LrPlan make_lr_plan(const fire_problem* p, int Wc, int KS) {
  LrPlan Q;
  std::memset(&Q, 0, sizeof(Q));
  const size_t es = elem_size(p);
  const size_t n = p->n_el, W = Wc, G = W * n, DN = NDET * n, K8 = (size_t)p->n_nuc * NENV_ORB, R = W * KS;
  size_t o = make_plan(p, Wc, false).total;
  auto take = [&](size_t& field, size_t count, size_t bytes_per) {
    o = (o + 255) / 256 * 256;
    field = o;
    o += count * bytes_per;
  };
  take(Q.vals, G * F, es);
  take(Q.B, W * NDET * n * (size_t)ainv_ld((int)n), es);
  const size_t WM = W * CLUSTER_KMAX;  // moved slots: one per walker, up to a cluster's size
  take(Q.S, R, 4);
  take(Q.S_cnt, W, 4);
  take(Q.en_cnt_p, WM, 4);
  take(Q.en_idx_p, WM * p->cap_nuc, 4);
  take(Q.counts_p, W * 4, 4);
  take(Q.acc, W, 4);
  take(Q.moved, WM, 4);
  take(Q.re_p, WM * 3, es);
  take(Q.E5p, WM * 5 * F, es);
  take(Q.HS, R * F, es);
  take(Q.B1S, R * F, es);
  take(Q.hS, R * F, es);
  take(Q.rawU, R * DN, es);
  take(Q.rawD, R * DN, es);
  take(Q.coefE, NDET * WM * K8, es);
  take(Q.coefD, NDET * WM * K8, es);
  take(Q.env_p, WM * DN, es);
  take(Q.env_pD, WM * DN, es);
  take(Q.aS, R * HEADS, es);
  take(Q.vS, R * F, es);
  take(Q.oS, R * 2, es);
  take(Q.V, W * NDET * KS * n, es);
  take(Q.Zb, W * NDET * n * KS, es);
  take(Q.Qb, W * NDET * KS * n, es);
  take(Q.Minv, W * NDET * KS * KS, 8);
  take(Q.ld_p, W * NDET, 8);
  take(Q.sd_p, W * NDET, 8);
  take(Q.lp0, W, es);
  take(Q.sgn0, W, es);
  take(Q.sgn_p, W, es);
  take(Q.ecp_acc, W, 8);
  take(Q.ecp_pt, W * 4, 8);
  Q.total = (o + 255) / 256 * 256;
  return Q;
}

int choose_chunk_lr(const fire_problem* p, size_t ws_bytes, int KS) {
  const int B = p->n_walkers;
  if (p->chunk_walkers > 0) {
    const int c = std::min(B, p->chunk_walkers);
    return make_lr_plan(p, c, KS).total <= ws_bytes ? c : 0;
  }
  int lo = 0, hi = B;
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (make_lr_plan(p, mid, KS).total <= ws_bytes) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// the attention readout MLP 512 -> 256 -> 256 -> 2 on the value rows RX [W][512] -> JAx [W][2] (the value
// path's part of stage_jastrow)
template <typename T>
void readout_value(Ctx<T>& c) {
  const int Wc = c.Wc;
  auto layer = [&](size_t in, size_t out, const T* Wt, const T* b, int K) {
    GemmP<T> q = gp0<T>();
    q.A = c.template buf<T>(in); q.lda = K; q.B = Wt; q.ldb = F; q.bias = b; q.C = c.template buf<T>(out);
    q.ldc = F; q.M = Wc; q.N = F; q.K = K; q.ld_aux = F;
    gemm<T, EPI_SILU_X>(c, q);
  };
  layer(c.P.RX, c.P.R1X, c.W.w[FIRE_P_ATT_OUT1_W], c.W.w[FIRE_P_ATT_OUT1_B], 2 * F);
  layer(c.P.R1X, c.P.R2X, c.W.w[FIRE_P_ATT_OUT2_W], c.W.w[FIRE_P_ATT_OUT2_B], F);
  GemmP<T> g = gp0<T>();
  g.A = c.template buf<T>(c.P.R2X); g.lda = F; g.B = c.W.w[FIRE_P_ATT_OUT3_W]; g.ldb = 2;
  g.bias = c.W.w[FIRE_P_ATT_OUT3_B]; g.bias_period = 1; g.C = c.template buf<T>(c.P.JAx); g.ldc = 2; g.M = Wc;
  g.N = 2; g.K = F;
  gemm<T, EPI_PLAIN>(c, g);
}

// State of one chunk: the value path with the inverse kept (Gauss-Jordan instead of the LU), the attention value
// rows, and log|psi| (and its sign, if sign is not null) of the chunk's walkers into logpsi[w0_out + w]
// (log_psi_with_state, wave_function.py:226-247).
template <typename T>
cudaError_t chunk_state(Ctx<T>& c, const LrPlan& Q, void* logpsi, void* sign, int w0_out) {
  setup_ctx(c, false);
  stage_neighbors(c, false);
  stage_embedding<T, 0>(c);
  stage_update<T, 0>(c);
  stage_orbitals<T, 0>(c);
  {
    Prof pr("gauss_jordan", c.s);
    if constexpr (sizeof(T) == 8)
      launch_gjg<double, T, T, true>(c, c.template buf<T>(c.P.Apl), (const T*)nullptr, c.template buf<T>(Q.B));
    else
      launch_gjg<df64, T, T, true>(c, c.template buf<T>(c.P.Apl),
                                   c.comp ? c.template buf<T>(c.P.Apl_lo) : nullptr, c.template buf<T>(Q.B));
  }
  stage_jastrow<T, 0>(c);
  const Planes B2{c.P.B2X, 0, 0}, VL{Q.vals, 0, 0};
  linear_layer<T>(c, false, B2, VL, c.W.w[PR_V_W_S1], c.W.w[FIRE_P_ATT_V_B], F, F, c.Wc * c.p->n_el, 0, nullptr);
  AssembleOut o;
  std::memset(&o, 0, sizeof(o));
  o.logpsi = logpsi;
  o.sign = sign;
  g_nlaunch++;
  k_assemble<T, false><<<c.Wc, 256, 3 * c.p->n_el * sizeof(double), c.s>>>(
      c.p->n_el, c.p->n_up, c.p->n_nuc, w0_out, c.r, c.R, c.Z, c.W, c.template buf<double>(c.P.ld),
      c.template buf<double>(c.P.sd), nullptr, nullptr, c.template buf<T>(c.P.JAx), nullptr, nullptr,
      c.template buf<T>(c.P.JMx), nullptr, nullptr, o, c.status);
  return cudaPeekAtLastError();
}

// log|psi'| (into c.P.lpn) and its sign (into sgn_out, may be null) of the chunk's proposal c.P.rn, in which walker w
// moved the electrons moved[w][0..KM) (the plan's moved buffer, padded with FIRE_NO_NEIGHBOUR), from the state; the
// proposal's rows stay in the plan's scratch for the commit.
template <typename T>
cudaError_t lr_evaluate(Ctx<T>& c, const LrPlan& Q, int KS, int KM, T* rr, int32_t* static_max, T* sgn_out,
                        int mover_spin = -1) {
  const fire_problem* p = c.p;
  const int n = p->n_el, nu = p->n_up, N = p->n_nuc, Wc = c.Wc, DN = NDET * n, rows = Wc * KS;
  const int K8 = N * NENV_ORB;
  cudaStream_t s = c.s;
  T* rn = c.template buf<T>(c.P.rn);
  T* r_chunk = rr + (size_t)c.w0 * n * 3;
  int* S = c.template buf<int>(Q.S);
  int* S_cnt = c.template buf<int>(Q.S_cnt);
  const int* moved = c.template buf<int>(Q.moved);
  Prof pr("low_rank_step", s);
  g_nlaunch++;
  k_lr_select<T><<<Wc, 256, 0, s>>>(r_chunk, rn, n, nu, moved, KM, c.R, N, (T)p->cutoff, (T)p->cutoff_1el, c.nb, KS, S,
                                    S_cnt, c.template buf<T>(Q.re_p), c.template buf<int>(Q.en_cnt_p),
                                    c.template buf<int>(Q.en_idx_p), c.template buf<int>(Q.counts_p), static_max,
                                    c.status);
  // ElecInit of the moved electrons (KM rows per walker), then their GLU / Dense / Dense
  {
    const int ME = Wc * KM;
    Nbr nbe = c.nb;
    nbe.en_cnt = c.template buf<int>(Q.en_cnt_p);
    nbe.en_idx = c.template buf<int>(Q.en_idx_p);
    T* E5a = c.template buf<T>(c.P.E5a);
    T* Z1 = c.template buf<T>(c.P.Z1);
    g_nlaunch++;
    k_elec_init<T, 0><<<ME, 256, 0, s>>>(c.template buf<T>(Q.re_p), c.R, nbe, c.W, (T)(1.0 / p->cutoff_1el), E5a);
    GemmP<T> g = gp0<T>();
    g.A = E5a; g.lda = F; g.B = c.W.w[FIRE_P_EI_GLU_W]; g.ldb = 2 * F; g.C = Z1; g.ldc = 2 * F;
    g.M = ME; g.N = 2 * F; g.K = F;
    gemm<T, EPI_PLAIN>(c, g);
    g_nlaunch++;
    k_glu<T, 0><<<nblk((long)ME * F), 256, 0, s>>>(Z1, E5a, ME);
    g = gp0<T>();
    g.A = E5a; g.lda = F; g.B = c.W.w[FIRE_P_EI_DENSE_W]; g.ldb = F; g.C = Z1; g.ldc = F;
    g.bias = c.W.w[FIRE_P_EI_DENSE_B]; g.bias_period = 1; g.M = ME; g.N = F; g.K = F;
    gemm<T, EPI_PLAIN>(c, g);
    g_nlaunch++;
    k_silu5<T, 0><<<nblk((long)ME * F), 256, 0, s>>>(Z1, ME);
    g = gp0<T>();
    g.A = Z1; g.lda = F; g.B = c.W.w[FIRE_P_EI_OUT_W]; g.ldb = 5 * F; g.C = c.template buf<T>(Q.E5p);
    g.ldc = 5 * F; g.bias = c.W.w[FIRE_P_EI_OUT_B]; g.bias_period = 1; g.M = ME; g.N = 5 * F; g.K = F;
    gemm<T, EPI_PLAIN>(c, g);
  }
  // messages and update MLP of the changed centers
  g_nlaunch++;
  k_lr_contract<T><<<dim3(KS, Wc), 256, 0, s>>>(rn, n, nu, (T)p->cutoff, moved, KM, S, S_cnt, KS, c.W,
                                                c.template buf<T>(c.P.E5o), c.template buf<T>(Q.E5p),
                                                c.template buf<T>(Q.HS));
  const Planes HS{Q.HS, 0, 0}, B1S{Q.B1S, 0, 0}, hS{Q.hS, 0, 0};
  silu_layer<T>(c, false, HS, B1S, c.W.w[PR_UPD1_W_S0], c.W.w[FIRE_P_UPD1_B], F, F, rows, 0, nullptr, nullptr, 1, 0,
                0);
  silu_layer<T>(c, false, B1S, hS, c.W.w[FIRE_P_UPD2_W], c.W.w[FIRE_P_UPD2_B], F, F, rows, 0, nullptr, nullptr, 1, 0,
                0);
  // raw orbital rows of the changed centers (both spins' contractions, then each row's own)
  for (int sp = 0; sp < 2; ++sp) {
    GemmP<T> g = gp0<T>();
    g.A = c.template buf<T>(Q.hS); g.lda = F; g.B = c.W.w[sp == 0 ? PR_ORB_UP_W_S1 : PR_ORB_DN_W_S1]; g.ldb = DN;
    g.bias = c.W.w[sp == 0 ? FIRE_P_ORB_UP_B : FIRE_P_ORB_DN_B]; g.bias_period = 1;
    g.C = c.template buf<T>(sp == 0 ? Q.rawU : Q.rawD); g.ldc = DN; g.M = rows; g.N = DN; g.K = F;
    gemm<T, EPI_PLAIN>(c, g);
  }
  g_nlaunch++;
  k_lr_orb<T><<<dim3(KS, Wc), 256, 0, s>>>(S, S_cnt, KS, nu, DN, c.template buf<T>(Q.rawU),
                                           c.template buf<T>(Q.rawD));
  // envelope row of the moved electron at its new position: coefficients of its own spin (zero in the other spin's
  // set), both spins' contractions, their sum; when every walker moves an electron of one spin (mover_spin >= 0, the
  // sequential single-electron sweep) that spin's contractions alone, straight into env_p
  {
    T* coefU = c.template buf<T>(Q.coefE);
    T* coefD = c.template buf<T>(Q.coefD);
    g_nlaunch++;
    const int ME = Wc * KM;
    k_lr_env_coef<T><<<nblk((long)ME * K8), 256, 0, s>>>(rn, c.R, c.W.w[PR_ENV_UP_SP], c.W.w[PR_ENV_DN_SP], moved,
                                                         KM, n, nu, N, Wc, coefU, coefD);
    if (mover_spin >= 0) {
      for (int d = 0; d < NDET; ++d) {
        GemmP<T> g = gp0<T>();
        g.A = (mover_spin == 0 ? coefU : coefD) + (size_t)d * ME * K8; g.lda = K8;
        g.B = c.W.w[mover_spin == 0 ? PR_ENV_UP_PI : PR_ENV_DN_PI] + (size_t)d * K8 * n; g.ldb = n;
        g.C = c.template buf<T>(Q.env_p) + (size_t)d * n; g.ldc = DN; g.M = ME; g.N = n;
        g.K = K8; g.n_el = 1; g.env_ns = 1; g.env_soff = 0; g.env_nv = 1;
        gemm<T, EPI_ENV>(c, g);
      }
    } else {
    for (int sp = 0; sp < 2; ++sp)
      for (int d = 0; d < NDET; ++d) {
        GemmP<T> g = gp0<T>();
        g.A = (sp == 0 ? coefU : coefD) + (size_t)d * ME * K8; g.lda = K8;
        g.B = c.W.w[sp == 0 ? PR_ENV_UP_PI : PR_ENV_DN_PI] + (size_t)d * K8 * n; g.ldb = n;
        g.C = c.template buf<T>(sp == 0 ? Q.env_p : Q.env_pD) + (size_t)d * n; g.ldc = DN; g.M = ME; g.N = n;
        g.K = K8; g.n_el = 1; g.env_ns = 1; g.env_soff = 0; g.env_nv = 1;
        gemm<T, EPI_ENV>(c, g);
      }
    g_nlaunch++;
    k_lr_env_add<T><<<nblk((long)ME * DN), 256, 0, s>>>((long)ME * DN, c.template buf<T>(Q.env_p),
                                                        c.template buf<T>(Q.env_pD));
    }
  }
  // determinant lemma
  {
    const size_t smem = sizeof(double) * (size_t)KS * KS + 2 * sizeof(T) * (size_t)KS * 33;
    cudaFuncSetAttribute(k_lr_det<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    g_nlaunch++;
    k_lr_det<T><<<dim3(NDET, Wc), 256, smem, s>>>(
        S, S_cnt, KS, n, moved, KM, c.template buf<T>(Q.rawU), c.template buf<T>(c.P.env), c.template buf<T>(Q.env_p),
        c.template buf<T>(c.P.Apl), c.template buf<T>(Q.B), c.template buf<double>(c.P.ld),
        c.template buf<double>(c.P.sd), c.template buf<T>(Q.V), c.template buf<double>(Q.Minv),
        c.template buf<double>(Q.ld_p), c.template buf<double>(Q.sd_p));
  }
  // Jastrow rows of the changed centers, the sums with the state's other rows, the readout
  {
    g_nlaunch++;
    k_narrow<T, HEADS, 1, false><<<rows, 256, 0, s>>>(c.template buf<T>(Q.hS), nullptr, nullptr, c.nb, c.L,
                                                      c.W.w[PR_QK_W_S1], c.W.w[PR_QK_B], nullptr, nullptr,
                                                      c.template buf<T>(Q.aS), nullptr, nullptr, c.status, nullptr,
                                                      nullptr);
    const Planes vS{Q.vS, 0, 0};
    linear_layer<T>(c, false, hS, vS, c.W.w[PR_V_W_S1], c.W.w[FIRE_P_ATT_V_B], F, F, rows, 0, nullptr);
    silu_layer<T>(c, false, hS, HS, c.W.w[PR_JMLP1_W_S1], c.W.w[FIRE_P_JMLP1_B], F, F, rows, 0, nullptr, nullptr, 1,
                  0, 0);
    silu_layer<T>(c, false, HS, B1S, c.W.w[FIRE_P_JMLP2_W], c.W.w[FIRE_P_JMLP2_B], F, F, rows, 0, nullptr, nullptr,
                  1, 0, 0);
    g_nlaunch++;
    k_narrow<T, 2, 0, false><<<rows, 256, 0, s>>>(c.template buf<T>(Q.B1S), nullptr, nullptr, c.nb, c.L,
                                                  c.W.w[FIRE_P_JMLP3_W], c.W.w[FIRE_P_JMLP3_B],
                                                  c.W.w[FIRE_P_MLP_SCALE], c.W.w[PR_SCALARS] + 1,
                                                  c.template buf<T>(Q.oS), nullptr, nullptr, c.status, nullptr,
                                                  nullptr);
    g_nlaunch++;
    k_lr_jsums<T><<<Wc, 256, 0, s>>>(n, nu, S, S_cnt, KS, c.template buf<T>(c.P.aX), c.template buf<T>(Q.vals),
                                     c.template buf<T>(c.P.Xo2), c.template buf<T>(Q.aS), c.template buf<T>(Q.vS),
                                     c.template buf<T>(Q.oS), c.template buf<T>(c.P.Ax), c.template buf<T>(c.P.JMx));
    g_nlaunch++;
    k_readout_in<T, false><<<Wc, 512, 0, s>>>(n, c.template buf<T>(c.P.Ax), nullptr, nullptr,
                                              c.template buf<T>(c.P.RX), nullptr, nullptr);
    readout_value<T>(c);
  }
  // log|psi'| and the Metropolis test
  AssembleOut o;
  std::memset(&o, 0, sizeof(o));
  o.logpsi = c.template buf<T>(c.P.lpn);
  o.sign = sgn_out;
  g_nlaunch++;
  k_assemble<T, false><<<Wc, 256, 3 * n * sizeof(double), s>>>(
      n, nu, N, 0, rn, c.R, c.Z, c.W, c.template buf<double>(Q.ld_p), c.template buf<double>(Q.sd_p), nullptr,
      nullptr, c.template buf<T>(c.P.JAx), nullptr, nullptr, c.template buf<T>(c.P.JMx), nullptr, nullptr, o,
      c.status);
  return cudaPeekAtLastError();
}

// One low-rank Metropolis step of the chunk: the proposal c.P.rn (walker w moved electron moved[w]) evaluated from the
// state, the Metropolis test with the proposals' log ratios plr (may be null), and on acceptance the state's rows and
// the Woodbury update of the inverse.
template <typename T>
cudaError_t lr_step(Ctx<T>& c, const LrPlan& Q, int KS, int KM, T* rr, void* logpsi, int st, uint64_t seed,
                    uint64_t counter, const void* logu, int32_t* n_accept, int32_t* static_max, const T* plr,
                    int mover_spin = -1) {
  const fire_problem* p = c.p;
  const int n = p->n_el, Wc = c.Wc;
  cudaStream_t s = c.s;
  T* rn = c.template buf<T>(c.P.rn);
  int* S = c.template buf<int>(Q.S);
  int* S_cnt = c.template buf<int>(Q.S_cnt);
  int* acc = c.template buf<int>(Q.acc);
  const int* moved = c.template buf<int>(Q.moved);
  const cudaError_t ev = lr_evaluate<T>(c, Q, KS, KM, rr, static_max, nullptr, mover_spin);
  if (ev != cudaSuccess) return ev;
  T* lpn = c.template buf<T>(c.P.lpn);
  g_nlaunch++;
  k_accept<T><<<Wc, 128, 0, s>>>(rr, rn, reinterpret_cast<T*>(logpsi), lpn, n, c.w0, p->n_walkers, st, seed, counter,
                                 reinterpret_cast<const T*>(logu), n_accept, c.template buf<int>(Q.counts_p),
                                 static_max, plr, acc);
  // accepted walkers: rows into the state, Woodbury update of the inverse
  g_nlaunch++;
  k_lr_commit<T><<<dim3(KS + KM, Wc), 256, 0, s>>>(
      acc, S, S_cnt, KS, n, moved, KM, c.template buf<T>(Q.hS), c.template buf<T>(Q.rawU), c.template buf<T>(Q.env_p),
      c.template buf<T>(Q.aS), c.template buf<T>(Q.vS), c.template buf<T>(Q.oS), c.template buf<T>(Q.E5p),
      c.template buf<int>(Q.en_cnt_p), c.template buf<int>(Q.en_idx_p), c.template buf<int>(Q.counts_p),
      c.template buf<double>(Q.ld_p), c.template buf<double>(Q.sd_p), c.template buf<T>(c.P.B2X),
      c.template buf<T>(c.P.rawx), c.template buf<T>(c.P.env), c.template buf<T>(c.P.Apl), c.template buf<T>(c.P.aX),
      c.template buf<T>(Q.vals), c.template buf<T>(c.P.Xo2), c.template buf<T>(c.P.E5o), c.nb,
      c.template buf<double>(c.P.ld), c.template buf<double>(c.P.sd));
  const dim3 wg((n + 31) / 32, NDET, Wc);
  g_nlaunch += 3;
  k_lr_wb_z<T><<<wg, 256, 0, s>>>(acc, S_cnt, KS, n, c.template buf<T>(Q.B), c.template buf<T>(Q.V),
                                  c.template buf<T>(Q.Zb));
  k_lr_wb_q<T><<<wg, 256, 0, s>>>(acc, S, S_cnt, KS, n, c.template buf<T>(Q.B), c.template buf<double>(Q.Minv),
                                  c.template buf<T>(Q.Qb));
  k_lr_wb_apply<T><<<wg, 256, 0, s>>>(acc, S_cnt, KS, n, c.template buf<T>(Q.B), c.template buf<T>(Q.Zb),
                                      c.template buf<T>(Q.Qb));
  return cudaPeekAtLastError();
}

// The unit-sphere quadratures of make_spherical_grid: 1 and 2 points, the tetrahedron, the octahedron and the
// icosahedron (vertices the cyclic permutations of (0, +-1, +-phi) / sqrt(1 + phi^2), phi the golden ratio).
EcpQuad ecp_quadratures() {
  EcpQuad q;
  std::memset(&q, 0, sizeof(q));
  auto sph = [&](int row, double th, double ph) {
    q.p[row][0] = std::sin(th) * std::cos(ph);
    q.p[row][1] = std::sin(th) * std::sin(ph);
    q.p[row][2] = std::cos(th);
  };
  const double pi = 3.141592653589793;
  sph(0, 0.0, 0.0);
  sph(1, 0.0, 0.0);
  sph(2, pi, 0.0);
  const double tet = std::acos(-1.0 / 3.0);
  sph(3, 0.0, 0.0);
  sph(4, tet, 0.0);
  sph(5, tet, 2 * pi / 3);
  sph(6, tet, 4 * pi / 3);
  const double h = pi / 2;
  sph(7, 0.0, 0.0);
  sph(8, pi, 0.0);
  sph(9, h, 0.0);
  sph(10, h, h);
  sph(11, h, pi);
  sph(12, h, 3 * h);
  const double phi = (1.0 + std::sqrt(5.0)) / 2.0, x = phi / std::sqrt(1.0 + phi * phi), y = 1.0 / std::sqrt(1.0 + phi * phi);
  const double ico[12][3] = {{x, 0, -y}, {y, -x, 0}, {0, -y, x}, {x, 0, y},  {-y, -x, 0}, {0, y, -x},
                             {-x, 0, -y}, {-y, x, 0}, {0, y, x}, {-x, 0, y}, {y, x, 0},   {0, -y, -x}};
  for (int k = 0; k < 12; ++k)
    for (int c = 0; c < 3; ++c) q.p[13 + k][c] = ico[k][c];
  return q;
}

// Pseudopotential energy of every walker: per chunk the state from one value-path evaluation, the local term, and for
// every electron e and quadrature point k the low-rank log|psi| of the moved configurations, accumulated into the
// non-local term.
template <typename T>
fire_status run_ecp(const fire_problem* p, cudaStream_t s, const float* R, const float* Z, const void* prepared,
                    const void* r, const fire_ecp& ecp, int KS, uint64_t seed, uint64_t counter, const void* rot,
                    void* out, int32_t* static_max, void* ws, size_t wsb, int32_t* status) {
  const int Wc = choose_chunk_lr(p, wsb, KS);
  if (Wc <= 0) return FIRE_ERR_WORKSPACE;
  Ctx<T> c = make_ctx<T>(p, s, R, Z, prepared, status, ws, Wc, false);
  const LrPlan Q = make_lr_plan(p, Wc, KS);
  const EcpQuad qt = ecp_quadratures();
  T* rr = const_cast<T*>(reinterpret_cast<const T*>(r));  // read only: nothing is committed
  const int n = p->n_el;
  for (int w0 = 0; w0 < p->n_walkers; w0 += Wc) {
    c.w0 = w0;
    c.Wc = std::min(Wc, p->n_walkers - w0);
    c.r = rr + (size_t)w0 * n * 3;
    T* lp0 = c.template buf<T>(Q.lp0);
    T* sgn0 = c.template buf<T>(Q.sgn0);
    double* acc = c.template buf<double>(Q.ecp_acc);
    double* pt = c.template buf<double>(Q.ecp_pt);
    if (chunk_state<T>(c, Q, lp0, sgn0, 0) != cudaSuccess) return launch_status("pseudopotential state");
    g_nlaunch++;
    k_ecp_local<T><<<c.Wc, 256, 0, s>>>(c.r, n, R, ecp, acc);
    for (int e = 0; e < n; ++e)
      for (int k = 0; k < ecp.max_quad; ++k) {
        g_nlaunch++;
        k_ecp_point<T><<<c.Wc, 128, 0, s>>>(c.r, c.template buf<T>(c.P.rn), n, e, k, R, ecp, qt, w0, seed, counter,
                                            reinterpret_cast<const T*>(rot), pt, c.template buf<int>(Q.moved));
        if (lr_evaluate<T>(c, Q, KS, 1, rr, static_max, c.template buf<T>(Q.sgn_p)) != cudaSuccess)
          return launch_status("pseudopotential ratio");
        g_nlaunch++;
        k_ecp_accum<T><<<nblk(c.Wc), 256, 0, s>>>(c.Wc, pt, c.template buf<T>(c.P.lpn), c.template buf<T>(Q.sgn_p),
                                                  lp0, sgn0, ecp, acc);
      }
    g_nlaunch++;
    k_ecp_store<T><<<nblk(c.Wc), 256, 0, s>>>(c.Wc, w0, acc, reinterpret_cast<T*>(out));
  }
  return launch_status(__func__);
}

// Low-rank Metropolis block (mcmc_steps_low_rank): per chunk the state from one value-path evaluation, then every
// step from the state.  kind MC_SINGLE: proposal_single_electron (electron (offset + step) mod n moved by width
// eps); MC_JUMP: proposal_jump_to_atom (a random electron per walker to a random nucleus, width = sigma, the
// proposal's log ratio in the test); MC_CLUSTER: proposal_cluster_update (ck electrons at most within cradius of a
// sequential or random center, its validity in the test).
template <typename T>
fire_status run_mcmc_lr(const fire_problem* p, cudaStream_t s, const float* R, const float* Z, const void* prepared,
                        void* r, void* logpsi, int steps, int offset, float width, int KS, uint64_t seed,
                        uint64_t counter, const void* noise, const void* logu, int32_t* n_accept,
                        int32_t* static_max, void* ws, size_t wsb, int32_t* status, int kind = MC_SINGLE, int ck = 1,
                        float cradius = 0.f, int crandom = 0) {
  const int Wc = choose_chunk_lr(p, wsb, KS);
  if (Wc <= 0) return FIRE_ERR_WORKSPACE;
  Ctx<T> c = make_ctx<T>(p, s, R, Z, prepared, status, ws, Wc, false);
  // the Metropolis test only compares log|psi| values: plain value contractions for the state and the changed rows,
  // as in the blocks that evaluate every proposal in full (the pseudopotential energy keeps the compensated ones)
  c.comp = false;
  const LrPlan Q = make_lr_plan(p, Wc, KS);
  T* rr = reinterpret_cast<T*>(r);
  const int n = p->n_el;
  for (int w0 = 0; w0 < p->n_walkers; w0 += Wc) {
    c.w0 = w0;
    c.Wc = std::min(Wc, p->n_walkers - w0);
    c.r = rr + (size_t)w0 * n * 3;
    if (chunk_state<T>(c, Q, logpsi, nullptr, w0) != cudaSuccess) return launch_status("low-rank state");
    int* moved = c.template buf<int>(Q.moved);
    T* plr = (kind == MC_JUMP || kind == MC_CLUSTER) ? c.template buf<T>(c.P.plr) : nullptr;
    const int KM = kind == MC_CLUSTER ? ck : 1;
    for (int st = 0; st < steps; ++st) {
      g_nlaunch++;
      if (kind == MC_CLUSTER)
        k_propose_cluster<T><<<c.Wc, 32, 0, s>>>(rr + (size_t)w0 * n * 3, c.template buf<T>(c.P.rn), plr, n, w0,
                                                 p->n_walkers, st, offset, ck, (T)cradius, (T)width, crandom, seed,
                                                 counter, reinterpret_cast<const T*>(noise), moved);
      else if (kind == MC_JUMP)
        k_propose_jump<T><<<c.Wc, 128, 0, s>>>(rr + (size_t)w0 * n * 3, c.template buf<T>(c.P.rn), plr, n, w0,
                                               p->n_walkers, st, R, Z, p->n_nuc, (T)width, seed, counter,
                                               reinterpret_cast<const T*>(noise), moved);
      else
        k_propose_single<T><<<c.Wc, 128, 0, s>>>(rr + (size_t)w0 * n * 3, c.template buf<T>(c.P.rn), n, w0,
                                                 p->n_walkers, st, offset, (T)width, seed, counter,
                                                 reinterpret_cast<const T*>(noise), moved);
      // the sequential sweep moves electron (offset + st) mod n of every walker: one spin per step
      const int mover = kind == MC_SINGLE ? (int)(((long)offset + st) % n) : -1;
      const int mover_spin = mover < 0 ? -1 : (mover < p->n_up ? 0 : 1);
      if (lr_step<T>(c, Q, KS, KM, rr, logpsi, st, seed, counter, logu, n_accept, static_max, plr, mover_spin) !=
          cudaSuccess)
        return launch_status("low-rank step");
    }
  }
  return launch_status(__func__);
}

}  // namespace

namespace fire {
void prep_offsets_host(const fire_problem* p, int64_t* off) { prep_offsets(p, off); }
}  // namespace fire

// ================================================================================== C ABI
extern "C" {

int32_t fire_abi_version(void) { return FIRE_ABI_VERSION; }

fire_status fire_param_layout(const fire_problem* prob, int64_t* offsets) {
  if (!valid(prob) || !offsets) return FIRE_ERR_INVALID;
  blob_offsets(prob, offsets);
  return FIRE_OK;
}

fire_status fire_prepared_size(const fire_problem* prob, size_t* bytes) {
  if (!valid(prob) || !bytes) return FIRE_ERR_INVALID;
  int64_t off[PR_COUNT + 1];
  prep_offsets(prob, off);
  *bytes = (size_t)off[PR_COUNT] * elem_size(prob);
  if (prob->precision != FIRE_PREC_FP64) *bytes = prep64_offset(prob) + (size_t)off[PR_COUNT] * 8;
  return FIRE_OK;
}

fire_status fire_workspace_size(const fire_problem* prob, int32_t chunk, size_t* bytes) {
  if (!valid(prob) || !bytes) return FIRE_ERR_INVALID;
  const int c = chunk > 0 ? std::min(chunk, prob->n_walkers) : prob->n_walkers;
  *bytes = eloc_ws_bytes(prob, c, nullptr);
  return FIRE_OK;
}

fire_status fire_prepare_params(void* stream, const fire_problem* prob, const float* blob,
                                const int64_t* offsets_host, void* prepared, size_t prepared_bytes) {
  if (!valid(prob) || !blob || !offsets_host || !prepared) return FIRE_ERR_INVALID;
  int64_t ref[FIRE_P_COUNT + 1];
  blob_offsets(prob, ref);
  for (int k = 0; k <= FIRE_P_COUNT; ++k)
    if (offsets_host[k] != ref[k]) return FIRE_ERR_INVALID;
  size_t need = 0;
  fire_prepared_size(prob, &need);
  if (prepared_bytes < need) return FIRE_ERR_WORKSPACE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (prob->precision == FIRE_PREC_FP64) return prepare_impl<double>(s, prob, blob, offsets_host, prepared);
  fire_status st = prepare_impl<float>(s, prob, blob, offsets_host, prepared);
  if (st == FIRE_OK) {  // the FP64 copy of the refinement pass
    const fire_problem p64 = refine_problem64(prob, 1);
    st = prepare_impl<double>(s, &p64, blob, offsets_host,
                              reinterpret_cast<unsigned char*>(prepared) + prep64_offset(prob));
  }
  if (st != FIRE_OK || prob->precision != FIRE_PREC_MIXED) return st;
  int64_t off[PR_COUNT + 1];
  prep_offsets(prob, off);
  size_t to[TC_COUNT + 1];
  tc_offsets(prob, (size_t)off[PR_COUNT] * 4, to);
  unsigned char* base = reinterpret_cast<unsigned char*>(prepared);
  for (int k = 0; k < TC_COUNT; ++k) {
    size_t K, N;
    int cnt;
    tc_shape(k, prob, &K, &N, &cnt);
    __nv_bfloat16* hi = reinterpret_cast<__nv_bfloat16*>(base + to[k]);
    __nv_bfloat16* lo = hi + (size_t)cnt * N * K;
    for (int m = 0; m < cnt; ++m) {
      const float* src = reinterpret_cast<const float*>(prepared) + off[kTcSrc[k].slot] + (size_t)m * K * N;
      g_nlaunch++;
      if (tc_tiled(k, K))
        split_tiles(src, (int)K, (int)N, hi + (size_t)m * tc_tiles_bytes(K, N) / 2, s,
                    tc_grid(k, K)
                        ? reinterpret_cast<float*>(base + to[k] + tc_cs_offset(K, N, cnt)) + (size_t)m * N
                        : nullptr);
      else split_transpose(src, (int)K, (int)N, hi + (size_t)m * N * K, lo + (size_t)m * N * K, s);
    }
  }
  return launch_status(__func__);
}

fire_status fire_neighbors(void* stream, const fire_problem* prob, const void* r, const float* R,
                           const fire_neighbor_out* out, int32_t* status) {
  if (!valid(prob) || !r || !R || !out) return FIRE_ERR_INVALID;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  Nbr nb;
  std::memset(&nb, 0, sizeof(nb));
  nb.W = prob->n_walkers;
  nb.n = prob->n_el;
  nb.n_up = prob->n_up;
  nb.N = prob->n_nuc;
  nb.cap_p = prob->cap_pairs;
  nb.cap_nuc = prob->cap_nuc;
  const int n = prob->n_el;
  if (prob->precision == FIRE_PREC_FP64) {
    const size_t smem = 3 * n * sizeof(double) + (5 * n + 2) * sizeof(int);
    cudaFuncSetAttribute(k_neighbors<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    g_nlaunch++;
    k_neighbors<double><<<prob->n_walkers, 512, smem, s>>>(reinterpret_cast<const double*>(r), R,
                                                          (double)prob->cutoff, (double)prob->cutoff_1el, nb, *out,
                                                          status);
  } else {
    const size_t smem = 3 * n * sizeof(float) + (5 * n + 2) * sizeof(int);
    cudaFuncSetAttribute(k_neighbors<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    g_nlaunch++;
    k_neighbors<float><<<prob->n_walkers, 512, smem, s>>>(reinterpret_cast<const float*>(r), R, prob->cutoff,
                                                         prob->cutoff_1el, nb, *out, status);
  }
  return launch_status(__func__);
}

fire_status fire_triplets(void* stream, const fire_problem* prob, const void* r, int32_t cap_triplets,
                          int32_t* trip_in, int32_t* trip_k, int32_t* trip_kn, int32_t* trip_i, void* workspace,
                          size_t workspace_bytes, int32_t* status) {
  if (!valid(prob) || !r || !trip_in || !trip_k || !trip_kn || !trip_i || cap_triplets < 1)
    return FIRE_ERR_INVALID;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int n = prob->n_el, B = prob->n_walkers;
  const size_t need = (size_t)B * (n + (n + 1) + 2 * prob->cap_pairs + n + (size_t)n * prob->cap_nuc + 4) * 4 + 1024;
  if (workspace_bytes < need || !workspace) return FIRE_ERR_WORKSPACE;
  int* w = reinterpret_cast<int*>(workspace);
  Nbr nb;
  nb.W = B; nb.n = n; nb.n_up = prob->n_up; nb.N = prob->n_nuc; nb.cap_p = prob->cap_pairs; nb.cap_nuc = prob->cap_nuc;
  nb.deg = w; w += (size_t)B * n;
  nb.rowptr = w; w += (size_t)B * (n + 1);
  nb.nbr = w; w += (size_t)B * prob->cap_pairs;
  nb.rev = w; w += (size_t)B * prob->cap_pairs;
  nb.en_cnt = w; w += (size_t)B * n;
  nb.en_idx = w; w += (size_t)B * n * prob->cap_nuc;
  nb.counts = w;
  fire_neighbor_out ext;
  std::memset(&ext, 0, sizeof(ext));
  // R is not needed for the e-e structure; nuclei enter only the e-n lists, which are skipped here
  static_assert(sizeof(int) == 4, "int32");
  Nbr nb2 = nb;
  nb2.N = 0;
  if (prob->precision == FIRE_PREC_FP64) {
    const size_t smem = 3 * n * sizeof(double) + (5 * n + 2) * sizeof(int);
    cudaFuncSetAttribute(k_neighbors<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    g_nlaunch++;
    k_neighbors<double><<<B, 512, smem, s>>>(reinterpret_cast<const double*>(r), nullptr, (double)prob->cutoff,
                                            (double)prob->cutoff_1el, nb2, ext, status);
  } else {
    const size_t smem = 3 * n * sizeof(float) + (5 * n + 2) * sizeof(int);
    cudaFuncSetAttribute(k_neighbors<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    g_nlaunch++;
    k_neighbors<float><<<B, 512, smem, s>>>(reinterpret_cast<const float*>(r), nullptr, prob->cutoff,
                                           prob->cutoff_1el, nb2, ext, status);
  }
  g_nlaunch++;
  k_triplets<<<B, 256, 0, s>>>(nb, cap_triplets, trip_in, trip_k, trip_kn, trip_i, status);
  return launch_status(__func__);
}

fire_status fire_logpsi(void* stream, const fire_problem* prob, const float* R, const float* Z, const void* prepared,
                        const void* r, void* sign, void* logpsi, void* workspace, size_t workspace_bytes,
                        int32_t* status) {
  if (!valid(prob) || !R || !Z || !prepared || !r || !logpsi || !workspace) return FIRE_ERR_INVALID;
  if (prob->n_el > ELOC_MAX_EL) return FIRE_ERR_UNSUPPORTED;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (prob->precision == FIRE_PREC_FP64)
    return run_logpsi<double>(prob, s, R, Z, prepared, r, sign, logpsi, workspace, workspace_bytes, status);
  return run_logpsi<float>(prob, s, R, Z, prepared, r, sign, logpsi, workspace, workspace_bytes, status);
}

fire_status fire_logpsi_grad_workspace_size(const fire_problem* prob, int32_t chunk, size_t* bytes) {
  if (!valid(prob) || !bytes) return FIRE_ERR_INVALID;
  *bytes = fire::grad_workspace_bytes(prob, chunk);
  return FIRE_OK;
}

fire_status fire_logpsi_grad(void* stream, const fire_problem* prob, const float* R, const void* prepared,
                             const void* r, void* sign, void* logpsi, void* grad, void* workspace,
                             size_t workspace_bytes, int32_t* status) {
  if (!valid(prob) || !R || !prepared || !r || !sign || !logpsi || !grad || !workspace) return FIRE_ERR_INVALID;
  if (prob->n_el > ELOC_MAX_EL) return FIRE_ERR_UNSUPPORTED;
  int64_t off[FIRE_P_COUNT + 1];
  blob_offsets(prob, off);
  // the edge bias of each e-e filter follows its edge kernel in the blob (one reduction writes both)
  if (off[FIRE_P_EESAME_EDGE_B] != off[FIRE_P_EESAME_EDGE_W] + 4 * F ||
      off[FIRE_P_EEDIFF_EDGE_B] != off[FIRE_P_EEDIFF_EDGE_W] + 4 * F)
    return FIRE_ERR_UNSUPPORTED;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const fire_status st = fire::grad_dispatch(prob, s, R, prepared, r, sign, logpsi, grad, workspace,
                                             workspace_bytes, status);
  if (st != FIRE_OK) return st;
  return launch_status(__func__);
}

fire_status fire_local_energy(void* stream, const fire_problem* prob, const float* R, const float* Z,
                              const void* prepared, const void* r, void* logpsi, void* sign, void* e_loc,
                              double* e_stats, const fire_eloc_debug* debug, void* workspace, size_t workspace_bytes,
                              int32_t* status) {
  if (!valid(prob) || !R || !Z || !prepared || !r || !e_loc || !workspace) return FIRE_ERR_INVALID;
  if (prob->n_el > ELOC_MAX_EL) return FIRE_ERR_UNSUPPORTED;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (prob->precision == FIRE_PREC_FP64)
    return run_eloc<double>(prob, s, R, Z, prepared, r, logpsi, sign, e_loc, e_stats, debug, workspace,
                            workspace_bytes, status);
  return run_eloc<float>(prob, s, R, Z, prepared, r, logpsi, sign, e_loc, e_stats, debug, workspace, workspace_bytes,
                         status);
}

fire_status fire_embedding(void* stream, const fire_problem* prob, const float* R, const void* prepared, const void* r,
                           void* h_contract, void* h_update, void* workspace, size_t workspace_bytes,
                           int32_t* status) {
  if (!valid(prob) || !R || !prepared || !r || !workspace) return FIRE_ERR_INVALID;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (prob->precision == FIRE_PREC_FP64)
    return run_embedding<double>(prob, s, R, prepared, r, h_contract, h_update, workspace, workspace_bytes, status);
  return run_embedding<float>(prob, s, R, prepared, r, h_contract, h_update, workspace, workspace_bytes, status);
}

fire_status fire_mcmc_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                            const void* prepared, void* r, void* logpsi, int32_t steps, float width, uint64_t seed,
                            uint64_t counter, const void* replay_noise, const void* replay_log_u, int32_t* n_accept,
                            int32_t* static_max, void* workspace, size_t workspace_bytes, int32_t* status) {
  if (!valid(prob) || !R || !Z || !prepared || !r || !logpsi || !workspace || steps < 0) return FIRE_ERR_INVALID;
  if ((replay_noise == nullptr) != (replay_log_u == nullptr)) return FIRE_ERR_INVALID;
  if (prob->n_el > ELOC_MAX_EL) return FIRE_ERR_UNSUPPORTED;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (prob->precision == FIRE_PREC_FP64)
    return run_mcmc<double>(prob, s, R, Z, prepared, r, logpsi, steps, width, seed, counter, replay_noise,
                            replay_log_u, n_accept, static_max, workspace, workspace_bytes, status);
  return run_mcmc<float>(prob, s, R, Z, prepared, r, logpsi, steps, width, seed, counter, replay_noise, replay_log_u,
                         n_accept, static_max, workspace, workspace_bytes, status);
}

fire_status fire_mcmc_single_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                                   const void* prepared, void* r, void* logpsi, int32_t steps, int32_t step_offset,
                                   float width, uint64_t seed, uint64_t counter, const void* replay_noise,
                                   const void* replay_log_u, int32_t* n_accept, int32_t* static_max, void* workspace,
                                   size_t workspace_bytes, int32_t* status) {
  if (!valid(prob) || !R || !Z || !prepared || !r || !logpsi || !workspace || steps < 0 || step_offset < 0)
    return FIRE_ERR_INVALID;
  if ((replay_noise == nullptr) != (replay_log_u == nullptr)) return FIRE_ERR_INVALID;
  if (prob->n_el > ELOC_MAX_EL) return FIRE_ERR_UNSUPPORTED;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (prob->precision == FIRE_PREC_FP64)
    return run_mcmc<double>(prob, s, R, Z, prepared, r, logpsi, steps, width, seed, counter, replay_noise,
                            replay_log_u, n_accept, static_max, workspace, workspace_bytes, status, MC_SINGLE,
                            step_offset);
  return run_mcmc<float>(prob, s, R, Z, prepared, r, logpsi, steps, width, seed, counter, replay_noise, replay_log_u,
                         n_accept, static_max, workspace, workspace_bytes, status, MC_SINGLE, step_offset);
}

fire_status fire_mcmc_cluster_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                                    const void* prepared, void* r, void* logpsi, int32_t steps, int32_t step_offset,
                                    float width, int32_t max_cluster_size, float max_cluster_radius,
                                    int32_t random_sweep, uint64_t seed, uint64_t counter, const void* replay_draws,
                                    const void* replay_log_u, int32_t* n_accept, int32_t* static_max, void* workspace,
                                    size_t workspace_bytes, int32_t* status) {
  if (!valid(prob) || !R || !Z || !prepared || !r || !logpsi || !workspace || steps < 0 || step_offset < 0 ||
      max_cluster_size < 1 || !(max_cluster_radius >= 0.f))
    return FIRE_ERR_INVALID;
  if (max_cluster_size > CLUSTER_KMAX) return FIRE_ERR_UNSUPPORTED;
  if ((replay_draws == nullptr) != (replay_log_u == nullptr)) return FIRE_ERR_INVALID;
  const int k = std::min<int>(max_cluster_size, prob->n_el);
  if (prob->n_el > ELOC_MAX_EL) return FIRE_ERR_UNSUPPORTED;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (prob->precision == FIRE_PREC_FP64)
    return run_mcmc<double>(prob, s, R, Z, prepared, r, logpsi, steps, width, seed, counter, replay_draws,
                            replay_log_u, n_accept, static_max, workspace, workspace_bytes, status, MC_CLUSTER,
                            step_offset, k, max_cluster_radius, random_sweep ? 1 : 0);
  return run_mcmc<float>(prob, s, R, Z, prepared, r, logpsi, steps, width, seed, counter, replay_draws, replay_log_u,
                         n_accept, static_max, workspace, workspace_bytes, status, MC_CLUSTER, step_offset, k,
                         max_cluster_radius, random_sweep ? 1 : 0);
}

fire_status fire_mcmc_jump_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                                 const void* prepared, void* r, void* logpsi, int32_t steps, float sigma, uint64_t seed,
                                 uint64_t counter, const void* replay_draws, const void* replay_log_u,
                                 int32_t* n_accept, int32_t* static_max, void* workspace, size_t workspace_bytes,
                                 int32_t* status) {
  if (!valid(prob) || !R || !Z || !prepared || !r || !logpsi || !workspace || steps < 0 || !(sigma > 0.f))
    return FIRE_ERR_INVALID;
  if ((replay_draws == nullptr) != (replay_log_u == nullptr)) return FIRE_ERR_INVALID;
  if (prob->n_el > ELOC_MAX_EL) return FIRE_ERR_UNSUPPORTED;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (prob->precision == FIRE_PREC_FP64)
    return run_mcmc<double>(prob, s, R, Z, prepared, r, logpsi, steps, sigma, seed, counter, replay_draws,
                            replay_log_u, n_accept, static_max, workspace, workspace_bytes, status, MC_JUMP);
  return run_mcmc<float>(prob, s, R, Z, prepared, r, logpsi, steps, sigma, seed, counter, replay_draws, replay_log_u,
                         n_accept, static_max, workspace, workspace_bytes, status, MC_JUMP);
}

fire_status fire_low_rank_workspace_size(const fire_problem* prob, int32_t chunk, int32_t cap_changed,
                                         size_t* bytes) {
  if (!valid(prob) || !bytes || chunk < 1 || cap_changed < 1) return FIRE_ERR_INVALID;
  if (cap_changed > LR_KMAX) return FIRE_ERR_UNSUPPORTED;
  *bytes = make_lr_plan(prob, std::min(chunk, prob->n_walkers), std::min<int>(cap_changed, prob->n_el)).total;
  return FIRE_OK;
}

fire_status fire_mcmc_low_rank_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                                     const void* prepared, void* r, void* logpsi, int32_t steps, int32_t step_offset,
                                     float width, int32_t cap_changed, uint64_t seed, uint64_t counter,
                                     const void* replay_noise, const void* replay_log_u, int32_t* n_accept,
                                     int32_t* static_max, void* workspace, size_t workspace_bytes, int32_t* status) {
  if (!valid(prob) || !R || !Z || !prepared || !r || !logpsi || !workspace || steps < 0 || step_offset < 0 ||
      cap_changed < 1)
    return FIRE_ERR_INVALID;
  if ((replay_noise == nullptr) != (replay_log_u == nullptr)) return FIRE_ERR_INVALID;
  if (prob->n_el > ELOC_MAX_EL || cap_changed > LR_KMAX) return FIRE_ERR_UNSUPPORTED;
  const int KS = std::min<int>(cap_changed, prob->n_el);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (prob->precision == FIRE_PREC_FP64)
    return run_mcmc_lr<double>(prob, s, R, Z, prepared, r, logpsi, steps, step_offset, width, KS, seed, counter,
                               replay_noise, replay_log_u, n_accept, static_max, workspace, workspace_bytes, status);
  return run_mcmc_lr<float>(prob, s, R, Z, prepared, r, logpsi, steps, step_offset, width, KS, seed, counter,
                            replay_noise, replay_log_u, n_accept, static_max, workspace, workspace_bytes, status);
}

fire_status fire_mcmc_low_rank_jump_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                                          const void* prepared, void* r, void* logpsi, int32_t steps, float sigma,
                                          int32_t cap_changed, uint64_t seed, uint64_t counter,
                                          const void* replay_draws, const void* replay_log_u, int32_t* n_accept,
                                          int32_t* static_max, void* workspace, size_t workspace_bytes,
                                          int32_t* status) {
  if (!valid(prob) || !R || !Z || !prepared || !r || !logpsi || !workspace || steps < 0 || !(sigma > 0.f) ||
      cap_changed < 1)
    return FIRE_ERR_INVALID;
  if ((replay_draws == nullptr) != (replay_log_u == nullptr)) return FIRE_ERR_INVALID;
  if (prob->n_el > ELOC_MAX_EL || cap_changed > LR_KMAX) return FIRE_ERR_UNSUPPORTED;
  const int KS = std::min<int>(cap_changed, prob->n_el);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (prob->precision == FIRE_PREC_FP64)
    return run_mcmc_lr<double>(prob, s, R, Z, prepared, r, logpsi, steps, 0, sigma, KS, seed, counter, replay_draws,
                               replay_log_u, n_accept, static_max, workspace, workspace_bytes, status, MC_JUMP);
  return run_mcmc_lr<float>(prob, s, R, Z, prepared, r, logpsi, steps, 0, sigma, KS, seed, counter, replay_draws,
                            replay_log_u, n_accept, static_max, workspace, workspace_bytes, status, MC_JUMP);
}

fire_status fire_mcmc_low_rank_cluster_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                                             const void* prepared, void* r, void* logpsi, int32_t steps,
                                             int32_t step_offset, float width, int32_t max_cluster_size,
                                             float max_cluster_radius, int32_t random_sweep, int32_t cap_changed,
                                             uint64_t seed, uint64_t counter, const void* replay_draws,
                                             const void* replay_log_u, int32_t* n_accept, int32_t* static_max,
                                             void* workspace, size_t workspace_bytes, int32_t* status) {
  if (!valid(prob) || !R || !Z || !prepared || !r || !logpsi || !workspace || steps < 0 || step_offset < 0 ||
      max_cluster_size < 1 || !(max_cluster_radius >= 0.f) || cap_changed < 1)
    return FIRE_ERR_INVALID;
  if ((replay_draws == nullptr) != (replay_log_u == nullptr)) return FIRE_ERR_INVALID;
  if (max_cluster_size > CLUSTER_KMAX || prob->n_el > ELOC_MAX_EL || cap_changed > LR_KMAX)
    return FIRE_ERR_UNSUPPORTED;
  const int k = std::min<int>(max_cluster_size, prob->n_el);
  const int KS = std::min<int>(cap_changed, prob->n_el);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (prob->precision == FIRE_PREC_FP64)
    return run_mcmc_lr<double>(prob, s, R, Z, prepared, r, logpsi, steps, step_offset, width, KS, seed, counter,
                               replay_draws, replay_log_u, n_accept, static_max, workspace, workspace_bytes, status,
                               MC_CLUSTER, k, max_cluster_radius, random_sweep ? 1 : 0);
  return run_mcmc_lr<float>(prob, s, R, Z, prepared, r, logpsi, steps, step_offset, width, KS, seed, counter,
                            replay_draws, replay_log_u, n_accept, static_max, workspace, workspace_bytes, status,
                            MC_CLUSTER, k, max_cluster_radius, random_sweep ? 1 : 0);
}

fire_status fire_ecp_quadrature(int32_t n_points, double* points) {
  if (!points || !(n_points == 1 || n_points == 2 || n_points == 4 || n_points == 6 || n_points == 12))
    return FIRE_ERR_INVALID;
  const EcpQuad q = ecp_quadratures();
  const int row = ecp_quad_row(n_points);
  for (int k = 0; k < n_points; ++k)
    for (int c = 0; c < 3; ++c) points[3 * k + c] = q.p[row + k][c];
  return FIRE_OK;
}

fire_status fire_ecp_energy(void* stream, const fire_problem* prob, const float* R, const float* Z,
                            const void* prepared, const void* r, const fire_ecp* ecp, int32_t cap_changed,
                            uint64_t seed, uint64_t counter, const void* replay_rotations, void* e_ecp,
                            int32_t* static_max, void* workspace, size_t workspace_bytes, int32_t* status) {
  if (!valid(prob) || !R || !Z || !prepared || !r || !ecp || !e_ecp || !workspace || cap_changed < 1)
    return FIRE_ERR_INVALID;
  if (ecp->n_ecp < 1 || ecp->n_grid < 2 || ecp->n_l < 0 || ecp->n_l > 4 || !ecp->atom || !ecp->grid || !ecp->v_loc ||
      (ecp->n_l > 0 && !ecp->v_nl) || !ecp->cutoff || !ecp->n_quad || ecp->max_quad < 1 || ecp->max_quad > 12)
    return FIRE_ERR_INVALID;
  if (prob->n_el > ELOC_MAX_EL || cap_changed > LR_KMAX) return FIRE_ERR_UNSUPPORTED;
  const int KS = std::min<int>(cap_changed, prob->n_el);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (prob->precision == FIRE_PREC_FP64)
    return run_ecp<double>(prob, s, R, Z, prepared, r, *ecp, KS, seed, counter, replay_rotations, e_ecp, static_max,
                           workspace, workspace_bytes, status);
  return run_ecp<float>(prob, s, R, Z, prepared, r, *ecp, KS, seed, counter, replay_rotations, e_ecp, static_max,
                        workspace, workspace_bytes, status);
}

fire_status fire_potential_energy(void* stream, const fire_problem* prob, const void* r, const float* R,
                                  const float* Z, void* out) {
  if (!valid(prob) || !r || !R || !Z || !out) return FIRE_ERR_INVALID;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  g_nlaunch++;
  if (prob->precision == FIRE_PREC_FP64)
    k_potential<double><<<prob->n_walkers, 256, 0, s>>>(prob->n_el, prob->n_nuc, reinterpret_cast<const double*>(r),
                                                        R, Z, reinterpret_cast<double*>(out));
  else
    k_potential<float><<<prob->n_walkers, 256, 0, s>>>(prob->n_el, prob->n_nuc, reinterpret_cast<const float*>(r), R,
                                                       Z, reinterpret_cast<float*>(out));
  return launch_status(__func__);
}

fire_status fire_gemm_mixed(void* stream, int32_t M, int32_t N, int32_t K, const float* A, const float* W, float* C,
                            void* workspace, size_t workspace_bytes, int32_t* status) {
  if (M < 1 || N < 1 || K < 8 || K % 8 != 0 || !A || !W || !C || !workspace) return FIRE_ERR_INVALID;
  const size_t need = K <= 256 ? tc_tiles_bytes(K, N) + 4 * (size_t)N : 4 * (size_t)N * K;
  if (workspace_bytes < need) return FIRE_ERR_WORKSPACE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  __nv_bfloat16* hi = reinterpret_cast<__nv_bfloat16*>(workspace);
  g_nlaunch += 2;
  TcWeights wt{};
  if (K <= 256) {
    float* cs = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(workspace) + tc_tiles_bytes(K, N));
    split_tiles(W, K, N, hi, s, cs);
    wt.tiles = hi;
    wt.cs = cs;
  } else {
    split_transpose(W, K, N, hi, hi + (size_t)N * K, s);
    wt.hi = hi;
    wt.lo = hi + (size_t)N * K;
  }
  GemmP<float> g;
  std::memset(&g, 0, sizeof(g));
  g.A = A; g.lda = K; g.C = C; g.ldc = N; g.M = M; g.N = N; g.K = K; g.node_div = 1; g.M_scale = 1; g.env_nv = 1;
  const cudaError_t e = gemm_tc(EPI_PLAIN, N > 128 ? 256 : 128, g, wt, nullptr, status, s);
  if (e == cudaErrorInvalidValue) return FIRE_ERR_UNSUPPORTED;
  return launch_status(__func__);
}

fire_status fire_profile_enable(int32_t on) {
  for (auto& r : g_recs) {
    g_pool.push_back(r.a);
    g_pool.push_back(r.b);
  }
  g_recs.clear();
  g_prof = on != 0;
  g_nlaunch = 0;
  return FIRE_OK;
}

fire_status fire_profile_report(char* buf, size_t len) {
  if (!buf || len == 0) return FIRE_ERR_INVALID;
  std::vector<std::pair<const char*, std::pair<int, double>>> acc;
  for (auto& r : g_recs) {
    if (cudaEventSynchronize(r.b) != cudaSuccess) return launch_status("profile");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, r.a, r.b);
    bool found = false;
    for (auto& a : acc)
      if (std::strcmp(a.first, r.name) == 0) {
        a.second.first += 1;
        a.second.second += ms;
        found = true;
      }
    if (!found) acc.push_back({r.name, {1, (double)ms}});
  }
  size_t o = 0;
  buf[0] = 0;
  {
    const int w = std::snprintf(buf, len, "kernels_launched %lld 0\n", g_nlaunch);
    if (w > 0 && (size_t)w < len) o = (size_t)w;
  }
  for (auto& a : acc) {
    const int w = std::snprintf(buf + o, len - o, "%s %d %.6f\n", a.first, a.second.first, a.second.second);
    if (w < 0 || (size_t)w >= len - o) break;
    o += (size_t)w;
  }
  return FIRE_OK;
}

}  // extern "C"
