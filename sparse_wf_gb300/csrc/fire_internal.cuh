// fire_internal.cuh -- device-side data structures shared by the pipeline stages.
#pragma once
#include "fire_common.cuh"

namespace fire {

// Neighbour structure of one chunk of walkers (all walkers of a chunk share n, n_up, n_nuc).
// Per walker w and electron i the directed e-e pairs (i, j), j != i, |r_i - r_j| < cutoff, are
// stored CSR-style sorted by (i, j): the same row-major order as jnp.where in get_pair_indices
// (model/new_sparse_model.py:238-263).
struct Nbr {
  int W, n, n_up, N, cap_p, cap_nuc;
  int* deg;     // [W, n]        neighbours of i
  int* rowptr;  // [W, n + 1]    exclusive prefix of deg
  int* nbr;     // [W, cap_p]    neighbour j of pair p
  int* rev;     // [W, cap_p]    index of the reverse pair (j, i)
  int* en_cnt;  // [W, n]        e-n neighbours (capped at cap_nuc)
  int* en_idx;  // [W, n, cap_nuc] nucleus indices, ascending
  int* counts;  // [W, 4]        n_pairs_same, n_pairs_diff, n_triplets, n_neighbours_en
};

// Sparse forward-Laplacian layout of a chunk ("positions" = Jacobian rows of NodeWithFwdLap,
// sparse_fwd_lap.py:14-22).  Per walker w the positions of center i are
//   q = pos_off[w] + rowptr[w][i] + i + k,  k = 0 (self, dep = i) and k = 1..deg(i) (pair (i, j_k)),
// i.e. positions are sorted by center.  Jacobian plane rows are 3 * q + xyz.
// dep_pos lists, for every dep m, the positions (i, m), i in {m} + N(m): slot
//   pos_off[w] + rowptr[w][m] + m + k holds the global position of the k-th of them.
struct Layout {
  int* pos_off;  // [W + 1]
  int* pos_ctr;  // [cap_pos] global electron id (w * n + i) of the center
  int* pos_dep;  // [cap_pos] global electron id of the dependency
  int* dep_pos;  // [cap_pos] positions grouped by dependency
  int cap_pos;   // capacity = W * (n + cap_p)
};

// Split-BF16 weights of a tensor-core contraction: hi/lo planes [N][K] (K contiguous); the second set
// (spin-down weights of the orbital layer) may be null.
struct TcWeights {
  const __nv_bfloat16* hi;  // split weights transposed [N][K] (hi, lo): the streamed-weight kernel (K > 256)
  const __nv_bfloat16* lo;
  const __nv_bfloat16* tiles;   // split weights pre-tiled for the A-resident kernel (K <= 256: FP16 hi / lo of the
                                // column-scaled weights; the envelope kernel: BF16 hi / lo)
  const __nv_bfloat16* tiles2;  // the other spin's tiles, or nullptr
  const float* cs;              // K <= 256: the column scales of tiles [N] (powers of two), else nullptr
  const float* cs2;             // ... of tiles2
};
// Envelope derivative rows of the mixed path (k_env_tc): electrons of one spin block (ns per walker, offset
// soff) of Wc walkers, determinant d.  C = env + d n, row stride ldc floats, nv carrier rows per electron;
// vec = 4 / 2 / 1: widest store the alignment of C and ldc allows.
struct EnvTcP {
  const float* r;   // electron positions [W][n][3]
  const float* R;   // nuclei [N][3]
  const float* sp;  // softplus(sigma) [N][NDET][NENV_ORB]
  float* C;
  long ldc;
  int n, ns, soff, N, Wc, d, nv, vec;
  const float* cs;  // column scales of this determinant's weights [n] (powers of two)
};
// longest envelope contraction (8 N) that k_env_tc splits on an exact grid (hi parts of at most 2^(grid_hb + 1))
constexpr int ENV_TC_KMAX = 4096;
// k_detlap staging: up to chi positions per dependency (3 J rows each, DL_CMAX at most), contraction chunks of
// DL_OC elements in shared-memory rows of DL_LD (16-byte aligned; consecutive rows on distinct bank quads); + 4
// rows because a thread's strided tile rows may run past the last one; DL_STAGES chunks in flight.  Jobs with
// at most DL_CSPLIT positions run in small CTAs (128 threads, 4 per SM), the rest in 256-thread CTAs.
constexpr int DL_CMAX = 64, DL_CSPLIT = 44, DL_OC = 32, DL_LD = DL_OC + 4, DL_STAGES = 2;
__host__ __device__ constexpr int dl_jrows(int chi) { return 3 * chi + 4; }
__host__ __device__ constexpr int dl_stage_elems(int chi) { return (dl_jrows(chi) + chi + 4) * DL_LD; }
__host__ __device__ constexpr int dl_smem_elems(int chi) { return DL_STAGES * dl_stage_elems(chi); }
// Cluster proposals: at most CLUSTER_KMAX electrons per cluster, CLUSTER_TRIALS draws per step
// (proposal_cluster_update, mcmc.py:119-161).
constexpr int CLUSTER_KMAX = 16, CLUSTER_TRIALS = 5;
// Low-rank single-electron steps: at most LR_KMAX electrons in a step's changed set (the moved electron and its
// neighbours before and after the move); the k x k determinant-lemma matrix is eliminated in shared memory.
constexpr int LR_KMAX = 128;
// Unit-sphere quadratures of the pseudopotentials' non-local term, all five in one table passed by value: the 1-, 2-,
// 4-, 6- and 12-point grids at rows 0, 1, 3, 7 and 13 (make_spherical_grid, pseudopotentials.py:44-133).
struct EcpQuad {
  double p[25][3];
};
__host__ __device__ inline int ecp_quad_row(int n_points) {
  return n_points == 1 ? 0 : n_points == 2 ? 1 : n_points == 4 ? 3 : n_points == 6 ? 7 : 13;
}
// Largest electron count of the local-energy and value paths: the double-FP32 / FP64 elimination keeps two n x 17 panel buffers
// of eight-byte elements (plus ~2.5 KB) in shared memory, 288 n + 2496 bytes within the 227 KB per CTA.
constexpr int ELOC_MAX_EL = 798;
// Row length of the transposed orbital-matrix inverse handed from the elimination to the determinant
// Laplacian: room in front for the determinant's alignment shift (d n) mod 4 within the orbital plane, rounded
// to 4 elements (16-byte rows in FP32)
__host__ __device__ inline int ainv_ld(int n) { return (n + 6) / 4 * 4; }
// bytes of the pre-tiled split weights of a K x N matrix: 32 KB per 128-column x 64-deep tile
inline size_t tc_tiles_bytes(size_t K, size_t N) { return ((N + 127) / 128) * ((K + 63) / 64) * 32768; }

// Output pointers of the per-walker assembly (k_assemble).
struct AssembleOut {
  void* logpsi;
  void* sign;
  void* eloc;
  fire_eloc_debug dbg;
  const double* enn;  // input: nucleus-nucleus repulsion of the molecule (one value)
  // ill-conditioned walkers: their batch indices are appended to ref_idx while fewer than ref_cap are stored;
  // ref_cnt counts all of them (null: no flagging)
  int32_t* ref_idx;
  int32_t* ref_cnt;
  int32_t ref_cap;
  double ref_ratio;
  double ref_kappa;
  double ref_ks;
  double ref_kscond;
  // input: kappa_F of every orbital matrix of the launch [Wc * NDET] (null: the condition test is skipped)
  const double* cond;
  // output rows: walker w of the launch writes row wmap[w] when w < *wcnt and nothing otherwise (null: w0 + w)
  const int32_t* wmap;
  const int32_t* wcnt;
};

// A walker is ill-conditioned, and its orbital-matrix values are recomputed in FP64 by the refinement pass of
// the FP32 and mixed local energy, when the two terms that cancel in its kinetic energy exceed its local energy by
// the problem's refine_ratio or its refine_ks Hartree: (|lap log psi| + |grad log psi|^2) / 2 > refine_ratio |E_loc| or
// > refine_ks, or when its orbital matrices are ill-conditioned: sum_d |w_d| kappa_F(A_d) / |sum_d w_d| > refine_kappa,
// or when the product of the two, (|lap| + |grad|^2) / 2 times that condition number, exceeds refine_kscond
// (see fire.h).

// Prepared-parameter slot offsets (elements of the compute type) and the per-walker parameter gradient of log|psi|
// (fire_grad.cu), behind fire_logpsi_grad.
void prep_offsets_host(const fire_problem* p, int64_t* off);
size_t grad_workspace_bytes(const fire_problem* p, int chunk);
fire_status grad_dispatch(const fire_problem* p, cudaStream_t s, const float* R, const void* prepared, const void* r,
                          void* sign, void* logpsi, void* grad, void* ws, size_t ws_bytes, int32_t* status);

}  // namespace fire
