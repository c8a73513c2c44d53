/*
 * fire.h -- C ABI of the GB300-native FiRE local-energy hot path.
 *
 * All array pointers are DEVICE pointers owned by the caller, except where a
 * comment says "host".  No entry point allocates device memory: scratch space is
 * the caller's workspace, sized by fire_workspace_size().  Every call is
 * asynchronous on `stream`; failures detected on the device (capacity overflow,
 * non-finite results) are written to the int32 status word array `status`
 * (FIRE_STATUS_WORDS entries, device memory) and never trap.  The return value
 * reports argument errors and launch failures only.
 *
 * The entry points replace these functions of the reference (MScherbela/sparse_wf,
 * paths relative to its src/sparse_wf/):
 *   fire_neighbors      model/new_sparse_model.py:238-263 get_pair_indices,
 *                       :399-437 get_static_input, :476-481 get_neighbouring_nuclei
 *   fire_triplets       model/sparse_fwd_lap.py:252-291 _get_triplet_indices
 *   fire_logpsi         model/wave_function.py:183-198 MoonLikeWaveFunction.signed
 *   fire_logpsi_grad    preconditioner.py:185-191 jax.grad(log_p) per walker (the SPRING Jacobian rows)
 *   fire_local_energy   hamiltonian.py:69-81 local_energy (kinetic via
 *                       wave_function.py:215-221, potential via hamiltonian.py:15-26),
 *                       batched like update.py:95-100 and reduced like update.py:130-134
 *   fire_mcmc_block     mcmc.py:38-97 mcmc_steps_all_electron
 *   fire_mcmc_single_block  mcmc.py:100-111, 196-275 proposal_single_electron + mcmc_steps_low_rank
 *                       (each proposal evaluated in full, no low-rank state)
 *   fire_mcmc_jump_block    mcmc.py:164-193 proposal_jump_to_atom (make_mcmc's jump_steps)
 *   fire_mcmc_cluster_block mcmc.py:119-161 proposal_cluster_update (make_mcmc "cluster-update")
 *   fire_mcmc_low_rank_block  mcmc.py:100-111, 196-275 with model/wave_function.py:226-287
 *                       log_psi_with_state / log_psi_low_rank_update (the state-carrying single-electron block)
 *   fire_mcmc_low_rank_jump_block  mcmc.py:164-193 proposal_jump_to_atom with the low-rank state
 *   fire_mcmc_low_rank_cluster_block  mcmc.py:119-161 proposal_cluster_update with the low-rank state
 *   fire_ecp_energy     pseudopotentials.py:205-219, 272-398 local and non-local pseudopotential terms
 *   fire_embedding      model/new_sparse_model.py:483-551 NewSparseEmbedding.apply
 *                       (used by the initialiser, new_sparse_model.py:378-379)
 */
#ifndef FIRE_H
#define FIRE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FIRE_NO_NEIGHBOUR 1000000 /* model/graph_utils.py:14 NO_NEIGHBOUR */
#define FIRE_STATUS_WORDS 8
#define FIRE_ABI_VERSION 3

typedef enum {
  FIRE_OK = 0,
  FIRE_ERR_INVALID = 1,     /* bad argument (host-side check) */
  FIRE_ERR_UNSUPPORTED = 2, /* architecture/size outside what the kernels are built for */
  FIRE_ERR_WORKSPACE = 3,   /* workspace too small */
  FIRE_ERR_CUDA = 4         /* a launch failed; cudaGetLastError() has the cause */
} fire_status;

/* bits of status[0] (sticky; the caller clears the status array) */
#define FIRE_FLAG_PAIR_OVERFLOW 1     /* e-e pairs of a walker exceeded cap_pairs */
#define FIRE_FLAG_NUC_OVERFLOW 2      /* e-n neighbours of an electron exceeded cap_nuc */
#define FIRE_FLAG_NONFINITE 4         /* a non-finite log|psi| or E_loc was produced */
#define FIRE_FLAG_TRIPLET_OVERFLOW 8  /* triplet list exceeded its capacity */
#define FIRE_FLAG_SINGULAR 16         /* an orbital matrix had a zero pivot */
#define FIRE_FLAG_TIMEOUT 32          /* a bounded wait on a tensor-core completion barrier gave up */
#define FIRE_FLAG_CHANGED_OVERFLOW 64 /* a low-rank step's changed set exceeded cap_changed */
#define FIRE_FLAG_REFINE_OVERFLOW 128 /* more ill-conditioned walkers than refine_cap (status[5] = their number) */
/* status[1] = max pairs of any walker seen, status[2] = max e-n neighbours seen,
 * status[3] = max triplets (sum_m deg(m)^2) seen, status[4] = max changed set of a low-rank step seen,
 * status[5] = ill-conditioned walkers of the last fire_local_energy call (FP32 and mixed, refine_cap > 0);
 * the host grows capacities from these, like StaticScheduler (static_args.py:62-84). */

typedef enum {
  FIRE_PREC_FP32 = 0,  /* FP32 SIMT; value planes by compensated (twice-the-working-precision) dot products, the
                          orbital-matrix values as hi + lo float pairs; orbital LU and inverse in double-FP32
                          (48-bit significand) */
  FIRE_PREC_MIXED = 1, /* derivative planes of the contractions on tensor cores: K <= 256 with every row of A and
                          column of W scaled and split on the grid of its largest value into FP16 hi + lo (the
                          hi x hi sums exact in one FP32 accumulator, the three other products in a second, four
                          MMAs per product; ~2^-20 of a row's largest value per element), K > 256 (the envelope rows) in split BF16 (three products per
                          FP32 product); value planes, orbital LU and inverse as in FIRE_PREC_FP32 */
  FIRE_PREC_FP64 = 2   /* everything in FP64 (validation build of the same kernels) */
} fire_precision;

typedef struct {
  int32_t n_el;          /* electrons per walker */
  int32_t n_up;          /* spin-up electrons (the first n_up) */
  int32_t n_nuc;         /* nuclei */
  int32_t n_walkers;     /* walkers in this call */
  float cutoff;          /* e-e neighbour cutoff (bohr), embedding.new.cutoff */
  float cutoff_1el;      /* e-n neighbour cutoff (bohr), embedding.new.cutoff_1el */
  int32_t cap_pairs;     /* capacity: directed e-e pairs per walker (same + diff) */
  int32_t cap_nuc;       /* capacity: e-n neighbours per electron */
  int32_t precision;     /* fire_precision */
  int32_t chunk_walkers; /* walkers per internal pass; 0 = choose from the workspace */
  int32_t refine_cap;    /* FP32 / mixed fire_local_energy: at most this many ill-conditioned walkers per call are
                            evaluated again with FP64 orbital-matrix values (see fire_local_energy); 0 = none */
  float refine_ratio;    /* a walker is ill-conditioned when (|lap| + |grad|^2) / 2 > refine_ratio |E_loc|
                            (<= 0: FIRE_REFINE_RATIO) */
  float refine_kappa;    /* ... or when its determinant-weighted condition number
                            sum_d |w_d| kappa_F(A_d) / |sum_d w_d| exceeds refine_kappa (<= 0: FIRE_REFINE_KAPPA) */
  float refine_ks;       /* ... or when (|lap| + |grad|^2) / 2 exceeds refine_ks Hartree (<= 0: FIRE_REFINE_KS) */
  float refine_kscond;   /* ... or when (|lap| + |grad|^2) / 2 times that condition number exceeds refine_kscond Hartree
                            (<= 0: FIRE_REFINE_KSCOND) */
} fire_problem;

/* Defaults of the ill-conditioned test.  After compensation the FP32 value planes move E_loc by ~1e-7 of the
 * kinetic terms (|lap| + |grad|^2) / 2, randomly signed: the walkers above FIRE_REFINE_KS carry errors of a few mHa
 * and dominate the error of a batch mean, the walkers above FIRE_REFINE_RATIO |E_loc| (near a node) the relative
 * error of their own E_loc. */
#define FIRE_REFINE_RATIO 100.0f
#define FIRE_REFINE_KAPPA 1.0e6f
#define FIRE_REFINE_KS 1.0e5f
/* The compensated value planes leave E_loc errors of ~(1-4)e-12 (|lap| + |grad|^2) / 2 kappa on C40H82 walkers
 * (kappa the determinant-weighted condition number): the product bound catches the walkers whose terms and
 * conditioning are each below their own bound but whose error is several mHa. */
#define FIRE_REFINE_KSCOND 1.0e10f

/* Parameter slots of the flat parameter blob (float32), in blob order.  Shapes with
 * F = 256, D = 4 determinants, n = n_el, N = n_nuc are given by fire_param_layout. */
enum fire_param_slot {
  FIRE_P_EN_SCALES, FIRE_P_EN_KERNEL, FIRE_P_EN_BIAS, FIRE_P_EN_NUC_EMB,
  FIRE_P_EI_DIR_W, FIRE_P_EI_DIR_B, FIRE_P_EI_ENV_W, FIRE_P_EI_GAMMA_W, FIRE_P_EI_EDGE_W,
  FIRE_P_EI_LN_SCALE, FIRE_P_EI_LN_BIAS, FIRE_P_EI_GLU_W, FIRE_P_EI_DENSE_W, FIRE_P_EI_DENSE_B,
  FIRE_P_EI_OUT_W, FIRE_P_EI_OUT_B,
  FIRE_P_EESAME_SCALE, FIRE_P_EESAME_KERNEL, FIRE_P_EESAME_BIAS, FIRE_P_EESAME_DIR_W,
  FIRE_P_EESAME_DIR_B, FIRE_P_EESAME_ENV_W, FIRE_P_EESAME_GAMMA_W, FIRE_P_EESAME_EDGE_W,
  FIRE_P_EESAME_EDGE_B,
  FIRE_P_EEDIFF_SCALE, FIRE_P_EEDIFF_KERNEL, FIRE_P_EEDIFF_BIAS, FIRE_P_EEDIFF_DIR_W,
  FIRE_P_EEDIFF_DIR_B, FIRE_P_EEDIFF_ENV_W, FIRE_P_EEDIFF_GAMMA_W, FIRE_P_EEDIFF_EDGE_W,
  FIRE_P_EEDIFF_EDGE_B,
  FIRE_P_UPD1_W, FIRE_P_UPD1_B, FIRE_P_UPD2_W, FIRE_P_UPD2_B, FIRE_P_SCALES, FIRE_P_CUTOFF_PARAM,
  FIRE_P_ORB_UP_W, FIRE_P_ORB_UP_B, FIRE_P_ORB_DN_W, FIRE_P_ORB_DN_B,
  FIRE_P_ENV_UP_SIGMA, FIRE_P_ENV_UP_PI, FIRE_P_ENV_DN_SIGMA, FIRE_P_ENV_DN_PI,
  FIRE_P_CUSP,
  FIRE_P_JMLP1_W, FIRE_P_JMLP1_B, FIRE_P_JMLP2_W, FIRE_P_JMLP2_B, FIRE_P_JMLP3_W, FIRE_P_JMLP3_B,
  FIRE_P_MLP_SCALE, FIRE_P_LOG_BIAS,
  FIRE_P_ATT_KEYS, FIRE_P_ATT_Q_W, FIRE_P_ATT_Q_B, FIRE_P_ATT_V_W, FIRE_P_ATT_V_B,
  FIRE_P_ATT_OUT1_W, FIRE_P_ATT_OUT1_B, FIRE_P_ATT_OUT2_W, FIRE_P_ATT_OUT2_B,
  FIRE_P_ATT_OUT3_W, FIRE_P_ATT_OUT3_B, FIRE_P_ATT_SCALE, FIRE_P_ATT_BIAS,
  FIRE_P_COUNT
};

/* ---- sizes (host functions, no device work) -------------------------------------------------- */
int32_t fire_abi_version(void);

/* offsets[FIRE_P_COUNT + 1] (host): element offset of every slot, 64-element aligned;
 * offsets[FIRE_P_COUNT] = total blob length.  Mirrors the MoonLikeParams tree
 * (model/wave_function.py:54-57) flattened. */
fire_status fire_param_layout(const fire_problem* prob, int64_t* offsets);

/* bytes of the prepared-parameter buffer (derived weights: folded scales, fused attention
 * query/key weights, BF16 copies for the mixed path, FP64 copies for the refinement pass of the FP32 and
 * mixed local energy). */
fire_status fire_prepared_size(const fire_problem* prob, size_t* bytes);

/* bytes of workspace needed to process `chunk` walkers per pass (chunk <= 0: the whole batch). */
fire_status fire_workspace_size(const fire_problem* prob, int32_t chunk, size_t* bytes);

/* ---- parameters ------------------------------------------------------------------------------- */
/* Builds the prepared buffer from the float32 blob (device) and its offsets (host array). */
fire_status fire_prepare_params(void* stream, const fire_problem* prob, const float* blob,
                                const int64_t* offsets_host, void* prepared, size_t prepared_bytes);

/* ---- neighbour lists (bit-exact with get_pair_indices) ----------------------------------------- */
typedef struct {
  /* each may be NULL; per walker, padded with FIRE_NO_NEIGHBOUR (jac_* padding: n_el + P) */
  int32_t* ct_same; int32_t* nb_same; int32_t* jac_same; /* [B, cap_same] */
  int32_t* ct_diff; int32_t* nb_diff; int32_t* jac_diff; /* [B, cap_diff] */
  int32_t* jac_ctr; int32_t* jac_dep;                    /* [B, n_el + cap_same + cap_diff] */
  int32_t* en_idx;                                       /* [B, n_el, cap_nuc] */
  int32_t* counts;  /* [B, 4]: n_pairs_same, n_pairs_diff, n_triplets, n_neighbours_en */
  int32_t cap_same, cap_diff;
} fire_neighbor_out;

/* r: [B, n_el, 3] float32 (float64 when prob->precision == FIRE_PREC_FP64); R: [n_nuc, 3] float32 */
fire_status fire_neighbors(void* stream, const fire_problem* prob, const void* r, const float* R,
                           const fire_neighbor_out* out, int32_t* status);

/* Triplet index quadruples (in, k, kn, i) in _get_triplet_indices order, [B, cap_triplets] each,
 * total per walker n_el + 2P + sum_m deg(m)^2 (padded with FIRE_NO_NEIGHBOUR). */
fire_status fire_triplets(void* stream, const fire_problem* prob, const void* r, int32_t cap_triplets,
                          int32_t* trip_in, int32_t* trip_k, int32_t* trip_kn, int32_t* trip_i,
                          void* workspace, size_t workspace_bytes, int32_t* status);

/* Same outputs as fire_triplets, with no workspace argument and no allocation: the intermediate
 * neighbour structure lives in a static device array of FIRE_TRIPLETS_STATIC_MAX_WORDS int32 words
 * (16 MiB) per device.  No counterpart in the reference.  It serves callers that cannot allocate or
 * pass device scratch (a handler inside another runtime's executable, a host program without a memory
 * pool).  Needs n_walkers * (2 * n_el + 1 + 2 * cap_pairs) <= FIRE_TRIPLETS_STATIC_MAX_WORDS, else
 * FIRE_ERR_UNSUPPORTED before any CUDA call.  The first call on a device (that device current) looks
 * the array up with cudaGetSymbolAddress; make it before any stream capture.  The address is cached with
 * the CUDA context it belongs to: after cudaDeviceReset (or a new primary context) the next call looks it
 * up again, so make that call before any stream capture too.  The stream must belong
 * to the current device.  Calls that can overlap on one device (other streams, other host threads)
 * race on the shared array; calls ordered on one stream do not. */
#define FIRE_TRIPLETS_STATIC_MAX_WORDS (4 * 1024 * 1024)
fire_status fire_triplets_static(void* stream, const fire_problem* prob, const void* r, int32_t cap_triplets,
                                 int32_t* trip_in, int32_t* trip_k, int32_t* trip_kn, int32_t* trip_i,
                                 int32_t* status);

/* ---- wavefunction ----------------------------------------------------------------------------- */
/* sign, logpsi: [B] in the walkers' dtype */
fire_status fire_logpsi(void* stream, const fire_problem* prob, const float* R, const float* Z,
                        const void* prepared, const void* r, void* sign, void* logpsi,
                        void* workspace, size_t workspace_bytes, int32_t* status);

/* Per-walker gradient of log|psi| with respect to every parameter: the rows of the Jacobian that the dense SPRING
 * preconditioner contracts (preconditioner.py:185-191 jax.grad of log_p vmapped over the walkers, called from
 * update.py:177-191).  grad: [B, L] in the walkers' dtype with L = offsets[FIRE_P_COUNT] of fire_param_layout;
 * walker w's derivative with respect to blob element k is grad[w * L + k] (the padding between slots is 0).
 * sign, logpsi: [B] as fire_logpsi.  Reverse mode through the value path on the CUDA cores, the orbital matrices
 * inverted in double-FP32 (FP64 in the FP64 build); FIRE_PREC_MIXED computes it as FIRE_PREC_FP32.  The workspace
 * is sized by fire_logpsi_grad_workspace_size (walkers per pass: prob->chunk_walkers, else as many as fit). */
fire_status fire_logpsi_grad_workspace_size(const fire_problem* prob, int32_t chunk, size_t* bytes);
fire_status fire_logpsi_grad(void* stream, const fire_problem* prob, const float* R, const void* prepared,
                             const void* r, void* sign, void* logpsi, void* grad, void* workspace,
                             size_t workspace_bytes, int32_t* status);

/* Optional intermediate outputs of fire_local_energy (any pointer may be NULL). */
typedef struct {
  void* kinetic;   /* [B] */
  void* potential; /* [B] */
  double* logdet;  /* [B, 4] */
  double* sign_det;/* [B, 4] */
  void* jastrow;   /* [B] log Jastrow value */
  void* grad;      /* [B, n_el, 3] gradient of log|psi| */
  void* lap;       /* [B] Laplacian of log|psi| */
  int32_t* refined;/* [B] 1 for the walkers the refinement pass evaluated again, else 0 */
  double* cond;    /* [B] sum_d |w_d| kappa_F(A_d) / |sum_d w_d| of the first pass (w_d the signed determinant
                      weights, kappa_F = ||A||_F ||A^-1||_F of orbital matrix d); 0 in the FP64 build */
} fire_eloc_debug;

/* logpsi, sign, e_loc: [B] in the walkers' dtype (may be NULL except e_loc);
 * e_stats: [2] float64 = (mean, std) of e_loc over the batch (may be NULL).
 * Up to 798 electrons (the orbital matrices are eliminated in shared memory); larger problems return
 * FIRE_ERR_UNSUPPORTED, here and in fire_logpsi and the Metropolis blocks.
 * FP32 and mixed precision: near a node of psi, E_loc is the small difference of two large terms
 * (lap log psi and |grad log psi|^2), and the FP32 rounding of the value planes that lead to the orbital
 * matrices moves it by up to ~2e-6 of their size; an orbital matrix of large condition number amplifies that
 * rounding in the same way.  A walker whose (|lap| + |grad|^2) / 2 exceeds refine_ratio |E_loc| or refine_ks, whose
 * determinant-weighted condition number (debug->cond) exceeds refine_kappa, or whose E_loc is not finite is
 * ill-conditioned: with refine_cap > 0, up to refine_cap of them are evaluated once more after the batch, with
 * the values of the embedding, orbitals, envelopes and orbital matrices, their LU and inverse in FP64 (the
 * derivative planes on the FP32 CUDA cores), and their results replace the first ones.  status[5] reports how
 * many walkers were ill-conditioned; more than refine_cap sets FIRE_FLAG_REFINE_OVERFLOW (the others keep their
 * first results).  The workspace must then hold the refinement pass as well (fire_workspace_size does). */
fire_status fire_local_energy(void* stream, const fire_problem* prob, const float* R, const float* Z,
                              const void* prepared, const void* r, void* logpsi, void* sign,
                              void* e_loc, double* e_stats, const fire_eloc_debug* debug,
                              void* workspace, size_t workspace_bytes, int32_t* status);

/* Embedding value path for initialisation and stage checks:
 * h_contract [B, n, 256] = h0 + messages (before the first normalize scale),
 * h_update [B, n, 256] = SparseMLP(h_contract * scales[0]) (before scales[1]). Either may be NULL. */
fire_status fire_embedding(void* stream, const fire_problem* prob, const float* R, const void* prepared,
                           const void* r, void* h_contract, void* h_update, void* workspace,
                           size_t workspace_bytes, int32_t* status);

/* Metropolis block of all-electron Gaussian moves (mcmc.py:38-97).
 * r [B, n, 3] and logpsi [B] are updated in place (logpsi must hold log|psi(r)| on entry).
 * Proposals: r' = r + width * eps.  eps and u come from Philox4x32-10 keyed by (seed, counter,
 * step, walker) unless replay_noise [steps, B, n, 3] and replay_log_u [steps, B] are given.
 * n_accept [B] int32 (accepted moves per walker), may be NULL.
 * static_max [4] int32: max over steps/walkers of (n_pairs_same, n_pairs_diff, 0, n_neighbours_en)
 * of the proposals (the laplacian=False statics of mcmc.py:290-294), may be NULL. */
fire_status fire_mcmc_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                            const void* prepared, void* r, void* logpsi, int32_t steps, float width,
                            uint64_t seed, uint64_t counter, const void* replay_noise,
                            const void* replay_log_u, int32_t* n_accept, int32_t* static_max,
                            void* workspace, size_t workspace_bytes, int32_t* status);

/* Metropolis block of single-electron Gaussian moves: proposal_single_electron (mcmc.py:100-111) as run by
 * mcmc_steps_low_rank (mcmc.py:196-275).  Step s (0 <= s < steps) moves electron (step_offset + s) mod n of
 * every walker by width * eps, eps [3] ~ N(0, 1), and accepts if 2 (log|psi'| - log|psi|) > log u.
 * log|psi'| is a full value-path evaluation of the proposed configuration (the reference reaches the same
 * value by a low-rank update of a cached state, checked against the full evaluation in its
 * tests/test_low_rank.py:29-61; fire_mcmc_low_rank_block is that variant, this one costs a full evaluation
 * per step).
 * Draws from Philox4x32-10 keyed by (seed, counter, step, walker) unless replay_noise [steps, B, 3] and
 * replay_log_u [steps, B] are given.  Other arguments and outputs as fire_mcmc_block. */
fire_status fire_mcmc_single_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                                   const void* prepared, void* r, void* logpsi, int32_t steps, int32_t step_offset,
                                   float width, uint64_t seed, uint64_t counter, const void* replay_noise,
                                   const void* replay_log_u, int32_t* n_accept, int32_t* static_max,
                                   void* workspace, size_t workspace_bytes, int32_t* status);

/* Metropolis block of cluster updates: proposal_cluster_update (mcmc.py:119-161) as run by mcmc_steps_low_rank
 * (make_mcmc "cluster-update", mcmc.py:305-316).  Step s picks a center electron, (step_offset + s) mod n
 * (random_sweep = 0) or uniformly at random, and moves the k = min(max_cluster_size, n) electrons closest to it
 * (ties: lower index first) that lie within max_cluster_radius by width * eps (noise row i to the i-th closest);
 * of 5 draws the first whose moved center has the same closest set is proposed, else the step is rejected
 * (proposal log ratio log(0)).  log|psi'| is a full value-path evaluation.  Draws per step and walker: u_center,
 * then eps [5][k][3] (Philox4x32-10 keyed by (seed, counter, step, walker), or replay_draws [steps, B, 1 + 15 k]
 * with replay_log_u [steps, B]).  max_cluster_size <= 16.  Other arguments and outputs as fire_mcmc_block. */
fire_status fire_mcmc_cluster_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                                    const void* prepared, void* r, void* logpsi, int32_t steps, int32_t step_offset,
                                    float width, int32_t max_cluster_size, float max_cluster_radius,
                                    int32_t random_sweep, uint64_t seed, uint64_t counter,
                                    const void* replay_draws, const void* replay_log_u, int32_t* n_accept,
                                    int32_t* static_max, void* workspace, size_t workspace_bytes,
                                    int32_t* status);

/* Metropolis block of jumps to the nuclei: proposal_jump_to_atom (mcmc.py:164-193) as run by
 * mcmc_steps_low_rank for make_mcmc's jump_steps (mcmc.py:320-326).  Each step moves one random electron of
 * every walker to R_I + sigma * eps, nucleus I drawn with probability Z_I / sum Z, and accepts if
 * log(q(r_old) / q(r_new)) + 2 (log|psi'| - log|psi|) > log u, q(x) = sum_J Z_J exp(-|x - R_J|^2 / (2 sigma^2));
 * log|psi'| is a full value-path evaluation.  Draws per step and walker (u_electron, u_nucleus, eps[3]) from
 * Philox4x32-10 keyed by (seed, counter, step, walker), unless replay_draws [steps, B, 5] and replay_log_u
 * [steps, B] are given: electron = min(floor(u_electron n), n - 1), nucleus = the first J whose cumulative
 * charge exceeds u_nucleus sum Z.  Other arguments and outputs as fire_mcmc_block. */
fire_status fire_mcmc_jump_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                                 const void* prepared, void* r, void* logpsi, int32_t steps, float sigma,
                                 uint64_t seed, uint64_t counter, const void* replay_draws,
                                 const void* replay_log_u, int32_t* n_accept, int32_t* static_max,
                                 void* workspace, size_t workspace_bytes, int32_t* status);

/* Workspace of fire_mcmc_low_rank_block for `chunk` walkers per pass and a changed set of at most cap_changed
 * electrons per walker and step (cap_changed <= 128, else FIRE_ERR_UNSUPPORTED). */
fire_status fire_low_rank_workspace_size(const fire_problem* prob, int32_t chunk, int32_t cap_changed,
                                         size_t* bytes);

/* Metropolis block of single-electron moves evaluated by the low-rank update of a cached state:
 * mcmc_steps_low_rank (mcmc.py:196-275) with proposal_single_electron (mcmc.py:100-111) and
 * log_psi_with_state / log_psi_low_rank_update (model/wave_function.py:226-287).  Per chunk of walkers the state
 * comes from one value-path evaluation (log|psi| of r is written to logpsi) and keeps the inverse of every
 * orbital matrix.  Step s moves electron e = (step_offset + s) mod n; the changed set is e and every electron
 * within the cutoff of e before or after the move (get_low_rank_pair_indices, model/new_sparse_model.py:439-474).
 * Their embeddings, raw orbital and Jastrow rows are recomputed, e's ElecInit and envelope rows, and log|psi'|
 * follows from the determinant lemma det(A') = det(A) det(I + V A^-1[:, S]) with the Jastrow sums over all rows;
 * an accepted step writes the rows into the state and updates the inverses by the Woodbury identity
 * (model/utils.py:216-245).  Proposals, draws, acceptance, replay and n_accept as fire_mcmc_single_block.
 * static_max [7] int32: (n_pairs_same, n_pairs_diff, 0, n_neighbours_en) of the proposals, then the move statics
 * (n_changed_hout, n_changed_pair_same, n_changed_pair_diff) of get_static_input (model/new_sparse_model.py:414-424).
 * A changed set larger than cap_changed sets FIRE_FLAG_CHANGED_OVERFLOW (status[4] = the largest set seen) and
 * rejects that proposal: the caller reruns the block with a larger capacity.  Up to 798 electrons. */
fire_status fire_mcmc_low_rank_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                                     const void* prepared, void* r, void* logpsi, int32_t steps, int32_t step_offset,
                                     float width, int32_t cap_changed, uint64_t seed, uint64_t counter,
                                     const void* replay_noise, const void* replay_log_u, int32_t* n_accept,
                                     int32_t* static_max, void* workspace, size_t workspace_bytes, int32_t* status);

/* Effective core potentials of the pseudised nuclei (make_pseudopotential, pseudopotentials.py:411-457): the
 * channels on the radial grid as eval_ecp_on_grid (pseudopotentials.py:149-202) tabulates them.  Device arrays. */
typedef struct {
  int32_t n_ecp;          /* pseudised nuclei */
  int32_t n_grid;         /* radial grid points */
  int32_t n_l;            /* non-local channels l = 0 .. n_l - 1 (n_l <= 4) */
  int32_t max_quad;       /* host copy of the largest n_quad */
  const int32_t* atom;    /* [n_ecp] nucleus index of each pseudised nucleus */
  const double* grid;     /* [n_grid] ascending radii */
  const double* v_loc;    /* [n_ecp, n_grid] local channel */
  const double* v_nl;     /* [n_ecp, n_l, n_grid] non-local channels */
  const double* cutoff;   /* [n_ecp] radius beyond which the non-local channels are neglected */
  const int32_t* n_quad;  /* [n_ecp] quadrature points of each nucleus's sphere: 1, 2, 4, 6 or 12 */
} fire_ecp;

/* Metropolis block of jumps to the nuclei (proposal_jump_to_atom, mcmc.py:164-193, with its log ratio in the test)
 * evaluated by the low-rank update of a cached state: the proposals, draws and replay of fire_mcmc_jump_block,
 * each walker moving its own electron; state, capacity, workspace and static_max [7] as fire_mcmc_low_rank_block. */
fire_status fire_mcmc_low_rank_jump_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                                          const void* prepared, void* r, void* logpsi, int32_t steps, float sigma,
                                          int32_t cap_changed, uint64_t seed, uint64_t counter,
                                          const void* replay_draws, const void* replay_log_u, int32_t* n_accept,
                                          int32_t* static_max, void* workspace, size_t workspace_bytes,
                                          int32_t* status);

/* Metropolis block of cluster updates (proposal_cluster_update, mcmc.py:119-161, make_mcmc "cluster-update",
 * mcmc.py:305-316) evaluated by the low-rank update of a cached state: the proposals, draws and replay of
 * fire_mcmc_cluster_block, the moved set being the cluster's index list (the center's k closest electrons, those
 * beyond max_cluster_radius padded, whose padding enters the move statics like an out-of-range JAX gather: as
 * electron n - 1).  State, capacity, workspace and static_max [7] as fire_mcmc_low_rank_block. */
fire_status fire_mcmc_low_rank_cluster_block(void* stream, const fire_problem* prob, const float* R, const float* Z,
                                             const void* prepared, void* r, void* logpsi, int32_t steps,
                                             int32_t step_offset, float width, int32_t max_cluster_size,
                                             float max_cluster_radius, int32_t random_sweep, int32_t cap_changed,
                                             uint64_t seed, uint64_t counter, const void* replay_draws,
                                             const void* replay_log_u, int32_t* n_accept, int32_t* static_max,
                                             void* workspace, size_t workspace_bytes, int32_t* status);

/* The unit-sphere quadrature of n_points (1, 2, 4, 6 or 12) points fire_ecp_energy uses (make_spherical_grid,
 * pseudopotentials.py:44-133), points [n_points, 3] (host, float64); equal weights 1 / n_points.  Host only. */
fire_status fire_ecp_quadrature(int32_t n_points, double* points);

/* Pseudopotential energy of every walker, e_ecp [B] in the walkers' dtype.  The local term is summed over
 * electrons and pseudised nuclei (make_local_pseudopotential, pseudopotentials.py:205-219).  For the non-local
 * term (make_nonlocal_pseudopotential, :337-398), each electron within the cutoff of its closest pseudised nucleus
 * is moved to that nucleus's quadrature points (build_all_integration_points, :272-334), on a sphere through the
 * electron, rotated at random per walker and electron.  The sum is over l of v_l(d) w (2l + 1) P_l(cos theta)
 * psi'/psi, the ratios from the low-rank update of a cached state as in fire_mcmc_low_rank_block.  Rotations: the
 * columns of the Gram-Schmidt basis of two normal 3-vectors (random_rot_mat, :222-228) from Philox4x32-10 keyed by
 * (seed, counter, walker, electron), unless replay_rotations [B, n, 3, 3] (walkers' dtype, rot[x][y]) is given.
 * The Coulomb potential with the effective charges and the kinetic energy come from fire_local_energy called with
 * Z = the effective charges.  cap_changed, workspace (fire_low_rank_workspace_size) and static_max [7] as
 * fire_mcmc_low_rank_block. */
fire_status fire_ecp_energy(void* stream, const fire_problem* prob, const float* R, const float* Z,
                            const void* prepared, const void* r, const fire_ecp* ecp, int32_t cap_changed,
                            uint64_t seed, uint64_t counter, const void* replay_rotations, void* e_ecp,
                            int32_t* static_max, void* workspace, size_t workspace_bytes, int32_t* status);

/* Coulomb potential of every walker (hamiltonian.py:15-26): out [B] in the walkers' dtype. */
fire_status fire_potential_energy(void* stream, const fire_problem* prob, const void* r,
                                  const float* R, const float* Z, void* out);

/* ---- diagnostics (no counterpart in the reference) ----------------------------------------------- */
/* Per-stage device timing: while enabled, every stage and every contraction (GEMM) launch of the calls
 * above is bracketed by CUDA events on its stream.  fire_profile_enable(1) clears the records;
 * fire_profile_report waits for the recorded events and writes one line per stage,
 * "<stage> <launches> <total_ms>\n", into buf (host memory, NUL-terminated, truncated to len). */
fire_status fire_profile_enable(int32_t on);
fire_status fire_profile_report(char* buf, size_t len);

/* The mixed-precision tensor-core contraction alone: C[M, N] = A[M, K] W[K, N] (all float32, row-major,
 * device), on tcgen05.  K <= 256: rows of A and columns of W scaled and split on the grid of their largest
 * value into FP16 hi + lo, the hi x hi sums exact in one FP32 accumulator and the three other products in a second;
 * K > 256: elementwise split BF16, three BF16 products per element pair, one FP32 accumulator.  workspace: the
 * split weights, 32768 * ceil(N / 128) * ceil(K / 64) + 4 * N bytes for K <= 256 (tiles, column scales),
 * else 4 * N * K bytes.  K % 8 == 0, N % 4 == 0
 * and 16-byte aligned A and C (else FIRE_ERR_UNSUPPORTED); K > 256 streams the weights through the
 * pipeline instead of keeping them in shared memory. */
fire_status fire_gemm_mixed(void* stream, int32_t M, int32_t N, int32_t K, const float* A, const float* W, float* C,
                            void* workspace, size_t workspace_bytes, int32_t* status);

#ifdef __cplusplus
}
#endif
#endif /* FIRE_H */
