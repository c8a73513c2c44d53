// fire_kernels.cuh -- declarations of the kernels defined (and explicitly instantiated) in the
// stage translation units, so that the entry-point files (fire_api.cu, fire_triplets_static.cu) can
// launch them.  Only translation units that define none of these kernels include this header: one that
// sees these declarations before its own template definitions gets launch stubs without device code
// ("invalid device function").
#pragma once
#include "fire_df64.cuh"
#include "fire_internal.cuh"

namespace fire {

// fire_neighbors.cu
template <typename T>
__global__ void k_neighbors(const T* r, const float* R, T cutoff, T cutoff_1el, Nbr nb, fire_neighbor_out ext,
                            int32_t* status);
__global__ void k_triplets(Nbr nb, int cap_t, int32_t* t_in, int32_t* t_k, int32_t* t_kn, int32_t* t_i,
                           int32_t* status);
__global__ void k_pos_scan(Nbr nb, int* pos_off);
__global__ void k_layout(Nbr nb, Layout L);

// fire_embed.cu
template <typename T, int NT>
__global__ void k_elec_init(const T* r, const float* R, Nbr nb, Weights<T> W, T inv_cutoff1, T* E5);
template <typename T, int NT>
__global__ void k_glu(const T* Z, T* out, int G);
template <typename T, int NT>
__global__ void k_silu5(T* Z, int G);
template <typename T, int NT>
__global__ void k_edge_contract(const T* r, Nbr nb, Layout L, Weights<T> W, const T* E5o, T* X, T* Lp, T* Jp);
template <typename T>
__global__ void k_lr_contract(const T* rn, int n, int n_up, T cutoff, const int* moved, int KM, const int* S,
                              const int* S_cnt, int KS, Weights<T> W, const T* E5, const T* E5p, T* HS);

// fire_det.cu
// Orbital Laplacian rows from the plain contraction of the embedding's Laplacian rows (in place):
// lapA = lap_raw env + raw lap_env + 2 sum_xyz raw_jac env_jac  (the product rule of the orbital x envelope).
__global__ void k_orb_lap(float* lapA, const float* env, const float* raw, const float* rjs, long G, int DN);
template <typename T, int NV>
__global__ void k_env_coef(const T* r, const float* R, const T* sp, int n, int n_s, int s_off, int N, int Wn,
                           T* coef);
template <typename S, typename TI, typename TO, bool INV>
__global__ void k_gj_global(const TI* A, const TI* A_lo, int n, S* work, double* logdet, double* sign, double* cond, TO* Ainv,
                            int32_t* status);
constexpr int GJG_BW_DECL = 16, GJG_THREADS_DECL = 512;
template <typename T, int NT, int CLO, int CHI>
__global__ void k_detlap(Nbr nb, Layout L, const T* Jp, const T* Ainv, const T* lapA, double* grad, double* lap,
                         int32_t* status);

// fire_jastrow.cu
__global__ void k_nn_energy(const float* R, const float* Z, int N, double* out);
template <typename T, int NC, int ACT, bool FLM>
__global__ void k_narrow(const T* X, const T* Jp, const T* Lp, Nbr nb, Layout L, const T* Wn, const T* bn,
                         const T* post_scale, const T* post_shift, T* Xo, T* Jo, T* Lo, int32_t* status, T* D1o,
                         T* D2o);
template <typename T, bool FLM>
__global__ void k_mlp_sum(Nbr nb, Layout L, const T* Xo, const T* Jo, const T* Lo, T* ox, T* ol, T* oj);
template <typename T, bool FLM>
__global__ void k_att_sums(Nbr nb, Layout L, const T* aX, const T* aJ, const T* aL, const T* VX, const T* VJ,
                           const T* VL, T* Ax, T* Al, T* AJ);
template <typename T, bool FLM>
__global__ void k_readout_in(int n, const T* Ax, const T* Al, const T* AJ, T* RX, T* RJ, T* RL);
template <typename T, bool FLM>
__global__ void k_assemble(int n, int n_up, int N, int w0, const T* r, const float* R, const float* Z,
                           Weights<T> W, const double* ld, const double* sd, const double* dgrad, const double* dlap,
                           const T* JAx, const T* JAj, const T* JAl, const T* JMx, const T* JMj, const T* JMl,
                           AssembleOut out, int32_t* status);
template <typename T>
__global__ void k_potential(int n, int N, const T* r, const float* R, const float* Z, T* out);
template <typename T>
__global__ void k_stats(const T* e, int B, double* out);

// fire_mcmc.cu
template <typename T>
__global__ void k_propose(const T* r, T* rn, int n, int Wc, int w0, int B, int step, T width, uint64_t seed,
                          uint64_t counter, const T* replay);
template <typename T>
__global__ void k_propose_single(const T* r, T* rn, int n, int w0, int B, int step, int offset, T width,
                                 uint64_t seed, uint64_t counter, const T* replay, int* moved);

template <typename T>
__global__ void k_accept(T* r, const T* rn, T* logpsi, const T* logpsi_new, int n, int w0, int B, int step,
                         uint64_t seed, uint64_t counter, const T* replay_log_u, int32_t* n_accept, const int* counts,
                         int32_t* static_max, const T* plr, int32_t* acc_out);
template <typename T>
__global__ void k_propose_cluster(const T* r, T* rn, T* plr, int n, int w0, int B, int step, int offset, int k,
                                  T radius, T width, int random_sweep, uint64_t seed, uint64_t counter,
                                  const T* replay, int* moved_idx);
template <typename T>
__global__ void k_propose_jump(const T* r, T* rn, T* plr, int n, int w0, int B, int step, const float* R,
                               const float* Z, int N, T sigma, uint64_t seed, uint64_t counter, const T* replay,
                               int* moved);

// fire_lowrank.cu
template <typename T>
__global__ void k_lr_select(const T* r, const T* rn, int n, int n_up, const int* moved, int KM, const float* R, int N,
                            T cutoff, T cutoff_1el, Nbr nb, int KS, int* S, int* S_cnt, T* re_p, int* en_cnt_p,
                            int* en_idx_p, int* counts_p, int32_t* static_max, int32_t* status);
template <typename T>
__global__ void k_lr_env_coef(const T* rn, const float* R, const T* sp_up, const T* sp_dn, const int* moved, int KM,
                              int n, int n_up, int N, int Wc, T* coefU, T* coefD);
template <typename T>
__global__ void k_lr_env_add(long total, T* env_p, const T* env_d);
template <typename T>
__global__ void k_lr_orb(const int* S, const int* S_cnt, int KS, int n_up, int DN, T* rawU, const T* rawD);
template <typename T>
__global__ void k_lr_det(const int* S, const int* S_cnt, int KS, int n, const int* moved, int KM, const T* rawS,
                         const T* env,
                         const T* env_p, const T* Apl, const T* B, const double* ld, const double* sd, T* V,
                         double* Minv, double* ld_p, double* sd_p);
template <typename T>
__global__ void k_lr_jsums(int n, int n_up, const int* S, const int* S_cnt, int KS, const T* aX, const T* vals,
                           const T* Xo, const T* aS, const T* vS, const T* oS, T* Ax, T* JM);
template <typename T>
__global__ void k_lr_commit(const int* accf, const int* S, const int* S_cnt, int KS, int n, const int* moved, int KM,
                            const T* hS,
                            const T* rawS, const T* env_p, const T* aS, const T* vS, const T* oS, const T* E5p,
                            const int* en_cnt_p, const int* en_idx_p, const int* counts_p, const double* ld_p,
                            const double* sd_p, T* h, T* rawx, T* env, T* Apl, T* aX, T* vals, T* Xo, T* E5o, Nbr nb,
                            double* ld, double* sd);
template <typename T>
__global__ void k_lr_wb_z(const int* accf, const int* S_cnt, int KS, int n, const T* B, const T* V, T* Zb);
template <typename T>
__global__ void k_lr_wb_q(const int* accf, const int* S, const int* S_cnt, int KS, int n, const T* B,
                          const double* Minv, T* Qb);
template <typename T>
__global__ void k_lr_wb_apply(const int* accf, const int* S_cnt, int KS, int n, T* B, const T* Zb, const T* Qb);

// fire_ecp.cu
template <typename T>
__global__ void k_ecp_local(const T* r, int n, const float* R, fire_ecp ecp, double* acc);
template <typename T>
__global__ void k_ecp_point(const T* r, T* rn, int n, int e, int k, const float* R, fire_ecp ecp, EcpQuad qt, int w0,
                            uint64_t seed, uint64_t counter, const T* replay, double* pt, int* moved);
template <typename T>
__global__ void k_ecp_accum(int Wc, const double* pt, const T* lpn, const T* sgn_n, const T* lp0, const T* sgn0,
                            fire_ecp ecp, double* acc);
template <typename T>
__global__ void k_ecp_store(int Wc, int w0, const double* acc, T* out);

// fire_tc.cu (host launchers)
cudaError_t split_transpose(const float* W, int K, int N, __nv_bfloat16* hi, __nv_bfloat16* lo, cudaStream_t s);
// cs: FP16 scaled-grid split of every column (hi parts bounded for an exact sum over K), its scale into cs [N];
// nullptr: an elementwise BF16 split
cudaError_t split_tiles(const float* W, int K, int N, __nv_bfloat16* Bt, cudaStream_t s, float* cs);
// value_rows: the value plane only (128 electrons per tile), else the 4 derivative planes (32 electrons per tile)
cudaError_t env_tc(const EnvTcP& p, const __nv_bfloat16* Bt, int32_t* status, cudaStream_t s, bool value_rows);
template <typename T>
struct GemmP;
cudaError_t gemm_tc(int mode, int bn, const GemmP<float>& p, const TcWeights& wt, int* mask_buf, int32_t* status,
                    cudaStream_t s);

}  // namespace fire
