// fire_ecp.cu -- effective core potentials of the pseudised nuclei (pseudopotentials.py).
//
//  k_ecp_local  the local term: sum over electrons and pseudised nuclei of the local channel interpolated on the
//               radial grid (make_local_pseudopotential, 205-219).
//  k_ecp_point  quadrature point k of electron e for every walker: the electron moved onto the sphere through it
//               around its closest pseudised nucleus, rotated per walker and electron (get_integration_points /
//               build_all_integration_points, 261-334; random_rot_mat, 222-228); the log|psi| of the moved
//               configuration comes from the low-rank evaluation of fire_lowrank.cu.
//  k_ecp_accum  the non-local sum over l of v_l(d) w (2l + 1) P_l(cos theta) psi'/psi (make_nonlocal_pseudopotential,
//               337-398).
//  k_ecp_store  the accumulated energy into the caller's array.
#include "fire_internal.cuh"
#include "fire_philox.cuh"

namespace fire {

// Linear interpolation on an ascending grid, clamped to the end values outside it (jnp.interp).
__device__ __forceinline__ double ecp_interp(const double* xp, const double* fp, int m, double x) {
  if (!(x > xp[0])) return fp[0];
  if (x >= xp[m - 1]) return fp[m - 1];
  int lo = 0, hi = m - 1;  // xp[lo] < x < xp[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (xp[mid] <= x) lo = mid; else hi = mid;
  }
  const double slope = (fp[lo + 1] - fp[lo]) / (xp[lo + 1] - xp[lo]);
  return slope * (x - xp[lo]) + fp[lo];
}

// acc[w] = sum_i sum_a v_loc[a](|r_i - R_atom[a]|) (FP64).  One CTA (256 threads) per walker of the chunk.
template <typename T>
__global__ void __launch_bounds__(256) k_ecp_local(const T* __restrict__ r, int n, const float* __restrict__ R,
                                                   fire_ecp ecp, double* __restrict__ acc) {
  __shared__ double red[32];
  const int w = blockIdx.x;
  double s = 0.0;
  for (int q = threadIdx.x; q < n * ecp.n_ecp; q += blockDim.x) {
    const int i = q / ecp.n_ecp, a = q - i * ecp.n_ecp, I = ecp.atom[a];
    const T* ri = r + ((size_t)w * n + i) * 3;
    const double dx = (double)ri[0] - R[3 * I], dy = (double)ri[1] - R[3 * I + 1], dz = (double)ri[2] - R[3 * I + 2];
    s += ecp_interp(ecp.grid, ecp.v_loc + (size_t)a * ecp.n_grid, ecp.n_grid, sqrt(dx * dx + dy * dy + dz * dz));
  }
  double v[1] = {s};
  block_sum<double, 1>(v, red);
  if (threadIdx.x == 0) acc[w] = v[0];
}

// Quadrature point k of electron e for every walker of the chunk; one CTA (128 threads) per walker.  rn = r, and
// when e lies within the cutoff of its closest pseudised nucleus a (d = |r_e - R_a|, ties to the lower index) and
// a's grid has more than k points, electron e of rn moves to R_a + d (g_k rot), rot the walker's rotation for e:
// replay [B][n][3][3] (rot[x][y]) or the Gram-Schmidt columns of two normal 3-vectors from Philox4x32-10.
// pt [W][4] (double): the point's weight 1 / n_quad (0 when inactive), cos theta between g_k rot and r_e - R_a,
// d, a; moved [W] = e for the low-rank evaluation.
template <typename T>
__global__ void __launch_bounds__(128) k_ecp_point(const T* __restrict__ r, T* __restrict__ rn, int n, int e, int k,
                                                   const float* __restrict__ R, fire_ecp ecp, EcpQuad qt, int w0,
                                                   uint64_t seed, uint64_t counter, const T* __restrict__ replay,
                                                   double* __restrict__ pt, int* __restrict__ moved) {
  const int w = blockIdx.x;
  const long gw = w0 + w;
  const T* src = r + (size_t)w * 3 * n;
  T* dst = rn + (size_t)w * 3 * n;
  for (int q = threadIdx.x; q < 3 * n; q += blockDim.x) dst[q] = src[q];
  __syncthreads();
  if (threadIdx.x != 0) return;
  moved[w] = e;
  const double ex = src[3 * e], ey = src[3 * e + 1], ez = src[3 * e + 2];
  int ab = 0;
  double db = 0.0;
  for (int a = 0; a < ecp.n_ecp; ++a) {
    const int I = ecp.atom[a];
    const double dx = ex - R[3 * I], dy = ey - R[3 * I + 1], dz = ez - R[3 * I + 2];
    const double d = sqrt(dx * dx + dy * dy + dz * dz);
    if (a == 0 || d < db) {
      ab = a;
      db = d;
    }
  }
  double* o = pt + (size_t)w * 4;
  const int nq = ecp.n_quad[ab];
  o[2] = db;
  o[3] = ab;
  if (!(db < ecp.cutoff[ab]) || k >= nq) {
    o[0] = 0.0;
    o[1] = 0.0;
    return;
  }
  double rot[3][3];
  if (replay) {
    const T* q = replay + ((size_t)gw * n + e) * 9;
    for (int x = 0; x < 3; ++x)
      for (int y = 0; y < 3; ++y) rot[x][y] = (double)q[3 * x + y];
  } else {
    double u[6];
    for (int h = 0; h < 2; ++h) {
      // own counter domain (0xFFFFFFF0, 0xFFFFFFEF): the proposals use 0xFFFFFFFB .. 0xFFFFFFFF
      uint32_t ctr[4] = {(uint32_t)e, (uint32_t)gw, 0xFFFFFFF0u - (uint32_t)h, (uint32_t)counter};
      philox10(ctr, seed ^ (counter >> 32) * 0x9E3779B97F4A7C15ull);
      const double r1 = sqrt(-2.0 * log(u01(ctr[0]))), t1 = 6.283185307179586 * u01(ctr[1]);
      const double r2 = sqrt(-2.0 * log(u01(ctr[2]))), t2 = 6.283185307179586 * u01(ctr[3]);
      u[3 * h] = r1 * cos(t1);
      u[3 * h + 1] = r1 * sin(t1);
      u[3 * h + 2] = r2 * cos(t2);
    }
    double v1[3] = {u[0], u[1], u[2]}, v2[3] = {u[3], u[4], u[5]};
    const double n1 = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
    for (int x = 0; x < 3; ++x) v1[x] /= n1;
    const double pr = v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2];
    for (int x = 0; x < 3; ++x) v2[x] -= v1[x] * pr;
    const double n2 = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
    for (int x = 0; x < 3; ++x) v2[x] /= n2;
    const double v3[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
    for (int x = 0; x < 3; ++x) {
      rot[x][0] = v1[x];
      rot[x][1] = v2[x];
      rot[x][2] = v3[x];
    }
  }
  const double* g = qt.p[ecp_quad_row(nq) + k];
  const int I = ecp.atom[ab];
  const double ux = (ex - R[3 * I]) / db, uy = (ey - R[3 * I + 1]) / db, uz = (ez - R[3 * I + 2]) / db;
  double gr[3];
  for (int y = 0; y < 3; ++y) gr[y] = g[0] * rot[0][y] + g[1] * rot[1][y] + g[2] * rot[2][y];
  for (int y = 0; y < 3; ++y) dst[3 * e + y] = (T)((double)R[3 * I + y] + db * gr[y]);
  o[0] = 1.0 / nq;
  o[1] = gr[0] * ux + gr[1] * uy + gr[2] * uz;
}

// acc[w] += sum_l v_l(d) (2l + 1) P_l(cos theta) w psi'/psi for the walkers whose point is active, psi'/psi =
// sgn' sgn exp(logpsi' - logpsi).  One thread per walker of the chunk.
template <typename T>
__global__ void k_ecp_accum(int Wc, const double* __restrict__ pt, const T* __restrict__ lpn,
                            const T* __restrict__ sgn_n, const T* __restrict__ lp0, const T* __restrict__ sgn0,
                            fire_ecp ecp, double* __restrict__ acc) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= Wc) return;
  const double* o = pt + (size_t)w * 4;
  if (!(o[0] > 0.0)) return;
  const double ratio = (double)sgn_n[w] * (double)sgn0[w] * exp((double)lpn[w] - (double)lp0[w]);
  const int a = (int)o[3];
  const double c = o[1], d = o[2];
  const double P[4] = {1.0, c, 0.5 * (3.0 * c * c - 1.0), 0.5 * (5.0 * c * c * c - 3.0 * c)};
  double s = 0.0;
  for (int l = 0; l < ecp.n_l; ++l)
    s += ecp_interp(ecp.grid, ecp.v_nl + ((size_t)a * ecp.n_l + l) * ecp.n_grid, ecp.n_grid, d) * (2 * l + 1) * P[l];
  acc[w] += s * o[0] * ratio;
}

template <typename T>
__global__ void k_ecp_store(int Wc, int w0, const double* __restrict__ acc, T* __restrict__ out) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w < Wc) out[w0 + w] = (T)acc[w];
}

#define FIRE_INST_ECP(T)                                                                                         \
  template __global__ void k_ecp_local<T>(const T*, int, const float*, fire_ecp, double*);                     \
  template __global__ void k_ecp_point<T>(const T*, T*, int, int, int, const float*, fire_ecp, EcpQuad, int,     \
                                          uint64_t, uint64_t, const T*, double*, int*);                        \
  template __global__ void k_ecp_accum<T>(int, const double*, const T*, const T*, const T*, const T*, fire_ecp, \
                                          double*);                                                            \
  template __global__ void k_ecp_store<T>(int, int, const double*, T*);
FIRE_INST_ECP(float)
FIRE_INST_ECP(double)

}  // namespace fire
