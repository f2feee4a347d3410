// Backward sweep of the discrete adjoint of recorded ESDIRK64 reactor integrations (the forward is
// sf_integrate_record_batch): gradients of the temperature at the end time and of the smoothed ignition delay with
// respect to every reaction's ln A and E_a, and with respect to the initial state, for a whole batch at once.
//
// Reactors are ordered by their step count, longest first, so that backward step m (counted from each reactor's
// last step) works on a prefix of that order: every per-reactor buffer (adjoint state, gradient) keeps one slot per
// reactor across the sweep, no compaction or scatter between steps. Per step m, over the na(m) reactors with more
// than m steps:
//   1. gather the recorded step (h, six stage states) of each reactor;
//   2. right-hand sides and Jacobians at the 6 na stage states (the 32-lane batched chemistry kernel);
//   3. the factors of the transposed implicit stage systems h gamma J_s^T - I, s = 1..5 (one warp per system);
//   4. the clamp mask of the step update (entries the forward step clamped at 0 carry no derivative);
//   5. the stage recursion, backwards over the stages, one warp per reactor for all outputs:
//        c_s = h b_s lam' + sum_{l>s} h a_ls Ybar_l (+ h gamma qd_s),   w_s = solve(h gamma J_s^T - I, -c_s)
//        (w_0 = c_0),   Ybar_s = J_s^T w_s + qd_s,   lam = lam' + sum_s Ybar_s,
//      qd_s the smoothed-delay quadrature term h b_s g'(T_s) e_T;
//   6. the parameter adjoint sum_s w_s^T df/dtheta(Y_s), one rate evaluation per stage state for all outputs.
// The host reads the step counts once; the sweep makes about six launches per step and no synchronization.
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "esdirk64.cuh"
#include "sf_internal.h"
#include "warp_lu.cuh"

namespace sfgb {
namespace {

// smoothed ignition delay: g(T) = 1 - 1 / (1 + exp(-(T - T0 - 400 K) / 20 K))
constexpr double kDtIgn = 400.;
constexpr double kWidth = 20.;
constexpr int kWarps = 4;  // warps per CTA of the LU and stage kernels

struct AdjBufs {
  int n, O, neq, tix, cap;
  const double *rec;
  int *order, *steps;          // sorted: reactor of slot a, its step count
  double *ps, *T0s;            // sorted pressures and initial temperatures
  double *Y6, *K6, *J6, *pres6, *h;
  double *LU, *dinv;  // factors of warp_lu_pd and the reciprocals of their pivots
  int *perm;          // final row permutation of each factorization
  double *lam, *lamp, *W, *Ybar;
  double *grad;                // [n][O][2 nr], sorted slots
  double quad[8];              // 1 for a smoothed-delay output
};

// sorted copies and initial adjoint states
__global__ void k_adj_setup(AdjBufs B, const int *counts, const double *pressures, double pressure, const double *T0,
                            const int *kinds_dev, int two_nr)
{
  const int a = blockIdx.x;
  if (a >= B.n) return;
  const int r = B.order[a];
  if (threadIdx.x == 0) {
    B.steps[a] = counts[(size_t)r * 4];
    B.ps[a] = pressures ? pressures[r] : pressure;
    B.T0s[a] = T0 ? T0[r] : 0.;
  }
  for (int e = threadIdx.x; e < B.O * B.neq; e += blockDim.x) {
    const int o = e / B.neq, j = e - o * B.neq;
    B.lam[(size_t)a * B.O * B.neq + e] = (kinds_dev[o] == SF_ADJ_T_END && j == B.tix) ? 1. : 0.;
  }
  for (int e = threadIdx.x; e < B.O * two_nr; e += blockDim.x) B.grad[(size_t)a * B.O * two_nr + e] = 0.;
}

// step m of every active slot: h, the six stage states, per-stage pressures
__global__ void k_adj_gather(AdjBufs B, int m, int na)
{
  const int a = blockIdx.x;
  if (a >= na) return;
  const int r = B.order[a];
  const int idx = B.steps[a] - 1 - m;
  const size_t row = 2 + 6 * (size_t)B.neq;
  const double *src = B.rec + ((size_t)r * B.cap + idx) * row;
  for (int e = threadIdx.x; e < 6 * B.neq; e += blockDim.x) B.Y6[(size_t)a * 6 * B.neq + e] = src[2 + e];
  if (threadIdx.x < 6) B.pres6[(size_t)a * 6 + threadIdx.x] = B.ps[a];
  if (threadIdx.x == 0) B.h[a] = src[1];
}

// factors of h gamma J_s^T - I for s = 1..5, system a*5 + s-1, one warp each: the row permutation and the
// reciprocals of the pivots are kept, so that the stage solves multiply instead of dividing on their serial sweeps
__global__ void k_adj_lu(AdjBufs B, int na)
{
  extern __shared__ __align__(16) unsigned char sm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m = B.neq;
  const size_t mm = (size_t)m * m;
  double *A = reinterpret_cast<double *>(sm) + (size_t)w * (mm + m);
  double *di = A + mm;
  int *pv = reinterpret_cast<int *>(reinterpret_cast<double *>(sm) + (size_t)kWarps * (mm + m)) + w * m;
  for (int sys = blockIdx.x * kWarps + w; sys < na * 5; sys += gridDim.x * kWarps) {
    const int a = sys / 5, s = sys - a * 5 + 1;
    const double g = B.h[a] * kGamma;
    const double *J = B.J6 + ((size_t)a * 6 + s) * mm;
    // J is column-major: f = c*m + r holds J[r][c]; A = g J^T - I holds J[r][c] at row c, column r
    for (size_t f = lane; f < mm; f += 32) {
      const int c = (int)(f / m), r = (int)(f - (size_t)c * m);
      A[(size_t)r * m + c] = g * J[f] - (r == c ? 1. : 0.);
    }
    __syncwarp();
    warp_lu_pd(A, m, pv, di);
    __syncwarp();
    double *LU = B.LU + (size_t)sys * mm;
    for (size_t e = lane; e < mm; e += 32) LU[e] = A[e];
    for (int k = lane; k < m; k += 32) {
      B.perm[(size_t)sys * m + k] = pv[k];
      B.dinv[(size_t)sys * m + k] = di[k];
    }
    __syncwarp();
  }
}

// lam' = lam with the entries the forward step's clamp acted on zeroed (the update Y0 + h sum_s b_s f_s < 0)
__global__ void k_adj_lamp(AdjBufs B, int na)
{
  const long long tot = (long long)na * B.neq;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(t / B.neq), j = (int)(t - (long long)a * B.neq);
    const double *K = B.K6 + (size_t)a * 6 * B.neq + j;
    double sum = 0.;
    for (int s = 0; s < 6; ++s) sum += c_b[s] * K[(size_t)s * B.neq];
    const double v = B.Y6[(size_t)a * 6 * B.neq + j] + B.h[a] * sum;
    const double keep = v >= 0. ? 1. : 0.;
    for (int o = 0; o < B.O; ++o) {
      const size_t e = ((size_t)a * B.O + o) * B.neq + j;
      B.lamp[e] = B.lam[e] * keep;
    }
  }
}

// the stage recursion of one reactor for all outputs, one warp
__global__ void k_adj_stages(AdjBufs B, int na)
{
  extern __shared__ __align__(16) unsigned char sm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m = B.neq, O = B.O, tix = B.tix;
  const size_t mm = (size_t)m * m;
  double *LU = reinterpret_cast<double *>(sm) + (size_t)w * (mm + 3 * m);
  double *x = LU + mm, *cv = x + m, *di = cv + m;
  int *pv = reinterpret_cast<int *>(reinterpret_cast<double *>(sm) + (size_t)kWarps * (mm + 3 * m)) + w * m;
  for (int a = blockIdx.x * kWarps + w; a < na; a += gridDim.x * kWarps) {
    const double h = B.h[a];
    for (int s = 5; s >= 0; --s) {
      if (s >= 1) {
        const size_t sys = (size_t)a * 5 + s - 1;
        for (size_t e = lane; e < mm; e += 32) LU[e] = B.LU[sys * mm + e];
        for (int k = lane; k < m; k += 32) {
          pv[k] = B.perm[sys * m + k];
          di[k] = B.dinv[sys * m + k];
        }
      }
      const double Ts = B.Y6[((size_t)a * 6 + s) * m + tix];
      const double sg = 1. / (1. + exp(-((Ts - B.T0s[a] - kDtIgn) / kWidth)));
      const double dg = -sg * (1. - sg) / kWidth;
      const double *J = B.J6 + ((size_t)a * 6 + s) * mm;
      for (int o = 0; o < O; ++o) {
        const size_t base = ((size_t)a * O + o);
        const double qdT = ((h * c_b[s]) * dg) * B.quad[o];
        __syncwarp();
        for (int j = lane; j < m; j += 32) {
          double c = (h * c_b[s]) * B.lamp[base * m + j];
          for (int l = s + 1; l < 6; ++l)
            if (c_a[l][s] != 0.) c = c + (h * c_a[l][s]) * B.Ybar[(base * 6 + l) * m + j];
          if (s >= 1) c = c + (h * kGamma) * (j == tix ? qdT : 0.);
          cv[j] = s >= 1 ? -c : c;
        }
        __syncwarp();
        if (s >= 1) {  // (h gamma J_s^T - I) w = -c, the right-hand side loaded in pivot order
          for (int i = lane; i < m; i += 32) x[i] = cv[pv[i]];
          warp_lu_solve_pd(LU, m, di, x);
        } else {
          for (int i = lane; i < m; i += 32) x[i] = cv[i];
        }
        __syncwarp();
        for (int j = lane; j < m; j += 32) B.W[(base * 6 + s) * m + j] = x[j];
        // Ybar_s = J_s^T w + qd_s: lane i walks column i of J (contiguous)
        for (int i = lane; i < m; i += 32) {
          const double *col = J + (size_t)i * m;
          double acc = 0.;
          for (int j = 0; j < m; ++j) acc = fma(col[j], x[j], acc);
          B.Ybar[(base * 6 + s) * m + i] = acc + (i == tix ? qdT : 0.);
        }
        __syncwarp();
      }
    }
    for (int o = 0; o < O; ++o) {
      const size_t base = (size_t)a * O + o;
      for (int j = lane; j < m; j += 32) {
        double sum = 0.;
        for (int s = 0; s < 6; ++s) sum += B.Ybar[(base * 6 + s) * m + j];
        B.lam[base * m + j] = B.lamp[base * m + j] + sum;
      }
    }
    __syncwarp();
  }
}

// results back in the caller's reactor order
__global__ void k_adj_scatter(AdjBufs B, int two_nr, double *out_theta, double *out_q0)
{
  const int a = blockIdx.x;
  if (a >= B.n) return;
  const int r = B.order[a];
  for (int e = threadIdx.x; e < B.O * two_nr; e += blockDim.x)
    out_theta[(size_t)r * B.O * two_nr + e] = B.grad[(size_t)a * B.O * two_nr + e];
  if (out_q0)
    for (int e = threadIdx.x; e < B.O * B.neq; e += blockDim.x)
      out_q0[(size_t)r * B.O * B.neq + e] = B.lam[(size_t)a * B.O * B.neq + e];
}

size_t up(size_t b) { return (b + 255) & ~(size_t)255; }

struct AdjLayout {
  size_t off[20];
  size_t bytes;
};

// 0 order, 1 steps, 2 ps, 3 T0s, 4 Y6, 5 K6, 6 J6, 7 pres6, 8 h, 9 LU, 10 perm, 11 lam, 12 lamp, 13 W, 14 Ybar,
// 15 grad, 16 output kinds, 17 dinv
AdjLayout adj_layout(const sf_mech *mech, int configuration, int n, int O)
{
  const HostMech &hm = mech->m;
  const size_t neq = configuration == 1 ? hm.dm.ns + 1 : hm.dm.ns;
  const size_t nr = hm.dm.nr;
  const size_t N = n;
  const size_t sizes[18] = {N * 4, N * 4, N * 8, N * 8, 6 * N * neq * 8, 6 * N * neq * 8, 6 * N * neq * neq * 8,
                            6 * N * 8, N * 8, 5 * N * neq * neq * 8, 5 * N * neq * 4, N * O * neq * 8,
                            N * O * neq * 8, N * O * 6 * neq * 8, N * O * 6 * neq * 8, N * O * 2 * nr * 8, 64, 5 * N * neq * 8};
  AdjLayout L{};
  size_t o = 0;
  for (int k = 0; k < 18; ++k) {
    L.off[k] = o;
    o += up(sizes[k]);
  }
  L.bytes = o;
  return L;
}

}  // namespace
}  // namespace sfgb

using namespace sfgb;

extern "C" {

size_t sf_adjoint_workspace_size(const sf_mech *mech, const sf_reactor_params *params, int n, int n_outputs)
{
  if (!mech || !params || n < 0 || n_outputs < 1 || n_outputs > 8) return 0;
  try {
    return adj_layout(mech, params->configuration, n, n_outputs).bytes;
  } catch (sf_error &e) {
    set_error(e.what());
    return 0;
  }
}

int sf_adjoint_batch(const sf_mech *mech, const sf_reactor_params *params, int n, const double *trajectory,
                     int capacity_steps, const int *counts, const double *pressures, const double *T0,
                     int n_outputs, const int *output_kinds, double *out_grad_theta, double *out_grad_q0,
                     void *workspace, size_t workspace_bytes, void *stream)
{
  try {
    if (!mech || !params || n < 0 || n_outputs < 1 || n_outputs > 8 || !output_kinds ||
        (n > 0 && (!trajectory || !counts || !out_grad_theta || capacity_steps < 1)))
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "sf_adjoint_batch: bad argument");
    if (params->open || params->heat_transfer != 0)
      throw sf_error(SF_ERR_UNSUPPORTED, "adjoints cover closed adiabatic reactors");
    if (params->configuration != 0 && params->configuration != 1)
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad configuration");
    bool any_tau = false;
    for (int o = 0; o < n_outputs; ++o) {
      if (output_kinds[o] != SF_ADJ_T_END && output_kinds[o] != SF_ADJ_TAU_S)
        throw sf_error(SF_ERR_INVALID_ARGUMENT, "unknown adjoint output kind");
      any_tau = any_tau || output_kinds[o] == SF_ADJ_TAU_S;
    }
    if (any_tau && !T0) throw sf_error(SF_ERR_INVALID_ARGUMENT, "the smoothed ignition delay needs T0");
    if (n == 0) return SF_OK;
    const HostMech &hm = mech->m;
    const AdjLayout L = adj_layout(mech, params->configuration, n, n_outputs);
    if (!workspace || workspace_bytes < L.bytes)
      throw sf_error(SF_ERR_WORKSPACE, "workspace smaller than sf_adjoint_workspace_size reports");
    cudaStream_t st = (cudaStream_t)stream;
    char *w = static_cast<char *>(workspace);
    auto at = [&](int k) { return w + L.off[k]; };
    const int ns = hm.dm.ns, nr = hm.dm.nr;
    AdjBufs B{};
    B.n = n;
    B.O = n_outputs;
    B.neq = params->configuration == 1 ? ns + 1 : ns;
    B.tix = params->configuration == 1 ? 1 : 0;
    B.cap = capacity_steps;
    B.rec = trajectory;
    B.order = reinterpret_cast<int *>(at(0));
    B.steps = reinterpret_cast<int *>(at(1));
    B.ps = reinterpret_cast<double *>(at(2));
    B.T0s = reinterpret_cast<double *>(at(3));
    B.Y6 = reinterpret_cast<double *>(at(4));
    B.K6 = reinterpret_cast<double *>(at(5));
    B.J6 = reinterpret_cast<double *>(at(6));
    B.pres6 = reinterpret_cast<double *>(at(7));
    B.h = reinterpret_cast<double *>(at(8));
    B.LU = reinterpret_cast<double *>(at(9));
    B.perm = reinterpret_cast<int *>(at(10));
    B.dinv = reinterpret_cast<double *>(at(17));
    B.lam = reinterpret_cast<double *>(at(11));
    B.lamp = reinterpret_cast<double *>(at(12));
    B.W = reinterpret_cast<double *>(at(13));
    B.Ybar = reinterpret_cast<double *>(at(14));
    B.grad = reinterpret_cast<double *>(at(15));
    int *kinds_dev = reinterpret_cast<int *>(at(16));
    for (int o = 0; o < n_outputs; ++o) B.quad[o] = output_kinds[o] == SF_ADJ_TAU_S ? 1. : 0.;

    // step counts: the one read back of the sweep
    std::vector<int> hc((size_t)n * 4);
    CUDA_THROW(cudaMemcpyAsync(hc.data(), counts, hc.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_THROW(cudaStreamSynchronize(st));
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return hc[(size_t)x * 4] > hc[(size_t)y * 4]; });
    std::vector<int> sorted_steps(n);
    for (int a = 0; a < n; ++a) {
      sorted_steps[a] = hc[(size_t)order[a] * 4];
      if (sorted_steps[a] < 0 || sorted_steps[a] > capacity_steps)
        throw sf_error(SF_ERR_INVALID_ARGUMENT, "a reactor's step count exceeds the trajectory's capacity");
    }
    CUDA_THROW(cudaMemcpyAsync(B.order, order.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, st));
    CUDA_THROW(cudaMemcpyAsync(kinds_dev, output_kinds, (size_t)n_outputs * sizeof(int), cudaMemcpyHostToDevice, st));
    const int two_nr = 2 * nr;
    k_adj_setup<<<n, 128, 0, st>>>(B, counts, pressures, params->pressure, T0, kinds_dev, two_nr);
    CUDA_THROW(cudaGetLastError());

    int dev, nsm;
    CUDA_THROW(cudaGetDevice(&dev));
    CUDA_THROW(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const size_t mm = (size_t)B.neq * B.neq;
    const size_t smem_lu = kWarps * ((mm + B.neq) * 8 + B.neq * 4);
    const size_t smem_st = kWarps * ((mm + 3 * B.neq) * 8 + B.neq * 4);
    ensure_dynamic_smem((const void *)k_adj_lu, smem_lu);
    ensure_dynamic_smem((const void *)k_adj_stages, smem_st);
    const int nmax = sorted_steps[0];
    int na = n;
    for (int m = 0; m < nmax; ++m) {
      while (na > 0 && sorted_steps[na - 1] <= m) --na;
      k_adj_gather<<<na, 128, 0, st>>>(B, m, na);
      CUDA_THROW(cudaGetLastError());
      // 32 lanes per state: a few thousand stage states are too few for the thread-per-state kernels
      reactor_jac_lanes(mech, params, 0, 6 * na, B.Y6, params->configuration == 0 ? B.pres6 : nullptr, B.K6, B.J6,
                        32, st);
      const long long lu_need = ((long long)na * 5 + kWarps - 1) / kWarps;
      k_adj_lu<<<(int)std::min<long long>(lu_need, (long long)nsm * 8), 32 * kWarps, smem_lu, st>>>(B, na);
      CUDA_THROW(cudaGetLastError());
      const long long lp = ((long long)na * B.neq + 255) / 256;
      k_adj_lamp<<<(int)std::min<long long>(lp, 4096), 256, 0, st>>>(B, na);
      CUDA_THROW(cudaGetLastError());
      const long long st_need = ((long long)na + kWarps - 1) / kWarps;
      k_adj_stages<<<(int)std::min<long long>(st_need, (long long)nsm * 8), 32 * kWarps, smem_st, st>>>(B, na);
      CUDA_THROW(cudaGetLastError());
      launch_rate_param_adjoint(hm, params->configuration, params->pressure, na, n_outputs, 6, B.Y6,
                                params->configuration == 0 ? B.ps : nullptr, B.W, B.grad, st);
    }
    k_adj_scatter<<<n, 128, 0, st>>>(B, two_nr, out_grad_theta, out_grad_q0);
    CUDA_THROW(cudaGetLastError());
    return SF_OK;
  } catch (sf_error &e) {
    set_error(e.what());
    return e.code;
  }
}

}  // extern "C"
