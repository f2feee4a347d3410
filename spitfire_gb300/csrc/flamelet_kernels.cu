// Flamelet kernels: the adiabatic flamelet right-hand side and its block-tridiagonal ("BTDDOD": block diagonal,
// diagonal off-diagonals) Jacobian for a batch of flamelets with different grids, and the block-Thomas algebra.
//
// Reference: src/spitfire/griffon/src/flamelet_kernels.cpp:31-90 (stencils, COO indices), :1039-1218
// (flamelet_rhs), :1220-1409 (flamelet_jacobian); src/btddod_matrix_kernels.cpp:19-465.
//
// Points of all flamelets are flattened: flamelet f owns interior points offsets_z[f] .. offsets_z[f+1]-1. One state
// group evaluates one point (isobaric chemistry via reactor_eval, then the mixture-fraction stencils). The
// block-Thomas factorization and solve are sequential in mixture fraction, so one CTA (factorization) or one warp
// (solve) works through one flamelet, parallel within each block.
#include "reactor_eval.cuh"
#include "sf_internal.h"
#include "warp_lu.cuh"
#include "eig_device.cuh"

namespace sfgb {
namespace {

struct FlmParams {
  DevMech m;
  const void *blob;
  int *status;
  ScratchLayout L;
  Progs pg;
  int n_flamelets, n_points;
  const int *offz;        // device [nf+1]
  const long long *offv;  // device [nf+1]
  double pressure;
  const double *oxy, *fuel;  // [nf][ns]
  const double *cmajor, *csub, *csup, *mc, *nc, *chi;
  int eflux, vcp;
  const double *state;
  double *out_rhs;
  double *out_values;
  int scale_offset;
  int rates_option;
  double prefactor;
  double *eflux_store;  // if set: the enthalpy-flux diagonal correction is stored here (per point) instead
  int groups_per_cta;
};

__device__ __forceinline__ int find_flamelet(const int *offz, int nf, int p)
{
  int lo = 0, hi = nf - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (offz[mid] <= p) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// cp of the mixture at a state [T, Y_0..Y_{ns-2}] (lanes over species, group reduction)
template <int G>
__device__ __forceinline__ double cp_of_state(const DevMech &m, const Blob &b, const Group<G> &grp, const double *st)
{
  const int ns = m.ns;
  const double T = st[0], logT = log(T), invT = 1. / T;
  double ys = 0., cp = 0.;
  for (int i = grp.lane; i < ns - 1; i += G) {
    const SpeciesThermo th = species_thermo(m, b, i, T, logT, invT, false);
    cp += st[1 + i] * th.cp;
    ys += st[1 + i];
  }
  ys = grp.sum(ys);
  cp = grp.sum(cp);
  const SpeciesThermo thn = species_thermo(m, b, ns - 1, T, logT, invT, false);
  return cp + (1. - ys) * thn.cp;
}

struct BlockWriter {
  double *blk;  // column-major ns x ns
  int ns;
  const double *cmaj;  // [ns] of this point
  int scale;
  double pref;
  __device__ __forceinline__ void operator()(int row, int col, double v) const
  {
    double x = v + (row == col ? cmaj[row] : 0.);
    if (scale) x = pref * x - (row == col ? 1. : 0.);
    blk[col * ns + row] = x;
  }
};

template <int G, bool JAC>
__global__ void __launch_bounds__(256) flamelet_point_kernel(const FlmParams p)
{
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint64_t bar;
  const DevMech &m = p.m;
  if (!stage_to_smem(smem, p.blob, m.blob_bytes, &bar, p.status)) return;
  const Blob b = blob_at(m, smem);
  const ScratchLayout &L = p.L;
  const int gid = threadIdx.x / G;
  // per group: Griffon scratch + ns doubles for the (unused) right-hand side of the Jacobian evaluation
  double *scr = reinterpret_cast<double *>(smem + m.blob_bytes) + (size_t)gid * ((JAC ? L.total : L.total_rhs) + m.ns + 2);
  const Group<G> grp;
  const int lane = grp.lane;
  const int ns = m.ns;
  ReactorCfg cfg{};
  cfg.configuration = 0;
  cfg.heat = 0;
  cfg.option = JAC ? p.rates_option : 0;
  NoJ noj;
  for (int pt = blockIdx.x * p.groups_per_cta + gid; pt < p.n_points; pt += gridDim.x * p.groups_per_cta) {
    const int f = find_flamelet(p.offz, p.n_flamelets, pt);
    const int z0 = p.offz[f], nzi = p.offz[f + 1] - z0;
    const int iz = pt - z0;
    const double *st = p.state + (size_t)pt * ns;
    const double *oxy = p.oxy + (size_t)f * ns;
    const double *fuel = p.fuel + (size_t)f * ns;
    const double *sm1 = iz == 0 ? oxy : st - ns;
    const double *sp1 = iz == nzi - 1 ? fuel : st + ns;
    const double mcf = p.mc[pt], ncf = p.nc[pt], chi = p.chi[pt];
    if (!JAC) {
      double *out = p.out_rhs + (size_t)pt * ns;
      reactor_eval<G, false>(m, b, L, scr, grp, st, p.pressure, cfg, p.pg, out, noj);
      // enthalpy-flux and variable-cp terms of the temperature equation (flamelet_kernels.cpp:1141-1206)
      double cp = 0.;
      for (int i = lane; i < ns; i += G) cp += scr[L.y + i] * scr[L.cpv + i];
      cp = grp.sum(cp);
      const double dTdZ = mcf * sm1[0] + ncf * sp1[0];
      double extra = 0.;
      if (p.eflux) {
        const double cpn = scr[L.cpv + ns - 1];
        double s = 0.;
        for (int j = lane; j < ns - 1; j += G) s += (scr[L.cpv + j] - cpn) * (mcf * sm1[1 + j] + ncf * sp1[1 + j]);
        s = grp.sum(s);
        extra += 0.5 * chi / cp * dTdZ * s;
      }
      if (p.vcp) {
        const double cpm = cp_of_state<G>(m, b, grp, sm1);
        const double cpp = cp_of_state<G>(m, b, grp, sp1);
        extra += 0.5 * chi * (mcf * cpm + ncf * cpp) / cp * dTdZ;
      }
      grp.sync();
      // mixture-fraction diffusion (flamelet_kernels.cpp:1208-1217)
      const double *cma = p.cmajor + (size_t)pt * ns, *csb = p.csub + (size_t)pt * ns, *csp = p.csup + (size_t)pt * ns;
      for (int i = lane; i < ns; i += G) {
        double v = out[i] + (i == 0 ? extra : 0.);
        v += cma[i] * st[i] + csb[i] * sm1[i] + csp[i] * sp1[i];
        out[i] = v;
      }
      grp.sync();
    } else {
      // block of this point in the flamelet's BTDDOD value array
      double *vals = p.out_values + p.offv[f];
      double *blk = vals + (size_t)iz * ns * ns;
      BlockWriter bw{blk, ns, p.cmajor + (size_t)pt * ns, p.scale_offset, p.prefactor};
      double *rhs_tmp = scr + L.total;
      reactor_eval<G, true>(m, b, L, scr, grp, st, p.pressure, cfg, p.pg, rhs_tmp, bw);
      if (p.eflux) {
        // approximate diagonal correction of the enthalpy-flux term (flamelet_kernels.cpp:1350-1381)
        double cp = 0., cps = 0.;
        for (int i = lane; i < ns; i += G) {
          cp += scr[L.y + i] * scr[L.cpv + i];
          cps += scr[L.y + i] * scr[L.dcp + i];
        }
        cp = grp.sum(cp);
        cps = grp.sum(cps);
        const double cpm = cp_of_state<G>(m, b, grp, sm1);
        const double cpp = cp_of_state<G>(m, b, grp, sp1);
        const double dTdZ = mcf * sm1[0] + ncf * sp1[0];
        const double dcpdZ = mcf * cpm + ncf * cpp;
        const double f1 = 0.5 * chi / cp * dTdZ * dcpdZ;
        grp.sync();
        if (lane == 0) {
          const double corr = (p.scale_offset ? p.prefactor : 1.) * f1 / cp * cps;
          if (p.eflux_store)
            p.eflux_store[(size_t)pt * ns] = corr;
          else
            blk[0] -= corr;
        }
      } else if (p.eflux_store && lane == 0) {
        p.eflux_store[(size_t)pt * ns] = 0.;
      }
      // off-diagonals: sub row iz (iz >= 1) and super row iz (iz <= nzi-2) (flamelet_kernels.cpp:1383-1394)
      const long long sub_off = (long long)nzi * ns * ns, sup_off = sub_off + (long long)(nzi - 1) * ns;
      const double sc = p.scale_offset ? p.prefactor : 1.;
      for (int q = lane; q < ns; q += G) {
        if (iz >= 1) vals[sub_off + (long long)(iz - 1) * ns + q] = sc * p.csub[(size_t)pt * ns + q];
        if (iz <= nzi - 2) vals[sup_off + (long long)iz * ns + q] = sc * p.csup[(size_t)pt * ns + q];
      }
      grp.sync();
    }
  }
}

// Pseudo-time-step eigenvalue bound (flamelet_kernels.cpp:1329-1341): for each point, max(max Re(lambda) - diffterm,
// 0) of the transformed isobaric chemistry block (the block before the diffusion diagonal and the enthalpy-flux
// correction are added), written to all ns entries of the point; then the held-back enthalpy-flux correction is
// applied to the block. One warp per point, the block in shared memory.
__global__ void flamelet_expeig_kernel(int n_points, int nf, int ns, const int *offz, const long long *offv,
                                       double *values, const double *cmajor, double diffterm, double *expeig,
                                       int *status, int warps)
{
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *A = reinterpret_cast<double *>(smem) + (size_t)w * (ns * ns + ns);
  double *work = A + ns * ns;
  for (int pt = blockIdx.x * warps + w; pt < n_points; pt += gridDim.x * warps) {
    const int f = find_flamelet(offz, nf, pt);
    const int iz = pt - offz[f];
    double *blk = values + offv[f] + (size_t)iz * ns * ns;
    for (int e = lane; e < ns * ns; e += 32) {
      const int col = e / ns, row = e - col * ns;
      A[e] = blk[e] - (row == col ? cmajor[(size_t)pt * ns + row] : 0.);
    }
    __syncwarp();
    double mx;
    const bool ok = warp_max_real_eig(A, ns, work, &mx);
    if (!ok && lane == 0) report_error(status, DEVERR_WAIT_TIMEOUT);
    const double corr = expeig[(size_t)pt * ns];
    __syncwarp();
    const double e = fmax(mx - diffterm, 0.);
    for (int q = lane; q < ns; q += 32) expeig[(size_t)pt * ns + q] = e;
    if (lane == 0) blk[0] -= corr;
    __syncwarp();
  }
}

// ------------------------------------------------------------------------------- block-Thomas (BTDDOD) algebra
// Factorization (btddod_matrix_kernels.cpp:19-80): D_0 = LU; for i >= 1: L_i = diag(sub_{i-1}) D_{i-1}^-1,
// D_i <- D_i - L_i diag(sup_{i-1}), LU(D_i). One CTA per flamelet, D_{i-1} factors and D_i in shared memory.
constexpr int kFactorThreads = 256;

__device__ void cta_lu(double *A, int n, int *piv, double *red_v, int *red_i)
{
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  for (int k = 0; k < n; ++k) {
    if (warp == 0) {
      double best = -1.;
      int bi = k;
      for (int i = k + lane; i < n; i += 32) {
        const double v = fabs(A[i + k * n]);
        if (v > best) { best = v; bi = i; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (lane == 0) {
        piv[k] = bi;
        red_i[0] = bi;
      }
    }
    __syncthreads();
    const int bi = red_i[0];
    if (bi != k)
      for (int j = tid; j < n; j += nt) {
        const double t = A[k + j * n];
        A[k + j * n] = A[bi + j * n];
        A[bi + j * n] = t;
      }
    __syncthreads();
    const double pv = A[k + k * n];
    if (pv != 0.) {
      const double inv = 1. / pv;
      for (int i = k + 1 + tid; i < n; i += nt) A[i + k * n] *= inv;
    }
    __syncthreads();
    if (pv != 0.) {
      const int r = n - k - 1;
      for (int t = tid; t < r * r; t += nt) {
        const int jj = t / r, ii = t - jj * r;
        A[(k + 1 + ii) + (k + 1 + jj) * n] -= A[(k + 1 + ii) + k * n] * A[k + (k + 1 + jj) * n];
      }
    }
    __syncthreads();
  }
  (void)red_v;
}

// X <- LU^-1 X for `ncols` right-hand-side columns (column-major, leading dimension n), columns split over warps.
__device__ void cta_lu_solve_cols(const double *LU, const int *piv, int n, double *X, int ncols)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int c = warp; c < ncols; c += nw) {
    double *x = X + (size_t)c * n;
    if (lane == 0)
      for (int k = 0; k < n; ++k) {
        const int p = piv[k];
        if (p != k) { const double t = x[k]; x[k] = x[p]; x[p] = t; }
      }
    __syncwarp();
    for (int j = 0; j < n; ++j) {
      const double xj = x[j];
      for (int i = j + 1 + lane; i < n; i += 32) x[i] -= LU[i + j * n] * xj;
      __syncwarp();
    }
    for (int j = n - 1; j >= 0; --j) {
      if (lane == 0) x[j] /= LU[j + j * n];
      __syncwarp();
      const double xj = x[j];
      for (int i = lane; i < j; i += 32) x[i] -= LU[i + j * n] * xj;
      __syncwarp();
    }
  }
}

__global__ void __launch_bounds__(kFactorThreads) btddod_factor_kernel(int nf, int ns, const int *offz,
                                                                       const long long *offv, double *values,
                                                                       double *lvals, int *pivots)
{
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red_v[32];
  __shared__ int red_i[32];
  const int f = blockIdx.x;
  if (f >= nf) return;
  const int z0 = offz[f], nb = offz[f + 1] - z0;
  const int bs2 = ns * ns;
  double *vals = values + offv[f];
  double *lv = lvals + (size_t)z0 * bs2;
  int *pv = pivots + (size_t)z0 * ns;
  const double *sub = vals + (size_t)nb * bs2;
  const double *sup = sub + (size_t)(nb - 1) * ns;
  double *Dprev = reinterpret_cast<double *>(smem);  // factors of D_{i-1}
  double *Dcur = Dprev + bs2;                         // D_i
  double *Lc = Dcur + bs2;                            // L_i
  int *ppiv = reinterpret_cast<int *>(Lc + bs2);      // pivots of D_{i-1}
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < bs2; e += nt) Dprev[e] = vals[e];
  __syncthreads();
  cta_lu(Dprev, ns, ppiv, red_v, red_i);
  for (int e = tid; e < bs2; e += nt) vals[e] = Dprev[e];
  for (int k = tid; k < ns; k += nt) pv[k] = ppiv[k];
  __syncthreads();
  for (int i = 1; i < nb; ++i) {
    // L_i = diag(sub_{i-1}) * D_{i-1}^-1: solve D_{i-1} X = I, then scale rows
    for (int e = tid; e < bs2; e += nt) {
      const int col = e / ns, row = e - col * ns;
      Lc[e] = row == col ? 1. : 0.;
      Dcur[e] = vals[(size_t)i * bs2 + e];
    }
    __syncthreads();
    cta_lu_solve_cols(Dprev, ppiv, ns, Lc, ns);
    __syncthreads();
    const double *sb = sub + (size_t)(i - 1) * ns;
    const double *sp = sup + (size_t)(i - 1) * ns;
    for (int e = tid; e < bs2; e += nt) {
      const int col = e / ns, row = e - col * ns;
      const double l = Lc[e] * sb[row];
      Lc[e] = l;
      lv[(size_t)i * bs2 + e] = l;
      Dcur[e] += -sp[col] * l;
    }
    __syncthreads();
    cta_lu(Dcur, ns, ppiv, red_v, red_i);
    for (int e = tid; e < bs2; e += nt) {
      vals[(size_t)i * bs2 + e] = Dcur[e];
      Dprev[e] = Dcur[e];
    }
    for (int k = tid; k < ns; k += nt) pv[(size_t)i * ns + k] = ppiv[k];
    __syncthreads();
  }
}

// Solve (btddod_matrix_kernels.cpp:82-119), one warp per flamelet:
//   y_0 = b_0, y_i = b_i - L_i y_{i-1};  x_{nb-1} = D^-1 y_{nb-1};  x_i = D_i^-1 (y_i - sup_i o x_{i+1})
__global__ void btddod_solve_kernel(int nf, int ns, const int *offz, const long long *offv, const double *values,
                                    const double *lvals, const int *pivots, const double *rhs, double *x)
{
  const int f = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (f >= nf) return;
  const int lane = threadIdx.x & 31;
  const int z0 = offz[f], nb = offz[f + 1] - z0;
  const int bs2 = ns * ns;
  const double *vals = values + offv[f];
  const double *lv = lvals + (size_t)z0 * bs2;
  const int *pv = pivots + (size_t)z0 * ns;
  const double *sup = vals + (size_t)nb * bs2 + (size_t)(nb - 1) * ns;
  const double *b = rhs + (size_t)z0 * ns;
  double *xs = x + (size_t)z0 * ns;
  // forward sweep into x (y values)
  for (int k = lane; k < ns; k += 32) xs[k] = b[k];
  __syncwarp();
  for (int i = 1; i < nb; ++i) {
    const double *Li = lv + (size_t)i * bs2;
    const double *yp = xs + (size_t)(i - 1) * ns;
    for (int r = lane; r < ns; r += 32) {
      double v = b[(size_t)i * ns + r];
      for (int c = 0; c < ns; ++c) v += Li[(size_t)c * ns + r] * (-yp[c]);
      xs[(size_t)i * ns + r] = v;
    }
    __syncwarp();
  }
  // backward sweep with the block LU factors (serial triangular solves per block)
  for (int i = nb - 1; i >= 0; --i) {
    double *xi = xs + (size_t)i * ns;
    if (i < nb - 1) {
      for (int j = lane; j < ns; j += 32) xi[j] -= sup[(size_t)i * ns + j] * xs[(size_t)(i + 1) * ns + j];
      __syncwarp();
    }
    warp_lu_solve(vals + (size_t)i * bs2, ns, pv + (size_t)i * ns, xi);
    __syncwarp();
  }
}

// y = A x (btddod_matrix_kernels.cpp:121-160), one warp per flamelet
__global__ void btddod_matvec_kernel(int nf, int ns, const int *offz, const long long *offv, const double *values,
                                     const double *x, double *y)
{
  const int f = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (f >= nf) return;
  const int lane = threadIdx.x & 31;
  const int z0 = offz[f], nb = offz[f + 1] - z0;
  const int bs2 = ns * ns;
  const double *vals = values + offv[f];
  const double *sub = vals + (size_t)nb * bs2;
  const double *sup = sub + (size_t)(nb - 1) * ns;
  const double *xs = x + (size_t)z0 * ns;
  double *ys = y + (size_t)z0 * ns;
  for (int i = 0; i < nb; ++i)
    for (int r = lane; r < ns; r += 32) {
      double v = 0.;
      for (int c = 0; c < ns; ++c) v += vals[(size_t)i * bs2 + (size_t)c * ns + r] * xs[(size_t)i * ns + c];
      if (i >= 1) v += sub[(size_t)(i - 1) * ns + r] * xs[(size_t)(i - 1) * ns + r];
      if (i <= nb - 2) v += sup[(size_t)i * ns + r] * xs[(size_t)(i + 1) * ns + r];
      ys[(size_t)i * ns + r] = v;
    }
}

// A <- matrix_scale*A + diag_scale*diag(d) (btddod_matrix_kernels.cpp:448-465), one CTA per flamelet
__global__ void btddod_scale_diag_kernel(int nf, int ns, const int *offz, const long long *offv, double *values,
                                         double ms, const double *diag, double ds)
{
  const int f = blockIdx.x;
  if (f >= nf) return;
  const int z0 = offz[f], nb = offz[f + 1] - z0;
  const long long ne = (long long)ns * (nb * ns + 2 * (nb - 1));
  double *vals = values + offv[f];
  for (long long e = threadIdx.x; e < ne; e += blockDim.x) vals[e] *= ms;
  __syncthreads();
  for (int e = threadIdx.x; e < nb * ns; e += blockDim.x) {
    const int iz = e / ns, q = e - iz * ns;
    vals[(size_t)iz * ns * ns + (size_t)q * (ns + 1)] += ds * diag[(size_t)z0 * ns + e];
  }
}

int launch_points(HostMech &hm, FlmParams &p, bool jac, cudaStream_t st)
{
  const int G = 32;
  const auto &progs = hm.programs_for(G);
  p.m = hm.dm;
  p.blob = hm.d_blob;
  p.status = hm.d_status;
  p.L = hm.sl;
  p.pg.w = progs.progs[0];
  p.pg.full = progs.progs[1];
  p.pg.j = progs.progs[2];
  int dev, smem_max, nsm;
  CUDA_THROW(cudaGetDevice(&dev));
  CUDA_THROW(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  CUDA_THROW(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const size_t per = (size_t)((jac ? hm.sl.total : hm.sl.total_rhs) + hm.dm.ns + 2) * 8;
  const size_t avail = (size_t)smem_max - hm.dm.blob_bytes - 64;
  int groups = (int)std::min<size_t>(avail / per, 256 / G);
  if (groups < 1) throw sf_error(SF_ERR_UNSUPPORTED, "mechanism too large for the flamelet kernels");
  p.groups_per_cta = groups;
  const size_t smem = hm.dm.blob_bytes + per * groups;
  void (*k)(const FlmParams) = jac ? flamelet_point_kernel<32, true> : flamelet_point_kernel<32, false>;
  CUDA_THROW(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int bps = std::max(1, (int)((size_t)smem_max / smem));
  const int grid = (int)std::max<long long>(1, std::min<long long>(((long long)p.n_points + groups - 1) / groups,
                                                                   (long long)nsm * bps));
  k<<<grid, groups * G, smem, st>>>(p);
  CUDA_THROW(cudaGetLastError());
  return SF_OK;
}

void fill(FlmParams &p, const sf_flamelet_batch *fb)
{
  if (!fb || fb->n_flamelets < 1 || !fb->offsets_z || !fb->offsets_v || !fb->offsets_z_host || !fb->oxy_state ||
      !fb->fuel_state || !fb->cmajor || !fb->csub || !fb->csup || !fb->mcoeff || !fb->ncoeff || !fb->chi)
    throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad flamelet batch");
  p.n_flamelets = fb->n_flamelets;
  p.n_points = fb->offsets_z_host[fb->n_flamelets];
  for (int f = 0; f < fb->n_flamelets; ++f)
    if (fb->offsets_z_host[f + 1] - fb->offsets_z_host[f] < 2)
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "every flamelet needs at least two interior points");
  p.offz = fb->offsets_z;
  p.offv = fb->offsets_v;
  p.pressure = fb->pressure;
  p.oxy = fb->oxy_state;
  p.fuel = fb->fuel_state;
  p.cmajor = fb->cmajor;
  p.csub = fb->csub;
  p.csup = fb->csup;
  p.mc = fb->mcoeff;
  p.nc = fb->ncoeff;
  p.chi = fb->chi;
  p.eflux = fb->include_enthalpy_flux;
  p.vcp = fb->include_variable_cp;
}

template <class F>
int guarded(F f)
{
  try {
    return f();
  } catch (sf_error &e) {
    set_error(e.what());
    return e.code;
  }
}

int check_launch()
{
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return SF_ERR_CUDA;
  }
  return SF_OK;
}

}  // namespace
}  // namespace sfgb

using namespace sfgb;

extern "C" {

int sf_flamelet_stencils(const sf_mech *mech, const double *dz, int nzi, const double *chi, const double *invLe,
                         double *cmaj, double *csub, double *csup, double *mc, double *nc)
{
  if (!mech || !dz || !chi || !invLe || !cmaj || !csub || !csup || !mc || !nc || nzi < 1) {
    set_error("sf_flamelet_stencils: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  const int ns = mech->m.dm.ns;
  for (int i = 0; i < nzi; ++i) {  // flamelet_kernels.cpp:31-48
    const double dzt = dz[i] + dz[i + 1];
    for (int l = 0; l < ns; ++l) {
      cmaj[i * ns + l] = -chi[1 + i] / (dz[i] * dz[i + 1]) * invLe[l];
      csub[i * ns + l] = chi[1 + i] / (dzt * dz[i]) * invLe[l];
      csup[i * ns + l] = chi[1 + i] / (dzt * dz[i + 1]) * invLe[l];
    }
    nc[i] = 1 / (dz[i] + dz[i + 1]);
    mc[i] = -nc[i];
  }
  return SF_OK;
}

int sf_flamelet_jac_indices(const sf_mech *mech, int nzi, int *rows, int *cols)
{
  if (!mech || !rows || !cols || nzi < 1) {
    set_error("sf_flamelet_jac_indices: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  const int ns = mech->m.dm.ns;
  int idx = 0;  // flamelet_kernels.cpp:50-90
  for (int iz = 0; iz < nzi; ++iz)
    for (int iq = 0; iq < ns; ++iq)
      for (int jq = 0; jq < ns; ++jq) {
        rows[idx] = iz * ns + jq;
        cols[idx] = iz * ns + iq;
        ++idx;
      }
  for (int iz = 1; iz < nzi; ++iz)
    for (int iq = 0; iq < ns; ++iq) {
      rows[idx] = iz * ns + iq;
      cols[idx] = iz * ns + iq - ns;
      ++idx;
    }
  for (int iz = 0; iz < nzi - 1; ++iz)
    for (int iq = 0; iq < ns; ++iq) {
      rows[idx] = iz * ns + iq;
      cols[idx] = iz * ns + iq + ns;
      ++idx;
    }
  return SF_OK;
}

int sf_flamelet_rhs_batch(const sf_mech *mech, const sf_flamelet_batch *fb, const double *state, double *out_rhs,
                          void *stream)
{
  return guarded([&] {
    if (!mech || !state || !out_rhs) throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad argument");
    FlmParams p{};
    fill(p, fb);
    p.state = state;
    p.out_rhs = out_rhs;
    return launch_points(const_cast<HostMech &>(mech->m), p, false, (cudaStream_t)stream);
  });
}

int sf_flamelet_jac_batch(const sf_mech *mech, const sf_flamelet_batch *fb, const double *state, int rates_option,
                          int scale_and_offset, double prefactor, double diffterm, double *out_expeig,
                          double *out_values, void *stream)
{
  return guarded([&] {
    if (!mech || !state || !out_values) throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad argument");
    if (rates_option < 0 || rates_option > 2)
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "rates option must be 0, 1 or 2");
    if (out_expeig && scale_and_offset)
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "eigenvalue bounds need scale_and_offset = 0 (as flamelet.py calls it)");
    FlmParams p{};
    fill(p, fb);
    p.state = state;
    p.out_values = out_values;
    p.scale_offset = scale_and_offset;
    p.rates_option = rates_option;
    p.prefactor = prefactor;
    p.eflux_store = out_expeig;
    HostMech &hm = const_cast<HostMech &>(mech->m);
    cudaStream_t st = (cudaStream_t)stream;
    launch_points(hm, p, true, st);
    if (out_expeig) {
      const int ns = hm.dm.ns;
      int dev, smem_max, nsm;
      CUDA_THROW(cudaGetDevice(&dev));
      CUDA_THROW(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
      CUDA_THROW(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
      const size_t per = (size_t)(ns * ns + ns) * 8;
      const int warps = (int)std::min<size_t>(8, (size_t)smem_max / per);
      if (warps < 1) throw sf_error(SF_ERR_UNSUPPORTED, "block too large for the eigenvalue kernel");
      CUDA_THROW(cudaFuncSetAttribute(flamelet_expeig_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(per * warps)));
      const int grid = (int)std::min<long long>((long long)nsm * 2, ((long long)p.n_points + warps - 1) / warps);
      flamelet_expeig_kernel<<<grid, 32 * warps, per * warps, st>>>(p.n_points, p.n_flamelets, ns, p.offz, p.offv,
                                                                    out_values, p.cmajor, diffterm, out_expeig,
                                                                    hm.d_status, warps);
      CUDA_THROW(cudaGetLastError());
    }
    return SF_OK;
  });
}

int sf_btddod_factor_batch(int nf, int ns, const int *offz, const long long *offv, const int *offz_host,
                           double *values, double *l_values, int *pivots, void *stream)
{
  if (nf < 1 || ns < 1 || ns > 128 || !offz || !offv || !values || !l_values || !pivots) {
    set_error("sf_btddod_factor_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  (void)offz_host;
  const size_t smem = (size_t)3 * ns * ns * 8 + (size_t)ns * 4 + 16;
  return guarded([&] {
    int dev, smem_max;
    CUDA_THROW(cudaGetDevice(&dev));
    CUDA_THROW(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    if (smem > (size_t)smem_max)
      throw sf_error(SF_ERR_UNSUPPORTED, "block size too large for the shared-memory block-Thomas factorization");
    CUDA_THROW(cudaFuncSetAttribute(btddod_factor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    btddod_factor_kernel<<<nf, kFactorThreads, smem, (cudaStream_t)stream>>>(nf, ns, offz, offv, values, l_values,
                                                                             pivots);
    return check_launch();
  });
}

int sf_btddod_solve_batch(int nf, int ns, const int *offz, const long long *offv, const int *offz_host,
                          const double *values, const double *l_values, const int *pivots, const double *rhs,
                          double *out_x, void *stream)
{
  if (nf < 1 || ns < 1 || !offz || !offv || !values || !l_values || !pivots || !rhs || !out_x) {
    set_error("sf_btddod_solve_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  (void)offz_host;
  btddod_solve_kernel<<<(nf + 3) / 4, 128, 0, (cudaStream_t)stream>>>(nf, ns, offz, offv, values, l_values, pivots,
                                                                      rhs, out_x);
  return check_launch();
}

int sf_btddod_matvec_batch(int nf, int ns, const int *offz, const long long *offv, const double *values,
                           const double *x, double *out_y, void *stream)
{
  if (nf < 1 || ns < 1 || !offz || !offv || !values || !x || !out_y) {
    set_error("sf_btddod_matvec_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  btddod_matvec_kernel<<<(nf + 3) / 4, 128, 0, (cudaStream_t)stream>>>(nf, ns, offz, offv, values, x, out_y);
  return check_launch();
}

int sf_btddod_scale_and_add_diagonal_batch(int nf, int ns, const int *offz, const long long *offv,
                                           const int *offz_host, double *values, double ms, const double *diag,
                                           double ds, void *stream)
{
  if (nf < 1 || ns < 1 || !offz || !offv || !values || !diag) {
    set_error("sf_btddod_scale_and_add_diagonal_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  (void)offz_host;
  btddod_scale_diag_kernel<<<nf, 256, 0, (cudaStream_t)stream>>>(nf, ns, offz, offv, values, ms, diag, ds);
  return check_launch();
}

}  // extern "C"
