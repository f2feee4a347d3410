// Batched steady flamelet solvers on the device: damped Newton (flamelet.py:1352-1485) and pseudo-transient
// continuation (psitc, flamelet.py:1487-1703) for every flamelet of a batch at once, each flamelet with its own
// iteration count, line search, Jacobian age, pseudo-time steps and restarts. The host runs the control loop; every
// vector operation, norm and per-flamelet decision runs on the device, over the batch's residual, Jacobian,
// eigenvalue-bound and block-Thomas kernels. The host reads back a few flags per iteration (whether any flamelet
// still iterates, needs a new Jacobian, cuts its step or failed), the only synchronizations of the loop.
//
// Per-flamelet state (iteration count, residual norm, step damping, masks) lives in the workspace; masks are int
// arrays [nf] that the batch kernels take as their `active` argument. Every operation mirrors the reference's
// arithmetic (weighted infinity norms with 1e3 on the temperature, halving line search, ds updates), so the
// iteration counts are the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "esdirk64.cuh"
#include "sf_internal.h"

namespace sfgb {
namespace {

constexpr int kThreads = 256;

// torch.minimum's rule: NaN if either operand is NaN
__device__ __forceinline__ double nan_min(double a, double b) { return (a != a || b != b) ? a + b : fmin(a, b); }

int grid_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + kThreads - 1) / kThreads, 4096)); }

// point -> flamelet
__global__ void k_point_map(int nf, const int *offz, int *map)
{
  const int f = blockIdx.x;
  if (f >= nf) return;
  for (int p = offz[f] + threadIdx.x; p < offz[f + 1]; p += blockDim.x) map[p] = f;
}

// Per-flamelet reductions over its dofs: mode 0 the weighted infinity norm (|v|, times 1e-3 on the temperature
// rows), 1 the minimum, 2 1.0 if any value is not finite. One block per flamelet.
__global__ void k_reduce(int nf, int ns, const int *offz, const double *v, int mode, double *out)
{
  __shared__ double red[kThreads];
  const int f = blockIdx.x;
  if (f >= nf) return;
  const long long lo = (long long)offz[f] * ns, hi = (long long)offz[f + 1] * ns;
  const double inv_t = 1. / 1.e3;
  double acc = mode == 1 ? INFINITY : 0.;
  for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const double x = v[i];
    if (mode == 0) {
      const double w = ((i - lo) % ns == 0) ? fabs(x * inv_t) : fabs(x * 1.);
      acc = fmax(acc, w);
      if (w != w) acc = w;  // NaN wins, as torch's amax does
    } else if (mode == 1) {
      acc = nan_min(acc, x);
    } else if (!isfinite(x)) {
      acc = 1.;
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      const double a = red[threadIdx.x], b = red[threadIdx.x + o];
      red[threadIdx.x] = mode == 1 ? nan_min(a, b) : ((a != a) ? a : ((b != b) ? b : fmax(a, b)));
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[f] = red[0];
}

// dof-parallel updates, masked per flamelet
enum DofOp {
  SELECT = 0,      // dst = m ? a : dst
  ADD_SELECT = 1,  // dst = m ? a + b : dst
  ADD_ALL = 2,     // dst = a + b (every dof)
  SCALE_SELECT = 3,  // dst = m ? dst * s[f] : dst
  ZERO_ELSE_NUM = 4, // dst = m ? nan_to_num(dst) : 0 (nan -> 0, +-inf -> +-DBL_MAX)
  BIG_NUM = 5,     // dst = nan_to_num(dst, nan=1e300, posinf=1e300, neginf=-1e300)
  CLAMP0 = 6,      // dst = max(dst, 0)
  EXPAND_SELECT = 7, // dst = m ? s[f] : dst
  RECIP = 8        // dst = 1 / a
};

__global__ void k_dof(long long N, int ns, int op, const int *map, const int *m, const double *a, const double *b,
                      const double *s, double *dst)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const int f = map ? map[i / ns] : 0;
    const bool on = m ? m[f] != 0 : true;
    switch (op) {
    case SELECT: if (on) dst[i] = a[i]; break;
    case ADD_SELECT: if (on) dst[i] = a[i] + b[i]; break;
    case ADD_ALL: dst[i] = a[i] + b[i]; break;
    case SCALE_SELECT: if (on) dst[i] = dst[i] * s[f]; break;
    case ZERO_ELSE_NUM: {
      const double x = dst[i];
      dst[i] = !on ? 0. : (x != x ? 0. : (isinf(x) ? (x > 0 ? 1.7976931348623157e308 : -1.7976931348623157e308) : x));
      break;
    }
    case BIG_NUM: {
      const double x = dst[i];
      if (x != x) dst[i] = 1e300;
      else if (isinf(x)) dst[i] = x > 0 ? 1e300 : -1e300;
      break;
    }
    case CLAMP0: dst[i] = dst[i] < 0. ? 0. : dst[i]; break;  // torch.clamp(min=0) keeps NaN
    case EXPAND_SELECT: if (on) dst[i] = s[f]; break;
    case RECIP: dst[i] = 1. / a[i]; break;
    }
  }
}

// psitc pseudo-time step: new = min(min(safety / (expeig + 1e-16), ramp * ds), ds_max) per dof (into tmp)
__global__ void k_ds_candidate(long long N, const double *expeig, const double *ds, double safety, double ramp,
                               double dsmax, double *tmp)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
    tmp[i] = nan_min(nan_min(safety / (expeig[i] + 1.e-16), ramp * ds[i]), dsmax);
}

// ds = need ? (first ? mn[f] : tmp) : ds
__global__ void k_ds_apply(long long N, int ns, const int *map, const int *need, const int *first, const double *mn,
                           const double *tmp, double *ds)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const int f = map[i / ns];
    if (need[f]) ds[i] = first[f] ? mn[f] : tmp[i];
  }
}

// ---------------------------------------------------------------------------------- per-flamelet control state
struct Ctl {
  int *run, *failed, *it, *evalj, *go, *need, *cut, *bad, *okgo, *rst, *first, *depth, *jac_age;
  double *res, *norm_old, *nnew, *alpha, *mins, *fin, *dsi, *mn;
  int *flags;  // [4] any-flags read by the host
};

enum CtlOp {
  NEWTON_BEGIN = 0,   // go = run & !failed & res > tol & it < maxit; it += go; need = go & evalj; flags: go, need
  NEWTON_AFTER_J = 1, // evalj &= !need
  FAIL_NONFINITE = 2, // failed |= go & fin; go &= !fin
  LS_CUT = 3,         // cut = go & nnew > mfls * norm_old & alpha > 0.001; alpha = cut ? alpha/2 : alpha; flag
  LS_EVALJ = 4,       // evalj |= cut
  NEWTON_END = 5,     // res = go ? nnew : res; failed |= go & (res > maxres | mins < minvar)
  PSITC_BEGIN = 6,    // go = run & !dead & res > tol & it < maxit; it += go; need = go & evalj; first; flags
  PSITC_AFTER_J = 7,  // jac_age = need ? 0 : jac_age
  PSITC_AGE = 8,      // jac_age += go & !need; evalj = go ? (jac_age == 8 | res > 1e-2) : evalj
  PSITC_BAD_SOLVE = 9,  // bad = go & fin
  PSITC_BAD_RHS = 10,   // bad |= go & fin; okgo = go & !bad; alpha = 1
  PSITC_END = 11,     // res = okgo ? nnew : res; bad |= okgo & (res > maxres | mins < minvar); restart logic; flags
  LS_INIT = 12,       // alpha = 1
  NEWTON_FINISH = 13, // conv = run & !failed & res <= tol & it <= maxit -> out
  PSITC_FINISH = 14   // conv = run & !dead & res <= tol -> out
};

struct CtlArgs {
  int op, nf;
  double tol, mfls, maxres, minvar, ds_init_decrease;
  int maxit, max_depth, adaptive, global_ds;
  int *out_conv, *out_it;
};

__global__ void k_ctl(Ctl c, CtlArgs a)
{
  for (int f = threadIdx.x; f < a.nf; f += blockDim.x) {
    switch (a.op) {
    case NEWTON_BEGIN: {
      const int go = c.run[f] && !c.failed[f] && c.res[f] > a.tol && c.it[f] < a.maxit;
      c.go[f] = go;
      c.it[f] += go;
      c.need[f] = go && c.evalj[f];
      if (go) atomicOr(&c.flags[0], 1);
      if (c.need[f]) atomicOr(&c.flags[1], 1);
      break;
    }
    case NEWTON_AFTER_J: c.evalj[f] = c.evalj[f] && !c.need[f]; break;
    case FAIL_NONFINITE: {
      const int bad = c.go[f] && c.fin[f] != 0.;
      c.failed[f] = c.failed[f] || bad;
      c.go[f] = c.go[f] && !bad;
      break;
    }
    case LS_INIT: c.alpha[f] = 1.; break;
    case LS_CUT: {
      const int cut = c.go[f] && c.nnew[f] > a.mfls * c.norm_old[f] && c.alpha[f] > 0.001;
      c.cut[f] = cut;
      if (cut) {
        c.alpha[f] = c.alpha[f] * 0.5;
        atomicOr(&c.flags[2], 1);
      }
      break;
    }
    case LS_EVALJ: c.evalj[f] = c.evalj[f] || c.cut[f]; break;
    case NEWTON_END:
      if (c.go[f]) {
        c.res[f] = c.nnew[f];
        if (c.res[f] > a.maxres) c.failed[f] = 1;
        if (c.mins[f] < a.minvar) c.failed[f] = 1;
      }
      break;
    case PSITC_BEGIN: {
      const int go = c.run[f] && !c.failed[f] && c.res[f] > a.tol && c.it[f] < a.maxit;
      c.go[f] = go;
      c.it[f] += go;
      c.need[f] = go && c.evalj[f];
      c.first[f] = c.need[f] && (c.it[f] == 1 || a.global_ds);
      if (go) atomicOr(&c.flags[0], 1);
      if (c.need[f]) atomicOr(&c.flags[1], 1);
      break;
    }
    case PSITC_AFTER_J: if (c.need[f]) c.jac_age[f] = 0; break;
    case PSITC_AGE:
      if (c.go[f] && !c.need[f]) c.jac_age[f] += 1;
      if (c.go[f]) c.evalj[f] = (c.jac_age[f] == 8) || (c.res[f] > 1.e-2);
      break;
    case PSITC_BAD_SOLVE: c.bad[f] = c.go[f] && c.fin[f] != 0.; break;
    case PSITC_BAD_RHS:
      c.bad[f] = c.bad[f] || (c.go[f] && c.fin[f] != 0.);
      c.okgo[f] = c.go[f] && !c.bad[f];
      c.alpha[f] = 1.;
      break;
    case PSITC_END: {
      if (c.okgo[f]) {
        c.res[f] = c.nnew[f];
        if (c.res[f] > a.maxres || c.mins[f] < a.minvar) c.bad[f] = 1;
      }
      c.rst[f] = 0;
      if (c.bad[f]) {
        const int give_up = c.depth[f] > a.max_depth || !a.adaptive;
        if (give_up) {
          c.failed[f] = 1;  // dead
        } else {
          c.rst[f] = 1;
          c.depth[f] += 1;
          c.dsi[f] = c.dsi[f] / a.ds_init_decrease;
          c.it[f] = 0;
          c.jac_age[f] = 0;
          c.res[f] = a.tol + 1.;
          c.evalj[f] = 1;
          atomicOr(&c.flags[3], 1);
        }
      }
      break;
    }
    case NEWTON_FINISH:
      a.out_conv[f] = c.run[f] && !c.failed[f] && c.res[f] <= a.tol && c.it[f] <= a.maxit;
      a.out_it[f] = c.it[f];
      break;
    case PSITC_FINISH:
      a.out_conv[f] = c.run[f] && !c.failed[f] && c.res[f] <= a.tol;
      a.out_it[f] = c.it[f];
      break;
    }
  }
}

__global__ void k_ctl_init(Ctl c, int nf, const int *active, double res0, double dsi0)
{
  for (int f = threadIdx.x; f < nf; f += blockDim.x) {
    c.run[f] = active ? (active[f] != 0) : 1;
    c.failed[f] = 0;
    c.it[f] = 0;
    c.evalj[f] = 1;
    c.res[f] = res0;
    c.depth[f] = 0;
    c.jac_age[f] = 0;
    c.dsi[f] = dsi0;
    c.alpha[f] = 1.;
  }
}

__global__ void k_flags_clear(int *flags)
{
  if (threadIdx.x < 4) flags[threadIdx.x] = 0;
}

// ---------------------------------------------------------------------------------------------- workspace
struct Layout {
  long long N, V, P;
  int nf;
  size_t bytes;
  size_t off[32];
};

size_t up(size_t b) { return (b + 255) & ~(size_t)255; }

// 0 values, 1 lvalues, 2 pivots, 3 rhs, 4 rhs_new, 5 dstate, 6 trial, 7 expeig, 8 ds, 9 tmp, 10 initial, 11 zeros,
// 12 map, 13 ctl ints (13 x nf), 14 ctl doubles (8 x nf), 15 flags, 16 eigenvalue kernel counter
Layout layout(const sf_mech *mech, const sf_flamelet_batch *fb)
{
  Layout L{};
  const int ns = mech->m.dm.ns;
  L.nf = fb->n_flamelets;
  L.P = fb->offsets_z_host[L.nf];
  L.N = L.P * ns;
  L.V = 0;
  for (int f = 0; f < L.nf; ++f) {
    const long long nb = fb->offsets_z_host[f + 1] - fb->offsets_z_host[f];
    L.V += (long long)ns * (nb * ns + 2 * (nb - 1));
  }
  const size_t sizes[17] = {(size_t)L.V * 8, (size_t)L.P * ns * ns * 8, (size_t)L.P * ns * 4,
                            (size_t)L.N * 8, (size_t)L.N * 8, (size_t)L.N * 8, (size_t)L.N * 8, (size_t)L.N * 8,
                            (size_t)L.N * 8, (size_t)L.N * 8, (size_t)L.N * 8, (size_t)L.N * 8, (size_t)L.P * 4,
                            (size_t)13 * L.nf * 4, (size_t)8 * L.nf * 8, 16,
                            std::max<size_t>(256, sf_flamelet_jac_workspace_size(mech, 1))};
  size_t o = 0;
  for (int k = 0; k < 17; ++k) {
    L.off[k] = o;
    o += up(sizes[k]);
  }
  L.bytes = o;
  return L;
}

struct Solver {
  const sf_mech *mech;
  sf_flamelet_batch fb;  // a copy whose active mask this solver sets per call
  Layout L;
  int ns;
  cudaStream_t st;
  char *w;
  double *values, *lvalues, *rhs, *rhs_new, *dstate, *trial, *expeig, *ds, *tmp, *initial, *zeros;
  int *pivots, *map;
  Ctl c;
  void *eig_ws;

  template <class T>
  T *at(int k) const { return reinterpret_cast<T *>(w + L.off[k]); }

  Solver(const sf_mech *m, const sf_flamelet_batch *b, void *ws, cudaStream_t s) : mech(m), fb(*b), st(s)
  {
    L = layout(m, b);
    ns = m->m.dm.ns;
    w = static_cast<char *>(ws);
    values = at<double>(0);
    lvalues = at<double>(1);
    pivots = at<int>(2);
    rhs = at<double>(3);
    rhs_new = at<double>(4);
    dstate = at<double>(5);
    trial = at<double>(6);
    expeig = at<double>(7);
    ds = at<double>(8);
    tmp = at<double>(9);
    initial = at<double>(10);
    zeros = at<double>(11);
    map = at<int>(12);
    int *ci = at<int>(13);
    const int nf = L.nf;
    c.run = ci;
    c.failed = ci + nf;
    c.it = ci + 2 * nf;
    c.evalj = ci + 3 * nf;
    c.go = ci + 4 * nf;
    c.need = ci + 5 * nf;
    c.cut = ci + 6 * nf;
    c.bad = ci + 7 * nf;
    c.okgo = ci + 8 * nf;
    c.rst = ci + 9 * nf;
    c.first = ci + 10 * nf;
    c.depth = ci + 11 * nf;
    c.jac_age = ci + 12 * nf;
    double *cd = at<double>(14);
    c.res = cd;
    c.norm_old = cd + nf;
    c.nnew = cd + 2 * nf;
    c.alpha = cd + 3 * nf;
    c.mins = cd + 4 * nf;
    c.fin = cd + 5 * nf;
    c.dsi = cd + 6 * nf;
    c.mn = cd + 7 * nf;
    c.flags = at<int>(15);
    eig_ws = at<char>(16);
    fb.active = nullptr;
    fb.prefactor = nullptr;
    fb.diffterm = nullptr;
  }

  void check(int rc) const
  {
    if (rc != SF_OK) throw sf_error(rc, sf_last_error());
  }
  void cuda() const { CUDA_THROW(cudaGetLastError()); }

  void dof(int op, const int *m, const double *a, const double *b, const double *s, double *dst)
  {
    k_dof<<<grid_for(L.N), kThreads, 0, st>>>(L.N, ns, op, map, m, a, b, s, dst);
    cuda();
  }
  void reduce(const double *v, int mode, double *out)
  {
    k_reduce<<<L.nf, kThreads, 0, st>>>(L.nf, ns, fb.offsets_z, v, mode, out);
    cuda();
  }
  void ctl(CtlArgs a)
  {
    a.nf = L.nf;
    k_ctl<<<1, 1024, 0, st>>>(c, a);
    cuda();
  }
  void clear_flags()
  {
    k_flags_clear<<<1, 32, 0, st>>>(c.flags);
    cuda();
  }
  void read_flags(int *h)
  {
    CUDA_THROW(cudaMemcpyAsync(h, c.flags, 4 * sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_THROW(cudaStreamSynchronize(st));
  }
  void rhs_of(const double *x, const int *m, double *out)
  {
    fb.active = m;
    const int rc = sf_flamelet_rhs_batch(mech, &fb, x, out, st);
    fb.active = nullptr;
    check(rc);
  }
  void factor(const int *m)
  {
    check(sf_btddod_factor_batch(L.nf, ns, fb.offsets_z, fb.offsets_v, fb.offsets_z_host, values, lvalues, pivots,
                                 m, st));
  }
  void solve(const double *b, double *x, const int *m)
  {
    check(sf_btddod_solve_batch(L.nf, ns, fb.offsets_z, fb.offsets_v, fb.offsets_z_host, values, lvalues, pivots, b,
                                x, m, st));
  }
  void scale_diag(double ms, const double *d, double dsc, const int *m)
  {
    check(sf_btddod_scale_and_add_diagonal_batch(L.nf, ns, fb.offsets_z, fb.offsets_v, fb.offsets_z_host, values,
                                                 ms, d, dsc, m, st));
  }
  void setup_common(const double *state, const int *active, double res0, double dsi0)
  {
    k_point_map<<<L.nf, kThreads, 0, st>>>(L.nf, fb.offsets_z, map);
    cuda();
    k_ctl_init<<<1, 1024, 0, st>>>(c, L.nf, active, res0, dsi0);
    cuda();
    CUDA_THROW(cudaMemsetAsync(zeros, 0, (size_t)L.N * 8, st));
    CUDA_THROW(cudaMemsetAsync(dstate, 0, (size_t)L.N * 8, st));
    CUDA_THROW(cudaMemcpyAsync(initial, state, (size_t)L.N * 8, cudaMemcpyDeviceToDevice, st));
  }
};

// ------------------------------------------------------------------------- transient step attempt (ESDIRK64)
// Elementwise arithmetic below is written with explicit roundings (no fused multiply-adds), in the order the
// batch's host-loop integrator evaluates it with separate tensor operations, so both give the same bits.
struct AttBufs {
  long long N;
  int ns, nf;
  const int *map;
  double *k;  // 6 stage derivatives, N each
  double *Y, *fs, *resid, *prior, *dx, *dstate, *eterm;
  const double *dt;  // [nf]
  double *state;
};

__global__ void k_att_stage_start(AttBufs a, int st)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += (long long)gridDim.x * blockDim.x) {
    const double dtd = a.dt[a.map[i / a.ns]];
    double pr = __dmul_rn(c_a[st][0], a.k[i]);
    for (int j = 1; j < st; ++j) pr = __dadd_rn(pr, __dmul_rn(c_a[st][j], a.k[(long long)j * a.N + i]));
    a.prior[i] = pr;
    const double f = a.k[(long long)(st - 1) * a.N + i];
    a.fs[i] = f;
    a.resid[i] = __dsub_rn(__dmul_rn(dtd, __dadd_rn(__dmul_rn(kGamma, f), pr)), __dsub_rn(a.Y[i], a.state[i]));
  }
}

// Y <- Y - dx where go
__global__ void k_att_newton_update(AttBufs a, const int *go)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += (long long)gridDim.x * blockDim.x)
    if (go[a.map[i / a.ns]]) a.Y[i] = __dsub_rn(a.Y[i], a.dx[i]);
}

// residual at the new iterate where go
__global__ void k_att_newton_resid(AttBufs a, const int *go)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += (long long)gridDim.x * blockDim.x) {
    const int f = a.map[i / a.ns];
    if (go[f])
      a.resid[i] = __dsub_rn(__dmul_rn(a.dt[f], __dadd_rn(__dmul_rn(kGamma, a.fs[i]), a.prior[i])),
                             __dsub_rn(a.Y[i], a.state[i]));
  }
}

// the step dt * sum_s b_s k_s and the error term dt * sum_s (b_s - bhat_s) k_s
__global__ void k_att_step(AttBufs a)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += (long long)gridDim.x * blockDim.x) {
    const double dtd = a.dt[a.map[i / a.ns]];
    double ds = __dmul_rn(c_b[0], a.k[i]);
    double de = __dmul_rn(__dsub_rn(c_b[0], c_bh[0]), a.k[i]);
    for (int j = 1; j < 6; ++j) {
      const double kj = a.k[(long long)j * a.N + i];
      ds = __dadd_rn(ds, __dmul_rn(c_b[j], kj));
      de = __dadd_rn(de, __dmul_rn(__dsub_rn(c_b[j], c_bh[j]), kj));
    }
    a.dstate[i] = __dmul_rn(dtd, ds);
    a.eterm[i] = __dmul_rn(dtd, de);
  }
}

// state <- max(state + step, 0) where the flamelet runs and its step is finite (fin[f] == 0: no non-finite entry)
__global__ void k_att_accept(AttBufs a, const int *run, const double *nonfinite)
{
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.N; i += (long long)gridDim.x * blockDim.x) {
    const int f = a.map[i / a.ns];
    if (run[f] && nonfinite[f] == 0.) {
      const double v = __dadd_rn(a.state[i], a.dstate[i]);
      a.state[i] = v < 0. ? 0. : v;
    }
  }
}

// per-flamelet bookkeeping of the attempt: 0 start of a stage (go = run, conv = 0), 1 newton += go,
// 2 convergence test (nrm < tol) and the any-go flag, 3 end of a stage (nl_ok &= conv | !run),
// 4 start of the attempt (prefactors gamma * dt, nl_ok = 1)
struct AttCtl {
  const int *run;
  int *go, *conv, *nl_ok, *newton, *flags;
  double *nrm, *pref;
  const double *dt;
};

__global__ void k_att_ctl(AttCtl c, int nf, int op, double tol)
{
  for (int f = threadIdx.x; f < nf; f += blockDim.x) {
    switch (op) {
    case 0: c.go[f] = c.run[f] != 0; c.conv[f] = 0; break;
    case 1: c.newton[f] += c.go[f]; break;
    case 2:
      if (c.go[f] && c.nrm[f] < tol) {
        c.conv[f] = 1;
        c.go[f] = 0;
      }
      if (c.go[f]) atomicOr(&c.flags[0], 1);
      break;
    case 3: c.nl_ok[f] = c.nl_ok[f] && (c.conv[f] || !c.run[f]); break;
    case 4: c.pref[f] = __dmul_rn(c.dt[f], kGamma); c.nl_ok[f] = 1; break;
    }
  }
}

// Workspace of an attempt: 0 values, 1 lvalues, 2 pivots (the iteration matrix factors, kept from one attempt to
// the next), 3 stage derivatives (6 N), 4 Y, 5 fs, 6 resid, 7 prior, 8 dx, 9 dstate, 10 eterm, 11 map,
// 12 ints (go, conv, flags), 13 doubles (nrm, pref)
Layout att_layout(const sf_mech *mech, const sf_flamelet_batch *fb)
{
  Layout L{};
  const int ns = mech->m.dm.ns;
  L.nf = fb->n_flamelets;
  L.P = fb->offsets_z_host[L.nf];
  L.N = L.P * ns;
  L.V = 0;
  for (int f = 0; f < L.nf; ++f) {
    const long long nb = fb->offsets_z_host[f + 1] - fb->offsets_z_host[f];
    L.V += (long long)ns * (nb * ns + 2 * (nb - 1));
  }
  const size_t N8 = (size_t)L.N * 8;
  const size_t sizes[14] = {(size_t)L.V * 8, (size_t)L.P * ns * ns * 8, (size_t)L.P * ns * 4, 6 * N8, N8, N8, N8,
                            N8, N8, N8, N8, (size_t)L.P * 4, (size_t)(2 * L.nf + 16) * 4, (size_t)2 * L.nf * 8};
  size_t o = 0;
  for (int k = 0; k < 14; ++k) {
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

size_t sf_flamelet_steady_workspace_size(const sf_mech *mech, const sf_flamelet_batch *fb)
{
  if (!mech || !fb || fb->n_flamelets < 1 || !fb->offsets_z_host) return 0;
  return layout(mech, fb).bytes;
}

int sf_flamelet_steady_newton_batch(const sf_mech *mech, const sf_flamelet_batch *fb, double *state,
                                    const int *active, double tolerance, int max_iterations,
                                    double max_factor_line_search, double max_allowed_residual,
                                    double min_allowable_state_var, int rates_option, int *out_converged,
                                    int *out_iterations, void *workspace, size_t workspace_bytes, void *stream)
{
  try {
    if (!mech || !fb || !state || !out_converged || !out_iterations || max_iterations < 0)
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "sf_flamelet_steady_newton_batch: bad argument");
    if (!workspace || workspace_bytes < sf_flamelet_steady_workspace_size(mech, fb))
      throw sf_error(SF_ERR_WORKSPACE, "workspace smaller than sf_flamelet_steady_workspace_size reports");
    Solver S(mech, fb, workspace, (cudaStream_t)stream);
    S.setup_common(state, active, tolerance + 1., 1.);
    CtlArgs a{};
    a.tol = tolerance;
    a.maxit = max_iterations;
    a.mfls = max_factor_line_search;
    a.maxres = max_allowed_residual;
    a.minvar = min_allowable_state_var;
    S.rhs_of(state, S.c.run, S.rhs);
    int h[4];
    for (int pass = 0; pass <= max_iterations; ++pass) {
      S.clear_flags();
      a.op = NEWTON_BEGIN;
      S.ctl(a);
      S.read_flags(h);
      if (!h[0]) break;
      if (h[1]) {
        S.fb.active = S.c.need;
        S.check(sf_flamelet_jac_batch(mech, &S.fb, state, rates_option, 0, 0., 0., nullptr, S.values, nullptr, 0,
                                      S.st));
        S.fb.active = nullptr;
        S.scale_diag(-1., S.zeros, 0., S.c.need);  // J <- -J
        S.factor(S.c.need);
        a.op = NEWTON_AFTER_J;
        S.ctl(a);
      }
      S.solve(S.rhs, S.dstate, S.c.go);
      S.reduce(S.dstate, 2, S.c.fin);
      a.op = FAIL_NONFINITE;
      S.ctl(a);
      S.dof(ZERO_ELSE_NUM, S.c.go, nullptr, nullptr, nullptr, S.dstate);  // go: the step, others 0
      S.reduce(S.rhs, 0, S.c.norm_old);
      S.dof(ADD_ALL, nullptr, state, S.dstate, nullptr, S.trial);
      S.rhs_of(S.trial, S.c.go, S.rhs_new);
      S.reduce(S.rhs_new, 2, S.c.fin);
      a.op = FAIL_NONFINITE;
      S.ctl(a);
      a.op = LS_INIT;
      S.ctl(a);
      for (int ls = 0; ls < 12; ++ls) {
        S.reduce(S.rhs_new, 0, S.c.nnew);
        S.clear_flags();
        a.op = LS_CUT;
        S.ctl(a);
        S.read_flags(h);
        if (!h[2]) break;
        S.dof(SCALE_SELECT, S.c.cut, nullptr, nullptr, S.c.alpha, S.dstate);
        S.dof(ADD_ALL, nullptr, state, S.dstate, nullptr, S.trial);
        S.rhs_of(S.trial, S.c.cut, S.tmp);
        S.dof(SELECT, S.c.cut, S.tmp, nullptr, nullptr, S.rhs_new);
        a.op = LS_EVALJ;
        S.ctl(a);
      }
      S.dof(ADD_SELECT, S.c.go, state, S.dstate, nullptr, state);
      S.dof(SELECT, S.c.go, S.rhs_new, nullptr, nullptr, S.rhs);
      S.reduce(S.rhs, 0, S.c.nnew);
      S.reduce(state, 1, S.c.mins);
      a.op = NEWTON_END;
      S.ctl(a);
    }
    S.dof(CLAMP0, nullptr, nullptr, nullptr, nullptr, state);
    a.op = NEWTON_FINISH;
    a.out_conv = out_converged;
    a.out_it = out_iterations;
    S.ctl(a);
    return SF_OK;
  } catch (sf_error &e) {
    set_error(e.what());
    return e.code;
  }
}

int sf_flamelet_steady_psitc_batch(const sf_mech *mech, const sf_flamelet_batch *fb, double *state,
                                   const int *active, const double *diffterm, double tolerance, int max_iterations,
                                   double min_allowable_state_var, double ds_init, double ds_init_decrease,
                                   int global_ds, double ds_safety, double ds_ramp, double ds_max,
                                   double max_factor_line_search, double max_allowed_residual,
                                   int max_recursion_depth, int adaptive_restart, int rates_option,
                                   int *out_converged, int *out_iterations, double *out_min_ds, void *workspace,
                                   size_t workspace_bytes, void *stream)
{
  try {
    if (!mech || !fb || !state || !diffterm || !out_converged || !out_iterations || max_iterations < 0)
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "sf_flamelet_steady_psitc_batch: bad argument");
    if (!workspace || workspace_bytes < sf_flamelet_steady_workspace_size(mech, fb))
      throw sf_error(SF_ERR_WORKSPACE, "workspace smaller than sf_flamelet_steady_workspace_size reports");
    Solver S(mech, fb, workspace, (cudaStream_t)stream);
    S.setup_common(state, active, tolerance + 1., ds_init);
    S.dof(EXPAND_SELECT, nullptr, nullptr, nullptr, S.c.dsi, S.ds);  // ds = expand(dsi)
    CtlArgs a{};
    a.tol = tolerance;
    a.maxit = max_iterations;
    a.mfls = max_factor_line_search;
    a.maxres = max_allowed_residual;
    a.minvar = min_allowable_state_var;
    a.ds_init_decrease = ds_init_decrease;
    a.max_depth = max_recursion_depth;
    a.adaptive = adaptive_restart ? 1 : 0;
    a.global_ds = global_ds ? 1 : 0;
    S.rhs_of(state, S.c.run, S.rhs);
    const long long total_cap = (long long)(max_iterations + 1) * (max_recursion_depth + 3);
    int h[4];
    for (long long pass = 0; pass < total_cap; ++pass) {
      S.clear_flags();
      a.op = PSITC_BEGIN;
      S.ctl(a);
      S.read_flags(h);
      if (!h[0]) break;
      if (h[1]) {
        sf_flamelet_batch j = S.fb;
        j.active = S.c.need;
        j.diffterm = diffterm;
        S.check(sf_flamelet_jac_batch(mech, &j, state, rates_option, 0, 0., 0., S.expeig, S.values, S.eig_ws,
                                      sf_flamelet_jac_workspace_size(mech, 1), S.st));
        k_ds_candidate<<<grid_for(S.L.N), kThreads, 0, S.st>>>(S.L.N, S.expeig, S.ds, ds_safety, ds_ramp, ds_max,
                                                                S.tmp);
        S.cuda();
        S.reduce(S.tmp, 1, S.c.mn);
        k_ds_apply<<<grid_for(S.L.N), kThreads, 0, S.st>>>(S.L.N, S.ns, S.map, S.c.need, S.c.first, S.c.mn, S.tmp,
                                                            S.ds);
        S.cuda();
        S.dof(RECIP, nullptr, S.ds, nullptr, nullptr, S.tmp);  // 1 / ds
        S.scale_diag(-1., S.tmp, 1., S.c.need);              // J <- -J + diag(1 / ds)
        S.factor(S.c.need);
        a.op = PSITC_AFTER_J;
        S.ctl(a);
      }
      a.op = PSITC_AGE;
      S.ctl(a);
      S.solve(S.rhs, S.dstate, S.c.go);
      S.reduce(S.dstate, 2, S.c.fin);
      a.op = PSITC_BAD_SOLVE;
      S.ctl(a);
      S.dof(ZERO_ELSE_NUM, S.c.go, nullptr, nullptr, nullptr, S.dstate);
      S.reduce(S.rhs, 0, S.c.norm_old);
      S.dof(ADD_ALL, nullptr, state, S.dstate, nullptr, S.trial);
      S.rhs_of(S.trial, S.c.go, S.rhs_new);
      S.reduce(S.rhs_new, 2, S.c.fin);
      a.op = PSITC_BAD_RHS;  // also okgo and alpha = 1
      S.ctl(a);
      S.dof(BIG_NUM, nullptr, nullptr, nullptr, nullptr, S.rhs_new);
      for (int ls = 0; ls < 12; ++ls) {
        S.reduce(S.rhs_new, 0, S.c.nnew);
        S.clear_flags();
        int *save_go = S.c.go;
        S.c.go = S.c.okgo;  // the line search runs over the flamelets whose step is finite
        a.op = LS_CUT;
        S.ctl(a);
        S.c.go = save_go;
        S.read_flags(h);
        if (!h[2]) break;
        S.dof(SCALE_SELECT, S.c.cut, nullptr, nullptr, S.c.alpha, S.dstate);
        S.dof(ADD_ALL, nullptr, state, S.dstate, nullptr, S.trial);
        S.rhs_of(S.trial, S.c.cut, S.tmp);
        S.dof(SELECT, S.c.cut, S.tmp, nullptr, nullptr, S.rhs_new);
        a.op = LS_EVALJ;
        S.ctl(a);
      }
      S.dof(ADD_SELECT, S.c.okgo, state, S.dstate, nullptr, state);
      S.dof(SELECT, S.c.okgo, S.rhs_new, nullptr, nullptr, S.rhs);
      S.reduce(S.rhs, 0, S.c.nnew);
      S.reduce(state, 1, S.c.mins);
      S.clear_flags();
      a.op = PSITC_END;  // residual, failure tests and the restart bookkeeping
      S.ctl(a);
      S.read_flags(h);
      if (h[3]) {  // restart the failed flamelets from the initial guess with a smaller first pseudo-time step
        S.dof(SELECT, S.c.rst, S.initial, nullptr, nullptr, state);
        S.dof(EXPAND_SELECT, S.c.rst, nullptr, nullptr, S.c.dsi, S.ds);
        S.rhs_of(state, S.c.rst, S.tmp);
        S.dof(SELECT, S.c.rst, S.tmp, nullptr, nullptr, S.rhs);
      }
    }
    S.dof(CLAMP0, nullptr, nullptr, nullptr, nullptr, state);
    a.op = PSITC_FINISH;
    a.out_conv = out_converged;
    a.out_it = out_iterations;
    S.ctl(a);
    if (out_min_ds) S.reduce(S.ds, 1, out_min_ds);
    return SF_OK;
  } catch (sf_error &e) {
    set_error(e.what());
    return e.code;
  }
}

size_t sf_flamelet_esdirk_workspace_size(const sf_mech *mech, const sf_flamelet_batch *fb)
{
  if (!mech || !fb || fb->n_flamelets < 1 || !fb->offsets_z_host) return 0;
  return att_layout(mech, fb).bytes;
}

int sf_flamelet_esdirk_attempt_batch(const sf_mech *mech, const sf_flamelet_batch *fb, double *state,
                                     const double *dt, const int *run, const int *setup, int any_setup,
                                     double nonlinear_tolerance, int max_nonlinear_iter, int rates_option,
                                     double *out_err, double *out_step_norm, double *out_nonfinite, int *out_nl_ok,
                                     int *inout_newton, void *workspace, size_t workspace_bytes, void *stream)
{
  try {
    if (!mech || !fb || !state || !dt || !run || !setup || !out_err || !out_step_norm || !out_nonfinite ||
        !out_nl_ok || !inout_newton || max_nonlinear_iter < 1)
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "sf_flamelet_esdirk_attempt_batch: bad argument");
    if (!workspace || workspace_bytes < sf_flamelet_esdirk_workspace_size(mech, fb))
      throw sf_error(SF_ERR_WORKSPACE, "workspace smaller than sf_flamelet_esdirk_workspace_size reports");
    const Layout L = att_layout(mech, fb);
    const int ns = mech->m.dm.ns, nf = L.nf;
    cudaStream_t st = (cudaStream_t)stream;
    char *w = static_cast<char *>(workspace);
    double *values = reinterpret_cast<double *>(w + L.off[0]);
    double *lvalues = reinterpret_cast<double *>(w + L.off[1]);
    int *pivots = reinterpret_cast<int *>(w + L.off[2]);
    AttBufs a{};
    a.N = L.N;
    a.ns = ns;
    a.nf = nf;
    a.k = reinterpret_cast<double *>(w + L.off[3]);
    a.Y = reinterpret_cast<double *>(w + L.off[4]);
    a.fs = reinterpret_cast<double *>(w + L.off[5]);
    a.resid = reinterpret_cast<double *>(w + L.off[6]);
    a.prior = reinterpret_cast<double *>(w + L.off[7]);
    a.dx = reinterpret_cast<double *>(w + L.off[8]);
    a.dstate = reinterpret_cast<double *>(w + L.off[9]);
    a.eterm = reinterpret_cast<double *>(w + L.off[10]);
    int *map = reinterpret_cast<int *>(w + L.off[11]);
    a.map = map;
    a.dt = dt;
    a.state = state;
    int *ci = reinterpret_cast<int *>(w + L.off[12]);
    double *cd = reinterpret_cast<double *>(w + L.off[13]);
    AttCtl c{};
    c.run = run;
    c.go = ci;
    c.conv = ci + nf;
    c.flags = ci + 2 * nf;
    c.nl_ok = out_nl_ok;
    c.newton = inout_newton;
    c.nrm = cd;
    c.pref = cd + nf;
    c.dt = dt;
    const int grid = grid_for(L.N);
    auto cuda = [] { CUDA_THROW(cudaGetLastError()); };
    auto ctl = [&](int op) {
      k_att_ctl<<<1, 1024, 0, st>>>(c, nf, op, nonlinear_tolerance);
      cuda();
    };
    auto reduce = [&](const double *v, int mode, double *out) {
      k_reduce<<<nf, kThreads, 0, st>>>(nf, ns, fb->offsets_z, v, mode, out);
      cuda();
    };
    auto check = [](int rc) {
      if (rc != SF_OK) throw sf_error(rc, sf_last_error());
    };
    sf_flamelet_batch b = *fb;
    b.diffterm = nullptr;
    b.prefactor = nullptr;
    k_point_map<<<nf, kThreads, 0, st>>>(nf, fb->offsets_z, map);
    cuda();
    ctl(4);  // prefactors gamma * dt; nl_ok = 1
    if (any_setup) {
      // the iteration matrix gamma dt J - I of every flamelet that needs a new one, with its own prefactor
      b.active = setup;
      b.prefactor = c.pref;
      check(sf_flamelet_jac_batch(mech, &b, state, rates_option, 1, 0., 0., nullptr, values, nullptr, 0, stream));
      b.prefactor = nullptr;
      check(sf_btddod_factor_batch(nf, ns, fb->offsets_z, fb->offsets_v, fb->offsets_z_host, values, lvalues, pivots,
                                   setup, stream));
    }
    b.active = run;
    check(sf_flamelet_rhs_batch(mech, &b, state, a.k, stream));  // k_0
    CUDA_THROW(cudaMemcpyAsync(a.Y, state, (size_t)L.N * 8, cudaMemcpyDeviceToDevice, st));
    int hflag = 0;
    for (int s = 1; s < 6; ++s) {
      k_att_stage_start<<<grid, kThreads, 0, st>>>(a, s);
      cuda();
      ctl(0);
      for (int it = 0; it < max_nonlinear_iter; ++it) {
        ctl(1);
        check(sf_btddod_solve_batch(nf, ns, fb->offsets_z, fb->offsets_v, fb->offsets_z_host, values, lvalues,
                                    pivots, a.resid, a.dx, c.go, stream));
        k_att_newton_update<<<grid, kThreads, 0, st>>>(a, c.go);
        cuda();
        b.active = c.go;
        check(sf_flamelet_rhs_batch(mech, &b, a.Y, a.fs, stream));
        k_att_newton_resid<<<grid, kThreads, 0, st>>>(a, c.go);
        cuda();
        reduce(a.resid, 0, c.nrm);
        CUDA_THROW(cudaMemsetAsync(c.flags, 0, sizeof(int), st));
        ctl(2);
        CUDA_THROW(cudaMemcpyAsync(&hflag, c.flags, sizeof(int), cudaMemcpyDeviceToHost, st));
        CUDA_THROW(cudaStreamSynchronize(st));
        if (!hflag) break;
      }
      CUDA_THROW(cudaMemcpyAsync(a.k + (size_t)s * L.N, a.fs, (size_t)L.N * 8, cudaMemcpyDeviceToDevice, st));
      ctl(3);
    }
    k_att_step<<<grid, kThreads, 0, st>>>(a);
    cuda();
    reduce(a.eterm, 0, out_err);
    reduce(a.dstate, 0, out_step_norm);
    reduce(a.dstate, 2, out_nonfinite);
    k_att_accept<<<grid, kThreads, 0, st>>>(a, run, out_nonfinite);
    cuda();
    return SF_OK;
  } catch (sf_error &e) {
    set_error(e.what());
    return e.code;
  }
}

}  // extern "C"
