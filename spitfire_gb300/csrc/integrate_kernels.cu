// Batched adaptive ESDIRK64 integration of closed homogeneous reactors in one persistent launch.
//
// One warp integrates one reactor at a time and takes the next unfinished reactor from an atomic work queue when
// it is done, so reactors with ten times more steps than others do not hold the rest back. Everything a reactor
// needs between steps lives in the warp's shared memory: the state, the six stage derivatives, the Newton
// iteration matrix A = dt*gamma*J - I and its LU factors, and the Griffon scratch of the right-hand side and
// Jacobian evaluations.
//
// The step logic restates the reference's default reactor integration exactly, so that the accepted-step sequence
// (and therefore the ignition delay, the end time of the first accepted step with T > T0 + delta) is the same:
//   odesolve governor        src/spitfire/time/integrator.py:520-640 (Jacobian setup policy :100-130, failed
//                            steps :82-97, stop rules :629-640)
//   KennedyCarpenterS6P4Q3   src/spitfire/time/methods.py:441-612 (tableau :464-500)
//   SimpleNewtonSolver       src/spitfire/time/nonlinear.py:185-268 (frozen Jacobian, inf-norm test, 20 iterations)
//   PIController             src/spitfire/time/stepcontrol.py:84-101 (after the first step the P factor is 1)
//   HomogeneousReactor       src/spitfire/chemistry/reactors.py:429-611 (weights 1/[1e3 on T], clamp of negative
//                            entries after each step)
#include "reactor_eval.cuh"
#include "sf_internal.h"
#include "warp_lu.cuh"
#include "esdirk64.cuh"

namespace sfgb {
namespace {

// Gather batch of the reactor evaluations inside the integrator: unbatched measured fastest there (the warp's scratch
// is in shared memory or L2, and the integrator kernel has no registers to spare for operands in flight).
constexpr int kIntegratorUnroll = 1;

struct IntParams {
  DevMech m;
  const void *blob;
  int *status;
  ScratchLayout L;
  Progs pg;
  ReactorCfg cfg;
  sf_integrate_params ip;
  int n, neq, prec;
  double pressure;
  const double *pressures, *q0;
  double *out_q, *out_t;
  int *out_counts, *out_status;
  unsigned int *queue;
  size_t per_warp;  // doubles of shared memory per warp
  double *rec;      // optional trajectory record: [n][rec_cap][2 + 6 neq] = (t_n, dt_n, stage values Y_1..Y_6)
  int rec_cap;
  double *gscratch; // if set: Griffon scratch of every resident warp in global memory ([grid * warps][L.total])
  double *gmat;     // if set: iteration matrix (and FP32 factors) of every resident warp in global memory
  size_t mat_doubles;
  int warps;
};

// First time in [t0, t0 + h] at which the cubic Hermite interpolant of a quantity with end values y0, y1 and end
// derivatives d0, d1 reaches thr (y0 <= thr < y1): the first of 16 equal sub-intervals with a crossing, then 48
// bisections. Uniform arithmetic in every lane.
__device__ __forceinline__ double hermite_crossing(double t0, double h, double y0, double y1, double d0, double d1,
                                                   double thr)
{
  auto p = [&](double s) {
    const double s2 = s * s, s3 = s2 * s;
    return (2. * s3 - 3. * s2 + 1.) * y0 + (s3 - 2. * s2 + s) * h * d0 + (3. * s2 - 2. * s3) * y1 +
           (s3 - s2) * h * d1;
  };
  double lo = 0., hi = 1.;
  for (int j = 1; j <= 16; ++j) {
    const double s = j / 16.;
    if (p(s) >= thr) {
      lo = (j - 1) / 16.;
      hi = s;
      break;
    }
  }
  for (int it = 0; it < 48; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (p(mid) >= thr) hi = mid;
    else lo = mid;
  }
  return t0 + hi * h;
}

// Writes A = pref * J - I straight from the Jacobian evaluation.
struct IterMatrix {
  double *A;
  int neq;
  double pref;
  __device__ __forceinline__ void operator()(int row, int col, double v) const
  {
    A[col * neq + row] = pref * v - (row == col ? 1. : 0.);
  }
};

// Time-dependent reactor parameters at integration-local time t: every column of the time table is its 4-point
// (cubic) Lagrange interpolant in time, held constant beyond the table's ends. At a spacing of the first time step
// the interpolation error, fourth order in the spacing, is far below the rounding of the values, so the right-hand
// side sees the parameter functions themselves. Sets the parameters of time_columns in cf; the feed mass fractions
// go to ybuf (ns doubles of the warp's shared memory), which cf.yin then points to.
__device__ __noinline__ void apply_time_params(const IntParams &p, ReactorCfg &cf, double t, double *ybuf, int ns)
{
  const sf_integrate_params &ip = p.ip;
  const double *tab = ip.time_table;
  const int W = ip.time_width, last = ip.time_points - 1;
  const double u = (t - ip.time_t0) / ip.time_dt;
  // stencil rows r0 .. r0 + rows - 1 with weights w (a single row beyond the ends)
  int r0 = 0, rows = 1;
  double w[4] = {1., 0., 0., 0.};
  if (!(u > 0.)) {
    r0 = 0;
  } else if (u >= (double)last) {
    r0 = last;
  } else if (last < 3) {
    r0 = (int)u;
    rows = 2;
    w[1] = u - (double)r0;
    w[0] = 1. - w[1];
  } else {
    const int i = (int)u;
    r0 = i < 1 ? 0 : (i + 2 > last ? last - 3 : i - 1);  // stencil shifted inside the table at its ends
    rows = 4;
    const double x0 = u - (double)r0, x1 = x0 - 1., x2 = x0 - 2., x3 = x0 - 3.;
    w[0] = -x1 * x2 * x3 * (1. / 6.);
    w[1] = x0 * x2 * x3 * 0.5;
    w[2] = -x0 * x1 * x3 * 0.5;
    w[3] = x0 * x1 * x2 * (1. / 6.);
  }
  auto val = [&](int c) {
    double v = 0.;
    for (int k = 0; k < rows; ++k) v += w[k] * tab[(size_t)(r0 + k) * W + c];
    return v;
  };
  const int m = ip.time_columns;
  int c = 0;
  if (m & SF_TIME_FEED_T) cf.Tin = val(c++);
  if (m & SF_TIME_MIXING_TAU) cf.tau = val(c++);
  if (m & SF_TIME_CONV_T) cf.Tc = val(c++);
  if (m & SF_TIME_CONV_H) cf.hc = val(c++);
  if (m & SF_TIME_RAD_T) cf.Tr = val(c++);
  if (m & SF_TIME_RAD_EPS) cf.eps = val(c++);
  if ((m & SF_TIME_FEED_Y) && ybuf) {
    __syncwarp();
    for (int k = threadIdx.x & 31; k < ns; k += 32) ybuf[k] = val(c + k);
    __syncwarp();
    cf.yin = ybuf;
  }
}

__device__ __forceinline__ double warp_max(double v)
{
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// The right-hand side of a step's first stage and of every Newton iteration, as one function that both call sites
// share. Inlined twice, its code did not stay in the instruction caches while the resident warps ran different
// phases of their steps (ncu: instruction-fetch stalls, "no instruction", were the largest stall reason); one
// shared copy ran the 8192-reactor GRI ignition batch 4.8 % faster with the same results bit for bit. Making the
// Jacobian evaluation and the LU separate functions as well was slower (register spills in the Jacobian).
template <bool OPEN>
__device__ __noinline__ void int_rhs(const IntParams &p, Blob b, double *scr, const double *q, double pres,
                                     const ReactorCfg &cf, double *out)
{
  const Group<32> grp;
  NoJ noj;
  reactor_eval<32, false, kIntegratorUnroll, OPEN>(p.m, b, p.L, scr, grp, q, pres, cf, p.pg, out, noj);
}

// p is a __grid_constant__ parameter so that int_rhs reads it in place, without a per-thread copy.
template <bool OPEN>
__global__ void __launch_bounds__(256) integrate_kernel(const __grid_constant__ IntParams p)
{
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint64_t bar;
  const DevMech &m = p.m;
  if (!stage_to_smem(smem, p.blob, m.blob_bytes, &bar, p.status)) return;
  const Blob b = blob_at(m, smem);
  const ScratchLayout &L = p.L;
  const Group<32> grp;
  const int lane = grp.lane;
  const int warp = threadIdx.x >> 5;
  const int neq = p.neq;
  const sf_integrate_params &ip = p.ip;
  double *base = reinterpret_cast<double *>(smem + m.blob_bytes) + (size_t)warp * p.per_warp;
  const size_t slot = (size_t)blockIdx.x * p.warps + warp;  // this warp's global slots
  // iteration matrix: in shared memory, or with the FP32 factors in this warp's global slot (L2-resident)
  double *A = p.gmat ? p.gmat + slot * p.mat_doubles : base;  // neq*neq
  double *y = p.gmat ? base : A + neq * neq;              // current state
  double *Y = y + neq;                                    // stage iterate
  double *res = Y + neq;                                  // Newton residual / step update
  double *f = res + neq;                                  // RHS at the iterate
  double *prior = f + neq;                                // sum_j a_sj k_j
  double *x = prior + neq;                                // linear-solve work vector
  double *k = x + neq;                                    // 6 stage derivatives
  // Griffon scratch: in shared memory, or in this warp's slot of the global scratch array (L2-resident)
  double *scr = p.gscratch ? p.gscratch + slot * L.total : k + 6 * neq;
  double *after = p.gscratch ? k + 6 * neq : scr + L.total;
  const int lu32_doubles = (p.prec == 1 && !p.gmat) ? (neq * neq + 1) / 2 : 0;
  // FP32 factors (precision 1)
  float *LU32 = p.gmat ? reinterpret_cast<float *>(A + neq * neq) : reinterpret_cast<float *>(after);
  float *xf = reinterpret_cast<float *>(after + lu32_doubles);  // 2*neq floats
  // row permutation of the factorization, then the reciprocals of U's diagonal (double, or float for precision 1)
  int *piv = reinterpret_cast<int *>(after + (p.prec == 1 ? lu32_doubles + neq : 0));
  double *dinv = after + (p.prec == 1 ? lu32_doubles + neq : 0) + (neq + 1) / 2 + 1;
  float *rf = xf + neq;
  const int Tidx = p.cfg.configuration == 1 ? 1 : 0;
  // feed mass fractions of a time table: the last ns doubles of the warp's shared region
  double *ybuf = (p.ip.time_table && (p.ip.time_columns & SF_TIME_FEED_Y)) ? base + p.per_warp - m.ns : nullptr;

  for (;;) {
    unsigned int r = 0;
    if (lane == 0) r = atomicAdd(p.queue, 1u);
    r = __shfl_sync(0xffffffffu, r, 0);
    if (r >= (unsigned)p.n) break;
    const double pres = p.cfg.configuration == 1 ? 0. : (p.pressures ? p.pressures[r] : p.pressure);
    for (int i = lane; i < neq; i += 32) y[i] = p.q0[(size_t)r * neq + i];
    __syncwarp();
    const double T0 = y[Tidx];
    // reactor options with the feed temperature of the current evaluation; t_rhs: time of the most recent
    // right-hand side, whose feed the next Jacobian uses
    ReactorCfg cf = p.cfg;
    double t_rhs = ip.time_jac_t0;
    double t = 0., dt = ip.first_time_step;
    double tau_interp = nan("");  // first crossing of T0 + delta, Hermite-interpolated
    bool setup = true;
    int count = 0, nsteps = 0, nnewton = 0, njac = 0, nfail = 0, status = 0, attempts = 0;
    const bool coerce = ip.stop_at_time > 0.;
    for (;;) {
      if (++attempts > ip.max_attempts) {
        status = SF_INT_MAX_STEPS;
        break;
      }
      if (coerce && t + dt > ip.stop_at_time) dt = ip.stop_at_time - t;
      if (setup) {
        IterMatrix im{A, neq, dt * kGamma};
        if (p.ip.time_table) apply_time_params(p, cf, t_rhs, ybuf, m.ns);
        reactor_eval<32, true, kIntegratorUnroll, OPEN>(m, b, L, scr, grp, y, pres, cf, p.pg, f, im);
        __syncwarp();
        if (p.prec == 1) {
          for (int e = lane; e < neq * neq; e += 32) LU32[e] = (float)A[e];
          __syncwarp();
          warp_lu_pd(LU32, neq, piv, reinterpret_cast<float *>(dinv));
        } else {
          warp_lu_pd(A, neq, piv, dinv);
        }
        __syncwarp();
        ++njac;
      }
      ++count;
      // trajectory record of this attempt (slot of the next accepted step; a rejected attempt is overwritten)
      double *slot = nullptr;
      if (p.rec) {
        if (nsteps >= p.rec_cap) {
          status = SF_INT_RECORD_FULL;
          break;
        }
        slot = p.rec + ((size_t)r * p.rec_cap + nsteps) * (2 + 6 * (size_t)neq);
        if (lane == 0) {
          slot[0] = t;
          slot[1] = dt;
        }
        for (int i = lane; i < neq; i += 32) slot[2 + i] = y[i];
      }
      // ---------------- one ESDIRK64 step (methods.py:502-612)
      t_rhs = t;
      if (p.ip.time_table) apply_time_params(p, cf, t_rhs, ybuf, m.ns);
      int_rhs<OPEN>(p, b, scr, y, pres, cf, k);
      for (int i = lane; i < neq; i += 32) Y[i] = y[i];
      __syncwarp();
      bool nl_ok = true;
      for (int s = 1; s < 6; ++s) {
        const double *kprev = k + (s - 1) * neq;
        t_rhs = t + c_c[s] * dt;
        if (p.ip.time_table) apply_time_params(p, cf, t_rhs, ybuf, m.ns);
        for (int i = lane; i < neq; i += 32) {
          double pr = 0.;
          for (int j = s - 1; j >= 0; --j) pr += c_a[s][j] * k[j * neq + i];  // a_s,s-1 k_s-1 + ... + a_s1 k_1
          prior[i] = pr;
          res[i] = dt * (kGamma * kprev[i] + pr) - (Y[i] - y[i]);
        }
        __syncwarp();
        bool conv = false;
        for (int it = 1; it <= ip.max_nonlinear_iter; ++it) {
          // dx = A^-1 res
          if (p.prec == 1) {
            // FP32 triangular solves of the FP32 factors, FP64 residual refinement r = res - A x
            for (int i = lane; i < neq; i += 32) xf[i] = (float)res[piv[i]];
            warp_lu_solve_pd(LU32, neq, reinterpret_cast<const float *>(dinv), xf);
            for (int i = lane; i < neq; i += 32) x[i] = (double)xf[i];
            __syncwarp();
            for (int sweep = 0; sweep < ip.refine_sweeps; ++sweep) {
              for (int i = lane; i < neq; i += 32) {
                const int pi = piv[i];  // the residual of row perm[i], in the factors' row order
                double rr = res[pi];
                for (int j = 0; j < neq; ++j) rr = fma(-A[j * neq + pi], x[j], rr);
                rf[i] = (float)rr;
              }
              warp_lu_solve_pd(LU32, neq, reinterpret_cast<const float *>(dinv), rf);
              for (int i = lane; i < neq; i += 32) x[i] += (double)rf[i];
              __syncwarp();
            }
          } else {
            for (int i = lane; i < neq; i += 32) x[i] = res[piv[i]];
            warp_lu_solve_pd(A, neq, dinv, x);
          }
          for (int i = lane; i < neq; i += 32) Y[i] -= x[i];
          __syncwarp();
          int_rhs<OPEN>(p, b, scr, Y, pres, cf, f);
          double nrm = 0.;
          for (int i = lane; i < neq; i += 32) {
            res[i] = dt * (kGamma * f[i] + prior[i]) - (Y[i] - y[i]);
            nrm = fmax(nrm, fabs(res[i]) * (i == Tidx ? 1.e-3 : 1.));
          }
          nrm = warp_max(nrm);
          ++nnewton;
          __syncwarp();
          if (nrm < ip.nonlinear_tolerance) {
            conv = true;
            break;
          }
        }
        for (int i = lane; i < neq; i += 32) k[s * neq + i] = f[i];
        if (slot)
          for (int i = lane; i < neq; i += 32) slot[2 + (size_t)s * neq + i] = Y[i];
        __syncwarp();
        if (!conv) nl_ok = false;
      }
      // ---------------- update, error estimate, residual
      double err = 0., rsd = 0.;
      bool finite = true;
      for (int i = lane; i < neq; i += 32) {
        double ds = 0., dh = 0.;
        for (int j = 0; j < 6; ++j) {
          ds += c_b[j] * k[j * neq + i];
          dh += c_bh[j] * k[j * neq + i];
        }
        ds *= dt;
        dh *= dt;
        res[i] = ds;
        const double wi = (i == Tidx) ? 1.e-3 : 1.;
        err = fmax(err, fabs((ds - dh) * wi));
        rsd = fmax(rsd, fabs(ds * wi));
        finite = finite && isfinite(ds);
      }
      err = warp_max(err);
      rsd = warp_max(rsd) / dt;
      finite = __all_sync(0xffffffffu, finite);
      const double T_start = y[Tidx];
      __syncwarp();
      const double recent = dt;
      if (finite) {
        for (int i = lane; i < neq; i += 32) {
          const double v = y[i] + res[i];
          y[i] = v < 0. ? 0. : v;  // post_step_callback (reactors.py:506-508)
        }
        __syncwarp();
        if (ip.delta_temperature_ignition > 0. && isnan(tau_interp) &&
            y[Tidx] > T0 + ip.delta_temperature_ignition)  // this step crossed: dT/dt at its ends are k_1 and k_6
          tau_interp = hermite_crossing(t, dt, T_start, y[Tidx], k[Tidx], k[5 * neq + Tidx],
                                        T0 + ip.delta_temperature_ignition);
        t += dt;
        ++nsteps;
        if (err < 1.e-16)
          dt = fmin(dt * 1.1, ip.max_time_step);
        else
          dt = fmin(dt * fmin(1.1, pow(ip.transient_tolerance / err, 0.1333333333)), ip.max_time_step);
        if (count == ip.maximum_steps_per_jacobian) {
          count = 0;
          setup = true;
        } else if (!nl_ok) {
          dt *= 0.8;
          setup = true;
        } else if (dt > recent * 1.05 || dt < recent * 0.9) {
          setup = true;
        } else {
          setup = false;
        }
      } else {
        dt *= 0.8;
        setup = true;
        ++nfail;
      }
      // ---------------- stop rules (integrator.py:629-640, reactors.py:774-787)
      bool cont = true;
      if (ip.delta_temperature_ignition > 0.) {
        const bool ignited = y[Tidx] > T0 + ip.delta_temperature_ignition;
        if (rsd > ip.minimum_allowable_residual) {
          cont = !ignited;
          status = ignited ? SF_INT_IGNITED : 0;
        } else {
          status = SF_INT_NO_IGNITION;
          break;
        }
      }
      if (nsteps < ip.minimum_time_step_count) {
        cont = true;
        if (status == SF_INT_IGNITED) status = 0;
      }
      if (nsteps > ip.maximum_time_step_count) {
        cont = false;
        status = SF_INT_MAX_STEPS;
      } else if (coerce && t >= ip.stop_at_time) {
        cont = false;
        if (status == 0) status = SF_INT_DONE;
      } else if (ip.stop_at_steady > 0. && rsd < ip.stop_at_steady) {
        cont = false;
        status = SF_INT_STEADY;
      }
      if (!cont) break;
    }
    for (int i = lane; i < neq; i += 32) p.out_q[(size_t)r * neq + i] = y[i];
    if (lane == 0) {
      p.out_t[r] = t;
      p.out_counts[4 * (size_t)r + 0] = nsteps;
      p.out_counts[4 * (size_t)r + 1] = nnewton;
      p.out_counts[4 * (size_t)r + 2] = njac;
      p.out_counts[4 * (size_t)r + 3] = nfail;
      p.out_status[r] = status;
      if (ip.ignition_time_interp) ip.ignition_time_interp[r] = tau_interp;
    }
    __syncwarp();
  }
}

// Memory placement of an integrating warp's data: 0 all in shared memory, 1 the Griffon scratch in a global
// (L2-resident) slot, 2 the iteration matrix and FP32 factors there too. The built-in choice (knob value 0) is 2:
// with 8 warps per block it ran the 8192-reactor GRI ignition batch at 2,292 ignitions/s, against 1,771 for
// placement 1 and 5 warps; placement 0 leaves room for two warps per block. Knob value 3 selects placement 0.
int integrate_placement(const HostMech &hm)
{
  const int v = hm.tune[SF_TUNE_INTEGRATE_SCRATCH];
  return v == 0 ? 2 : (v == 3 ? 0 : v);
}

// Shared memory per warp. global_scratch: the Griffon scratch lives in a global slot; global_matrix: the iteration
// matrix and the FP32 factors too, leaving the vectors and pivots in shared memory.
size_t per_warp_doubles(const HostMech &hm, int neq, int prec, bool global_scratch, bool global_matrix,
                        bool feed_y_table = false)
{
  const size_t n2 = (size_t)neq * neq;
  return (global_matrix ? 0 : n2) + 12 * (size_t)neq + (global_scratch ? 0 : hm.sl.total) +
         (prec == 1 ? (global_matrix ? 0 : (n2 + 1) / 2) + (size_t)neq : 0) + ((size_t)neq + 1) / 2 + 2 +
         (size_t)neq +                           // reciprocals of U's diagonal
         (feed_y_table ? (size_t)hm.dm.ns : 0);  // interpolated feed mass fractions
}

size_t matrix_doubles(int neq, int prec)
{
  const size_t n2 = (size_t)neq * neq;
  return n2 + (prec == 1 ? (n2 + 1) / 2 : 0);
}

struct IntShape {
  int warps, grid;
  size_t per_warp, smem, scratch_bytes, mat_bytes;
};

// Warps per block and grid of the persistent launch (autotuned knobs, else as many warps as fit)
IntShape integrate_shape(const HostMech &hm, int neq, int prec, int n, bool feed_y_table = false)
{
  int dev, smem_max, nsm;
  CUDA_THROW(cudaGetDevice(&dev));
  CUDA_THROW(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  CUDA_THROW(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  IntShape s{};
  const int place = integrate_placement(hm);
  const bool gs = place >= 1, gm = place == 2;
  s.per_warp = per_warp_doubles(hm, neq, prec, gs, gm, feed_y_table);
  const size_t avail = (size_t)smem_max - hm.dm.blob_bytes - 64;
  int fit = (int)std::min<size_t>(8, avail / (s.per_warp * 8));
  if (fit < 1) throw sf_error(SF_ERR_UNSUPPORTED, "mechanism too large for the shared-memory integrator");
  const int want = hm.tune[SF_TUNE_INTEGRATE_WARPS];
  s.warps = (want > 0 && want < fit) ? want : fit;
  s.smem = hm.dm.blob_bytes + (size_t)s.warps * s.per_warp * 8;
  const int per_sm = std::max(1, (int)((size_t)smem_max / s.smem));
  s.grid = (int)std::max<long long>(1, std::min<long long>((long long)nsm * per_sm, ((long long)n + s.warps - 1) / s.warps));
  s.scratch_bytes = gs ? (size_t)nsm * per_sm * s.warps * hm.sl.total * 8 : 0;
  s.mat_bytes = gm ? (size_t)nsm * per_sm * s.warps * matrix_doubles(neq, prec) * 8 : 0;
  return s;
}

}  // namespace
}  // namespace sfgb

using namespace sfgb;

extern "C" {

size_t sf_integrate_workspace_size(const sf_mech *mech, const sf_reactor_params *params, int n)
{
  if (!mech || !params) return 256;
  try {
    const HostMech &hm = mech->m;
    const int neq = params->configuration == 1 ? hm.dm.ns + 1 : hm.dm.ns;
    // both linear precisions, with or without a feed mass-fraction table: the largest scratch need
    size_t most = 0;
    for (int prec = 0; prec <= 1; ++prec)
      for (int fy = 0; fy <= 1; ++fy) {
        const IntShape a = integrate_shape(hm, neq, prec, n < 1 ? 1 : n, fy != 0);
        most = std::max(most, a.scratch_bytes + a.mat_bytes);
      }
    return 256 + most;
  } catch (...) {
    return 256;
  }
}

static int integrate_impl(const sf_mech *mech, const sf_reactor_params *rp, const sf_integrate_params *ip, int n,
                          const double *q0, const double *pressures, double *out_q, double *out_t, int *out_counts,
                          int *out_status, void *workspace, size_t workspace_bytes, double *record, int record_cap,
                          void *stream)
{
  try {
    if (!mech || !rp || !ip || n < 0 || (n > 0 && (!q0 || !out_q || !out_t || !out_counts || !out_status)))
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "sf_integrate_batch: bad argument");
    if (rp->configuration != 0 && rp->configuration != 1) throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad configuration");
    if (rp->heat_transfer < 0 || rp->heat_transfer > 2) throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad heat_transfer");
    if (rp->open) {
      if (!rp->inflow_Y || !(rp->tau > 0.))
        throw sf_error(SF_ERR_INVALID_ARGUMENT, "open reactor needs feed mass fractions and a positive mixing time");
      const bool t_table = ip->time_table && (ip->time_columns & SF_TIME_FEED_T);
      if (!t_table && !(rp->inflow_temperature > 0.))
        throw sf_error(SF_ERR_INVALID_ARGUMENT, "open reactor needs a feed temperature (constant or table)");
    }
    if (ip->time_table) {
      const int m = ip->time_columns;
      int width = 0;
      for (int bit = 1; bit <= SF_TIME_RAD_EPS; bit <<= 1) width += (m & bit) ? 1 : 0;
      if (m & SF_TIME_FEED_Y) width += mech->m.dm.ns;
      if (m & ~127) throw sf_error(SF_ERR_INVALID_ARGUMENT, "unknown bit in time_columns");
      if (ip->time_points < 2 || !(ip->time_dt > 0.) || ip->time_width < width)
        throw sf_error(SF_ERR_INVALID_ARGUMENT, "time table needs >= 2 points, a positive spacing and a column for "
                                                "every parameter of time_columns");
    }
    if (ip->linear_precision != 0 && ip->linear_precision != 1)
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "linear_precision must be 0 or 1");
    if (ip->rates_option < 0 || ip->rates_option > 2) throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad rates option");
    if (ip->max_nonlinear_iter < 1 || ip->maximum_steps_per_jacobian < 1 || ip->max_attempts < 1 ||
        !(ip->first_time_step > 0.))
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad integration controls");
    if (!workspace || workspace_bytes < 256) throw sf_error(SF_ERR_WORKSPACE, "workspace too small");
    if (mech->m.dm.ns + 1 > 128) throw sf_error(SF_ERR_UNSUPPORTED, "the integrator supports up to 127 species");
    if (n == 0) return SF_OK;
    HostMech &hm = const_cast<HostMech &>(mech->m);
    const auto &progs = hm.programs_for(32);
    IntParams p{};
    p.m = hm.dm;
    p.blob = hm.d_blob;
    p.status = hm.d_status;
    p.L = hm.sl;
    p.pg.w = progs.progs[0];
    p.pg.full = progs.progs[1];
    p.pg.j = progs.progs[2];
    p.cfg.configuration = rp->configuration;
    p.cfg.heat = rp->heat_transfer;
    p.cfg.option = ip->rates_option;
    p.cfg.Tc = rp->fluid_temperature;
    p.cfg.Tr = rp->surface_temperature;
    p.cfg.hc = rp->h_convection;
    p.cfg.eps = rp->eps_radiation;
    p.cfg.SoV = rp->surface_area_to_volume;
    p.cfg.open = rp->open ? 1 : 0;
    p.cfg.tau = rp->tau;
    p.cfg.rho_in = rp->inflow_density;
    p.cfg.Tin = rp->inflow_temperature;
    p.cfg.yin = rp->inflow_Y;
    p.ip = *ip;
    if (p.ip.maximum_time_step_count <= 0) p.ip.maximum_time_step_count = 2147483647;
    p.n = n;
    p.neq = rp->configuration == 1 ? hm.dm.ns + 1 : hm.dm.ns;
    p.prec = ip->linear_precision;
    p.pressure = rp->pressure;
    p.pressures = pressures;
    p.q0 = q0;
    p.out_q = out_q;
    p.out_t = out_t;
    p.out_counts = out_counts;
    p.out_status = out_status;
    p.queue = static_cast<unsigned int *>(workspace);
    p.rec = record;
    p.rec_cap = record_cap;
    const IntShape sh = integrate_shape(hm, p.neq, p.prec, n,
                                        ip->time_table && (ip->time_columns & SF_TIME_FEED_Y));
    if (workspace_bytes < 256 + sh.scratch_bytes + sh.mat_bytes)
      throw sf_error(SF_ERR_WORKSPACE, "workspace smaller than sf_integrate_workspace_size reports");
    p.per_warp = sh.per_warp;
    p.warps = sh.warps;
    p.gscratch = sh.scratch_bytes ? reinterpret_cast<double *>(static_cast<char *>(workspace) + 256) : nullptr;
    p.gmat = sh.mat_bytes ? reinterpret_cast<double *>(static_cast<char *>(workspace) + 256 + sh.scratch_bytes)
                          : nullptr;
    p.mat_doubles = matrix_doubles(p.neq, p.prec);
    auto kern = p.cfg.open ? integrate_kernel<true> : integrate_kernel<false>;
    ensure_dynamic_smem((const void *)kern, sh.smem);
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_THROW(cudaMemsetAsync(workspace, 0, 256, st));
    kern<<<sh.grid, 32 * sh.warps, sh.smem, st>>>(p);
    CUDA_THROW(cudaGetLastError());
    return SF_OK;
  } catch (sf_error &e) {
    set_error(e.what());
    return e.code;
  }
}

int sf_integrate_batch(const sf_mech *mech, const sf_reactor_params *rp, const sf_integrate_params *ip, int n,
                       const double *q0, const double *pressures, double *out_q, double *out_t, int *out_counts,
                       int *out_status, void *workspace, size_t workspace_bytes, void *stream)
{
  return integrate_impl(mech, rp, ip, n, q0, pressures, out_q, out_t, out_counts, out_status, workspace,
                        workspace_bytes, nullptr, 0, stream);
}

int sf_integrate_record_batch(const sf_mech *mech, const sf_reactor_params *rp, const sf_integrate_params *ip, int n,
                              const double *q0, const double *pressures, double *out_q, double *out_t,
                              int *out_counts, int *out_status, void *workspace, size_t workspace_bytes,
                              double *trajectory, int capacity_steps, void *stream)
{
  if (n > 0 && (!trajectory || capacity_steps < 1)) {
    set_error("sf_integrate_record_batch: trajectory buffer and a positive capacity are required");
    return SF_ERR_INVALID_ARGUMENT;
  }
  return integrate_impl(mech, rp, ip, n, q0, pressures, out_q, out_t, out_counts, out_status, workspace,
                        workspace_bytes, trajectory, capacity_steps, stream);
}

}  // extern "C"
