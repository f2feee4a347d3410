// The plain single-state GPU form of the reactor Jacobian, kept as the comparison point for the batched kernels:
// one thread per state, the mechanism read from global memory (no shared-memory staging), per-state scratch in a
// global workspace laid out one state after another (the reference's memory layout), and Griffon's dense
// per-reaction scatter of every reaction's derivative into all ns-1 Y columns
// (rates_sensitivities_exact.cpp:1001-1026) followed by the dense assembly of chem_jac_isochoric /
// chem_jac_isobaric (isochoric_reactor_kernels.cpp:61-104, isobaric_reactor_kernels.cpp:57-100, :319-343).
// Also: the plain form of the batched ignition integrator, one thread per reactor running the same ESDIRK64 step
// logic over plain_state and a serial LU (the comparison point of integrate_kernels.cu), and the thermodynamic
// property kernel behind sf_thermo_batch (thermodynamics_kernels.cpp:18-382).
#include "chem_device.cuh"
#include "esdirk64.cuh"
#include "sf_internal.h"

#include <mutex>

namespace sfgb {

namespace {

struct PlainParams {
  DevMech m;
  const void *blob;
  ScratchLayout L;
  int n, configuration;
  double pressure;
  const double *q, *pressures;
  double *out_rhs, *out_J, *ws;
  size_t per_state;
};

// One state, Griffon's plain serial form: thermodynamics, then every reaction's rate (JAC: and derivatives, scattered
// densely into all ns-1 Y columns, rates_sensitivities_exact.cpp:1001-1026), then the reactor right-hand side
// (JAC: and the dense assembly of chem_jac_isochoric / chem_jac_isobaric + transform). scr, S ((ns+1)^2) and dq (ns)
// are this thread's scratch.
template <bool JAC>
__device__ void plain_state(const DevMech &m, const Blob &b, const ScratchLayout &L, double *scr, double *S, double *dq,
                            bool iso, double pressure, const double *qs, double *rhs, double *J)
{
  const int ns = m.ns, nr = m.nr, n1 = ns + 1;
  const int neq = iso ? ns + 1 : ns;
  double T, rho;
  double ysum = 0.;
  for (int i = 0; i < ns - 1; ++i) {
    scr[L.y + i] = qs[(iso ? 2 : 1) + i];
    ysum += scr[L.y + i];
  }
  scr[L.y + ns - 1] = 1. - ysum;
  double sim = 0.;
  for (int i = 0; i < ns; ++i) sim += scr[L.y + i] * b.d[m.d_invmw + i];
  const double mmw = 1. / sim;
  if (iso) {
    rho = qs[0];
    T = qs[1];
  } else {
    T = qs[0];
    rho = pressure * mmw / (T * m.Ru);
  }
  StateCtx s;
  s.T = T; s.logT = log(T); s.invT = 1. / T; s.rho = rho; s.invRho = 1. / rho; s.mmw = mmw; s.invM = 1. / mmw;
  s.ct = rho / mmw; s.port = m.pref * s.invT * m.invRu; s.invport = 1. / s.port; s.option = 0;
  double cpmix = 0., cpsens = 0.;
  for (int i = 0; i < ns; ++i) {
    const double invmw = b.d[m.d_invmw + i];
    scr[L.C + i] = scr[L.y + i] * rho * invmw;
    const SpeciesThermo th = species_thermo(m, b, i, T, s.logT, s.invT, JAC);
    store_gibbs_factor(scr, L, i, th.g * s.invT * m.invRu, b.d + m.d_exptab);
    scr[L.eh + i] = iso ? th.h - m.Ru * T * invmw : th.h;
    scr[L.cpv + i] = iso ? th.cp - m.Ru * invmw : th.cp;
    if (JAC) {
      scr[L.dB + i] = th.dB;
      scr[L.dcp + i] = th.dcp;
      cpsens += scr[L.y + i] * th.dcp;
    }
    cpmix += scr[L.y + i] * th.cp;
  }
  const double cmix = iso ? cpmix - m.Ru / mmw : cpmix;
  if (JAC)
    for (int i = 0; i < n1 * n1; ++i) S[i] = 0.;
  for (int i = 0; i < ns; ++i) scr[L.w + i] = 0.;
  double EA = 0., EB = 0.;
  for (int r = 0; r < nr; ++r) {
    eval_reaction<JAC>(m, b, L, scr, s, r, &EA, &EB);
    if (JAC) {
      // dense dq/dY over all columns
      const int di = b.i[m.i_dense + r];
      const double al = di >= 0 ? scr[L.alpha + di] : 0., be = di >= 0 ? scr[L.beta + di] : 0.;
      for (int k = 0; k < ns - 1; ++k) dq[k] = al * b.d[m.d_u + k] + be;
      for (int j = b.i[m.i_slot_off + r]; j < b.i[m.i_slot_off + r + 1]; ++j)
        dq[b.i[m.i_slot + j] & 0xFFFF] += scr[L.D + j];
    }
    for (int j = b.i[m.i_net_off + r]; j < b.i[m.i_net_off + r + 1]; ++j) {
      const int i = b.i[m.i_net + j] & 0xFFFF;
      const double c = b.d[m.d_netc + j];
      scr[L.w + i] += c * scr[L.q + r];
      if (JAC) {
        S[i] += c * scr[L.dqdrho + r];
        S[i + n1] += c * scr[L.dqdT + r];
        for (int k = 0; k < ns - 1; ++k) S[i + (2 + k) * n1] += c * dq[k];
      }
    }
  }
  // assembly (dense inner products as chem_jac_*)
  const double invRho = s.invRho, iC = 1. / cmix, iRC = 1. / (rho * cmix);
  double swe = 0., sre = 0., ste = 0., swc = 0.;
  for (int i = 0; i < ns; ++i) {
    swe += scr[L.w + i] * scr[L.eh + i];
    if (JAC) {
      sre += S[i] * scr[L.eh + i];
      ste += S[i + n1] * scr[L.eh + i];
      swc += scr[L.w + i] * scr[L.cpv + i];
    }
  }
  const double rhsT = -swe / (rho * cmix);
  const int tix = iso ? 1 : 0;
  if (iso) rhs[0] = 0.;
  rhs[tix] = rhsT;
  for (int i = 0; i < ns - 1; ++i) rhs[tix + 1 + i] = scr[L.w + i] * invRho;
  if (!JAC) return;
  const double JTrho = -iRC * sre - invRho * rhsT;
  const double JTT = -iC * (invRho * (ste + swc) + rhsT * cpsens);
  const double cpn = scr[L.cpv + ns - 1];
  if (iso) {
    for (int k = 0; k < neq; ++k) J[k * neq] = 0.;
    J[1] = JTrho;
    J[neq + 1] = JTT;
    for (int i = 0; i < ns - 1; ++i) {
      J[2 + i] = invRho * (S[i] - invRho * scr[L.w + i]);
      J[neq + 2 + i] = invRho * S[i + n1];
    }
    for (int k = 0; k < ns - 1; ++k) {
      double te = 0.;
      for (int i = 0; i < ns; ++i) te += S[i + (2 + k) * n1] * scr[L.eh + i];
      J[(2 + k) * neq + 1] = -iC * te - rhsT * (scr[L.cpv + k] - cpn) * iC;
      for (int i = 0; i < ns - 1; ++i) J[(2 + k) * neq + 2 + i] = S[i + (2 + k) * n1];
    }
  } else {
    const double roT = rho / T, nrm = -rho * mmw;
    J[0] = JTT - roT * JTrho;
    for (int i = 0; i < ns - 1; ++i) {
      const double pjr = invRho * (S[i] - invRho * scr[L.w + i]);
      J[1 + i] = invRho * S[i + n1] - roT * pjr;
    }
    for (int k = 0; k < ns - 1; ++k) {
      const double u = b.d[m.d_u + k];
      double te = 0.;
      for (int i = 0; i < ns; ++i) te += S[i + (2 + k) * n1] * scr[L.eh + i];
      J[(1 + k) * ns] = -iC * te - rhsT * (scr[L.cpv + k] - cpn) * iC + nrm * u * JTrho;
      for (int i = 0; i < ns - 1; ++i) {
        const double pjr = invRho * (S[i] - invRho * scr[L.w + i]);
        J[(1 + k) * ns + 1 + i] = S[i + (2 + k) * n1] + nrm * u * pjr;
      }
    }
  }
}

__global__ void __launch_bounds__(128) plain_jac_kernel(const PlainParams p)
{
  const int st = blockIdx.x * blockDim.x + threadIdx.x;
  if (st >= p.n) return;
  const DevMech &m = p.m;
  const Blob b = blob_at(m, p.blob);
  const ScratchLayout &L = p.L;
  const int ns = m.ns, n1 = ns + 1;
  double *scr = p.ws + (size_t)st * p.per_state;
  double *S = scr + L.total;        // (ns+1)^2, Y columns scaled by 1/rho
  double *dq = S + (size_t)n1 * n1; // ns
  const bool iso = p.configuration == 1;
  const int neq = iso ? ns + 1 : ns;
  const double pres = iso ? 0. : (p.pressures ? p.pressures[st] : p.pressure);
  plain_state<true>(m, b, L, scr, S, dq, iso, pres, p.q + (size_t)st * neq, p.out_rhs + (size_t)st * neq,
                    p.out_J + (size_t)st * neq * neq);
}

// ------------------------------------------------------------------------------------------ plain integrator
struct PlainIntParams {
  DevMech m;
  const void *blob;
  ScratchLayout L;
  int n, configuration;
  double pressure;
  const double *pressures, *q0;
  sf_integrate_params ip;
  double *out_q, *out_t;
  int *out_counts, *out_status;
  double *ws;
  size_t per_reactor;
};

// LU with partial pivoting of a column-major n x n matrix (pivot: the first largest |a|, as idamax), serial
__device__ void plain_lu(double *A, int n, int *piv)
{
  for (int k = 0; k < n; ++k) {
    int pr = k;
    double best = fabs(A[(size_t)k * n + k]);
    for (int i = k + 1; i < n; ++i) {
      const double v = fabs(A[(size_t)k * n + i]);
      if (v > best) {
        best = v;
        pr = i;
      }
    }
    piv[k] = pr;
    if (pr != k)
      for (int j = 0; j < n; ++j) {
        const double t = A[(size_t)j * n + k];
        A[(size_t)j * n + k] = A[(size_t)j * n + pr];
        A[(size_t)j * n + pr] = t;
      }
    const double inv = 1. / A[(size_t)k * n + k];
    for (int i = k + 1; i < n; ++i) A[(size_t)k * n + i] *= inv;
    for (int j = k + 1; j < n; ++j) {
      const double u = A[(size_t)j * n + k];
      for (int i = k + 1; i < n; ++i) A[(size_t)j * n + i] -= A[(size_t)k * n + i] * u;
    }
  }
}

// Solve with the factors of plain_lu: row interchanges, unit-lower forward and upper backward substitution
__device__ void plain_lu_solve(const double *A, int n, const int *piv, double *x)
{
  for (int k = 0; k < n; ++k)
    if (piv[k] != k) {
      const double t = x[k];
      x[k] = x[piv[k]];
      x[piv[k]] = t;
    }
  for (int j = 0; j < n; ++j) {
    const double xj = x[j];
    for (int i = j + 1; i < n; ++i) x[i] -= A[(size_t)j * n + i] * xj;
  }
  for (int j = n - 1; j >= 0; --j) {
    x[j] /= A[(size_t)j * n + j];
    const double xj = x[j];
    for (int i = 0; i < j; ++i) x[i] -= A[(size_t)j * n + i] * xj;
  }
}

// One thread integrates one closed adiabatic reactor with the step logic of integrate_kernel (odesolve, ESDIRK64,
// frozen-Jacobian Newton, PI control, Jacobian setup policy and stop rules), all serial per thread, the state,
// iteration matrix and Griffon scratch in the thread's global workspace.
__global__ void __launch_bounds__(32) plain_integrate_kernel(const PlainIntParams p)
{
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= p.n) return;
  const DevMech &m = p.m;
  const Blob b = blob_at(m, p.blob);
  const ScratchLayout &L = p.L;
  const int ns = m.ns, n1 = ns + 1;
  const bool iso = p.configuration == 1;
  const int neq = iso ? ns + 1 : ns;
  const sf_integrate_params &ip = p.ip;
  double *scr = p.ws + (size_t)r * p.per_reactor;
  double *S = scr + L.total;
  double *dq = S + (size_t)n1 * n1;
  double *A = dq + ns + 1;
  double *y = A + (size_t)neq * neq, *Y = y + neq, *res = Y + neq, *f = res + neq, *prior = f + neq, *x = prior + neq;
  double *k = x + neq;
  int *piv = reinterpret_cast<int *>(k + 6 * neq);
  const double pres = iso ? 0. : (p.pressures ? p.pressures[r] : p.pressure);
  for (int i = 0; i < neq; ++i) y[i] = p.q0[(size_t)r * neq + i];
  const int Tidx = iso ? 1 : 0;
  const double T0 = y[Tidx];
  double t = 0., dt = ip.first_time_step;
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
      plain_state<true>(m, b, L, scr, S, dq, iso, pres, y, f, A);
      const double pref = dt * kGamma;
      for (int c = 0; c < neq; ++c)
        for (int i = 0; i < neq; ++i) A[(size_t)c * neq + i] = pref * A[(size_t)c * neq + i] - (i == c ? 1. : 0.);
      plain_lu(A, neq, piv);
      ++njac;
    }
    ++count;
    plain_state<false>(m, b, L, scr, S, dq, iso, pres, y, k, nullptr);
    for (int i = 0; i < neq; ++i) Y[i] = y[i];
    bool nl_ok = true;
    for (int s = 1; s < 6; ++s) {
      const double *kprev = k + (s - 1) * neq;
      for (int i = 0; i < neq; ++i) {
        double pr = 0.;
        for (int j = s - 1; j >= 0; --j) pr += c_a[s][j] * k[j * neq + i];
        prior[i] = pr;
        res[i] = dt * (kGamma * kprev[i] + pr) - (Y[i] - y[i]);
      }
      bool conv = false;
      for (int it = 1; it <= ip.max_nonlinear_iter; ++it) {
        for (int i = 0; i < neq; ++i) x[i] = res[i];
        plain_lu_solve(A, neq, piv, x);
        for (int i = 0; i < neq; ++i) Y[i] -= x[i];
        plain_state<false>(m, b, L, scr, S, dq, iso, pres, Y, f, nullptr);
        double nrm = 0.;
        for (int i = 0; i < neq; ++i) {
          res[i] = dt * (kGamma * f[i] + prior[i]) - (Y[i] - y[i]);
          nrm = fmax(nrm, fabs(res[i]) * (i == Tidx ? 1.e-3 : 1.));
        }
        ++nnewton;
        if (nrm < ip.nonlinear_tolerance) {
          conv = true;
          break;
        }
      }
      for (int i = 0; i < neq; ++i) k[s * neq + i] = f[i];
      if (!conv) nl_ok = false;
    }
    double err = 0., rsd = 0.;
    bool finite = true;
    for (int i = 0; i < neq; ++i) {
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
    rsd /= dt;
    const double recent = dt;
    if (finite) {
      for (int i = 0; i < neq; ++i) {
        const double v = y[i] + res[i];
        y[i] = v < 0. ? 0. : v;  // post_step_callback (reactors.py:506-508)
      }
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
  for (int i = 0; i < neq; ++i) p.out_q[(size_t)r * neq + i] = y[i];
  p.out_t[r] = t;
  p.out_counts[4 * (size_t)r + 0] = nsteps;
  p.out_counts[4 * (size_t)r + 1] = nnewton;
  p.out_counts[4 * (size_t)r + 2] = njac;
  p.out_counts[4 * (size_t)r + 3] = nfail;
  p.out_status[r] = status;
}

size_t plain_reactor_doubles(const HostMech &hm, int neq)
{
  const size_t ns = hm.dm.ns, n1 = ns + 1;
  return (size_t)hm.sl.total + n1 * n1 + ns + 1 + (size_t)neq * neq + 12 * (size_t)neq + ((size_t)neq + 1) / 2 + 1;
}

struct ThermoParams {
  DevMech m;
  const void *blob;
  int n, what;
  const double *T, *Y;
  double *out;
};

__global__ void thermo_kernel(const ThermoParams p)
{
  const int st = blockIdx.x * blockDim.x + threadIdx.x;
  if (st >= p.n) return;
  const DevMech &m = p.m;
  const Blob b = blob_at(m, p.blob);
  const int ns = m.ns;
  const double T = p.T[st], logT = log(T), invT = 1. / T;
  const double *y = p.Y + (size_t)st * ns;
  double mix = 0., sim = 0.;
  const bool per_species = (p.what >= 4 && p.what <= 7) || p.what == 10;
  for (int i = 0; i < ns; ++i) {
    const double invmw = b.d[m.d_invmw + i];
    sim += y[i] * invmw;
    const SpeciesThermo th = species_thermo(m, b, i, T, logT, invT, p.what >= 9);
    double v;
    switch (p.what) {
    case 0: case 4: v = th.cp; break;
    case 1: v = th.cp; break;
    case 5: v = th.cp - m.Ru * invmw; break;
    case 2: case 6: v = th.h; break;
    case 3: case 7: v = th.h - m.Ru * T * invmw; break;
    case 9: case 10: v = th.dcp; break;
    default: v = 0.;
    }
    if (per_species)
      p.out[(size_t)st * ns + i] = v;
    else
      mix += y[i] * v;
  }
  if (!per_species) {
    if (p.what == 8) mix = 1. / sim;
    if (p.what == 1) mix -= m.Ru * sim;
    p.out[st] = mix;
  }
}

}  // namespace
}  // namespace sfgb

using namespace sfgb;

extern "C" {

size_t sf_reactor_jac_plain_workspace_size(const sf_mech *mech, int n)
{
  if (!mech || n < 0) return 0;
  const int ns = mech->m.dm.ns;
  return (size_t)n * ((size_t)mech->m.sl.total + (size_t)(ns + 1) * (ns + 1) + ns + 2) * sizeof(double);
}

int sf_reactor_jac_plain_batch(const sf_mech *mech, const sf_reactor_params *rp, int n, const double *q,
                               const double *pressures, double *out_rhs, double *out_jac, void *workspace,
                               size_t workspace_bytes, void *stream)
{
  if (!mech || !rp || n < 0 || (n > 0 && (!q || !out_rhs || !out_jac))) {
    set_error("sf_reactor_jac_plain_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  if (rp->open || rp->heat_transfer != 0) {
    set_error("sf_reactor_jac_plain_batch: only closed adiabatic reactors");
    return SF_ERR_UNSUPPORTED;
  }
  if (workspace_bytes < sf_reactor_jac_plain_workspace_size(mech, n) || (n > 0 && !workspace)) {
    set_error("sf_reactor_jac_plain_batch: workspace too small");
    return SF_ERR_WORKSPACE;
  }
  if (n == 0) return SF_OK;
  PlainParams p{};
  p.m = mech->m.dm;
  p.blob = mech->m.d_blob;
  p.L = mech->m.sl;
  p.n = n;
  p.configuration = rp->configuration;
  p.pressure = rp->pressure;
  p.q = q;
  p.pressures = pressures;
  p.out_rhs = out_rhs;
  p.out_J = out_jac;
  p.ws = (double *)workspace;
  const int ns = p.m.ns;
  p.per_state = (size_t)p.L.total + (size_t)(ns + 1) * (ns + 1) + ns + 2;
  plain_jac_kernel<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(p);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return SF_ERR_CUDA;
  }
  return SF_OK;
}

size_t sf_integrate_plain_workspace_size(const sf_mech *mech, const sf_reactor_params *params, int n)
{
  if (!mech || !params || n < 0) return 0;
  const int neq = params->configuration == 1 ? mech->m.dm.ns + 1 : mech->m.dm.ns;
  return (size_t)n * plain_reactor_doubles(mech->m, neq) * sizeof(double);
}

int sf_integrate_plain_batch(const sf_mech *mech, const sf_reactor_params *rp, const sf_integrate_params *ip, int n,
                             const double *q0, const double *pressures, double *out_q, double *out_t, int *out_counts,
                             int *out_status, void *workspace, size_t workspace_bytes, void *stream)
{
  if (!mech || !rp || !ip || n < 0 || (n > 0 && (!q0 || !out_q || !out_t || !out_counts || !out_status))) {
    set_error("sf_integrate_plain_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  if (rp->open || rp->heat_transfer != 0 || (rp->configuration != 0 && rp->configuration != 1)) {
    set_error("sf_integrate_plain_batch: the plain form covers closed adiabatic reactors");
    return SF_ERR_UNSUPPORTED;
  }
  if (ip->max_nonlinear_iter < 1 || ip->maximum_steps_per_jacobian < 1 || ip->max_attempts < 1 ||
      !(ip->first_time_step > 0.)) {
    set_error("sf_integrate_plain_batch: bad integration controls");
    return SF_ERR_INVALID_ARGUMENT;
  }
  if (workspace_bytes < sf_integrate_plain_workspace_size(mech, rp, n) || (n > 0 && !workspace)) {
    set_error("sf_integrate_plain_batch: workspace too small");
    return SF_ERR_WORKSPACE;
  }
  if (n == 0) return SF_OK;
  PlainIntParams p{};
  p.m = mech->m.dm;
  p.blob = mech->m.d_blob;
  p.L = mech->m.sl;
  p.n = n;
  p.configuration = rp->configuration;
  p.pressure = rp->pressure;
  p.pressures = pressures;
  p.q0 = q0;
  p.ip = *ip;
  if (p.ip.maximum_time_step_count <= 0) p.ip.maximum_time_step_count = 2147483647;
  p.out_q = out_q;
  p.out_t = out_t;
  p.out_counts = out_counts;
  p.out_status = out_status;
  p.ws = static_cast<double *>(workspace);
  const int neq = rp->configuration == 1 ? p.m.ns + 1 : p.m.ns;
  p.per_reactor = plain_reactor_doubles(mech->m, neq);
  // one warp per block so that even a small batch spreads over the SMs
  plain_integrate_kernel<<<(n + 31) / 32, 32, 0, (cudaStream_t)stream>>>(p);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return SF_ERR_CUDA;
  }
  return SF_OK;
}

int sf_thermo_batch(const sf_mech *mech, int what, int n, const double *T, const double *Y, double *out, void *stream)
{
  if (!mech || n < 0 || what < 0 || what > 10 || (n > 0 && (!T || !Y || !out))) {
    set_error("sf_thermo_batch: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  if (n == 0) return SF_OK;
  ThermoParams p{};
  p.m = mech->m.dm;
  p.blob = mech->m.d_blob;
  p.n = n;
  p.what = what;
  p.T = T;
  p.Y = Y;
  p.out = out;
  thermo_kernel<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(p);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return SF_ERR_CUDA;
  }
  return SF_OK;
}

}  // extern "C"

// ======================================================================= plain Jacobian without any allocation
// Some callers cannot allocate device memory at the point where they evaluate Jacobians: a host code that hands
// all device memory to its own pool allocator and forbids raw cudaMalloc, or a caller that must not allocate
// while other work is being recorded on its streams. sf_reactor_jac_plain_batch_static gives them the plain
// Jacobian evaluation with its per-state scratch taken from a fixed array in device global memory that this
// library owns for the lifetime of the process (on every device that loads the library), instead of a
// caller-provided workspace.
namespace sfgb {
namespace {

// Fixed scratch: SF_PLAIN_STATIC_SCRATCH_BYTES (32 MiB) per device, shared by every call of
// sf_reactor_jac_plain_batch_static on that device.
static __device__ __align__(256) double g_plain_static_scratch[SF_PLAIN_STATIC_SCRATCH_BYTES / sizeof(double)];

constexpr int kMaxStaticDevices = 64;
double *g_static_scratch_ptr[kMaxStaticDevices] = {nullptr};
std::mutex g_static_scratch_mutex;

// Device address of the fixed scratch on the current device. The host-side symbol is only a stand-in for the
// device array, so the address is obtained once per device (with that device current) and cached.
int static_scratch_address(double **out)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    return SF_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxStaticDevices) {
    set_error("sf_reactor_jac_plain_batch_static: device index out of range");
    return SF_ERR_INVALID_ARGUMENT;
  }
  std::lock_guard<std::mutex> lock(g_static_scratch_mutex);
  if (!g_static_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_plain_static_scratch);
    if (e != cudaSuccess || !p) {
      set_error(std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
      return SF_ERR_CUDA;
    }
    g_static_scratch_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_static_scratch_ptr[dev];
  return SF_OK;
}

}  // namespace
}  // namespace sfgb

extern "C" int sf_reactor_jac_plain_batch_static(const sf_mech *mech, const sf_reactor_params *rp, int n,
                                                 const double *q, const double *pressures, double *out_rhs,
                                                 double *out_jac, void *stream)
{
  if (!mech || !rp || n < 0 || (n > 0 && (!q || !out_rhs || !out_jac))) {
    set_error("sf_reactor_jac_plain_batch_static: bad argument");
    return SF_ERR_INVALID_ARGUMENT;
  }
  if (rp->open || rp->heat_transfer != 0) {
    set_error("sf_reactor_jac_plain_batch_static: only closed adiabatic reactors");
    return SF_ERR_UNSUPPORTED;
  }
  const int ns = mech->m.dm.ns;
  const size_t per_state = (size_t)mech->m.sl.total + (size_t)(ns + 1) * (ns + 1) + ns + 2;
  const size_t capacity = SF_PLAIN_STATIC_SCRATCH_BYTES / sizeof(double) / per_state;
  if ((size_t)n > capacity) {
    set_error("sf_reactor_jac_plain_batch_static: " + std::to_string(n) + " states exceed the fixed scratch (" +
              std::to_string(capacity) + " states of this mechanism fit in " +
              std::to_string(SF_PLAIN_STATIC_SCRATCH_BYTES >> 20) + " MiB); split the batch");
    return SF_ERR_WORKSPACE;
  }
  if (n == 0) return SF_OK;
  double *scratch = nullptr;
  const int rc = static_scratch_address(&scratch);
  if (rc != SF_OK) return rc;
  // every value a state reads from its scratch slice is written earlier in the same launch (the S block and
  // the species sums are zeroed per state), so leftover contents of earlier calls need no clearing
  PlainParams p{};
  p.m = mech->m.dm;
  p.blob = mech->m.d_blob;
  p.L = mech->m.sl;
  p.n = n;
  p.configuration = rp->configuration;
  p.pressure = rp->pressure;
  p.q = q;
  p.pressures = pressures;
  p.out_rhs = out_rhs;
  p.out_J = out_jac;
  p.ws = scratch;
  p.per_state = per_state;
  plain_jac_kernel<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(p);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(cudaGetErrorString(e));
    return SF_ERR_CUDA;
  }
  return SF_OK;
}
