// The plain single-state GPU form of the reactor Jacobian, kept as the comparison point for the batched kernels:
// one thread per state, the mechanism read from global memory (no shared-memory staging), per-state scratch in a
// global workspace laid out one state after another (the reference's memory layout), and Griffon's dense
// per-reaction scatter of every reaction's derivative into all ns-1 Y columns
// (rates_sensitivities_exact.cpp:1001-1026) followed by the dense assembly of chem_jac_isochoric /
// chem_jac_isobaric (isochoric_reactor_kernels.cpp:61-104, isobaric_reactor_kernels.cpp:57-100, :319-343).
// Also: the thermodynamic property kernel behind sf_thermo_batch (thermodynamics_kernels.cpp:18-382).
#include "chem_device.cuh"
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

__global__ void __launch_bounds__(128) plain_jac_kernel(const PlainParams p)
{
  const int st = blockIdx.x * blockDim.x + threadIdx.x;
  if (st >= p.n) return;
  const DevMech &m = p.m;
  const Blob b = blob_at(m, p.blob);
  const ScratchLayout &L = p.L;
  const int ns = m.ns, nr = m.nr, n1 = ns + 1;
  double *scr = p.ws + (size_t)st * p.per_state;
  double *S = scr + L.total;        // (ns+1)^2, Y columns scaled by 1/rho
  double *dq = S + (size_t)n1 * n1; // ns
  const bool iso = p.configuration == 1;
  const int neq = iso ? ns + 1 : ns;
  const double *qs = p.q + (size_t)st * neq;
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
    rho = (p.pressures ? p.pressures[st] : p.pressure) * mmw / (T * m.Ru);
  }
  StateCtx s;
  s.T = T; s.logT = log(T); s.invT = 1. / T; s.rho = rho; s.invRho = 1. / rho; s.mmw = mmw; s.invM = 1. / mmw;
  s.ct = rho / mmw; s.port = m.pref * s.invT * m.invRu; s.invport = 1. / s.port; s.option = 0;
  double cpmix = 0., cpsens = 0.;
  for (int i = 0; i < ns; ++i) {
    const double invmw = b.d[m.d_invmw + i];
    scr[L.C + i] = scr[L.y + i] * rho * invmw;
    const SpeciesThermo th = species_thermo(m, b, i, T, s.logT, s.invT, true);
    store_gibbs_factor(scr, L, i, th.g * s.invT * m.invRu);
    scr[L.eh + i] = iso ? th.h - m.Ru * T * invmw : th.h;
    scr[L.cpv + i] = iso ? th.cp - m.Ru * invmw : th.cp;
    scr[L.dB + i] = th.dB;
    scr[L.dcp + i] = th.dcp;
    cpmix += scr[L.y + i] * th.cp;
    cpsens += scr[L.y + i] * th.dcp;
  }
  const double cmix = iso ? cpmix - m.Ru / mmw : cpmix;
  for (int i = 0; i < n1 * n1; ++i) S[i] = 0.;
  for (int i = 0; i < ns; ++i) scr[L.w + i] = 0.;
  double EA = 0., EB = 0.;
  for (int r = 0; r < nr; ++r) {
    eval_reaction<true>(m, b, L, scr, s, r, &EA, &EB);
    // dense dq/dY over all columns
    const int di = b.i[m.i_dense + r];
    const double al = di >= 0 ? scr[L.alpha + di] : 0., be = di >= 0 ? scr[L.beta + di] : 0.;
    for (int k = 0; k < ns - 1; ++k) dq[k] = al * b.d[m.d_u + k] + be;
    for (int j = b.i[m.i_slot_off + r]; j < b.i[m.i_slot_off + r + 1]; ++j) dq[b.i[m.i_slot + j] & 0xFFFF] += scr[L.D + j];
    for (int j = b.i[m.i_net_off + r]; j < b.i[m.i_net_off + r + 1]; ++j) {
      const int i = b.i[m.i_net + j] & 0xFFFF;
      const double c = b.d[m.d_netc + j];
      scr[L.w + i] += c * scr[L.q + r];
      S[i] += c * scr[L.dqdrho + r];
      S[i + n1] += c * scr[L.dqdT + r];
      for (int k = 0; k < ns - 1; ++k) S[i + (2 + k) * n1] += c * dq[k];
    }
  }
  // assembly (dense inner products as chem_jac_*)
  const double invRho = s.invRho, iC = 1. / cmix, iRC = 1. / (rho * cmix);
  double swe = 0., sre = 0., ste = 0., swc = 0.;
  for (int i = 0; i < ns; ++i) {
    swe += scr[L.w + i] * scr[L.eh + i];
    sre += S[i] * scr[L.eh + i];
    ste += S[i + n1] * scr[L.eh + i];
    swc += scr[L.w + i] * scr[L.cpv + i];
  }
  const double rhsT = -swe / (rho * cmix);
  double *rhs = p.out_rhs + (size_t)st * neq;
  double *J = p.out_J + (size_t)st * neq * neq;
  const int tix = iso ? 1 : 0;
  if (iso) rhs[0] = 0.;
  rhs[tix] = rhsT;
  for (int i = 0; i < ns - 1; ++i) rhs[tix + 1 + i] = scr[L.w + i] * invRho;
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
