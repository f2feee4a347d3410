// Batched thermochemistry kernels: production rates, rate sensitivities, reactor right-hand sides and analytical
// Jacobians (isochoric and isobaric), one state group of G lanes per state.
//
// Phases per state (group-synchronous):
//   P0  load the state; mixture molecular weight and density              (reduction over species)
//   P1  concentrations and species thermodynamics                         (lanes over species)
//   P2  reaction rates q_r and, for Jacobians, their derivatives           (lanes over reactions)
//   P3  species gathers w_i, S_rho_i, S_T_i, P_i, Q_i                      (gather program)
//   P4  right-hand side, rho/T columns, dense-term coefficients            (lanes over species)
//   P5  Y-block of the Jacobian and T-row sums                             (gather program)
//   P6  T row of the Jacobian                                              (lanes over columns)
// Reference: isochoric_reactor_kernels.cpp:18-333, isobaric_reactor_kernels.cpp:19-343,
//            chemistry_kernels.cpp:35-483, rates_sensitivities_exact.cpp:33-1028.
#include "reactor_eval.cuh"
#include "sf_internal.h"

namespace sfgb {

// MODE_RHS_OPEN / MODE_JAC_OPEN: the reactor modes of open (mass-exchange) reactors, compiled with the feed terms;
// the closed modes compile them out.
enum Mode { MODE_RATES = 0, MODE_SENS = 1, MODE_RHS = 2, MODE_JAC = 3, MODE_RHS_OPEN = 4, MODE_JAC_OPEN = 5 };

__host__ __device__ constexpr int base_mode(int mode) { return mode >= MODE_RHS_OPEN ? mode - 2 : mode; }
__host__ __device__ constexpr bool jac_mode(int mode) { return base_mode(mode) == MODE_JAC || mode == MODE_SENS; }

struct KParams {
  DevMech m;
  const void *blob;
  int *status;
  ScratchLayout L;
  DevProgram prog_w, prog_full, prog_j;
  int n;
  int option;
  // inputs
  const double *T, *rho, *Y;      // RATES / SENS
  const double *q, *pressures;    // RHS / JAC
  int configuration;              // 0 isobaric, 1 isochoric
  int heat;                       // 0 adiabatic, 1 isothermal, 2 diathermal
  double pressure, Tc, Tr, hc, eps, SoV;
  // outputs
  double *out_w, *out_S, *out_rhs, *out_J;
  int groups_per_cta;
  double *gscratch;  // thread-per-state kernels: interleaved per-warp scratch in global memory
  // open reactors: feed
  int open;
  double tau, rho_in, Tin;
  const double *yin;
};

template <int G>
struct JWriter {
  double *J;
  int ld;       // leading dimension (neq or ns+1)
  int roff;     // row offset of species rows
  int coff;     // column offset of Y columns
  double scale;
  __device__ __forceinline__ void operator()(int row, int col, double v) const
  {
    J[(size_t)(coff + col) * ld + roff + row] = v * scale;
  }
};

// Column-major neq x neq block in global memory.
struct GlobalJ {
  double *J;
  int neq;
  __device__ __forceinline__ void operator()(int row, int col, double v) const { J[(size_t)col * neq + row] = v; }
};

// One state: the body shared by the state-group kernel (scratch in shared memory) and the thread-per-state kernel
// (interleaved scratch in global memory).
template <int G, int MODE, class S>
__device__ __forceinline__ void eval_state(const KParams &p, const DevMech &m, const Blob &b, const ScratchLayout &L,
                                           S scr, const Group<G> &grp, const Progs &pg, const ReactorCfg &cfg, int st)
{
  constexpr bool JAC = jac_mode(MODE);
  constexpr bool OPEN = MODE >= MODE_RHS_OPEN;
  const int lane = grp.lane;
  const int ns = m.ns;
  const int neq = p.configuration == 1 ? ns + 1 : ns;
  if (base_mode(MODE) == MODE_RHS || base_mode(MODE) == MODE_JAC) {
    const double *qs = p.q + (size_t)st * neq;
    const double pres = p.configuration == 1 ? 0. : (p.pressures ? p.pressures[st] : p.pressure);
    GlobalJ gj{JAC ? p.out_J + (size_t)st * neq * neq : nullptr, neq};
    reactor_eval<G, JAC, default_unroll(G), OPEN>(m, b, L, scr, grp, qs, pres, cfg, pg, p.out_rhs + (size_t)st * neq,
                                                  gj);
    return;
  }
  // ---------------- production rates / sensitivities at (T, rho, Y)
  const double T = p.T[st], rho = p.rho[st];
  for (int i = lane; i < ns; i += G) scr[L.y + i] = p.Y[(size_t)st * ns + i];
  grp.sync();
  double sim = 0.;
  for (int i = lane; i < ns; i += G) sim += scr[L.y + i] * b.d[m.d_invmw + i];
  sim = grp.sum(sim);
  const double mmw = 1. / sim;
  StateCtx s;
  s.T = T;
  s.logT = log(T);
  s.invT = 1. / T;
  s.rho = rho;
  s.invRho = 1. / rho;
  s.mmw = mmw;
  s.invM = 1. / mmw;
  s.ct = rho / mmw;
  s.port = m.pref * s.invT * m.invRu;
  s.invport = 1. / s.port;
  s.option = p.option;
  prep_species<G, JAC>(m, b, L, scr, grp, s, false, MODE == MODE_SENS);
  reactions_and_gathers<G, JAC>(m, b, L, scr, grp, s, pg);
  if (MODE == MODE_RATES) {
    for (int i = lane; i < ns; i += G) p.out_w[(size_t)st * ns + i] = scr[L.w + i];
    grp.sync();
    return;
  }
  // Griffon's (ns+1)^2 column-major sensitivity block (rates_sensitivities_exact.cpp:1001-1026)
  const int n1 = ns + 1;
  double *Sb = p.out_S + (size_t)st * n1 * n1;
  for (int i = lane; i < ns; i += G) {
    p.out_w[(size_t)st * ns + i] = scr[L.w + i];
    Sb[i] = scr[L.Srho + i];
    Sb[n1 + i] = scr[L.ST + i];
  }
  for (int k = lane; k < n1; k += G) Sb[k * n1 + ns] = 0.;
  grp.sync();
  JWriter<G> jw{Sb, n1, 0, 2, rho};
  run_program<G>(p.prog_j, lane, b.d, scr, jw);
  grp.sync();
}

__device__ __forceinline__ ReactorCfg cfg_of(const KParams &p)
{
  ReactorCfg cfg;
  cfg.configuration = p.configuration;
  cfg.heat = p.heat;
  cfg.option = p.option;
  cfg.Tc = p.Tc;
  cfg.Tr = p.Tr;
  cfg.hc = p.hc;
  cfg.eps = p.eps;
  cfg.SoV = p.SoV;
  cfg.open = p.open;
  cfg.tau = p.tau;
  cfg.rho_in = p.rho_in;
  cfg.Tin = p.Tin;
  cfg.yin = p.yin;
  return cfg;
}

template <int G, int MODE>
__global__ void __launch_bounds__(256) chem_kernel(const KParams p)
{
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint64_t bar;
  const DevMech &m = p.m;
  if (!stage_to_smem(smem, p.blob, m.blob_bytes, &bar, p.status)) return;
  const Blob b = blob_at(m, smem);
  const ScratchLayout &L = p.L;
  const int gid = threadIdx.x / G;
  const int scr_doubles = jac_mode(MODE) ? L.total : L.total_rhs;
  double *scr = reinterpret_cast<double *>(smem + m.blob_bytes) + (size_t)gid * scr_doubles;
  const Group<G> grp;
  const Progs pg{p.prog_w, p.prog_full, p.prog_j};
  const ReactorCfg cfg = cfg_of(p);
  for (int st = blockIdx.x * p.groups_per_cta + gid; st < p.n; st += gridDim.x * p.groups_per_cta)
    eval_state<G, MODE>(p, m, b, L, scr, grp, pg, cfg, st);
}

// Thread per state: the 32 lanes of a warp evaluate 32 states in lockstep (the same mechanism, so the same
// instruction stream), each FP64 instruction carrying 32 useful lanes. Scratch is interleaved per warp in global
// memory (L2/HBM); the mechanism blob is in shared memory, read by all lanes at once.
template <int MODE>
__global__ void __launch_bounds__(128) chem_kernel_tps(const KParams p)
{
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint64_t bar;
  const DevMech &m = p.m;
  if (!stage_to_smem(smem, p.blob, m.blob_bytes, &bar, p.status)) return;
  const Blob b = blob_at(m, smem);
  const ScratchLayout &L = p.L;
  const int lane = threadIdx.x & 31;
  const int wg = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int nwg = gridDim.x * (blockDim.x >> 5);
  const int scr_doubles = jac_mode(MODE) ? L.total : L.total_rhs;
  const ScrStrided scr{p.gscratch + (size_t)wg * scr_doubles * 32 + lane};
  const Group<1> grp;
  const Progs pg{p.prog_w, p.prog_full, p.prog_j};
  const ReactorCfg cfg = cfg_of(p);
  for (int base = wg * 32; base < p.n; base += nwg * 32) {
    const int st = base + lane;
    if (st < p.n) eval_state<1, MODE>(p, m, b, L, scr, grp, pg, cfg, st);
  }
}

// Interleaved scratch of the thread-per-state kernels: one slot of 32 x (per-state scratch) doubles per warp of
// the launch, at most one per warp that can be resident at once (the CTAS knob, else the occupancy of the kernel at
// the blob's shared memory). The caller's workspace holds the slots.
constexpr int kTpsThreads = 128;

size_t tps_resident_warps(const HostMech &hm)
{
  int dev, nsm;
  CUDA_THROW(cudaGetDevice(&dev));
  CUDA_THROW(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  int ctas = hm.tune[SF_TUNE_TPS_CTAS];
  if (ctas <= 0) {
    const size_t smem = hm.dm.blob_bytes;
    ensure_dynamic_smem((const void *)chem_kernel_tps<MODE_JAC>, smem);
    CUDA_THROW(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctas, chem_kernel_tps<MODE_JAC>, kTpsThreads, smem));
    if (ctas < 1) throw sf_error(SF_ERR_UNSUPPORTED, "mechanism too large for the thread-per-state kernels");
  }
  return (size_t)nsm * ctas * (kTpsThreads / 32);
}

size_t tps_scratch_bytes(const HostMech &hm, int mode, long long n)
{
  if (n <= 0) return 0;
  const size_t per_warp = (size_t)32 * (jac_mode(mode) ? hm.sl.total : hm.sl.total_rhs) * 8;
  const size_t wpb = kTpsThreads / 32;  // whole blocks: every warp of a launch has a slot
  const size_t warps = std::min<size_t>(((size_t)((n + 31) / 32) + wpb - 1) / wpb * wpb, tps_resident_warps(hm));
  return per_warp * warps;
}

// ------------------------------------------------------------------------------------------------ launchers
namespace {

int pick_group(const DevMech &m) { return m.nr >= 96 || m.ns >= 24 ? 32 : (m.nr >= 24 ? 16 : 8); }

template <int MODE>
int launch_tps(const HostMech &hm, KParams &p, cudaStream_t st, void *ws, size_t ws_bytes)
{
  const auto &progs = hm.programs_for(1);
  p.m = hm.dm;
  p.blob = hm.d_blob;
  p.status = hm.d_status;
  p.L = hm.sl;
  p.prog_w = progs.progs[0];
  p.prog_full = progs.progs[1];
  p.prog_j = (MODE == MODE_SENS) ? progs.progs[3] : progs.progs[2];
  if (p.n == 0) return SF_OK;
  const size_t per_warp = (size_t)32 * (jac_mode(MODE) ? hm.sl.total : hm.sl.total_rhs) * 8;
  const size_t need_bytes = tps_scratch_bytes(hm, MODE, p.n);
  if (!ws || ws_bytes < need_bytes)
    throw sf_error(SF_ERR_WORKSPACE, "workspace smaller than sf_chem_workspace_size reports (" +
                                         std::to_string(need_bytes) + " bytes for these states)");
  // slots of whole 4-warp blocks: a launch never has more warps than the workspace has slots
  const long long blocks_avail = (long long)(ws_bytes / per_warp) / (kTpsThreads / 32);
  const long long max_blocks = std::max<long long>(1, (long long)(tps_resident_warps(hm) / (kTpsThreads / 32)));
  p.gscratch = static_cast<double *>(ws);
  const size_t smem = hm.dm.blob_bytes;
  ensure_dynamic_smem((const void *)chem_kernel_tps<MODE>, smem);
  const long long need = ((long long)p.n + kTpsThreads - 1) / kTpsThreads;
  const int grid = (int)std::max<long long>(1, std::min(need, std::min(blocks_avail, max_blocks)));
  chem_kernel_tps<MODE><<<grid, kTpsThreads, smem, st>>>(p);
  CUDA_THROW(cudaGetLastError());
  return SF_OK;
}

template <int MODE>
int launch_mode(const HostMech &hm, KParams &p, cudaStream_t st, int G_req, void *ws, size_t ws_bytes)
{
  if (G_req == 1) return launch_tps<MODE>(hm, p, st, ws, ws_bytes);
  const int G = G_req > 0 ? G_req : pick_group(hm.dm);
  const auto &progs = hm.programs_for(G);
  p.m = hm.dm;
  p.blob = hm.d_blob;
  p.status = hm.d_status;
  p.L = hm.sl;
  p.prog_w = progs.progs[0];
  p.prog_full = progs.progs[1];
  p.prog_j = (MODE == MODE_SENS) ? progs.progs[3] : progs.progs[2];
  const int scr_doubles = jac_mode(MODE) ? hm.sl.total : hm.sl.total_rhs;
  int dev;
  CUDA_THROW(cudaGetDevice(&dev));
  int smem_max, nsm;
  CUDA_THROW(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  CUDA_THROW(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const size_t per_group = (size_t)scr_doubles * 8;
  const size_t avail = (size_t)smem_max - hm.dm.blob_bytes - 64;
  if ((size_t)smem_max <= (size_t)hm.dm.blob_bytes + per_group)
    throw sf_error(SF_ERR_UNSUPPORTED, "mechanism too large for the shared-memory kernels");
  int groups = (int)std::min<size_t>(avail / per_group, 256 / G);
  groups = std::max(groups, 1);
  p.groups_per_cta = groups;
  const size_t smem = hm.dm.blob_bytes + per_group * groups;
  const int threads = groups * G;
  void (*kern)(const KParams);
  switch (G) {
  case 8: kern = chem_kernel<8, MODE>; break;
  case 16: kern = chem_kernel<16, MODE>; break;
  default: kern = chem_kernel<32, MODE>; break;
  }
  ensure_dynamic_smem((const void *)kern, smem);
  const int blocks_per_sm = std::max(1, (int)(((size_t)smem_max) / smem));
  const long long need = ((long long)p.n + groups - 1) / groups;
  const int grid = (int)std::max<long long>(1, std::min<long long>(need, (long long)nsm * blocks_per_sm));
  if (p.n == 0) return SF_OK;
  kern<<<grid, threads, smem, st>>>(p);
  CUDA_THROW(cudaGetLastError());
  return SF_OK;
}

}  // namespace

int chem_launch(const HostMech &hm, int mode, KParams &p, cudaStream_t st, int G, void *ws, size_t ws_bytes)
{
  switch (mode) {
  case MODE_RATES: return launch_mode<MODE_RATES>(hm, p, st, G, ws, ws_bytes);
  case MODE_SENS: return launch_mode<MODE_SENS>(hm, p, st, G, ws, ws_bytes);
  case MODE_RHS:
    return p.open ? launch_mode<MODE_RHS_OPEN>(hm, p, st, G, ws, ws_bytes)
                  : launch_mode<MODE_RHS>(hm, p, st, G, ws, ws_bytes);
  default:
    return p.open ? launch_mode<MODE_JAC_OPEN>(hm, p, st, G, ws, ws_bytes)
                  : launch_mode<MODE_JAC>(hm, p, st, G, ws, ws_bytes);
  }
}

}  // namespace sfgb

// ================================================================================================== C ABI
using namespace sfgb;

namespace {
thread_local std::string t_err;
template <class F>
int guard(F f)
{
  try {
    t_err.clear();
    return f();
  } catch (sf_error &e) {
    t_err = e.what();
    return e.code;
  } catch (std::exception &e) {
    t_err = e.what();
    return SF_ERR_INVALID_ARGUMENT;
  }
}
// lanes per state for a kernel family: the autotuned value if one was set, else the built-in rule
int group_of(const HostMech &hm, int knob)
{
  const int g = hm.tune[knob];
  return (g == 1 || g == 8 || g == 16 || g == 32) ? g : 0;
}
}  // namespace

void sfgb::set_error(const std::string &msg) { t_err = msg; }

extern "C" {

const char *sf_last_error(void) { return t_err.c_str(); }

int sf_mech_set_tuning(sf_mech *mech, int knob, int value)
{
  if (!mech || knob < 0 || knob >= SF_TUNE_KNOBS) {
    t_err = "sf_mech_set_tuning: bad argument";
    return SF_ERR_INVALID_ARGUMENT;
  }
  const bool ok = (knob <= SF_TUNE_GROUP_JAC) ? (value == 0 || value == 1 || value == 8 || value == 16 || value == 32)
                  : (knob == SF_TUNE_INTEGRATE_WARPS) ? (value >= 0 && value <= 8)
                  : (knob == SF_TUNE_TPS_CTAS) ? (value >= 0 && value <= 16)
                  : (knob == SF_TUNE_INTEGRATE_SCRATCH) ? (value >= 0 && value <= 3)
                  : (value >= 0 && value <= 2);
  if (!ok) {
    t_err = "sf_mech_set_tuning: value out of range for this knob";
    return SF_ERR_INVALID_ARGUMENT;
  }
  mech->m.tune[knob] = value;
  return SF_OK;
}

int sf_mech_layout(const sf_mech *mech, int *scratch_rhs_doubles, int *scratch_total_doubles,
                   long long *blob_bytes)
{
  if (!mech) {
    t_err = "sf_mech_layout: null mechanism";
    return SF_ERR_INVALID_ARGUMENT;
  }
  if (scratch_rhs_doubles) *scratch_rhs_doubles = mech->m.sl.total_rhs;
  if (scratch_total_doubles) *scratch_total_doubles = mech->m.sl.total;
  if (blob_bytes) *blob_bytes = (long long)mech->m.dm.blob_bytes;
  return SF_OK;
}

int sf_mech_get_tuning(const sf_mech *mech, int knob, int *value)
{
  if (!mech || !value || knob < 0 || knob >= SF_TUNE_KNOBS) {
    t_err = "sf_mech_get_tuning: bad argument";
    return SF_ERR_INVALID_ARGUMENT;
  }
  *value = mech->m.tune[knob];
  return SF_OK;
}
const char *sf_version(void) { return "spitfire_gb300 0.1 (sm_103a)"; }

int sf_mech_create(const sf_mech_desc *desc, sf_mech **out)
{
  return guard([&] {
    if (!desc || !out) throw sf_error(SF_ERR_INVALID_ARGUMENT, "null argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw sf_error(SF_ERR_NO_DEVICE, "no CUDA device");
    auto *m = new sf_mech();
    try {
      m->m.build(desc);
    } catch (...) {
      delete m;
      throw;
    }
    *out = m;
    return SF_OK;
  });
}

int sf_mech_destroy(sf_mech *m)
{
  delete m;
  return SF_OK;
}

int sf_mech_info(const sf_mech *m, int *ns, int *nr, int *counts)
{
  return guard([&] {
    if (!m) throw sf_error(SF_ERR_INVALID_ARGUMENT, "null mechanism");
    if (ns) *ns = m->m.dm.ns;
    if (nr) *nr = m->m.dm.nr;
    if (counts) {
      int c[6] = {0, 0, 0, 0, 0, 0};
      for (const auto &x : m->m.rx) {
        c[x.kind - 1]++;
        if (x.dense) c[4]++;
        if (x.has_orders) c[5]++;
      }
      for (int i = 0; i < 6; ++i) counts[i] = c[i];
    }
    return SF_OK;
  });
}

int sf_production_rates_batch(const sf_mech *mech, int n, const double *T, const double *rho, const double *Y,
                              double *out_w, void *workspace, size_t workspace_bytes, void *stream)
{
  return guard([&] {
    if (!mech || n < 0 || (n > 0 && (!T || !rho || !Y || !out_w))) throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad argument");
    KParams p{};
    p.n = n;
    p.T = T;
    p.rho = rho;
    p.Y = Y;
    p.out_w = out_w;
    p.configuration = 0;
    return chem_launch(mech->m, MODE_RATES, p, (cudaStream_t)stream, group_of(mech->m, SF_TUNE_GROUP_RATES),
                       workspace, workspace_bytes);
  });
}

int sf_rates_sens_batch(const sf_mech *mech, int n, const double *rho, const double *T, const double *Y, int option,
                        double *out_w, double *out_sens, void *workspace, size_t workspace_bytes, void *stream)
{
  return guard([&] {
    if (!mech || n < 0 || (n > 0 && (!T || !rho || !Y || !out_w || !out_sens)))
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad argument");
    if (option < 0 || option > 2) throw sf_error(SF_ERR_INVALID_ARGUMENT, "rates sensitivity option must be 0, 1 or 2");
    KParams p{};
    p.n = n;
    p.T = T;
    p.rho = rho;
    p.Y = Y;
    p.option = option;
    p.out_w = out_w;
    p.out_S = out_sens;
    return chem_launch(mech->m, MODE_SENS, p, (cudaStream_t)stream, group_of(mech->m, SF_TUNE_GROUP_SENS),
                       workspace, workspace_bytes);
  });
}

static void fill_reactor(KParams &p, const sf_reactor_params *rp)
{
  if (!rp) throw sf_error(SF_ERR_INVALID_ARGUMENT, "null reactor params");
  if (rp->configuration != 0 && rp->configuration != 1) throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad configuration");
  if (rp->heat_transfer < 0 || rp->heat_transfer > 2) throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad heat_transfer");
  if (rp->open) {
    if (!rp->inflow_Y) throw sf_error(SF_ERR_INVALID_ARGUMENT, "open reactor without feed mass fractions");
    if (!(rp->tau > 0.)) throw sf_error(SF_ERR_INVALID_ARGUMENT, "open reactor needs a positive mixing time");
    if (!(rp->inflow_temperature > 0.)) throw sf_error(SF_ERR_INVALID_ARGUMENT, "open reactor needs a feed temperature");
  }
  p.open = rp->open ? 1 : 0;
  p.tau = rp->tau;
  p.rho_in = rp->inflow_density;
  p.Tin = rp->inflow_temperature;
  p.yin = rp->inflow_Y;
  p.configuration = rp->configuration;
  p.heat = rp->heat_transfer;
  p.pressure = rp->pressure;
  p.Tc = rp->fluid_temperature;
  p.Tr = rp->surface_temperature;
  p.hc = rp->h_convection;
  p.eps = rp->eps_radiation;
  p.SoV = rp->surface_area_to_volume;
}

int sf_reactor_rhs_batch(const sf_mech *mech, const sf_reactor_params *rp, int n, const double *q,
                         const double *pressures, double *out_rhs, void *workspace, size_t workspace_bytes,
                         void *stream)
{
  return guard([&] {
    if (!mech || n < 0 || (n > 0 && (!q || !out_rhs))) throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad argument");
    KParams p{};
    fill_reactor(p, rp);
    p.n = n;
    p.q = q;
    p.pressures = pressures;
    p.out_rhs = out_rhs;
    return chem_launch(mech->m, MODE_RHS, p, (cudaStream_t)stream, group_of(mech->m, SF_TUNE_GROUP_RHS), workspace,
                       workspace_bytes);
  });
}

int sf_reactor_jac_batch(const sf_mech *mech, const sf_reactor_params *rp, int rates_option, int n, const double *q,
                         const double *pressures, double *out_rhs, double *out_jac, void *workspace,
                         size_t workspace_bytes, void *stream)
{
  return guard([&] {
    if (!mech || n < 0 || (n > 0 && (!q || !out_rhs || !out_jac))) throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad argument");
    if (rates_option < 0 || rates_option > 2) throw sf_error(SF_ERR_INVALID_ARGUMENT, "rates option must be 0, 1 or 2");
    KParams p{};
    fill_reactor(p, rp);
    p.n = n;
    p.q = q;
    p.pressures = pressures;
    p.option = rates_option;
    p.out_rhs = out_rhs;
    p.out_J = out_jac;
    return chem_launch(mech->m, MODE_JAC, p, (cudaStream_t)stream, group_of(mech->m, SF_TUNE_GROUP_JAC), workspace,
                       workspace_bytes);
  });
}

size_t sf_chem_workspace_size(const sf_mech *mech, int kind, int n)
{
  if (!mech || n <= 0 || kind < SF_CHEM_RATES || kind > SF_CHEM_JAC) return 0;
  static const int knob[4] = {SF_TUNE_GROUP_RATES, SF_TUNE_GROUP_SENS, SF_TUNE_GROUP_RHS, SF_TUNE_GROUP_JAC};
  static const int mode[4] = {MODE_RATES, MODE_SENS, MODE_RHS, MODE_JAC};
  if (group_of(mech->m, knob[kind]) != 1) return 0;
  try {
    return tps_scratch_bytes(mech->m, mode[kind], n);
  } catch (sf_error &e) {
    t_err = e.what();
    return 0;
  }
}

size_t sf_reactor_jac_host_workspace_size(const sf_mech *mech, const sf_reactor_params *rp, int n)
{
  if (!mech || !rp || n < 0) return 0;
  const size_t neq = (size_t)mech->m.dm.ns + (rp->configuration == 1 ? 1 : 0);
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  return up(n * neq * 8) + up((size_t)n * 8) + up(n * neq * 8) + up(n * neq * neq * 8) +
         sf_chem_workspace_size(mech, SF_CHEM_JAC, n);
}

int sf_reactor_jac_host_batch(const sf_mech *mech, const sf_reactor_params *rp, int rates_option, int n,
                              const double *q_host, const double *pressures_host, double *out_rhs_host,
                              double *out_jac_host, int chunk_states, void *workspace, size_t workspace_bytes,
                              void *stream)
{
  return guard([&]() -> int {
    if (!mech || !rp || n < 0 || (n > 0 && (!q_host || !out_rhs_host || !out_jac_host)))
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad argument");
    if (rates_option < 0 || rates_option > 2) throw sf_error(SF_ERR_INVALID_ARGUMENT, "rates option must be 0, 1 or 2");
    if (n == 0) return SF_OK;
    if (!workspace || workspace_bytes < sf_reactor_jac_host_workspace_size(mech, rp, n))
      throw sf_error(SF_ERR_WORKSPACE, "workspace smaller than sf_reactor_jac_host_workspace_size reports");
    HostMech &hm = const_cast<HostMech &>(mech->m);
    // the copy stream and chunk events belong to the mechanism: calls from several threads take turns here (each
    // event wait captures its own record), their copies sharing the copy stream
    std::lock_guard<std::mutex> lock(hm.host_batch_mutex);
    const size_t neq = (size_t)hm.dm.ns + (rp->configuration == 1 ? 1 : 0);
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    char *w = static_cast<char *>(workspace);
    const size_t io_bytes = up(n * neq * 8) + up((size_t)n * 8) + up(n * neq * 8) + up(n * neq * neq * 8);
    double *q = reinterpret_cast<double *>(w);
    double *pr = reinterpret_cast<double *>(w + up(n * neq * 8));
    double *rhs = reinterpret_cast<double *>(w + up(n * neq * 8) + up((size_t)n * 8));
    double *J = reinterpret_cast<double *>(w + up(n * neq * 8) + up((size_t)n * 8) + up(n * neq * 8));
    void *kws = w + io_bytes;  // the kernel's scratch: every chunk runs on `stream`, one after another
    const size_t kws_bytes = workspace_bytes - io_bytes;
    cudaStream_t st = (cudaStream_t)stream;
    const int G = group_of(hm, SF_TUNE_GROUP_JAC);
    // chunk: by default the states one wave of the thread-per-state kernel covers (its resident warps), else half
    int chunk = chunk_states;
    if (chunk <= 0) chunk = G == 1 ? (int)std::min<size_t>((size_t)n, tps_resident_warps(hm) * 32) : (n + 1) / 2;
    chunk = std::max(1, std::min(chunk, n));
    const int nchunks = (n + chunk - 1) / chunk;
    if (!hm.copy_stream) CUDA_THROW(cudaStreamCreateWithFlags(&hm.copy_stream, cudaStreamNonBlocking));
    while ((int)hm.events.size() < nchunks + 1) {
      cudaEvent_t e;
      CUDA_THROW(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      hm.events.push_back(e);
    }
    // inputs, then per chunk: the Jacobians on the caller's stream and their copies back on the copy stream, so that
    // a chunk's copies overlap the next chunk's kernel
    CUDA_THROW(cudaMemcpyAsync(q, q_host, n * neq * 8, cudaMemcpyHostToDevice, st));
    if (pressures_host) CUDA_THROW(cudaMemcpyAsync(pr, pressures_host, (size_t)n * 8, cudaMemcpyHostToDevice, st));
    for (int c = 0; c < nchunks; ++c) {
      const size_t a = (size_t)c * chunk;
      const int m = (int)std::min<size_t>(chunk, n - a);
      KParams p{};
      fill_reactor(p, rp);
      p.n = m;
      p.q = q + a * neq;
      p.pressures = pressures_host ? pr + a : nullptr;
      p.option = rates_option;
      p.out_rhs = rhs + a * neq;
      p.out_J = J + a * neq * neq;
      const int rc = chem_launch(hm, MODE_JAC, p, st, G, kws, kws_bytes);
      if (rc != SF_OK) return (int)rc;
      CUDA_THROW(cudaEventRecord(hm.events[c], st));
      CUDA_THROW(cudaStreamWaitEvent(hm.copy_stream, hm.events[c], 0));
      CUDA_THROW(cudaMemcpyAsync(out_rhs_host + a * neq, rhs + a * neq, (size_t)m * neq * 8, cudaMemcpyDeviceToHost,
                                 hm.copy_stream));
      CUDA_THROW(cudaMemcpyAsync(out_jac_host + a * neq * neq, J + a * neq * neq, (size_t)m * neq * neq * 8,
                                 cudaMemcpyDeviceToHost, hm.copy_stream));
    }
    CUDA_THROW(cudaEventRecord(hm.events[nchunks], hm.copy_stream));
    CUDA_THROW(cudaStreamWaitEvent(st, hm.events[nchunks], 0));
    return SF_OK;
  });
}

int sf_device_status(const sf_mech *mech, int clear)
{
  if (!mech || !mech->m.d_status) return -1;
  int v = 0;
  if (cudaMemcpy(&v, mech->m.d_status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  if (clear && v) cudaMemset(mech->m.d_status, 0, sizeof(int));
  return v;
}

}  // extern "C"

// Reactor right-hand sides and Jacobians with an explicit lane width G (8, 16 or 32 lanes per state: shared-memory
// scratch, no workspace), for callers whose batch is too small for the thread-per-state shape the autotuner may have
// chosen for large batches.
void sfgb::reactor_jac_lanes(const sf_mech *mech, const sf_reactor_params *rp, int rates_option, int n,
                             const double *q, const double *pressures, double *out_rhs, double *out_jac, int G,
                             cudaStream_t st)
{
  if (G != 8 && G != 16 && G != 32) throw sf_error(SF_ERR_INVALID_ARGUMENT, "lane width must be 8, 16 or 32");
  KParams p{};
  fill_reactor(p, rp);
  p.n = n;
  p.q = q;
  p.pressures = pressures;
  p.option = rates_option;
  p.out_rhs = out_rhs;
  p.out_J = out_jac;
  const int rc = chem_launch(mech->m, MODE_JAC, p, st, G, nullptr, 0);
  if (rc != SF_OK) throw sf_error(rc, "reactor Jacobian launch failed");
}
