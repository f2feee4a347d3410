// Parameter adjoint of the reactor right-hand side: for reactor states q and adjoint vectors w, the products
// w^T df/dtheta for the rate parameters theta = (ln A_r, E_a,r) of every reaction r (the forward, or for falloff
// reactions the high-pressure, Arrhenius coefficients).
//
// The net rate of progress q_r is linear in the forward rate constant k_r except through the falloff blending
// factor of Lindemann/Troe reactions, whose reduced pressure is Pr = k0 [M] / k_inf. With s_r = dq_r / d ln k_r:
//   simple, three-body:  s_r = q_r
//   Lindemann:           s_r = q_r Pr / (1 + Pr)
//   Troe:                s_r = q_r (Pr / (1 + Pr) - d ln F / d ln Pr), F from the production-rate form of
//                        chemistry_kernels.cpp:280-312 (log10 F = log10 Fc / (1 + f1^2))
// and d ln k_r / d ln A_r = 1, d ln k_r / d E_a,r = -1 / (R T) (E_a in J/kmol, R = 8314.46 J/kmol/K).
// The reaction's column of df/dtheta is s_r times its column of the species production: the mass production
// nu_sr M_s enters dY_s/dt = w_s / rho and dT/dt = -sum_s e_s w_s / (rho c) (c = cp isobaric, cv isochoric; e the
// species enthalpy or energy), so w^T df/d ln A_r = s_r sum_s nu_sr M_s (w_Y_s - w_T e_s / c) / rho, where the
// last species is not a state variable (w_Y = 0 there).
#include "reactor_eval.cuh"
#include "sf_internal.h"

namespace sfgb {
namespace {

struct AdjParams {
  DevMech m;
  const void *blob;
  int *status;
  ScratchLayout L;
  Progs pg;
  ReactorCfg cfg;
  int n_items, stages, neq;
  int wsets;                // adjoint vector sets per state (e.g. one per output)
  double pressure;
  const double *pressures;  // [n_items] or null
  const double *q;          // [n_items][stages][neq]
  const double *w;          // [n_items][wsets][stages][neq]
  double *out;              // [n_items][wsets][2 nr], accumulated
  int groups_per_cta;
};

// d ln q_r / d ln k_r (the factor s_r / q_r above) of a falloff reaction at the state of the group's scratch
__device__ double falloff_factor(const DevMech &m, const Blob &b, const ScratchLayout &L, const double *scr,
                                 const StateCtx &s, int r, int kind, int kform, int info)
{
  const double *kc = b.d + m.d_kf + 3 * r;
  double kf;
  switch (kform) {
  case 0: kf = kc[0]; break;
  case 1: kf = kc[0] * s.T; break;
  case 2: kf = kc[0] * s.T * s.T; break;
  case 3: kf = kc[0] * s.invT; break;
  default: kf = kc[0] * tab_exp(kc[1] * s.logT - kc[2] * s.invT, b.d + m.d_exptab); break;
  }
  const double *y = scr + L.y;
  const int t0 = b.i[m.i_tb_off + r], t1 = b.i[m.i_tb_off + r + 1];
  double sumtb = 0.;
  for (int j = t0; j < t1; ++j) sumtb += b.d[m.d_tbeff + j] * y[b.i[m.i_tb + j]];
  const double M = b.d[m.d_beff + r] * s.ct + s.rho * sumtb;
  const int f = b.i[m.i_fall + r];
  const double *kp = b.d + m.d_kp + 3 * f;
  const double pr = kp[0] * tab_exp(kp[1] * s.logT - kp[2] * s.invT, b.d + m.d_exptab) / kf * M;
  double fac = pr / (1. + pr);
  if (kind == 4 && pr > 1.e-300) {
    const double *tr = b.d + m.d_troe + 4 * f;
    const int terms = (info >> RI_TROE_SHIFT) & 7;
    double fc = 0.;
    if (terms & 1) fc += (1 - tr[0]) * tab_exp(-s.T / tr[1], b.d + m.d_exptab);
    if (terms & 2) fc += tr[0] * tab_exp(-s.T / tr[2], b.d + m.d_exptab);
    if (terms & 4) fc += tab_exp(-s.invT * tr[3], b.d + m.d_exptab);
    const double lfc = log10(fc);
    const double nn = 0.75 - 1.27 * lfc;
    const double lpc = log10(pr) + (-0.4 - 0.67 * lfc);
    const double den = nn - 0.14 * lpc;
    const double f1 = lpc / den;
    const double g = 1. + f1 * f1;
    // d log10 F / d log10 Pr = log10 Fc * (-2 f1 / g^2) * d f1 / d lpc, d f1 / d lpc = nn / den^2
    fac -= lfc * (-2. * f1 / (g * g)) * nn / (den * den);
  }
  return fac;
}

template <int G>
__global__ void __launch_bounds__(256) rate_param_adjoint_kernel(const AdjParams p)
{
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ uint64_t bar;
  const DevMech &m = p.m;
  if (!stage_to_smem(smem, p.blob, m.blob_bytes, &bar, p.status)) return;
  const Blob b = blob_at(m, smem);
  const ScratchLayout &L = p.L;
  const int gid = threadIdx.x / G;
  double *scr = reinterpret_cast<double *>(smem + m.blob_bytes) + (size_t)gid * (L.total_rhs + p.neq + 2);
  double *rhs_tmp = scr + L.total_rhs;
  const Group<G> grp;
  const int lane = grp.lane;
  const int ns = m.ns, nr = m.nr, neq = p.neq;
  const bool isochoric = p.cfg.configuration == 1;
  const int tix = isochoric ? 1 : 0;
  NoJ noj;
  for (int it = blockIdx.x * p.groups_per_cta + gid; it < p.n_items; it += gridDim.x * p.groups_per_cta) {
    const double pres = isochoric ? 0. : (p.pressures ? p.pressures[it] : p.pressure);
    for (int st = 0; st < p.stages; ++st) {
      const double *qs = p.q + ((size_t)it * p.stages + st) * neq;
      reactor_eval<G, false, default_unroll(G), false>(m, b, L, scr, grp, qs, pres, p.cfg, p.pg, rhs_tmp, noj);
      // state quantities (as in reactor_eval)
      const double T = qs[tix];
      double sim = 0., cmix = 0.;
      for (int i = lane; i < ns; i += G) {
        sim += scr[L.y + i] * b.d[m.d_invmw + i];
        cmix += scr[L.y + i] * scr[L.cpv + i];
      }
      sim = grp.sum(sim);
      cmix = grp.sum(cmix);
      const double mmw = 1. / sim;
      const double rho = isochoric ? qs[0] : pres * mmw / (T * m.Ru);
      StateCtx s;
      s.T = T;
      s.logT = log(T);
      s.invT = 1. / T;
      s.rho = rho;
      s.invRho = 1. / rho;
      s.mmw = mmw;
      s.invM = sim;
      s.ct = rho * sim;
      for (int r = lane; r < nr; r += G) {
        const int info = b.i[m.i_info + r];
        const int kind = (info >> RI_KIND_SHIFT) & 7;
        const int kform = (info >> RI_KFORM_SHIFT) & 7;
        double sr = scr[L.q + r];
        if (kind == 3 || kind == 4) sr *= falloff_factor(m, b, L, scr, s, r, kind, kform, info);
        const int n0 = b.i[m.i_net_off + r], n1 = b.i[m.i_net_off + r + 1];
        const int ro = b.i[m.i_orig + r];  // reported in the order the mechanism was described
        for (int o = 0; o < p.wsets; ++o) {  // the rates above serve every adjoint vector of this state
          const double *w = p.w + (((size_t)it * p.wsets + o) * p.stages + st) * neq;
          double *out = p.out + ((size_t)it * p.wsets + o) * 2 * nr;
          const double wTc = w[tix] / cmix;
          double B = 0.;
          for (int j = n0; j < n1; ++j) {
            const int sp = b.i[m.i_net + j] & 0xFFFF;
            const double wy = sp < ns - 1 ? w[tix + 1 + sp] : 0.;
            B += b.d[m.d_netc + j] * (wy - wTc * scr[L.eh + sp]);
          }
          const double g = sr * B * s.invRho;
          out[2 * ro] += g;
          out[2 * ro + 1] += -g * s.invT * m.invRu;
        }
      }
      grp.sync();
    }
  }
}

}  // namespace

void launch_rate_param_adjoint(const HostMech &hm, int configuration, double pressure, int n_items, int wsets,
                               int stages, const double *q, const double *pressures, const double *w, double *out,
                               cudaStream_t st)
{
  if (n_items == 0) return;
  constexpr int G = 32;
  const auto &progs = hm.programs_for(G);
  AdjParams p{};
  p.m = hm.dm;
  p.blob = hm.d_blob;
  p.status = hm.d_status;
  p.L = hm.sl;
  p.pg.w = progs.progs[0];
  p.pg.full = progs.progs[1];
  p.pg.j = progs.progs[2];
  p.cfg.configuration = configuration;
  p.cfg.heat = 0;
  p.cfg.option = 0;
  p.n_items = n_items;
  p.stages = stages;
  p.wsets = wsets;
  p.neq = configuration == 1 ? hm.dm.ns + 1 : hm.dm.ns;
  p.pressure = pressure;
  p.pressures = pressures;
  p.q = q;
  p.w = w;
  p.out = out;
  int dev, smem_max, nsm;
  CUDA_THROW(cudaGetDevice(&dev));
  CUDA_THROW(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  CUDA_THROW(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const size_t per = (size_t)(hm.sl.total_rhs + p.neq + 2) * 8;
  const size_t avail = (size_t)smem_max - hm.dm.blob_bytes - 64;
  const int groups = (int)std::min<size_t>(avail / per, 256 / G);
  if (groups < 1) throw sf_error(SF_ERR_UNSUPPORTED, "mechanism too large for the parameter-adjoint kernel");
  p.groups_per_cta = groups;
  const size_t smem = hm.dm.blob_bytes + per * groups;
  ensure_dynamic_smem((const void *)rate_param_adjoint_kernel<G>, smem);
  const int bps = std::max(1, (int)((size_t)smem_max / smem));
  const int grid = (int)std::max<long long>(
      1, std::min<long long>(((long long)n_items + groups - 1) / groups, (long long)nsm * bps));
  rate_param_adjoint_kernel<G><<<grid, groups * G, smem, st>>>(p);
  CUDA_THROW(cudaGetLastError());
}

}  // namespace sfgb

using namespace sfgb;

extern "C" {

int sf_rate_param_adjoint_batch(const sf_mech *mech, const sf_reactor_params *rp, int n_items, int stages,
                                const double *q, const double *pressures, const double *w, double *out_grad,
                                void *stream)
{
  try {
    if (!mech || !rp || n_items < 0 || stages < 1 || (n_items > 0 && (!q || !w || !out_grad)))
      throw sf_error(SF_ERR_INVALID_ARGUMENT, "sf_rate_param_adjoint_batch: bad argument");
    if (rp->open || rp->heat_transfer != 0)
      throw sf_error(SF_ERR_UNSUPPORTED, "parameter adjoints cover closed adiabatic reactors");
    if (rp->configuration != 0 && rp->configuration != 1) throw sf_error(SF_ERR_INVALID_ARGUMENT, "bad configuration");
    launch_rate_param_adjoint(mech->m, rp->configuration, rp->pressure, n_items, 1, stages, q, pressures, w,
                              out_grad, (cudaStream_t)stream);
    return SF_OK;
  } catch (sf_error &e) {
    set_error(e.what());
    return e.code;
  }
}

}  // extern "C"
