/*
 * ORACLE -- test infrastructure, not the product.
 *
 * A CPU restatement of Spitfire's Griffon chemistry engine (sandialabs/Spitfire v1.3.0,
 * src/spitfire/griffon/src/, all .cpp files), used only by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * --impl reference legs as the checker and the timed CPU baseline. Nothing in spitfire_gb300/ links or calls it.
 *
 * Parity pinning: tests/test_oracle_golden.py checks every function here against golden vectors produced by the
 * reference Griffon itself (compiled unmodified from its sources by `make -C oracle ref`, fixtures written by
 * tests/golden/make_golden.py).
 *
 * Scope restated (file:line in src/spitfire/griffon/):
 *   mechanism finalize            src/chemistry_setup.cpp:102-130 (NASA7 scaling), :406-419 (efficiencies), :459-732
 *   thermodynamics                src/thermodynamics_kernels.cpp:18-382
 *   production rates              src/chemistry_kernels.cpp:35-463
 *   rate sensitivities (0, 1, 2)  src/rates_sensitivities_exact.cpp:33-1028, _sparse.cpp (same values),
 *                                 _no_tbaf_sens.cpp (dCtbaf terms dropped)
 *   reactors                      src/isochoric_reactor_kernels.cpp:18-333, src/isobaric_reactor_kernels.cpp:19-343
 *   flamelets                     src/flamelet_kernels.cpp:31-90, :1039-1409 (eigenvalue option not restated)
 *   block-tridiagonal algebra     src/btddod_matrix_kernels.cpp:19-465, LU as LAPACK dgetrf/dgetrs
 * The loops are restated with general products over reactant/product lists instead of the reference's unrolled
 * order classes, so results agree with the reference to rounding, not bit for bit.
 */
#include "spitfire_gb300.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Rxn {
  int kind = SF_RXN_SIMPLE;
  bool reversible = true;
  bool has_orders = false;
  std::vector<int> reac, reac_nu, prod, prod_nu;  // prod_nu positive
  std::vector<int> net; std::vector<int> net_nu; std::vector<double> net_mw;
  std::vector<int> tb; std::vector<double> tb_eff;  // tb_eff = invMW*(eff - default)
  std::vector<int> sp; std::vector<double> sp_order; std::vector<bool> sp_nonzero;
  double base_eff = 1.;
  double kf[3] = {0, 0, 0}, kp[3] = {0, 0, 0}, troe[4] = {0, 0, 0, 0};
  int kform = 4;         // 0 const, 1 linear, 2 quadratic, 3 reciprocal, 4 arrhenius
  int troe_terms = 0;    // bit 0: (1-A)exp(-T/T3) term present, bit 1: A exp(-T/T1), bit 2: exp(-T2/T)
  int sum_nu = 0, sum_reac_nu = 0, sum_prod_nu = 0;
  bool is_dense = false;
  std::vector<int> sens;
};

struct Mech {
  int ns = 0, nr = 0;
  double Ru = 0, pref = 0;
  std::vector<double> mw, invmw;
  std::vector<int> thermo;
  std::vector<std::array<double, 15>> c;  // Griffon NASA7 storage, chemistry_setup.cpp:102-130
  std::vector<double> tmin, tmax;
  std::vector<std::vector<double>> c9;
  std::vector<Rxn> rx;
};

std::string g_err;

// ---------------------------------------------------------------------------------------------- mechanism
Mech *build(const sf_mech_desc *d)
{
  Mech *m = new Mech();
  m->ns = d->n_species;
  m->nr = d->n_reactions;
  m->Ru = d->gas_constant;
  m->pref = d->ref_pressure;
  const int ns = m->ns;
  m->mw.assign(d->molecular_weights, d->molecular_weights + ns);
  for (double w : m->mw) m->invmw.push_back(1. / w);
  m->thermo.assign(d->thermo_kind, d->thermo_kind + ns);
  m->c.resize(ns);
  m->tmin.resize(ns);
  m->tmax.resize(ns);
  m->c9.resize(ns);
  for (int k = 0; k < ns; ++k) {
    const double *t = d->thermo_coefs + 20 * k;
    auto &c = m->c[k];
    c.fill(0.);
    if (m->thermo[k] == SF_THERMO_NASA7) {
      m->tmin[k] = t[0];
      m->tmax[k] = t[2];
      c[0] = t[1];
      for (int j = 0; j < 7; ++j) c[1 + j] = t[10 + j] * m->Ru;  // high
      for (int j = 0; j < 7; ++j) c[8 + j] = t[3 + j] * m->Ru;   // low
      c[2] /= 2.; c[3] /= 6.; c[4] /= 12.; c[5] /= 20.;
      c[9] /= 2.; c[10] /= 6.; c[11] /= 12.; c[12] /= 20.;
    } else if (m->thermo[k] == SF_THERMO_CONST) {
      m->tmin[k] = t[0];
      m->tmax[k] = t[1];
      c[0] = t[2]; c[1] = t[3]; c[2] = t[4]; c[3] = t[5];
    } else if (m->thermo[k] == SF_THERMO_NASA9) {
      const double *a = d->nasa9_coefs + d->nasa9_offsets[k];
      const int len = d->nasa9_offsets[k + 1] - d->nasa9_offsets[k];
      auto &v = m->c9[k];
      v.assign(a, a + len);
      const int nreg = (int)v[0];
      for (int r = 0; r < nreg; ++r)
        for (int j = 2; j < 11; ++j) v[1 + r * 11 + j] *= m->Ru;  // chemistry_setup.cpp:132-150
      m->tmin[k] = v[1];
      m->tmax[k] = v[1 + (nreg - 1) * 11 + 1];
    }
  }
  for (int r = 0; r < m->nr; ++r) {
    Rxn x;
    x.kind = d->rxn_kind[r];
    x.reversible = d->rxn_reversible[r] != 0;
    for (int j = 0; j < 3; ++j) x.kf[j] = d->rxn_kfwd[3 * r + j];
    if (x.kind == SF_RXN_LINDEMANN || x.kind == SF_RXN_TROE)
      for (int j = 0; j < 3; ++j) x.kp[j] = d->rxn_kflf[3 * r + j];
    if (x.kind == SF_RXN_TROE)
      for (int j = 0; j < 4; ++j) x.troe[j] = d->rxn_troe[4 * r + j];
    for (int i = d->reac_offsets[r]; i < d->reac_offsets[r + 1]; ++i) {
      x.reac.push_back(d->reac_species[i]);
      x.reac_nu.push_back(d->reac_stoich[i]);
    }
    for (int i = d->prod_offsets[r]; i < d->prod_offsets[r + 1]; ++i) {
      x.prod.push_back(d->prod_species[i]);
      x.prod_nu.push_back(d->prod_stoich[i]);
    }
    if (x.kind != SF_RXN_SIMPLE) {
      x.base_eff = d->rxn_default_eff[r];
      for (int i = d->eff_offsets[r]; i < d->eff_offsets[r + 1]; ++i) {
        const int s = d->eff_species[i];
        x.tb.push_back(s);
        x.tb_eff.push_back(m->invmw[s] * (d->eff_values[i] - x.base_eff));  // chemistry_setup.cpp:406-419
      }
    }
    if (d->order_offsets && d->order_offsets[r + 1] > d->order_offsets[r]) {
      x.has_orders = true;
      for (int i = d->order_offsets[r]; i < d->order_offsets[r + 1]; ++i) {
        x.sp.push_back(d->order_species[i]);
        x.sp_order.push_back(d->order_values[i]);
        x.sp_nonzero.push_back(std::abs(d->order_values[i]) > 1.e-12);
      }
    }
    // net stoichiometry in ascending species-index order (std::map<int,...>, chemistry_setup.cpp:462-510)
    std::map<int, int> net;
    x.sum_nu = 0;
    for (size_t i = 0; i < x.reac.size(); ++i) { net[x.reac[i]] += x.reac_nu[i]; x.sum_nu += x.reac_nu[i]; }
    for (size_t i = 0; i < x.prod.size(); ++i) { net[x.prod[i]] -= x.prod_nu[i]; x.sum_nu -= x.prod_nu[i]; }
    for (auto &kv : net)
      if (kv.second != 0) {
        x.net.push_back(kv.first);
        x.net_nu.push_back(kv.second);
        x.net_mw.push_back(1. / m->invmw[kv.first]);
      }
    if (x.net.size() < 2 || x.net.size() > 8) {
      delete m;
      throw std::runtime_error("reaction " + std::to_string(r) + ": bad number of net reacting species");
    }
    x.sum_reac_nu = 0;
    for (int v : x.reac_nu) x.sum_reac_nu += std::abs(v);
    x.sum_prod_nu = 0;
    for (int v : x.prod_nu) x.sum_prod_nu += std::abs(v);
    // is_dense / sens_indices (chemistry_setup.cpp:543-602)
    x.is_dense = x.kind != SF_RXN_SIMPLE;
    auto has_last = [&](const std::vector<int> &v) {
      for (int s : v) if (s == ns - 1) return true;
      return false;
    };
    if (has_last(x.net) || has_last(x.reac) || has_last(x.prod) || has_last(x.tb)) x.is_dense = true;
    if (!x.is_dense) {
      for (const auto *v : {&x.reac, &x.prod, &x.tb})
        for (int s : *v)
          if (std::find(x.sens.begin(), x.sens.end(), s) == x.sens.end()) x.sens.push_back(s);
    }
    // rate-constant temperature form (chemistry_setup.cpp:670-688)
    if (std::abs(x.kf[2]) < 1.e-6) {
      if (std::abs(x.kf[1]) < 1.e-6) x.kform = 0;
      else if (std::abs(x.kf[1] - 1) < 1.e-6) x.kform = 1;
      else if (std::abs(x.kf[1] - 2) < 1.e-6) x.kform = 2;
      else if (std::abs(x.kf[1] + 1) < 1.e-6) x.kform = 3;
      else x.kform = 4;
    } else x.kform = 4;
    // Troe terms present (chemistry_setup.cpp:690-730): troe = [A, T3, T1, T2]
    if (x.kind == SF_RXN_TROE) {
      x.troe_terms = (std::abs(x.troe[1]) > 1.e-8 ? 1 : 0) | (std::abs(x.troe[2]) > 1.e-8 ? 2 : 0) |
                     (std::abs(x.troe[3]) > 1.e-8 ? 4 : 0);
      if (x.troe_terms == 0) {
        delete m;
        throw std::runtime_error("Troe reaction without Troe terms");
      }
    }
    m->rx.push_back(x);
  }
  return m;
}

// ---------------------------------------------------------------------------------------------- thermodynamics
inline double mmw_of(const Mech &m, const double *y)
{
  double s = 0.;
  for (int i = 0; i < m.ns; ++i) s += m.invmw[i] * y[i];
  return 1. / s;
}

// thermodynamics_kernels.cpp:45-131
void cp_mix_species(const Mech &m, double t, const double *y, double *cpmix, double *cpi)
{
  *cpmix = 0.;
  for (int i = 0; i < m.ns; ++i) {
    const auto &c = m.c[i];
    const double mn = m.tmin[i], mx = m.tmax[i];
    double v = 0.;
    if (m.thermo[i] == SF_THERMO_CONST) {
      v = m.invmw[i] * c[3];
    } else if (m.thermo[i] == SF_THERMO_NASA7) {
      double tt = t;
      int base = 8;
      if (t <= c[0] && t >= mn) { tt = t; base = 8; }
      else if (t > c[0] && t <= mx) { tt = t; base = 1; }
      else if (t < mn) { tt = mn; base = 8; }
      else { tt = mx; base = 1; }
      v = m.invmw[i] * (c[base] + tt * (2. * c[base + 1] + tt * (6. * c[base + 2] + tt * (12. * c[base + 3] +
                                                                                        20. * tt * c[base + 4]))));
    } else {
      const auto &c9 = m.c9[i];
      const int nreg = (int)c9[0];
      const double *a = nullptr;
      double tt = t;
      if (t < mn) { tt = mn; a = &c9[3]; }
      else if (t > mx) { tt = mx; a = &c9[1 + (nreg - 1) * 11 + 2]; }
      else
        for (int k = 0; k < nreg; ++k)
          if (t >= c9[1 + k * 11] && t < c9[1 + k * 11 + 1]) { a = &c9[1 + k * 11 + 2]; break; }
      if (!a) { cpi[i] = 0.; continue; }
      const double it = 1. / tt;
      v = m.invmw[i] * (it * (a[1] + it * a[0]) + a[2] + tt * (a[3] + tt * (a[4] + tt * (a[5] + tt * a[6]))));
    }
    cpi[i] = v;
    *cpmix += y[i] * v;
  }
}

// thermodynamics_kernels.cpp:183-260
void cp_sens(const Mech &m, double t, const double *y, double *mix, double *spec)
{
  *mix = 0.;
  for (int i = 0; i < m.ns; ++i) {
    const auto &c = m.c[i];
    double v = 0.;
    if (m.thermo[i] == SF_THERMO_NASA7) {
      if (t <= c[0] && t >= m.tmin[i])
        v = m.invmw[i] * (2. * c[9] + t * (12. * c[10] + t * (36. * c[11] + 80. * t * c[12])));
      else if (t > c[0] && t <= m.tmax[i])
        v = m.invmw[i] * (2. * c[2] + t * (12. * c[3] + t * (36. * c[4] + 80. * t * c[5])));
    } else if (m.thermo[i] == SF_THERMO_NASA9) {
      const auto &c9 = m.c9[i];
      const int nreg = (int)c9[0];
      if (!(t < m.tmin[i] || t > m.tmax[i])) {
        const double it = 1. / t;
        for (int k = 0; k < nreg; ++k)
          if (t >= c9[1 + k * 11] && t < c9[1 + k * 11 + 1]) {
            const double *a = &c9[1 + k * 11 + 2];
            v = m.invmw[i] * (-it * it * (a[1] + it * 2.0 * a[0]) + a[3] + t * (2.0 * a[4] + t * (3.0 * a[5] + t * 4.0 * a[6])));
            break;
          }
      }
    }
    spec[i] = v;
    *mix += y[i] * v;
  }
}

// thermodynamics_kernels.cpp:262-351
void enthalpies(const Mech &m, double t, double *h)
{
  for (int i = 0; i < m.ns; ++i) {
    const auto &c = m.c[i];
    const double mn = m.tmin[i], mx = m.tmax[i];
    if (m.thermo[i] == SF_THERMO_CONST) {
      h[i] = m.invmw[i] * (c[1] + c[3] * (t - c[0]));
    } else if (m.thermo[i] == SF_THERMO_NASA7) {
      if ((t <= c[0] && t >= mn) || (t > c[0] && t <= mx)) {
        const int b = (t <= c[0]) ? 8 : 1;
        const double c0 = (t <= c[0]) ? c[13] : c[6];
        h[i] = m.invmw[i] * (c0 + t * (c[b] + t * (c[b + 1] + t * (2. * c[b + 2] + t * (3. * c[b + 3] + t * 4. * c[b + 4])))));
      } else {
        // linear extrapolation with the boundary cp (same function as thermodynamics_kernels.cpp:300-311)
        const double tb = (t < mn) ? mn : mx;
        const int b = (t < mn) ? 8 : 1;
        const double c0 = (t < mn) ? c[13] : c[6];
        const double hb = c0 + tb * (c[b] + tb * (c[b + 1] + tb * (2. * c[b + 2] + tb * (3. * c[b + 3] + tb * 4. * c[b + 4]))));
        const double cpb = c[b] + tb * (2. * c[b + 1] + tb * (6. * c[b + 2] + tb * (12. * c[b + 3] + 20. * tb * c[b + 4])));
        h[i] = m.invmw[i] * (hb + cpb * (t - tb));
      }
    } else {
      const auto &c9 = m.c9[i];
      const int nreg = (int)c9[0];
      auto hfun = [&](const double *a, double tt) {
        const double it = 1. / tt, lt = std::log(tt);
        return m.invmw[i] * tt * (it * (a[7] + lt * a[1] - a[0] * it) + a[2] +
                                  tt * (0.5 * a[3] + tt * (0.3333333333333333 * a[4] + tt * (0.25 * a[5] + tt * 0.2 * a[6]))));
      };
      auto cpfun = [&](const double *a, double tt) {
        const double it = 1. / tt;
        return m.invmw[i] * (it * (a[1] + it * a[0]) + a[2] + tt * (a[3] + tt * (a[4] + tt * (a[5] + tt * a[6]))));
      };
      if (t < mn) {
        const double *a = &c9[3];
        h[i] = hfun(a, mn) + cpfun(a, mn) * (t - mn);
      } else if (t > mx) {
        const double *a = &c9[1 + (nreg - 1) * 11 + 2];
        h[i] = hfun(a, mx) + cpfun(a, mx) * (t - mx);
      } else {
        h[i] = 0.;
        for (int k = 0; k < nreg; ++k)
          if (t >= c9[1 + k * 11] && t < c9[1 + k * 11 + 1]) { h[i] = hfun(&c9[1 + k * 11 + 2], t); break; }
      }
    }
  }
}

void energies(const Mech &m, double t, double *e)
{
  enthalpies(m, t, e);
  const double RT = m.Ru * t;
  for (int i = 0; i < m.ns; ++i) e[i] -= RT * m.invmw[i];
}

// Gibbs energies g_i and d(g_i/RT)/dT-like term B_i (chemistry_kernels.cpp:56-97,
// rates_sensitivities_exact.cpp:83-124)
void gibbs(const Mech &m, double T, double *g, double *dB)
{
  const double invT = 1. / T, logT = std::log(T), invRu = 1. / m.Ru, Ru = m.Ru;
  for (int n = 0; n < m.ns; ++n) {
    const auto &c = m.c[n];
    if (m.thermo[n] == SF_THERMO_NASA7) {
      if (T <= c[0]) {
        g[n] = c[13] + T * (c[8] - c[14] - c[8] * logT - T * (c[9] + T * (c[10] + T * (c[11] + T * c[12]))));
        if (dB) dB[n] = invRu * ((c[8] - Ru) * invT + c[9] + T * (2 * c[10] + T * (3 * c[11] + T * 4 * c[12])) + c[13] * invT * invT);
      } else {
        g[n] = c[6] + T * (c[1] - c[7] - c[1] * logT - T * (c[2] + T * (c[3] + T * (c[4] + T * c[5]))));
        if (dB) dB[n] = invRu * ((c[1] - Ru) * invT + c[2] + T * (2 * c[3] + T * (3 * c[4] + T * 4 * c[5])) + c[6] * invT * invT);
      }
    } else if (m.thermo[n] == SF_THERMO_CONST) {
      g[n] = c[1] + c[3] * (T - c[0]) - T * (c[2] + c[3] * (logT - std::log(c[0])));
      if (dB) dB[n] = invT * (m.mw[n] * invRu * (c[3] - invT * (c[3] * c[0] - c[1])) - 1);
    } else {
      const auto &c9 = m.c9[n];
      const int nreg = (int)c9[0];
      for (int k = 0; k < nreg; ++k) {
        // production_rates selects the region with Tlo < T < Thi; the sensitivities use T < Thi or the last
        // region (chemistry_kernels.cpp:74-86 vs rates_sensitivities_exact.cpp:100-112); the latter is used here.
        if (T < c9[1 + k * 11 + 1] || k == nreg - 1) {
          const double *a = &c9[1 + k * 11 + 2];
          g[n] = a[7] - 0.5 * a[0] * invT + a[1] * (logT + 1.0) -
                 T * (a[2] * (logT - 1.0) + a[8] + T * (0.5 * a[3] + T * (0.1666666666666666 * a[4] + T * (0.0833333333333333 * a[5] + T * 0.05 * a[6]))));
          if (dB) dB[n] = invRu * (invT * (a[2] - Ru + invT * (a[7] + a[1] * logT - invT * a[0])) + 0.5 * a[3] +
                                   T * (a[4] * 0.3333333333333333 + T * (0.25 * a[5] + T * 0.2 * a[6])));
          break;
        }
      }
    }
  }
}

inline double arrh(const double *k, double logT, double invT) { return k[0] * std::exp(k[1] * logT - k[2] * invT); }
inline double arrh_sens_over_k(const double *k, double invT) { return invT * (k[1] + k[2] * invT); }

inline double kf_of(const Rxn &x, double T, double invT, double logT)
{
  switch (x.kform) {
  case 0: return x.kf[0];
  case 1: return x.kf[0] * T;
  case 2: return x.kf[0] * T * T;
  case 3: return x.kf[0] * invT;
  default: return arrh(x.kf, logT, invT);
  }
}

inline double third_body(const Rxn &x, const double *y, double rho, double ct)
{
  double m = x.base_eff * ct;
  double s = 0.;
  for (size_t i = 0; i < x.tb.size(); ++i) s += x.tb_eff[i] * y[x.tb[i]];
  return m + rho * s;
}

inline double log10_fcent(const Rxn &x, double T, double invT)
{
  const double *tr = x.troe;
  double f = 0.;
  if (x.troe_terms & 1) f += (1 - tr[0]) * std::exp(-T / tr[1]);
  if (x.troe_terms & 2) f += tr[0] * std::exp(-T / tr[2]);
  if (x.troe_terms & 4) f += std::exp(-invT * tr[3]);
  return std::log10(f);
}

// chemistry_kernels.cpp:35-463
void production_rates(const Mech &m, double T, double rho, double mmw, const double *y, double *w)
{
  const int ns = m.ns;
  const double invT = 1. / T, logT = std::log(T), conc = rho / mmw;
  const double invRu = 1. / m.Ru, port = m.pref * invT * invRu;
  std::vector<double> g(ns);
  gibbs(m, T, g.data(), nullptr);
  for (int i = 0; i < ns; ++i) w[i] = 0.;
  for (const Rxn &x : m.rx) {
    double k = kf_of(x, T, invT, logT);
    if (x.kind == SF_RXN_THIRD_BODY) {
      k *= third_body(x, y, rho, conc);
    } else if (x.kind == SF_RXN_LINDEMANN) {
      k /= (1 + k / (arrh(x.kp, logT, invT) * third_body(x, y, rho, conc)));
    } else if (x.kind == SF_RXN_TROE) {
      const double pr = arrh(x.kp, logT, invT) / k * third_body(x, y, rho, conc);
      const double lfc = log10_fcent(x, T, invT);
      const double lpc = std::log10(std::max(pr, 1.e-300)) + (-0.4 - 0.67 * lfc);
      const double f1 = lpc / ((0.75 - 1.27 * lfc) - 0.14 * lpc);
      k = k * std::pow(10, lfc / (1 + f1 * f1)) * pr / (1 + pr);
    }
    double kr = 0.;
    if (x.has_orders) {
      for (size_t i = 0; i < x.sp.size(); ++i)
        if (x.sp_nonzero[i]) k *= std::pow(std::max(y[x.sp[i]] * rho * m.invmw[x.sp[i]], 0.), x.sp_order[i]);
    } else {
      if (x.reversible) {
        double sg = 0.;
        for (size_t i = 0; i < x.net.size(); ++i) sg += x.net_nu[i] * g[x.net[i]];
        kr = k * std::exp(x.sum_nu * std::log(port) - invT * invRu * sg);
      }
      for (size_t i = 0; i < x.reac.size(); ++i) {
        const double C = y[x.reac[i]] * rho * m.invmw[x.reac[i]];
        for (int p = 0; p < x.reac_nu[i]; ++p) k *= C;
      }
      if (x.reversible)
        for (size_t i = 0; i < x.prod.size(); ++i) {
          const double C = y[x.prod[i]] * rho * m.invmw[x.prod[i]];
          for (int p = 0; p < x.prod_nu[i]; ++p) kr *= C;
        }
    }
    for (size_t i = 0; i < x.net.size(); ++i) w[x.net[i]] -= x.net_nu[i] * x.net_mw[i] * (k - kr);
  }
}

// Net rate of progress q_r of every reaction (as production_rates computes it) and s_r = dq_r / d ln k_r, k_r the
// forward (high-pressure for falloff) rate constant: k_r enters q_r linearly except through Pr = k0 [M] / k_inf of
// the falloff factor, so s_r = q_r for simple and three-body reactions, q_r Pr/(1+Pr) for Lindemann and
// q_r (Pr/(1+Pr) - d ln F / d ln Pr) for Troe (log10 F = log10 Fc / (1 + f1^2)). Project-written: the reference has
// no parameter sensitivities.
void rate_param_sens(const Mech &m, double T, double rho, double mmw, const double *y, double *q, double *sr)
{
  const int ns = m.ns;
  const double invT = 1. / T, logT = std::log(T), conc = rho / mmw;
  const double invRu = 1. / m.Ru, port = m.pref * invT * invRu;
  std::vector<double> g(ns);
  gibbs(m, T, g.data(), nullptr);
  int r = 0;
  for (const Rxn &x : m.rx) {
    double k = kf_of(x, T, invT, logT);
    double fac = 1.;
    if (x.kind == SF_RXN_THIRD_BODY) {
      k *= third_body(x, y, rho, conc);
    } else if (x.kind == SF_RXN_LINDEMANN) {
      const double pr = arrh(x.kp, logT, invT) / k * third_body(x, y, rho, conc);
      k /= (1 + k / (arrh(x.kp, logT, invT) * third_body(x, y, rho, conc)));
      fac = pr / (1 + pr);
    } else if (x.kind == SF_RXN_TROE) {
      const double pr = arrh(x.kp, logT, invT) / k * third_body(x, y, rho, conc);
      const double lfc = log10_fcent(x, T, invT);
      const double lpc = std::log10(std::max(pr, 1.e-300)) + (-0.4 - 0.67 * lfc);
      const double nn = 0.75 - 1.27 * lfc;
      const double den = nn - 0.14 * lpc;
      const double f1 = lpc / den;
      k = k * std::pow(10, lfc / (1 + f1 * f1)) * pr / (1 + pr);
      fac = pr / (1 + pr);
      if (pr > 1.e-300) fac -= lfc * (-2. * f1 / ((1 + f1 * f1) * (1 + f1 * f1))) * nn / (den * den);
    }
    double kr = 0.;
    if (x.has_orders) {
      for (size_t i = 0; i < x.sp.size(); ++i)
        if (x.sp_nonzero[i]) k *= std::pow(std::max(y[x.sp[i]] * rho * m.invmw[x.sp[i]], 0.), x.sp_order[i]);
    } else {
      if (x.reversible) {
        double sg = 0.;
        for (size_t i = 0; i < x.net.size(); ++i) sg += x.net_nu[i] * g[x.net[i]];
        kr = k * std::exp(x.sum_nu * std::log(port) - invT * invRu * sg);
      }
      for (size_t i = 0; i < x.reac.size(); ++i) {
        const double C = y[x.reac[i]] * rho * m.invmw[x.reac[i]];
        for (int p = 0; p < x.reac_nu[i]; ++p) k *= C;
      }
      if (x.reversible)
        for (size_t i = 0; i < x.prod.size(); ++i) {
          const double C = y[x.prod[i]] * rho * m.invmw[x.prod[i]];
          for (int p = 0; p < x.prod_nu[i]; ++p) kr *= C;
        }
    }
    q[r] = k - kr;
    sr[r] = (k - kr) * fac;
    ++r;
  }
}

// d(prod_j C_j^nu_j)/dY_s for the species at list position `at` (its stoich counted once), times rho/M_s
inline double dprod(const Mech &m, const std::vector<int> &idx, const std::vector<int> &nu, const double *y,
                    double rho, int at)
{
  double v = rho * m.invmw[idx[at]] * nu[at];
  for (size_t i = 0; i < idx.size(); ++i) {
    const double C = y[idx[i]] * rho * m.invmw[idx[i]];
    const int p = (int)i == at ? nu[i] - 1 : nu[i];
    for (int q = 0; q < p; ++q) v *= C;
  }
  return v;
}

// rates_sensitivities_exact.cpp:33-1028 (option 0), _sparse (option 2, same values), _no_tbaf (option 1)
void rates_sens(const Mech &m, double T, double rho, double mmw, const double *y, int option, double *w,
                double *S)
{
  const int ns = m.ns, nsp1 = ns + 1;
  const double invT = 1. / T, logT = std::log(T), invM = 1. / mmw, ct = rho * invM;
  const double invRu = 1. / m.Ru;
  std::vector<double> g(ns), dB(ns), dRdY(ns), dCdY(ns), dqdY(ns);
  gibbs(m, T, g.data(), dB.data());
  for (int i = 0; i < ns; ++i) w[i] = 0.;
  for (int i = 0; i < nsp1 * nsp1; ++i) S[i] = 0.;
  double Kc_prev = 0., dKc_prev = 0.;  // the reference keeps Kc from the previous reaction when n_net > 6
  for (const Rxn &x : m.rx) {
    std::fill(dRdY.begin(), dRdY.end(), 0.);
    std::fill(dCdY.begin(), dCdY.end(), 0.);
    const double kf = kf_of(x, T, invT, logT);
    double Rnet = 0., dRdrho = 0., dRdT = 0.;
    // option 1 (rates_sensitivities_no_tbaf_sens.cpp:153-175) treats every reaction with its mass-action orders,
    // ignoring special orders
    if (x.has_orders && option != 1) {
      double sumo = 0.;
      Rnet = kf;
      for (size_t i = 0; i < x.sp.size(); ++i)
        if (x.sp_nonzero[i]) {
          Rnet *= std::pow(std::max(y[x.sp[i]] * rho * m.invmw[x.sp[i]], 0.), x.sp_order[i]);
          sumo += x.sp_order[i];
        }
      dRdrho = Rnet / ct * invM * sumo;
      dRdT = Rnet * arrh_sens_over_k(x.kf, invT);
      int last_at = -1;
      for (size_t j = 0; j < x.sp.size(); ++j) {
        const int s = x.sp[j];
        if (s == ns - 1) { last_at = (int)j; continue; }
        if (!x.sp_nonzero[j]) continue;
        double mr = kf;
        for (size_t l = 0; l < x.sp.size(); ++l) {
          const double C = y[x.sp[l]] * rho * m.invmw[x.sp[l]];
          if (l != j) {
            if (x.sp_nonzero[l]) mr *= std::pow(std::max(C, 0.), x.sp_order[l]);
          } else if (x.sp_order[l] > 1) {
            mr *= x.sp_order[l] * rho * m.invmw[x.sp[l]] * std::pow(std::max(C, 1.e-16), x.sp_order[l] - 1.);
          } else {
            mr *= x.sp_order[l] * rho * m.invmw[x.sp[l]] / std::pow(std::max(C, 1.e-16), 1. - x.sp_order[l]);
          }
        }
        dRdY[s] = mr;
      }
      if (last_at >= 0 && x.sp_nonzero[last_at]) {
        double t = kf;
        for (size_t i = 0; i < x.sp.size(); ++i) {
          const double C = y[x.sp[i]] * rho * m.invmw[x.sp[i]];
          if ((int)i != last_at) {
            if (x.sp_nonzero[i]) t *= std::pow(C, x.sp_order[i]);
          } else {
            t *= x.sp_order[i] * rho * m.invmw[x.sp[i]] * std::pow(std::max(C, 1.e-16), x.sp_order[i] - 1.);
          }
        }
        for (int s = 0; s < ns - 1; ++s) dRdY[s] -= t;
      }
    } else {
      double Rf = kf;
      for (size_t i = 0; i < x.reac.size(); ++i) {
        const double C = y[x.reac[i]] * rho * m.invmw[x.reac[i]];
        for (int p = 0; p < x.reac_nu[i]; ++p) Rf *= C;
      }
      Rnet = Rf;
      dRdrho = Rf / ct * invM * x.sum_reac_nu;
      dRdT = Rf * arrh_sens_over_k(x.kf, invT);
      // reactant entries are assigned first, then the closure species (index ns-1) is subtracted from every
      // column (rates_sensitivities_exact.cpp:289-432)
      for (size_t i = 0; i < x.reac.size(); ++i)
        if (x.reac[i] != ns - 1) dRdY[x.reac[i]] = kf * dprod(m, x.reac, x.reac_nu, y, rho, (int)i);
      for (size_t i = 0; i < x.reac.size(); ++i)
        if (x.reac[i] == ns - 1) {
          const double v = kf * dprod(m, x.reac, x.reac_nu, y, rho, (int)i);
          for (int s = 0; s < ns - 1; ++s) dRdY[s] -= v;
        }
      if (x.reversible) {
        double Kc = Kc_prev, dKc = dKc_prev;
        const int nn = (int)x.net.size();
        if (nn >= 2 && nn <= 6) {  // rates_sensitivities_exact.cpp:531-558
          double sg = 0., sb = 0.;
          for (int i = 0; i < nn; ++i) { sg += x.net_nu[i] * g[x.net[i]]; sb += x.net_nu[i] * dB[x.net[i]]; }
          Kc = std::exp(-(x.sum_nu * std::log(m.pref * invT * invRu) - invT * invRu * sg));
          dKc = -sb;
        }
        Kc_prev = Kc;
        dKc_prev = dKc;
        const double kr = kf / Kc;
        double Rr = kr;
        for (size_t i = 0; i < x.prod.size(); ++i) {
          const double C = y[x.prod[i]] * rho * m.invmw[x.prod[i]];
          for (int p = 0; p < x.prod_nu[i]; ++p) Rr *= C;
        }
        Rnet -= Rr;
        dRdrho -= Rr / ct * invM * x.sum_prod_nu;
        dRdT -= Rr * (arrh_sens_over_k(x.kf, invT) - dKc);
        for (size_t i = 0; i < x.prod.size(); ++i) {
          const double v = kr * dprod(m, x.prod, x.prod_nu, y, rho, (int)i);
          if (x.prod[i] != ns - 1) dRdY[x.prod[i]] -= v;
          else for (int s = 0; s < ns - 1; ++s) dRdY[s] += v;
        }
      }
    }

    double Ctbaf = 1., dCdrho = 0., dCdT = 0.;
    if (x.kind == SF_RXN_THIRD_BODY) {
      Ctbaf = third_body(x, y, rho, ct);
      dCdrho = x.base_eff * invM;
      for (size_t i = 0; i < x.tb.size(); ++i) dCdrho += x.tb_eff[i] * y[x.tb[i]];
      for (int s = 0; s < ns - 1; ++s) dCdY[s] = rho * x.base_eff * (m.invmw[s] - m.invmw[ns - 1]);
      for (size_t i = 0; i < x.tb.size(); ++i) dCdY[x.tb[i]] += rho * x.tb_eff[i];
      for (size_t i = 0; i < x.tb.size(); ++i)
        if (x.tb[i] == ns - 1) { for (int s = 0; s < ns - 1; ++s) dCdY[s] -= rho * x.tb_eff[i]; break; }
    } else if (x.kind == SF_RXN_LINDEMANN || x.kind == SF_RXN_TROE) {
      const double M = third_body(x, y, rho, ct);
      const double kpf = arrh(x.kp, logT, invT) / kf;
      const double pr = kpf * M;
      const double dlogk = arrh_sens_over_k(x.kp, invT) - arrh_sens_over_k(x.kf, invT);
      double fac;  // d Ctbaf / d M
      if (x.kind == SF_RXN_LINDEMANN) {
        Ctbaf = pr / (1. + pr);
        dCdT = Ctbaf / (1. + pr) * dlogk;
        fac = kpf / ((1. + pr) * (1. + pr));
      } else {
        const double *tr = x.troe;
        const double e1 = std::exp(-T / tr[1]), e2 = std::exp(-T / tr[2]), e3 = std::exp(-invT * tr[3]);
        double fc = 0., dfc = 0.;
        if (x.troe_terms & 1) { fc += (1 - tr[0]) * e1; dfc += (tr[0] - 1) / tr[1] * e1; }
        if (x.troe_terms & 2) { fc += tr[0] * e2; dfc += -tr[0] / tr[2] * e2; }
        if (x.troe_terms & 4) { fc += e3; dfc += e3 * tr[3] * invT * invT; }
        const double l10pr = std::log10(std::max(pr, 1.e-300));
        const double l10fc = std::log10(std::max(fc, 1.e-300));
        const double lfc = std::log(std::max(fc, 1.e-300));
        const double ln10 = std::log(10.);
        const double a = l10pr - 0.67 * l10fc - 0.4;
        const double b = -0.14 * l10pr - 1.1762 * l10fc + 0.806;
        const double gt = 1 / (1 + (a / b) * (a / b));
        const double F = std::pow(fc, gt);
        Ctbaf = F * pr / (1 + pr);
        const double dFdT = F * (gt / fc * dfc + lfc * (-2.0 * gt * gt / ln10 * a / (b * b * b) *
                                                       ((b + 0.14 * a) * dlogk - (0.67 * b - 1.1762 * a) * dfc / fc)));
        dCdT = 1. / (1. + 1. / pr) * dFdT + F * pr / ((1. + pr) * (1. + pr)) * dlogk;
        fac = kpf * (-2.0 / (1. + pr) * F * lfc * gt * gt / ln10 * a / (b * b * b) * (b + 0.14 * a) +
                     F / ((1. + pr) * (1 + pr)));
      }
      dCdrho = fac * x.base_eff * invM;
      for (size_t i = 0; i < x.tb.size(); ++i) dCdrho += fac * x.tb_eff[i] * y[x.tb[i]];
      const double fr = fac * rho;
      for (int s = 0; s < ns - 1; ++s) dCdY[s] = fr * x.base_eff * (m.invmw[s] - m.invmw[ns - 1]);
      for (size_t i = 0; i < x.tb.size(); ++i) dCdY[x.tb[i]] += fr * x.tb_eff[i];
      for (size_t i = 0; i < x.tb.size(); ++i)
        if (x.tb[i] == ns - 1) { for (int s = 0; s < ns - 1; ++s) dCdY[s] -= fr * x.tb_eff[i]; break; }
    }
    const bool tbaf = option != 1;
    const double q = Rnet * Ctbaf;
    const double dqdrho = dRdrho * Ctbaf + (tbaf ? dCdrho * Rnet : 0.);
    const double dqdT = dRdT * Ctbaf + (tbaf ? dCdT * Rnet : 0.);
    // dq/dY once per reaction (rates_sensitivities_exact.cpp:1001-1010), then scattered to each net species
    for (int s = 0; s < ns - 1; ++s) dqdY[s] = dRdY[s] * Ctbaf + (tbaf ? dCdY[s] * Rnet : 0.);
    for (size_t i = 0; i < x.net.size(); ++i) {
      const int idx = x.net[i];
      const double f = -x.net_nu[i] * x.net_mw[i];
      w[idx] += f * q;
      S[idx] += f * dqdrho;
      S[idx + nsp1] += f * dqdT;
      double *Sc = S + idx + 2 * nsp1;
      for (int s = 0; s < ns - 1; ++s) Sc[nsp1 * s] += f * dqdY[s];
    }
  }
}

// ---------------------------------------------------------------------------------------------- reactors
inline double inner(int n, const double *a, const double *b)
{
  double d = 0.;
  for (int i = 0; i < n; ++i) d += b[i] * a[i];
  return d;
}

void extract_y(const Mech &m, const double *ynm1, double *y)
{
  y[m.ns - 1] = 1.;
  for (int j = 0; j < m.ns - 1; ++j) { y[j] = ynm1[j]; y[m.ns - 1] -= y[j]; }
}

// isochoric_reactor_kernels.cpp:184-242
void rhs_isochoric(const Mech &m, const sf_reactor_params &P, const double *q, double *rhs)
{
  const int ns = m.ns;
  std::vector<double> y(ns), cvi(ns), e(ns), w(ns);
  const double rho = q[0], T = q[1];
  extract_y(m, q + 2, y.data());
  const double mmw = mmw_of(m, y.data());
  const double p = rho * T * m.Ru / mmw;
  double cv;
  cp_mix_species(m, T, y.data(), &cv, cvi.data());
  cv -= m.Ru / mmw;
  for (int i = 0; i < ns; ++i) cvi[i] -= m.Ru * m.invmw[i];
  energies(m, T, e.data());
  production_rates(m, T, rho, mmw, y.data(), w.data());
  rhs[0] = 0.;
  rhs[1] = -inner(ns, w.data(), e.data()) / (rho * cv);
  for (int i = 0; i < ns - 1; ++i) rhs[2 + i] = w[i] / rho;
  if (P.open) {
    std::vector<double> ein(ns);
    energies(m, P.inflow_temperature, ein.data());
    const double *yin = P.inflow_Y;
    double r1 = (ein[ns - 1] - e[ns - 1]) * yin[ns - 1];
    std::vector<double> mr(ns + 1);
    for (int i = 0; i < ns - 1; ++i) { r1 += (ein[i] - e[i]) * yin[i]; mr[2 + i] = yin[i] - y[i]; }
    mr[0] = (P.inflow_density - rho) / P.tau;
    mr[1] = r1 / cv;
    for (int i = 1; i < ns + 1; ++i) mr[i] *= 1. / P.tau * P.inflow_density / rho;
    for (int i = 0; i < ns + 1; ++i) rhs[i] += mr[i];
    (void)p;
  }
  if (P.heat_transfer == 1) rhs[1] = 0.;
  else if (P.heat_transfer == 2) {
    const double Ts = P.surface_temperature;
    rhs[1] += P.surface_area_to_volume / (rho * cv) *
              (P.h_convection * (P.fluid_temperature - T) + P.eps_radiation * 5.67e-8 * (Ts * Ts * Ts * Ts - T * T * T * T));
  }
}

// isochoric_reactor_kernels.cpp:244-333 with chem_jac_isochoric (:61-104), mass_jac (:106-154), heat_jac (:156-182)
void jac_isochoric(const Mech &m, const sf_reactor_params &P, int opt, const double *q, double *rhs, double *J)
{
  const int ns = m.ns, n1 = ns + 1;
  std::vector<double> y(ns), cvi(ns), cvis(ns), e(ns), w(ns), S(n1 * n1);
  const double rho = q[0], T = q[1];
  extract_y(m, q + 2, y.data());
  const double mmw = mmw_of(m, y.data());
  double cv, cvT;
  cp_mix_species(m, T, y.data(), &cv, cvi.data());
  cv -= m.Ru / mmw;
  for (int i = 0; i < ns; ++i) cvi[i] -= m.Ru * m.invmw[i];
  cp_sens(m, T, y.data(), &cvT, cvis.data());
  energies(m, T, e.data());
  rates_sens(m, T, rho, mmw, y.data(), opt, w.data(), S.data());
  const double iR = 1. / rho, iCv = 1. / cv, iRCv = 1. / (rho * cv);
  rhs[0] = 0.;
  rhs[1] = -inner(ns, w.data(), e.data()) / (rho * cv);
  for (int i = 0; i < ns - 1; ++i) rhs[2 + i] = w[i] * iR;
  J[0] = 0.;
  J[1] = -iRCv * inner(ns, S.data(), e.data()) - iR * rhs[1];
  for (int i = 0; i < ns - 1; ++i) J[2 + i] = iR * (S[i] - iR * w[i]);
  J[n1] = 0.;
  J[n1 + 1] = -iCv * (iR * (inner(ns, &S[n1], e.data()) + inner(ns, w.data(), cvi.data())) + rhs[1] * cvT);
  for (int i = 0; i < ns - 1; ++i) J[n1 + 2 + i] = iR * S[n1 + i];
  const double cvn = cvi[ns - 1];
  for (int k = 0; k < ns - 1; ++k) {
    const int c0 = (2 + k) * n1;
    J[c0] = 0.;
    J[c0 + 1] = -iRCv * inner(ns, &S[c0], e.data()) - rhs[1] * (cvi[k] - cvn) * iCv;
    for (int i = 0; i < ns - 1; ++i) J[c0 + 2 + i] = iR * S[c0 + i];
  }
  if (P.open) {
    std::vector<double> ein(ns), mr(n1);
    energies(m, P.inflow_temperature, ein.data());
    const double *yin = P.inflow_Y;
    double r1 = (ein[ns - 1] - e[ns - 1]) * yin[ns - 1];
    for (int i = 0; i < ns - 1; ++i) { r1 += (ein[i] - e[i]) * yin[i]; mr[2 + i] = yin[i] - y[i]; }
    const double itau = 1. / P.tau;
    mr[0] = (P.inflow_density - rho) * itau;
    mr[1] = r1 / cv;
    for (int i = 1; i < n1; ++i) mr[i] *= itau * P.inflow_density * iR;
    for (int i = 0; i < n1; ++i) rhs[i] += mr[i];
    J[0] += -itau;
    for (int i = 0; i < ns; ++i) J[1 + i] += -iR * mr[1 + i];
    J[n1 + 1] += -iCv * (itau * iR * (P.inflow_density * inner(ns, yin, cvi.data())) + cvT * mr[1]);
    for (int k = 0; k < ns - 1; ++k) {
      const int c0 = (2 + k) * n1;
      J[c0 + 1] += -iCv * mr[1] * (cvi[k] - cvn);
      J[c0 + 2 + k] += -itau * P.inflow_density / rho;
    }
  }
  if (P.heat_transfer == 1) {
    for (int k = 0; k < n1; ++k) J[k * n1 + 1] = 0.;
    rhs[1] = 0.;
  } else if (P.heat_transfer == 2) {
    const double Ts = P.surface_temperature;
    const double hq = P.surface_area_to_volume * iRCv *
                      (P.h_convection * (P.fluid_temperature - T) + P.eps_radiation * 5.67e-8 * (Ts * Ts * Ts * Ts - T * T * T * T));
    rhs[1] += hq;
    J[1] += -hq / rho;
    J[n1 + 1] += -iCv * cvT * hq - P.surface_area_to_volume * iRCv * (P.h_convection + 4. * P.eps_radiation * 5.67e-8 * T * T * T);
    for (int k = 0; k < ns - 1; ++k) J[(2 + k) * n1 + 1] += iCv * hq * (cvn - cvi[k]);
  }
}

// isobaric_reactor_kernels.cpp:170-219
void rhs_isobaric(const Mech &m, const sf_reactor_params &P, double p, const double *q, double *rhs)
{
  const int ns = m.ns;
  std::vector<double> y(ns), cpi(ns), h(ns), w(ns);
  const double T = q[0];
  extract_y(m, q + 1, y.data());
  const double mmw = mmw_of(m, y.data());
  const double rho = p * mmw / (T * m.Ru);
  double cp;
  cp_mix_species(m, T, y.data(), &cp, cpi.data());
  enthalpies(m, T, h.data());
  production_rates(m, T, rho, mmw, y.data(), w.data());
  rhs[0] = -inner(ns, w.data(), h.data()) / (rho * cp);
  for (int i = 0; i < ns - 1; ++i) rhs[1 + i] = w[i] / rho;
  if (P.open) {
    std::vector<double> hin(ns);
    enthalpies(m, P.inflow_temperature, hin.data());
    const double *yin = P.inflow_Y;
    double r0 = (hin[ns - 1] - h[ns - 1]) * yin[ns - 1];
    std::vector<double> mr(ns);
    for (int i = 0; i < ns - 1; ++i) { r0 += (hin[i] - h[i]) * yin[i]; mr[1 + i] = yin[i] - y[i]; }
    mr[0] = r0 / cp;
    for (int i = 0; i < ns; ++i) rhs[i] += mr[i] / P.tau;
  }
  if (P.heat_transfer == 1) rhs[0] = 0.;
  else if (P.heat_transfer == 2) {
    const double Ts = P.surface_temperature;
    rhs[0] += P.surface_area_to_volume / (rho * cp) *
              (P.h_convection * (P.fluid_temperature - T) + P.eps_radiation * 5.67e-8 * (Ts * Ts * Ts * Ts - T * T * T * T));
  }
}

// chem_jac_isobaric (isobaric_reactor_kernels.cpp:57-100): primitive n x (n+1) Jacobian, columns rho, T, Y
void chem_primjac_isobaric(const Mech &m, double rho, double cp, const double *cpi, double cpT, const double *h,
                           const double *w, const double *S, double *rhs, double *PJ)
{
  const int ns = m.ns, n1 = ns + 1;
  rhs[0] = -inner(ns, w, h) / (rho * cp);
  for (int i = 0; i < ns - 1; ++i) rhs[1 + i] = w[i] / rho;
  const double iRCp = 1. / (rho * cp), iR = 1. / rho, iCp = 1. / cp;
  PJ[0] = -iRCp * inner(ns, S, h) - iR * rhs[0];
  for (int i = 0; i < ns - 1; ++i) PJ[1 + i] = iR * (S[i] - iR * w[i]);
  PJ[ns] = -iRCp * (inner(ns, &S[n1], h) + inner(ns, w, cpi)) - rhs[0] * cpT * iCp;
  for (int i = 0; i < ns - 1; ++i) PJ[ns + 1 + i] = S[n1 + i] * iR;
  const double cpn = cpi[ns - 1];
  for (int k = 0; k < ns - 1; ++k) {
    const int r0 = (2 + k) * ns;
    PJ[r0] = -iRCp * inner(ns, &S[(2 + k) * n1], h) - rhs[0] * (cpi[k] - cpn) * iCp;
    for (int i = 0; i < ns - 1; ++i) PJ[r0 + 1 + i] = iR * S[(2 + k) * n1 + i];
  }
}

// transform_isobaric_primitive_jacobian (isobaric_reactor_kernels.cpp:319-343)
void transform_isobaric(const Mech &m, double rho, double T, double mmw, const double *PJ, double *J)
{
  const int ns = m.ns;
  const double roT = rho / T;
  for (int i = 0; i < ns; ++i) J[i] = PJ[ns + i] - roT * PJ[i];
  const double nrm = -rho * mmw;
  for (int k = 0; k < ns - 1; ++k)
    for (int i = 0; i < ns; ++i)
      J[(1 + k) * ns + i] = PJ[(2 + k) * ns + i] + nrm * (m.invmw[k] - m.invmw[ns - 1]) * PJ[i];
}

// isobaric_reactor_kernels.cpp:221-317
void jac_isobaric(const Mech &m, const sf_reactor_params &P, int opt, double p, const double *q, double *rhs,
                  double *J)
{
  const int ns = m.ns, n1 = ns + 1;
  std::vector<double> y(ns), cpi(ns), cpis(ns), h(ns), w(ns), S(n1 * n1), PJ(ns * n1);
  const double T = q[0];
  extract_y(m, q + 1, y.data());
  const double mmw = mmw_of(m, y.data());
  const double rho = p * mmw / (T * m.Ru);
  double cp, cpT;
  cp_mix_species(m, T, y.data(), &cp, cpi.data());
  enthalpies(m, T, h.data());
  cp_sens(m, T, y.data(), &cpT, cpis.data());
  rates_sens(m, T, rho, mmw, y.data(), opt, w.data(), S.data());
  chem_primjac_isobaric(m, rho, cp, cpi.data(), cpT, h.data(), w.data(), S.data(), rhs, PJ.data());
  if (P.open) {
    std::vector<double> hin(ns), mr(ns);
    enthalpies(m, P.inflow_temperature, hin.data());
    const double *yin = P.inflow_Y;
    const double itau = 1. / P.tau, iCp = 1. / cp;
    double r0 = (hin[ns - 1] - h[ns - 1]) * yin[ns - 1];
    for (int i = 0; i < ns - 1; ++i) { r0 += (hin[i] - h[i]) * yin[i]; mr[1 + i] = yin[i] - y[i]; }
    mr[0] = r0 / cp;
    for (int i = 0; i < ns; ++i) mr[i] *= itau;
    PJ[ns] += -iCp * (cpT * mr[0] + itau * inner(ns, yin, cpi.data()));
    for (int k = 0; k < ns - 1; ++k) {
      PJ[(2 + k) * ns] += -mr[0] * (cpi[k] - cpi[ns - 1]) * iCp;
      PJ[(2 + k) * ns + 1 + k] += -itau;
    }
    for (int i = 0; i < ns; ++i) rhs[i] += mr[i];
  }
  if (P.heat_transfer == 1) {
    for (int k = 0; k < n1; ++k) PJ[k * ns] = 0.;
    rhs[0] = 0.;
  } else if (P.heat_transfer == 2) {
    const double Ts = P.surface_temperature, iRCp = 1. / (rho * cp), iCp = 1. / cp;
    const double hq = P.surface_area_to_volume * iRCp *
                      (P.h_convection * (P.fluid_temperature - T) + P.eps_radiation * 5.67e-8 * (Ts * Ts * Ts * Ts - T * T * T * T));
    PJ[0] += -hq / rho;
    PJ[ns] += -iCp * cpT * hq - P.surface_area_to_volume * iRCp * (P.h_convection + 4. * P.eps_radiation * 5.67e-8 * T * T * T);
    for (int k = 0; k < ns - 1; ++k) PJ[(2 + k) * ns] += iCp * hq * (cpi[ns - 1] - cpi[k]);
    rhs[0] += hq;
  }
  transform_isobaric(m, rho, T, mmw, PJ.data(), J);
}

// ---------------------------------------------------------------------------------------------- dense LU
// Partial-pivoting LU of a column-major n x n matrix (the factorization LAPACK dgetrf computes), 0-based pivots.
int lu_factor(int n, double *A, int *piv)
{
  int info = 0;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double mx = std::abs(A[k + k * n]);
    for (int i = k + 1; i < n; ++i)
      if (std::abs(A[i + k * n]) > mx) { mx = std::abs(A[i + k * n]); p = i; }
    piv[k] = p;
    if (A[p + k * n] == 0.) { if (!info) info = k + 1; continue; }
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(A[k + j * n], A[p + j * n]);
    const double inv = 1. / A[k + k * n];
    for (int i = k + 1; i < n; ++i) A[i + k * n] *= inv;
    for (int j = k + 1; j < n; ++j) {
      const double a = A[k + j * n];
      if (a != 0.)
        for (int i = k + 1; i < n; ++i) A[i + j * n] -= A[i + k * n] * a;
    }
  }
  return info;
}

void lu_solve(int n, const double *LU, const int *piv, double *b)
{
  for (int k = 0; k < n; ++k) std::swap(b[k], b[piv[k]]);
  for (int j = 0; j < n; ++j)
    for (int i = j + 1; i < n; ++i) b[i] -= LU[i + j * n] * b[j];
  for (int j = n - 1; j >= 0; --j) {
    b[j] /= LU[j + j * n];
    for (int i = 0; i < j; ++i) b[i] -= LU[i + j * n] * b[j];
  }
}

// ---------------------------------------------------------------------------------------------- flamelets
void flamelet_rhs(const Mech &m, const double *state, double p, const double *oxy, const double *fuel, bool adiabatic,
                  const double *Tc, const double *hc, const double *Tr, const double *hr, int nzi, const double *cmajor,
                  const double *csub, const double *csup, const double *mc, const double *nc, const double *chi,
                  bool eflux, bool vcp, bool scaled, double *out)
{
  const int ns = m.ns;
  double maxT = -1, maxT4 = -1;
  if (scaled) {
    for (int i = 0; i < nzi; ++i) maxT = std::max(maxT, state[i * ns]);
    maxT4 = maxT * maxT * maxT * maxT;
  }
  std::vector<double> y(ns), cpz(nzi), cpg(nzi), h(ns), w(ns), cpi(ns);
  auto cp_at = [&](const double *st) {
    std::vector<double> yy(ns), ci(ns);
    extract_y(m, st + 1, yy.data());
    double c;
    cp_mix_species(m, st[0], yy.data(), &c, ci.data());
    return c;
  };
  if (vcp) {
    for (int i = 0; i < nzi; ++i) cpg[i] = cp_at(&state[i * ns]);
    for (int i = 0; i < nzi; ++i) {
      if (i == 0) cpz[i] = mc[i] * cp_at(oxy) + nc[i] * cpg[1];
      else if (i == nzi - 1) cpz[i] = mc[i] * cpg[nzi - 2] + nc[i] * cp_at(fuel);
      else cpz[i] = mc[i] * cpg[i - 1] + nc[i] * cpg[i + 1];
    }
  }
  for (int i = 0; i < nzi; ++i) {
    const double T = state[i * ns];
    extract_y(m, &state[i * ns + 1], y.data());
    const double mmw = mmw_of(m, y.data());
    const double rho = p * mmw / (T * m.Ru);
    double cp;
    cp_mix_species(m, T, y.data(), &cp, cpi.data());
    enthalpies(m, T, h.data());
    production_rates(m, T, rho, mmw, y.data(), w.data());
    out[i * ns] = -inner(ns, w.data(), h.data()) / (rho * cp);
    for (int k = 0; k < ns - 1; ++k) out[i * ns + 1 + k] = w[k] / rho;
    if (!adiabatic) {
      double q;
      if (scaled) {
        const double Tr4 = Tr[i] * Tr[i] * Tr[i] * Tr[i];
        q = hc[i] * (Tc[i] - T) / (maxT - Tc[i]) + hr[i] * 5.67e-8 * (Tr4 - T * T * T * T) / (maxT4 - Tr4);
      } else {
        q = hc[i] * (Tc[i] - T) + hr[i] * 5.67e-8 * (Tr[i] * Tr[i] * Tr[i] * Tr[i] - T * T * T * T);
      }
      out[i * ns] += q / (rho * cp);
    }
    const double *sm = (i == 0) ? oxy : &state[(i - 1) * ns];
    const double *sp = (i == nzi - 1) ? fuel : &state[(i + 1) * ns];
    const double dTdZ = mc[i] * sm[0] + nc[i] * sp[0];
    if (eflux) {
      const double cpn = cpi[ns - 1];
      double s = 0.;
      for (int j = 0; j < ns - 1; ++j) s += (cpi[j] - cpn) * (mc[i] * sm[1 + j] + nc[i] * sp[1 + j]);
      out[i * ns] += 0.5 * chi[i] / cp * dTdZ * s;
    }
    if (vcp) out[i * ns] += 0.5 * chi[i] * cpz[i] / cp * dTdZ;
  }
  const int end = (nzi - 1) * ns;
  for (int i = ns; i < end; ++i) out[i] += cmajor[i] * state[i] + csub[i] * state[i - ns] + csup[i] * state[i + ns];
  for (int j = 0; j < ns; ++j) {
    out[j] += cmajor[j] * state[j] + csub[j] * oxy[j] + csup[j] * state[j + ns];
    out[end + j] += cmajor[end + j] * state[end + j] + csub[end + j] * state[end + j - ns] + csup[end + j] * fuel[j];
  }
}

// flamelet_kernels.cpp:1220-1409 without the eigenvalue option. out_jac is fully written (off-diagonals set,
// not accumulated, i.e. the reference called on a zeroed buffer).
void flamelet_jacobian(const Mech &m, const double *state, double p, const double *oxy, const double *fuel,
                       bool adiabatic, const double *Tc, const double *hc, const double *Tr, const double *hr, int nzi,
                       const double *cmajor, const double *csub, const double *csup, const double *mc,
                       const double *nc, const double *chi, bool scale_offset, double pref, int opt, bool eflux,
                       bool scaled, double *J)
{
  const int ns = m.ns, n1 = ns + 1, bs = ns * ns;
  double maxT = -1, maxT4 = -1;
  if (scaled) {
    for (int i = 0; i < nzi; ++i) maxT = std::max(maxT, state[i * ns]);
    maxT4 = maxT * maxT * maxT * maxT;
  }
  std::vector<double> cp(nzi), cpT(nzi), y(ns), cpi(ns), cpis(ns), h(ns), w(ns), S(n1 * n1), PJ(ns * n1), rt(ns);
  for (int iz = 0; iz < nzi; ++iz) {
    const double T = state[iz * ns];
    extract_y(m, &state[iz * ns + 1], y.data());
    const double mmw = mmw_of(m, y.data());
    const double rho = p * mmw / (T * m.Ru);
    cp_mix_species(m, T, y.data(), &cp[iz], cpi.data());
    enthalpies(m, T, h.data());
    cp_sens(m, T, y.data(), &cpT[iz], cpis.data());
    rates_sens(m, T, rho, mmw, y.data(), opt, w.data(), S.data());
    chem_primjac_isobaric(m, rho, cp[iz], cpi.data(), cpT[iz], h.data(), w.data(), S.data(), rt.data(), PJ.data());
    if (!adiabatic) {
      const double iRCp = 1. / (rho * cp[iz]), iCp = 1. / cp[iz];
      double q;
      if (scaled) {
        const double Tr4 = Tr[iz] * Tr[iz] * Tr[iz] * Tr[iz];
        q = (hc[iz] * (Tc[iz] - T) / (maxT - Tc[iz]) + hr[iz] * 5.67e-8 * (Tr4 - T * T * T * T) / (maxT4 - Tr4)) * iRCp;
        PJ[ns] -= iCp * cpT[iz] * q + iRCp * (hc[iz] / (maxT - Tc[iz]) + 4. * hr[iz] / (maxT4 - Tr4) * 5.67e-8 * T * T * T);
      } else {
        q = (hc[iz] * (Tc[iz] - T) + hr[iz] * 5.67e-8 * (Tr[iz] * Tr[iz] * Tr[iz] * Tr[iz] - T * T * T * T)) * iRCp;
        PJ[ns] -= iCp * cpT[iz] * q + iRCp * (hc[iz] + 4. * hr[iz] * 5.67e-8 * T * T * T);
      }
      PJ[0] -= q / rho;
      // the reference loops k < nSpec+1 here (flamelet_kernels.cpp:1316-1319), reading past cpi; the
      // restatement stops at the last Y column
      for (int k = 0; k < ns - 1; ++k) PJ[(2 + k) * ns] += iCp * q * (cpi[ns - 1] - cpi[k]);
    }
    transform_isobaric(m, rho, T, mmw, PJ.data(), &J[iz * bs]);
    for (int iq = 0; iq < ns; ++iq) J[iz * bs + iq * (ns + 1)] += cmajor[iz * ns + iq];
  }
  if (eflux) {
    auto cp_at = [&](const double *st) {
      std::vector<double> yy(ns), ci(ns);
      extract_y(m, st + 1, yy.data());
      double c;
      cp_mix_species(m, st[0], yy.data(), &c, ci.data());
      return c;
    };
    for (int i = 0; i < nzi; ++i) {
      double dTdZ, dcpdZ;
      if (i == 0) {
        dTdZ = mc[i] * oxy[0] + nc[i] * state[(i + 1) * ns];
        dcpdZ = mc[i] * cp_at(oxy) + nc[i] * cp[i + 1];
      } else if (i == nzi - 1) {
        dTdZ = mc[i] * state[(i - 1) * ns] + nc[i] * fuel[0];
        dcpdZ = mc[i] * cp[i - 1] + nc[i] * cp_at(fuel);
      } else {
        dTdZ = mc[i] * state[(i - 1) * ns] + nc[i] * state[(i + 1) * ns];
        dcpdZ = mc[i] * cp[i - 1] + nc[i] * cp[i + 1];
      }
      const double f1 = 0.5 * chi[i] / cp[i] * dTdZ * dcpdZ;
      J[i * bs] -= f1 / cp[i] * cpT[i];
    }
  }
  const int off = (nzi - 1) * ns;
  int idx = nzi * bs;
  for (int iz = 1; iz < nzi; ++iz)
    for (int iq = 0; iq < ns; ++iq) {
      J[idx] = csub[iz * ns + iq];
      J[off + idx] = csup[(iz - 1) * ns + iq];
      ++idx;
    }
  if (scale_offset) {
    const int ne = ns * (nzi * ns + 2 * (nzi - 1));
    for (int i = 0; i < ne; ++i) J[i] *= pref;
    for (int iz = 0; iz < nzi; ++iz)
      for (int iq = 0; iq < ns; ++iq) J[iz * bs + iq * (ns + 1)] -= 1.;
  }
}

// btddod_matrix_kernels.cpp:19-80
void btddod_factor(double *d, int nb, int bs, double *l, int *piv)
{
  const int ne = bs * bs, noff = (nb - 1) * bs, nbd = nb * ne;
  const double *sub = &d[nbd];
  const double *sup = &d[nbd + noff];
  lu_factor(bs, d, piv);
  for (int i = 1; i < nb; ++i) {
    const int o1 = i * ne, om = o1 - ne;
    for (int l2 = 0; l2 < ne; ++l2) l[o1 + l2] = 0.;
    for (int j = 0; j < bs; ++j) l[o1 + j * (bs + 1)] = 1.;
    for (int j = 0; j < bs; ++j) lu_solve(bs, &d[om], &piv[(i - 1) * bs], &l[o1 + j * bs]);
    const int b = (i - 1) * bs;
    for (int j = 0; j < bs; ++j)
      for (int k = 0; k < bs; ++k) l[o1 + j * bs + k] *= sub[b + k];
    for (int j = 0; j < bs; ++j) {
      const double fac = -sup[b + j];
      for (int k = 0; k < bs; ++k) d[o1 + j * bs + k] += fac * l[o1 + j * bs + k];
    }
    lu_factor(bs, &d[o1], &piv[i * bs]);
  }
}

// btddod_matrix_kernels.cpp:82-119
void btddod_solve(const double *d, const double *l, const int *piv, const double *rhs, int nb, int bs, double *x)
{
  const int ne = bs * bs, noff = (nb - 1) * bs, nbd = nb * ne;
  const double *sup = &d[nbd + noff];
  std::vector<double> y(nb * bs), t(bs);
  for (int i = 0; i < bs; ++i) y[i] = rhs[i];
  for (int i = 1; i < nb; ++i) {
    for (int k = 0; k < bs; ++k) y[i * bs + k] = rhs[i * bs + k];
    for (int c = 0; c < bs; ++c) {
      const double a = -y[(i - 1) * bs + c];
      for (int r = 0; r < bs; ++r) y[i * bs + r] += l[i * ne + c * bs + r] * a;
    }
  }
  const int last = nb - 1;
  for (int k = 0; k < bs; ++k) x[last * bs + k] = y[last * bs + k];
  lu_solve(bs, &d[last * ne], &piv[last * bs], &x[last * bs]);
  for (int i = nb - 2; i >= 0; --i) {
    for (int j = 0; j < bs; ++j) x[i * bs + j] = y[i * bs + j] - sup[i * bs + j] * x[(i + 1) * bs + j];
    lu_solve(bs, &d[i * ne], &piv[i * bs], &x[i * bs]);
  }
}

// btddod_matrix_kernels.cpp:121-160
void btddod_matvec(const double *a, const double *x, int nb, int bs, double *y)
{
  const int ne = bs * bs, noff = (nb - 1) * bs, nbd = nb * ne;
  for (int i = 0; i < nb * bs; ++i) y[i] = 0.;
  for (int i = 0; i < nb; ++i)
    for (int c = 0; c < bs; ++c)
      for (int r = 0; r < bs; ++r) y[i * bs + r] += a[i * ne + c * bs + r] * x[i * bs + c];
  const double *sub = &a[nbd];
  const double *sup = &a[nbd + noff];
  for (int i = 1; i < nb; ++i)
    for (int q = 0; q < bs; ++q) y[i * bs + q] += sub[(i - 1) * bs + q] * x[(i - 1) * bs + q];
  for (int i = 0; i < nb - 1; ++i)
    for (int q = 0; q < bs; ++q) y[i * bs + q] += sup[i * bs + q] * x[(i + 1) * bs + q];
}

template <class F>
int guarded(F f)
{
  try {
    f();
    return 0;
  } catch (std::exception &e) {
    g_err = e.what();
    return SF_ERR_MECHANISM;
  }
}

}  // namespace

// =============================================================================================== C interface
extern "C" {

const char *oracle_last_error(void) { return g_err.c_str(); }

int oracle_mech_create(const sf_mech_desc *d, void **out)
{
  return guarded([&] { *out = build(d); });
}

void oracle_mech_destroy(void *m) { delete static_cast<Mech *>(m); }

int oracle_set_threads(int n)
{
#ifdef _OPENMP
  omp_set_num_threads(n);
  return n;
#else
  (void)n;
  return 1;
#endif
}

int oracle_thermo(const void *mp, int what, int n, const double *T, const double *Y, double *out)
{
  const Mech &m = *static_cast<const Mech *>(mp);
  const int ns = m.ns;
#pragma omp parallel for schedule(static) if (n >= 64)
  for (int s = 0; s < n; ++s) {
    std::vector<double> a(ns), b(ns);
    const double *y = Y + (size_t)s * ns;
    const double t = T[s];
    double mix;
    switch (what) {
    case 0: cp_mix_species(m, t, y, &mix, a.data()); out[s] = mix; break;
    case 1: cp_mix_species(m, t, y, &mix, a.data()); out[s] = mix - m.Ru / mmw_of(m, y); break;
    case 2: enthalpies(m, t, a.data()); out[s] = inner(ns, a.data(), y); break;
    case 3: energies(m, t, a.data()); out[s] = inner(ns, a.data(), y); break;
    case 4: cp_mix_species(m, t, y, &mix, out + (size_t)s * ns); break;
    case 5:
      cp_mix_species(m, t, y, &mix, out + (size_t)s * ns);
      for (int i = 0; i < ns; ++i) out[(size_t)s * ns + i] -= m.Ru * m.invmw[i];
      break;
    case 6: enthalpies(m, t, out + (size_t)s * ns); break;
    case 7: energies(m, t, out + (size_t)s * ns); break;
    case 8: out[s] = mmw_of(m, y); break;
    case 9: cp_sens(m, t, y, &mix, a.data()); out[s] = mix; break;
    case 10: cp_sens(m, t, y, &mix, out + (size_t)s * ns); break;
    }
  }
  return 0;
}

int oracle_production_rates(const void *mp, int n, const double *T, const double *rho, const double *Y, double *w)
{
  const Mech &m = *static_cast<const Mech *>(mp);
#pragma omp parallel for schedule(static) if (n >= 64)
  for (int s = 0; s < n; ++s) {
    const double *y = Y + (size_t)s * m.ns;
    production_rates(m, T[s], rho[s], mmw_of(m, y), y, w + (size_t)s * m.ns);
  }
  return 0;
}

int oracle_rates_sens(const void *mp, int n, const double *rho, const double *T, const double *Y, int opt, double *w,
                      double *S)
{
  const Mech &m = *static_cast<const Mech *>(mp);
  const size_t n1 = m.ns + 1;
#pragma omp parallel for schedule(static) if (n >= 64)
  for (int s = 0; s < n; ++s) {
    const double *y = Y + (size_t)s * m.ns;
    rates_sens(m, T[s], rho[s], mmw_of(m, y), y, opt, w + (size_t)s * m.ns, S + (size_t)s * n1 * n1);
  }
  return 0;
}

int oracle_reactor_rhs(const void *mp, const sf_reactor_params *P, int n, const double *q, const double *pres,
                       double *rhs)
{
  const Mech &m = *static_cast<const Mech *>(mp);
  const int neq = P->configuration == 0 ? m.ns : m.ns + 1;
#pragma omp parallel for schedule(static) if (n >= 64)
  for (int s = 0; s < n; ++s) {
    if (P->configuration == 0)
      rhs_isobaric(m, *P, pres ? pres[s] : P->pressure, q + (size_t)s * neq, rhs + (size_t)s * neq);
    else
      rhs_isochoric(m, *P, q + (size_t)s * neq, rhs + (size_t)s * neq);
  }
  return 0;
}

int oracle_reactor_jac(const void *mp, const sf_reactor_params *P, int opt, int n, const double *q, const double *pres,
                       double *rhs, double *J)
{
  const Mech &m = *static_cast<const Mech *>(mp);
  const int neq = P->configuration == 0 ? m.ns : m.ns + 1;
#pragma omp parallel for schedule(static) if (n >= 64)
  for (int s = 0; s < n; ++s) {
    if (P->configuration == 0)
      jac_isobaric(m, *P, opt, pres ? pres[s] : P->pressure, q + (size_t)s * neq, rhs + (size_t)s * neq,
                   J + (size_t)s * neq * neq);
    else
      jac_isochoric(m, *P, opt, q + (size_t)s * neq, rhs + (size_t)s * neq, J + (size_t)s * neq * neq);
  }
  return 0;
}

int oracle_rate_param_sens(const void *mp, int n, const double *T, const double *rho, const double *Y, double *q,
                           double *sr)
{
  const Mech &m = *static_cast<const Mech *>(mp);
  const int nr = (int)m.rx.size();
#pragma omp parallel for schedule(static) if (n >= 64)
  for (int i = 0; i < n; ++i) {
    const double *y = Y + (size_t)i * m.ns;
    double sim = 0.;
    for (int s = 0; s < m.ns; ++s) sim += y[s] * m.invmw[s];
    rate_param_sens(m, T[i], rho[i], 1. / sim, y, q + (size_t)i * nr, sr + (size_t)i * nr);
  }
  return 0;
}

int oracle_lu_factor(int n, int m, double *A, int *piv, int *info)
{
#pragma omp parallel for schedule(static) if (n >= 64)
  for (int s = 0; s < n; ++s) {
    const int r = lu_factor(m, A + (size_t)s * m * m, piv + (size_t)s * m);
    if (info) info[s] = r;
  }
  return 0;
}

int oracle_lu_solve(int n, int m, const double *LU, const int *piv, double *b)
{
#pragma omp parallel for schedule(static) if (n >= 64)
  for (int s = 0; s < n; ++s) lu_solve(m, LU + (size_t)s * m * m, piv + (size_t)s * m, b + (size_t)s * m);
  return 0;
}

int oracle_flamelet_stencils(const void *mp, const double *dz, int nzi, const double *chi, const double *invLe,
                             double *cmaj, double *csub, double *csup, double *mc, double *nc)
{
  const Mech &m = *static_cast<const Mech *>(mp);
  const int ns = m.ns;
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
  return 0;
}

int oracle_flamelet_rhs(const void *mp, const double *state, double p, const double *oxy, const double *fuel,
                        int adiabatic, const double *Tc, const double *hc, const double *Tr, const double *hr, int nzi,
                        const double *cmajor, const double *csub, const double *csup, const double *mc,
                        const double *nc, const double *chi, int eflux, int vcp, int scaled, double *out)
{
  const Mech &m = *static_cast<const Mech *>(mp);
  flamelet_rhs(m, state, p, oxy, fuel, adiabatic, Tc, hc, Tr, hr, nzi, cmajor, csub, csup, mc, nc, chi, eflux, vcp,
               scaled, out);
  return 0;
}

int oracle_flamelet_jacobian(const void *mp, const double *state, double p, const double *oxy, const double *fuel,
                             int adiabatic, const double *Tc, const double *hc, const double *Tr, const double *hr,
                             int nzi, const double *cmajor, const double *csub, const double *csup, const double *mc,
                             const double *nc, const double *chi, int scale_offset, double pref, int opt, int eflux,
                             int scaled, double *J)
{
  const Mech &m = *static_cast<const Mech *>(mp);
  flamelet_jacobian(m, state, p, oxy, fuel, adiabatic, Tc, hc, Tr, hr, nzi, cmajor, csub, csup, mc, nc, chi,
                    scale_offset, pref, opt, eflux, scaled, J);
  return 0;
}

int oracle_btddod_full_factorize(double *d, int nb, int bs, double *l, int *piv)
{
  btddod_factor(d, nb, bs, l, piv);
  return 0;
}

int oracle_btddod_full_solve(const double *d, const double *l, const int *piv, const double *rhs, int nb, int bs,
                             double *x)
{
  btddod_solve(d, l, piv, rhs, nb, bs, x);
  return 0;
}

int oracle_btddod_full_matvec(const double *a, const double *x, int nb, int bs, double *y)
{
  btddod_matvec(a, x, nb, bs, y);
  return 0;
}

}  // extern "C"
