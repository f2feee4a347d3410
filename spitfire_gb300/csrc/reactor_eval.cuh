// Per-state evaluation of the reactor right-hand side and analytical Jacobian by one state group, shared by the
// batched Jacobian kernel (chem_kernels.cu) and the persistent integrator (integrate_kernels.cu).
//
// Phases (group-synchronous):
//   P0  load the state; mixture molecular weight and density              (reduction over species)
//   P1  concentrations and species thermodynamics                         (lanes over species)
//   P2  reaction rates q_r and, for Jacobians, their derivatives           (lanes over reactions)
//   P3  species gathers w_i (and S_rho_i, S_T_i, P_i, Q_i)                 (gather program)
//   P4  right-hand side, rho/T columns, dense-term coefficients            (lanes over species)
//   P5  Y block of the Jacobian and T-row sums                             (gather program)
//   P6  T row of the Jacobian                                              (lanes over columns)
// Reference: isochoric_reactor_kernels.cpp:18-333, isobaric_reactor_kernels.cpp:19-343.
#pragma once
#include "chem_device.cuh"

namespace sfgb {

struct ReactorCfg {
  int configuration;  // 0 isobaric (q = [T, Y]), 1 isochoric (q = [rho, T, Y])
  int heat;           // 0 adiabatic, 1 isothermal, 2 diathermal
  int option;         // rates-sensitivity option
  double Tc, Tr, hc, eps, SoV;
  int open;           // mass exchange with a feed of temperature Tin, mass fractions yin[ns] (device), density
  double tau, rho_in, Tin;  // rho_in (isochoric), over the mixing time tau
  const double *yin;
};

struct Progs {
  DevProgram w, full, j;
};

struct SpeciesSums {
  double cpmix, cpsens;
};

// P1: concentrations and thermodynamics of every species; y must already be in scratch.
template <int G, bool JAC, class S>
__device__ __forceinline__ SpeciesSums prep_species(const DevMech &m, const Blob &b, const ScratchLayout &L,
                                                    S scr, const Group<G> &grp, const StateCtx &s,
                                                    bool isochoric, bool want_eh)
{
  const int ns = m.ns, lane = grp.lane;
  double cpmix = 0., cpsens = 0.;
  for (int i = lane; i < ns; i += G) {
    const double yi = scr[L.y + i];
    const double invmw = b.d[m.d_invmw + i];
    scr[L.C + i] = yi * s.rho * invmw;
    const SpeciesThermo th = species_thermo(m, b, i, s.T, s.logT, s.invT, JAC);
    store_gibbs_factor(scr, L, i, th.g * s.invT * m.invRu, b.d + m.d_exptab);
    if (want_eh) {
      scr[L.eh + i] = isochoric ? th.h - m.Ru * s.T * invmw : th.h;
      scr[L.cpv + i] = isochoric ? th.cp - m.Ru * invmw : th.cp;
      cpmix += yi * th.cp;
    } else {
      scr[L.eh + i] = 0.;
    }
    // gather destinations start at zero: an entry with no contributions (an inert species) is never written
    scr[L.w + i] = 0.;
    if (JAC) {
      scr[L.dB + i] = th.dB;
      scr[L.dcp + i] = th.dcp;
      cpsens += yi * th.dcp;
      scr[L.Srho + i] = 0.;
      scr[L.ST + i] = 0.;
      scr[L.P + i] = 0.;
      scr[L.Q + i] = 0.;
    }
  }
  SpeciesSums r;
  r.cpmix = grp.sum(cpmix);
  r.cpsens = JAC ? grp.sum(cpsens) : 0.;
  grp.sync();
  return r;
}

// P2 + P3: reaction rates (and derivatives) and the species gathers. Returns (EA, EB) of the T-row dense terms.
template <int G, bool JAC, int U = default_unroll(G), class S>
__device__ __forceinline__ double2 reactions_and_gathers(const DevMech &m, const Blob &b, const ScratchLayout &L,
                                                         S scr, const Group<G> &grp, const StateCtx &s,
                                                         const Progs &pg)
{
  double EA = 0., EB = 0.;
  for (int r = grp.lane; r < m.nr; r += G) eval_reaction<JAC>(m, b, L, scr, s, r, &EA, &EB);
  if (JAC) {
    EA = grp.sum(EA);
    EB = grp.sum(EB);
  }
  grp.sync();
  NoJ noj;
  run_program<G, U>(JAC ? pg.full : pg.w, grp.lane, b.d, scr, noj);
  grp.sync();
  return make_double2(EA, EB);
}

// Reactor right-hand side (and, with JAC, the analytical Jacobian) of the state qs (neq values, any memory space).
// rhs receives neq values; jset(row, col, value) receives every Jacobian entry exactly once.
// U: gather batch (loads in flight per lane); smaller batches use fewer registers. OPEN = false compiles the feed
// terms of open reactors out (c.open is then ignored).
template <int G, bool JAC, int U = default_unroll(G), bool OPEN = true, class JSet, class S>
__device__ void reactor_eval(const DevMech &m, const Blob &b, const ScratchLayout &L, S scr,
                             const Group<G> &grp, const double *qs, double pres, const ReactorCfg &c,
                             const Progs &pg, double *rhs, JSet &jset)
{
  const int ns = m.ns, lane = grp.lane;
  const bool isochoric = c.configuration == 1;
  const bool open_ = OPEN && c.open;
  const int neq = isochoric ? ns + 1 : ns;
  // ---------------- P0
  double T, rho = 0.;
  if (isochoric) {
    rho = qs[0];
    T = qs[1];
  } else {
    T = qs[0];
  }
  double sy = 0.;
  for (int i = lane; i < ns - 1; i += G) {
    const double yi = qs[(isochoric ? 2 : 1) + i];
    scr[L.y + i] = yi;
    sy += yi;
  }
  sy = grp.sum(sy);
  if (lane == 0) scr[L.y + ns - 1] = 1. - sy;  // extract_y (combustion_kernels.h:526-535)
  grp.sync();
  double sim = 0.;
  for (int i = lane; i < ns; i += G) sim += scr[L.y + i] * b.d[m.d_invmw + i];
  sim = grp.sum(sim);
  const double mmw = 1. / sim;
  if (!isochoric) rho = pres * mmw / (T * m.Ru);
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
  s.option = c.option;
  // ---------------- P1-P3
  const SpeciesSums sums = prep_species<G, JAC>(m, b, L, scr, grp, s, isochoric, true);
  const double2 E = reactions_and_gathers<G, JAC, U>(m, b, L, scr, grp, s, pg);
  const double EA = E.x, EB = E.y;
  const double cmix = isochoric ? sums.cpmix - m.Ru / mmw : sums.cpmix;  // cv or cp
  const double cpsens = sums.cpsens;
  // feed of an open reactor (isochoric_reactor_kernels.cpp:39-154, isobaric_reactor_kernels.cpp:31-168):
  // fe = sum_i (e_i(Tin) - e_i(T)) yin_i (enthalpies when isobaric), fc = sum_i yin_i cv_i(T) (cp_i)
  double fe = 0., fc = 0.;
  if (open_) {
    const double Tin = c.Tin, lTin = log(Tin), iTin = 1. / Tin;
    for (int i = lane; i < ns; i += G) {
      const SpeciesThermo th = species_thermo(m, b, i, Tin, lTin, iTin, false);
      const double ein = isochoric ? th.h - m.Ru * Tin * b.d[m.d_invmw + i] : th.h;
      const double yi = c.yin[i];
      fe += (ein - scr[L.eh + i]) * yi;
      fc += yi * scr[L.cpv + i];
    }
    fe = grp.sum(fe);
    fc = grp.sum(fc);
  }
  // mass-exchange factor of the species and energy equations: rho_in / (tau rho) isochoric, 1 / tau isobaric
  const double itau = open_ ? 1. / c.tau : 0.;
  const double mfac = open_ ? (isochoric ? itau * c.rho_in / rho : itau) : 0.;
  const double mrT = open_ ? fe / cmix * mfac : 0.;  // feed term of the temperature equation

  // ---------------- P4: right-hand side and rho/T columns
  double swe = 0., sre = 0., ste = 0., swc = 0.;
  for (int i = lane; i < ns; i += G) {
    const double e = scr[L.eh + i];
    swe += scr[L.w + i] * e;
    if (JAC) {
      sre += scr[L.Srho + i] * e;
      ste += scr[L.ST + i] * e;
      swc += scr[L.w + i] * scr[L.cpv + i];
    }
  }
  swe = grp.sum(swe);
  if (JAC) {
    sre = grp.sum(sre);
    ste = grp.sum(ste);
    swc = grp.sum(swc);
  }
  const double invRho = s.invRho;
  const double iC = 1. / cmix, iRC = 1. / (rho * cmix);
  const double rhsT = -swe / (rho * cmix);
  double qheat = 0.;
  if (c.heat == 2)
    qheat = c.SoV / (rho * cmix) * (c.hc * (c.Tc - T) + c.eps * 5.67e-8 * (c.Tr * c.Tr * c.Tr * c.Tr - T * T * T * T));
  const int tix = isochoric ? 1 : 0;  // index of T in the state
  for (int i = lane; i < ns - 1; i += G) {
    double v = scr[L.w + i] * invRho;
    if (open_) v += (c.yin[i] - scr[L.y + i]) * mfac;
    rhs[tix + 1 + i] = v;
  }
  if (lane == 0) {
    if (isochoric) rhs[0] = open_ ? (c.rho_in - rho) * itau : 0.;
    rhs[tix] = c.heat == 1 ? 0. : (open_ ? rhsT + qheat + mrT : rhsT + qheat);
  }
  if (!JAC) {
    grp.sync();
    return;
  }
  // primitive rho and T columns of the T row (chem_jac_isochoric / chem_jac_isobaric)
  const double JTrho = -iRC * sre - invRho * rhsT;
  const double JTT = -iC * (invRho * (ste + swc) + rhsT * cpsens);
  const double cpv_last = scr[L.cpv + ns - 1];
  if (isochoric) {
    for (int i = lane; i < ns - 1; i += G) {
      double v = invRho * (scr[L.Srho + i] - invRho * scr[L.w + i]);
      if (open_) v -= (c.yin[i] - scr[L.y + i]) * mfac * invRho;
      jset(2 + i, 0, v);
      jset(2 + i, 1, invRho * scr[L.ST + i]);
    }
  } else {
    // isobaric transform (isobaric_reactor_kernels.cpp:319-343): T column = PJ_T - rho/T * PJ_rho, and the Y
    // columns get (-rho*mmw) * u_k * PJ_rho, folded into P
    const double roT = rho / T, nrm = -rho * mmw;
    for (int i = lane; i < ns - 1; i += G) {
      const double pjr = invRho * (scr[L.Srho + i] - invRho * scr[L.w + i]);
      const double pjt = invRho * scr[L.ST + i];
      jset(1 + i, 0, pjt - roT * pjr);
      scr[L.P + i] += nrm * pjr;
    }
  }
  for (int k = lane; k < ns; k += G) scr[L.trow + k] = 0.;
  grp.sync();

  // ---------------- P5: Y block (species rows/columns) and T-row sums; an open reactor's feed adds -mfac on the
  // diagonal (rho_in / (tau rho) isochoric, 1 / tau isobaric)
  {
    const int off = isochoric ? 2 : 1;
    const bool diag = open_;
    const double dyy = -mfac;
    auto yblock = [&](int row, int col, double v) {
      if (diag && row == col) v += dyy;
      jset(off + row, off + col, v);
    };
    run_program<G, U>(pg.j, lane, b.d, scr, yblock);
  }
  grp.sync();

  // ---------------- P6: T row (and the zero rho row of the isochoric Jacobian)
  const double iso_heat = (c.heat == 1) ? 0. : 1.;
  if (isochoric) {
    for (int k = lane; k < ns - 1; k += G) {
      const double ts = scr[L.trow + k] + b.d[m.d_u + k] * EA + EB;
      double v = -iC * ts - rhsT * (scr[L.cpv + k] - cpv_last) * iC;
      if (open_) v += -iC * mrT * (scr[L.cpv + k] - cpv_last);
      if (c.heat == 2) v += iC * qheat * (cpv_last - scr[L.cpv + k]);
      jset(1, 2 + k, v * iso_heat);
    }
    for (int k = lane; k < neq; k += G) jset(0, k, (k == 0 && open_) ? -itau : 0.);
    if (lane == 0) {
      double j10 = JTrho, j11 = JTT;
      if (open_) {
        j10 += -mrT * invRho;
        j11 += -iC * (itau * invRho * c.rho_in * fc + cpsens * mrT);
      }
      if (c.heat == 2) {
        j10 += -qheat / rho;
        j11 += -iC * cpsens * qheat - c.SoV * iRC * (c.hc + 4. * c.eps * 5.67e-8 * T * T * T);
      }
      jset(1, 0, j10 * iso_heat);
      jset(1, 1, j11 * iso_heat);
    }
  } else {
    const double roT = rho / T, nrm = -rho * mmw;
    double pjr = JTrho, pjt = JTT;
    if (open_) pjt += -iC * (cpsens * mrT + itau * fc);
    if (c.heat == 2) {
      pjr += -qheat / rho;
      pjt += -iC * cpsens * qheat - c.SoV * iRC * (c.hc + 4. * c.eps * 5.67e-8 * T * T * T);
    }
    pjr *= iso_heat;
    pjt *= iso_heat;
    for (int k = lane; k < ns - 1; k += G) {
      const double ts = scr[L.trow + k] + b.d[m.d_u + k] * EA + EB;
      double v = -iC * ts - rhsT * (scr[L.cpv + k] - cpv_last) * iC;
      if (open_) v += -mrT * (scr[L.cpv + k] - cpv_last) * iC;
      if (c.heat == 2) v += iC * qheat * (cpv_last - scr[L.cpv + k]);
      jset(0, 1 + k, v * iso_heat + nrm * b.d[m.d_u + k] * pjr);
    }
    if (lane == 0) jset(0, 0, pjt - roT * pjr);
  }
  grp.sync();
}

}  // namespace sfgb
