"""ORACLE -- test infrastructure, not the product.

CPU checks of the reactor parameter gradients (project-written; the reference computes no parameter
sensitivities). Parameters theta are (ln A_r, E_a,r) per reaction r in the mechanism's internal order (the setter
order: simple, three-body, Lindemann, Troe), interleaved [ln A_0, E_a,0, ln A_1, ...]; A is the forward or, for
falloff reactions, the high-pressure pre-exponential factor, E_a its activation energy in J/kmol.

* ``frozen_integrate``: the oracle ESDIRK64 integration (oracle/integrate.py) on a given step-size sequence (the
  Jacobian set up at the start of every step, as the defaults do), recording the stage values of every step.
* ``outputs``: the final temperature and the smoothed ignition delay
      tau_s = sum_n h_n sum_s b_s g(T(Y_ns)),  g(T) = 1 - 1 / (1 + exp(-(T - T0 - dT_ign) / width)),
  i.e. the ESDIRK64 quadrature of the time spent below T0 + dT_ign, smoothed over `width` kelvin.
* ``forward_sensitivity``: dy/dtheta propagated through the same stages (exact stage Jacobians), giving both
  outputs' gradients; ``fd_gradient``: central finite differences on the frozen step sequence with perturbed
  mechanisms (relative step 1e-6 in ln A and in E_a).
"""

import copy

import numpy as np
from scipy.linalg import lu_factor, lu_solve

import integrate as I
import oracle as orc

RU = 8314.46261815324
DT_IGN = 400.
WIDTH = 20.


def g_smooth(T, T0, dT=DT_IGN, width=WIDTH):
    return 1. - 1. / (1. + np.exp(-(T - T0 - dT) / width))


def dg_smooth(T, T0, dT=DT_IGN, width=WIDTH):
    s = 1. / (1. + np.exp(-(T - T0 - dT) / width))
    return -s * (1. - s) / width


def frozen_integrate(prob, q0, dts, nonlinear_tolerance=1.e-12, max_nonlinear_iter=20):
    """ESDIRK64 steps of sizes dts from q0 (no error control). Returns (final state, stages [N][6][neq])."""
    from scipy.linalg.lapack import dgetrf, dgetrs
    neq = q0.size
    w = np.ones(neq)
    w[prob.Tidx] = 1.e-3
    state = np.array(q0, dtype=np.float64)
    stages = np.zeros((len(dts), 6, neq))
    for n, dt in enumerate(dts):
        Jm = prob.jac(state) * (dt * I.GAMMA)
        Jm[np.diag_indices(neq)] -= 1.
        lu, piv, _ = dgetrf(Jm)
        k = np.zeros((6, neq))
        k[0] = prob.rhs(state)
        stages[n, 0] = state
        Y = state.copy()
        for s in range(1, 6):
            prior = I.A[s, :s] @ k[:s]
            resid = dt * (I.GAMMA * k[s - 1] + prior) - (Y - state)
            f = k[s - 1]
            for it in range(max_nonlinear_iter):
                Y = Y - dgetrs(lu, piv, resid)[0]
                f = prob.rhs(Y)
                resid = dt * (I.GAMMA * f + prior) - (Y - state)
                if np.max(np.abs(resid * w)) < nonlinear_tolerance:
                    break
            k[s] = f
            stages[n, s] = Y
        state = state + dt * (I.B @ k)
        state[state < 0.] = 0.
    return state, stages


def outputs(final_state, stages, dts, Tidx, T0):
    tau = 0.
    for n, dt in enumerate(dts):
        tau += dt * float(I.B @ g_smooth(stages[n, :, Tidx], T0))
    return final_state[Tidx], tau


class ParamJacobian:
    """df/dtheta of the closed adiabatic isobaric or isochoric reactor right-hand side at a state."""

    def __init__(self, spec, og, configuration, pressure):
        self.spec, self.og = spec, og
        self.configuration = configuration
        self.pressure = pressure
        ns = spec.n_species
        self.ns = ns
        self.neq = ns if configuration == 'isobaric' else ns + 1
        self.tix = 0 if configuration == 'isobaric' else 1
        mw = spec.molecular_weights
        idx = {n: i for i, n in enumerate(spec.species_names)}
        nr = len(spec.mech_data['reactions'])
        self.nu = np.zeros((nr, ns))  # net stoichiometry nu_sr (products - reactants), mass-weighted below
        for r, rx in enumerate(spec.mech_data['reactions']):
            for sp, v in rx[1].items():
                self.nu[r, idx[sp]] -= v
            for sp, v in rx[2].items():
                self.nu[r, idx[sp]] += v
        self.numw = self.nu * mw[None, :]

    def __call__(self, q):
        og, ns, tix = self.og, self.ns, self.tix
        T = q[tix]
        Y = np.hstack([q[tix + 1:], 1. - np.sum(q[tix + 1:])])
        mmw = 1. / np.sum(Y / self.spec.molecular_weights)
        rho = q[0] if self.configuration == 'isochoric' else self.pressure * mmw / (RU * T)
        _, sr = og.rate_param_sens_batch(np.array([T]), np.array([rho]), Y[None, :])
        sr = sr[0]
        e = np.zeros(ns)
        if self.configuration == 'isobaric':
            og.species_enthalpies(T, e)
            c = og.cp_mix(T, Y)
        else:
            og.species_energies(T, e)
            c = og.cv_mix(T, Y)
        col = np.zeros((self.neq, self.numw.shape[0]))
        col[tix] = -(self.numw @ e) / (rho * c)
        col[tix + 1:] = (self.numw[:, :ns - 1] / rho).T
        F = np.zeros((self.neq, 2 * self.numw.shape[0]))
        F[:, 0::2] = col * sr[None, :]
        F[:, 1::2] = col * (-sr / (RU * T))[None, :]
        return F


def forward_sensitivity(prob, pj, q0, dts, stages):
    """Gradients (dT_end/dtheta, dtau_s/dtheta) by forward sensitivities through the recorded stages."""
    neq = q0.size
    P = pj.numw.shape[0] * 2
    S = np.zeros((neq, P))
    dtau = np.zeros(P)
    T0 = q0[prob.Tidx]
    for n, dt in enumerate(dts):
        K = np.zeros((6, neq, P))
        SY = np.zeros((6, neq, P))
        for s in range(6):
            Ys = stages[n, s]
            J = prob.jac(Ys)
            F = pj(Ys)
            rhs = S + dt * np.tensordot(I.A[s, :s], K[:s], axes=(0, 0)) if s > 0 else S.copy()
            if s == 0:
                SY[s] = S
            else:
                M = np.eye(neq) - dt * I.GAMMA * J
                SY[s] = lu_solve(lu_factor(M), rhs + dt * I.GAMMA * F)
            K[s] = J @ SY[s] + F
            dtau += dt * I.B[s] * dg_smooth(Ys[prob.Tidx], T0) * SY[s][prob.Tidx]
        # the post-step clamp: clamped entries have zero sensitivity
        v = stages[n, 0] + dt * (I.B @ np.array([prob.rhs(stages[n, s]) for s in range(6)]))
        S = S + dt * np.tensordot(I.B, K, axes=(0, 0))
        S[v < 0.] = 0.
    return S[prob.Tidx].copy(), dtau


def perturbed(spec, r, which, factor):
    """Copy of the mechanism with reaction r's ln A shifted by `factor` (which=0) or E_a scaled by (1+factor)
    (which=1; an E_a of zero is shifted by factor * 1e3 R instead)."""
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    md = copy.deepcopy(spec.mech_data)
    t = list(md['reactions'][r])
    if which == 0:
        t[4] = t[4] * np.exp(factor)
    else:
        t[6] = t[6] * (1. + factor) if t[6] != 0. else factor * 1.e3 * RU
    md['reactions'][r] = tuple(t)
    sp = ChemicalMechanismSpec(mech_data=md)
    og = orc.OracleGriffon()
    sp._populate_griffon(og)
    return sp, og


def fd_gradient(spec, configuration, pressure, q0, dts, params, rel=1.e-6):
    """Central finite differences of (T_end, tau_s) for the parameter indices `params` (interleaved layout)."""
    out = np.zeros((2, len(params)))
    T0 = q0[0 if configuration == 'isobaric' else 1]
    for k, p in enumerate(params):
        r, which = divmod(p, 2)
        ea = spec.mech_data['reactions'][r][6]
        vals = []
        for sgn in (1., -1.):
            sp, og = perturbed(spec, r, which, sgn * rel)
            prob = I.ReactorProblem(og, configuration, pressure=pressure)
            fs, st = frozen_integrate(prob, q0, dts)
            vals.append(outputs(fs, st, dts, prob.Tidx, T0))
        step = 2. * rel if which == 0 else 2. * (rel * ea if ea != 0. else rel * 1.e3 * RU)
        out[:, k] = (np.array(vals[0]) - np.array(vals[1])) / step
    return out
