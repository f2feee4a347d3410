"""ORACLE -- test infrastructure, not the product.

CPU restatement of Spitfire's transient flamelet integration and of the transient enthalpy-defect expansion:

* ``FlameletTransientProblem``: what Flamelet.integrate hands odesolve (spitfire/chemistry/flamelet.py:1046-1213).
  * The right-hand side is the FlameletOperator's (oracle Griffon).
  * The linear setup is _*_setup_block_thomas (flamelet.py:756-761, 881-886): prefactor * J - I in BTDDOD form,
    factorized by the reference's block-Thomas algorithm (oracle.btddod_full_factorize).
  * The linear solve is _solve_block_thomas (flamelet.py:911-915).
  * The norm weighting is 1 / variable scales: 1e-3 on temperatures (flamelet.py:613-614).
* ``integrate_for_heat_loss`` (flamelet.py:1263-1286), with integrate()'s defaults:
  * oracle.integrate.integrate (odesolve + ESDIRK64 + simple Newton + PI control);
  * the Jacobian reused for up to 10 steps, at least 40 steps, negative entries clipped after every step;
  * stopped when max(state) < (1 + 0.05) max(T_oxy, T_fuel), or when the step residual falls below 1e-4.
* ``transient_defect_entries`` (tabulation.py:339-406): one dissipation rate's trajectory subsampled every
  h_stoich_spacing of stoichiometric enthalpy, first and last states always kept, as the unstructured table
  entries {(chi_st, defect_st): data}.

Used by tests/ to pin the GPU transient integrator and defect library: against the reference's own trajectory
(tests/golden/nonadiabatic_transient_slfm_gold.npz) and against the reference test's gold library.
"""

import numpy as np

import oracle as orc
from integrate import integrate


class FlameletTransientProblem:
    def __init__(self, op):
        self.op = op
        n = op.nzi * op.ns
        self.weights = np.ones(n)
        self.weights[::op.ns] = 1.e-3
        self._fac = None

    def rhs(self, q, t=0.):
        return self.op.rhs(q)

    def linear_setup(self, q, prefactor):
        J = self.op.jac(q, scale_and_offset=True, prefactor=prefactor)
        self._fac = orc.btddod_full_factorize(J, self.op.nzi, self.op.ns)

    def linear_solve(self, r):
        d, l, piv = self._fac
        return orc.btddod_full_solve(d, l, piv, r, self.op.nzi, self.op.ns)


def integrate_for_heat_loss(op, state0, T_bc_max, temperature_tolerance=0.05, steady_tolerance=1.e-4,
                            first_time_step=1.e-6, max_time_step=1.e-3, transient_tolerance=1.e-10,
                            minimum_time_step_count=40, maximum_steps_per_jacobian=10, nonlinear_tolerance=1.e-12):
    """Returns the oracle.integrate.integrate result with every accepted step (times, states)."""
    def stop(t, state, residual, nsteps):
        return np.max(state) < (1. + temperature_tolerance) * T_bc_max or residual < steady_tolerance

    return integrate(FlameletTransientProblem(op), np.asarray(state0, dtype=np.float64),
                     first_time_step=first_time_step, max_time_step=max_time_step,
                     transient_tolerance=transient_tolerance, nonlinear_tolerance=nonlinear_tolerance,
                     minimum_time_step_count=minimum_time_step_count,
                     maximum_steps_per_jacobian=maximum_steps_per_jacobian, save_each_step=True,
                     stop_criteria=stop)


def _interp(x, xp, fp):
    return float(np.interp(x, xp, fp))


def transient_defect_entries(og, chi_st, z, z_st, states, oxy_state, fuel_state, pressure, species_names,
                             h_stoich_spacing):
    """tabulation.py:376-404 for one dissipation rate. states: [nt, nzi*ns] interior states (the first the
    adiabatic one); oxy_state / fuel_state: [T, Y_0..Y_{ns-2}] of the boundaries. Returns {(chi_st, g_st): data}
    with the library's quantities over the full grid, enthalpy from the oracle Griffon."""
    ns = len(species_names)
    nt = states.shape[0]
    nz = z.size

    def full(st):
        T = np.empty(nz)
        Y = np.empty((nz, ns))
        T[0], T[-1] = oxy_state[0], fuel_state[0]
        T[1:-1] = st[::ns]
        for b, bs in ((0, oxy_state), (nz - 1, fuel_state)):
            Y[b, :-1] = bs[1:]
        for i in range(ns - 1):
            Y[1:-1, i] = st[1 + i::ns]
        Y[:, -1] = 1. - Y[:, :-1].sum(axis=1)
        return T, Y

    TY = [full(states[i]) for i in range(nt)]
    h_tz = np.array([[og.enthalpy_mix(T[k], Y[k]) for k in range(nz)] for T, Y in TY])
    h_ad = h_tz[0]
    indices = [0]
    last = _interp(z_st, z, h_ad)
    for i in range(nt):
        this = _interp(z_st, z, h_tz[i])
        if last - this > h_stoich_spacing:
            indices.append(i)
            last = this
    if nt - 1 not in indices:
        indices.append(nt - 1)
    out = {}
    for i in indices:
        T, Y = TY[i]
        defect = h_tz[i] - h_ad
        g = _interp(z_st, z, defect)
        data = {'enthalpy_defect': defect.copy(), 'enthalpy_cons': h_ad.copy(), 'enthalpy': h_tz[i].copy(),
                'mixture_fraction': z.copy(), 'temperature': T.copy(), 'pressure': np.full(nz, pressure)}
        for k, n in enumerate(species_names):
            data['mass fraction ' + n] = Y[:, k].copy()
        out[(chi_st, g)] = data
    return out
