"""Adiabatic steady laminar flamelet (SLFM) libraries on the GPU flamelet solvers.

``build_adiabatic_slfm_library`` keeps the interface and behaviour of spitfire/chemistry/tabulation.py:229-336:
a sequential continuation in the dissipation rate, each flamelet started from the previous converged profile,
solved with compute_steady_state (Newton, then pseudo-transient continuation), stopped at extinction
(max(T - T_linear) < 10 K, :299) unless include_extinguished, and returned as a ``Library`` over
(mixture_fraction, dissipation_rate_stoich or _max). The first flamelet starts from the Burke-Schumann profile:
the reference starts it from Cantera's HP equilibrium, which is not available here; both starts converge to the
burning steady solution the solver tolerance defines.

``solve_steady_flamelets`` solves any number of independent flamelets (own grids, dissipation rates, initial
profiles) at once, every solver iteration one batched launch per operation over all of them.
"""

from time import perf_counter

import numpy as np

from .flamelet import FlameletBatch, FlameletSetup, FlameletSpec, compute_dissipation_rate
from .library import Dimension, Library

_mixture_fraction_name = 'mixture_fraction'
_dissipation_rate_name = 'dissipation_rate'
_stoich_suffix = '_stoich'


def _spec_copy(fs, **changes):
    d = dict(fs.__dict__)
    d.update(changes)
    return FlameletSpec(**d)


def _library_of(setup, state):
    ns = setup.mech.n_species
    st = np.asarray(state).reshape(setup.nzi, ns)
    full = np.vstack([setup.state_oxy, st, setup.state_fuel])
    props = {'temperature': full[:, 0], 'pressure': np.full(setup.z.size, setup.pressure)}
    names = setup.mech.species_names
    last = np.ones(setup.z.size)
    for i, sp in enumerate(names[:-1]):
        props['mass fraction ' + sp] = full[:, 1 + i]
        last = last - full[:, 1 + i]
    props['mass fraction ' + names[-1]] = last
    return props


def solve_steady_flamelets(setups, tolerance=1.e-6):
    """Steady states of a batch of adiabatic flamelets (compute_steady_state per flamelet, all advanced together).
    Returns (states: list of numpy arrays or None where a flamelet did not converge, method per flamelet)."""
    b = FlameletBatch(setups)
    out, conv, how = b.compute_steady_state(tolerance=tolerance)
    out = out.cpu().numpy()
    conv = conv.cpu().numpy()
    newton = how['newton'].cpu().numpy()
    states, methods = [], []
    for f, s in enumerate(setups):
        lo, hi = b.offz_host[f] * b.ns, b.offz_host[f + 1] * b.ns
        states.append(out[lo:hi].copy() if conv[f] else None)
        methods.append(None if not conv[f] else ('newton' if newton[f] else 'psitc'))
    return states, methods


def build_adiabatic_slfm_library(flamelet_specs, diss_rate_values=np.logspace(-3, 2, 16),
                                 diss_rate_ref='stoichiometric', verbose=True, solver_verbose=False,
                                 _return_intermediates=False, include_extinguished=False, diss_rate_log_scaled=True):
    if isinstance(flamelet_specs, dict):
        flamelet_specs = FlameletSpec(**flamelet_specs)
    m = flamelet_specs.mech_spec
    fs = _spec_copy(flamelet_specs, initial_condition='Burke-Schumann', dissipation_rate=None,
                    max_dissipation_rate=None, stoich_dissipation_rate=None)
    t00 = perf_counter()
    if verbose:
        print('-' * 82)
        print('building adiabatic SLFM library (GPU flamelet solvers)')
        print(f'- {m.n_species} species, {m.n_reactions} reactions')
        print(f'- stoichiometric mixture fraction: {m.stoich_mixture_fraction(fs.fuel_stream, fs.oxy_stream):.3f}')
        print('-' * 82)
    suffix = _stoich_suffix if diss_rate_ref == 'stoichiometric' else '_max'
    x_values = []
    table = {}
    z = None
    ic = 'Burke-Schumann'
    for idx, chival in enumerate(np.asarray(diss_rate_values, dtype=np.float64)):
        key = 'max_dissipation_rate' if diss_rate_ref == 'maximum' else 'stoich_dissipation_rate'
        setup = FlameletSetup(_spec_copy(fs, initial_condition=ic, **{key: float(chival)}))
        z = setup.z
        if verbose:
            print(f'{idx + 1:4}/{len(diss_rate_values):4} (chi{suffix} = {chival:8.1e} 1/s) ', end='', flush=True)
        t0 = perf_counter()
        states, methods = solve_steady_flamelets([setup])
        if states[0] is None:
            raise RuntimeError(f'steady flamelet solve failed at chi{suffix} = {chival}')
        state = states[0]
        T = state[::m.n_species]
        if np.max(T - setup.linear_temperature) < 10. and not include_extinguished:
            if verbose:
                print(' extinction detected, stopping. The extinguished state will not be included in the table.')
            break
        if verbose:
            print(f' converged in {perf_counter() - t0:6.2f} s ({methods[0]}), T_max = {np.max(T):6.1f}')
        chi_st = compute_dissipation_rate(np.array([setup.z_st]), setup.max_dissipation_rate, setup.form)[0]
        x_values.append(chi_st)
        table[chi_st] = _library_of(setup, state)
        if _return_intermediates:
            table[chi_st]['adiabatic_state'] = state.copy()
        ic = state.copy()
    if _return_intermediates:
        return table, z, np.array(x_values)
    lib = Library(Dimension(_mixture_fraction_name, z),
                  Dimension(_dissipation_rate_name + _stoich_suffix, np.array(x_values), diss_rate_log_scaled))
    lib.extra_attributes['mech_spec'] = m
    for q in table[x_values[-1]]:
        lib[q] = lib.get_empty_dataset()
        for ix, x in enumerate(x_values):
            lib[q][:, ix] = table[x][q]
    if verbose:
        print(f'library built in {perf_counter() - t00:6.2f} s')
    return lib
