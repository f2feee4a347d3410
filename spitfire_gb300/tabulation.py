"""Steady laminar flamelet (SLFM) libraries on the GPU flamelet solvers: adiabatic, and nonadiabatic with an
enthalpy-defect dimension from quasisteady or transient heat loss.

``build_adiabatic_slfm_library`` keeps the interface and behaviour of spitfire/chemistry/tabulation.py:229-336:
a sequential continuation in the dissipation rate, each flamelet started from the previous converged profile,
solved with compute_steady_state (Newton, then pseudo-transient continuation), stopped at extinction
(max(T - T_linear) < 10 K, :299) unless include_extinguished, and returned as a ``Library`` over
(mixture_fraction, dissipation_rate_stoich or _max). The first flamelet starts from the Burke-Schumann profile:
the reference starts it from Cantera's HP equilibrium, which is not available here; both starts converge to the
burning steady solution the solver tolerance defines.

``build_nonadiabatic_defect_steady_slfm_library`` keeps the interface of tabulation.py:786-845: for every burning
dissipation rate of the adiabatic library, a continuation in the convection coefficient of a heat-loss flamelet
(linear reference temperature profile, no radiation) until extinction (tabulation.py:408-519), the solutions
subsampled every h_stoich_spacing of stoichiometric enthalpy, then interpolated onto n_defect_st uniformly spaced
stoichiometric enthalpy defects (tabulation.py:594-665) and returned over (mixture_fraction,
dissipation_rate_stoich, enthalpy_defect_stoich). The continuations of all dissipation rates advance together,
each step one batched steady solve.

``build_nonadiabatic_defect_transient_slfm_library`` keeps the interface of tabulation.py:727-784: the same
defect dimension from transient heat loss instead, every burning dissipation rate's heat-loss flamelet integrated
in time (ESDIRK64 on the GPU kernels) until its temperature profile is nearly linear, all of them in one batch.

The unstrained libraries need no flamelet solve and keep the reference's interfaces as well:
``build_unreacted_library``, ``build_adiabatic_bs_library`` and ``build_nonadiabatic_defect_bs_library``
(tabulation.py:55-226). The equilibrium variants need Cantera's equilibrium solver and raise NotImplementedError.

``solve_steady_flamelets`` solves any number of independent flamelets (own grids, dissipation rates, initial
profiles) at once, every solver iteration one batched launch per operation over all of them.
"""

from time import perf_counter

import numpy as np

from .flamelet import Flamelet, FlameletBatch, FlameletSetup, FlameletSpec, compute_dissipation_rate
from .library import Dimension, Library

_mixture_fraction_name = 'mixture_fraction'
_dissipation_rate_name = 'dissipation_rate'
_enthalpy_defect_name = 'enthalpy_defect'
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


def _as_spec(flamelet_specs, **changes):
    fs = FlameletSpec(**flamelet_specs) if isinstance(flamelet_specs, dict) else flamelet_specs
    return _spec_copy(fs, **changes)


def build_unreacted_library(flamelet_specs, verbose=True):
    """Nonreacting library over the mixture fraction (tabulation.py:55-72): the streams mixed at constant enthalpy
    and pressure, no reaction."""
    f = Flamelet(_as_spec(flamelet_specs, initial_condition='unreacted'))
    return f.make_library_from_interior_state(f.initial_interior_state)


def build_adiabatic_bs_library(flamelet_specs, verbose=True):
    """Burke-Schumann (infinitely fast one-step combustion) library over the mixture fraction (tabulation.py:
    96-113)."""
    f = Flamelet(_as_spec(flamelet_specs, initial_condition='Burke-Schumann'))
    return f.make_library_from_interior_state(f.initial_interior_state)


def build_adiabatic_eq_library(flamelet_specs, verbose=True):
    """tabulation.py:75-93 needs Cantera's HP equilibrium, which is not available."""
    raise NotImplementedError('equilibrium libraries need Cantera\'s equilibrium solver, which is not available')


def build_nonadiabatic_defect_bs_library(flamelet_specs, n_defect_st=16, verbose=True):
    """Burke-Schumann library with a presumed triangular enthalpy defect (tabulation.py:116-187, 209-226): the
    adiabatic profile's enthalpy lowered by g fz(Z) (fz = Z / Z_st below the stoichiometric mixture fraction,
    (1 - Z) / (1 - Z_st) above) for n_defect_st stoichiometric defects g from 0 down to the defect of the profile
    cooled to the linear temperature, the temperature solved from each enthalpy at fixed composition and
    pressure. Returns a Library over (mixture_fraction, enthalpy_defect_stoich)."""
    fs = _as_spec(flamelet_specs, initial_condition='Burke-Schumann')
    m = fs.mech_spec
    fuel, oxy = fs.fuel_stream, fs.oxy_stream
    z_st = m.stoich_mixture_fraction(fuel, oxy)
    f = Flamelet(fs)
    ns = m.n_species
    state_ad = f.initial_interior_state
    ad = f.make_library_from_interior_state(state_ad)
    h_ad = _enthalpy_of_props(m, ad)
    z = f.mixfrac_grid
    cooled = state_ad.copy()
    cooled[::ns] = z[1:-1] * fuel.T + (1. - z[1:-1]) * oxy.T
    h_ce = _enthalpy_of_props(m, f.make_library_from_interior_state(cooled))
    defect_ext = float(np.interp(z_st, z, h_ad)) - float(np.interp(z_st, z, h_ce))
    defects = np.linspace(-defect_ext, 0., n_defect_st)[::-1]
    lib = Library(Dimension(_mixture_fraction_name, z), Dimension(_enthalpy_defect_name + _stoich_suffix, defects))
    lib.extra_attributes['mech_spec'] = m
    fz = np.where(z <= z_st, z / z_st, (1. - z) / (1. - z_st))
    names = m.species_names
    Y = np.stack([np.asarray(ad['mass fraction ' + n]) for n in names], axis=-1)
    props = {q: lib.get_empty_dataset() for q in list(ad.props) + ['enthalpy_defect', 'enthalpy_cons', 'enthalpy',
                                                                   _mixture_fraction_name]}
    T = np.array(ad['temperature'], dtype=np.float64)
    for ig, g in enumerate(defects):
        h = h_ad + g * fz
        T[1:-1] = m.temperature_from_enthalpy_vec(h[1:-1], Y[1:-1], 1500.)
        for q in ad.props:
            props[q][:, ig] = T if q == 'temperature' else np.asarray(ad[q])
        props['enthalpy_defect'][:, ig] = h - h_ad
        props['enthalpy_cons'][:, ig] = h_ad
        props['enthalpy'][:, ig] = h
        props[_mixture_fraction_name][:, ig] = z
    for q, v in props.items():
        lib[q] = v
    return lib


def build_nonadiabatic_defect_eq_library(flamelet_specs, n_defect_st=16, verbose=True):
    """tabulation.py:189-206 needs Cantera's HP equilibrium, which is not available."""
    raise NotImplementedError('equilibrium libraries need Cantera\'s equilibrium solver, which is not available')


def solve_steady_flamelets(setups, tolerance=1.e-6):
    """Steady states of a batch of adiabatic flamelets (compute_steady_state per flamelet, all advanced together).
    Returns (states: list of numpy arrays or None where a flamelet did not converge, method per flamelet)."""
    b = FlameletBatch(setups)
    out, conv, how = b.compute_steady_state(tolerance=tolerance)
    out = out.cpu().numpy()
    conv = conv.cpu().numpy()
    newton = how['newton'].cpu().numpy()
    esdirk = how['esdirk'].cpu().numpy()
    states, methods = [], []
    for f, s in enumerate(setups):
        lo, hi = b.offz_host[f] * b.ns, b.offz_host[f + 1] * b.ns
        states.append(out[lo:hi].copy() if conv[f] else None)
        methods.append(None if not conv[f] else ('newton' if newton[f] else ('esdirk' if esdirk[f] else 'psitc')))
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


# ------------------------------------------------------------------------------------------------------ heat loss
def _mixture_enthalpy(m, T, Y):
    """Mass-specific mixture enthalpy of states T[...] and Y[..., ns] (the quantity Cantera's enthalpy_mass gives
    analysis.compute_specific_enthalpy, from the same NASA7 polynomials)."""
    T = np.asarray(T, dtype=np.float64)
    hs, _ = m.species_h_cp_host_vec(T.ravel())
    return (hs * np.asarray(Y).reshape(-1, m.n_species)).sum(1).reshape(T.shape)


def _enthalpy_of_props(m, props):
    names = m.species_names
    Y = np.stack([props['mass fraction ' + n] for n in names], axis=-1)
    return _mixture_enthalpy(m, props['temperature'], Y)


def _expand_defect_steady(flamelet_specs, table, chis, h_stoich_spacing, verbose):
    """Quasisteady heat-loss continuation of every dissipation rate (tabulation.py:408-519), all advanced together:
    convection coefficient h += dh from 0 with dh = 0.1, dh *= min(max(sqrt(0.1 / diff), 0.1), 2) after each solve
    (diff: largest relative change of the interior state), until the maximum of the interior state drops below
    max(T_oxy, T_fuel) + 10 (extinction) or h reaches 1e10. Returns the unstructured table {(chi_st, g_st): data}."""
    m = flamelet_specs.mech_spec
    fs = _spec_copy(flamelet_specs, heat_transfer='nonadiabatic', scale_heat_loss_by_temp_range=False,
                    scale_convection_by_dissipation=False, use_linear_ref_temp_profile=True,
                    radiative_emissivity=0., convection_coefficient=0., dissipation_rate=None,
                    max_dissipation_rate=None)
    t_ext = max(flamelet_specs.oxy_stream.T, flamelet_specs.fuel_stream.T) + 10.
    k = len(chis)
    hval = np.zeros(k)
    dh = np.full(k, 0.1)
    diff_target = 0.1
    hval_max = 1.e10
    state = [table[c]['adiabatic_state'].copy() for c in chis]
    state_old = [x.copy() for x in state]
    running = np.ones(k, dtype=bool)
    hvalues = [[0.] for _ in chis]
    solutions = [[{q: v for q, v in table[c].items() if q != 'adiabatic_state'}] for c in chis]
    z = None
    setup0 = None
    it = 0
    while running.any():
        it += 1
        idx = np.flatnonzero(running)
        hval[idx] += dh[idx]
        setups = [FlameletSetup(_spec_copy(fs, stoich_dissipation_rate=float(chis[i]),
                                           convection_coefficient=float(hval[i]), initial_condition=state[i]))
                  for i in idx]
        setup0 = setups[0]
        z = setup0.z
        states, methods = solve_steady_flamelets(setups)
        for j, i in enumerate(idx):
            if states[j] is None:
                raise RuntimeError(f'steady heat-loss flamelet solve failed at chi_st = {chis[i]}, h = {hval[i]}')
            cur = states[j]
            diff = np.max(np.abs(cur - state_old[i]) / (np.abs(cur) + 1.e-4))
            extinguished = np.max(cur) < t_ext
            state[i] = cur
            state_old[i] = cur.copy()
            dh[i] *= np.min([np.max([np.sqrt(diff_target / diff), 0.1]), 2.])
            hvalues[i].append(hval[i])
            solutions[i].append(_library_of(setups[j], cur))
            if extinguished or hval[i] >= hval_max:
                running[i] = False
        if verbose:
            print(f'  heat-loss step {it:4d}: {int(running.sum())} of {k} flamelets still burning', flush=True)
    z_st = m.stoich_mixture_fraction(flamelet_specs.fuel_stream, flamelet_specs.oxy_stream)
    out = {}
    for i, chi in enumerate(chis):
        sols = solutions[i]
        h_tz = np.stack([_enthalpy_of_props(m, sol) for sol in sols], axis=1)  # [nz, nt]
        h_ad = h_tz[:, 0]
        nt = h_tz.shape[1]
        indices = [0]
        last_hst = np.interp(z_st, z, h_ad)
        for t in range(nt - 1):
            this_hst = np.interp(z_st, z, h_tz[:, t])
            if last_hst - this_hst > h_stoich_spacing:
                indices.append(t)
                last_hst = this_hst
        for t in indices:
            defect = h_tz[:, t] - h_ad
            gst = float(np.interp(z_st, z, defect))
            data = {'enthalpy_defect': defect.copy(), 'enthalpy_cons': h_ad.copy(), 'enthalpy': h_tz[:, t].copy(),
                    _mixture_fraction_name: z.copy()}
            for q, v in sols[t].items():
                data[q] = np.asarray(v).copy()
            out[(chi, gst)] = data
    return out


def _structure_defect(unstructured, n_defect_st, extend=False):
    """tabulation.py:594-665: every quantity of every dissipation rate interpolated onto n_defect_st uniformly spaced
    stoichiometric defects between the smallest and largest of all flamelets (piecewise linear, constant beyond a
    flamelet's own range; enthalpy and enthalpy_defect extrapolated linearly when extend). Returns (table, sorted
    dissipation rates, defects in decreasing order)."""
    gs = np.array([g for (_, g) in unstructured])
    gmin, gmax = float(gs.min()), float(gs.max())
    space = np.linspace(gmin, gmax, n_defect_st)
    if extend:
        sp = abs(space[1] - space[0])
        space = np.linspace(gmin - 2 * sp, gmax, n_defect_st + 2)
    chis = sorted({c for (c, _) in unstructured})
    table = {}
    for chi in chis:
        gl = np.array(sorted(g for (c, g) in unstructured if c == chi))
        first = unstructured[(chi, gl[0])]
        for q in first:
            Y = np.stack([unstructured[(chi, g)][q] for g in gl], axis=0)  # [ng, nz]
            for gs_ in space:
                if extend and q in ('enthalpy', 'enthalpy_defect') and gl.size > 1 and not gl[0] <= gs_ <= gl[-1]:
                    lo = 0 if gs_ < gl[0] else gl.size - 2
                    w = (gs_ - gl[lo]) / (gl[lo + 1] - gl[lo])
                    val = Y[lo] + w * (Y[lo + 1] - Y[lo])
                elif gl.size == 1:
                    val = Y[0].copy()
                else:
                    val = np.array([np.interp(gs_, gl, Y[:, iz]) for iz in range(Y.shape[1])])
                table.setdefault((chi, gs_), {})[q] = val
                if q in ('density', 'temperature') and np.any(val < 1.e-14):
                    raise ValueError(f'{q} < 1.e-14 detected!')
    return table, np.array(chis), space[::-1]


def build_nonadiabatic_defect_steady_slfm_library(flamelet_specs, diss_rate_values=np.logspace(-3, 2, 16),
                                                  diss_rate_ref='stoichiometric', verbose=True,
                                                  solver_verbose=False, h_stoich_spacing=10.e3, num_procs=1,
                                                  integration_args=None, n_defect_st=32, extend_defect_dim=False,
                                                  diss_rate_log_scaled=True):
    """SLFM library with an enthalpy-defect dimension from quasisteady heat loss (tabulation.py:786-845); see the
    module docstring. num_procs and integration_args are accepted for interface compatibility: the continuations
    already run together on the device, and no time integration is involved."""
    if isinstance(flamelet_specs, dict):
        flamelet_specs = FlameletSpec(**flamelet_specs)
    m = flamelet_specs.mech_spec
    t00 = perf_counter()
    table, z, x_values = build_adiabatic_slfm_library(flamelet_specs, diss_rate_values, diss_rate_ref,
                                                      verbose, solver_verbose, _return_intermediates=True)
    if verbose:
        print('expanding (steady) enthalpy defect dimension ...', flush=True)
    unstructured = _expand_defect_steady(flamelet_specs, table, list(x_values), h_stoich_spacing, verbose)
    lib = _defect_library(m, unstructured, n_defect_st, extend_defect_dim, diss_rate_log_scaled)
    if verbose:
        print(f'library built in {perf_counter() - t00:6.2f} s')
    return lib


def _defect_library(m, unstructured, n_defect_st, extend_defect_dim, diss_rate_log_scaled):
    """The structured defect table as a Library over (mixture_fraction, dissipation_rate_stoich,
    enthalpy_defect_stoich) (tabulation.py:694-724)."""
    st, xs, gs = _structure_defect(unstructured, n_defect_st, extend_defect_dim)
    key0 = next(iter(st))
    lib = Library(Dimension(_mixture_fraction_name, st[key0][_mixture_fraction_name]),
                  Dimension(_dissipation_rate_name + _stoich_suffix, xs, diss_rate_log_scaled),
                  Dimension(_enthalpy_defect_name + _stoich_suffix, gs))
    lib.extra_attributes['mech_spec'] = m
    for q in st[key0]:
        vals = lib.get_empty_dataset()
        for ix, x in enumerate(xs):
            for ig, g in enumerate(gs):
                vals[:, ix, ig] = st[(x, g)][q]
        lib[q] = vals
    return lib


def _expand_defect_transient(flamelet_specs, table, chis, h_stoich_spacing, integration_args, verbose):
    """Transient heat loss of every dissipation rate (tabulation.py:339-406), all integrated together: each
    flamelet starts from its adiabatic steady state with scaled convective heat loss (coefficient 1e7 unless the
    specs give one, scaled by the temperature range and the dissipation rate, linear reference temperature profile,
    no radiation) and runs until its temperature profile is nearly linear or it is steady (integrate_for_heat_loss,
    flamelet.py:1263-1286). Flamelets whose integration fails are retried with a 100x lower tolerance, as the
    reference does, down to 1e-15. Each trajectory is subsampled every h_stoich_spacing of stoichiometric enthalpy,
    the first and last states always kept. Returns the unstructured table {(chi_st, g_st): data}."""
    m = flamelet_specs.mech_spec
    hc = flamelet_specs.convection_coefficient if flamelet_specs.convection_coefficient is not None else 1.e7
    fs = _spec_copy(flamelet_specs, heat_transfer='nonadiabatic', scale_heat_loss_by_temp_range=True,
                    scale_convection_by_dissipation=True, use_linear_ref_temp_profile=True,
                    convection_coefficient=hc, radiative_emissivity=0., dissipation_rate=None,
                    max_dissipation_rate=None)
    args = {'first_time_step': 1.e-9, 'max_time_step': 1.e-1}
    args.update(integration_args or {})
    for key in ('write_log', 'log_rate', 'print_exception_on_failure', 'linear_solver'):
        args.pop(key, None)
    tol = args.pop('transient_tolerance', 1.e-8)
    temperature_tolerance = args.pop('temperature_tolerance', 0.05)
    steady_tolerance = args.pop('steady_tolerance', 1.e-4)
    T_bc_max = max(flamelet_specs.oxy_stream.T, flamelet_specs.fuel_stream.T)

    def stop(f, t, state, residual, steps):
        return np.max(state) < (1. + temperature_tolerance) * T_bc_max or residual < steady_tolerance

    pending = list(range(len(chis)))
    done = {}
    while pending:
        if tol <= 1.e-15:
            raise RuntimeError('transient heat-loss integration failed for chi_st = '
                               + ', '.join(f'{chis[i]:.3e}' for i in pending))
        setups = [FlameletSetup(_spec_copy(fs, stoich_dissipation_rate=float(chis[i]),
                                           initial_condition=table[chis[i]]['adiabatic_state'])) for i in pending]
        traj, stats = FlameletBatch(setups).integrate(stop_criteria=stop, transient_tolerance=tol, **args)
        retry = []
        for j, i in enumerate(pending):
            ok = stats['status'][j] != 4 and np.all(np.isfinite(traj[j][1][-1]))
            if ok:
                done[i] = (setups[j], traj[j])
            else:
                retry.append(i)
        if verbose:
            print(f'  transient heat loss at tolerance {tol:.1e}: {len(pending) - len(retry)} of {len(pending)} '
                  f'flamelets done', flush=True)
        pending = retry
        tol *= 1.e-2
    z_st = m.stoich_mixture_fraction(flamelet_specs.fuel_stream, flamelet_specs.oxy_stream)
    out = {}
    for i, chi in enumerate(chis):
        setup, (times, states) = done[i]
        z = setup.z
        sols = [_library_of(setup, st) for st in states]
        h_tz = np.stack([_enthalpy_of_props(m, sol) for sol in sols], axis=0)  # [nt, nz]
        h_ad = h_tz[0]
        nt = h_tz.shape[0]
        indices = [0]
        last_hst = np.interp(z_st, z, h_ad)
        for t in range(nt):
            this_hst = np.interp(z_st, z, h_tz[t])
            if last_hst - this_hst > h_stoich_spacing:
                indices.append(t)
                last_hst = this_hst
        if nt - 1 not in indices:
            indices.append(nt - 1)
        for t in indices:
            defect = h_tz[t] - h_ad
            gst = float(np.interp(z_st, z, defect))
            data = {'enthalpy_defect': defect.copy(), 'enthalpy_cons': h_ad.copy(), 'enthalpy': h_tz[t].copy(),
                    _mixture_fraction_name: z.copy()}
            for q, v in sols[t].items():
                data[q] = np.asarray(v).copy()
            out[(chi, gst)] = data
    return out


def build_nonadiabatic_defect_transient_slfm_library(flamelet_specs, diss_rate_values=np.logspace(-3, 2, 16),
                                                     diss_rate_ref='stoichiometric', verbose=True,
                                                     solver_verbose=False, h_stoich_spacing=10.e3, num_procs=1,
                                                     integration_args=None, n_defect_st=32,
                                                     extend_defect_dim=False, diss_rate_log_scaled=True):
    """SLFM library with an enthalpy-defect dimension from transient heat loss (tabulation.py:727-784): the adiabatic
    library, then every burning dissipation rate's heat-loss flamelet integrated in time on the GPU (all of them in
    one batch), subsampled, and interpolated onto n_defect_st stoichiometric enthalpy defects. num_procs is accepted
    for interface compatibility: the integrations already run together on the device. integration_args go to the
    heat-loss integration as in the reference (transient_tolerance, first_time_step, max_time_step, ...)."""
    if isinstance(flamelet_specs, dict):
        flamelet_specs = FlameletSpec(**flamelet_specs)
    m = flamelet_specs.mech_spec
    t00 = perf_counter()
    table, z, x_values = build_adiabatic_slfm_library(flamelet_specs, diss_rate_values, diss_rate_ref,
                                                      verbose, solver_verbose, _return_intermediates=True)
    if verbose:
        print('expanding (transient) enthalpy defect dimension ...', flush=True)
    unstructured = _expand_defect_transient(flamelet_specs, table, list(x_values), h_stoich_spacing,
                                            integration_args, verbose)
    lib = _defect_library(m, unstructured, n_defect_st, extend_defect_dim, diss_rate_log_scaled)
    if verbose:
        print(f'library built in {perf_counter() - t00:6.2f} s')
    return lib
