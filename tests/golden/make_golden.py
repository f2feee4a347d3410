"""Generate the golden fixtures of tests/golden from the reference Spitfire itself.

Runs only where the reference sources exist (this needs the reference Griffon built by `make -C oracle ref` and
the reference's Python modules, loaded by oracle/ref_harness.py). The fixtures pin the oracle:

  kernels_<mech>.npz   seeded states and the reference Griffon's production rates, rate sensitivities (options
                       0, 1, 2) and isochoric / isobaric reactor right-hand sides and Jacobians
  ignition_ref.json    ignition delays, accepted-step counts and final temperatures from the reference
                       HomogeneousReactor.compute_ignition_delay (reference odesolve + ESDIRK64 + Newton + PI)
  h2_mech_data.json    the Cantera-converted mech_data embedded in tests/tabulation/adiabatic_slfm/gold.pkl
  closed_reactor_gold.npz  the reference's stored closed-reactor trajectories (tests/reactor/closed_reactors/gold.pkl)
  open_kernels_<mech>.npz  seeded states with a feed and the reference Griffon's open-reactor (mass exchange)
                       right-hand sides and Jacobians, isochoric and isobaric, adiabatic / isothermal / diathermal
  open_reactor_gold.npz    the reference's stored open-reactor trajectory under an oscillating feed temperature
                       (tests/reactor/oscillating_feed_temperature/gold.pkl)
  flamelet_ref.npz     reference Flamelet (flamelet.py) residuals, BTDDOD Jacobians (plain, scaled, with eigenvalue
                       bounds), block-Thomas solves and matvecs, and steady Newton / psitc solutions with iteration
                       counts, for an H2 and a GRI-3.0 flamelet started from a Burke-Schumann profile
  adiabatic_slfm_gold.npz  temperature and mass fractions of tests/tabulation/adiabatic_slfm/gold.pkl
  flamelet_nonad_ref.npz   reference Flamelet residuals and BTDDOD Jacobians with heat loss (convection and
                       radiation per point; unscaled, and scaled by the temperature range with the linear reference
                       temperature profile) for the flamelet cases
  nonadiabatic_steady_slfm_gold.npz  dimensions, temperature, mass fractions and enthalpy defect of
                       tests/tabulation/nonadiabatic_defect_steady_slfm/gold.pkl

  nonadiabatic_transient_slfm_gold.npz  the reference's transient heat-loss trajectory of one H2 flamelet
                       (times, temperatures, sampled mass fractions, heat-loss parameters), its adiabatic
                       ignition transient from the linear profile to t = 2 ms, and the dimensions,
                       temperature, mass fractions and enthalpy defect of
                       tests/tabulation/nonadiabatic_defect_transient_slfm/gold.pkl

  structure_defect_ref.npz  a seeded unstructured defect table and the reference's structured interpolation of
                       it (tabulation.py:594-665), without and with the extended defect range

  adiabatic_unreacted_gold.npz, adiabatic_burke_schumann_gold.npz, nonadiabatic_defect_burke_schumann_gold.npz
                       dimensions and properties (all but viscosity) of the reference's unstrained library golds

  dropin_ref.npz       the reference's single-state PyCombustionKernels methods called directly: every thermo getter
                       at temperatures inside and outside the NASA7 ranges, flamelet_stencils, flamelet_jac_indices,
                       flamelet_rhs and flamelet_jacobian (adiabatic and nonadiabatic, each flag combination its
                       callers use, rates options 0/1/2) on the flamelet cases, and the ten module-level
                       py_btddod_* functions on seeded block-diagonally dominant matrices of several sizes

  reference_<name>_gold.pkl  byte copies of the reference's pickled gold libraries
                       (tests/tabulation/<name>/gold.pkl): the reader of reference-written libraries is tested on them

Usage:  python tests/golden/make_golden.py --reference PATH [kernels] [ignition] [gold] [flamelets] [open] [nonadiabatic]
                                           [transient] [structure] [unstrained] [dropin] [libraries]
"""
import json
import os
import pickle
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'oracle'))
sys.path.insert(0, os.path.join(ROOT, 'tests'))
REF = None     # the reference checkout: --reference PATH, or SPITFIRE_REFERENCE
MECHS = None


def seeded_states(spec, n, seed):
    rng = np.random.default_rng(seed)
    ns = spec.n_species
    T = rng.uniform(300., 2800., n)
    p = 101325. * np.exp(rng.uniform(0., np.log(40.), n))
    Y = rng.dirichlet(0.5 * np.ones(ns), n)
    mmw = 1. / (Y / spec.molecular_weights).sum(1)
    rho = p * mmw / (8314.46261815324 * T)
    return T, p, Y, rho


def kernels():
    import ref_harness as rh
    for fname, phase, name, n in [('h2-burke.yaml', 'h2-burke', 'h2-burke', 16),
                                  ('methane-gri30.yaml', 'methane-gri30', 'methane-gri30', 6),
                                  ('reaction_test_mechanism.yaml', None, 'reaction-test', 13)]:
        ref = rh.ReferenceMechanism(os.path.join(MECHS, fname), phase)
        g = ref.griffon
        ns = ref.n_species
        T, p, Y, rho = seeded_states(ref, n, 4242)
        w = np.zeros((n, ns))
        S = np.zeros((3, n, (ns + 1) ** 2))
        for i in range(n):
            g.production_rates(T[i], rho[i], Y[i], w[i])
            for opt in range(3):
                g.prod_rates_primitive_sensitivities(rho[i], T[i], Y[i], opt, S[opt, i])
        yin = np.zeros(ns)
        qiv = np.hstack([rho[:, None], T[:, None], Y[:, :-1]])
        qib = np.hstack([T[:, None], Y[:, :-1]])
        riv = np.zeros((n, ns + 1))
        Jiv = np.zeros((n, (ns + 1) ** 2))
        rib = np.zeros((n, ns))
        Jib = np.zeros((n, ns * ns))
        rib_rhs = np.zeros((n, ns))
        riv_rhs = np.zeros((n, ns + 1))
        for i in range(n):
            g.reactor_jac_isochoric(qiv[i], 0., 0., yin, 1., 0., 0., 0., 0., 1., 0, False, 0, riv[i], Jiv[i])
            g.reactor_rhs_isochoric(qiv[i], 0., 0., yin, 1., 0., 0., 0., 0., 1., 0, False, riv_rhs[i])
            g.reactor_jac_isobaric(qib[i], p[i], 0., yin, 1., 0., 0., 0., 0., 1., 0, False, 0, 0, rib[i], Jib[i])
            g.reactor_rhs_isobaric(qib[i], p[i], 0., yin, 1., 0., 0., 0., 0., 1., 0, False, rib_rhs[i])
        np.savez_compressed(os.path.join(HERE, f'kernels_{name}.npz'), T=T, p=p, Y=Y, rho=rho, w=w, S=S, qiv=qiv,
                            qib=qib, jac_rhs_iv=riv, Jiv=Jiv, rhs_iv=riv_rhs, jac_rhs_ib=rib, Jib=Jib, rhs_ib=rib_rhs)
        print('kernels', name, n)


OPEN_HEAT = {'adiabatic': 0, 'isothermal': 1, 'diathermal': 2}
# convection / radiation parameters of the diathermal cases: Tc, Tr, h, eps, surface-to-volume
OPEN_DIATHERMAL = (600., 900., 50., 0.3, 20.)


def open_kernels():
    import ref_harness as rh
    for fname, phase, name, n in [('h2-burke.yaml', 'h2-burke', 'h2-burke', 12),
                                  ('methane-gri30.yaml', 'methane-gri30', 'methane-gri30', 4)]:
        ref = rh.ReferenceMechanism(os.path.join(MECHS, fname), phase)
        g = ref.griffon
        ns = ref.n_species
        T, p, Y, rho = seeded_states(ref, n, 4343)
        rng = np.random.default_rng(4344)
        Tin = rng.uniform(300., 1500., n)
        Yin = rng.dirichlet(0.5 * np.ones(ns), n)
        tau = np.exp(rng.uniform(np.log(1.e-6), np.log(1.e-2), n))
        rhoin = rho * rng.uniform(0.5, 2., n)
        qiv = np.hstack([rho[:, None], T[:, None], Y[:, :-1]])
        qib = np.hstack([T[:, None], Y[:, :-1]])
        arrs = dict(T=T, p=p, Y=Y, rho=rho, Tin=Tin, Yin=Yin, tau=tau, rhoin=rhoin, qiv=qiv, qib=qib)
        Tc, Tr, hc, eps, sov = OPEN_DIATHERMAL
        for heat, ho in OPEN_HEAT.items():
            riv, Jiv = np.zeros((n, ns + 1)), np.zeros((n, (ns + 1) ** 2))
            rib, Jib = np.zeros((n, ns)), np.zeros((n, ns * ns))
            riv_r, rib_r = np.zeros((n, ns + 1)), np.zeros((n, ns))
            for i in range(n):
                g.reactor_rhs_isochoric(qiv[i], rhoin[i], Tin[i], Yin[i], tau[i], Tc, Tr, hc, eps, sov, ho, True,
                                        riv_r[i])
                g.reactor_jac_isochoric(qiv[i], rhoin[i], Tin[i], Yin[i], tau[i], Tc, Tr, hc, eps, sov, ho, True, 0,
                                        riv[i], Jiv[i])
                g.reactor_rhs_isobaric(qib[i], p[i], Tin[i], Yin[i], tau[i], Tc, Tr, hc, eps, sov, ho, True,
                                       rib_r[i])
                g.reactor_jac_isobaric(qib[i], p[i], Tin[i], Yin[i], tau[i], Tc, Tr, hc, eps, sov, ho, True, 0, 0,
                                       rib[i], Jib[i])
            arrs.update({f'{heat}_rhs_iv': riv_r, f'{heat}_jac_rhs_iv': riv, f'{heat}_Jiv': Jiv,
                         f'{heat}_rhs_ib': rib_r, f'{heat}_jac_rhs_ib': rib, f'{heat}_Jib': Jib})
        np.savez_compressed(os.path.join(HERE, f'open_kernels_{name}.npz'), **arrs)
        print('open kernels', name, n)
    t, T, Y = pickle.load(open(os.path.join(REF, 'tests', 'reactor', 'oscillating_feed_temperature', 'gold.pkl'),
                               'rb'))
    np.savez_compressed(os.path.join(HERE, 'open_reactor_gold.npz'), t=np.asarray(t), T=np.asarray(T),
                        Y=np.asarray(Y))
    print('open reactor gold', np.asarray(t).shape)


IGNITION_CASES = [
    # (mechanism, phase, configuration, T0, phi, p_atm, fuel)
    ('h2-burke.yaml', 'h2-burke', 'isobaric', 1200., 1.0, 1.0, 'H2'),
    ('h2-burke.yaml', 'h2-burke', 'isochoric', 1200., 1.0, 1.0, 'H2'),
    ('h2-burke.yaml', 'h2-burke', 'isobaric', 1000., 0.6, 5.0, 'H2'),
    ('methane-gri30.yaml', 'methane-gri30', 'isobaric', 1200., 1.0, 1.0, 'CH4'),
    ('methane-gri30.yaml', 'methane-gri30', 'isobaric', 1400., 0.7, 10.0, 'CH4'),
    ('methane-gri30.yaml', 'methane-gri30', 'isobaric', 1100., 1.8, 3.0, 'CH4'),
    ('methane-gri30.yaml', 'methane-gri30', 'isobaric', 1300., 1.3, 20.0, 'CH4'),
    ('methane-gri30.yaml', 'methane-gri30', 'isochoric', 1250., 1.0, 2.0, 'CH4'),
]


def ignition():
    import ref_harness as rh
    from spitfire_gb300.mechanism import Stream
    ns_ref = rh.load_reference()
    out = []
    for fname, phase, conf, T0, phi, patm, fuel in IGNITION_CASES:
        ref = rh.ReferenceMechanism(os.path.join(MECHS, fname), phase)
        spec = ref.spec
        X = np.zeros(spec.n_species)
        if fuel == 'H2':
            X[spec.species_index('H2')] = 2. * phi
            X[spec.species_index('O2')] = 1.
            X[spec.species_index('N2')] = 3.76
        else:
            X[spec.species_index('CH4')] = phi
            X[spec.species_index('O2')] = 2.
            X[spec.species_index('N2')] = 2. * 3.76
        Y = X * spec.molecular_weights
        Y /= Y.sum()
        mix = Stream(spec, T0, patm * 101325., Y)
        r = ns_ref.reactors.HomogeneousReactor(ref, mix, conf, 'adiabatic', 'closed')
        tau, lib = r.compute_ignition_delay(return_solution=True)
        times = lib.time_values
        Tf = lib['temperature'][-1]
        out.append(dict(mechanism=phase, configuration=conf, T0=T0, phi=phi, p=patm * 101325., Y0=Y.tolist(),
                        tau=float(tau), steps=int(times.size - 1), T_final=float(Tf)))
        print(out[-1]['mechanism'], conf, T0, phi, patm, tau, times.size - 1)
    with open(os.path.join(HERE, 'ignition_ref.json'), 'w') as f:
        json.dump(out, f, indent=1)


class _Stub:
    def __init__(self, *a, **k):
        pass

    def __setstate__(self, st):
        self.__dict__['_st'] = st


class _U(pickle.Unpickler):
    def find_class(self, mod, name):
        if mod.startswith('spitfire'):
            return type(name, (_Stub,), {})
        return super().find_class(mod, name)


def gold():
    d = _U(open(os.path.join(REF, 'tests', 'tabulation', 'adiabatic_slfm', 'gold.pkl'), 'rb')).load()
    md = d._st['extra_attributes']['mech_spec']._st['mech_data']
    conv = json.loads(json.dumps(md, default=float))
    with open(os.path.join(HERE, 'h2_mech_data.json'), 'w') as f:
        json.dump(conv, f)
    g = pickle.load(open(os.path.join(REF, 'tests', 'reactor', 'closed_reactors', 'gold.pkl'), 'rb'))
    arrs = {}
    for k, (t, T, Y) in g.items():
        key = k.replace(', ', '_').replace(' ', '_')
        arrs[key + '_t'] = np.asarray(t)
        arrs[key + '_T'] = np.asarray(T)
        arrs[key + '_Y'] = np.asarray(Y)
    np.savez_compressed(os.path.join(HERE, 'closed_reactor_gold.npz'), **arrs)
    print('gold', list(g.keys()))


def flamelets():
    import ref_harness as rh
    from flamelet_cases import FLAMELET_CASES, flamelet_case_setup
    from spitfire_gb300.flamelet import burke_schumann_state, clustered_grid
    ns_ref = rh.load_reference()
    G = ns_ref.griffon
    out = {}
    for case in FLAMELET_CASES:
        name, fname, phase = case[:3]
        ref = rh.ReferenceMechanism(os.path.join(MECHS, fname), phase)
        spec = ref.spec
        oxy, fuel, kw = flamelet_case_setup(spec, case)
        zst = spec.stoich_mixture_fraction(fuel, oxy)
        z, _ = clustered_grid(kw['grid_points'], zst, 4.)
        ic = burke_schumann_state(spec, oxy, fuel, z, 101325.)
        F = ns_ref.flamelet.Flamelet(ns_ref.flamelet.FlameletSpec(mech_spec=ref, initial_condition=ic, **kw))
        nzi, ns = F._nz_interior, F._n_equations
        rng = np.random.default_rng(case[-1])
        st = ic * (1. + 0.02 * rng.standard_normal(ic.size))
        st = np.abs(st)
        pre = name + '_'
        out[pre + 'z'] = F._z
        out[pre + 'chi'] = F._x
        out[pre + 'oxy'] = F._state_oxy
        out[pre + 'fuel'] = F._state_fuel
        out[pre + 'ic'] = ic
        out[pre + 'state'] = st
        for ef in (0, 1):
            for vc in (0, 1):
                F._include_enthalpy_flux, F._include_variable_cp = bool(ef), bool(vc)
                out[pre + f'rhs_e{ef}v{vc}'] = F._adiabatic_rhs(0., st)
            F._include_enthalpy_flux, F._include_variable_cp = bool(ef), True
            out[pre + f'jac_e{ef}'] = F._adiabatic_jac(st)
        F._include_enthalpy_flux, F._include_variable_cp = True, True
        out[pre + 'jac_scaled'] = F._adiabatic_jac_offset_scaled(st, 1.e-3)
        diffterm = 4. * F._max_dissipation_rate
        vals, expeig = F._adiabatic_jac_and_eig(st, diffterm)
        out[pre + 'jac_eig'] = vals
        out[pre + 'expeig'] = expeig
        out[pre + 'diffterm'] = np.array(diffterm)
        # block-Thomas algebra on -J, and on -J + diag(1/ds)
        J = -out[pre + 'jac_e1']
        b = rng.standard_normal(nzi * ns)
        y = np.zeros(nzi * ns)
        G.py_btddod_full_matvec(J, b, nzi, ns, y)
        out[pre + 'matvec_b'] = b
        out[pre + 'matvec_y'] = y
        Jf = J.copy()
        lv = np.zeros(nzi * ns * ns)
        pv = np.zeros(J.size, dtype=np.int32)
        G.py_btddod_full_factorize(Jf, nzi, ns, lv, pv)
        x = np.zeros(nzi * ns)
        G.py_btddod_full_solve(Jf, lv, pv, b, nzi, ns, x)
        out[pre + 'solve_x'] = x
        ds = np.exp(rng.uniform(np.log(1e-6), np.log(1e-2), nzi * ns))
        Js = out[pre + 'jac_e1'].copy()
        G.py_btddod_scale_and_add_diagonal(Js, -1., 1. / ds, 1., nzi, ns)
        out[pre + 'scaled_ds'] = ds
        out[pre + 'scaled_values'] = Js
        # steady solvers from the Burke-Schumann profile
        F._include_enthalpy_flux, F._include_variable_cp = True, True
        lib, it, conv = F.steady_solve_newton(initial_guess=ic, tolerance=1.e-6, max_iterations=38, verbose=False)
        out[pre + 'newton_conv'] = np.array(bool(conv))
        out[pre + 'newton_iters'] = np.array(it if conv else -1)
        out[pre + 'newton_state'] = F._current_state.copy() if conv else np.zeros(0)
        F2 = ns_ref.flamelet.Flamelet(ns_ref.flamelet.FlameletSpec(mech_spec=ref, initial_condition=ic, **kw))
        lib, it, conv, mds = F2.steady_solve_psitc(initial_guess=ic, tolerance=1.e-6, max_iterations=400,
                                                   verbose=False)
        out[pre + 'psitc_conv'] = np.array(bool(conv))
        out[pre + 'psitc_iters'] = np.array(it if conv else -1)
        out[pre + 'psitc_state'] = F2._current_state.copy() if conv else np.zeros(0)
        out[pre + 'psitc_min_ds'] = np.array(mds)
        # continuation step like the SLFM builder: Newton at 1.5 chi_st from the converged psitc profile
        kw3 = dict(kw, stoich_dissipation_rate=1.5 * kw['stoich_dissipation_rate'])
        F3 = ns_ref.flamelet.Flamelet(ns_ref.flamelet.FlameletSpec(mech_spec=ref,
                                                                   initial_condition=F2._current_state.copy(), **kw3))
        lib, it, conv = F3.steady_solve_newton(tolerance=1.e-6, max_iterations=38, verbose=False)
        out[pre + 'cont_conv'] = np.array(bool(conv))
        out[pre + 'cont_iters'] = np.array(it if conv else -1)
        out[pre + 'cont_state'] = F3._current_state.copy() if conv else np.zeros(0)
        print(name, 'nzi', nzi, 'newton', out[pre + 'newton_conv'], out[pre + 'newton_iters'], 'psitc',
              out[pre + 'psitc_conv'], out[pre + 'psitc_iters'], 'continuation newton', out[pre + 'cont_conv'],
              out[pre + 'cont_iters'])
    np.savez_compressed(os.path.join(HERE, 'flamelet_ref.npz'), **out)


def nonadiabatic():
    import ref_harness as rh
    from flamelet_cases import FLAMELET_CASES, flamelet_case_setup
    from spitfire_gb300.flamelet import burke_schumann_state, clustered_grid
    ns_ref = rh.load_reference()
    out = {}
    for case in FLAMELET_CASES:
        name, fname, phase = case[:3]
        ref = rh.ReferenceMechanism(os.path.join(MECHS, fname), phase)
        spec = ref.spec
        oxy, fuel, kw = flamelet_case_setup(spec, case)
        zst = spec.stoich_mixture_fraction(fuel, oxy)
        z, _ = clustered_grid(kw['grid_points'], zst, 4.)
        ic = burke_schumann_state(spec, oxy, fuel, z, 101325.)
        rng = np.random.default_rng(case[-1] + 100)
        st = np.abs(ic * (1. + 0.02 * rng.standard_normal(ic.size)))
        nzi = z.size - 2
        variants = {
            # per-point convection / radiation parameters, unscaled
            'plain': dict(heat_transfer='nonadiabatic', convection_temperature=rng.uniform(300., 600., nzi),
                          radiation_temperature=rng.uniform(300., 900., nzi),
                          convection_coefficient=rng.uniform(1.e3, 1.e5, nzi),
                          radiative_emissivity=rng.uniform(0.1, 0.9, nzi)),
            # the transient defect builder's options (tabulation.py:341-348)
            'scaled': dict(heat_transfer='nonadiabatic', scale_heat_loss_by_temp_range=True,
                           scale_convection_by_dissipation=True, use_linear_ref_temp_profile=True,
                           convection_coefficient=1.e7, radiative_emissivity=0.5),
        }
        pre = name + '_'
        out[pre + 'state'] = st
        for vname, hk in variants.items():
            F = ns_ref.flamelet.Flamelet(ns_ref.flamelet.FlameletSpec(mech_spec=ref, initial_condition=ic,
                                                                      **dict(kw, **hk)))
            v = pre + vname + '_'
            out[v + 'T_conv'] = np.asarray(F._T_conv)
            out[v + 'T_rad'] = np.asarray(F._T_rad)
            out[v + 'h_conv'] = np.asarray(F._h_conv)
            out[v + 'h_rad'] = np.asarray(F._h_rad)
            for q in ('convection_temperature', 'radiation_temperature', 'convection_coefficient',
                      'radiative_emissivity'):
                if q in hk:
                    out[v + 'arg_' + q] = np.asarray(hk[q])
            out[v + 'rhs'] = F._nonadiabatic_rhs(0., st)
            out[v + 'jac'] = F._nonadiabatic_jac(st)
        print('nonadiabatic flamelet kernels', name, nzi)
    np.savez_compressed(os.path.join(HERE, 'flamelet_nonad_ref.npz'), **out)
    d = _U(open(os.path.join(REF, 'tests', 'tabulation', 'nonadiabatic_defect_steady_slfm', 'gold.pkl'), 'rb')).load()
    st = d._st
    arrs = {}
    for i in range(len(st['dim_ordering'])):
        n = st['dim_ordering'][i]
        arrs['dim%d_name' % i] = np.array(n)
        arrs['dim%d_values' % i] = np.asarray(st['dimensions'][n]['values'])
    for k, v in st['properties'].items():
        if k in ('temperature', 'enthalpy_defect', 'enthalpy', 'pressure') or k.startswith('mass fraction'):
            arrs['prop:' + k] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, 'nonadiabatic_steady_slfm_gold.npz'), **arrs)
    print('nonadiabatic steady slfm gold', np.asarray(st['properties']['temperature']).shape)


def transient():
    """The reference's transient heat-loss integration (Flamelet.integrate_for_heat_loss) of the H2 flamelet of
    tests/tabulation/nonadiabatic_defect_transient_slfm (air 1200 K / H2 300 K, 34 points) at chi_st = 1, started
    from the reference's own adiabatic steady solution with the transient defect builder's settings
    (tabulation.py:341-352), and that test's gold library."""
    import ref_harness as rh
    ns_ref = rh.load_reference()
    ref = rh.ReferenceMechanism(os.path.join(MECHS, 'h2-burke.yaml'), 'h2-burke')
    spec = ref.spec
    air = spec.stream(stp_air=True)
    air.TP = 1200., 101325.
    fuel = spec.stream('TPY', (300., 101325., 'H2:1'))
    FSpec, Fl = ns_ref.flamelet.FlameletSpec, ns_ref.flamelet.Flamelet
    base = dict(mech_spec=ref, oxy_stream=air, fuel_stream=fuel, grid_points=34)
    # the reference's Burke-Schumann start needs Cantera stream enthalpies: the same profile from this project's
    # burke_schumann_state on the reference's grid instead
    from spitfire_gb300.flamelet import burke_schumann_state
    z = np.asarray(Fl(FSpec(initial_condition='linear-TY', stoich_dissipation_rate=1., **base))._z)
    ic = burke_schumann_state(spec, air, fuel, z, 101325.)
    f0 = Fl(FSpec(initial_condition=ic, stoich_dissipation_rate=1., **base))
    f0.compute_steady_state(tolerance=1.e-6)
    ad = np.copy(f0._current_state)
    heat = dict(heat_transfer='nonadiabatic', scale_heat_loss_by_temp_range=True,
                scale_convection_by_dissipation=True, use_linear_ref_temp_profile=True,
                convection_coefficient=1.e7, radiative_emissivity=0.)
    f1 = Fl(FSpec(initial_condition=ad, stoich_dissipation_rate=1., **dict(base, **heat)))
    lib = f1.integrate_for_heat_loss(first_time_step=1.e-9, max_time_step=1.e-1, transient_tolerance=1.e-10,
                                     write_log=False, log_rate=100, print_exception_on_failure=False)
    t = np.asarray(lib.dim('time').values)
    T = np.asarray(lib['temperature'])
    names = spec.species_names
    Y = np.stack([np.asarray(lib['mass fraction ' + n]) for n in names], axis=-1)
    pick = np.unique(np.r_[np.arange(0, t.size, 25), t.size - 1])
    out = dict(z=np.asarray(f1._z), adiabatic_state=ad, times=t, T=T, pick=pick, Y_pick=Y[pick],
               T_conv=np.asarray(f1._T_conv), h_conv=np.asarray(f1._h_conv), T_rad=np.asarray(f1._T_rad),
               h_rad=np.asarray(f1._h_rad))
    print('transient heat loss: steps', t.size - 1, 'final max T', T[-1].max())
    # an adiabatic flamelet igniting from the linear T/Y profile (the hot air side ignites the mixing layer)
    f2 = Fl(FSpec(initial_condition='linear-TY', stoich_dissipation_rate=1., **base))
    lib2 = f2.integrate_to_time(2.e-3, first_time_step=1.e-6, transient_tolerance=1.e-10, write_log=False)
    out['ign_ic'] = np.asarray(f2._initial_state)
    out['ign_times'] = np.asarray(lib2.dim('time').values)
    out['ign_T'] = np.asarray(lib2['temperature'])
    print('adiabatic ignition transient: steps', out['ign_times'].size - 1, 'final max T', out['ign_T'][-1].max())
    d = _U(open(os.path.join(REF, 'tests', 'tabulation', 'nonadiabatic_defect_transient_slfm', 'gold.pkl'),
                'rb')).load()
    st = d._st
    for i in range(len(st['dim_ordering'])):
        n = st['dim_ordering'][i]
        out['dim%d_name' % i] = np.array(n)
        out['dim%d_values' % i] = np.asarray(st['dimensions'][n]['values'])
    for k, v in st['properties'].items():
        if k in ('temperature', 'enthalpy_defect', 'enthalpy', 'pressure') or k.startswith('mass fraction'):
            out['prop:' + k] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, 'nonadiabatic_transient_slfm_gold.npz'), **out)
    print('nonadiabatic transient slfm gold', np.asarray(st['properties']['temperature']).shape)


def structure():
    """The reference's interpolation onto the structured enthalpy-defect dimension (tabulation.py:594-665), on a
    seeded unstructured table of three dissipation rates with 4-7 ragged defects each, without and with the
    extended defect range."""
    ns_ref = rh_load()
    rng = np.random.default_rng(77)
    nz = 5
    table = {}
    out = {}
    chis = [0.3, 1.7, 9.1]
    for ci, chi in enumerate(chis):
        ng = 4 + ci + (ci == 2)
        gs = np.sort(-rng.uniform(0., 4.e6, ng))
        gs[-1] = 0.
        out['g_%d' % ci] = gs
        for gi, g in enumerate(gs):
            d = {'temperature': rng.uniform(300., 2200., nz), 'enthalpy': rng.uniform(-1.e6, 1.e6, nz),
                 'enthalpy_defect': g * rng.uniform(0.5, 1.5, nz), 'mass fraction X': rng.uniform(0., 1., nz),
                 'mixture_fraction': np.linspace(0., 1., nz)}
            table[(chi, float(g))] = d
            for q, v in d.items():
                out['in_%d_%d_%s' % (ci, gi, q)] = v
    out['chis'] = np.array(chis)
    for ext in (False, True):
        st, xs, gs = ns_ref.tabulation._interpolate_to_structured_defect_dimension(table, 6, extend=ext)
        tag = 'ext' if ext else 'plain'
        out[tag + '_x'] = xs
        out[tag + '_g'] = gs
        for ix, x in enumerate(xs):
            for ig, g in enumerate(gs):
                for q, v in st[(x, g)].items():
                    out['%s_%d_%d_%s' % (tag, ix, ig, q)] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, 'structure_defect_ref.npz'), **out)
    print('structured defect dimension', len(table), 'entries')


def unstrained():
    """Dimensions and properties of the reference's unstrained library golds (tests/tabulation/adiabatic_unreacted,
    adiabatic_burke_schumann, nonadiabatic_defect_burke_schumann: h2-burke, air 1200 K / H2 300 K, 34 points),
    all but viscosity."""
    for name in ('adiabatic_unreacted', 'adiabatic_burke_schumann', 'nonadiabatic_defect_burke_schumann'):
        d = _U(open(os.path.join(REF, 'tests', 'tabulation', name, 'gold.pkl'), 'rb')).load()
        st = d._st
        arrs = {}
        for i in range(len(st['dim_ordering'])):
            n = st['dim_ordering'][i]
            arrs['dim%d_name' % i] = np.array(n)
            arrs['dim%d_values' % i] = np.asarray(st['dimensions'][n]['values'])
        for k, v in st['properties'].items():
            if k != 'viscosity':
                arrs['prop:' + k] = np.asarray(v)
        np.savez_compressed(os.path.join(HERE, name + '_gold.npz'), **arrs)
        print(name, sorted(k for k in arrs if not k.startswith('prop:mass'))[:12])


def rh_load():
    import ref_harness as rh
    return rh.load_reference()


def slfm_gold():
    d = _U(open(os.path.join(REF, 'tests', 'tabulation', 'adiabatic_slfm', 'gold.pkl'), 'rb')).load()
    st = d._st
    dims = st['dimensions']
    order = [st['dim_ordering'][i] for i in range(len(st['dim_ordering']))]
    arrs = {}
    for i, n in enumerate(order):
        dd = dims[n]
        dd = dd._st if hasattr(dd, '_st') else dd
        arrs['dim%d_name' % i] = np.array(n)
        arrs['dim%d_values' % i] = np.asarray(dd['_values'] if '_values' in dd else dd['values'])
    for k, v in st['properties'].items():
        if k == 'temperature' or k.startswith('mass fraction') or k == 'pressure':
            arrs['prop:' + k] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, 'adiabatic_slfm_gold.npz'), **arrs)
    print('slfm gold', order, [a.shape for a in arrs.values()][:4])


def dropin():
    import ref_harness as rh
    from flamelet_cases import FLAMELET_CASES, flamelet_case_setup
    from spitfire_gb300.flamelet import burke_schumann_state, clustered_grid
    ns_ref = rh.load_reference()
    G = ns_ref.griffon
    out = {}
    for case in FLAMELET_CASES:
        name, fname, phase = case[:3]
        ref = rh.ReferenceMechanism(os.path.join(MECHS, fname), phase)
        g = ref.griffon
        ns = ref.n_species
        pre = name + '_'
        # thermodynamics, in and outside [Tmin, Tmax] of the NASA7 fits
        rng = np.random.default_rng(77 + ns)
        Ts = np.array([200., 300., 999., 1000., 1500., 2999., 3500., 6000.])
        Y = rng.dirichlet(0.5 * np.ones(ns), Ts.size)
        p = 101325. * np.exp(rng.uniform(0., np.log(40.), Ts.size))
        th = {k: [] for k in ('mmw', 'x', 'rho', 'p', 'cp', 'cv', 'h', 'e', 'cpi', 'cvi', 'hi', 'ei', 'dcpdT')}
        for T, y, pp in zip(Ts, Y, p):
            v = np.zeros(ns)
            th['mmw'].append(g.mixture_molecular_weight(y))
            g.mole_fractions(y, v)
            th['x'].append(v.copy())
            rho = g.ideal_gas_density(pp, T, y)
            th['rho'].append(rho)
            th['p'].append(g.ideal_gas_pressure(rho, T, y))
            th['cp'].append(g.cp_mix(T, y))
            th['cv'].append(g.cv_mix(T, y))
            th['h'].append(g.enthalpy_mix(T, y))
            th['e'].append(g.energy_mix(T, y))
            for k, f in (('cpi', g.species_cp), ('cvi', g.species_cv), ('hi', g.species_enthalpies),
                         ('ei', g.species_energies)):
                f(T, v)
                th[k].append(v.copy())
            g.dcpdT_species(T, y, v)
            th['dcpdT'].append(v.copy())
        out[pre + 'thermo_T'] = Ts
        out[pre + 'thermo_Y'] = Y
        out[pre + 'thermo_p'] = p
        for k, v in th.items():
            out[pre + 'thermo_' + k] = np.array(v)
        # flamelet methods with the argument lists of the reference's Flamelet closures (flamelet.py:623-915)
        oxy, fuel, kw = flamelet_case_setup(spec := ref.spec, case)
        zst = spec.stoich_mixture_fraction(fuel, oxy)
        z, _ = clustered_grid(kw['grid_points'], zst, 4.)
        ic = burke_schumann_state(spec, oxy, fuel, z, 101325.)
        F = ns_ref.flamelet.Flamelet(ns_ref.flamelet.FlameletSpec(mech_spec=ref, initial_condition=ic, **kw))
        nzi = F._nz_interior
        st = np.abs(ic * (1. + 0.02 * rng.standard_normal(ic.size)))
        dz, chi, invle = F._dz, F._x, 1. / F._lewis_numbers
        cma, csb, csp = np.zeros(nzi * ns), np.zeros(nzi * ns), np.zeros(nzi * ns)
        mc, nc = np.zeros(nzi), np.zeros(nzi)
        g.flamelet_stencils(dz, nzi, chi, invle, cma, csb, csp, mc, nc)
        nel = ns * (nzi * ns + 2 * (nzi - 1))
        rows, cols = np.zeros(nel, dtype=np.int32), np.zeros(nel, dtype=np.int32)
        g.flamelet_jac_indices(nzi, rows, cols)
        for k, v in (('dz', dz), ('chi', chi), ('invle', invle), ('cmajor', cma), ('csub', csb), ('csup', csp),
                     ('mcoeff', mc), ('ncoeff', nc), ('rows', rows), ('cols', cols), ('state', st),
                     ('oxy', F._state_oxy), ('fuel', F._state_fuel)):
            out[pre + 'flm_' + k] = v
        Tc = 300. + 1500. * rng.uniform(size=nzi)
        Tr = 300. + 1500. * rng.uniform(size=nzi)
        hc = 1.e5 * rng.uniform(size=nzi)
        hr = rng.uniform(size=nzi)
        for k, v in (('Tc', Tc), ('Tr', Tr), ('hc', hc), ('hr', hr)):
            out[pre + 'flm_' + k] = v
        null = np.zeros(1)
        heat = {'ad': (True, null, null, null, null, False), 'na': (False, Tc, Tr, hc, hr, False),
                'ns': (False, Tc, Tr, hc / 1.e3, hr, True)}
        for hk, (adb, a1, a2, a3, a4, scaled) in heat.items():
            for ef in (0, 1):
                for vc in (0, 1):
                    r = np.zeros(nzi * ns)
                    g.flamelet_rhs(st, F._pressure, F._state_oxy, F._state_fuel, adb, a1, a2, a3, a4, nzi, cma, csb,
                                   csp, mc, nc, chi, bool(ef), bool(vc), scaled, r)
                    out[pre + f'flm_rhs_{hk}_e{ef}v{vc}'] = r
        diffterm = 4. * F._max_dissipation_rate
        jac_cases = {'plain_r0': ('ad', False, 0., False, 0., 0, True), 'plain_r1': ('ad', False, 0., False, 0., 1, True),
                     'plain_r2': ('ad', False, 0., False, 0., 2, True), 'plain_e0': ('ad', False, 0., False, 0., 0, False),
                     'scaled': ('ad', False, 0., True, 1.e-3, 0, True), 'eig': ('ad', True, diffterm, False, 0., 0, True),
                     'eig_scaled': ('ad', True, diffterm, True, 1.e-3, 0, True),
                     'na': ('na', False, 0., False, 0., 0, True), 'ns': ('ns', False, 0., False, 0., 0, True)}
        if ns > 20:  # the larger mechanism: a subset, to keep the fixture small
            jac_cases = {k: jac_cases[k] for k in ('plain_r1', 'eig_scaled', 'ns')}
        for jk, (hk, eig, dt, sc, pf, ropt, ef) in jac_cases.items():
            adb, a1, a2, a3, a4, scaled = heat[hk]
            v = np.zeros(nel)
            e = np.zeros(nzi * ns)
            g.flamelet_jacobian(st, F._pressure, F._state_oxy, F._state_fuel, adb, a1, a2, a3, a4, nzi, cma, csb, csp,
                                mc, nc, chi, eig, dt, sc, pf, ropt, 0, ef, True, scaled, e, v)
            out[pre + f'flm_jac_{jk}'] = v
            if eig:
                out[pre + f'flm_expeig_{jk}'] = e
        out[pre + 'flm_diffterm'] = np.array(diffterm)
        print('dropin', name, 'nzi', nzi)
    # module-level block algebra on seeded block-diagonally dominant BTDDOD matrices
    for nb, bs in ((7, 5), (3, 53), (1, 3), (2, 11)):
        rng = np.random.default_rng(1000 * nb + bs)
        nv = bs * (nb * bs + 2 * (nb - 1))
        A = rng.standard_normal(nv)
        for i in range(nb):
            A[i * bs * bs: (i + 1) * bs * bs: bs + 1] += 3. * bs
        x = rng.standard_normal(nb * bs)
        pre = f'bt{nb}x{bs}_'
        out[pre + 'A'] = A
        out[pre + 'x'] = x
        y = np.zeros(nb * bs)
        if nb > 1:  # with one block the reference adds both end couplings from outside its arrays
            G.py_btddod_full_matvec(A, x, nb, bs, y)
            out[pre + 'full_matvec'] = y.copy()
        G.py_btddod_blockdiag_matvec(A, x, nb, bs, y)
        out[pre + 'blockdiag_matvec'] = y.copy()
        piv = np.zeros(nb * bs, dtype=np.int32)
        fac = np.zeros(nb * bs * bs)
        G.py_btddod_blockdiag_factorize(A, nb, bs, piv, fac)
        G.py_btddod_blockdiag_solve(piv, fac, x, nb, bs, y)
        out[pre + 'blockdiag_solve'] = y.copy()
        G.py_btddod_lowerfulltriangle_solve(piv, fac, A, x, nb, bs, y)
        out[pre + 'lower_solve'] = y.copy()
        G.py_btddod_upperfulltriangle_solve(piv, fac, A, x, nb, bs, y)
        out[pre + 'upper_solve'] = y.copy()
        Af = A.copy()
        lv = np.zeros(nb * bs * bs)
        pv = np.zeros(nv, dtype=np.int32)
        G.py_btddod_full_factorize(Af, nb, bs, lv, pv)
        G.py_btddod_full_solve(Af, lv, pv, x, nb, bs, y)
        out[pre + 'full_solve'] = y.copy()
        B = rng.standard_normal(nb * bs * bs)
        out[pre + 'B'] = B
        As = A.copy()
        G.py_btddod_scale_and_add_scaled_block_diagonal(As, 0.7, B, -1.3, nb, bs)
        out[pre + 'scaled_block'] = As
        d = rng.standard_normal(nb * bs)
        out[pre + 'd'] = d
        As = A.copy()
        G.py_btddod_scale_and_add_diagonal(As, -1., d, 2.5, nb, bs)
        out[pre + 'scaled_diag'] = As
    np.savez_compressed(os.path.join(HERE, 'dropin_ref.npz'), **out)


def libraries():
    import shutil
    for name in ('adiabatic_slfm', 'nonadiabatic_defect_burke_schumann'):
        shutil.copyfile(os.path.join(REF, 'tests', 'tabulation', name, 'gold.pkl'),
                        os.path.join(HERE, f'reference_{name}_gold.pkl'))


if __name__ == '__main__':
    args = sys.argv[1:]
    if '--reference' in args:
        i = args.index('--reference')
        os.environ['SPITFIRE_REFERENCE'] = args[i + 1]
        del args[i:i + 2]
    REF = os.environ.get('SPITFIRE_REFERENCE')
    if not REF or not os.path.isdir(os.path.join(REF, 'tests', 'test_mechanisms')):
        sys.exit('give the reference checkout: --reference PATH (or set SPITFIRE_REFERENCE)')
    MECHS = os.path.join(REF, 'tests', 'test_mechanisms')
    what = args or ['kernels', 'ignition', 'gold', 'flamelets']
    if 'flamelets' in what:
        slfm_gold()
        flamelets()
    if 'gold' in what:
        gold()
    if 'kernels' in what:
        kernels()
    if 'ignition' in what:
        ignition()
    if 'open' in what:
        open_kernels()
    if 'nonadiabatic' in what:
        nonadiabatic()
    if 'transient' in what:
        transient()
    if 'structure' in what:
        structure()
    if 'unstrained' in what:
        unstrained()
    if 'dropin' in what:
        dropin()
    if 'libraries' in what:
        libraries()
