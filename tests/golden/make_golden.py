"""Generate the golden fixtures of tests/golden from the reference Spitfire itself.

Runs only where the reference sources exist (this needs the reference Griffon built by `make -C oracle ref` and
the reference's Python modules, loaded by oracle/ref_harness.py). The fixtures pin the oracle:

  kernels_<mech>.npz   seeded states and the reference Griffon's production rates, rate sensitivities (options
                       0, 1, 2) and isochoric / isobaric reactor right-hand sides and Jacobians
  ignition_ref.json    ignition delays, accepted-step counts and final temperatures from the reference
                       HomogeneousReactor.compute_ignition_delay (reference odesolve + ESDIRK64 + Newton + PI)
  h2_mech_data.json    the Cantera-converted mech_data embedded in tests/tabulation/adiabatic_slfm/gold.pkl
  closed_reactor_gold.npz  the reference's stored closed-reactor trajectories (tests/reactor/closed_reactors/gold.pkl)

Usage:  python tests/golden/make_golden.py [kernels] [ignition] [gold]
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
REF = os.environ.get('SPITFIRE_REFERENCE', '/root/reference')
MECHS = os.path.join(REF, 'tests', 'test_mechanisms')


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


if __name__ == '__main__':
    what = sys.argv[1:] or ['kernels', 'ignition', 'gold']
    if 'gold' in what:
        gold()
    if 'kernels' in what:
        kernels()
    if 'ignition' in what:
        ignition()
