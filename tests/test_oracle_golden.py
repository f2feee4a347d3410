"""The oracle (CPU restatement) pinned against golden vectors produced by the reference Spitfire itself
(tests/golden/make_golden.py): loader, Griffon kernels, and ESDIRK64 reactor integration."""
import json
import os

import numpy as np
import pytest

from helpers import colmajor, pair, rownorm_err

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def test_loader_matches_cantera_converted_mech_data():
    """The project YAML loader reproduces the mech_data Cantera produced for h2-burke (embedded in the
    reference's tests/tabulation/adiabatic_slfm/gold.pkl)."""
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    gold = json.load(open(os.path.join(GOLD, 'h2_mech_data.json')))
    spec = ChemicalMechanismSpec.bundled('h2-burke')
    md = json.loads(json.dumps(spec.mech_data, default=float))
    for k in ('ref_pressure', 'ref_temperature', 'elements', 'gas_constant', 'element_mw_map'):
        assert md[k] == gold[k], k
    assert list(md['species']) == list(gold['species'])
    for s in gold['species']:
        assert md['species'][s]['atom_map'] == gold['species'][s]['atom_map']
        assert list(md['species'][s]['cp']) == list(gold['species'][s]['cp'])
    assert len(md['reactions']) == len(gold['reactions'])
    for a, b in zip(md['reactions'], gold['reactions']):
        assert list(a) == list(b)


@pytest.mark.parametrize('name', ['h2-burke', 'methane-gri30', 'reaction-test'])
def test_oracle_kernels_match_reference(name):
    import oracle as orc
    from spitfire_gb300._desc import reactor_params
    g = np.load(os.path.join(GOLD, f'kernels_{name}.npz'))
    spec, og = pair(name)
    ns = spec.n_species
    w = og.production_rates_batch(g['T'], g['rho'], g['Y'])
    assert rownorm_err(w, g['w']) <= 1e-13
    for opt in range(3):
        _, S = og.rates_sens_batch(g['rho'], g['T'], g['Y'], opt)
        assert rownorm_err(colmajor(S, ns + 1)[:, :ns], colmajor(g['S'][opt], ns + 1)[:, :ns]) <= 1e-13, opt
    yin = np.zeros(ns)
    Piv = reactor_params('isochoric')
    Piv.inflow_Y = orc._p(yin)
    Pib = reactor_params('isobaric')
    Pib.inflow_Y = orc._p(yin)
    assert rownorm_err(og.reactor_rhs_batch(Piv, g['qiv']), g['rhs_iv']) <= 1e-13
    assert rownorm_err(og.reactor_rhs_batch(Pib, g['qib'], pressures=g['p']), g['rhs_ib']) <= 1e-13
    r, J = og.reactor_jac_batch(Piv, g['qiv'], 0)
    rb, Jb = og.reactor_jac_batch(Pib, g['qib'], 0, pressures=g['p'])
    assert rownorm_err(r, g['jac_rhs_iv']) <= 1e-13
    assert rownorm_err(rb, g['jac_rhs_ib']) <= 1e-13
    # temperature rows of the artificial reaction-test mechanism are pure cancellation (terms ~1e21, value ~1e-2)
    riv = slice(2, None) if name == 'reaction-test' else slice(0, None)
    rib = slice(1, None) if name == 'reaction-test' else slice(0, None)
    assert rownorm_err(colmajor(J, ns + 1)[:, riv], colmajor(g['Jiv'], ns + 1)[:, riv]) <= 1e-13
    assert rownorm_err(colmajor(Jb, ns)[:, rib], colmajor(g['Jib'], ns)[:, rib]) <= 1e-13


def _case_problem(case):
    import integrate as I
    name = case['mechanism']
    spec, og = pair(name)
    prob = I.ReactorProblem(og, case['configuration'], pressure=case['p'])
    Y = np.array(case['Y0'])
    T0 = case['T0']
    if case['configuration'] == 'isobaric':
        q0 = np.hstack([[T0], Y[:-1]])
    else:
        rho = case['p'] * (1. / (Y / spec.molecular_weights).sum()) / (8314.46261815324 * T0)
        q0 = np.hstack([[rho, T0], Y[:-1]])
    return prob, q0


CASES = json.load(open(os.path.join(GOLD, 'ignition_ref.json')))


@pytest.mark.parametrize('case', CASES, ids=[f"{c['mechanism']}-{c['configuration']}-{c['T0']:.0f}K-{c['phi']}"
                                             for c in CASES])
def test_oracle_ignition_matches_reference(case):
    import integrate as I
    prob, q0 = _case_problem(case)
    tau, r = I.ignition_delay(prob, q0)
    assert r['status'] == I.STATUS['ignited']
    assert r['steps'] == case['steps']
    assert abs(tau - case['tau']) / case['tau'] <= 1e-9


def test_oracle_closed_reactor_trajectory_matches_gold():
    """tests/reactor/closed_reactors/gold.pkl ('cp, adiabatic'): h2-burke, X = 2:1:3.74 H2:O2:N2, 1200 K, 1 atm,
    integrate_to_steady (steady tolerance 1e-6); the reference stored 517 steps. The reference's own test compares
    with rtol 1e-4 (tests/reactor/closed_reactors/test.py:26-28): the accepted-step sequence of adaptive ESDIRK
    moves by ~1e-5 when a Newton solve lands next to its 1e-12 tolerance and its iteration count flips under
    rounding-level differences (the reference run here differs from its own gold file by 1.9e-5 in time)."""
    import integrate as I
    g = np.load(os.path.join(GOLD, 'closed_reactor_gold.npz'))
    t, T, Y = g['cp_adiabatic_t'], g['cp_adiabatic_T'], g['cp_adiabatic_Y']
    spec, og = pair('h2-burke')
    prob = I.ReactorProblem(og, 'isobaric', pressure=101325.)
    q0 = np.hstack([[T[0]], Y[:-1, 0]])
    r = I.integrate(prob, q0, stop_at_steady=1e-6, save_each_step=True)
    assert r['steps'] == t.size - 1
    assert np.max(np.abs(r['times'] - t) / np.maximum(t, 1e-300)) <= 1e-4
    assert np.max(np.abs(r['states'][:, 0] - T) / T) <= 1e-4


def test_oracle_forward_sensitivity_matches_finite_differences():
    """The CPU forward sensitivity (test infrastructure for the adjoint) against central differences on a frozen
    step sequence, H2 isobaric reactor, all 54 parameters (normwise 1e-6 of the largest gradient)."""
    import integrate as I
    import oracle as orc
    import sensitivity as SE
    orc.set_threads(1)
    spec, og = pair('h2-burke')
    X = np.zeros(spec.n_species)
    X[spec.species_index('H2')], X[spec.species_index('O2')], X[spec.species_index('N2')] = 2., 1., 3.76
    Y = X * spec.molecular_weights
    Y /= Y.sum()
    q0 = np.hstack([1100., Y[:-1]])
    prob = I.ReactorProblem(og, 'isobaric', pressure=101325.)
    r = I.integrate(prob, q0, stop_at_time=1.e-4, save_each_step=True)
    dts = np.diff(r['times'])
    fs, st = SE.frozen_integrate(prob, q0, dts)
    pj = SE.ParamJacobian(spec, og, 'isobaric', 101325.)
    gT, gtau = SE.forward_sensitivity(prob, pj, q0, dts, st)
    fd = SE.fd_gradient(spec, 'isobaric', 101325., q0, dts, list(range(gT.size)))
    for g, f in ((gT, fd[0]), (gtau, fd[1])):
        for c in (0, 1):
            assert np.max(np.abs(g[c::2] - f[c::2])) / np.max(np.abs(g[c::2])) < 1e-6


def test_oracle_rate_parameter_sensitivity_matches_finite_differences():
    import copy
    import oracle as orc
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    spec, og = pair('methane-gri30')
    d = W.gri_states(spec, 4, seed=5)
    q, s = og.rate_param_sens_batch(d['T'], d['rho'], d['Y'])
    kinds = [r[0] for r in spec.mech_data['reactions']]
    picks = [i for i, k in enumerate(kinds) if k.startswith('Troe')][:4] + \
            [i for i, k in enumerate(kinds) if k.startswith('Lindemann')][:2] + [0, 100, 250]
    for r in picks:
        vals = []
        for sgn in (1., -1.):
            md = copy.deepcopy(spec.mech_data)
            t = list(md['reactions'][r])
            t[4] *= np.exp(sgn * 1e-6)
            md['reactions'][r] = tuple(t)
            sp2 = ChemicalMechanismSpec(mech_data=md)
            g2 = orc.OracleGriffon()
            sp2._populate_griffon(g2)
            vals.append(g2.rate_param_sens_batch(d['T'], d['rho'], d['Y'])[0][:, r])
        fd = (vals[0] - vals[1]) / 2e-6
        assert np.max(np.abs(fd - s[:, r]) / np.abs(s[:, r])) < 1e-7, (kinds[r], r)


OPEN_DIATHERMAL = (600., 900., 50., 0.3, 20.)  # Tc, Tr, h, eps, surface-to-volume (tests/golden/make_golden.py)


@pytest.mark.parametrize('name', ['h2-burke', 'methane-gri30'])
def test_oracle_open_reactor_kernels_match_reference(name):
    """Open (mass-exchange) reactor right-hand sides and Jacobians, isochoric and isobaric, each heat-transfer
    option, with a per-state feed (temperature, mass fractions, residence time, density)."""
    g = np.load(os.path.join(GOLD, f'open_kernels_{name}.npz'))
    spec, og = pair(name)
    ns = spec.n_species
    Tc, Tr, hc, eps, sov = OPEN_DIATHERMAL
    for heat, ho in (('adiabatic', 0), ('isothermal', 1), ('diathermal', 2)):
        for i in range(g['T'].size):
            feed = (g['Tin'][i], g['Yin'][i], g['tau'][i], Tc, Tr, hc, eps, sov, ho, True)
            r = np.zeros(ns + 1)
            rj, J = np.zeros(ns + 1), np.zeros((ns + 1) ** 2)
            og.reactor_rhs_isochoric(g['qiv'][i], g['rhoin'][i], *feed, r)
            og.reactor_jac_isochoric(g['qiv'][i], g['rhoin'][i], *feed, 0, rj, J)
            assert rownorm_err(r, g[f'{heat}_rhs_iv'][i]) <= 1e-13
            assert rownorm_err(rj, g[f'{heat}_jac_rhs_iv'][i]) <= 1e-13
            assert rownorm_err(colmajor(J, ns + 1), colmajor(g[f'{heat}_Jiv'][i], ns + 1)) <= 1e-13
            r = np.zeros(ns)
            rj, J = np.zeros(ns), np.zeros(ns * ns)
            og.reactor_rhs_isobaric(g['qib'][i], g['p'][i], *feed, r)
            og.reactor_jac_isobaric(g['qib'][i], g['p'][i], *feed, 0, 0, rj, J)
            assert rownorm_err(r, g[f'{heat}_rhs_ib'][i]) <= 1e-13
            assert rownorm_err(rj, g[f'{heat}_jac_rhs_ib'][i]) <= 1e-13
            assert rownorm_err(colmajor(J, ns), colmajor(g[f'{heat}_Jib'][i], ns)) <= 1e-13


def oscillating_feed_case(spec):
    """tests/reactor/oscillating_feed_temperature/rebless.py: h2-burke, stoichiometric H2/air (air = O2:N2 1:3.74
    at 300 K) at 800 K and 1 atm, isobaric adiabatic open reactor with mixing time 1e-5 s, feed = the initial
    mixture with temperature 800 + 400 sin(2 pi 10 t), integrated to t = 0.1 s."""
    air = spec.stream(stp_air=True)
    fuel = spec.stream('X', 'H2:1')
    mix = spec.mix_for_equivalence_ratio(1.0, fuel, air)
    mix.TP = 800., 101325.
    return mix, (lambda t: 800. + 400. * np.sin(2. * np.pi * 10. * t))


def test_oracle_open_reactor_trajectory_matches_gold():
    """The reference's oscillating-feed gold (1720 steps) under the reference test's own tolerances
    (rtol 1e-3, atol 1e-8 on t, T and Y; tests/reactor/oscillating_feed_temperature/test.py)."""
    import integrate as I
    g = np.load(os.path.join(GOLD, 'open_reactor_gold.npz'))
    spec, og = pair('h2-burke')
    mix, feed_T = oscillating_feed_case(spec)
    Y0 = np.array(mix.Y)
    prob = I.OpenReactorProblem(og, 'isobaric', feed_T, Y0, 1.e-5, pressure=101325.)
    q0 = np.hstack([[mix.T], Y0[:-1]])
    r = I.integrate(prob, q0, stop_at_time=0.1, save_each_step=True)
    assert r['times'].size == g['t'].size
    np.testing.assert_allclose(r['times'], g['t'], rtol=1e-3, atol=1e-8)
    np.testing.assert_allclose(r['states'][:, 0], g['T'], rtol=1e-3, atol=1e-8)
    Y = np.vstack([r['states'][:, 1:].T, 1. - r['states'][:, 1:].sum(1)])
    np.testing.assert_allclose(Y, g['Y'], rtol=1e-3, atol=1e-8)
