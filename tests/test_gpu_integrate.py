"""GPU batched ESDIRK64 integration against the reference's own ignition delays (tests/golden/ignition_ref.json,
made by the reference HomogeneousReactor) and against the oracle integrator.

Bars: ignition delay within 1e-6 relative of the reference and of the oracle; accepted-step counts equal. The
FP32-LU + FP64-refinement variant is compared with the all-FP64 result (its error is reported, bound 1e-4).
"""
import json
import os

import numpy as np
import pytest

from helpers import pair

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
CASES = json.load(open(os.path.join(GOLD, 'ignition_ref.json')))


def _q0(spec, case):
    Y = np.array(case['Y0'])
    if case['configuration'] == 'isobaric':
        return np.hstack([[case['T0']], Y[:-1]])
    rho = case['p'] / (Y / spec.molecular_weights).sum() / (8314.46261815324 * case['T0'])
    return np.hstack([[rho, case['T0']], Y[:-1]])


@pytest.mark.parametrize('group', sorted({(c['mechanism'], c['configuration']) for c in CASES}))
def test_ignition_delays_match_reference(cuda, group):
    from spitfire_gb300.reactors import BatchIntegrator
    mech, conf = group
    cases = [c for c in CASES if (c['mechanism'], c['configuration']) == group]
    spec, og = pair(mech)
    q0 = np.array([_q0(spec, c) for c in cases])
    pres = np.array([c['p'] for c in cases])
    bi = BatchIntegrator(spec, conf, pressure=pres[0])
    kw = dict(pressures=pres) if conf == 'isobaric' else {}
    if conf == 'isochoric':
        assert np.allclose(pres, pres[0])
    out = bi.run(q0, delta_temperature_ignition=400., **kw)
    tau = out['t'].cpu().numpy()
    counts = out['counts'].cpu().numpy()
    status = out['status'].cpu().numpy()
    for i, c in enumerate(cases):
        assert status[i] == 2, (c, status[i])
        assert abs(tau[i] - c['tau']) / c['tau'] <= 1e-6, (c, tau[i])
        assert counts[i, 0] == c['steps'], (c, counts[i])
    assert spec.griffon.device_status() == 0


def test_batched_ignition_matches_oracle(cuda):
    """16 isobaric GRI-3.0 reactors from the batched-ignition distribution (T0 900-1500 K, phi 0.5-2, p 1-20 atm)
    against the oracle integrator, reactor by reactor."""
    import integrate as I
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.reactors import BatchIntegrator
    spec, og = pair('methane-gri30')
    d = W.ignition_batch(spec, 16, seed=77, T_range=(1050., 1500.))
    bi = BatchIntegrator(spec, 'isobaric')
    out = bi.run(d['q0'], pressures=d['p'], delta_temperature_ignition=400., stop_at_time=0.1)
    tau = out['t'].cpu().numpy()
    ti = out['t_interp'].cpu().numpy()
    st = out['status'].cpu().numpy()
    cnt = out['counts'].cpu().numpy()
    for i in range(16):
        prob = I.ReactorProblem(og, 'isobaric', pressure=d['p'][i])
        r = I.integrate(prob, d['q0'][i], delta_temperature_ignition=400., stop_at_time=0.1)
        assert st[i] == r['status'], i
        assert cnt[i, 0] == r['steps'], (i, cnt[i], r['steps'])
        assert abs(tau[i] - r['t']) / r['t'] <= 1e-6, (i, tau[i], r['t'])
        # the Hermite-interpolated delay: the oracle's, and inside the crossing step (no later than its end)
        if r['t_interp'] is None:
            assert np.isnan(ti[i]), i
        else:
            assert abs(ti[i] - r['t_interp']) / r['t_interp'] <= 1e-6, (i, ti[i], r['t_interp'])
            assert ti[i] <= tau[i] * (1. + 1e-12), i


def test_fp32_lu_variant_error_is_small(cuda):
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.reactors import BatchIntegrator
    spec, og = pair('methane-gri30')
    d = W.ignition_batch(spec, 32, seed=78, T_range=(1100., 1500.))
    o64 = BatchIntegrator(spec, 'isobaric').run(d['q0'], pressures=d['p'], delta_temperature_ignition=400.,
                                                stop_at_time=0.1)
    o32 = BatchIntegrator(spec, 'isobaric', linear_precision=1, refine_sweeps=2).run(
        d['q0'], pressures=d['p'], delta_temperature_ignition=400., stop_at_time=0.1)
    t64, t32 = o64['t'].cpu().numpy(), o32['t'].cpu().numpy()
    rel = np.abs(t32 - t64) / t64
    print('FP32-LU + 2 FP64 refinement sweeps: max rel. ignition-delay error vs FP64 LU %.2e' % rel.max())
    assert rel.max() <= 1e-4


def test_graph_replay_and_drop_in_reactor(cuda):
    import torch
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.mechanism import Stream
    from spitfire_gb300.reactors import BatchIntegrator, HomogeneousReactor
    spec, og = pair('h2-burke')
    c = [c for c in CASES if c['mechanism'] == 'h2-burke' and c['configuration'] == 'isobaric'][0]
    mix = Stream(spec, c['T0'], c['p'], np.array(c['Y0']))
    r = HomogeneousReactor(spec, mix, 'isobaric', 'adiabatic', 'closed')
    tau = r.compute_ignition_delay()
    assert abs(tau - c['tau']) / c['tau'] <= 1e-6
    assert r.last_counts['steps'] == c['steps']
    q0 = np.repeat(_q0(spec, c)[None, :], 64, axis=0)
    bi = BatchIntegrator(spec, 'isobaric', pressure=c['p'])
    out = bi.run(q0, graph=True, delta_temperature_ignition=400.)
    torch.cuda.synchronize()
    t1 = out['t'].clone()
    bi.replay()
    torch.cuda.synchronize()
    assert torch.equal(t1, bi._graph[3]['t'])
    assert abs(float(t1[0]) - c['tau']) / c['tau'] <= 1e-6


def test_autotuned_shapes_do_not_change_results(cuda):
    """The autotuner's candidates (lanes per state of the Jacobian kernel; integrator scratch placement and warps
    per block) give bit-identical results (the tuner itself checks this), and the chosen shapes are applied."""
    from spitfire_gb300 import autotune as AT
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.reactors import BatchIntegrator
    spec, og = pair('methane-gri30')
    d = W.gri_states(spec, 2048, seed=31)
    res = AT.tune_chemistry(spec, W.isochoric_state(d), kinds=('rhs', 'jac'))
    assert AT.get_tuning(spec, 'group_jac') == res['group_jac'][0]
    b = W.ignition_batch(spec, 256, seed=32, T_range=(1200., 1500.))
    bi = BatchIntegrator(spec, 'isobaric')
    best, times = AT.tune_integrator(bi, b['q0'], pressures=b['p'], delta_temperature_ignition=400.,
                                     stop_at_time=0.1)
    assert (AT.get_tuning(spec, 'integrate_scratch'), AT.get_tuning(spec, 'integrate_warps')) == best
    assert len(times) >= 2
    out = bi.run(b['q0'], pressures=b['p'], delta_temperature_ignition=400., stop_at_time=0.1)
    import integrate as I
    for i in range(0, 256, 64):
        r = I.integrate(I.ReactorProblem(og, 'isobaric', pressure=b['p'][i]), b['q0'][i],
                        delta_temperature_ignition=400., stop_at_time=0.1)
        assert abs(out['t'][i].item() - r['t']) / r['t'] <= 1e-6
    for k in AT.KNOBS:
        AT.set_tuning(spec, k, 0)


def _h2_air_mix(spec, T):
    air = spec.stream(stp_air=True)
    fuel = spec.stream('X', 'H2:1')
    mix = spec.mix_for_equivalence_ratio(1.0, fuel, air)
    mix.TP = T, 101325.
    return mix


@pytest.mark.parametrize('key', ['cp_adiabatic', 'cp_isothermal', 'cv_adiabatic', 'cv_isothermal'])
def test_drop_in_reactor_trajectories_match_closed_gold(cuda, key):
    """tests/reactor/closed_reactors: HomogeneousReactor(...).integrate_to_steady() for the four closed reactors,
    every accepted step against the reference's stored trajectory under its own test's tolerances (rtol 1e-4,
    atol 1e-8 on t, T and Y) and step for step."""
    from spitfire_gb300.reactors import HomogeneousReactor
    g = np.load(os.path.join(GOLD, 'closed_reactor_gold.npz'))
    spec, og = pair('h2-burke')
    conf = 'isobaric' if key.startswith('cp') else 'isochoric'
    heat = key.split('_')[1]
    r = HomogeneousReactor(spec, _h2_air_mix(spec, 1200.), conf, heat, 'closed')
    out = r.integrate_to_steady()
    t, T = out.time_values, out['temperature']
    Y = np.array([out['mass fraction ' + s] for s in spec.species_names])
    assert t.size == g[key + '_t'].size, (t.size, g[key + '_t'].size)
    np.testing.assert_allclose(t, g[key + '_t'], rtol=1e-4, atol=1e-8)
    np.testing.assert_allclose(T, g[key + '_T'], rtol=1e-4, atol=1e-8)
    np.testing.assert_allclose(Y, g[key + '_Y'], rtol=1e-4, atol=1e-8)


def test_open_reactor_oscillating_feed_matches_gold(cuda):
    """tests/reactor/oscillating_feed_temperature: an open isobaric H2/air reactor (mixing time 1e-5 s) whose feed
    temperature is 800 + 400 sin(2 pi 10 t), integrated to 0.1 s through the drop-in reactor; every step against
    the reference's stored trajectory (rtol 1e-3, atol 1e-8, the reference test's tolerances) and the step count
    against the oracle's."""
    import integrate as I
    from spitfire_gb300.reactors import HomogeneousReactor
    from test_oracle_golden import oscillating_feed_case
    g = np.load(os.path.join(GOLD, 'open_reactor_gold.npz'))
    spec, og = pair('h2-burke')
    mix, feed_T = oscillating_feed_case(spec)
    feed = spec.copy_stream(mix)
    r = HomogeneousReactor(spec, mix, configuration='isobaric', heat_transfer='adiabatic', mass_transfer='open',
                           mixing_tau=1.e-5, feed_temperature=feed_T, feed_mass_fractions=feed.Y)
    out = r.integrate_to_time(0.1, transient_tolerance=1.e-10, write_log=False, log_rate=200)
    t, T = out.time_values, out['temperature']
    Y = np.array([out['mass fraction ' + s] for s in spec.species_names])
    np.testing.assert_allclose(t, g['t'], rtol=1e-3, atol=1e-8)
    np.testing.assert_allclose(T, g['T'], rtol=1e-3, atol=1e-8)
    np.testing.assert_allclose(Y, g['Y'], rtol=1e-3, atol=1e-8)
    Y0 = np.array(mix.Y)
    ro = I.integrate(I.OpenReactorProblem(og, 'isobaric', feed_T, Y0, 1.e-5), np.hstack([[mix.T], Y0[:-1]]),
                     stop_at_time=0.1)
    assert abs(r.last_counts['steps'] - ro['steps']) <= 2, (r.last_counts, ro['steps'])


@pytest.mark.parametrize('configuration', ['isobaric', 'isochoric'])
@pytest.mark.parametrize('heat', ['adiabatic', 'diathermal'])
def test_open_reactor_batch_matches_oracle(cuda, configuration, heat):
    """A batch of open GRI-3.0 reactors with a constant feed (and, diathermal, convection and radiation) against
    the oracle integrator reactor by reactor: status and accepted steps equal, final state within 1e-6."""
    import integrate as I
    import oracle as orc
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.reactors import BatchIntegrator
    spec, og = pair('methane-gri30')
    n = 6
    d = W.ignition_batch(spec, n, seed=91, T_range=(1100., 1400.))
    ns = spec.n_species
    yin = np.array(d['q0'][0, 1:].tolist() + [1. - d['q0'][0, 1:].sum()])
    Tin, tau = 900., 2.e-3
    q0 = d['q0']
    if configuration == 'isochoric':
        mw = spec.molecular_weights
        Yf = np.hstack([q0[:, 1:], 1. - q0[:, 1:].sum(1, keepdims=True)])
        rho = 101325. / (8314.46261815324 * q0[:, 0] * (Yf / mw).sum(1))
        q0 = np.hstack([rho[:, None], q0])
    rho_in = 0.4
    dia = dict(convection_temperature=500., radiation_temperature=600., convection_coefficient=20.,
               radiative_emissivity=0.5, surface_area_to_volume=30.) if heat == 'diathermal' else {}
    bi = BatchIntegrator(spec, configuration, heat, pressure=101325., mass_transfer='open', mixing_tau=tau,
                         feed_temperature=Tin, feed_mass_fractions=yin, feed_density=rho_in, **dia)
    out = bi.run(q0, stop_at_time=5.e-3)
    qg, st, cnt = out['q'].cpu().numpy(), out['status'].cpu().numpy(), out['counts'].cpu().numpy()
    for i in range(n):
        prob = I.OpenReactorProblem(og, configuration, Tin, yin, tau, pressure=101325.,
                                    heat='diathermal' if dia else 'adiabatic', feed_density=rho_in)
        if dia:
            prob.P.fluid_temperature, prob.P.surface_temperature = 500., 600.
            prob.P.h_convection, prob.P.eps_radiation, prob.P.surface_area_to_volume = 20., 0.5, 30.
        r = I.integrate(prob, q0[i], stop_at_time=5.e-3)
        assert st[i] == r['status'], i
        assert cnt[i, 0] == r['steps'], (i, cnt[i], r['steps'])
        assert np.max(np.abs(qg[i] - r['state']) / np.maximum(np.abs(r['state']), 1e-3)) <= 1e-6, i
    assert spec.griffon.device_status() == 0
    del orc, ns


def test_plain_integrator_form_matches_reference_and_oracle(cuda):
    """The plain single-state GPU form of the integrator (one thread per reactor): the reference's H2 ignition delays
    with their step counts, and GRI reactors of the batched-ignition distribution against the oracle."""
    import integrate as I
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.reactors import BatchIntegrator
    for conf in ('isobaric', 'isochoric'):
        cases = [c for c in CASES if c['mechanism'] == 'h2-burke' and c['configuration'] == conf]
        spec, og = pair('h2-burke')
        q0 = np.array([_q0(spec, c) for c in cases])
        pres = np.array([c['p'] for c in cases])
        bi = BatchIntegrator(spec, conf, pressure=pres[0])
        out = bi.run_plain(q0, delta_temperature_ignition=400., **(dict(pressures=pres) if conf == 'isobaric' else {}))
        tau, cnt, st = out['t'].cpu().numpy(), out['counts'].cpu().numpy(), out['status'].cpu().numpy()
        for i, c in enumerate(cases):
            assert st[i] == 2 and cnt[i, 0] == c['steps'], (c, st[i], cnt[i])
            assert abs(tau[i] - c['tau']) / c['tau'] <= 1e-6, (c, tau[i])
    spec, og = pair('methane-gri30')
    d = W.ignition_batch(spec, 4, seed=77, T_range=(1300., 1500.))
    out = BatchIntegrator(spec, 'isobaric').run_plain(d['q0'], pressures=d['p'], delta_temperature_ignition=400.,
                                                      stop_at_time=0.1)
    tau, cnt = out['t'].cpu().numpy(), out['counts'].cpu().numpy()
    for i in range(4):
        r = I.integrate(I.ReactorProblem(og, 'isobaric', pressure=d['p'][i]), d['q0'][i],
                        delta_temperature_ignition=400., stop_at_time=0.1)
        assert cnt[i, 0] == r['steps'], (i, cnt[i], r['steps'])
        assert abs(tau[i] - r['t']) / r['t'] <= 1e-6, (i, tau[i], r['t'])
    assert spec.griffon.device_status() == 0


def _time_dependent_params(spec, yin):
    """Functions of time for every parameter the reference lets vary (reactors.py:253-341)."""
    yn2 = np.zeros(spec.n_species)
    yn2[spec.species_index('N2')] = 1.
    w = 2. * np.pi
    return dict(feed_temperature=lambda t: 900. + 200. * np.sin(w * t / 2.e-3),
                mixing_tau=lambda t: 2.e-3 * (1. + 0.5 * np.sin(w * t / 3.e-3)),
                feed_mass_fractions=lambda t: (1. - 0.25 * (1. - np.cos(w * t / 4.e-3))) * yin +
                0.25 * (1. - np.cos(w * t / 4.e-3)) * yn2,
                convection_temperature=lambda t: 500. + 2.e4 * t,
                convection_coefficient=lambda t: 20. * (1. + 200. * t),
                radiation_temperature=lambda t: 600. - 50. * np.sin(w * t / 2.5e-3),
                radiative_emissivity=lambda t: 0.5 + 0.2 * np.sin(w * t / 3.5e-3))


@pytest.mark.parametrize('configuration', ['isobaric', 'isochoric'])
def test_time_dependent_parameters_match_oracle(cuda, configuration):
    """Open, diathermal GRI-3.0 reactors whose feed temperature, feed mass fractions, mixing time, convection and
    radiation temperatures, convection coefficient and emissivity all vary in time (and, isochoric, whose feed
    density is a function the reference evaluates at t = 0 only): the batched integrator against the oracle's
    restatement of the reference's closures, reactor by reactor (status and accepted steps equal, final state
    within 1e-6), and the drop-in HomogeneousReactor with the same functions."""
    import integrate as I
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.reactors import BatchIntegrator, HomogeneousReactor
    spec, og = pair('methane-gri30')
    n = 4
    d = W.ignition_batch(spec, n, seed=93, T_range=(1150., 1400.))
    yin = np.array(d['q0'][0, 1:].tolist() + [1. - d['q0'][0, 1:].sum()])
    q0 = d['q0']
    if configuration == 'isochoric':
        mw = spec.molecular_weights
        Yf = np.hstack([q0[:, 1:], 1. - q0[:, 1:].sum(1, keepdims=True)])
        rho = 101325. / (8314.46261815324 * q0[:, 0] * (Yf / mw).sum(1))
        q0 = np.hstack([rho[:, None], q0])
    fn = _time_dependent_params(spec, yin)
    rho_in = lambda t: 0.4 + 100. * t  # evaluated at t = 0 only, as the reference does
    bi = BatchIntegrator(spec, configuration, 'diathermal', pressure=101325., mass_transfer='open',
                         feed_density=rho_in, surface_area_to_volume=30., **fn)
    out = bi.run(q0, stop_at_time=5.e-3)
    qg, st, cnt = out['q'].cpu().numpy(), out['status'].cpu().numpy(), out['counts'].cpu().numpy()
    for i in range(n):
        prob = I.OpenReactorProblem(og, configuration, fn['feed_temperature'], fn['feed_mass_fractions'],
                                    fn['mixing_tau'], pressure=101325., heat='diathermal', feed_density=rho_in,
                                    convection_temperature=fn['convection_temperature'],
                                    radiation_temperature=fn['radiation_temperature'],
                                    convection_coefficient=fn['convection_coefficient'],
                                    radiative_emissivity=fn['radiative_emissivity'], surface_area_to_volume=30.)
        r = I.integrate(prob, q0[i], stop_at_time=5.e-3)
        assert st[i] == r['status'], i
        assert cnt[i, 0] == r['steps'], (i, cnt[i], r['steps'])
        assert np.max(np.abs(qg[i] - r['state']) / np.maximum(np.abs(r['state']), 1e-3)) <= 1e-6, i
    # the drop-in reactor: the same functions through HomogeneousReactor, against the batch's first reactor
    mix = spec.stream('TPY', (float(d['T0'][0]), 101325., {s: float(v) for s, v in zip(spec.species_names, d['Y'][0])}))
    hr = HomogeneousReactor(spec, mix, configuration=configuration, heat_transfer='diathermal',
                            mass_transfer='open', feed_density=rho_in,
                            shape_dimension_dict={'shape': 'cube', 'char. length': 0.2}, **fn)  # 30 1/m
    lib = hr.integrate_to_time(5.e-3)
    assert hr.last_counts['steps'] == cnt[0, 0], (hr.last_counts, cnt[0])
    Ti = 1 if configuration == 'isochoric' else 0
    assert abs(lib['temperature'][-1] - qg[0, Ti]) / qg[0, Ti] < 1e-9
    assert spec.griffon.device_status() == 0
