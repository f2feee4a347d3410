"""CPU: the flamelet oracle and the flamelet setup logic against the reference Flamelet's own outputs
(tests/golden/flamelet_ref.npz, made by tests/golden/make_golden.py from the reference flamelet.py over the
reference Griffon built unmodified).

Pins (1) the grid, dissipation-rate profile and boundary states of spitfire_gb300.flamelet.FlameletSetup,
(2) the oracle's flamelet residual, BTDDOD Jacobian (plain, scaled, enthalpy-flux on/off) and block-Thomas
algebra, (3) the eigenvalue bound semantics (numpy eigvals of the chemistry block vs Griffon's dgeev path), and
(4) the oracle's restatement of steady_solve_newton / steady_solve_psitc: same convergence, same iteration counts,
same converged profiles as the reference solvers.
"""
import numpy as np
import pytest

import flamelet_cases as FC
from helpers import pair

CASES = [c[0] for c in FC.FLAMELET_CASES]


def _op(name, **kw):
    import flamelet_steady as FS
    d = FC.golden()
    spec, og = pair(FC.BUNDLED[name])
    op = FS.FlameletOperator(og, d[name + '_z'], d[name + '_chi'], d[name + '_oxy'], d[name + '_fuel'], **kw)
    return d, spec, og, op


@pytest.mark.parametrize('name', CASES)
def test_setup_matches_reference_flamelet(name):
    from spitfire_gb300.flamelet import FlameletSetup, FlameletSpec
    d = FC.golden()
    spec, _ = pair(FC.BUNDLED[name])
    oxy, fuel, kw = FC.flamelet_case_setup(spec, FC.case(name))
    s = FlameletSetup(FlameletSpec(mech_spec=spec, initial_condition='Burke-Schumann', **kw))
    assert np.allclose(s.z, d[name + '_z'], rtol=1e-14, atol=1e-15)
    assert np.allclose(s.x, d[name + '_chi'], rtol=1e-12, atol=1e-14)
    assert np.allclose(s.state_oxy, d[name + '_oxy'], rtol=1e-14, atol=1e-16)
    assert np.allclose(s.state_fuel, d[name + '_fuel'], rtol=1e-14, atol=1e-16)
    assert np.allclose(s.initial_state, d[name + '_ic'], rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize('name', CASES)
def test_oracle_flamelet_kernels_match_reference(name):
    d, spec, og, op = _op(name)
    st = d[name + '_state']
    ns = op.ns
    for ef in (0, 1):
        for vc in (0, 1):
            assert FC.vec_err(op.rhs(st, eflux=ef, vcp=vc), d[name + f'_rhs_e{ef}v{vc}'], ns) < 1e-12, (ef, vc)
        assert FC.btddod_row_err(op.jac(st, eflux=ef), d[name + f'_jac_e{ef}'], op.nzi, ns) < 1e-12, ef
    assert FC.btddod_row_err(op.jac(st, scale_and_offset=True, prefactor=1.e-3), d[name + '_jac_scaled'], op.nzi,
                             ns) < 1e-12
    assert FC.btddod_row_err(op.jac(st), d[name + '_jac_eig'], op.nzi, ns) < 1e-12


@pytest.mark.parametrize('name', CASES)
def test_eigenvalue_bound_matches_reference(name):
    d, spec, og, op = _op(name)
    e = op.expeig(d[name + '_state'], float(d[name + '_diffterm']))
    ref = d[name + '_expeig']
    assert np.all((e > 0) == (ref > 0))
    assert np.max(np.abs(e - ref) / np.maximum(np.abs(ref), 1.)) < 1e-8


@pytest.mark.parametrize('name', CASES)
def test_oracle_block_thomas_matches_reference(name):
    import oracle as orc
    d, spec, og, op = _op(name)
    nzi, ns = op.nzi, op.ns
    J = -d[name + '_jac_e1']
    y = orc.btddod_full_matvec(J, d[name + '_matvec_b'], nzi, ns)
    assert FC.vec_err(y, d[name + '_matvec_y'], ns) < 1e-13
    x = orc.btddod_full_solve(*orc.btddod_full_factorize(J, nzi, ns), d[name + '_matvec_b'], nzi, ns)
    ref = d[name + '_solve_x']
    assert np.max(np.abs(x - ref)) / np.max(np.abs(ref)) < 1e-9
    # componentwise backward error of the reference's own solution under the oracle's matvec
    b = d[name + '_matvec_b']
    r = orc.btddod_full_matvec(J, ref, nzi, ns) - b
    scale = orc.btddod_full_matvec(np.abs(J), np.abs(ref), nzi, ns) + np.abs(b)
    assert np.max(np.abs(r) / scale) < 1e-10


@pytest.mark.parametrize('name', CASES)
def test_oracle_steady_solvers_match_reference(name):
    import flamelet_steady as FS
    d, spec, og, op = _op(name)
    ic = d[name + '_ic']
    s, it, conv = FS.steady_solve_newton(op, ic, tolerance=1.e-6, max_iterations=38)
    assert conv == bool(d[name + '_newton_conv'])
    s, it, conv, mds = FS.steady_solve_psitc(op, ic, tolerance=1.e-6, max_iterations=400)
    assert conv and bool(d[name + '_psitc_conv'])
    assert it == int(d[name + '_psitc_iters'])
    ref = d[name + '_psitc_state']
    assert FC.vec_err(s, ref, op.ns) < 1e-6
    assert np.max(np.abs(s[::op.ns] - ref[::op.ns]) / ref[::op.ns]) < 1e-8


@pytest.mark.parametrize('name', CASES)
def test_oracle_continuation_newton_matches_reference(name):
    import flamelet_steady as FS
    from spitfire_gb300.flamelet import FlameletSetup, FlameletSpec
    d = FC.golden()
    spec, og = pair(FC.BUNDLED[name])
    oxy, fuel, kw = FC.flamelet_case_setup(spec, FC.case(name))
    kw['stoich_dissipation_rate'] *= 1.5
    s = FlameletSetup(FlameletSpec(mech_spec=spec, initial_condition=d[name + '_psitc_state'], **kw))
    op = FS.FlameletOperator(og, s.z, s.x, s.state_oxy, s.state_fuel)
    st, it, conv = FS.steady_solve_newton(op, s.initial_state, tolerance=1.e-6, max_iterations=38)
    assert conv and bool(d[name + '_cont_conv'])
    assert it == int(d[name + '_cont_iters'])
    ref = d[name + '_cont_state']
    assert np.max(np.abs(st[::op.ns] - ref[::op.ns]) / ref[::op.ns]) < 1e-8
    assert FC.vec_err(st, ref, op.ns) < 1e-6


def _slfm_inputs():
    d = np.load(FC.os.path.join(FC.GOLD, 'adiabatic_slfm_gold.npz'))
    spec, og = pair('h2-burke')
    air = spec.stream(stp_air=True)
    air.TP = 1200., 101325.
    fuel = spec.stream('TPY', (300., 101325., 'H2:1'))
    return d, spec, og, dict(mech_spec=spec, oxy_stream=air, fuel_stream=fuel, grid_points=34)


def test_oracle_slfm_continuation_matches_reference_gold():
    """The reference's adiabatic SLFM gold (tests/tabulation/adiabatic_slfm: h2-burke, air 1200 K / H2 300 K, 34
    points, chi_st = logspace(0, 1, 8)) rebuilt by the sequential continuation on the oracle solvers from a
    Burke-Schumann start (the reference starts from Cantera's HP equilibrium), within the reference test's own
    rtol = atol = 1e-6."""
    import flamelet_steady as FS
    from spitfire_gb300.flamelet import FlameletSetup, FlameletSpec, compute_dissipation_rate
    d, spec, og, kw = _slfm_inputs()
    assert str(d['dim0_name']) == 'mixture_fraction' and str(d['dim1_name']) == 'dissipation_rate_stoich'
    ic = 'Burke-Schumann'
    ns = spec.n_species
    chis = []
    for ix, chi in enumerate(np.logspace(0, 1, 8)):
        s = FlameletSetup(FlameletSpec(initial_condition=ic, stoich_dissipation_rate=chi, **kw))
        op = FS.FlameletOperator(og, s.z, s.x, s.state_oxy, s.state_fuel)
        st, how, it = FS.compute_steady_state(op, s.initial_state)
        assert st is not None
        T = np.hstack([s.state_oxy[0], st[::ns], s.state_fuel[0]])
        np.testing.assert_allclose(T, d['prop:temperature'][:, ix], rtol=1e-6, atol=1e-6)
        for k, name in enumerate(spec.species_names[:-1]):
            Y = np.hstack([s.state_oxy[1 + k], st[1 + k::ns], s.state_fuel[1 + k]])
            np.testing.assert_allclose(Y, d['prop:mass fraction ' + name][:, ix], rtol=1e-6, atol=1e-6)
        chis.append(compute_dissipation_rate(np.array([s.z_st]), s.max_dissipation_rate, s.form)[0])
        ic = st
    np.testing.assert_allclose(s.z, d['dim0_values'], rtol=1e-14)
    np.testing.assert_allclose(chis, d['dim1_values'], rtol=1e-12)


def _nonad_op(name, variant):
    import flamelet_steady as FS
    d = FC.golden()
    g = np.load(FC.GOLD + '/flamelet_nonad_ref.npz')
    spec, og = pair(FC.BUNDLED[name])
    v = f'{name}_{variant}_'
    heat = dict(T_conv=g[v + 'T_conv'], T_rad=g[v + 'T_rad'], h_conv=g[v + 'h_conv'], h_rad=g[v + 'h_rad'],
                scaled=variant == 'scaled')
    op = FS.FlameletOperator(og, d[name + '_z'], d[name + '_chi'], d[name + '_oxy'], d[name + '_fuel'],
                             heat_loss=heat)
    return g, v, op, spec


@pytest.mark.parametrize('name', CASES)
@pytest.mark.parametrize('variant', ['plain', 'scaled'])
def test_oracle_nonadiabatic_flamelet_kernels_match_reference(name, variant):
    """Heat-loss terms (convection and radiation per point; and scaled by the temperature range with the linear
    reference temperature profile and dissipation-scaled coefficients) against the reference Flamelet's
    _nonadiabatic_rhs / _nonadiabatic_jac (tests/golden/flamelet_nonad_ref.npz)."""
    g, v, op, spec = _nonad_op(name, variant)
    st = g[name + '_state']
    ns = op.ns
    assert FC.vec_err(op.rhs(st), g[v + 'rhs'], ns) < 1e-12
    assert FC.btddod_row_err(op.jac(st), g[v + 'jac'], op.nzi, ns) < 1e-12


@pytest.mark.parametrize('name', CASES)
@pytest.mark.parametrize('variant', ['plain', 'scaled'])
def test_nonadiabatic_setup_matches_reference(name, variant):
    """FlameletSetup's heat-loss arrays (flamelet.py:479-519) equal the reference Flamelet's."""
    from spitfire_gb300.flamelet import FlameletSetup, FlameletSpec
    g = np.load(FC.GOLD + '/flamelet_nonad_ref.npz')
    spec, _ = pair(FC.BUNDLED[name])
    oxy, fuel, kw = FC.flamelet_case_setup(spec, FC.case(name))
    v = f'{name}_{variant}_'
    if variant == 'plain':
        hk = dict(heat_transfer='nonadiabatic', convection_temperature=g[v + 'arg_convection_temperature'],
                  radiation_temperature=g[v + 'arg_radiation_temperature'],
                  convection_coefficient=g[v + 'arg_convection_coefficient'],
                  radiative_emissivity=g[v + 'arg_radiative_emissivity'])
    else:
        hk = dict(heat_transfer='nonadiabatic', scale_heat_loss_by_temp_range=True,
                  scale_convection_by_dissipation=True, use_linear_ref_temp_profile=True,
                  convection_coefficient=1.e7, radiative_emissivity=0.5)
    s = FlameletSetup(FlameletSpec(mech_spec=spec, initial_condition='Burke-Schumann', **dict(kw, **hk)))
    for a, k in ((s.T_conv, 'T_conv'), (s.T_rad, 'T_rad'), (s.h_conv, 'h_conv'), (s.h_rad, 'h_rad')):
        assert np.allclose(a, g[v + k], rtol=1e-13, atol=0.), k
    assert s.scale_heat_loss_by_temp_range == (variant == 'scaled')
