"""Host-side mechanism utilities (spitfire_gb300/mechanism.py) and reactor front-end logic on CPU: the mechanism API
basics of the reference's tests/mechanism/test_mechanisms_and_streams.py, pickling, the stream utilities around
stoichiometry, and HomogeneousReactor glue that needs no device."""
import pickle

import numpy as np
import pytest

from spitfire_gb300.mechanism import ChemicalMechanismSpec


def test_mechanism_simple_api_and_serialization():
    m = ChemicalMechanismSpec.bundled('h2-burke')
    for i, n in enumerate(m.species_names):
        assert m.species_index(n) == i
        assert m.molecular_weight(i) == m.molecular_weight(n)
    with pytest.raises(Exception):
        m.molecular_weight(list())
    m2 = pickle.loads(pickle.dumps(m))
    assert m2.mech_data['species'] == m.mech_data['species']
    assert m2.mech_data['reactions'] == m.mech_data['reactions']
    assert m2.n_species == m.n_species and m2.n_reactions == m.n_reactions


def test_mix_fuels_for_stoich_mixture_fraction():
    """Methane diluted with nitrogen to a stoichiometric mixture fraction of 0.2 with air (mechanism.py:724-757),
    and a target the two fuels cannot reach."""
    m = ChemicalMechanismSpec.bundled('methane-gri30')
    air = m.stream(stp_air=True)
    ch4 = m.stream('TPX', (300., 101325., 'CH4:1'))
    n2 = m.stream('TPX', (300., 101325., 'N2:1'))
    assert abs(m.stoich_mixture_fraction(ch4, air) - 0.0554) < 1e-3
    mix = m.mix_fuels_for_stoich_mixture_fraction(ch4, n2, 0.2, air)
    assert abs(m.stoich_mixture_fraction(mix, air) - 0.2) < 1e-12
    x = mix.X
    assert abs(x[m.species_index('CH4')] + x[m.species_index('N2')] - 1.) < 1e-12
    with pytest.raises(ValueError):
        m.mix_fuels_for_stoich_mixture_fraction(ch4, n2, 0.01, air)


def test_reactor_steady_after_ignition_composition(monkeypatch):
    """HomogeneousReactor.integrate_to_steady_after_ignition as two GPU integrations, checked on CPU with the
    integrations replaced by stand-ins: the first stops at ignition without the small-residual give-up, the
    second starts from the last accepted step size with the rest of the minimum step count, and the trajectories
    join at the ignition state without repeating it. Also current_pressure and n_reactions."""
    from spitfire_gb300.library import Dimension, Library
    from spitfire_gb300.reactors import HomogeneousReactor
    m = ChemicalMechanismSpec.bundled('h2-burke')
    mix = m.stream('TPX', (1200., 101325., 'H2:2 O2:1 N2:3.76'))
    r = HomogeneousReactor(m, mix, 'isobaric', 'adiabatic', 'closed')
    assert r.n_reactions == m.n_reactions and r.current_pressure == 101325.
    calls = []

    def traj(t, T):
        lib = Library(Dimension('time', np.asarray(t)))
        lib['temperature'] = np.asarray(T, dtype=np.float64)
        return lib

    def fake_ignition(save_first_and_last_only=False, **controls):
        calls.append(('ignition', controls))
        return traj([0., 1e-6, 3e-6, 7e-6], [1200., 1300., 1700., 2400.])

    def fake_steady(stop_at_steady=None, **kw):
        calls.append(('steady', dict(kw, stop_at_steady=stop_at_steady)))
        return traj([7e-6, 1.5e-5, 3e-5], [2400., 2450., 2460.])

    monkeypatch.setattr(r, '_integrate', fake_ignition)
    monkeypatch.setattr(r, 'integrate', fake_steady)
    lib = r.integrate_to_steady_after_ignition(steady_tolerance=1e-5, minimum_time_step_count=40)
    (k1, c1), (k2, c2) = calls
    assert k1 == 'ignition' and c1['delta_temperature_ignition'] == 400. and c1['minimum_allowable_residual'] == 0.
    assert k2 == 'steady' and c2['stop_at_steady'] == 1e-5
    assert c2['first_time_step'] == 7e-6 - 3e-6 and c2['minimum_time_step_count'] == 37
    np.testing.assert_array_equal(lib.dim('time').values, [0., 1e-6, 3e-6, 7e-6, 1.5e-5, 3e-5])
    np.testing.assert_array_equal(lib['temperature'], [1200., 1300., 1700., 2400., 2450., 2460.])
    calls.clear()
    fl = r.integrate_to_steady_after_ignition(save_first_and_last_only=True)
    np.testing.assert_array_equal(fl.dim('time').values, [0., 3e-5])


def test_reactor_front_end_accepts_every_configuration():
    """Every combination the reference's reactor coverage test builds (tests/reactor/test_reactor_coverage.py:
    isobaric and isochoric, closed and open with a feed, adiabatic, isothermal and diathermal over every supported
    shape) constructs on the host with the reference's argument names; an unknown shape or a diathermal reactor
    without its coefficients is rejected."""
    from spitfire_gb300.reactors import HomogeneousReactor
    m = ChemicalMechanismSpec.bundled('h2-burke')
    air = m.stream(stp_air=True)
    fuel = m.stream('X', 'H2:1')
    mix = m.mix_for_equivalence_ratio(1.0, fuel, air)
    mix.TP = 1200., 101325.
    feed = m.copy_stream(mix)
    n = 0
    for configuration in ('isobaric', 'isochoric'):
        for mass_transfer in ('closed', 'open'):
            for heat_transfer in ('adiabatic', 'isothermal', 'diathermal'):
                shapes = list(HomogeneousReactor.get_supported_reactor_shapes()) if heat_transfer == 'diathermal' \
                    else [None]
                for shape in shapes:
                    kw = {}
                    if mass_transfer == 'open':
                        kw.update(feed_temperature=feed.T, feed_mass_fractions=feed.Y, mixing_tau=1.e-3)
                        if configuration == 'isochoric':
                            kw['feed_density'] = feed.density
                    if heat_transfer == 'diathermal':
                        kw.update(convection_coefficient=1., convection_temperature=300., radiative_emissivity=1.,
                                  radiation_temperature=300.,
                                  shape_dimension_dict={'shape': shape, 'char. length': 1.e-3})
                    r = HomogeneousReactor(m, mix, configuration=configuration, heat_transfer=heat_transfer,
                                           mass_transfer=mass_transfer, **kw)
                    assert r.n_equations == m.n_species + (1 if configuration == 'isochoric' else 0)
                    n += 1
    assert n > 12
    with pytest.raises(Exception):
        HomogeneousReactor(m, mix, 'isobaric', 'diathermal', 'closed', convection_coefficient=1.,
                           convection_temperature=300., radiative_emissivity=1., radiation_temperature=300.,
                           shape_dimension_dict={'shape': 'dodecahedron-ish', 'char. length': 1.e-3})
    with pytest.raises(Exception):
        HomogeneousReactor(m, mix, 'isobaric', 'diathermal', 'closed')
