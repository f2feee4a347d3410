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
