"""Host-side mechanism utilities (spitfire_gb300/mechanism.py) on CPU: the mechanism API basics of the reference's
tests/mechanism/test_mechanisms_and_streams.py, pickling, and the stream utilities around stoichiometry."""
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
