"""Host-side tabulation logic against the reference's own functions (CPU).

tests/golden/structure_defect_ref.npz holds a seeded unstructured enthalpy-defect table (three dissipation rates
with 4, 5 and 7 ragged defects) and the reference's interpolation of it onto the structured defect dimension
(tabulation.py:594-665), without and with the extended range. spitfire_gb300.tabulation._structure_defect, which
both defect-library builders use, must reproduce both to rounding. And the unstrained libraries (unreacted,
Burke-Schumann, Burke-Schumann with a presumed enthalpy defect), which need no flamelet solve, against the
reference tests' gold libraries.
"""
import os

import numpy as np
import pytest

import flamelet_cases as FC


def _table(d):
    chis = d['chis']
    table = {}
    qs = ('temperature', 'enthalpy', 'enthalpy_defect', 'mass fraction X', 'mixture_fraction')
    for ci, chi in enumerate(chis):
        for gi, g in enumerate(d['g_%d' % ci]):
            table[(float(chi), float(g))] = {q: d['in_%d_%d_%s' % (ci, gi, q)] for q in qs}
    return table, qs


def test_structured_defect_dimension_matches_reference():
    from spitfire_gb300.tabulation import _structure_defect
    d = np.load(os.path.join(FC.GOLD, 'structure_defect_ref.npz'))
    table, qs = _table(d)
    for ext, tag in ((False, 'plain'), (True, 'ext')):
        st, xs, gs = _structure_defect(table, 6, extend=ext)
        np.testing.assert_allclose(xs, d[tag + '_x'], rtol=0, atol=0)
        np.testing.assert_allclose(gs, d[tag + '_g'], rtol=1e-15)
        for ix, x in enumerate(xs):
            for ig, g in enumerate(gs):
                for q in qs:
                    np.testing.assert_allclose(st[(x, g)][q], d['%s_%d_%d_%s' % (tag, ix, ig, q)], rtol=1e-12,
                                               atol=1e-9, err_msg=f'{tag} {ix} {ig} {q}')


def _unstrained_case():
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    m = ChemicalMechanismSpec.bundled('h2-burke')
    air = m.stream(stp_air=True)
    air.TP = 1200., 101325.
    fuel = m.stream('TPY', (300., 101325., 'H2:1'))
    return m, dict(mech_spec=m, oxy_stream=air, fuel_stream=fuel, grid_points=34)



@pytest.mark.parametrize('name,builder', [('adiabatic_unreacted', 'build_unreacted_library'),
                                          ('adiabatic_burke_schumann', 'build_adiabatic_bs_library'),
                                          ('nonadiabatic_defect_burke_schumann',
                                           'build_nonadiabatic_defect_bs_library')])
def test_unstrained_libraries_match_reference_gold(name, builder):
    """The reference's unstrained library tests (tests/tabulation/<name>: h2-burke, air 1200 K / H2 300 K, 34
    points) with the same post-processing (enthalpy, cv, cp, density, pressure; viscosity needs Cantera's transport
    data): dimensions to rounding, every property within 1e-8 of its largest magnitude. The temperatures come from
    enthalpy by Newton's method on the mechanism's NASA7 polynomials, as Cantera's do; the two solvers agree to
    about 1e-9."""
    from spitfire_gb300 import analysis as A
    from spitfire_gb300 import tabulation as TB
    m, specs = _unstrained_case()
    lib = getattr(TB, builder)(specs, verbose=False)
    for f in (A.compute_specific_enthalpy, A.compute_isochoric_specific_heat, A.compute_isobaric_specific_heat,
              A.compute_density, A.compute_pressure):
        lib = f(m, lib)
    g = np.load(os.path.join(FC.GOLD, name + '_gold.npz'))
    for i, dn in enumerate(lib.dim_names):
        assert str(g['dim%d_name' % i]) == dn
        np.testing.assert_allclose(lib.dims[i].values, g['dim%d_values' % i], rtol=1e-12, atol=1e-9)
    keys = [k for k in g.files if k.startswith('prop:')]
    assert len(keys) >= 5 + m.n_species
    for k in keys:
        a, b = np.asarray(lib[k[5:]]), g[k]
        assert a.shape == b.shape, k
        assert np.max(np.abs(a - b)) <= 1e-8 * max(np.max(np.abs(b)), 1e-300), k


def test_equilibrium_libraries_need_cantera():
    from spitfire_gb300 import tabulation as TB
    m, specs = _unstrained_case()
    with pytest.raises(NotImplementedError):
        TB.build_adiabatic_eq_library(specs)
    with pytest.raises(NotImplementedError):
        TB.build_nonadiabatic_defect_eq_library(specs)
