"""Host-side tabulation logic against the reference's own functions (CPU).

tests/golden/structure_defect_ref.npz holds a seeded unstructured enthalpy-defect table (three dissipation rates
with 4, 5 and 7 ragged defects) and the reference's interpolation of it onto the structured defect dimension
(tabulation.py:594-665), without and with the extended range. spitfire_gb300.tabulation._structure_defect, which
both defect-library builders use, must reproduce both to rounding.
"""
import os

import numpy as np

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
