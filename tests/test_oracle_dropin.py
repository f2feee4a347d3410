"""CPU: the oracle's single-state thermodynamics, flamelet stencils, residuals and Jacobians, and its block-Thomas
algebra against the reference's own PyCombustionKernels methods and py_btddod_* functions called directly
(tests/golden/dropin_ref.npz, made by tests/golden/make_golden.py from the reference Griffon built unmodified).
"""
import os

import numpy as np
import pytest

import flamelet_cases as FC
from helpers import pair

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
CASES = [c[0] for c in FC.FLAMELET_CASES]
TOL = 1e-10


def fixture():
    return np.load(os.path.join(GOLD, 'dropin_ref.npz'))


def rel(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize('name', CASES)
def test_oracle_thermo(name):
    d = fixture()
    _, og = pair(FC.BUNDLED[name])
    pre = name + '_thermo_'
    ns = og.n_species
    v = np.zeros(ns)
    for i, (T, y, p) in enumerate(zip(d[pre + 'T'], d[pre + 'Y'], d[pre + 'p'])):
        assert rel(og.mixture_molecular_weight(y), d[pre + 'mmw'][i]) < 1e-14
        assert rel(og.ideal_gas_density(p, T, y), d[pre + 'rho'][i]) < 1e-14
        assert rel(og.cp_mix(T, y), d[pre + 'cp'][i]) < 1e-13
        assert rel(og.cv_mix(T, y), d[pre + 'cv'][i]) < 1e-13
        assert rel(og.enthalpy_mix(T, y), d[pre + 'h'][i]) < 1e-12
        assert rel(og.energy_mix(T, y), d[pre + 'e'][i]) < 1e-12
        for k, f in (('cpi', og.species_cp), ('cvi', og.species_cv), ('hi', og.species_enthalpies),
                     ('ei', og.species_energies)):
            f(T, v)
            assert rel(v, d[pre + k][i]) < 1e-13, (k, T)
        og.dcpdT_species(T, y, v)
        assert rel(v, d[pre + 'dcpdT'][i]) < 1e-13


@pytest.mark.parametrize('name', CASES)
def test_oracle_flamelet_methods(name):
    d = fixture()
    _, og = pair(FC.BUNDLED[name])
    f = lambda k: d[name + '_flm_' + k]
    ns, nzi = og.n_species, f('cmajor').size // og.n_species
    outs = [np.zeros(nzi * ns) for _ in range(3)] + [np.zeros(nzi), np.zeros(nzi)]
    og.flamelet_stencils(f('dz'), nzi, f('chi'), f('invle'), *outs)
    for k, o in zip(('cmajor', 'csub', 'csup', 'mcoeff', 'ncoeff'), outs):
        np.testing.assert_array_equal(o, f(k))
    null = np.zeros(1)
    heat = {'ad': (True, null, null, null, null, False), 'na': (False, f('Tc'), f('Tr'), f('hc'), f('hr'), False),
            'ns': (False, f('Tc'), f('Tr'), f('hc') / 1.e3, f('hr'), True)}
    args = lambda hk: (f('state'), 101325., f('oxy'), f('fuel')) + heat[hk][:5] + \
        (nzi, f('cmajor'), f('csub'), f('csup'), f('mcoeff'), f('ncoeff'), f('chi'))
    for hk in heat:
        for ef in (0, 1):
            for vc in (0, 1):
                r = np.zeros(nzi * ns)
                og.flamelet_rhs(*args(hk), bool(ef), bool(vc), heat[hk][5], r)
                assert FC.vec_err(r, f(f'rhs_{hk}_e{ef}v{vc}'), ns) < TOL, (hk, ef, vc)
    for jk, (hk, sc, pf, ropt) in {'plain_r1': ('ad', False, 0., 1), 'ns': ('ns', False, 0., 0),
                                   'scaled': ('ad', True, 1.e-3, 0)}.items():
        if name + '_flm_jac_' + jk not in d:
            continue
        st, p, oxy, fuel, adb, a1, a2, a3, a4, nz, cma, csb, csp, mc, nc, chi = args(hk)
        v = og.flamelet_jacobian_values(st, p, oxy, fuel, adb, a1, a2, a3, a4, nz, cma, csb, csp, mc, nc, chi, sc, pf,
                                        ropt, True, heat[hk][5])
        assert FC.btddod_row_err(v, f('jac_' + jk), nzi, ns) < TOL, jk


def test_oracle_block_thomas():
    import oracle as orc
    d = fixture()
    for key in [k[:-2] for k in d.files if k.startswith('bt') and k.endswith('_A')]:
        nb, bs = (int(v) for v in key[2:].split('x'))
        A, x = d[key + '_A'], d[key + '_x']
        if key + '_full_matvec' in d:
            assert rel(orc.btddod_full_matvec(A, x, nb, bs), d[key + '_full_matvec']) < 1e-14
        fac, lv, piv = orc.btddod_full_factorize(A, nb, bs)
        assert rel(orc.btddod_full_solve(fac, lv, piv, x, nb, bs), d[key + '_full_solve']) < 1e-12
