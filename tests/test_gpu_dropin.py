"""GPU: the drop-in surface with the reference's own names and argument lists, against the reference.

Every single-state method of spitfire_gb300.griffon.PyCombustionKernels and every module-level py_btddod_*
function is called exactly as the reference's callers call spitfire.griffon.griffon (griffon.pyx:556-866,
:1009-1113), and compared with what the reference Griffon returned for the same arguments
(tests/golden/dropin_ref.npz, kernels_<mech>.npz and open_kernels_<mech>.npz, made by tests/golden/make_golden.py).
Bars: 1e-10 relative (row-normwise for Jacobians, per variable for point-major vectors); stencils and indices
exactly; eigenvalue bounds to the tolerance two backward-stable eigensolvers share.
"""
import os

import numpy as np
import pytest

import flamelet_cases as FC
from helpers import colmajor, rownorm_err

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
CASES = [c[0] for c in FC.FLAMELET_CASES]
TOL = 1e-10


def fixture(name='dropin_ref'):
    return np.load(os.path.join(GOLD, name + '.npz'))


def rel(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def spec_of(name):
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    return ChemicalMechanismSpec.bundled(name)


@pytest.mark.parametrize('name', CASES)
def test_thermo_methods(cuda, name):
    """mixture_molecular_weight, mole_fractions, ideal_gas_density/pressure, cp/cv/enthalpy/energy_mix,
    species_cp/cv/enthalpies/energies and dcpdT_species (griffon.pyx:684-761), including temperatures outside the
    NASA7 fit ranges (cp clamped, enthalpy extrapolated)."""
    d = fixture()
    g = spec_of(FC.BUNDLED[name]).griffon
    pre = name + '_thermo_'
    ns = g.n_species
    v = np.zeros(ns)
    for i, (T, y, p) in enumerate(zip(d[pre + 'T'], d[pre + 'Y'], d[pre + 'p'])):
        assert rel(g.mixture_molecular_weight(y), d[pre + 'mmw'][i]) < TOL
        g.mole_fractions(y, v)
        assert rel(v, d[pre + 'x'][i]) < TOL
        rho = g.ideal_gas_density(p, T, y)
        assert rel(rho, d[pre + 'rho'][i]) < TOL
        assert rel(g.ideal_gas_pressure(rho, T, y), d[pre + 'p'][i]) < TOL
        for k, f in (('cp', g.cp_mix), ('cv', g.cv_mix), ('h', g.enthalpy_mix), ('e', g.energy_mix)):
            assert rel(f(T, y), d[pre + k][i]) < TOL, (k, T)
        for k, f in (('cpi', g.species_cp), ('cvi', g.species_cv), ('hi', g.species_enthalpies),
                     ('ei', g.species_energies)):
            v[:] = np.nan
            f(T, v)
            assert rel(v, d[pre + k][i]) < TOL, (k, T)
        v[:] = np.nan
        g.dcpdT_species(T, y, v)
        assert rel(v, d[pre + 'dcpdT'][i]) < TOL, T


@pytest.mark.parametrize('name', ['h2-burke', 'methane-gri30'])
def test_kinetics_and_closed_reactor_methods(cuda, name):
    """production_rates(T, rho, Y, out) with its first argument taken as the temperature (griffon.pyx:763-768),
    prod_rates_primitive_sensitivities for options 0/1/2, and the closed reactor right-hand sides and Jacobians,
    with the argument lists the reference fixtures were made with."""
    d = fixture('kernels_' + name)
    g = spec_of(name).griffon
    ns = g.n_species
    yin = np.zeros(ns)
    for i in range(d['T'].size):
        w = np.full(ns, np.nan)
        g.production_rates(d['T'][i], d['rho'][i], d['Y'][i], w)
        assert rownorm_err(w, d['w'][i]) <= TOL
        for opt in range(3):
            S = np.full((ns + 1) ** 2, np.nan)
            g.prod_rates_primitive_sensitivities(d['rho'][i], d['T'][i], d['Y'][i], opt, S)
            assert rownorm_err(colmajor(S, ns + 1)[:ns], colmajor(d['S'][opt, i], ns + 1)[:ns]) <= TOL, opt
        r, J = np.zeros(ns + 1), np.zeros((ns + 1) ** 2)
        g.reactor_jac_isochoric(d['qiv'][i], 0., 0., yin, 1., 0., 0., 0., 0., 1., 0, False, 0, r, J)
        assert rownorm_err(r, d['jac_rhs_iv'][i]) <= TOL
        assert rownorm_err(colmajor(J, ns + 1), colmajor(d['Jiv'][i], ns + 1)) <= TOL
        g.reactor_rhs_isochoric(d['qiv'][i], 0., 0., yin, 1., 0., 0., 0., 0., 1., 0, False, r)
        assert rownorm_err(r, d['rhs_iv'][i]) <= TOL
        r, J = np.zeros(ns), np.zeros(ns * ns)
        g.reactor_jac_isobaric(d['qib'][i], d['p'][i], 0., yin, 1., 0., 0., 0., 0., 1., 0, False, 0, 0, r, J)
        assert rownorm_err(r, d['jac_rhs_ib'][i]) <= TOL
        assert rownorm_err(colmajor(J, ns), colmajor(d['Jib'][i], ns)) <= TOL
        g.reactor_rhs_isobaric(d['qib'][i], d['p'][i], 0., yin, 1., 0., 0., 0., 0., 1., 0, False, r)
        assert rownorm_err(r, d['rhs_ib'][i]) <= TOL
        # a sensitivity transform other than 0 ('exact') leaves the Jacobian argument as it was
        # (isobaric_reactor_kernels.cpp:305-311); the right-hand side is still written
        J[:] = -7.
        r[:] = np.nan
        g.reactor_jac_isobaric(d['qib'][i], d['p'][i], 0., yin, 1., 0., 0., 0., 0., 1., 0, False, 0, 1, r, J)
        assert np.all(J == -7.)
        assert rownorm_err(r, d['jac_rhs_ib'][i]) <= TOL


@pytest.mark.parametrize('name', ['h2-burke', 'methane-gri30'])
@pytest.mark.parametrize('heat', ['adiabatic', 'isothermal', 'diathermal'])
def test_open_reactor_methods(cuda, name, heat):
    """Open (mass-exchange) reactors through the single-state methods, each heat-transfer option."""
    d = fixture('open_kernels_' + name)
    g = spec_of(name).griffon
    ns = g.n_species
    ho = {'adiabatic': 0, 'isothermal': 1, 'diathermal': 2}[heat]
    Tc, Tr, hc, eps, sov = 600., 900., 50., 0.3, 20.
    for i in range(d['T'].size):
        r, J = np.zeros(ns + 1), np.zeros((ns + 1) ** 2)
        args = (d['rhoin'][i], d['Tin'][i], d['Yin'][i], d['tau'][i], Tc, Tr, hc, eps, sov, ho, True)
        g.reactor_rhs_isochoric(d['qiv'][i], *args, r)
        assert rownorm_err(r, d[f'{heat}_rhs_iv'][i]) <= TOL
        g.reactor_jac_isochoric(d['qiv'][i], *args, 0, r, J)
        assert rownorm_err(r, d[f'{heat}_jac_rhs_iv'][i]) <= TOL
        assert rownorm_err(colmajor(J, ns + 1), colmajor(d[f'{heat}_Jiv'][i], ns + 1)) <= TOL
        r, J = np.zeros(ns), np.zeros(ns * ns)
        args = (d['p'][i], d['Tin'][i], d['Yin'][i], d['tau'][i], Tc, Tr, hc, eps, sov, ho, True)
        g.reactor_rhs_isobaric(d['qib'][i], *args, r)
        assert rownorm_err(r, d[f'{heat}_rhs_ib'][i]) <= TOL
        g.reactor_jac_isobaric(d['qib'][i], *args, 0, 0, r, J)
        assert rownorm_err(r, d[f'{heat}_jac_rhs_ib'][i]) <= TOL
        assert rownorm_err(colmajor(J, ns), colmajor(d[f'{heat}_Jib'][i], ns)) <= TOL


@pytest.mark.parametrize('name', CASES)
def test_flamelet_methods(cuda, name):
    """flamelet_stencils, flamelet_jac_indices, flamelet_rhs and flamelet_jacobian (griffon.pyx:556-679) with the
    argument lists of the reference's Flamelet closures (flamelet.py:623-915): adiabatic, nonadiabatic with plain
    and temperature-range scaled heat loss (the Python order T_conv, T_rad, h_conv, h_rad), enthalpy flux and
    variable cp on and off, rates options, eigenvalue bounds, and the scaled-and-offset form."""
    d = fixture()
    g = spec_of(FC.BUNDLED[name]).griffon
    f = lambda k: d[name + '_flm_' + k]
    ns = g.n_species
    nzi = f('cmajor').size // ns
    outs = [np.zeros(nzi * ns) for _ in range(3)] + [np.zeros(nzi), np.zeros(nzi)]
    g.flamelet_stencils(f('dz'), nzi, f('chi'), f('invle'), *outs)
    for k, o in zip(('cmajor', 'csub', 'csup', 'mcoeff', 'ncoeff'), outs):
        np.testing.assert_allclose(o, f(k), rtol=1e-15, atol=0)
    nel = ns * (nzi * ns + 2 * (nzi - 1))
    rows, cols = np.zeros(nel, dtype=np.int32), np.zeros(nel, dtype=np.int32)
    g.flamelet_jac_indices(nzi, rows, cols)
    np.testing.assert_array_equal(rows, f('rows'))
    np.testing.assert_array_equal(cols, f('cols'))
    null = np.zeros(1)
    heat = {'ad': (True, null, null, null, null, False), 'na': (False, f('Tc'), f('Tr'), f('hc'), f('hr'), False),
            'ns': (False, f('Tc'), f('Tr'), f('hc') / 1.e3, f('hr'), True)}
    head = lambda hk: (f('state'), 101325., f('oxy'), f('fuel')) + heat[hk][:5] + \
        (nzi, f('cmajor'), f('csub'), f('csup'), f('mcoeff'), f('ncoeff'), f('chi'))
    for hk in heat:
        for ef in (0, 1):
            for vc in (0, 1):
                r = np.full(nzi * ns, np.nan)
                g.flamelet_rhs(*head(hk), bool(ef), bool(vc), heat[hk][5], r)
                assert FC.vec_err(r, f(f'rhs_{hk}_e{ef}v{vc}'), ns) < TOL, (hk, ef, vc)
    diffterm = float(f('diffterm'))
    cases = {'plain_r0': ('ad', False, 0., False, 0., 0, True), 'plain_r1': ('ad', False, 0., False, 0., 1, True),
             'plain_r2': ('ad', False, 0., False, 0., 2, True), 'plain_e0': ('ad', False, 0., False, 0., 0, False),
             'scaled': ('ad', False, 0., True, 1.e-3, 0, True), 'eig': ('ad', True, diffterm, False, 0., 0, True),
             'eig_scaled': ('ad', True, diffterm, True, 1.e-3, 0, True),
             'na': ('na', False, 0., False, 0., 0, True), 'ns': ('ns', False, 0., False, 0., 0, True)}
    # scale of each point's chemistry block, for the eigenvalue tolerance
    v0 = np.zeros(nel)
    g.flamelet_jacobian(*head('ad'), False, 0., False, 0., 0, 0, True, True, False, null, v0)
    blocks = np.swapaxes(v0[:nzi * ns * ns].reshape(nzi, ns, ns), 1, 2)
    fro = np.array([np.linalg.norm(blocks[i] - np.diag(f('cmajor')[i * ns:(i + 1) * ns])) for i in range(nzi)])
    ran = 0
    for jk, (hk, eig, dt, sc, pf, ropt, ef) in cases.items():
        if name + '_flm_jac_' + jk not in d:
            continue
        v = np.full(nel, np.nan)
        e = np.full(nzi * ns, np.nan)
        g.flamelet_jacobian(*head(hk), eig, dt, sc, pf, ropt, 0, ef, True, heat[hk][5], e, v)
        assert FC.btddod_row_err(v, f('jac_' + jk), nzi, ns) < TOL, jk
        if eig:
            ref = f('expeig_' + jk)
            tol = 1e-13 * np.repeat(fro, ns) + 1e-8 * np.maximum(np.abs(ref), 1.)
            assert np.all(np.abs(e - ref) <= tol), jk
        ran += 1
    assert ran >= 3
    with pytest.raises(ValueError):
        g.flamelet_jacobian(*head('ad'), False, 0., False, 0., 0, 1, True, True, False, null, np.zeros(nel))


def _bt_keys(d):
    return [k[:-2] for k in d.files if k.startswith('bt') and k.endswith('_A')]


def test_py_btddod_functions(cuda):
    """The ten module-level py_btddod_* functions (griffon.pyx:1009-1113) on numpy arguments, as the reference's
    flamelet.py passes them, against the reference's results on seeded block-diagonally dominant matrices of 1 to
    7 blocks and block sizes 3 to 53."""
    from spitfire_gb300 import griffon as G
    d = fixture()
    keys = _bt_keys(d)
    assert len(keys) >= 4
    for key in keys:
        nb, bs = (int(v) for v in key[2:].split('x'))
        A, x = d[key + '_A'], d[key + '_x']
        n = nb * bs
        y = np.full(n, np.nan)
        if key + '_full_matvec' in d:
            G.py_btddod_full_matvec(A, x, nb, bs, y)
            assert rel(y, d[key + '_full_matvec']) < TOL, key
        G.py_btddod_blockdiag_matvec(A, x, nb, bs, y)
        assert rel(y, d[key + '_blockdiag_matvec']) < TOL, key
        piv = np.zeros(n, dtype=np.int32)
        fac = np.zeros(n * bs)
        G.py_btddod_blockdiag_factorize(A, nb, bs, piv, fac)
        G.py_btddod_blockdiag_solve(piv, fac, x, nb, bs, y)
        assert rel(y, d[key + '_blockdiag_solve']) < TOL, key
        G.py_btddod_lowerfulltriangle_solve(piv, fac, A, x, nb, bs, y)
        assert rel(y, d[key + '_lower_solve']) < TOL, key
        G.py_btddod_upperfulltriangle_solve(piv, fac, A, x, nb, bs, y)
        assert rel(y, d[key + '_upper_solve']) < TOL, key
        Af = A.copy()
        lv = np.zeros(n * bs)
        pv = np.zeros(A.size, dtype=np.int32)  # flamelet.py sizes its pivot array as the values
        G.py_btddod_full_factorize(Af, nb, bs, lv, pv)
        y[:] = np.nan
        G.py_btddod_full_solve(Af, lv, pv, x, nb, bs, y)
        assert rel(y, d[key + '_full_solve']) < TOL, key
        As = A.copy()
        G.py_btddod_scale_and_add_scaled_block_diagonal(As, 0.7, d[key + '_B'], -1.3, nb, bs)
        assert rel(As, d[key + '_scaled_block']) < 1e-15, key
        As = A.copy()
        G.py_btddod_scale_and_add_diagonal(As, -1., d[key + '_d'], 2.5, nb, bs)
        assert rel(As, d[key + '_scaled_diag']) < 1e-15, key


def test_py_btddod_on_device_tensors(cuda):
    """The same functions on torch CUDA tensors work in place, without host copies."""
    import torch
    from spitfire_gb300 import griffon as G
    d = fixture()
    key = [k for k in _bt_keys(d) if k.endswith('x53')][0]
    nb, bs = (int(v) for v in key[2:].split('x'))
    t = lambda a, dt=torch.float64: torch.tensor(a, dtype=dt, device='cuda')
    A, x = t(d[key + '_A']), t(d[key + '_x'])
    lv, pv = torch.zeros(nb * bs * bs, dtype=torch.float64, device='cuda'), torch.zeros(nb * bs, dtype=torch.int32,
                                                                                        device='cuda')
    y = torch.empty(nb * bs, dtype=torch.float64, device='cuda')
    G.py_btddod_full_matvec(A, x, nb, bs, y)
    assert rel(y.cpu().numpy(), d[key + '_full_matvec']) < TOL
    G.py_btddod_full_factorize(A, nb, bs, lv, pv)
    G.py_btddod_full_solve(A, lv, pv, x, nb, bs, y)
    assert rel(y.cpu().numpy(), d[key + '_full_solve']) < TOL
    with pytest.raises(TypeError):
        G.py_btddod_full_solve(A, lv, pv, x, nb, bs, y.cpu().numpy().astype(np.float32))
