"""GPU flamelet path against the reference Flamelet (tests/golden/flamelet_ref.npz) and the oracle.

A batch holds the reference's golden flamelet plus two more flamelets of the same mechanism with other grids and
dissipation rates, so every launch covers ragged batches. Bars: residuals and Jacobian rows 1e-10 (row-normwise,
FP64); eigenvalue bounds 1e-13 ||A||_F + 1e-8 max(|lambda|, 1) (two backward-stable eigenvalue algorithms agree
to a multiple of eps ||A||, and chemistry blocks reach ||A||_F ~ 1e11); block-Thomas solutions 1e-9 normwise; steady solvers:
same convergence and iteration counts as the reference solvers, temperatures within 1e-6 relative (the solvers'
own tolerance), mass fractions within 1e-6 per species of the species' maximum.
"""
import numpy as np
import pytest

import flamelet_cases as FC
from helpers import pair

pytestmark = pytest.mark.gpu
CASES = [c[0] for c in FC.FLAMELET_CASES]


def _setups(name, extra=True):
    from spitfire_gb300.flamelet import FlameletSetup, FlameletSpec
    d = FC.golden()
    spec, og = pair(FC.BUNDLED[name])
    oxy, fuel, kw = FC.flamelet_case_setup(spec, FC.case(name))
    setups = [FlameletSetup(FlameletSpec(mech_spec=spec, initial_condition=d[name + '_state'], **kw))]
    if extra:
        rng = np.random.default_rng(5)
        for npts, chi in ((9, 0.3), (21, 5.)):
            s = FlameletSetup(FlameletSpec(mech_spec=spec, initial_condition='Burke-Schumann',
                                           **dict(kw, grid_points=npts, stoich_dissipation_rate=chi)))
            s.initial_state = np.abs(s.initial_state * (1. + 0.02 * rng.standard_normal(s.initial_state.size)))
            setups.append(s)
    return d, spec, og, setups


def _ops(og, setups):
    import flamelet_steady as FS
    return [FS.FlameletOperator(og, s.z, s.x, s.state_oxy, s.state_fuel) for s in setups]


def _split(b, v, per='z'):
    v = v.cpu().numpy()
    out = []
    for f in range(b.nf):
        if per == 'z':
            out.append(v[b.offz_host[f] * b.ns:b.offz_host[f + 1] * b.ns])
        else:
            out.append(v[b.offv_host[f]:b.offv_host[f + 1]])
    return out


@pytest.mark.parametrize('name', CASES)
def test_flamelet_rhs_and_jacobian(cuda, name):
    from spitfire_gb300.flamelet import FlameletBatch
    d, spec, og, setups = _setups(name)
    b = FlameletBatch(setups)
    ops = _ops(og, setups)
    ns = b.ns
    st = b.initial_state()
    states = [s.initial_state for s in setups]
    for ef in (0, 1):
        for vc in (0, 1):
            b.fb.include_enthalpy_flux, b.fb.include_variable_cp = ef, vc
            r = _split(b, b.rhs(st))
            assert FC.vec_err(r[0], d[name + f'_rhs_e{ef}v{vc}'], ns) < 1e-10, (ef, vc)
            for f in range(b.nf):
                assert FC.vec_err(r[f], ops[f].rhs(states[f], eflux=ef, vcp=vc), ns) < 1e-10, (f, ef, vc)
        b.fb.include_variable_cp = 1
        J = _split(b, b.jacobian(st).clone(), 'v')
        assert FC.btddod_row_err(J[0], d[name + f'_jac_e{ef}'], setups[0].nzi, ns) < 1e-10, ef
        for f in range(b.nf):
            assert FC.btddod_row_err(J[f], ops[f].jac(states[f], eflux=ef), setups[f].nzi, ns) < 1e-10, (f, ef)
    b.fb.include_enthalpy_flux, b.fb.include_variable_cp = 1, 1
    J = _split(b, b.jacobian(st, scale_and_offset=True, prefactor=1.e-3).clone(), 'v')
    assert FC.btddod_row_err(J[0], d[name + '_jac_scaled'], setups[0].nzi, ns) < 1e-10
    for f in range(b.nf):
        ref = ops[f].jac(states[f], scale_and_offset=True, prefactor=1.e-3)
        assert FC.btddod_row_err(J[f], ref, setups[f].nzi, ns) < 1e-10, f
    assert spec.griffon.device_status() == 0


@pytest.mark.parametrize('name', CASES)
def test_flamelet_eigenvalue_bounds(cuda, name):
    from spitfire_gb300.flamelet import FlameletBatch
    d, spec, og, setups = _setups(name)
    b = FlameletBatch(setups)
    ops = _ops(og, setups)
    st = b.initial_state()
    dt = float(d[name + '_diffterm'])
    vals, e = b.jacobian(st, eig=True, diffterm=dt)
    J = _split(b, vals.clone(), 'v')
    e = _split(b, e)
    # values are the plain Jacobian (eigenvalues do not change them)
    assert FC.btddod_row_err(J[0], d[name + '_jac_eig'], setups[0].nzi, b.ns) < 1e-10
    ref = d[name + '_expeig']
    assert FC.eig_err(e[0], ref, ops[0], setups[0].initial_state) < 1.
    for f in range(b.nf):
        o = ops[f].expeig(setups[f].initial_state, dt)
        assert FC.eig_err(e[f], o, ops[f], setups[f].initial_state) < 1., f
    # per-flamelet diffusion term, as steady_solve_psitc uses it
    e2 = _split(b, b.expeig_per_flamelet_diffterm(st))
    for f in range(b.nf):
        o = ops[f].expeig(setups[f].initial_state, 4. * setups[f].max_dissipation_rate)
        assert FC.eig_err(e2[f], o, ops[f], setups[f].initial_state) < 1., f
    assert spec.griffon.device_status() == 0


@pytest.mark.parametrize('name', CASES)
def test_block_thomas_factor_solve_matvec_scale(cuda, name):
    import torch
    import oracle as orc
    from spitfire_gb300.flamelet import FlameletBatch
    d, spec, og, setups = _setups(name)
    b = FlameletBatch(setups)
    ops = _ops(og, setups)
    ns = b.ns
    st = b.initial_state()
    rng = np.random.default_rng(9)
    x = torch.tensor(rng.standard_normal(b.npts * ns), dtype=torch.float64, device='cuda')
    J0 = [ops[f].jac(setups[f].initial_state) for f in range(b.nf)]
    # matvec with -J
    b.jacobian(st)
    b.values.neg_()
    y = _split(b, b.matvec(x))
    xs = _split(b, x)
    for f in range(b.nf):
        ref = orc.btddod_full_matvec(-J0[f], xs[f], setups[f].nzi, ns)
        assert FC.vec_err(y[f], ref, ns) < 1e-10, f
    # golden flamelet: the reference's matvec / solve on -J at its own vector
    g = torch.zeros(b.npts * ns, dtype=torch.float64, device='cuda')
    g[:setups[0].nzi * ns] = torch.tensor(d[name + '_matvec_b'], device='cuda')
    assert FC.vec_err(_split(b, b.matvec(g))[0], d[name + '_matvec_y'], ns) < 1e-10
    b.factor()
    sol = _split(b, b.solve(g))[0]
    ref = d[name + '_solve_x']
    assert np.max(np.abs(sol - ref)) / np.max(np.abs(ref)) < 1e-9
    xsol = _split(b, b.solve(x))
    for f in range(b.nf):
        dd, l, piv = orc.btddod_full_factorize(-J0[f], setups[f].nzi, ns)
        ref = orc.btddod_full_solve(dd, l, piv, xs[f], setups[f].nzi, ns)
        assert np.max(np.abs(xsol[f] - ref)) / np.max(np.abs(ref)) < 1e-9, f
    # -J + diag(1/ds) against the reference's scale_and_add_diagonal
    b.jacobian(st)
    ds = torch.tensor(np.exp(rng.uniform(np.log(1e-6), np.log(1e-2), b.npts * ns)), device='cuda')
    ds[:setups[0].nzi * ns] = torch.tensor(d[name + '_scaled_ds'], device='cuda')
    b.scale_and_add_diagonal(-1., 1. / ds, 1.)
    S = _split(b, b.values.clone(), 'v')
    assert FC.btddod_row_err(S[0], d[name + '_scaled_values'], setups[0].nzi, ns) < 1e-10
    assert spec.griffon.device_status() == 0


@pytest.mark.parametrize('name', CASES)
def test_batched_steady_solvers_match_reference(cuda, name):
    """psitc from the Burke-Schumann profile (Newton fails there, as in the reference) and a Newton continuation
    step at 1.5 chi_st, in one batch with two other flamelets; the golden flamelet must follow the reference
    solvers' iteration counts and converge to their profiles, the others must match the oracle solvers."""
    import torch
    import flamelet_steady as FS
    from spitfire_gb300.flamelet import FlameletBatch, FlameletSetup, FlameletSpec
    d, spec, og, setups = _setups(name)
    setups[0].initial_state = d[name + '_ic'].copy()
    b = FlameletBatch(setups)
    ops = _ops(og, setups)
    ns = b.ns
    init = b.initial_state()
    s, conv, it = b.steady_solve_newton(init, tolerance=1.e-6, max_iterations=38)
    assert bool(conv[0]) == bool(d[name + '_newton_conv'])
    s, conv, it = b.steady_solve_psitc(init, tolerance=1.e-6, max_iterations=400)
    conv, it = conv.cpu().numpy(), it.cpu().numpy()
    st = _split(b, s)
    assert conv[0] and it[0] == int(d[name + '_psitc_iters']), (conv, it)
    ref = d[name + '_psitc_state']
    assert np.max(np.abs(st[0][::ns] - ref[::ns]) / ref[::ns]) < 1e-6
    assert FC.vec_err(st[0], ref, ns) < 1e-6
    for f in range(1, b.nf):
        o, oit, oconv, _ = FS.steady_solve_psitc(ops[f], setups[f].initial_state)
        assert bool(conv[f]) == oconv, f
        if oconv:
            assert it[f] == oit, (f, it[f], oit)
            assert FC.vec_err(st[f], o, ns) < 1e-6
    # continuation Newton step
    oxy, fuel, kw = FC.flamelet_case_setup(spec, FC.case(name))
    kw['stoich_dissipation_rate'] *= 1.5
    s3 = FlameletSetup(FlameletSpec(mech_spec=spec, initial_condition=ref.copy(), **kw))
    b3 = FlameletBatch([s3])
    out, conv, it = b3.steady_solve_newton(b3.initial_state(), tolerance=1.e-6, max_iterations=38)
    assert bool(conv[0]) and int(it[0]) == int(d[name + '_cont_iters'])
    r3 = d[name + '_cont_state']
    o3 = out.cpu().numpy()
    assert np.max(np.abs(o3[::ns] - r3[::ns]) / r3[::ns]) < 1e-6
    assert FC.vec_err(o3, r3, ns) < 1e-6
    assert spec.griffon.device_status() == 0


def test_flamelet_drop_in_compute_steady_state(cuda):
    from spitfire_gb300.flamelet import Flamelet
    d = FC.golden()
    spec, og = pair('h2-burke')
    oxy, fuel, kw = FC.flamelet_case_setup(spec, FC.case('h2'))
    f = Flamelet(dict(mech_spec=spec, initial_condition='Burke-Schumann', **kw))
    lib = f.compute_steady_state(tolerance=1.e-6)
    ref = d['h2_psitc_state']
    T = lib['temperature'][1:-1]
    assert np.max(np.abs(T - ref[::spec.n_species]) / ref[::spec.n_species]) < 1e-6
    assert abs(lib['temperature'][0] - oxy.T) < 1e-12 and abs(lib['temperature'][-1] - fuel.T) < 1e-12
    ysum = sum(lib['mass fraction ' + n] for n in spec.species_names)
    assert np.allclose(ysum, 1., atol=1e-12)


def test_adiabatic_slfm_library_matches_reference_gold(cuda):
    """tests/tabulation/adiabatic_slfm of the reference (h2-burke, air 1200 K / H2 300 K, 34 points,
    chi_st = logspace(0, 1, 8)) through the drop-in build_adiabatic_slfm_library; the reference test's bars
    (rtol = atol = 1e-6) on temperature, pressure and every mass fraction, and the library dimensions."""
    import os
    from spitfire_gb300.library import Library
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    from spitfire_gb300.tabulation import build_adiabatic_slfm_library
    g = np.load(os.path.join(FC.GOLD, 'adiabatic_slfm_gold.npz'))
    m = ChemicalMechanismSpec.bundled('h2-burke')
    air = m.stream(stp_air=True)
    air.TP = 1200., 101325.
    fuel = m.stream('TPY', (300., 101325., 'H2:1'))
    lib = build_adiabatic_slfm_library(dict(mech_spec=m, oxy_stream=air, fuel_stream=fuel, grid_points=34),
                                       verbose=False, diss_rate_values=np.logspace(0, 1, 8),
                                       diss_rate_log_scaled=True)
    assert lib.dim_names == ['mixture_fraction', 'dissipation_rate_stoich']
    np.testing.assert_allclose(lib.dims[0].values, g['dim0_values'], rtol=1e-14)
    np.testing.assert_allclose(lib.dims[1].values, g['dim1_values'], rtol=1e-12)
    assert lib.dims[1].log_scaled
    keys = [k for k in g.files if k.startswith('prop:')]
    assert len(keys) == 2 + m.n_species
    for k in keys:
        np.testing.assert_allclose(lib[k[5:]], g[k], rtol=1e-6, atol=1e-6, err_msg=k)
    # the pickle round trip keeps everything
    import tempfile
    with tempfile.TemporaryDirectory() as t:
        p = os.path.join(t, 'slfm.pkl')
        lib.extra_attributes.pop('mech_spec')
        lib.save_to_file(p)
        l2 = Library.load_from_file(p)
        for k in keys:
            assert np.array_equal(l2[k[5:]], lib[k[5:]])


@pytest.mark.parametrize('name', CASES)
@pytest.mark.parametrize('variant', ['plain', 'scaled'])
def test_nonadiabatic_flamelet_rhs_and_jacobian(cuda, name, variant):
    """Heat loss on the GPU: a batch of the reference's nonadiabatic flamelet (tests/golden/flamelet_nonad_ref.npz),
    an adiabatic flamelet and a nonadiabatic flamelet on another grid; residuals and Jacobians against the reference
    and the oracle at the same bars."""
    import flamelet_steady as FS
    from spitfire_gb300.flamelet import FlameletBatch, FlameletSetup, FlameletSpec
    g = np.load(FC.GOLD + '/flamelet_nonad_ref.npz')
    d = FC.golden()
    spec, og = pair(FC.BUNDLED[name])
    oxy, fuel, kw = FC.flamelet_case_setup(spec, FC.case(name))
    v = f'{name}_{variant}_'
    if variant == 'plain':
        hk = dict(heat_transfer='nonadiabatic', convection_temperature=g[v + 'arg_convection_temperature'],
                  radiation_temperature=g[v + 'arg_radiation_temperature'],
                  convection_coefficient=g[v + 'arg_convection_coefficient'],
                  radiative_emissivity=g[v + 'arg_radiative_emissivity'])
        hk2 = dict(heat_transfer='nonadiabatic', convection_temperature=400., radiation_temperature=500.,
                   convection_coefficient=3.e4, radiative_emissivity=0.4)
    else:
        hk = dict(heat_transfer='nonadiabatic', scale_heat_loss_by_temp_range=True,
                  scale_convection_by_dissipation=True, use_linear_ref_temp_profile=True,
                  convection_coefficient=1.e7, radiative_emissivity=0.5)
        hk2 = dict(hk, convection_coefficient=3.e6)
    st0 = g[name + '_state']
    s0 = FlameletSetup(FlameletSpec(mech_spec=spec, initial_condition=st0, **dict(kw, **hk)))
    s1 = FlameletSetup(FlameletSpec(mech_spec=spec, initial_condition='Burke-Schumann',
                                    **dict(kw, grid_points=13, stoich_dissipation_rate=3.)))
    s2 = FlameletSetup(FlameletSpec(mech_spec=spec, initial_condition='Burke-Schumann',
                                    **dict(kw, grid_points=19, stoich_dissipation_rate=0.5, **hk2)))
    rng = np.random.default_rng(7)
    for s in (s1, s2):
        s.initial_state = np.abs(s.initial_state * (1. + 0.02 * rng.standard_normal(s.initial_state.size)))
    setups = [s0, s1, s2]
    b = FlameletBatch(setups)
    ops = [FS.FlameletOperator(og, s.z, s.x, s.state_oxy, s.state_fuel,
                               heat_loss=None if s.heat_transfer == 'adiabatic' else
                               dict(T_conv=s.T_conv, T_rad=s.T_rad, h_conv=s.h_conv, h_rad=s.h_rad,
                                    scaled=s.scale_heat_loss_by_temp_range)) for s in setups]
    ns = b.ns
    st = b.initial_state()
    r = _split(b, b.rhs(st))
    assert FC.vec_err(r[0], g[v + 'rhs'], ns) < 1e-10
    J = _split(b, b.jacobian(st).clone(), 'v')
    assert FC.btddod_row_err(J[0], g[v + 'jac'], s0.nzi, ns) < 1e-10
    for f, s in enumerate(setups):
        assert FC.vec_err(r[f], ops[f].rhs(s.initial_state), ns) < 1e-10, f
        assert FC.btddod_row_err(J[f], ops[f].jac(s.initial_state), s.nzi, ns) < 1e-10, f
    assert spec.griffon.device_status() == 0
    del d


def test_nonadiabatic_steady_slfm_library_matches_reference_gold(cuda):
    """tests/tabulation/nonadiabatic_defect_steady_slfm of the reference (h2-burke, air 1200 K / H2 300 K, 34
    points, chi_st = logspace(0, 1, 4), 32 stoichiometric enthalpy defects) through the drop-in
    build_nonadiabatic_defect_steady_slfm_library; the reference test's bars (rtol 2e-4, atol 1e-4) on temperature,
    pressure, every mass fraction, the enthalpy and the enthalpy defect, and the library dimensions. As in the
    reference test (rebless.py), the enthalpy is recomputed from the library's states afterwards."""
    import os
    from spitfire_gb300.analysis import compute_specific_enthalpy
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    from spitfire_gb300.tabulation import build_nonadiabatic_defect_steady_slfm_library
    g = np.load(os.path.join(FC.GOLD, 'nonadiabatic_steady_slfm_gold.npz'))
    m = ChemicalMechanismSpec.bundled('h2-burke')
    air = m.stream(stp_air=True)
    air.TP = 1200., 101325.
    fuel = m.stream('TPY', (300., 101325., 'H2:1'))
    lib = build_nonadiabatic_defect_steady_slfm_library(
        dict(mech_spec=m, oxy_stream=air, fuel_stream=fuel, grid_points=34), verbose=False,
        diss_rate_values=np.logspace(0, 1, 4), diss_rate_log_scaled=True,
        integration_args={'transient_tolerance': 1e-10}, num_procs=1)
    lib = compute_specific_enthalpy(m, lib)
    assert lib.dim_names == ['mixture_fraction', 'dissipation_rate_stoich', 'enthalpy_defect_stoich']
    np.testing.assert_allclose(lib.dims[0].values, g['dim0_values'], rtol=1e-14)
    np.testing.assert_allclose(lib.dims[1].values, g['dim1_values'], rtol=1e-12)
    np.testing.assert_allclose(lib.dims[2].values, g['dim2_values'], rtol=2e-4, atol=1e-4)
    keys = [k for k in g.files if k.startswith('prop:')]
    assert len(keys) == 4 + m.n_species
    for k in keys:
        np.testing.assert_allclose(lib[k[5:]], g[k], rtol=2e-4, atol=1e-4, err_msg=k)


@pytest.mark.parametrize('name', CASES)
def test_block_thomas_short_flamelets(cuda, name):
    """Flamelets of 2 to 5 interior points (the fewest the flamelet Jacobian takes), where the twisted
    elimination's halves are empty or one block long, in one ragged batch: the factorization and solve against the
    reference's block-Thomas algorithm (the oracle)."""
    import torch
    import oracle as orc
    from spitfire_gb300.flamelet import FlameletBatch, FlameletSetup, FlameletSpec
    d, spec, og, setups0 = _setups(name, extra=False)
    oxy, fuel, kw = FC.flamelet_case_setup(spec, FC.case(name))
    rng = np.random.default_rng(21)
    setups = []
    for nzi in (2, 3, 4, 5):
        s = FlameletSetup(FlameletSpec(mech_spec=spec, initial_condition='Burke-Schumann',
                                       **dict(kw, grid_points=nzi + 2, stoich_dissipation_rate=2.)))
        assert s.nzi == nzi
        s.initial_state = np.abs(s.initial_state * (1. + 0.02 * rng.standard_normal(s.initial_state.size)))
        setups.append(s)
    b = FlameletBatch(setups)
    ops = _ops(og, setups)
    ns = b.ns
    x = torch.tensor(rng.standard_normal(b.npts * ns), dtype=torch.float64, device='cuda')
    b.jacobian(b.initial_state())
    b.values.neg_()
    b.factor()
    xsol = _split(b, b.solve(x))
    xs = _split(b, x)
    for f, s in enumerate(setups):
        dd, l, piv = orc.btddod_full_factorize(-ops[f].jac(s.initial_state), s.nzi, ns)
        ref = orc.btddod_full_solve(dd, l, piv, xs[f], s.nzi, ns)
        assert np.max(np.abs(xsol[f] - ref)) / np.max(np.abs(ref)) < 1e-9, f
    assert spec.griffon.device_status() == 0


def test_heat_loss_integration_matches_reference_trajectory(cuda):
    """Flamelet.integrate_for_heat_loss on the GPU kernels (ESDIRK64, simple Newton, PI control, block-Thomas
    setups) against the reference's own heat-loss trajectory of the H2 flamelet of
    tests/tabulation/nonadiabatic_defect_transient_slfm at chi_st = 1
    (tests/golden/nonadiabatic_transient_slfm_gold.npz): the same accepted-step count, step times and interior temperatures within 1e-7 relative, sampled mass
    fractions within 1e-5 relative (1e-9 absolute)."""
    import os
    from spitfire_gb300.flamelet import Flamelet, FlameletSpec
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    g = np.load(os.path.join(FC.GOLD, 'nonadiabatic_transient_slfm_gold.npz'))
    m = ChemicalMechanismSpec.bundled('h2-burke')
    air = m.stream(stp_air=True)
    air.TP = 1200., 101325.
    fuel = m.stream('TPY', (300., 101325., 'H2:1'))
    f = Flamelet(FlameletSpec(mech_spec=m, oxy_stream=air, fuel_stream=fuel, grid_points=34,
                              initial_condition=g['adiabatic_state'], stoich_dissipation_rate=1.,
                              heat_transfer='nonadiabatic', scale_heat_loss_by_temp_range=True,
                              scale_convection_by_dissipation=True, use_linear_ref_temp_profile=True,
                              convection_coefficient=1.e7, radiative_emissivity=0.))
    lib = f.integrate_for_heat_loss(first_time_step=1.e-9, max_time_step=1.e-1, transient_tolerance=1.e-10)
    t = lib.dim('time').values
    assert t.size == g['times'].size
    np.testing.assert_allclose(t, g['times'], rtol=1e-7)
    np.testing.assert_allclose(lib['temperature'], g['T'], rtol=1e-7)
    pick = g['pick']
    for i, n in enumerate(m.species_names):
        np.testing.assert_allclose(lib['mass fraction ' + n][pick], g['Y_pick'][:, :, i], rtol=1e-5, atol=1e-9,
                                   err_msg=n)
    assert m.griffon.device_status() == 0


def test_nonadiabatic_transient_slfm_library_matches_reference_gold(cuda):
    """tests/tabulation/nonadiabatic_defect_transient_slfm of the reference (h2-burke, air 1200 K / H2 300 K, 34
    points, chi_st = logspace(0, 1, 4), transient_tolerance 1e-10, 32 stoichiometric enthalpy defects) through the
    drop-in build_nonadiabatic_defect_transient_slfm_library: that test's bars (rtol 2e-4, atol 1e-4) on
    temperature, pressure, every mass fraction, the enthalpy and the enthalpy defect, and the library dimensions;
    the enthalpy recomputed from the library's states afterwards, as that test does."""
    import os
    from spitfire_gb300.analysis import compute_specific_enthalpy
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    from spitfire_gb300.tabulation import build_nonadiabatic_defect_transient_slfm_library
    g = np.load(os.path.join(FC.GOLD, 'nonadiabatic_transient_slfm_gold.npz'))
    m = ChemicalMechanismSpec.bundled('h2-burke')
    air = m.stream(stp_air=True)
    air.TP = 1200., 101325.
    fuel = m.stream('TPY', (300., 101325., 'H2:1'))
    lib = build_nonadiabatic_defect_transient_slfm_library(
        dict(mech_spec=m, oxy_stream=air, fuel_stream=fuel, grid_points=34), verbose=False,
        diss_rate_values=np.logspace(0, 1, 4), integration_args={'transient_tolerance': 1e-10}, num_procs=1)
    lib = compute_specific_enthalpy(m, lib)
    assert lib.dim_names == ['mixture_fraction', 'dissipation_rate_stoich', 'enthalpy_defect_stoich']
    np.testing.assert_allclose(lib.dims[0].values, g['dim0_values'], rtol=1e-14)
    np.testing.assert_allclose(lib.dims[1].values, g['dim1_values'], rtol=1e-12)
    np.testing.assert_allclose(lib.dims[2].values, g['dim2_values'], rtol=2e-4, atol=1e-4)
    keys = [k for k in g.files if k.startswith('prop:')]
    assert len(keys) == 4 + m.n_species
    for k in keys:
        np.testing.assert_allclose(lib[k[5:]], g[k], rtol=2e-4, atol=1e-4, err_msg=k)


@pytest.mark.parametrize('name', CASES)
def test_integrate_to_steady_matches_oracle_and_newton(cuda, name):
    """The ESDIRK64 path compute_steady_state falls back to (integrate_to_steady with steady tolerance 1e-6,
    transient tolerance 1e-8, steps up to 1e4 from 1e-8): from the case's perturbed Burke-Schumann profile, the
    accepted-step count of the oracle's restatement of odesolve within two steps and final states within 1e-5
    relative. The run stops when the step residual falls below 1e-6, and in the last steps the residual sits at the
    threshold to rounding (h2: 177 steps here, 178 in the oracle). The steady temperatures of the batched Newton
    solver agree within 1e-4 relative."""
    import torch
    import flamelet_steady as FS
    import flamelet_transient as FT
    from integrate import integrate
    from spitfire_gb300.flamelet import FlameletBatch
    d, spec, og, setups = _setups(name, extra=False)
    s = setups[0]
    b = FlameletBatch(setups)
    st0 = torch.tensor(s.initial_state, dtype=torch.float64, device='cuda')
    kw = dict(stop_at_steady=1.e-6, transient_tolerance=1.e-8, max_time_step=1.e4, first_time_step=1.e-8,
              maximum_steps_per_jacobian=10)
    traj, stats = b.integrate(st0, save_each_step=False, **kw)
    op = FS.FlameletOperator(og, s.z, s.x, s.state_oxy, s.state_fuel)
    r = integrate(FT.FlameletTransientProblem(op), s.initial_state, **kw)
    assert stats['status'][0] == 3
    assert abs(int(stats['steps'][0]) - r['steps']) <= 2
    np.testing.assert_allclose(traj[0][1][-1], r['state'], rtol=1e-5, atol=1e-10)
    newton, conv, _ = b.compute_steady_state(st0)
    assert bool(conv[0])
    ns = spec.n_species
    np.testing.assert_allclose(traj[0][1][-1][::ns], newton.cpu().numpy()[::ns], rtol=1e-4)


def test_adiabatic_ignition_transient_matches_reference(cuda):
    """Flamelet.integrate_to_time on the GPU kernels for an adiabatic H2 flamelet igniting from the linear T/Y
    profile (air 1200 K / H2 300 K, 34 points, chi_st = 1) to t = 2 ms, against the reference's own run
    (tests/golden/nonadiabatic_transient_slfm_gold.npz, 1216 accepted steps): the step count within three (over
    a thousand step-size decisions, rounding may move one), and the temperatures at the end time within 1e-6
    relative."""
    import os
    from spitfire_gb300.flamelet import Flamelet, FlameletSpec
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    g = np.load(os.path.join(FC.GOLD, 'nonadiabatic_transient_slfm_gold.npz'))
    m = ChemicalMechanismSpec.bundled('h2-burke')
    air = m.stream(stp_air=True)
    air.TP = 1200., 101325.
    fuel = m.stream('TPY', (300., 101325., 'H2:1'))
    f = Flamelet(FlameletSpec(mech_spec=m, oxy_stream=air, fuel_stream=fuel, grid_points=34,
                              initial_condition='linear-TY', stoich_dissipation_rate=1.))
    lib = f.integrate_to_time(2.e-3, first_time_step=1.e-6, transient_tolerance=1.e-10)
    t = lib.dim('time').values
    assert abs(t.size - g['ign_times'].size) <= 3
    assert t[-1] == 2.e-3
    np.testing.assert_allclose(lib['temperature'][-1], g['ign_T'][-1], rtol=1e-6)
    assert m.griffon.device_status() == 0


@pytest.mark.parametrize('name', CASES)
def test_native_steady_solvers_match_host_loop(cuda, name):
    """sf_flamelet_steady_newton_batch / sf_flamelet_steady_psitc_batch against the same solvers with their control
    loop on the host (FlameletBatch.steady_solve_*_host): both run the same device operations in the same order,
    so states, convergence flags, iteration counts and the last pseudo-time steps agree bit for bit, with a run
    mask, with failures that restart psitc (a low max_allowed_residual) and with a restart depth that gives up."""
    import torch
    from spitfire_gb300.flamelet import FlameletBatch
    d, spec, og, setups = _setups(name)
    setups[0].initial_state = d[name + '_ic'].copy()
    b = FlameletBatch(setups)
    init = b.initial_state()
    mask = torch.tensor([True, False, True], device=init.device)
    for kw in (dict(tolerance=1.e-6, max_iterations=38), dict(tolerance=1.e-6, max_iterations=38, active=mask),
               dict(tolerance=1.e-6, max_iterations=5, max_factor_line_search=1.01)):
        a = b.steady_solve_newton(init, **kw)
        h = b.steady_solve_newton_host(init, **kw)
        assert torch.equal(a[1], h[1]) and torch.equal(a[2], h[2]), (kw, a[1:], h[1:])
        assert torch.equal(a[0], h[0]), kw
    for kw in (dict(tolerance=1.e-6, max_iterations=400), dict(tolerance=1.e-6, max_iterations=400, active=~mask),
               dict(tolerance=1.e-6, max_iterations=60, max_allowed_residual=30., max_recursion_depth=2),
               dict(tolerance=1.e-6, max_iterations=60, global_ds=True, ds_init=10.),
               dict(tolerance=1.e-6, max_iterations=60, max_allowed_residual=30., adaptive_restart=False)):
        a = b.steady_solve_psitc(init, **kw)
        mds_a = b.last_psitc_min_ds.clone()
        h = b.steady_solve_psitc_host(init, **kw)
        mds_h = b.last_psitc_min_ds.clone()
        assert torch.equal(a[1], h[1]) and torch.equal(a[2], h[2]), (kw, a[1:], h[1:])
        assert torch.equal(a[0], h[0]), kw
        assert torch.equal(mds_a, mds_h), (kw, mds_a, mds_h)
    assert spec.griffon.device_status() == 0


def test_native_transient_attempts_match_host_attempts(cuda):
    """The transient integrator's native step attempt (sf_flamelet_esdirk_attempt_batch) against the same attempt as
    torch operations (host_attempts=True) on a ragged batch of a nonadiabatic and an adiabatic H2 flamelet of
    different grids and dissipation rates: bit-identical step times, states and counters over the whole run, with
    Jacobian reuse, rejected steps and an end time."""
    import os
    from spitfire_gb300.flamelet import FlameletBatch, FlameletSetup, FlameletSpec, _integrate_batch
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    g = np.load(os.path.join(FC.GOLD, 'nonadiabatic_transient_slfm_gold.npz'))
    m = ChemicalMechanismSpec.bundled('h2-burke')
    air = m.stream(stp_air=True)
    air.TP = 1200., 101325.
    fuel = m.stream('TPY', (300., 101325., 'H2:1'))
    common = dict(mech_spec=m, oxy_stream=air, fuel_stream=fuel)
    heat = FlameletSetup(FlameletSpec(grid_points=34, initial_condition=g['adiabatic_state'],
                                      stoich_dissipation_rate=1., heat_transfer='nonadiabatic',
                                      scale_heat_loss_by_temp_range=True, scale_convection_by_dissipation=True,
                                      use_linear_ref_temp_profile=True, convection_coefficient=1.e7,
                                      radiative_emissivity=0., **common))
    ign = FlameletSetup(FlameletSpec(grid_points=21, initial_condition='linear-TY', stoich_dissipation_rate=3.,
                                     **common))
    # 2e-5 s: the heat-loss flamelet is still burning (its loss coefficient is divided by max T - T_conv, which
    # vanishes once it has cooled to the oxidizer temperature), the other is igniting
    kw = dict(stop_at_time=2.e-5, first_time_step=1.e-8, max_time_step=1.e-4, transient_tolerance=1.e-10,
              maximum_steps_per_jacobian=5, max_attempts=5000)
    b = FlameletBatch([heat, ign])
    tn, sn = _integrate_batch(b, **kw)
    b2 = FlameletBatch([heat, ign])
    th, sh = _integrate_batch(b2, host_attempts=True, **kw)
    for key in ('steps', 'failed_steps', 'newton_iters', 'jac_setups', 'status'):
        assert np.array_equal(sn[key], sh[key]), (key, sn[key], sh[key])
    assert sn['steps'].min() > 20 and (sn['status'] == 1).all()
    for f in range(2):
        assert np.array_equal(tn[f][0], th[f][0]), f
        assert np.array_equal(tn[f][1], th[f][1]), f
    assert m.griffon.device_status() == 0
