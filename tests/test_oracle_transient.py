"""Oracle transient flamelet integration and transient enthalpy-defect library against the reference (CPU).

Pins oracle/flamelet_transient.py: the heat-loss integration of one H2 flamelet against the reference's own
trajectory (tests/golden/nonadiabatic_transient_slfm_gold.npz, made by tests/golden/make_golden.py transient): the
same accepted-step count, step times within 1e-7 and temperatures within 1e-7 relative. And the whole transient
defect library of the reference test tests/tabulation/nonadiabatic_defect_transient_slfm against its gold within
that test's bars (rtol 2e-4, atol 1e-4).
"""
import os

import numpy as np

import flamelet_cases as FC
from helpers import pair

GOLD = os.path.join(FC.GOLD, 'nonadiabatic_transient_slfm_gold.npz')
HEAT = dict(heat_transfer='nonadiabatic', scale_heat_loss_by_temp_range=True, scale_convection_by_dissipation=True,
            use_linear_ref_temp_profile=True, convection_coefficient=1.e7, radiative_emissivity=0.)


def _streams(spec):
    air = spec.stream(stp_air=True)
    air.TP = 1200., 101325.
    fuel = spec.stream('TPY', (300., 101325., 'H2:1'))
    return air, fuel


def _heat_op(og, s):
    import flamelet_steady as FS
    return FS.FlameletOperator(og, s.z, s.x, s.state_oxy, s.state_fuel,
                               heat_loss=dict(T_conv=s.T_conv, T_rad=s.T_rad, h_conv=s.h_conv, h_rad=s.h_rad,
                                              scaled=s.scale_heat_loss_by_temp_range))


def test_oracle_heat_loss_integration_matches_reference_trajectory():
    import flamelet_transient as FT
    from spitfire_gb300.flamelet import FlameletSetup, FlameletSpec
    g = np.load(GOLD)
    spec, og = pair('h2-burke')
    air, fuel = _streams(spec)
    s = FlameletSetup(FlameletSpec(mech_spec=spec, oxy_stream=air, fuel_stream=fuel, grid_points=34,
                                   initial_condition=g['adiabatic_state'], stoich_dissipation_rate=1., **HEAT))
    np.testing.assert_allclose(s.z, g['z'], rtol=1e-14)
    for a, b in ((s.T_conv, 'T_conv'), (s.h_conv, 'h_conv'), (s.T_rad, 'T_rad'), (s.h_rad, 'h_rad')):
        np.testing.assert_allclose(a, g[b], rtol=1e-13, atol=0., err_msg=b)
    r = FT.integrate_for_heat_loss(_heat_op(og, s), g['adiabatic_state'], max(air.T, fuel.T),
                                   first_time_step=1.e-9, max_time_step=1.e-1, transient_tolerance=1.e-10)
    assert r['steps'] == g['times'].size - 1
    np.testing.assert_allclose(r['times'], g['times'], rtol=1e-7)
    ns = spec.n_species
    np.testing.assert_allclose(r['states'][:, ::ns], g['T'][:, 1:-1], rtol=1e-7)
    pick = g['pick']
    for i in range(ns - 1):
        np.testing.assert_allclose(r['states'][pick, 1 + i::ns], g['Y_pick'][:, 1:-1, i], rtol=1e-5, atol=1e-9)


def oracle_transient_library(h_stoich_spacing=10.e3, n_defect_st=32, diss_rate_values=np.logspace(0, 1, 4),
                             transient_tolerance=1.e-10):
    """The reference test's library built from the oracle: the adiabatic continuation in the stoichiometric
    dissipation rate (oracle compute_steady_state, the first flamelet from the Burke-Schumann profile), each rate's
    heat-loss integration, the defect subsampling, then the structured defect dimension (the same host-side
    interpolation the GPU builder uses). Returns (dims, props)."""
    import flamelet_steady as FS
    import flamelet_transient as FT
    from spitfire_gb300.flamelet import FlameletSetup, FlameletSpec, compute_dissipation_rate
    from spitfire_gb300.tabulation import _structure_defect
    spec, og = pair('h2-burke')
    air, fuel = _streams(spec)
    names = spec.species_names
    unstructured = {}
    ic = 'Burke-Schumann'
    for chi in diss_rate_values:
        s = FlameletSetup(FlameletSpec(mech_spec=spec, oxy_stream=air, fuel_stream=fuel, grid_points=34,
                                       initial_condition=ic, stoich_dissipation_rate=float(chi)))
        op = FS.FlameletOperator(og, s.z, s.x, s.state_oxy, s.state_fuel)
        ad, how, it = FS.compute_steady_state(op, s.initial_state)
        assert ad is not None
        ic = ad
        chi_st = compute_dissipation_rate(np.array([s.z_st]), s.max_dissipation_rate, s.form)[0]
        sh = FlameletSetup(FlameletSpec(mech_spec=spec, oxy_stream=air, fuel_stream=fuel, grid_points=34,
                                        initial_condition=ad, stoich_dissipation_rate=float(chi), **HEAT))
        r = FT.integrate_for_heat_loss(_heat_op(og, sh), ad, max(air.T, fuel.T), first_time_step=1.e-9,
                                       max_time_step=1.e-1, transient_tolerance=transient_tolerance)
        unstructured.update(FT.transient_defect_entries(og, chi_st, sh.z, sh.z_st, r['states'], sh.state_oxy,
                                                        sh.state_fuel, sh.pressure, names, h_stoich_spacing))
    table, xs, gs = _structure_defect(unstructured, n_defect_st)
    key0 = next(iter(table))
    nz = table[key0]['mixture_fraction'].size
    props = {}
    for q in table[key0]:
        v = np.empty((nz, xs.size, gs.size))
        for ix, x in enumerate(xs):
            for ig, gg in enumerate(gs):
                v[:, ix, ig] = table[(x, gg)][q]
        props[q] = v
    # the reference test recomputes the enthalpy from the library's states (analysis.compute_specific_enthalpy)
    Y = np.stack([props['mass fraction ' + n] for n in names], axis=-1)
    T = props['temperature']
    props['enthalpy'] = np.array([og.enthalpy_mix(t, y) for t, y in zip(T.ravel(), Y.reshape(-1, len(names)))]
                                 ).reshape(T.shape)
    return (table[key0]['mixture_fraction'], xs, gs), props


def test_oracle_transient_defect_library_matches_reference_gold():
    g = np.load(GOLD)
    (z, xs, gs), props = oracle_transient_library()
    np.testing.assert_allclose(z, g['dim0_values'], rtol=1e-14)
    np.testing.assert_allclose(xs, g['dim1_values'], rtol=1e-12)
    np.testing.assert_allclose(gs, g['dim2_values'], rtol=2e-4, atol=1e-4)
    keys = [k for k in g.files if k.startswith('prop:')]
    for k in keys:
        np.testing.assert_allclose(props[k[5:]], g[k], rtol=2e-4, atol=1e-4, err_msg=k)


def test_oracle_adiabatic_ignition_transient_matches_reference():
    """An adiabatic H2 flamelet (same streams and grid) igniting from the linear T/Y profile, integrated to
    t = 2 ms by the reference's Flamelet.integrate_to_time (first step 1e-6, tolerance 1e-10): the oracle takes
    the same accepted steps, with step times and temperatures within 1e-7 relative."""
    import flamelet_steady as FS
    import flamelet_transient as FT
    from integrate import integrate
    from spitfire_gb300.flamelet import FlameletSetup, FlameletSpec
    g = np.load(GOLD)
    spec, og = pair('h2-burke')
    air, fuel = _streams(spec)
    s = FlameletSetup(FlameletSpec(mech_spec=spec, oxy_stream=air, fuel_stream=fuel, grid_points=34,
                                   initial_condition='linear-TY', stoich_dissipation_rate=1.))
    np.testing.assert_allclose(s.initial_state, g['ign_ic'], rtol=1e-14)
    op = FS.FlameletOperator(og, s.z, s.x, s.state_oxy, s.state_fuel)
    r = integrate(FT.FlameletTransientProblem(op), s.initial_state, stop_at_time=2.e-3, first_time_step=1.e-6,
                  max_time_step=1.e-3, transient_tolerance=1.e-10, maximum_steps_per_jacobian=10,
                  save_each_step=True)
    assert r['steps'] == g['ign_times'].size - 1
    np.testing.assert_allclose(r['times'], g['ign_times'], rtol=1e-7)
    np.testing.assert_allclose(r['states'][:, ::spec.n_species], g['ign_T'][:, 1:-1], rtol=1e-7)
