"""GPU parity of the batched kernels against the oracle (CPU restatement of Griffon), through the C ABI.

Bar: row-normwise relative error <= 1e-10 in FP64 (per state, max_i |gpu_i - ref_i| / max_j |ref_ij| over each
row of the RHS / Jacobian / sensitivity block).
"""
import numpy as np
import pytest

from helpers import colmajor, pair, rownorm_err
from spitfire_gb300 import workloads as W
from spitfire_gb300._desc import reactor_params

pytestmark = pytest.mark.gpu
TOL = 1e-10
UNIT_MECHS = ['unit-rev_troe4_withN_withNTB', 'unit-rev_lindemann_withN_withNTB', 'unit-rev_3body_withN_withN_nonUnity',
              'unit-rev_elementary_withNreactant_generalstoich_in_products',
              'unit-rev_elementary_withNproduct_generalstoich_in_reactants', 'unit-irr_elementary_withN_withT',
              'unit-rev_troe3_noN_noNTB', 'unit-methane-lu30', 'unit-hydrogen-burke']


def random_states(spec, n, seed, T=(300., 2800.)):
    rng = np.random.default_rng(seed)
    ns = spec.n_species
    Tv = rng.uniform(*T, n)
    p = 101325. * np.exp(rng.uniform(0., np.log(40.), n))
    Y = rng.dirichlet(0.5 * np.ones(ns), n)
    mmw = 1. / (Y / spec.molecular_weights).sum(1)
    rho = p * mmw / (8314.46261815324 * Tv)
    return dict(T=Tv, p=p, Y=Y, rho=rho)


def gpu_np(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize('name', ['h2-burke', 'methane-gri30', 'reaction-test'] + UNIT_MECHS)
def test_production_rates_and_sensitivities(cuda, name):
    spec, og = pair(name)
    g = spec.griffon
    d = random_states(spec, 64, 7)
    w = gpu_np(g.production_rates_batch(d['T'], d['rho'], d['Y']))
    wo = og.production_rates_batch(d['T'], d['rho'], d['Y'])
    assert rownorm_err(w, wo) <= TOL
    ns = spec.n_species
    for opt in (0, 1, 2):
        w2, S = g.rates_sens_batch(d['rho'], d['T'], d['Y'], opt)
        wo2, So = og.rates_sens_batch(d['rho'], d['T'], d['Y'], opt)
        assert rownorm_err(gpu_np(w2), wo2) <= TOL, opt
        assert rownorm_err(colmajor(gpu_np(S), ns + 1)[:, :ns], colmajor(So, ns + 1)[:, :ns]) <= TOL, opt


@pytest.mark.parametrize('name', ['h2-burke', 'methane-gri30'] + UNIT_MECHS)
@pytest.mark.parametrize('configuration', ['isochoric', 'isobaric'])
@pytest.mark.parametrize('heat', ['adiabatic', 'isothermal', 'diathermal'])
def test_reactor_rhs_jac(cuda, name, configuration, heat):
    import oracle as orc
    spec, og = pair(name)
    g = spec.griffon
    d = random_states(spec, 48, 11)
    q = W.isochoric_state(d) if configuration == 'isochoric' else W.isobaric_state(d)
    neq = q.shape[1]
    P = reactor_params(configuration, heat, pressure=101325., fluid_temperature=600., surface_temperature=900.,
                       h_convection=50., eps_radiation=0.3, surface_area_to_volume=20.)
    yin = np.zeros(spec.n_species)
    P.inflow_Y = orc._p(yin)
    pres = d['p'] if configuration == 'isobaric' else None
    rhs = gpu_np(g.reactor_rhs_batch(P, q, pressures=pres))
    rhso = og.reactor_rhs_batch(P, q, pressures=pres)
    assert rownorm_err(rhs, rhso) <= TOL
    for opt in (0, 2):
        r2, J = g.reactor_jac_batch(P, q, opt, pressures=pres)
        ro2, Jo = og.reactor_jac_batch(P, q, opt, pressures=pres)
        assert rownorm_err(gpu_np(r2), ro2) <= TOL
        assert rownorm_err(colmajor(gpu_np(J), neq), colmajor(Jo, neq)) <= TOL


@pytest.mark.parametrize('name', ['h2-burke', 'methane-gri30'])
@pytest.mark.parametrize('configuration', ['isochoric', 'isobaric'])
def test_plain_kernel_matches(cuda, name, configuration):
    import oracle as orc
    spec, og = pair(name)
    g = spec.griffon
    d = W.h2_states(spec, 40) if name == 'h2-burke' else W.gri_states(spec, 40)
    q = W.isochoric_state(d) if configuration == 'isochoric' else W.isobaric_state(d)
    neq = q.shape[1]
    P = reactor_params(configuration, 'adiabatic', pressure=101325.)
    yin = np.zeros(spec.n_species)
    P.inflow_Y = orc._p(yin)
    pres = d['p'] if configuration == 'isobaric' else None
    r, J = g.reactor_jac_plain_batch(P, q, pressures=pres)
    ro, Jo = og.reactor_jac_batch(P, q, 0, pressures=pres)
    assert rownorm_err(gpu_np(r), ro) <= TOL
    assert rownorm_err(colmajor(gpu_np(J), neq), colmajor(Jo, neq)) <= TOL


def test_reaction_test_mechanism_jacobian_species_rows(cuda):
    """The artificial test mechanism has catastrophic cancellation in the temperature row (huge cp of species B);
    the species rows are compared."""
    import oracle as orc
    spec, og = pair('reaction-test')
    g = spec.griffon
    d = random_states(spec, 32, 3)
    q = W.isochoric_state(d)
    P = reactor_params('isochoric')
    yin = np.zeros(spec.n_species)
    P.inflow_Y = orc._p(yin)
    r, J = g.reactor_jac_batch(P, q, 0)
    ro, Jo = og.reactor_jac_batch(P, q, 0)
    n1 = spec.n_species + 1
    assert rownorm_err(colmajor(gpu_np(J), n1)[:, 2:], colmajor(Jo, n1)[:, 2:]) <= TOL


@pytest.mark.parametrize('precision', [0, 1])
def test_newton_lu_solve(cuda, precision):
    import torch
    import oracle as orc
    from spitfire_gb300 import _native as N
    spec, og = pair('methane-gri30')
    g = spec.griffon
    d = W.gri_states(spec, 64)
    q = W.isochoric_state(d)
    P = reactor_params('isochoric')
    yin = np.zeros(spec.n_species)
    P.inflow_Y = orc._p(yin)
    rhs, J = g.reactor_jac_batch(P, q, 0)
    n, m = q.shape
    gh = torch.tensor(d['gamma_h'], dtype=torch.float64, device='cuda')
    A = torch.empty_like(J)
    lu = torch.empty(n, m * m, dtype=torch.float64 if precision == 0 else torch.float32, device='cuda')
    piv = torch.empty(n, m, dtype=torch.int32, device='cuda')
    info = torch.empty(n, dtype=torch.int32, device='cuda')
    L = N.load()
    N.check(L.sf_newton_lu_batch(n, m, N.ptr(J), N.ptr(gh), precision, N.ptr(A), N.ptr(lu), N.ptr(piv), N.ptr(info),
                                 N.stream_handle()))
    x = torch.empty_like(rhs)
    N.check(L.sf_newton_solve_batch(n, m, N.ptr(A), N.ptr(lu), N.ptr(piv), precision, 2, N.ptr(rhs), N.ptr(x),
                                    N.stream_handle()))
    torch.cuda.synchronize()
    An = colmajor(gpu_np(A), m)
    xg, bg = gpu_np(x), gpu_np(rhs)
    # normwise backward error |b - A x| / (|A| |x| + |b|): the Newton matrices gamma*h*J - I are ill-conditioned,
    # so the forward error of any FP64 solver is cond(A) * eps; the backward error is what LU + refinement bound
    res = np.abs(bg - np.einsum('kij,kj->ki', An, xg)).max(1)
    scale = np.abs(An).sum(2).max(1) * np.abs(xg).max(1) + np.abs(bg).max(1)
    assert (gpu_np(info) == 0).all()
    assert (res / scale).max() <= (1e-14 if precision == 0 else 1e-13)
    # the same pivoted factorization as the oracle (LAPACK dgetrf semantics): solutions agree to cond * eps
    import oracle as orc
    LU, pv, inf = orc.lu_factor_batch(gpu_np(A))
    xo = orc.lu_solve_batch(LU, pv, bg)
    cond = np.array([np.linalg.cond(An[k], np.inf) for k in range(n)])
    fwd = np.abs(xg - xo).max(1) / np.abs(xo).max(1)
    assert (fwd <= 1e3 * cond * 2.2e-16 + 1e-13).all()


def _tps_check(spec, og, d, heats, rates=True, species_only=False):
    import oracle as orc
    g = spec.griffon
    if rates:
        w = gpu_np(g.production_rates_batch(d['T'], d['rho'], d['Y']))
        assert rownorm_err(w, og.production_rates_batch(d['T'], d['rho'], d['Y'])) <= TOL
        ns = spec.n_species
        for opt in (0, 1, 2):
            w2, S = g.rates_sens_batch(d['rho'], d['T'], d['Y'], opt)
            wo2, So = og.rates_sens_batch(d['rho'], d['T'], d['Y'], opt)
            assert rownorm_err(gpu_np(w2), wo2) <= TOL, opt
            assert rownorm_err(colmajor(gpu_np(S), ns + 1)[:, :ns], colmajor(So, ns + 1)[:, :ns]) <= TOL, opt
    for configuration in ('isochoric', 'isobaric'):
        q = W.isochoric_state(d) if configuration == 'isochoric' else W.isobaric_state(d)
        neq = q.shape[1]
        for heat in heats:
            P = reactor_params(configuration, heat, pressure=101325., fluid_temperature=600.,
                               surface_temperature=900., h_convection=50., eps_radiation=0.3,
                               surface_area_to_volume=20.)
            P.inflow_Y = orc._p(np.zeros(spec.n_species))
            pres = d['p'] if configuration == 'isobaric' else None
            # species entries only where the temperature row cancels catastrophically (the artificial test
            # mechanism, see the test above)
            sp = slice(neq - spec.n_species + 1, None) if species_only else slice(None)
            rhs = gpu_np(g.reactor_rhs_batch(P, q, pressures=pres))
            assert rownorm_err(rhs[:, sp], og.reactor_rhs_batch(P, q, pressures=pres)[:, sp]) <= TOL
            r2, J = g.reactor_jac_batch(P, q, 0, pressures=pres)
            ro2, Jo = og.reactor_jac_batch(P, q, 0, pressures=pres)
            assert rownorm_err(gpu_np(r2)[:, sp], ro2[:, sp]) <= TOL
            assert rownorm_err(colmajor(gpu_np(J), neq)[:, sp], colmajor(Jo, neq)[:, sp]) <= TOL
    assert g.device_status() == 0


def _tps_on(spec, ctas):
    from spitfire_gb300 import autotune as AT
    for k in ('group_rates', 'group_sens', 'group_rhs', 'group_jac'):
        AT.set_tuning(spec, k, 1)
    AT.set_tuning(spec, 'tps_ctas', ctas)


def _tps_off(spec):
    from spitfire_gb300 import autotune as AT
    for k in AT.KNOBS:
        AT.set_tuning(spec, k, 0)


@pytest.mark.parametrize('name', ['h2-burke', 'methane-gri30', 'reaction-test'] + UNIT_MECHS)
def test_thread_per_state_kernels(cuda, name):
    """Lanes-per-state knob 1 (each lane one state, scratch interleaved across the warp in global memory): rates,
    sensitivities, right-hand sides and Jacobians at the same bar, on a batch that is not a multiple of 32."""
    spec, og = pair(name)
    try:
        _tps_on(spec, 0)
        _tps_check(spec, og, random_states(spec, 100, 23), ('adiabatic', 'diathermal'),
                   species_only=name == 'reaction-test')
    finally:
        _tps_off(spec)


@pytest.mark.parametrize('name', ['h2-burke', 'methane-gri30'])
def test_thread_per_state_grid_stride(cuda, name):
    """One 4-warp block per SM and more states than resident lanes: the thread-per-state kernels loop over warp
    batches (ignition-range states of the workload distributions)."""
    spec, og = pair(name)
    n = 152 * 128 + 77
    d = W.h2_states(spec, n) if name == 'h2-burke' else W.gri_states(spec, n)
    try:
        _tps_on(spec, 1)
        _tps_check(spec, og, d, ('adiabatic',), rates=name == 'methane-gri30')
    finally:
        _tps_off(spec)


@pytest.mark.parametrize('name', ['h2-burke', 'methane-gri30', 'unit-rev_troe4_withN_withNTB', 'unit-methane-lu30'])
@pytest.mark.parametrize('configuration', ['isochoric', 'isobaric'])
@pytest.mark.parametrize('heat', ['adiabatic', 'isothermal', 'diathermal'])
@pytest.mark.parametrize('group', [0, 1])
def test_open_reactor_rhs_jac(cuda, name, configuration, heat, group):
    """Open (mass-exchange) reactors: feed temperature, mass fractions (a device array), mixing time and feed density,
    with the lane-group and thread-per-state kernels."""
    import oracle as orc
    import torch
    from spitfire_gb300 import autotune as AT
    spec, og = pair(name)
    g = spec.griffon
    d = random_states(spec, 70, 31)
    q = W.isochoric_state(d) if configuration == 'isochoric' else W.isobaric_state(d)
    neq = q.shape[1]
    rng = np.random.default_rng(32)
    yin = rng.dirichlet(0.5 * np.ones(spec.n_species))
    yin_d = torch.tensor(yin, dtype=torch.float64, device='cuda')
    kw = dict(pressure=101325., inflow_density=0.7, inflow_temperature=650., tau=3.e-4, fluid_temperature=600.,
              surface_temperature=900., h_convection=50., eps_radiation=0.3, surface_area_to_volume=20.)
    P = reactor_params(configuration, heat, True, inflow_Y_ptr=yin_d.data_ptr(), **kw)
    Po = reactor_params(configuration, heat, True, **kw)
    Po.inflow_Y = orc._p(yin)
    pres = d['p'] if configuration == 'isobaric' else None
    try:
        if group:
            AT.set_tuning(spec, 'group_rhs', 1)
            AT.set_tuning(spec, 'group_jac', 1)
        rhs = gpu_np(g.reactor_rhs_batch(P, q, pressures=pres))
        assert rownorm_err(rhs, og.reactor_rhs_batch(Po, q, pressures=pres)) <= TOL
        r2, J = g.reactor_jac_batch(P, q, 0, pressures=pres)
        ro2, Jo = og.reactor_jac_batch(Po, q, 0, pressures=pres)
        assert rownorm_err(gpu_np(r2), ro2) <= TOL
        assert rownorm_err(colmajor(gpu_np(J), neq), colmajor(Jo, neq)) <= TOL
        assert g.device_status() == 0
    finally:
        _tps_off(spec)


@pytest.mark.parametrize('group', [0, 1])
def test_host_buffer_jacobians_match_device_path(cuda, group):
    """sf_reactor_jac_host_batch (host states in, host results out, chunked with overlapped copies) gives the
    device entry point's results bit for bit, for pinned and pageable buffers (aligned or not) and several chunk
    sizes."""
    import torch
    from spitfire_gb300 import autotune as AT
    spec, og = pair('methane-gri30')
    g = spec.griffon
    n = 3000
    d = W.gri_states(spec, n, seed=41)
    qh = W.isochoric_state(d)
    neq = qh.shape[1]
    P = reactor_params('isochoric')
    try:
        if group:
            AT.set_tuning(spec, 'group_jac', 1)
        r_ref, J_ref = g.reactor_jac_batch(P, qh, 0)
        r_ref, J_ref = gpu_np(r_ref), gpu_np(J_ref)
        for chunk in (0, 1000, 777, n):
            qp = torch.from_numpy(qh).pin_memory()
            rh = torch.empty((n, neq), dtype=torch.float64).pin_memory()
            Jh = torch.empty((n, neq * neq), dtype=torch.float64).pin_memory()
            g.reactor_jac_host_batch(P, qp, rh, Jh, chunk_states=chunk)
            torch.cuda.synchronize()
            assert np.array_equal(rh.numpy(), r_ref) and np.array_equal(Jh.numpy(), J_ref), chunk
        rn, Jn = np.zeros((n, neq)), np.zeros((n, neq * neq))
        g.reactor_jac_host_batch(P, np.ascontiguousarray(qh), rn, Jn, chunk_states=1234)
        torch.cuda.synchronize()
        assert np.array_equal(rn, r_ref) and np.array_equal(Jn, J_ref)
        # pinned outputs at an 8-byte offset into their allocations
        rb = torch.empty(n * neq + 1, dtype=torch.float64).pin_memory()
        Jb = torch.empty(n * neq * neq + 1, dtype=torch.float64).pin_memory()
        rv, Jv = rb[1:].view(n, neq), Jb[1:].view(n, neq * neq)
        g.reactor_jac_host_batch(P, torch.from_numpy(qh).pin_memory(), rv, Jv)
        torch.cuda.synchronize()
        assert np.array_equal(rv.numpy(), r_ref) and np.array_equal(Jv.numpy(), J_ref)
        assert g.device_status() == 0
    finally:
        _tps_off(spec)
