"""Edge cases of the batched entry points on the GPU: empty batches (every call returns without launching and
without touching its null outputs), single-state batches of the thread-per-state kernels against the lane-group
kernels, and the native steady flamelet solvers with every flamelet masked out."""
import numpy as np
import pytest

from helpers import pair

pytestmark = pytest.mark.gpu


def test_empty_batches_return_without_work(cuda):
    import torch
    from spitfire_gb300 import workloads as W
    from spitfire_gb300._desc import reactor_params
    from spitfire_gb300.adjoint import ReactorAdjoint
    from spitfire_gb300.linalg import NewtonSystems
    from spitfire_gb300.reactors import BatchIntegrator
    spec, og = pair('methane-gri30')
    g = spec.griffon
    ns = spec.n_species
    e = lambda *shape: torch.empty(shape, dtype=torch.float64, device='cuda')
    assert g.thermo_batch(0, e(0), e(0, ns)).shape == (0,)
    assert g.production_rates_batch(e(0), e(0), e(0, ns)).shape == (0, ns)
    w, S = g.rates_sens_batch(e(0), e(0), e(0, ns), option=2)
    assert w.shape == (0, ns) and S.shape == (0, (ns + 1) ** 2)
    for conf, neq in (('isochoric', ns + 1), ('isobaric', ns)):
        P = reactor_params(conf)
        assert g.reactor_rhs_batch(P, e(0, neq)).shape == (0, neq)
        rhs, J = g.reactor_jac_batch(P, e(0, neq))
        assert rhs.shape == (0, neq) and J.shape == (0, neq * neq)
        qh = torch.empty((0, neq), dtype=torch.float64).pin_memory()
        g.reactor_jac_host_batch(P, qh, torch.empty((0, neq), dtype=torch.float64),
                                 torch.empty((0, neq * neq), dtype=torch.float64))
    ns_sys = NewtonSystems(0, ns + 1, 0).factor(e(0, (ns + 1) ** 2), e(0))
    assert ns_sys.solve(e(0, ns + 1)).shape == (0, ns + 1)
    bi = BatchIntegrator(spec, 'isobaric')
    out = bi.run(e(0, ns), pressures=e(0), delta_temperature_ignition=400., stop_at_time=0.1)
    assert out['q'].shape == (0, ns) and out['status'].numel() == 0
    adj = ReactorAdjoint(spec, 'isobaric')
    tr = adj.forward(e(0, ns), pressures=e(0), t_end=1.e-4)
    gr = adj.backward(tr)
    assert gr['theta'].shape[0] == 0 and gr['q0'].shape[0] == 0
    torch.cuda.synchronize()
    assert g.device_status() == 0
    # one state still works after the empty calls
    d = W.gri_states(spec, 1, seed=41)
    rhs, J = g.reactor_jac_batch(reactor_params('isochoric'), W.isochoric_state(d))
    assert bool(torch.isfinite(J).all())


@pytest.mark.parametrize('n', [1, 31, 33, 129])
def test_thread_per_state_partial_warps_match_lane_groups(cuda, n):
    """Batches that leave lanes or warps of the thread-per-state launch without a state (n below, at and just past
    a warp, and past a 4-warp block) give the lane-group kernel's results to rounding (1e-13 row-normwise: the two
    shapes sum per-species terms in different orders)."""
    import torch
    from helpers import colmajor, rownorm_err
    from spitfire_gb300 import autotune as AT
    from spitfire_gb300 import workloads as W
    from spitfire_gb300._desc import reactor_params
    spec, og = pair('methane-gri30')
    g = spec.griffon
    d = W.gri_states(spec, n, seed=43 + n)
    q = W.isochoric_state(d)
    P = reactor_params('isochoric')
    neq = q.shape[1]
    saved = AT.get_tuning(spec, 'group_jac')
    try:
        AT.set_tuning(spec, 'group_jac', 32)
        r32, J32 = g.reactor_jac_batch(P, q)
        AT.set_tuning(spec, 'group_jac', 1)
        r1, J1 = g.reactor_jac_batch(P, q)
    finally:
        AT.set_tuning(spec, 'group_jac', saved)
    torch.cuda.synchronize()
    assert rownorm_err(r1.cpu().numpy()[:, None, :], r32.cpu().numpy()[:, None, :]) < 1e-13
    assert rownorm_err(colmajor(J1.cpu().numpy(), neq), colmajor(J32.cpu().numpy(), neq)) < 1e-13
    assert g.device_status() == 0


def test_native_steady_solvers_with_every_flamelet_masked_out(cuda):
    """All flamelets inactive: the native solvers iterate nothing, report no convergence and zero iterations, and
    return the initial guess clamped at zero, as the host-loop solvers do."""
    import torch
    import flamelet_cases as FC
    from spitfire_gb300.flamelet import FlameletBatch, FlameletSetup, FlameletSpec
    spec, og = pair('h2-burke')
    oxy, fuel, kw = FC.flamelet_case_setup(spec, FC.case('h2'))
    setups = [FlameletSetup(FlameletSpec(mech_spec=spec, initial_condition='Burke-Schumann',
                                         **dict(kw, grid_points=npts))) for npts in (9, 14)]
    b = FlameletBatch(setups)
    init = b.initial_state()
    none = torch.zeros(b.nf, dtype=torch.bool, device=init.device)
    for solve, host in ((b.steady_solve_newton, b.steady_solve_newton_host),
                        (b.steady_solve_psitc, b.steady_solve_psitc_host)):
        s, conv, it = solve(init, active=none, tolerance=1.e-6, max_iterations=10)
        hs, hconv, hit = host(init, active=none, tolerance=1.e-6, max_iterations=10)
        assert not bool(conv.any()) and int(it.abs().sum()) == 0
        assert torch.equal(s, torch.clamp(init, min=0.)) and torch.equal(s, hs)
        assert torch.equal(conv, hconv) and torch.equal(it, hit)
    assert spec.griffon.device_status() == 0
