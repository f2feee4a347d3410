"""GPU adjoint gradients of reactor integrations with respect to ln A and E_a of every reaction.

There is no reference counterpart (the reference computes no parameter sensitivities); the checks are the oracle's
project-written CPU forward sensitivity (exact derivative of the same discrete step sequence) and central finite
differences of the oracle integration on the frozen step sequence (relative step 1e-6). Bars: the parameter-adjoint
kernel 1e-10 against the oracle; the batched adjoint 1e-7 normwise against the forward sensitivity; 1e-5 normwise
(relative to the largest gradient) against finite differences, whose own floor is the Newton tolerance (1e-12
weighted residual, about 1e-9 K per stage).
"""
import numpy as np
import pytest

from helpers import pair

pytestmark = pytest.mark.gpu


def _oracle_1thread():
    import oracle as orc
    orc.set_threads(1)


def test_rate_param_adjoint_kernel_matches_oracle(cuda):
    import torch
    import ctypes as C
    import sensitivity as SE
    from spitfire_gb300 import _native as N
    from spitfire_gb300 import workloads as W
    from spitfire_gb300._desc import reactor_params
    _oracle_1thread()
    for name in ('h2-burke', 'methane-gri30'):
        spec, og = pair(name)
        d = W.gri_states(spec, 6, seed=11) if name == 'methane-gri30' else W.h2_states(spec, 6, seed=11)
        q = W.isobaric_state(d)
        rng = np.random.default_rng(3)
        w = rng.standard_normal(q.shape)
        nr = len(spec.mech_data['reactions'])
        P = reactor_params('isobaric')
        out = torch.zeros((6, 2 * nr), dtype=torch.float64, device='cuda')
        qt = torch.tensor(q, device='cuda')
        wt = torch.tensor(w, device='cuda')
        pt = torch.tensor(d['p'], device='cuda')
        N.check(N.load().sf_rate_param_adjoint_batch(spec.griffon.handle, C.byref(P), 6, 1, N.ptr(qt), N.ptr(pt),
                                                     N.ptr(wt), N.ptr(out), N.stream_handle()))
        got = out.cpu().numpy()
        for i in range(6):
            F = SE.ParamJacobian(spec, og, 'isobaric', d['p'][i])(q[i])
            ref = w[i] @ F
            err = np.max(np.abs(got[i] - ref)) / np.max(np.abs(ref))
            assert err < 1e-10, (name, i, err)
    assert spec.griffon.device_status() == 0


def _h2_reactors(spec, n):
    X = np.zeros(spec.n_species)
    X[spec.species_index('H2')] = 2.
    X[spec.species_index('O2')] = 1.
    X[spec.species_index('N2')] = 3.76
    Y = X * spec.molecular_weights
    Y /= Y.sum()
    T0 = np.linspace(1000., 1200., n)
    return np.hstack([T0[:, None], np.repeat(Y[None, :-1], n, axis=0)])


def test_recording_does_not_change_the_integration(cuda):
    from spitfire_gb300.adjoint import ReactorAdjoint
    from spitfire_gb300.reactors import BatchIntegrator
    spec, og = pair('h2-burke')
    q0 = _h2_reactors(spec, 8)
    adj = ReactorAdjoint(spec, 'isobaric')
    tr = adj.forward(q0, t_end=2.e-4, capacity=64)  # grows the capacity on the way
    plain = BatchIntegrator(spec, 'isobaric').run(q0, stop_at_time=2.e-4)
    assert (tr.status.cpu().numpy() == 1).all()
    assert np.array_equal(tr.q_end.cpu().numpy(), plain['q'].cpu().numpy())
    assert np.array_equal(tr.counts.cpu().numpy(), plain['counts'].cpu().numpy())
    rec = tr.rec.cpu().numpy()
    st = tr.steps.cpu().numpy()
    for i in range(8):
        assert abs(rec[i, :st[i], 1].sum() - 2.e-4) < 1e-15
        assert rec[i, 0, 0] == 0. and np.all(np.diff(rec[i, :st[i], 0]) > 0)


def test_record_growth_reintegrates_only_the_reactors_that_ran_out(cuda):
    """A record too small for some reactors: those alone are integrated again into a larger record, and every
    reactor's record, counts and end state equal those of one run with a record that fits the whole batch."""
    from spitfire_gb300.adjoint import ReactorAdjoint
    spec, og = pair('h2-burke')
    q0 = _h2_reactors(spec, 8)
    adj = ReactorAdjoint(spec, 'isobaric')
    big = adj.forward(q0, t_end=2.e-4, capacity=4096)
    steps = big.steps.cpu().numpy()
    lo, hi = int(steps.min()), int(steps.max())
    cap = lo if lo < hi else lo - 1  # the shortest fit (when the counts differ), the others run out
    small = adj.forward(q0, t_end=2.e-4, capacity=cap)
    assert small.rec.shape[1] >= hi
    for a in ('steps', 'status', 'counts', 'q_end', 't_end'):
        assert np.array_equal(getattr(small, a).cpu().numpy(), getattr(big, a).cpu().numpy()), a
    # the smoothed delay sums over the record's whole length: another length may associate the sum differently
    assert np.allclose(small.tau_s.cpu().numpy(), big.tau_s.cpu().numpy(), rtol=1e-13, atol=0.)
    rb, rs = big.rec.cpu().numpy(), small.rec.cpu().numpy()
    for i in range(8):
        assert np.array_equal(rs[i, :steps[i]], rb[i, :steps[i]])
    g_big, g_small = adj.backward(big), adj.backward(small)
    assert np.array_equal(g_big['theta'].cpu().numpy(), g_small['theta'].cpu().numpy())


def _mid_ignition_gri(spec, seed):
    """A GRI-3.0 reactor of the adjoint workload and an end time inside its ignition: of 8 seeded reactors the one
    that ignites first, t_end = its smoothed ignition delay (both outputs then respond to the kinetics; after
    ignition the final temperature is the equilibrium one, and before it the smoothed delay is t_end whatever the
    rates, so in either case the gradients are rounding noise)."""
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.adjoint import ReactorAdjoint
    d = W.adjoint_batch(spec, 8, seed=seed)
    tr = ReactorAdjoint(spec, 'isobaric').forward(d['q0'], pressures=d['p'], t_end=5.e-3)
    tau = tr.tau_s.cpu().numpy()
    i = int(np.argmin(tau))
    assert tau[i] < 4.e-3
    return d['q0'][i:i + 1], d['p'][i:i + 1], float(tau[i])


@pytest.mark.parametrize('name', ['h2-burke', 'methane-gri30'])
def test_adjoint_matches_cpu_forward_sensitivity(cuda, name):
    import integrate as I
    import sensitivity as SE
    from spitfire_gb300.adjoint import ReactorAdjoint
    _oracle_1thread()
    spec, og = pair(name)
    if name == 'h2-burke':
        q0, p, t_end, n = _h2_reactors(spec, 3), np.full(3, 101325.), 2.e-4, 3
    else:
        q0, p, t_end = _mid_ignition_gri(spec, 21)
        n = 1
    adj = ReactorAdjoint(spec, 'isobaric')
    tr = adj.forward(q0, pressures=p, t_end=t_end)
    g = adj.backward(tr)
    theta = g['theta'].cpu().numpy()          # [n, 2, nr, 2], file order
    rec = tr.rec.cpu().numpy()
    steps = tr.steps.cpu().numpy()
    yi = spec.reaction_yaml_index
    pj = SE.ParamJacobian(spec, og, 'isobaric', p[0])
    for i in range(n):
        prob = I.ReactorProblem(og, 'isobaric', pressure=p[i])
        pj.pressure = p[i]
        dts = rec[i, :steps[i], 1]
        fs, stages = SE.frozen_integrate(prob, q0[i], dts)
        gpu_stages = rec[i, :steps[i], 2:].reshape(steps[i], 6, -1)
        assert np.max(np.abs(stages - gpu_stages)) / np.max(np.abs(gpu_stages)) < 1e-9
        T_end, tau = SE.outputs(fs, stages, dts, 0, q0[i, 0])
        assert abs(T_end - tr.T_end[i].item()) / T_end < 1e-10
        assert abs(tau - tr.tau_s[i].item()) / tau < 1e-9
        gT, gtau = SE.forward_sensitivity(prob, pj, q0[i], dts, stages)
        for o, ref in enumerate((gT, gtau)):
            ref_f = np.zeros_like(theta[i, o])
            ref_f[yi, 0] = ref[0::2]
            ref_f[yi, 1] = ref[1::2]
            for c in range(2):
                err = np.max(np.abs(theta[i, o, :, c] - ref_f[:, c])) / np.max(np.abs(ref_f[:, c]))
                assert err < 1e-7, (name, i, o, c, err)


def test_adjoint_matches_finite_differences(cuda):
    """One GRI-3.0 reactor of the adjoint workload (T0 1000-1400 K, phi 0.7-1.5, 10 atm) integrated into its
    ignition: the GPU gradients of both outputs against central differences for the 8 largest ln A and 4 largest
    E_a entries."""
    import sensitivity as SE
    from spitfire_gb300.adjoint import ReactorAdjoint
    _oracle_1thread()
    spec, og = pair('methane-gri30')
    q0, p, t_end = _mid_ignition_gri(spec, 22)
    d = {'q0': q0, 'p': p}
    adj = ReactorAdjoint(spec, 'isobaric')
    tr = adj.forward(d['q0'], pressures=d['p'], t_end=t_end)
    th = adj.backward(tr)['theta'].cpu().numpy()[0]   # [2, nr, 2] file order
    dts = tr.rec[0, :tr.steps[0].item(), 1].cpu().numpy()
    yi = spec.reaction_yaml_index
    inv = np.argsort(yi)                                # file position -> internal index
    for o in range(2):
        picks = [(int(r), 0) for r in np.argsort(-np.abs(th[o, :, 0]))[:8]] + \
                [(int(r), 1) for r in np.argsort(-np.abs(th[o, :, 1]))[:4]]
        params = [2 * int(inv[r]) + c for r, c in picks]
        fd = SE.fd_gradient(spec, 'isobaric', d['p'][0], d['q0'][0], dts, params)[o]
        got = np.array([th[o, r, c] for r, c in picks])
        for c in (0, 1):
            sel = [k for k, (r, cc) in enumerate(picks) if cc == c]
            scale = np.max(np.abs(th[o, :, c]))
            err = np.max(np.abs(got[sel] - fd[sel])) / scale
            assert err < 1e-5, (o, c, err, got[sel], fd[sel])


def test_autograd_function_and_batch(cuda):
    import torch
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.adjoint import ReactorAdjoint, ignition_outputs, nominal_parameters
    spec, og = pair('methane-gri30')
    d = W.adjoint_batch(spec, 16, seed=23)
    theta = torch.tensor(nominal_parameters(spec), dtype=torch.float64, requires_grad=True)
    out = ignition_outputs(theta, spec, d['q0'], d['p'], 5.e-3)
    wts = torch.tensor([[1., 0.], [0., 1.]], dtype=torch.float64, device=out.device).repeat(8, 1)
    (out * wts).sum().backward()
    adj = ReactorAdjoint(spec, 'isobaric')
    g = adj.backward(adj.forward(d['q0'], d['p'], 5.e-3))['theta']
    ref = (wts[:, :, None, None] * g).sum((0, 1)).cpu()
    assert torch.allclose(theta.grad, ref, rtol=1e-12, atol=0.)
    assert spec.griffon.device_status() == 0


@pytest.mark.parametrize('name,configuration,outputs', [
    ('methane-gri30', 'isobaric', ('T_end', 'tau_s')),
    ('methane-gri30', 'isobaric', ('tau_s',)),
    ('h2-burke', 'isochoric', ('tau_s', 'T_end'))])
def test_native_backward_matches_host_loop(cuda, name, configuration, outputs):
    """sf_adjoint_batch (ReactorAdjoint.backward) against the same recursion with its step loop in Python
    (backward_host) on a batch of reactors with different step counts: parameter and initial-state gradients agree
    to 1e-9 normwise (the two sum the stage terms in different orders), for either output order and for isochoric
    reactors."""
    import torch
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.adjoint import ReactorAdjoint
    spec, og = pair(name)
    adj = ReactorAdjoint(spec, configuration)
    if name == 'methane-gri30':
        d = W.adjoint_batch(spec, 12, seed=29)
        q0, p, t_end = d['q0'], d['p'], 5.e-3
    else:
        q0, p, t_end = _h2_reactors(spec, 5), np.full(5, 101325.), 3.e-4
        if configuration == 'isochoric':
            from spitfire_gb300.mechanism import GAS_CONSTANT
            Y = np.hstack([q0[:, 1:], 1. - q0[:, 1:].sum(1, keepdims=True)])
            rho = 101325. / (GAS_CONSTANT * q0[:, 0] * (Y / spec.molecular_weights).sum(1))
            q0 = np.hstack([rho[:, None], q0])
    tr = adj.forward(q0, pressures=p, t_end=t_end)
    steps = tr.steps.cpu().numpy()
    assert steps.min() < steps.max()
    a = adj.backward(tr, outputs=outputs)
    h = adj.backward_host(tr, outputs=outputs)
    for key in ('theta', 'q0'):
        x, y = a[key].cpu().numpy(), h[key].cpu().numpy()
        for o in range(len(outputs)):
            scale = np.max(np.abs(y[:, o]))
            assert scale > 0
            err = np.max(np.abs(x[:, o] - y[:, o])) / scale
            assert err < 1e-9, (key, o, err)
    assert spec.griffon.device_status() == 0
