"""The allocation-free plain Jacobian entry point (sf_reactor_jac_plain_batch_static) against the regular one.

sf_reactor_jac_plain_batch_static exists for callers that cannot allocate device memory where they evaluate
Jacobians (their memory manager owns all device allocations, or they must not allocate while recording work on
their streams); it takes its scratch from a fixed 32 MiB device array instead of a caller workspace. This file is
named so that pytest collects it last: a run that stops at its first failure has run every other test before.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import colmajor, rownorm_err
from spitfire_gb300 import workloads as W
from spitfire_gb300._desc import reactor_params

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _static_call(g, P, q, pressures=None):
    import torch
    from spitfire_gb300 import _native as N
    n, neq = q.shape
    rhs = torch.full((n, neq), float('nan'), dtype=torch.float64, device=q.device)
    J = torch.full((n, neq * neq), float('nan'), dtype=torch.float64, device=q.device)
    rc = N.load().sf_reactor_jac_plain_batch_static(g.handle, C.byref(P), n, N.ptr(q), N.ptr(pressures),
                                                     N.ptr(rhs), N.ptr(J), N.stream_handle())
    return rc, rhs, J


@pytest.mark.parametrize('name,configuration,n', [('methane-gri30', 'isochoric', 512),
                                                  ('methane-gri30', 'isobaric', 300),
                                                  ('h2-burke', 'isochoric', 4096)])
def test_static_scratch_matches_workspace_entry_point(cuda, name, configuration, n):
    import torch
    from spitfire_gb300 import _native as N
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    spec = ChemicalMechanismSpec.bundled(name)
    g = spec.griffon
    gen = W.gri_states if 'gri' in name else W.h2_states
    P = reactor_params(configuration, 'adiabatic', pressure=101325.)
    for call, seed in enumerate((2024, 2025)):  # two calls in a row, different states
        d = gen(spec, n, seed=seed)
        qh = W.isochoric_state(d) if configuration == 'isochoric' else W.isobaric_state(d)
        q = torch.tensor(qh, device=cuda)
        pr = torch.tensor(d['p'], device=cuda) if configuration == 'isobaric' else None
        rc, rhs_s, J_s = _static_call(g, P, q, pr)
        assert rc == 0, N.load().sf_last_error().decode()
        rhs_w, J_w = g.reactor_jac_plain_batch(P, q, pressures=pr)
        torch.cuda.synchronize()
        neq = q.shape[1]
        a_rhs, b_rhs = rhs_s.cpu().numpy(), rhs_w.cpu().numpy()
        a_J, b_J = J_s.cpu().numpy(), J_w.cpu().numpy()
        assert np.isfinite(a_J).all() and np.isfinite(a_rhs).all(), call
        assert rownorm_err(a_rhs, b_rhs) <= TOL, call
        assert rownorm_err(colmajor(a_J, neq), colmajor(b_J, neq)) <= TOL, call


def test_static_scratch_rejects_oversized_batch(cuda):
    import torch
    from spitfire_gb300 import _native as N
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    spec = ChemicalMechanismSpec.bundled('methane-gri30')
    g = spec.griffon
    d = W.gri_states(spec, 4096)
    q = torch.tensor(W.isochoric_state(d), device=cuda)
    rc, _, _ = _static_call(g, reactor_params('isochoric'), q)
    assert rc == 5  # SF_ERR_WORKSPACE
    assert 'exceed the fixed scratch' in N.load().sf_last_error().decode()
