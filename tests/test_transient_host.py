"""Host logic of the batched transient flamelet integrator (spitfire_gb300/flamelet.py: _integrate_batch) on CPU.

The integrator's device operations (right-hand side, scaled Jacobian, block-Thomas factor and solve, per-flamelet
norms) are supplied here by a CPU stand-in over the oracle's flamelet operator, so the step control, Newton
masking, Jacobian reuse and stop logic run as they do on the GPU. Against the reference's own heat-loss trajectory
(tests/golden/nonadiabatic_transient_slfm_gold.npz): the same accepted-step count, step times and temperatures
within 1e-7; and a ragged batch of two flamelets gives each the trajectory it has alone.
"""
import numpy as np
import torch

import flamelet_cases as FC
from helpers import pair
from test_oracle_transient import GOLD, HEAT, _heat_op, _streams


class CpuBatch:
    """The FlameletBatch operations _integrate_batch uses, on CPU tensors, from oracle flamelet operators."""

    def __init__(self, ops, states):
        import oracle as orc
        self.orc = orc
        self.ops = ops
        self.nf = len(ops)
        self.ns = ops[0].ns
        nz = [op.nzi for op in ops]
        self.offz_host = np.r_[0, np.cumsum(nz)].astype(np.int32)
        self.values = torch.zeros(1, dtype=torch.float64)
        self._init = torch.tensor(np.concatenate(states), dtype=torch.float64)
        self.dof_flamelet = torch.repeat_interleave(torch.arange(self.nf), torch.tensor(nz) * self.ns)
        w = torch.ones(self._init.numel(), dtype=torch.float64)
        w[::self.ns] = 1.e-3
        self.inv_scales = w
        self._J = [None] * self.nf
        self._fac = [None] * self.nf

    def _seg(self, f):
        return slice(int(self.offz_host[f]) * self.ns, int(self.offz_host[f + 1]) * self.ns)

    def _on(self, active):
        return range(self.nf) if active is None else [f for f in range(self.nf) if bool(active[f])]

    def initial_state(self):
        return self._init.clone()

    def rhs(self, state, out=None, active=None):
        out = torch.full_like(state, float('nan')) if out is None else out
        x = state.numpy()
        for f in self._on(active):
            out[self._seg(f)] = torch.from_numpy(self.ops[f].rhs(x[self._seg(f)]))
        return out

    def jacobian(self, state, scale_and_offset=False, prefactor=0., active=None):
        # prefactor: a number, or one per flamelet (as FlameletBatch.jacobian takes it)
        x = state.numpy()
        for f in self._on(active):
            pf = float(prefactor[f]) if torch.is_tensor(prefactor) else prefactor
            self._J[f] = self.ops[f].jac(x[self._seg(f)], scale_and_offset=scale_and_offset, prefactor=pf)

    def factor(self, active=None):
        for f in self._on(active):
            self._fac[f] = self.orc.btddod_full_factorize(self._J[f], self.ops[f].nzi, self.ns)

    def solve(self, r, out=None, active=None):
        out = torch.full_like(r, float('nan')) if out is None else out
        x = r.numpy()
        for f in self._on(active):
            d, l, piv = self._fac[f]
            out[self._seg(f)] = torch.from_numpy(
                self.orc.btddod_full_solve(d, l, piv, x[self._seg(f)], self.ops[f].nzi, self.ns))
        return out

    def expand(self, per_flamelet):
        return per_flamelet[self.dof_flamelet]

    def norms(self, v):
        out = torch.zeros(self.nf, dtype=torch.float64)
        return out.scatter_reduce(0, self.dof_flamelet, (v * self.inv_scales).abs(), reduce='amax',
                                  include_self=True)

    def finite(self, v):
        bad = torch.zeros(self.nf, dtype=torch.float64)
        bad = bad.scatter_reduce(0, self.dof_flamelet, (~torch.isfinite(v)).double(), reduce='amax',
                                 include_self=True)
        return bad == 0


def _case(chi=1., state=None):
    from spitfire_gb300.flamelet import FlameletSetup, FlameletSpec
    g = np.load(GOLD)
    spec, og = pair('h2-burke')
    air, fuel = _streams(spec)
    s = FlameletSetup(FlameletSpec(mech_spec=spec, oxy_stream=air, fuel_stream=fuel, grid_points=34,
                                   initial_condition=g['adiabatic_state'] if state is None else state,
                                   stoich_dissipation_rate=chi, **HEAT))
    return g, spec, og, s, max(air.T, fuel.T)


def _stop(T_bc_max):
    return lambda f, t, st, res, n: np.max(st) < 1.05 * T_bc_max or res < 1.e-4


def test_integrate_batch_host_logic_reproduces_reference_trajectory():
    from spitfire_gb300.flamelet import _integrate_batch
    g, spec, og, s, Tb = _case()
    b = CpuBatch([_heat_op(og, s)], [g['adiabatic_state']])
    traj, stats = _integrate_batch(b, host_attempts=True, stop_criteria=_stop(Tb), first_time_step=1.e-9,
                                   max_time_step=1.e-1, transient_tolerance=1.e-10)
    times, states = traj[0]
    assert stats['steps'][0] == g['times'].size - 1
    assert stats['status'][0] == 7
    np.testing.assert_allclose(times, g['times'], rtol=1e-7)
    np.testing.assert_allclose(states[:, ::spec.n_species], g['T'][:, 1:-1], rtol=1e-7)


def test_integrate_batch_ragged_flamelets_match_their_own_runs():
    """Two flamelets of different dissipation rates (and so different step sequences) in one batch: each follows
    the trajectory it has alone (the masks keep them independent)."""
    from spitfire_gb300.flamelet import _integrate_batch
    g, spec, og, s1, Tb = _case(1.)
    _, _, _, s2, _ = _case(3.)
    ops = [_heat_op(og, s1), _heat_op(og, s2)]
    st = [g['adiabatic_state'], g['adiabatic_state']]
    kw = dict(stop_criteria=_stop(Tb), first_time_step=1.e-9, max_time_step=1.e-1, transient_tolerance=1.e-10)
    both, sb = _integrate_batch(CpuBatch(ops, st), host_attempts=True, **kw)
    for f in range(2):
        alone, sa = _integrate_batch(CpuBatch([ops[f]], [st[f]]), host_attempts=True, **kw)
        assert sb['steps'][f] == sa['steps'][0]
        np.testing.assert_array_equal(both[f][0], alone[0][0])
        np.testing.assert_array_equal(both[f][1], alone[0][1])
    assert sb['steps'][0] != sb['steps'][1]


def test_flamelet_integrate_rejects_what_the_gpu_path_does_not_implement():
    """Flamelet.integrate fails loudly, before touching the device, for a non-default stepper, nonlinear solver,
    step controller or extra arguments, for another linear solver, without a stop rule, and for unknown
    arguments."""
    import pytest
    from spitfire_gb300.flamelet import Flamelet
    f = Flamelet.__new__(Flamelet)
    with pytest.raises(NotImplementedError):
        f.integrate(stop_at_time=1., stepper_type=object)
    with pytest.raises(NotImplementedError):
        f.integrate(stop_at_time=1., extra_stepcontrol_args={'kp': 0.})
    with pytest.raises(ValueError):
        f.integrate(stop_at_time=1., linear_solver='superlu')
    with pytest.raises(ValueError):
        f.integrate()
    with pytest.raises(TypeError):
        f.integrate(stop_at_time=1., bogus=1)


def test_integrate_batch_stop_at_time_active_mask_and_first_last_output():
    """stop_at_time clips the last step onto the end time (odesolve's coerced final step), matching the oracle's
    restatement step for step; a flamelet outside `active` is left at its initial state with no steps; without
    save_each_step only the first and last states come back."""
    import flamelet_transient as FT
    from integrate import integrate
    from spitfire_gb300.flamelet import _integrate_batch
    g, spec, og, s1, Tb = _case(1.)
    _, _, _, s2, _ = _case(3.)
    ops = [_heat_op(og, s1), _heat_op(og, s2)]
    st = [g['adiabatic_state'], g['adiabatic_state']]
    kw = dict(stop_at_time=2.e-5, first_time_step=1.e-9, max_time_step=1.e-1, transient_tolerance=1.e-10)
    traj, stats = _integrate_batch(CpuBatch(ops, st), host_attempts=True, active=np.array([True, False]),
                                   save_each_step=False, **kw)
    ref = integrate(FT.FlameletTransientProblem(ops[0]), st[0], **kw)
    assert stats['status'][0] == 1 and stats['steps'][0] == ref['steps']
    times, states = traj[0]
    assert times.shape == (2,) and states.shape[0] == 2
    assert times[-1] == 2.e-5
    np.testing.assert_allclose(states[-1], ref['state'], rtol=1e-8, atol=1e-12)  # stage sums ordered differently
    np.testing.assert_array_equal(states[0], st[0])
    assert stats['steps'][1] == 0 and stats['status'][1] == 0
    np.testing.assert_array_equal(traj[1][1][-1], st[1])
