"""Homogeneous reactors on the GPU: batched adaptive ESDIRK64 integration and a drop-in ``HomogeneousReactor``.

``BatchIntegrator`` integrates thousands of closed reactors of one mechanism and configuration in a single
persistent launch (``sf_integrate_batch``), with the reference's defaults (reactors.py:429-611): first time step
1e-6, maximum 1e6, PI target error 1e-10, Newton tolerance 1e-12 with weights 1/[1e3 on T], at least 40 steps,
Jacobian every step. Optionally the launch is captured once in a CUDA graph and replayed.

``HomogeneousReactor`` keeps the constructor and the integrate / compute_ignition_delay / integrate_to_steady /
integrate_to_time methods of ``spitfire.chemistry.reactors.HomogeneousReactor`` for closed reactors; it runs the
batched integrator with one reactor and returns the first and last states (the GPU path does not record
trajectories).
"""

import ctypes as C

import numpy as np

from . import _native as N
from ._desc import SfIntegrateParams, reactor_params

STATUS_NAMES = {0: 'running', 1: 'done', 2: 'ignited', 3: 'steady', 4: 'max_steps', 5: 'nan', 6: 'no_ignition',
                7: 'record_full'}


def _torch():
    import torch
    return torch


class BatchIntegrator:
    def __init__(self, mech, configuration='isobaric', heat_transfer='adiabatic', pressure=101325.,
                 linear_precision=0, refine_sweeps=2, rates_option=0):
        if configuration not in ('isobaric', 'isochoric'):
            raise ValueError('configuration must be isobaric or isochoric')
        self.mech = mech
        self.g = mech.griffon
        self.configuration = configuration
        self.params = reactor_params(configuration, heat_transfer, pressure=pressure)
        self.linear_precision = linear_precision
        self.refine_sweeps = refine_sweeps
        self.rates_option = rates_option
        self._graph = None

    def controls(self, stop_at_time=None, delta_temperature_ignition=None, stop_at_steady=None,
                 first_time_step=1.e-6, max_time_step=1.e6, transient_tolerance=1.e-10, nonlinear_tolerance=1.e-12,
                 minimum_time_step_count=40, maximum_time_step_count=None, max_nonlinear_iter=20,
                 maximum_steps_per_jacobian=1, minimum_allowable_residual=1.e-12, max_attempts=500000):
        ip = SfIntegrateParams()
        ip.first_time_step = first_time_step
        ip.max_time_step = max_time_step
        ip.transient_tolerance = transient_tolerance
        ip.nonlinear_tolerance = nonlinear_tolerance
        ip.minimum_time_step_count = minimum_time_step_count
        ip.maximum_time_step_count = 0 if maximum_time_step_count is None else int(maximum_time_step_count)
        ip.max_nonlinear_iter = max_nonlinear_iter
        ip.maximum_steps_per_jacobian = maximum_steps_per_jacobian
        ip.stop_at_time = stop_at_time if stop_at_time is not None else -1.
        ip.delta_temperature_ignition = delta_temperature_ignition if delta_temperature_ignition is not None else -1.
        ip.minimum_allowable_residual = minimum_allowable_residual
        ip.stop_at_steady = stop_at_steady if stop_at_steady is not None else -1.
        ip.linear_precision = self.linear_precision
        ip.refine_sweeps = self.refine_sweeps
        ip.rates_option = self.rates_option
        ip.max_attempts = max_attempts
        return ip

    def allocate(self, n):
        torch = _torch()
        neq = self.mech.n_species + (1 if self.configuration == 'isochoric' else 0)
        dev = torch.device('cuda', torch.cuda.current_device())
        return dict(q=torch.empty((n, neq), dtype=torch.float64, device=dev),
                    t=torch.empty(n, dtype=torch.float64, device=dev),
                    counts=torch.empty((n, 4), dtype=torch.int32, device=dev),
                    status=torch.empty(n, dtype=torch.int32, device=dev),
                    ws=torch.empty(self.workspace_bytes(n) // 4 + 1, dtype=torch.int32, device=dev))

    def workspace_bytes(self, n):
        return int(N.load().sf_integrate_workspace_size(self.g.handle, C.byref(self.params), int(n)))

    def launch(self, q0, pressures, out, ip):
        L = N.load()
        n = q0.shape[0]
        N.check(L.sf_integrate_batch(self.g.handle, C.byref(self.params), C.byref(ip), n, N.ptr(q0),
                                     N.ptr(pressures), N.ptr(out['q']), N.ptr(out['t']), N.ptr(out['counts']),
                                     N.ptr(out['status']), N.ptr(out['ws']), out['ws'].numel() * 4,
                                     N.stream_handle()))

    def run(self, q0, pressures=None, graph=False, **controls):
        """Integrate every row of q0 (isobaric [T, Y_0..Y_{ns-2}] or isochoric [rho, T, Y...]).

        Returns dict of CUDA tensors: q (final states), t (final times; the ignition delay when
        delta_temperature_ignition is given), counts [n, 4] (accepted steps, Newton iterations, Jacobian setups,
        failed steps), status (see STATUS_NAMES)."""
        torch = _torch()
        q0 = self.g._dev(q0)
        pr = self.g._dev(pressures) if pressures is not None else None
        ip = self.controls(**controls)
        out = self.allocate(q0.shape[0])
        if not graph:
            self.launch(q0, pr, out, ip)
            return out
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.launch(q0, pr, out, ip)  # first call builds the gather programs outside the capture
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch(q0, pr, out, ip)
        g.replay()
        self._graph = (g, q0, pr, out, ip)
        return out

    def replay(self):
        """Re-run the captured launch (same inputs, same outputs)."""
        if self._graph is None:
            raise RuntimeError('no captured launch; call run(..., graph=True) first')
        self._graph[0].replay()
        return self._graph[3]


class HomogeneousReactor:
    """Drop-in for spitfire.chemistry.reactors.HomogeneousReactor (closed reactors; reactors.py:27-794)."""

    def __init__(self, mech_spec, initial_mixture, configuration, heat_transfer, mass_transfer,
                 convection_temperature=None, radiation_temperature=None, convection_coefficient=None,
                 radiative_emissivity=None, shape_dimension_dict=None, mixing_tau=None, feed_temperature=None,
                 feed_mass_fractions=None, feed_density=None, rates_sensitivity_type='dense',
                 sensitivity_transform_type='exact', initial_time=0.):
        if mass_transfer != 'closed':
            raise NotImplementedError('open reactors are not on the GPU path')
        if heat_transfer not in ('adiabatic', 'isothermal'):
            raise NotImplementedError('the GPU integrator covers adiabatic and isothermal reactors')
        self._mechanism = mech_spec
        self._configuration = configuration
        self._heat_transfer = heat_transfer
        self._rates_sensitivity_option = {'dense': 0, 'no-TBAF': 1, 'sparse': 2}[rates_sensitivity_type]
        self._initial_pressure = initial_mixture.P
        self._initial_temperature = initial_mixture.T
        self._initial_mass_fractions = np.array(initial_mixture.Y)
        ns = mech_spec.n_species
        self._n_equations = ns if configuration == 'isobaric' else ns + 1
        if configuration == 'isobaric':
            self._temperature_index = 0
            self._initial_state = np.hstack([[initial_mixture.T], self._initial_mass_fractions[:-1]])
        else:
            self._temperature_index = 1
            self._initial_state = np.hstack([[initial_mixture.density, initial_mixture.T],
                                             self._initial_mass_fractions[:-1]])
        self._current_state = self._initial_state.copy()
        self._current_time = float(initial_time)
        self._last_info = None

    @property
    def initial_state(self):
        return self._initial_state.copy()

    @property
    def current_state(self):
        return self._current_state.copy()

    @property
    def current_time(self):
        return self._current_time

    @property
    def current_temperature(self):
        return self._current_state[self._temperature_index]

    @property
    def n_equations(self):
        return self._n_equations

    @property
    def last_counts(self):
        return self._last_info

    def _integrate(self, **controls):
        bi = BatchIntegrator(self._mechanism, self._configuration, self._heat_transfer,
                             pressure=self._initial_pressure, rates_option=self._rates_sensitivity_option)
        out = bi.run(self._current_state[None, :], **controls)
        st = int(out['status'][0])
        if st == 6:
            raise ValueError('From compute_ignition_delay(): residual < minimum allowable value, suggesting that '
                             'the reactor will not ignite.')
        q = out['q'][0].cpu().numpy()
        self._last_info = dict(zip(['steps', 'newton_iters', 'jac_setups', 'failed_steps'],
                                   out['counts'][0].cpu().numpy().tolist()), status=STATUS_NAMES.get(st, st))
        t_end = float(out['t'][0]) + self._current_time
        t0 = self._current_time
        self._current_state = q
        self._current_time = t_end
        from .library import Dimension, Library
        lib = Library(Dimension('time', np.array([t0, t_end])))
        states = np.vstack([self._initial_state if t0 == 0. else q, q])
        names = self._mechanism.species_names
        Tidx = self._temperature_index
        lib['temperature'] = states[:, Tidx]
        if self._configuration == 'isochoric':
            lib['density'] = states[:, 0]
        else:
            lib['pressure'] = np.full(2, self._initial_pressure)
        last = np.ones(2)
        for i, s in enumerate(names[:-1]):
            lib['mass fraction ' + s] = states[:, Tidx + 1 + i]
            last -= states[:, Tidx + 1 + i]
        lib['mass fraction ' + names[-1]] = last
        return lib

    def integrate(self, stop_at_time=None, stop_at_steady=None, first_time_step=1.e-6, max_time_step=1.e6,
                  minimum_time_step_count=40, transient_tolerance=1.e-10, maximum_steps_per_jacobian=1,
                  nonlinear_solve_tolerance=1.e-12, **kwargs):
        return self._integrate(stop_at_time=stop_at_time, stop_at_steady=stop_at_steady,
                               first_time_step=first_time_step, max_time_step=max_time_step,
                               minimum_time_step_count=minimum_time_step_count,
                               transient_tolerance=transient_tolerance,
                               maximum_steps_per_jacobian=maximum_steps_per_jacobian,
                               nonlinear_tolerance=nonlinear_solve_tolerance)

    def integrate_to_steady(self, steady_tolerance=1.e-6, **kwargs):
        return self.integrate(stop_at_steady=steady_tolerance, **kwargs)

    def integrate_to_time(self, final_time, **kwargs):
        return self.integrate(stop_at_time=final_time, **kwargs)

    def compute_ignition_delay(self, delta_temperature_ignition=400., minimum_allowable_residual=1.e-12,
                               return_solution=False, **kwargs):
        if self._heat_transfer == 'isothermal':
            raise ValueError('compute_ignition_delay() called on an isothermal reactor! This is not currently '
                             'supported!')
        lib = self._integrate(delta_temperature_ignition=delta_temperature_ignition,
                              minimum_allowable_residual=minimum_allowable_residual,
                              first_time_step=kwargs.get('first_time_step', 1.e-6),
                              max_time_step=kwargs.get('max_time_step', 1.e6),
                              minimum_time_step_count=kwargs.get('minimum_time_step_count', 40),
                              transient_tolerance=kwargs.get('transient_tolerance', 1.e-10),
                              nonlinear_tolerance=kwargs.get('nonlinear_solve_tolerance', 1.e-12),
                              stop_at_time=kwargs.get('stop_at_time'))
        tau = self._current_time
        return (tau, lib) if return_solution else tau
