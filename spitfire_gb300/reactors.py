"""Homogeneous reactors on the GPU: batched adaptive ESDIRK64 integration and a drop-in ``HomogeneousReactor``.

``BatchIntegrator`` integrates thousands of reactors of one mechanism, configuration and feed in a single persistent
launch (``sf_integrate_batch``), with the reference's defaults (reactors.py:429-611): first time step 1e-6, maximum
1e6, PI target error 1e-10, Newton tolerance 1e-12 with weights 1/[1e3 on T], at least 40 steps, Jacobian every
step. Closed or open (mass exchange with a feed whose temperature may vary in time), adiabatic, isothermal or
diathermal. Optionally the launch is captured once in a CUDA graph and replayed; ``run_recorded`` returns every
accepted step.

``HomogeneousReactor`` keeps the constructor and the integrate / compute_ignition_delay / integrate_to_steady /
integrate_to_time methods of ``spitfire.chemistry.reactors.HomogeneousReactor`` and returns the same output library
(every accepted step, or the first and last when ``save_first_and_last_only``).
"""

import ctypes as C

import numpy as np

from . import _native as N
from ._desc import TIME_PARAMS, SfIntegrateParams, reactor_params

STATUS_NAMES = {0: 'running', 1: 'done', 2: 'ignited', 3: 'steady', 4: 'max_steps', 5: 'nan', 6: 'no_ignition',
                7: 'record_full'}

# feed temperature tables: points per unit of the first time step over the horizon, and the bounds on their number
FEED_TABLE_MIN_POINTS = 1024
FEED_TABLE_MAX_POINTS = 1 << 21


def _torch():
    import torch
    return torch


def record_capacity(n, neq, free_bytes, most=1024, share=0.25):
    """The largest power of two up to `most` steps whose trajectory record for n reactors of neq equations
    ((2 + 6 neq) doubles per step) takes at most `share` of free_bytes; at least 64 steps."""
    cap = most
    while cap > 64 and n * cap * (2 + 6 * neq) * 8 > share * free_bytes:
        cap //= 2
    return cap


class BatchIntegrator:
    """Batched ESDIRK64 integration of reactors that share a mechanism, configuration, heat transfer and feed.

    heat_transfer 'diathermal' takes convection_temperature, radiation_temperature, convection_coefficient,
    radiative_emissivity and surface_area_to_volume. mass_transfer 'open' takes mixing_tau, the feed mass fractions
    feed_mass_fractions (ns values), feed_density (isochoric) and feed_temperature. Each of convection_temperature,
    radiation_temperature, convection_coefficient, radiative_emissivity, mixing_tau, feed_temperature and
    feed_mass_fractions may be a function of time (absolute time; an array of ns values for the mass fractions),
    as in the reference (reactors.py:253-341): it is evaluated on a table of integration times that the device
    interpolates, and every right-hand side takes the parameters at its own time, every Jacobian those of the most
    recent right-hand side. A feed_density function is evaluated once, at t = 0, as the reference does."""

    def __init__(self, mech, configuration='isobaric', heat_transfer='adiabatic', pressure=101325.,
                 linear_precision=0, refine_sweeps=2, rates_option=0, mass_transfer='closed', mixing_tau=None,
                 feed_temperature=None, feed_mass_fractions=None, feed_density=None, convection_temperature=None,
                 radiation_temperature=None, convection_coefficient=None, radiative_emissivity=None,
                 surface_area_to_volume=None):
        if configuration not in ('isobaric', 'isochoric'):
            raise ValueError('configuration must be isobaric or isochoric')
        if mass_transfer not in ('closed', 'open'):
            raise ValueError('mass_transfer must be closed or open')
        self.mech = mech
        self.g = mech.griffon
        self.configuration = configuration
        self.open = mass_transfer == 'open'
        value0 = lambda v: v(0.) if callable(v) else v
        self._time_funcs = {}  # parameter name -> function of absolute time
        kw = {}
        if heat_transfer == 'diathermal':
            for name, v in (('convection_temperature', convection_temperature),
                            ('radiation_temperature', radiation_temperature),
                            ('convection_coefficient', convection_coefficient),
                            ('radiative_emissivity', radiative_emissivity),
                            ('surface_area_to_volume', surface_area_to_volume)):
                if v is None:
                    raise ValueError(f'diathermal reactors need {name}')
                if callable(v):
                    if name == 'surface_area_to_volume':
                        raise ValueError('surface_area_to_volume is a constant (the reactor shape)')
                    self._time_funcs[name] = v
            kw = dict(fluid_temperature=float(value0(convection_temperature)),
                      surface_temperature=float(value0(radiation_temperature)),
                      h_convection=float(value0(convection_coefficient)),
                      eps_radiation=float(value0(radiative_emissivity)),
                      surface_area_to_volume=float(surface_area_to_volume))
        self._feed_Y = None
        if self.open:
            if mixing_tau is None or feed_temperature is None or feed_mass_fractions is None:
                raise ValueError('open reactors need mixing_tau, feed_temperature and feed_mass_fractions')
            if configuration == 'isochoric' and feed_density is None:
                raise ValueError('open isochoric reactors need feed_density')
            for name, v in (('mixing_tau', mixing_tau), ('feed_temperature', feed_temperature),
                            ('feed_mass_fractions', feed_mass_fractions)):
                if callable(v):
                    self._time_funcs[name] = v
            self._feed_Y = self.g._dev(np.asarray(value0(feed_mass_fractions), dtype=np.float64).reshape(-1))
            if self._feed_Y.numel() != mech.n_species:
                raise ValueError('feed_mass_fractions needs one value per species')
            # the reference evaluates a feed density function once, at t = 0 (reactors.py:280, never updated)
            kw.update(inflow_temperature=float(value0(feed_temperature)),
                      inflow_density=float(value0(feed_density) or 0.), tau=float(value0(mixing_tau)),
                      inflow_Y_ptr=self._feed_Y.data_ptr())
        self.params = reactor_params(configuration, heat_transfer, self.open, pressure=pressure, **kw)
        self.linear_precision = linear_precision
        self.refine_sweeps = refine_sweeps
        self.rates_option = rates_option
        self._graph = None
        self._table = None

    def _time_table(self, ta):
        """[len(ta), width] values of the time-dependent parameters at absolute times ta, columns in the order of
        their sf_time_param bits; and the bit mask."""
        ns = self.mech.n_species
        cols, mask = [], 0
        for name, bit in TIME_PARAMS:
            f = self._time_funcs.get(name)
            if f is None:
                continue
            mask |= bit
            if name == 'feed_mass_fractions':
                cols.append(np.array([np.asarray(f(x), dtype=np.float64).reshape(ns) for x in ta]))
                continue
            try:
                vals = np.asarray(f(ta), dtype=np.float64)
                if vals.shape != ta.shape:
                    raise ValueError
            except Exception:
                vals = np.array([float(f(x)) for x in ta])
            cols.append(vals[:, None])
        return np.ascontiguousarray(np.hstack(cols)), mask

    def controls(self, stop_at_time=None, delta_temperature_ignition=None, stop_at_steady=None,
                 first_time_step=1.e-6, max_time_step=1.e6, transient_tolerance=1.e-10, nonlinear_tolerance=1.e-12,
                 minimum_time_step_count=40, maximum_time_step_count=None, max_nonlinear_iter=20,
                 maximum_steps_per_jacobian=1, minimum_allowable_residual=1.e-12, max_attempts=500000,
                 time_offset=0., first_jacobian_feed_time=0., feed_horizon=1.):
        """Integration controls. time_offset: the reactors' current time (a parameter function is evaluated at
        time_offset + integration time). first_jacobian_feed_time: the absolute time whose parameters the first
        Jacobian takes (0 for a new reference reactor). feed_horizon: integration time a parameter table covers when
        stop_at_time is not given."""
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
        ip.time_jac_t0 = float(first_jacobian_feed_time) - float(time_offset)
        if self._time_funcs:
            horizon = stop_at_time if stop_at_time is not None else feed_horizon
            t_lo = min(0., ip.time_jac_t0)
            n = int(min(FEED_TABLE_MAX_POINTS,
                        max(FEED_TABLE_MIN_POINTS, np.ceil((horizon - t_lo) / first_time_step) + 1)))
            tl = np.linspace(t_lo, horizon, n)
            tab, mask = self._time_table(tl + float(time_offset))
            self._table = self.g._dev(tab)
            ip.time_table = C.cast(C.c_void_p(self._table.data_ptr()), C.POINTER(C.c_double))
            ip.time_points = n
            ip.time_width = tab.shape[1]
            ip.time_columns = mask
            ip.time_t0 = float(tl[0])
            ip.time_dt = float(tl[1] - tl[0])
        return ip

    def allocate(self, n):
        torch = _torch()
        neq = self.mech.n_species + (1 if self.configuration == 'isochoric' else 0)
        dev = torch.device('cuda', torch.cuda.current_device())
        return dict(q=torch.empty((n, neq), dtype=torch.float64, device=dev),
                    t=torch.empty(n, dtype=torch.float64, device=dev),
                    t_interp=torch.full((n,), float('nan'), dtype=torch.float64, device=dev),
                    counts=torch.empty((n, 4), dtype=torch.int32, device=dev),
                    status=torch.empty(n, dtype=torch.int32, device=dev),
                    ws=torch.empty(self.workspace_bytes(n) // 4 + 1, dtype=torch.int32, device=dev))

    def workspace_bytes(self, n):
        return int(N.load().sf_integrate_workspace_size(self.g.handle, C.byref(self.params), int(n)))

    def launch(self, q0, pressures, out, ip, record=None):
        L = N.load()
        n = q0.shape[0]
        # the Hermite-interpolated first crossing of T0 + delta beside the step-end delay
        ip.ignition_time_interp = C.cast(out['t_interp'].data_ptr(), C.POINTER(C.c_double)) \
            if ip.delta_temperature_ignition > 0. else None
        if record is None:
            N.check(L.sf_integrate_batch(self.g.handle, C.byref(self.params), C.byref(ip), n, N.ptr(q0),
                                         N.ptr(pressures), N.ptr(out['q']), N.ptr(out['t']), N.ptr(out['counts']),
                                         N.ptr(out['status']), N.ptr(out['ws']), out['ws'].numel() * 4,
                                         N.stream_handle()))
        else:
            N.check(L.sf_integrate_record_batch(self.g.handle, C.byref(self.params), C.byref(ip), n, N.ptr(q0),
                                                N.ptr(pressures), N.ptr(out['q']), N.ptr(out['t']),
                                                N.ptr(out['counts']), N.ptr(out['status']), N.ptr(out['ws']),
                                                out['ws'].numel() * 4, N.ptr(record), record.shape[1],
                                                N.stream_handle()))

    def record(self, q0, pressures, ip, capacity):
        """Recording integration (sf_integrate_record_batch) of every row of q0, into a record of `capacity` steps per
        reactor to start with. Reactors that fill their record (status 7) are integrated again, by themselves, into a
        record of twice the capacity, until every reactor fits; the others keep the results of the first launch. A
        reactor's integration does not depend on the rest of its batch, so the results are those of a single run
        with the final capacity, without integrating the whole batch again. Returns (out, record)."""
        torch = _torch()
        n, neq = q0.shape
        row = 2 + 6 * neq
        out = self.allocate(n)
        rec = torch.empty((n, capacity, row), dtype=torch.float64, device=q0.device)
        self.launch(q0, pressures, out, ip, record=rec)
        full = torch.nonzero(out['status'] == 7).flatten()
        while full.numel():
            capacity *= 2
            sub = self.allocate(full.numel())
            sub_rec = torch.empty((full.numel(), capacity, row), dtype=torch.float64, device=q0.device)
            self.launch(q0[full].contiguous(), None if pressures is None else pressures[full].contiguous(), sub, ip,
                        record=sub_rec)
            grown = torch.empty((n, capacity, row), dtype=torch.float64, device=q0.device)
            grown[:, :rec.shape[1]] = rec
            grown[full] = sub_rec
            rec = grown
            for k in ('q', 't', 't_interp', 'counts', 'status'):
                out[k][full] = sub[k]
            full = full[torch.nonzero(sub['status'] == 7).flatten()]
        return out, rec

    def default_record_capacity(self, n, most=1024, share=0.25):
        """Starting record capacity for n reactors: record_capacity with the device memory that is free now."""
        torch = _torch()
        neq = self.mech.n_species + (1 if self.configuration == 'isochoric' else 0)
        return record_capacity(n, neq, torch.cuda.mem_get_info()[0], most, share)

    def run(self, q0, pressures=None, graph=False, **controls):
        """Integrate every row of q0 (isobaric [T, Y_0..Y_{ns-2}] or isochoric [rho, T, Y...]).

        Returns dict of CUDA tensors: q (final states), t (final times; the ignition delay when
        delta_temperature_ignition is given), t_interp (with delta_temperature_ignition: the time T first reaches
        T0 + delta on the cubic Hermite interpolant of the crossing step, NaN if never), counts [n, 4] (accepted
        steps, Newton iterations, Jacobian setups, failed steps), status (see STATUS_NAMES)."""
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
        self._graph = (g, q0, pr, out, ip, self._table)
        return out

    def run_recorded(self, q0, pressures=None, capacity=None, **controls):
        """run() that also returns every accepted step: 'times' [n, steps + 1] and 'states' [n, steps + 1, neq]
        (host arrays, padded past each reactor's own step count with its final time and state), 'steps' [n].
        The record grows until every reactor fits (see record; capacity None: default_record_capacity)."""
        q0 = self.g._dev(q0)
        pr = self.g._dev(pressures) if pressures is not None else None
        ip = self.controls(**controls)
        n, neq = q0.shape
        out, rec = self.record(q0, pr, ip, capacity or self.default_record_capacity(n))
        steps = out['counts'][:, 0].cpu().numpy()
        smax = int(steps.max()) if n else 0
        r = rec[:, :smax].cpu().numpy()
        tf = out['t'].cpu().numpy()
        qf = out['q'].cpu().numpy()
        times = np.empty((n, smax + 1))
        states = np.empty((n, smax + 1, neq))
        for i in range(n):
            k = int(steps[i])
            times[i, :k] = r[i, :k, 0]
            states[i, :k] = r[i, :k, 2:2 + neq]
            times[i, k:] = tf[i]
            states[i, k:] = qf[i]
        out.update(times=times, states=states, steps=steps)
        return out

    def run_plain(self, q0, pressures=None, **controls):
        """The plain single-state GPU form (sf_integrate_plain_batch, one thread per reactor, same step logic): the
        comparison point of run(). Closed adiabatic reactors; returns the dict of run()."""
        torch = _torch()
        q0 = self.g._dev(q0)
        pr = self.g._dev(pressures) if pressures is not None else None
        ip = self.controls(**controls)
        n, neq = q0.shape
        dev = q0.device
        out = dict(q=torch.empty((n, neq), dtype=torch.float64, device=dev),
                   t=torch.empty(n, dtype=torch.float64, device=dev),
                   counts=torch.empty((n, 4), dtype=torch.int32, device=dev),
                   status=torch.empty(n, dtype=torch.int32, device=dev))
        L = N.load()
        nb = int(L.sf_integrate_plain_workspace_size(self.g.handle, C.byref(self.params), n))
        ws = torch.empty(nb // 8 + 1, dtype=torch.float64, device=dev)
        N.check(L.sf_integrate_plain_batch(self.g.handle, C.byref(self.params), C.byref(ip), n, N.ptr(q0), N.ptr(pr),
                                           N.ptr(out['q']), N.ptr(out['t']), N.ptr(out['counts']),
                                           N.ptr(out['status']), N.ptr(ws), ws.numel() * 8, N.stream_handle()))
        out['workspace'] = ws
        return out

    def replay(self):
        """Re-run the captured launch (same inputs, same outputs)."""
        if self._graph is None:
            raise RuntimeError('no captured launch; call run(..., graph=True) first')
        self._graph[0].replay()
        return self._graph[3]


# surface-to-volume ratio of a reactor shape from its characteristic length a or its volume v (the geometry of each
# solid; the reference's table is reactors.py:85-97)
_SOV = {'cube': (lambda a: 6. / a, lambda v: 6. / np.cbrt(v)),
        'sphere': (lambda a: 3. / a, lambda v: 3. / np.cbrt(3. * v / (4. * np.pi))),
        'capsule': (lambda a: 12. / (5. * a), lambda v: 12. / (5. * np.cbrt(3. * v / (10. * np.pi)))),
        'tetrahedron': (lambda a: 6. * np.sqrt(6.) / a, lambda v: 6. * np.sqrt(6.) / np.cbrt(12. * v / np.sqrt(2.))),
        'octahedron': (lambda a: 3. * np.sqrt(6.) / a, lambda v: 3. * np.sqrt(6.) / np.cbrt(3. * v / np.sqrt(2.))),
        'icosahedron': (lambda a: 12. * np.sqrt(3.) / ((3. + np.sqrt(5.)) * a),
                        lambda v: 12. * np.sqrt(3.) / ((3. + np.sqrt(5.)) *
                                                       np.cbrt(12. * v / 5. / (3. + np.sqrt(5.)))))}


def _surface_to_volume(shape_dimension_dict):
    d = shape_dimension_dict
    if d is None or 'shape' not in d:
        raise ValueError('diathermal reactors need shape_dimension_dict with a shape key')
    if d['shape'] not in _SOV:
        raise ValueError(f'unknown reactor shape {d["shape"]!r}; supported: {sorted(_SOV)}')
    if ('char. length' in d) == ('volume' in d):
        raise ValueError('shape_dimension_dict needs exactly one of the char. length or volume keys')
    l2s, v2s = _SOV[d['shape']]
    return float(l2s(d['char. length'])) if 'char. length' in d else float(v2s(d['volume']))


def _join_trajectories(lib1, lib2, first_and_last_only=False):
    """One Library over 'time' from two consecutive trajectories; the second starts at the first one's last
    state, which is kept once."""
    from .library import Dimension, Library
    t = np.concatenate([lib1.dim('time').values, lib2.dim('time').values[1:]])
    pick = np.array([0, t.size - 1]) if first_and_last_only else np.arange(t.size)
    out = Library(Dimension('time', t[pick]))
    for q in lib1.props:
        out[q] = np.concatenate([np.asarray(lib1[q]), np.asarray(lib2[q])[1:]])[pick]
    return out


class HomogeneousReactor:
    """Drop-in for spitfire.chemistry.reactors.HomogeneousReactor (reactors.py:27-794): closed or open (mass
    exchange with a feed), adiabatic, isothermal or diathermal, isobaric or isochoric. The convection and radiation
    temperatures, convection coefficient, emissivity, mixing time, feed temperature and feed mass fractions may be
    functions of time, tabulated for the device (see BatchIntegrator); a feed density function is evaluated at
    t = 0, as the reference does."""

    def __init__(self, mech_spec, initial_mixture, configuration, heat_transfer, mass_transfer,
                 convection_temperature=None, radiation_temperature=None, convection_coefficient=None,
                 radiative_emissivity=None, shape_dimension_dict=None, mixing_tau=None, feed_temperature=None,
                 feed_mass_fractions=None, feed_density=None, rates_sensitivity_type='dense',
                 sensitivity_transform_type='exact', initial_time=0.):
        configuration = configuration.lower()
        heat_transfer = heat_transfer.lower()
        mass_transfer = mass_transfer.lower()
        if configuration not in ('isobaric', 'isochoric'):
            raise ValueError(f'bad configuration {configuration!r}; use isobaric or isochoric')
        if heat_transfer not in ('adiabatic', 'isothermal', 'diathermal'):
            raise ValueError(f'bad heat transfer {heat_transfer!r}')
        if mass_transfer not in ('closed', 'open'):
            raise ValueError(f'bad mass transfer {mass_transfer!r}')
        self._mechanism = mech_spec
        self._configuration = configuration
        self._heat_transfer = heat_transfer
        self._mass_transfer = mass_transfer
        self._rates_sensitivity_option = {'dense': 0, 'no-TBAF': 1, 'sparse': 2}[rates_sensitivity_type]
        if sensitivity_transform_type != 'exact':
            raise ValueError('sensitivity_transform_type must be exact')
        self._options = dict(heat_transfer=heat_transfer, mass_transfer=mass_transfer)
        if heat_transfer == 'diathermal':
            self._options.update(convection_temperature=convection_temperature,
                                 radiation_temperature=radiation_temperature,
                                 convection_coefficient=convection_coefficient,
                                 radiative_emissivity=radiative_emissivity,
                                 surface_area_to_volume=_surface_to_volume(shape_dimension_dict))
        if mass_transfer == 'open':
            self._options.update(mixing_tau=mixing_tau, feed_temperature=feed_temperature,
                                 feed_mass_fractions=feed_mass_fractions,
                                 feed_density=feed_density if configuration == 'isochoric' else None)
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
        self._initial_time = float(initial_time)
        self._current_time = float(initial_time)
        self._integrations = 0
        self._last_info = None

    @property
    def initial_state(self):
        return self._initial_state.copy()

    @property
    def current_state(self):
        return self._current_state.copy()

    @property
    def initial_time(self):
        return self._initial_time

    @property
    def current_time(self):
        return self._current_time

    @property
    def initial_temperature(self):
        return self._initial_temperature

    @property
    def current_temperature(self):
        return self._current_state[self._temperature_index]

    @property
    def initial_pressure(self):
        return self._initial_pressure

    @property
    def current_pressure(self):
        """reactors.py:391-394: an isobaric reactor's constant pressure; for an isochoric one the ideal-gas pressure
        rho R T / M of the current state (the reference evaluates rho T M there, without the gas constant)."""
        if self._configuration == 'isobaric' or self._integrations == 0:
            return self._initial_pressure
        rho, T = self._current_state[0], self._current_state[1]
        Y = self.current_mass_fractions
        return float(rho * 8314.46261815324 * T * np.sum(Y / np.asarray(self._mechanism.molecular_weights)))

    @property
    def initial_mass_fractions(self):
        return self._initial_mass_fractions.copy()

    @property
    def current_mass_fractions(self):
        y = self._current_state[self._temperature_index + 1:]
        return np.hstack([y, 1. - y.sum()])

    @property
    def n_species(self):
        return self._mechanism.n_species

    @property
    def n_reactions(self):
        return self._mechanism.n_reactions

    @property
    def n_equations(self):
        return self._n_equations

    @property
    def last_counts(self):
        return self._last_info

    @classmethod
    def get_supported_reactor_shapes(cls):
        return _SOV.keys()

    def _integrate(self, save_first_and_last_only=False, **controls):
        bi = BatchIntegrator(self._mechanism, self._configuration, pressure=self._initial_pressure,
                             rates_option=self._rates_sensitivity_option, **self._options)
        # a new reference reactor's first Jacobian takes the feed at t = 0 (reactors.py:279-282); a continued one
        # the feed of its last right-hand side, at the current time
        controls['time_offset'] = self._current_time
        controls['first_jacobian_feed_time'] = 0. if self._integrations == 0 else self._current_time
        q0 = self._current_state[None, :]
        t0 = self._current_time
        if save_first_and_last_only:
            out = bi.run(q0, **controls)
        else:
            out = bi.run_recorded(q0, **controls)
        st = int(out['status'][0])
        if st == 6:
            raise ValueError('From compute_ignition_delay(): residual < minimum allowable value, suggesting that '
                             'the reactor will not ignite.')
        q = out['q'][0].cpu().numpy()
        self._last_info = dict(zip(['steps', 'newton_iters', 'jac_setups', 'failed_steps'],
                                   out['counts'][0].cpu().numpy().tolist()), status=STATUS_NAMES.get(st, st))
        t_end = float(out['t'][0]) + t0
        if save_first_and_last_only:
            times = np.array([t_end])
            states = q[None, :]
        else:
            k = int(out['steps'][0])
            times = out['times'][0, :k + 1] + t0
            states = out['states'][0, :k + 1]
        self._current_state = q
        self._current_time = t_end
        self._integrations += 1
        from .library import Dimension, Library
        lib = Library(Dimension('time', times))
        names = self._mechanism.species_names
        Tidx = self._temperature_index
        lib['temperature'] = states[:, Tidx].copy()
        if self._configuration == 'isochoric':
            lib['density'] = states[:, 0].copy()
        else:
            lib['pressure'] = np.full(times.size, self._initial_pressure)
        last = np.ones(times.size)
        for i, s in enumerate(names[:-1]):
            lib['mass fraction ' + s] = states[:, Tidx + 1 + i].copy()
            last -= states[:, Tidx + 1 + i]
        lib['mass fraction ' + names[-1]] = last
        return lib

    def integrate(self, stop_at_time=None, stop_at_steady=None, stop_criteria=None, first_time_step=1.e-6,
                  max_time_step=1.e6, minimum_time_step_count=40, transient_tolerance=1.e-10, write_log=False,
                  log_rate=100, maximum_steps_per_jacobian=1, nonlinear_solve_tolerance=1.e-12,
                  linear_solver='lapack', plot=None, save_first_and_last_only=False, **kwargs):
        """reactors.py:429-678. A stop_at_time of the reference is an absolute time; stop_criteria callables are
        not on the GPU path (integrate_to_steady and compute_ignition_delay are)."""
        if stop_criteria is not None:
            raise NotImplementedError('stop_criteria callables are not on the GPU path')
        return self._integrate(save_first_and_last_only=save_first_and_last_only,
                               stop_at_time=None if stop_at_time is None else stop_at_time - self._current_time,
                               stop_at_steady=stop_at_steady, first_time_step=first_time_step,
                               max_time_step=max_time_step, minimum_time_step_count=minimum_time_step_count,
                               transient_tolerance=transient_tolerance,
                               maximum_steps_per_jacobian=maximum_steps_per_jacobian,
                               nonlinear_tolerance=nonlinear_solve_tolerance)

    def integrate_to_steady(self, steady_tolerance=1.e-6, **kwargs):
        return self.integrate(stop_at_steady=steady_tolerance, **kwargs)

    def integrate_to_time(self, final_time, **kwargs):
        return self.integrate(stop_at_time=final_time, **kwargs)

    def integrate_to_steady_after_ignition(self, steady_tolerance=1.e-4, delta_temperature_ignition=400., **kwargs):
        """Integrate until the reactor has ignited (T > T0 + delta_temperature_ignition) and the step residual is
        below steady_tolerance (reactors.py:711-743), for slowly evolving mixtures whose first residuals are already
        small. The reference runs one integration with that stop criterion. Here it is two integrations of the GPU
        integrator: to ignition (its ignition stop rule, with no give-up on small residuals), then on to a steady
        state from there, starting from the last accepted step size and completing the minimum step count. The
        restart re-evaluates the Jacobian and restarts the step-size control at ignition, so the steps after
        ignition are not the reference's; both runs end at the same steady state within steady_tolerance.
        Returns the joined trajectory (first and last states only with save_first_and_last_only)."""
        if self._heat_transfer == 'isothermal':
            raise ValueError('integrate_to_steady_after_ignition() called on an isothermal reactor! This is not '
                             'currently supported!')
        if kwargs.get('stop_criteria') is not None or kwargs.get('stop_at_steady') is not None:
            raise ValueError('integrate_to_steady_after_ignition() sets its own stop rules')
        save_fl = kwargs.pop('save_first_and_last_only', False)
        min_steps = kwargs.get('minimum_time_step_count', 40)
        stop_at_time = kwargs.get('stop_at_time')
        lib1 = self._integrate(save_first_and_last_only=False, delta_temperature_ignition=delta_temperature_ignition,
                               minimum_allowable_residual=0.,
                               first_time_step=kwargs.get('first_time_step', 1.e-6),
                               max_time_step=kwargs.get('max_time_step', 1.e6),
                               minimum_time_step_count=min_steps,
                               transient_tolerance=kwargs.get('transient_tolerance', 1.e-10),
                               nonlinear_tolerance=kwargs.get('nonlinear_solve_tolerance', 1.e-12),
                               maximum_steps_per_jacobian=kwargs.get('maximum_steps_per_jacobian', 1),
                               stop_at_time=None if stop_at_time is None else stop_at_time - self._current_time)
        t1 = lib1.dim('time').values
        if stop_at_time is not None and self._current_time >= stop_at_time:
            return _join_trajectories(lib1, lib1[-1:], save_fl)
        steps1 = t1.size - 1
        rest = dict(kwargs)
        rest['minimum_time_step_count'] = max(0, min_steps - steps1)
        if t1.size > 1:
            rest['first_time_step'] = float(t1[-1] - t1[-2])
        lib2 = self.integrate(stop_at_steady=steady_tolerance, **rest)
        return _join_trajectories(lib1, lib2, save_fl)

    def compute_ignition_delay(self, delta_temperature_ignition=400., minimum_allowable_residual=1.e-12,
                               return_solution=False, **kwargs):
        if self._heat_transfer == 'isothermal':
            raise ValueError('compute_ignition_delay() called on an isothermal reactor! This is not currently '
                             'supported!')
        lib = self._integrate(save_first_and_last_only=not return_solution,
                              delta_temperature_ignition=delta_temperature_ignition,
                              minimum_allowable_residual=minimum_allowable_residual,
                              first_time_step=kwargs.get('first_time_step', 1.e-6),
                              max_time_step=kwargs.get('max_time_step', 1.e6),
                              minimum_time_step_count=kwargs.get('minimum_time_step_count', 40),
                              transient_tolerance=kwargs.get('transient_tolerance', 1.e-10),
                              nonlinear_tolerance=kwargs.get('nonlinear_solve_tolerance', 1.e-12),
                              maximum_steps_per_jacobian=kwargs.get('maximum_steps_per_jacobian', 1),
                              stop_at_time=None if kwargs.get('stop_at_time') is None
                              else kwargs['stop_at_time'] - self._current_time)
        tau = self._current_time
        return (tau, lib) if return_solution else tau
