"""ORACLE -- test infrastructure, not the product.

CPU restatement of Spitfire's reactor time integration, as HomogeneousReactor.integrate runs it with its
defaults: odesolve (src/spitfire/time/integrator.py:229-713) driving KennedyCarpenterS6P4Q3 (ESDIRK64,
time/methods.py:441-612) with SimpleNewtonSolver (time/nonlinear.py:143-268, frozen Jacobian) and PIController
(time/stepcontrol.py:50-117); the right-hand side and Jacobian come from the oracle's Griffon restatement and the
linear algebra from LAPACK dgetrf/dgetrs through scipy, as in chemistry/reactors.py:340-356.
Used by tests (ignition delays, step counts) and by the CPU baseline of the ignition benchmark.
"""

import numpy as np
from scipy.linalg.lapack import dgetrf, dgetrs

# ESDIRK64 tableau (methods.py:464-500)
GAMMA = 0.25
A = np.array([[0., 0., 0., 0., 0., 0.],
              [0.25, GAMMA, 0., 0., 0., 0.],
              [8611. / 62500., -1743. / 31250., GAMMA, 0., 0., 0.],
              [5012029. / 34652500., -654441. / 2922500., 174375. / 388108., GAMMA, 0., 0.],
              [15267082809. / 155376265600., -71443401. / 120774400., 730878875. / 902184768.,
               2285395. / 8070912., GAMMA, 0.],
              [82889. / 524892., 0., 15625. / 83664., 69875. / 102672., -2260. / 8211., GAMMA]])
B = A[5].copy()
BH = np.array([4586570599. / 29645900160., 0., 178811875. / 945068544., 814220225. / 1159782912.,
               -3700637. / 11593932., 61727. / 225920.])

STATUS = {'done': 1, 'ignited': 2, 'steady': 3, 'max_steps': 4, 'nan': 5, 'no_ignition': 6}


class ReactorProblem:
    """Reactor RHS/Jacobian closures (reactors.py:538-592) over the oracle Griffon. Diathermal reactors take
    convection_temperature, radiation_temperature, convection_coefficient, radiative_emissivity and
    surface_area_to_volume; any of the first four may be a function of time. As in the reference
    (_update_heat_transfer_parameters, reactors.py:324-328), every right-hand side evaluation refreshes them at its
    own time and the Jacobian uses the values the most recent right-hand side left (those at t = 0 before the
    first one, reactors.py:275-278)."""

    HEAT = (('convection_temperature', 'fluid_temperature'), ('radiation_temperature', 'surface_temperature'),
            ('convection_coefficient', 'h_convection'), ('radiative_emissivity', 'eps_radiation'))

    def __init__(self, og, configuration, pressure=101325., heat='adiabatic', convection_temperature=300.,
                 radiation_temperature=300., convection_coefficient=0., radiative_emissivity=0.,
                 surface_area_to_volume=1.):
        import oracle as orc
        from spitfire_gb300._desc import reactor_params
        self.og = og
        self.configuration = configuration
        self.pressure = pressure
        self.P = reactor_params(configuration, heat, pressure=pressure, surface_area_to_volume=surface_area_to_volume)
        self._funcs = {}
        given = dict(convection_temperature=convection_temperature, radiation_temperature=radiation_temperature,
                     convection_coefficient=convection_coefficient, radiative_emissivity=radiative_emissivity)
        for name, field in self.HEAT:
            v = given[name]
            if callable(v):
                self._funcs[field] = v
            setattr(self.P, field, v(0.) if callable(v) else v)
        self._yin = np.zeros(og.n_species)
        self.P.inflow_Y = orc._p(self._yin)
        self.Tidx = 0 if configuration == 'isobaric' else 1
        self.pres = np.array([pressure]) if configuration == 'isobaric' else None

    def _update(self, t):
        for field, f in self._funcs.items():
            if field == 'inflow_Y':
                self._yin[:] = np.asarray(f(t), dtype=np.float64)
            else:
                setattr(self.P, field, f(t))

    def rhs(self, q, t=0.):
        self._update(t)
        return self.og.reactor_rhs_batch(self.P, q[None, :], pressures=self.pres)[0]

    def jac(self, q):
        n = q.size
        _, J = self.og.reactor_jac_batch(self.P, q[None, :], 0, pressures=self.pres)
        return J[0].reshape((n, n), order='F')


class OpenReactorProblem(ReactorProblem):
    """Open (mass-exchange) reactor: a feed of temperature `feed_temperature`, mass fractions `feed_Y`, density
    `feed_density` (isochoric) and mixing time `tau`. The feed temperature, mass fractions and mixing time may be
    functions of time: as in the reference's closures (reactors.py:538-592 with _update_mass_transfer_parameters,
    :330-333) every right-hand side evaluation refreshes them at its own time, and the Jacobian uses the values the
    most recent right-hand side left (those at t = 0 before the first one, reactors.py:275-282). A feed density
    function is evaluated once, at t = 0, and never refreshed, as in the reference."""

    def __init__(self, og, configuration, feed_temperature, feed_Y, tau, pressure=101325., heat='adiabatic',
                 feed_density=0., **heat_params):
        import oracle as orc
        super().__init__(og, configuration, pressure=pressure, heat=heat, **heat_params)
        self.P.open = 1
        at0 = lambda v: v(0.) if callable(v) else v
        self.P.tau = at0(tau)
        self.P.inflow_density = at0(feed_density)
        self._yin = np.asarray(at0(feed_Y), dtype=np.float64).copy()
        self.P.inflow_Y = orc._p(self._yin)
        self.P.inflow_temperature = at0(feed_temperature)
        for field, v in (('inflow_temperature', feed_temperature), ('tau', tau), ('inflow_Y', feed_Y)):
            if callable(v):
                self._funcs[field] = v


C = A.sum(axis=1)  # stage times t + c_s dt


def integrate(prob, q0, first_time_step=1.e-6, max_time_step=1.e6, transient_tolerance=1.e-10,
              nonlinear_tolerance=1.e-12, minimum_time_step_count=40, maximum_time_step_count=np.inf,
              max_nonlinear_iter=20, maximum_steps_per_jacobian=1, stop_at_time=None, delta_temperature_ignition=None,
              minimum_allowable_residual=1.e-12, stop_at_steady=None, max_attempts=1000000, save_each_step=False,
              stop_criteria=None, post_step_clip=True):
    """Returns dict(state, t, steps, newton_iters, jac_setups, failed_steps, status, t_interp[, times, states]);
    t_interp: with delta_temperature_ignition, the Hermite-interpolated first crossing of T0 + delta (None if none).

    prob gives rhs(q, t) and either jac(q) (dense; LAPACK LU of dt*gamma*J - I) or linear_setup(q, prefactor) and
    linear_solve(r) (its own factorization of prefactor*J - I), and either Tidx (one temperature scaled by 1e3) or
    weights (the norm weighting, 1 / variable scales). stop_criteria(t, state, residual, steps) -> bool is checked
    after every attempt, before the minimum step count, as odesolve does (integrator.py:629-641)."""
    neq = q0.size
    if hasattr(prob, 'weights'):
        w = np.asarray(prob.weights, dtype=np.float64)
    else:
        w = np.ones(neq)
        w[prob.Tidx] = 1. / 1.e3  # 1 / variable_scales (reactors.py:321-322)
    T0 = q0[prob.Tidx] if delta_temperature_ignition is not None else None
    own_setup = hasattr(prob, 'linear_setup')
    state = q0.astype(np.float64).copy()
    t = 0.
    dt = first_time_step
    eval_setup = True
    setup_count = 0
    nsteps = 0
    nnewton = 0
    njac = 0
    nfail = 0
    lu = piv = None
    status = 0
    coerce = stop_at_time is not None
    times = [0.] if save_each_step else None
    states = [state.copy()] if save_each_step else None
    attempts = 0
    t_interp = None  # first crossing of T0 + delta, Hermite-interpolated over the crossing step
    while True:
        attempts += 1
        if attempts > max_attempts:
            status = STATUS['max_steps']
            break
        if coerce and t + dt > stop_at_time:
            dt = stop_at_time - t
        if eval_setup:
            if own_setup:
                prob.linear_setup(state, dt * GAMMA)
            else:
                Jm = prob.jac(state) * (dt * GAMMA)
                Jm[np.diag_indices(neq)] -= 1.
                lu, piv, _ = dgetrf(Jm)
            njac += 1
        setup_count += 1
        # ---- ESDIRK64 single step (methods.py:502-612)
        k = np.zeros((6, neq))
        k[0] = prob.rhs(state, t)
        Y = state.copy()
        nl_ok = True
        nl_slow = False
        for s in range(1, 6):
            prior = A[s, :s] @ k[:s]
            resid = dt * (GAMMA * k[s - 1] + prior) - (Y - state)
            conv = False
            f = k[s - 1]
            for it in range(1, max_nonlinear_iter + 1):
                dx = prob.linear_solve(resid) if own_setup else dgetrs(lu, piv, resid)[0]
                Y = Y - dx
                f = prob.rhs(Y, t + C[s] * dt)
                resid = dt * (GAMMA * f + prior) - (Y - state)
                nnewton += 1
                if np.max(np.abs(resid * w)) < nonlinear_tolerance:
                    conv = True
                    break
            k[s] = f
            if not conv:
                nl_ok = False
                nl_slow = True
        dstate = dt * (B @ k)
        dstate_h = dt * (BH @ k)
        err = np.max(np.abs((dstate - dstate_h) * w))
        residual = np.max(np.abs(dstate * w)) / dt
        # ---- governor (integrator.py:540-640)
        recent = dt
        if np.all(np.isfinite(dstate)):
            T_start = state[prob.Tidx] if T0 is not None else None
            state = state + dstate
            if post_step_clip:
                state[state < 0.] = 0.  # post_step_callback (reactors.py:506-508, flamelet.py:1119-1121)
            if T0 is not None and t_interp is None and state[prob.Tidx] > T0 + delta_temperature_ignition:
                t_interp = hermite_crossing(t, dt, T_start, state[prob.Tidx], k[0][prob.Tidx], k[5][prob.Tidx],
                                            T0 + delta_temperature_ignition)
            t = t + dt
            nsteps += 1
            if save_each_step:
                times.append(t)
                states.append(state.copy())
            # PI controller (stepcontrol.py:84-101): after a step the P factor is exactly 1
            if err < 1.e-16:
                dt = min(dt * 1.1, max_time_step)
            else:
                dt = min(dt * min(1.1, (transient_tolerance / err) ** 0.1333333333), max_time_step)
            # _check_linear_setup (integrator.py:100-130)
            if setup_count == maximum_steps_per_jacobian:
                setup_count = 0
                eval_setup = True
            elif nl_slow:
                dt *= 0.8
                eval_setup = True
            elif not nl_ok:
                dt *= 0.8
                eval_setup = True
            elif dt > recent * 1.05:
                eval_setup = True
            elif dt < recent * 0.9:
                eval_setup = True
            else:
                eval_setup = False
        else:
            dt *= 0.8
            eval_setup = True
            nfail += 1
        cont = True
        if stop_criteria is not None:
            cont = not stop_criteria(t, state, residual, nsteps)
        if delta_temperature_ignition is not None:
            ignited = state[prob.Tidx] > T0 + delta_temperature_ignition
            if residual > minimum_allowable_residual:
                cont = not ignited
                if ignited:
                    status = STATUS['ignited']
            else:
                status = STATUS['no_ignition']
                break
        if nsteps < minimum_time_step_count:
            cont = True
            if status == STATUS['ignited']:
                status = 0
        if nsteps > maximum_time_step_count:
            cont = False
            status = STATUS['max_steps']
        elif coerce and t >= stop_at_time:
            cont = False
            if status == 0:
                status = STATUS['done']
        elif stop_at_steady is not None and residual < stop_at_steady:
            cont = False
            status = STATUS['steady']
        if not cont:
            break
    out = dict(state=state, t=t, steps=nsteps, newton_iters=nnewton, jac_setups=njac, failed_steps=nfail,
               status=status, t_interp=t_interp)
    if save_each_step:
        out['times'] = np.array(times)
        out['states'] = np.array(states)
    return out


def hermite_crossing(t0, h, y0, y1, d0, d1, thr):
    """First time in [t0, t0 + h] at which the cubic Hermite interpolant (end values y0 <= thr < y1, end derivatives
    d0, d1) reaches thr: the first of 16 equal sub-intervals with a crossing, then 48 bisections. The GPU integrator
    refines its ignition delay the same way (a project-defined measure; the reference reports the step end)."""
    def p(s):
        s2, s3 = s * s, s * s * s
        return (2. * s3 - 3. * s2 + 1.) * y0 + (s3 - 2. * s2 + s) * h * d0 + (3. * s2 - 2. * s3) * y1 + \
            (s3 - s2) * h * d1
    lo, hi = 0., 1.
    for j in range(1, 17):
        if p(j / 16.) >= thr:
            lo, hi = (j - 1) / 16., j / 16.
            break
    for _ in range(48):
        mid = 0.5 * (lo + hi)
        if p(mid) >= thr:
            hi = mid
        else:
            lo = mid
    return t0 + hi * h


def ignition_delay(prob, q0, delta=400., **kw):
    r = integrate(prob, q0, delta_temperature_ignition=delta, **kw)
    return r['t'], r
