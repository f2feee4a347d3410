"""ORACLE -- test infrastructure, not the product.

CPU restatement of Spitfire's adiabatic steady-flamelet solvers on the oracle's Griffon restatement:

* ``FlameletOperator``: the closures ``_adiabatic_rhs`` / ``_adiabatic_jac`` / ``_adiabatic_jac_offset_scaled`` /
  ``_adiabatic_jac_and_eig`` (spitfire/chemistry/flamelet.py:642-735) over oracle/griffon_oracle.cpp, in the
  reference's calling convention (the full-grid dissipation rate is passed and indexed with the interior index,
  flamelet.py:654). The eigenvalue bound that Griffon gets from LAPACK dgeev (flamelet_kernels.cpp:1329-1341) is
  computed with numpy's eigvals.
* ``steady_solve_newton`` (flamelet.py:1352-1485), ``steady_solve_psitc`` (:1487-1703, with its adaptive restart)
  and ``compute_steady_state`` (:1705-1778, Newton with 38 iterations then psitc with 400).

Used by tests/ (to pin the GPU solvers and against the reference's own solver results) and by bench.py's CPU
baseline for the steady-flamelet workload.
"""

import numpy as np

import oracle as orc


class FlameletOperator:
    """heat_loss: None (adiabatic) or dict(T_conv, T_rad, h_conv, h_rad, scaled) over the interior points, the
    reference Flamelet's _T_conv, _T_rad, _h_conv, _h_rad and scale_heat_loss_by_temp_range."""

    def __init__(self, og, z, chi, oxy, fuel, pressure=101325., include_enthalpy_flux=True, include_variable_cp=True,
                 heat_loss=None):
        self.og = og
        self.heat_loss = heat_loss
        self.z = np.asarray(z, dtype=np.float64)
        self.chi = np.asarray(chi, dtype=np.float64)
        self.dz = self.z[1:] - self.z[:-1]
        self.nzi = self.z.size - 2
        self.ns = og.n_species
        self.oxy = np.asarray(oxy, dtype=np.float64)
        self.fuel = np.asarray(fuel, dtype=np.float64)
        self.pressure = pressure
        self.eflux = include_enthalpy_flux
        self.vcp = include_variable_cp
        n = self.nzi * self.ns
        self.cmajor, self.csub, self.csup = np.zeros(n), np.zeros(n), np.zeros(n)
        self.mc, self.nc = np.zeros(self.nzi), np.zeros(self.nzi)
        og.flamelet_stencils(self.dz, self.nzi, self.chi, np.ones(self.ns), self.cmajor, self.csub, self.csup,
                             self.mc, self.nc)
        self.null = np.zeros(1)
        self.scales = np.ones(n)
        self.scales[::self.ns] = 1.e3
        self.max_dissipation_rate = float(np.max(self.chi))

    def _heat(self):
        h = self.heat_loss
        if h is None:
            n = self.null
            return True, n, n, n, n, False
        return (False, np.asarray(h['T_conv'], dtype=np.float64), np.asarray(h['T_rad'], dtype=np.float64),
                np.asarray(h['h_conv'], dtype=np.float64), np.asarray(h['h_rad'], dtype=np.float64),
                bool(h.get('scaled', False)))

    def rhs(self, state, eflux=None, vcp=None):
        out = np.zeros(self.nzi * self.ns)
        adiabatic, Tc, Tr, hc, hr, scaled = self._heat()
        self.og.flamelet_rhs(state, self.pressure, self.oxy, self.fuel, adiabatic, Tc, Tr, hc, hr, self.nzi,
                             self.cmajor, self.csub, self.csup, self.mc, self.nc, self.chi,
                             self.eflux if eflux is None else eflux, self.vcp if vcp is None else vcp, scaled, out)
        return out

    def jac(self, state, eflux=None, scale_and_offset=False, prefactor=0.):
        adiabatic, Tc, Tr, hc, hr, scaled = self._heat()
        return self.og.flamelet_jacobian_values(state, self.pressure, self.oxy, self.fuel, adiabatic, Tc, Tr, hc, hr,
                                                self.nzi, self.cmajor, self.csub, self.csup, self.mc, self.nc,
                                                self.chi, scale_and_offset, prefactor, 0,
                                                self.eflux if eflux is None else eflux, scaled)

    def blocks(self, values):
        """[nzi, row, col] diagonal blocks of a BTDDOD value array."""
        ns = self.ns
        return np.swapaxes(values[:self.nzi * ns * ns].reshape(self.nzi, ns, ns), 1, 2)

    def expeig(self, state, diffterm):
        """Per row: max(max Re(lambda) - diffterm, 0) over the eigenvalues of the point's chemistry block (the
        block without the diffusion diagonal; the enthalpy-flux correction is applied after the eigenvalues in
        flamelet_kernels.cpp:1329-1381, so the block of the Jacobian without it is the one to use)."""
        B = self.blocks(self.jac(state, eflux=False))
        out = np.zeros(self.nzi * self.ns)
        for i in range(self.nzi):
            A = B[i] - np.diag(self.cmajor[i * self.ns:(i + 1) * self.ns])
            out[i * self.ns:(i + 1) * self.ns] = max(np.max(np.linalg.eigvals(A).real) - diffterm, 0.)
        return out

    def jac_and_eig(self, state, diffterm):
        return self.jac(state), self.expeig(state, diffterm)

    def norm(self, v):
        return float(np.max(np.abs(v / self.scales)))


def _factor(J, nzi, ns):
    return orc.btddod_full_factorize(J, nzi, ns)


def _solve(fac, b, nzi, ns):
    d, l, piv = fac
    return orc.btddod_full_solve(d, l, piv, b, nzi, ns)


def steady_solve_newton(op, state, tolerance=1.e-6, max_iterations=10, max_factor_line_search=1.5,
                        max_allowed_residual=1.e6, min_allowable_state_var=-1.e-6):
    """flamelet.py:1352-1485. Returns (state or None, iterations or None, converged)."""
    state = np.array(state, dtype=np.float64)
    nzi, ns = op.nzi, op.ns
    it = 0
    res = tolerance + 1.
    rhs = op.rhs(state)
    evaluate_jacobian = True
    fac = None
    while res > tolerance and it < max_iterations:
        it += 1
        if evaluate_jacobian:
            fac = _factor(-op.jac(state), nzi, ns)
            evaluate_jacobian = False
        dstate = _solve(fac, rhs, nzi, ns)
        if not np.all(np.isfinite(dstate)):
            return None, None, False
        norm_old = op.norm(rhs)
        alpha = 1.
        rhs = op.rhs(state + dstate)
        if not np.all(np.isfinite(rhs)):
            return None, None, False
        while op.norm(rhs) > max_factor_line_search * norm_old and alpha > 0.001:
            alpha *= 0.5
            dstate *= alpha
            rhs = op.rhs(state + dstate)
            evaluate_jacobian = True
        state += dstate
        res = op.norm(rhs)
        if res > max_allowed_residual or np.min(state) < min_allowable_state_var:
            return None, None, False
    state[state < 0] = 0.
    if it > max_iterations or res > tolerance:
        return None, None, False
    return state, it, True


def steady_solve_psitc(op, state, tolerance=1.e-6, max_iterations=400, min_allowable_state_var=-1.e-6, ds_init=1.,
                       ds_init_decrease=4., adaptive_restart=True, diffusion_factor=4., global_ds=False,
                       ds_safety=0.1, ds_ramp=1.1, ds_max=1.e4, max_factor_line_search=1.5,
                       max_allowed_residual=1.e6, max_recursion_depth=20, _recursion_depth=0):
    """flamelet.py:1487-1703. Returns (state or None, iterations or None, converged, min ds)."""
    args = dict(locals())
    del args['op'], args['state']
    initial = np.array(state, dtype=np.float64)
    state = initial.copy()
    nzi, ns = op.nzi, op.ns
    diffterm = diffusion_factor * op.max_dissipation_rate
    ds = np.full(nzi * ns, ds_init)
    it = 0
    jac_age = 0
    res = tolerance + 1.
    rhs = op.rhs(state)
    evaluate_jacobian = True
    fac = None

    def restart():
        if _recursion_depth > max_recursion_depth or not adaptive_restart:
            return None, None, False, float(np.min(ds))
        a = dict(args)
        a['ds_init'] = ds_init / ds_init_decrease
        a['_recursion_depth'] = _recursion_depth + 1
        return steady_solve_psitc(op, initial, **a)

    while res > tolerance and it < max_iterations:
        it += 1
        if evaluate_jacobian:
            J, expeig = op.jac_and_eig(state, diffterm)
            ds = np.minimum(np.minimum(ds_safety / (expeig + 1.e-16), ds_ramp * ds), ds_max)
            if global_ds or it == 1:
                ds[:] = np.min(ds)
            J = -J
            for iz in range(nzi):
                for q in range(ns):
                    J[iz * ns * ns + q * (ns + 1)] += 1. / ds[iz * ns + q]
            fac = _factor(J, nzi, ns)
            jac_age = 0
            evaluate_jacobian = False
        else:
            jac_age += 1
        evaluate_jacobian = (jac_age == 8) or res > 1.e-2
        dstate = _solve(fac, rhs, nzi, ns)
        if not np.all(np.isfinite(dstate)):
            return restart()
        norm_old = op.norm(rhs)
        alpha = 1.
        rhs = op.rhs(state + dstate)
        if not np.all(np.isfinite(rhs)):
            return restart()
        while op.norm(rhs) > max_factor_line_search * norm_old and alpha > 0.001:
            alpha *= 0.5
            dstate *= alpha
            rhs = op.rhs(state + dstate)
            evaluate_jacobian = True
        state += dstate
        res = op.norm(rhs)
        if res > max_allowed_residual or np.min(state) < min_allowable_state_var:
            return restart()
    state[state < 0] = 0.
    if it > max_iterations or res > tolerance:
        return None, None, False, float(np.min(ds))
    return state, it, True, float(np.min(ds))


def compute_steady_state(op, state, tolerance=1.e-6):
    """Newton (38 iterations) then psitc (400), flamelet.py:1705-1778 without the ESDIRK fallback.
    Returns (state or None, 'newton' | 'psitc' | None, iterations)."""
    s, it, conv = steady_solve_newton(op, state, tolerance=tolerance, max_iterations=38)
    if conv:
        return s, 'newton', it
    s, it, conv, _ = steady_solve_psitc(op, state, tolerance=tolerance, max_iterations=400)
    return (s, 'psitc', it) if conv else (None, None, None)
