"""ORACLE -- test infrastructure, not the product.

Python side of the CPU restatement of Griffon (oracle/griffon_oracle.cpp) and of Spitfire's time integration
(oracle/integrate.py). Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use it, as the
checker. ``OracleGriffon`` keeps the method names and positional conventions of the reference's
``PyCombustionKernels`` (griffon.pyx:220-987), including the quirk that ``production_rates``' first positional
argument is the temperature (griffon.pyx:763-768 -> chemistry_kernels.cpp:29-33) and that ``flamelet_rhs`` takes
``T_conv, T_rad, h_conv, h_rad`` but forwards ``T_conv, h_conv, T_rad, h_rad`` (griffon.pyx:586-609).
"""

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from spitfire_gb300._desc import GriffonSetters, SfReactorParams, reactor_params  # noqa: E402

_LIB = None
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build():
    """Compile the restatement (make -C oracle port); quick, no reference sources needed."""
    subprocess.check_call(['make', '-s', '-C', HERE, 'port'])


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, '_build', 'libgriffon_oracle.so')
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_mech_create.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
        L.oracle_mech_destroy.argtypes = [C.c_void_p]
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_thermo.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp]
        L.oracle_production_rates.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp]
        L.oracle_rates_sens.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, C.c_int, _dp, _dp]
        L.oracle_reactor_rhs.argtypes = [C.c_void_p, C.POINTER(SfReactorParams), C.c_int, _dp, _dp, _dp]
        L.oracle_reactor_jac.argtypes = [C.c_void_p, C.POINTER(SfReactorParams), C.c_int, C.c_int, _dp, _dp, _dp,
                                         _dp]
        L.oracle_lu_factor.argtypes = [C.c_int, C.c_int, _dp, _ip, _ip]
        L.oracle_rate_param_sens.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _dp]
        L.oracle_lu_solve.argtypes = [C.c_int, C.c_int, _dp, _ip, _dp]
        L.oracle_flamelet_stencils.argtypes = [C.c_void_p, _dp, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.oracle_flamelet_rhs.argtypes = [C.c_void_p, _dp, C.c_double, _dp, _dp, C.c_int, _dp, _dp, _dp, _dp, C.c_int,
                                          _dp, _dp, _dp, _dp, _dp, _dp, C.c_int, C.c_int, C.c_int, _dp]
        L.oracle_flamelet_jacobian.argtypes = [C.c_void_p, _dp, C.c_double, _dp, _dp, C.c_int, _dp, _dp, _dp, _dp,
                                               C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int, C.c_double, C.c_int,
                                               C.c_int, C.c_int, _dp]
        L.oracle_btddod_full_factorize.argtypes = [_dp, C.c_int, C.c_int, _dp, _ip]
        L.oracle_btddod_full_solve.argtypes = [_dp, _dp, _ip, _dp, C.c_int, C.c_int, _dp]
        L.oracle_btddod_full_matvec.argtypes = [_dp, _dp, C.c_int, C.c_int, _dp]
        _LIB = L
    return _LIB


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a):
    return a.ctypes.data_as(_dp)


def _pi(a):
    return a.ctypes.data_as(_ip)


def set_threads(n):
    return lib().oracle_set_threads(int(n))


class OracleGriffon(GriffonSetters):
    """CPU restatement with PyCombustionKernels-compatible methods (single state) plus batched helpers."""

    def __init__(self):
        self._rec = None
        self._h = None

    def _mechanism_changed(self):
        self._release()

    def _release(self):
        if self._h is not None:
            lib().oracle_mech_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self._release()
        except Exception:
            pass

    @property
    def handle(self):
        if self._h is None:
            h = C.c_void_p()
            d = self._rec.desc()
            rc = lib().oracle_mech_create(C.byref(d), C.byref(h))
            if rc != 0:
                raise ValueError(lib().oracle_last_error().decode())
            self._h = h
        return self._h

    @property
    def n_species(self):
        return len(self._rec.species)

    # ---------------------------------------------------------------- thermodynamics (griffon.pyx:684-761)
    def _thermo(self, what, T, Y, per_species):
        T = _d(np.atleast_1d(T))
        Y = _d(Y).reshape(T.size, -1)
        out = np.zeros((T.size, self.n_species) if per_species else T.size)
        lib().oracle_thermo(self.handle, what, T.size, _p(T), _p(Y), _p(out))
        return out

    def mixture_molecular_weight(self, y):
        return float(self._thermo(8, 300., y, False)[0])

    def cp_mix(self, T, y):
        return float(self._thermo(0, T, y, False)[0])

    def cv_mix(self, T, y):
        return float(self._thermo(1, T, y, False)[0])

    def enthalpy_mix(self, T, y):
        return float(self._thermo(2, T, y, False)[0])

    def energy_mix(self, T, y):
        return float(self._thermo(3, T, y, False)[0])

    def species_cp(self, T, out):
        out[:] = self._thermo(4, T, np.ones(self.n_species), True)[0]

    def species_cv(self, T, out):
        out[:] = self._thermo(5, T, np.ones(self.n_species), True)[0]

    def species_enthalpies(self, T, out):
        out[:] = self._thermo(6, T, np.ones(self.n_species), True)[0]

    def species_energies(self, T, out):
        out[:] = self._thermo(7, T, np.ones(self.n_species), True)[0]

    def dcpdT_species(self, T, y, out):
        out[:] = self._thermo(10, T, y, True)[0]

    def ideal_gas_density(self, p, T, y):
        return p * self.mixture_molecular_weight(y) / (T * self._rec.gas_constant)

    def ideal_gas_pressure(self, rho, T, y):
        return rho * T * self._rec.gas_constant / self.mixture_molecular_weight(y)

    # ---------------------------------------------------------------- kinetics
    def production_rates(self, density, temperature, mass_fractions, prodrates):
        """First argument is used as T (griffon.pyx:763-768 passes it into the C++ temperature slot)."""
        w = self.production_rates_batch(np.array([density]), np.array([temperature]), _d(mass_fractions)[None, :])
        prodrates[:] = w[0]

    def production_rates_batch(self, T, rho, Y):
        T, rho, Y = _d(T), _d(rho), _d(Y)
        out = np.zeros_like(Y)
        lib().oracle_production_rates(self.handle, T.size, _p(T), _p(rho), _p(Y), _p(out))
        return out

    def rate_param_sens_batch(self, T, rho, Y):
        """(q [n][nr], s [n][nr]): net rates of progress and their derivatives with respect to the log of the forward
        (high-pressure for falloff) rate constant, reactions in the internal (setter) order."""
        T, rho, Y = _d(T), _d(rho), _d(Y)
        nr = len(self._rec.reactions)
        q = np.zeros((T.size, nr))
        sr = np.zeros((T.size, nr))
        lib().oracle_rate_param_sens(self.handle, T.size, _p(T), _p(rho), _p(Y), _p(q), _p(sr))
        return q, sr

    def prod_rates_primitive_sensitivities(self, density, temperature, mass_fractions, rates_sensitivity_option,
                                           prod_rates_sens):
        w, S = self.rates_sens_batch(np.array([density]), np.array([temperature]), _d(mass_fractions)[None, :],
                                     rates_sensitivity_option)
        prod_rates_sens[:] = S[0]

    def rates_sens_batch(self, rho, T, Y, option=0):
        rho, T, Y = _d(rho), _d(T), _d(Y)
        n, ns = Y.shape
        w = np.zeros((n, ns))
        S = np.zeros((n, (ns + 1) ** 2))
        lib().oracle_rates_sens(self.handle, n, _p(rho), _p(T), _p(Y), int(option), _p(w), _p(S))
        return w, S

    # ---------------------------------------------------------------- reactors (griffon.pyx:788-866)
    def reactor_rhs_batch(self, params, q, pressures=None):
        q = _d(q)
        out = np.zeros_like(q)
        pp = _d(pressures) if pressures is not None else None
        lib().oracle_reactor_rhs(self.handle, C.byref(params), q.shape[0], _p(q), _p(pp) if pp is not None else None,
                                 _p(out))
        return out

    def reactor_jac_batch(self, params, q, rates_option=0, pressures=None):
        q = _d(q)
        n, neq = q.shape
        rhs = np.zeros_like(q)
        J = np.zeros((n, neq * neq))
        pp = _d(pressures) if pressures is not None else None
        lib().oracle_reactor_jac(self.handle, C.byref(params), int(rates_option), n, _p(q),
                                 _p(pp) if pp is not None else None, _p(rhs), _p(J))
        return rhs, J

    def _params(self, configuration, pressure_or_rho_in, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_):
        yin = _d(Yin)
        self._keep_yin = yin
        if configuration == 'isobaric':
            p = reactor_params('isobaric', heat, open_, pressure=pressure_or_rho_in, inflow_temperature=Tin,
                               tau=tau, fluid_temperature=Tc, surface_temperature=Tr, h_convection=hc,
                               eps_radiation=eps, surface_area_to_volume=SoV)
        else:
            p = reactor_params('isochoric', heat, open_, inflow_density=pressure_or_rho_in, inflow_temperature=Tin,
                               tau=tau, fluid_temperature=Tc, surface_temperature=Tr, h_convection=hc,
                               eps_radiation=eps, surface_area_to_volume=SoV)
        p.inflow_Y = _p(yin)
        return p

    def reactor_rhs_isobaric(self, state, pressure, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_, out):
        P = self._params('isobaric', pressure, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_)
        out[:] = self.reactor_rhs_batch(P, _d(state)[None, :])[0]

    def reactor_jac_isobaric(self, state, pressure, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_, ropt, topt,
                             out_rhs, out_jac):
        P = self._params('isobaric', pressure, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_)
        r, J = self.reactor_jac_batch(P, _d(state)[None, :], ropt)
        out_rhs[:] = r[0]
        out_jac[:] = J[0]

    def reactor_rhs_isochoric(self, state, rho_in, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_, out):
        P = self._params('isochoric', rho_in, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_)
        out[:] = self.reactor_rhs_batch(P, _d(state)[None, :])[0]

    def reactor_jac_isochoric(self, state, rho_in, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_, ropt, out_rhs,
                              out_jac):
        P = self._params('isochoric', rho_in, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_)
        r, J = self.reactor_jac_batch(P, _d(state)[None, :], ropt)
        out_rhs[:] = r[0]
        out_jac[:] = J[0]

    # ---------------------------------------------------------------- flamelets (griffon.pyx:556-679)
    def flamelet_stencils(self, dz, nzi, chi, invLe, cmajor, csub, csup, mcoeff, ncoeff):
        dz, chi, invLe = _d(dz), _d(chi), _d(invLe)
        lib().oracle_flamelet_stencils(self.handle, _p(dz), int(nzi), _p(chi), _p(invLe), _p(cmajor), _p(csub),
                                       _p(csup), _p(mcoeff), _p(ncoeff))

    def flamelet_rhs(self, state, pressure, oxy, fuel, adiabatic, T_convection, T_radiation, h_convection,
                     h_radiation, nzi, cmajor, csub, csup, mcoeff, ncoeff, chi, include_enthalpy_flux,
                     include_variable_cp, use_scaled_heat_loss, out_rhs):
        a = [_d(v) for v in (state, oxy, fuel, T_convection, h_convection, T_radiation, h_radiation, cmajor, csub,
                             csup, mcoeff, ncoeff, chi)]
        # forwarded as (T_conv, h_conv, T_rad, h_rad) like griffon.pyx:586-609
        lib().oracle_flamelet_rhs(self.handle, _p(a[0]), float(pressure), _p(a[1]), _p(a[2]), int(adiabatic),
                                  _p(a[3]), _p(a[4]), _p(a[5]), _p(a[6]), int(nzi), _p(a[7]), _p(a[8]), _p(a[9]),
                                  _p(a[10]), _p(a[11]), _p(a[12]), int(include_enthalpy_flux),
                                  int(include_variable_cp), int(use_scaled_heat_loss), _p(out_rhs))

    def flamelet_jacobian_values(self, state, pressure, oxy, fuel, adiabatic, T_convection, T_radiation,
                                 h_convection, h_radiation, nzi, cmajor, csub, csup, mcoeff, ncoeff, chi,
                                 scale_and_offset, prefactor, rates_sensitivity_option, include_enthalpy_flux,
                                 use_scaled_heat_loss):
        ns = self.n_species
        out = np.zeros(ns * (nzi * ns + 2 * (nzi - 1)))
        a = [_d(v) for v in (state, oxy, fuel, T_convection, h_convection, T_radiation, h_radiation, cmajor, csub,
                             csup, mcoeff, ncoeff, chi)]
        lib().oracle_flamelet_jacobian(self.handle, _p(a[0]), float(pressure), _p(a[1]), _p(a[2]), int(adiabatic),
                                       _p(a[3]), _p(a[4]), _p(a[5]), _p(a[6]), int(nzi), _p(a[7]), _p(a[8]),
                                       _p(a[9]), _p(a[10]), _p(a[11]), _p(a[12]), int(scale_and_offset),
                                       float(prefactor), int(rates_sensitivity_option), int(include_enthalpy_flux),
                                       int(use_scaled_heat_loss), _p(out))
        return out


# ------------------------------------------------------------------------------------- dense and BTDDOD algebra
def lu_factor_batch(A):
    A = _d(A).copy()
    n, mm = A.shape
    m = int(round(np.sqrt(mm)))
    piv = np.zeros((n, m), dtype=np.int32)
    info = np.zeros(n, dtype=np.int32)
    lib().oracle_lu_factor(n, m, _p(A), _pi(piv), _pi(info))
    return A, piv, info


def lu_solve_batch(LU, piv, b):
    b = _d(b).copy()
    n, m = b.shape
    lib().oracle_lu_solve(n, m, _p(_d(LU)), _pi(np.ascontiguousarray(piv, dtype=np.int32)), _p(b))
    return b


def btddod_full_factorize(values, nb, bs):
    d = _d(values).copy()
    l = np.zeros(nb * bs * bs)
    piv = np.zeros(nb * bs, dtype=np.int32)
    lib().oracle_btddod_full_factorize(_p(d), nb, bs, _p(l), _pi(piv))
    return d, l, piv


def btddod_full_solve(d, l, piv, rhs, nb, bs):
    x = np.zeros(nb * bs)
    lib().oracle_btddod_full_solve(_p(_d(d)), _p(_d(l)), _pi(np.ascontiguousarray(piv, dtype=np.int32)),
                                   _p(_d(rhs)), nb, bs, _p(x))
    return x


def btddod_full_matvec(values, x, nb, bs):
    y = np.zeros(nb * bs)
    lib().oracle_btddod_full_matvec(_p(_d(values)), _p(_d(x)), nb, bs, _p(y))
    return y


def oracle_mechanism(path, phase=None):
    """(ChemicalMechanismSpec from the project loader, OracleGriffon filled with the same setter sequence)."""
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    spec = ChemicalMechanismSpec(cantera_input=path, group_name=phase) if phase else \
        ChemicalMechanismSpec(cantera_input=path)
    g = OracleGriffon()
    spec._populate_griffon(g)
    return spec, g
