"""GPU-backed drop-in for Spitfire's ``spitfire.griffon.griffon.PyCombustionKernels`` (griffon.pyx:220-987).

The mechanism setters keep Griffon's names and argument order (griffon.pyx:234-551); the mechanism is built on
the current CUDA device at the first evaluation (``sf_mech_create``). Two kinds of evaluation methods exist:

* batched methods (``*_batch``) on torch CUDA float64 tensors with a leading batch dimension -- the hot path;
* the reference's single-state methods with its exact names, positional conventions and output-argument style
  on numpy arrays (e.g. ``production_rates(T, rho, y, out)`` -- the first positional argument is used as the
  temperature, as in griffon.pyx:763-768; ``flamelet_rhs(..., T_conv, T_rad, h_conv, h_rad, ...)`` as in
  griffon.pyx:580-620). They copy to the GPU, run the batched kernel for one state and copy back.

There is no CPU fallback: without the native library or a CUDA device these methods raise.
"""

import ctypes as C

import numpy as np

from . import _native as N
from ._desc import GriffonSetters, reactor_params


def _torch():
    import torch
    return torch


class PyCombustionKernels(GriffonSetters):
    def __init__(self):
        self._rec = None
        self._mech = None
        self._device = None

    # ------------------------------------------------------------------------------------------------ setup
    def _mechanism_changed(self):
        self._release()

    def _release(self):
        if self._mech is not None:
            try:
                N.load().sf_mech_destroy(self._mech)
            except Exception:
                pass
            self._mech = None

    def __del__(self):
        self._release()

    def __getstate__(self):
        return {'_rec': self._rec}

    def __setstate__(self, st):
        self._rec = st['_rec']
        self._mech = None
        self._device = None

    @property
    def handle(self):
        """Native mechanism on the current CUDA device (built on first use)."""
        torch = _torch()
        if not torch.cuda.is_available():
            raise N.NativeError('spitfire_gb300 needs a CUDA device (no CPU fallback)')
        dev = torch.cuda.current_device()
        if self._mech is not None and self._device != dev:
            self._release()
        if self._mech is None:
            if self._rec is None:
                raise ValueError('mechanism has no data; call the mechanism_* setters first')
            L = N.load()
            import ctypes as C
            h = C.c_void_p()
            N.check(L.sf_mech_create(C.byref(self._rec.desc()), C.byref(h)))
            self._mech = h
            self._device = dev
        return self._mech

    @property
    def n_species(self):
        return len(self._rec.species)

    @property
    def n_reactions(self):
        return len(self._rec.reactions)

    def scratch_layout(self):
        """{'rhs': doubles, 'total': doubles, 'blob_bytes': bytes} of the kernels' per-state scratch and blob."""
        a, b, c = C.c_int(), C.c_int(), C.c_longlong()
        N.check(N.load().sf_mech_layout(self.handle, C.byref(a), C.byref(b), C.byref(c)))
        return {'rhs': a.value, 'total': b.value, 'blob_bytes': c.value}

    def device_status(self, clear=True):
        return N.load().sf_device_status(self.handle, int(clear))

    def mechanism_counts(self):
        import ctypes as C
        ns, nr = C.c_int(), C.c_int()
        c = (C.c_int * 6)()
        N.check(N.load().sf_mech_info(self.handle, C.byref(ns), C.byref(nr), c))
        return dict(simple=c[0], three_body=c[1], lindemann=c[2], troe=c[3], dense=c[4], special_orders=c[5])

    # --------------------------------------------------------------------------------------- batched API
    @staticmethod
    def _dev(t):
        torch = _torch()
        t = torch.as_tensor(t, dtype=torch.float64)
        if not t.is_cuda:
            t = t.cuda()
        return t.contiguous()

    def thermo_batch(self, what, T, Y):
        """what: 0 cp, 1 cv, 2 h, 3 e, 4 cp_i, 5 cv_i, 6 h_i, 7 e_i, 8 mmw, 9 dcp/dT, 10 dcp_i/dT."""
        torch = _torch()
        T, Y = self._dev(T), self._dev(Y)
        n = T.numel()
        per = what in (4, 5, 6, 7, 10)
        out = torch.empty((n, self.n_species) if per else (n,), dtype=torch.float64, device=T.device)
        N.check(N.load().sf_thermo_batch(self.handle, what, n, N.ptr(T), N.ptr(Y), N.ptr(out), N.stream_handle()))
        return out

    def production_rates_batch(self, T, rho, Y, out=None):
        torch = _torch()
        T, rho, Y = self._dev(T), self._dev(rho), self._dev(Y)
        n = T.numel()
        out = torch.empty((n, self.n_species), dtype=torch.float64, device=T.device) if out is None else out
        N.check(N.load().sf_production_rates_batch(self.handle, n, N.ptr(T), N.ptr(rho), N.ptr(Y), N.ptr(out),
                                                   N.stream_handle()))
        return out

    def rates_sens_batch(self, rho, T, Y, option=0):
        torch = _torch()
        T, rho, Y = self._dev(T), self._dev(rho), self._dev(Y)
        n, ns = T.numel(), self.n_species
        w = torch.empty((n, ns), dtype=torch.float64, device=T.device)
        S = torch.empty((n, (ns + 1) ** 2), dtype=torch.float64, device=T.device)
        N.check(N.load().sf_rates_sens_batch(self.handle, n, N.ptr(rho), N.ptr(T), N.ptr(Y), int(option), N.ptr(w),
                                             N.ptr(S), N.stream_handle()))
        return w, S

    def reactor_params(self, configuration, **kw):
        return reactor_params(configuration, **kw)

    def reactor_rhs_batch(self, params, q, pressures=None, out=None):
        torch = _torch()
        q = self._dev(q)
        pr = self._dev(pressures) if pressures is not None else None
        out = torch.empty_like(q) if out is None else out
        import ctypes as C
        N.check(N.load().sf_reactor_rhs_batch(self.handle, C.byref(params), q.shape[0], N.ptr(q), N.ptr(pr),
                                              N.ptr(out), N.stream_handle()))
        return out

    def reactor_jac_batch(self, params, q, rates_option=0, pressures=None, out_rhs=None, out_jac=None):
        torch = _torch()
        q = self._dev(q)
        n, neq = q.shape
        pr = self._dev(pressures) if pressures is not None else None
        out_rhs = torch.empty_like(q) if out_rhs is None else out_rhs
        out_jac = torch.empty((n, neq * neq), dtype=torch.float64, device=q.device) if out_jac is None else out_jac
        import ctypes as C
        N.check(N.load().sf_reactor_jac_batch(self.handle, C.byref(params), int(rates_option), n, N.ptr(q),
                                              N.ptr(pr), N.ptr(out_rhs), N.ptr(out_jac), N.stream_handle()))
        return out_rhs, out_jac

    def reactor_jac_host_batch(self, params, q, out_rhs, out_jac, rates_option=0, pressures=None, chunk_states=0):
        """RHS and Jacobian of states in HOST memory into host outputs (sf_reactor_jac_host_batch): q [n, neq],
        out_rhs [n, neq], out_jac [n, neq*neq] (torch CPU tensors, pinned for asynchronous copies, or numpy arrays);
        the copies back overlap the computation of the next chunk. Returns on the current stream without waiting."""
        torch = _torch()
        import ctypes as C
        n = q.shape[0]
        L = N.load()
        need = int(L.sf_reactor_jac_host_workspace_size(self.handle, C.byref(params), n))
        ws = getattr(self, '_host_ws', None)
        if ws is None or ws.numel() * 8 < need:
            self._host_ws = ws = torch.empty(need // 8 + 1, dtype=torch.float64, device='cuda')
        hp = lambda a: (a.data_ptr() if hasattr(a, 'data_ptr') else a.ctypes.data) if a is not None else None
        N.check(L.sf_reactor_jac_host_batch(self.handle, C.byref(params), int(rates_option), n, hp(q), hp(pressures),
                                            hp(out_rhs), hp(out_jac), int(chunk_states), N.ptr(ws), ws.numel() * 8,
                                            N.stream_handle()))
        return out_rhs, out_jac

    def reactor_jac_plain_batch(self, params, q, pressures=None, workspace=None):
        """Plain single-state GPU form (one thread per state), the comparison point of the batched kernel."""
        torch = _torch()
        q = self._dev(q)
        n, neq = q.shape
        pr = self._dev(pressures) if pressures is not None else None
        L = N.load()
        nbytes = L.sf_reactor_jac_plain_workspace_size(self.handle, n)
        if workspace is None or workspace.numel() * workspace.element_size() < nbytes:
            workspace = torch.empty(nbytes // 8 + 1, dtype=torch.float64, device=q.device)
        out_rhs = torch.empty_like(q)
        out_jac = torch.empty((n, neq * neq), dtype=torch.float64, device=q.device)
        import ctypes as C
        N.check(L.sf_reactor_jac_plain_batch(self.handle, C.byref(params), n, N.ptr(q), N.ptr(pr), N.ptr(out_rhs),
                                             N.ptr(out_jac), N.ptr(workspace),
                                             workspace.numel() * workspace.element_size(), N.stream_handle()))
        return out_rhs, out_jac

    # ------------------------------------------------------------------ reference-named single-state methods
    def _np1(self, t):
        return t.detach().cpu().numpy()

    def mixture_molecular_weight(self, y):
        return float(self.thermo_batch(8, [300.], np.asarray(y)[None, :])[0])

    def mole_fractions(self, y, x):
        mmw = self.mixture_molecular_weight(y)
        x[:] = np.asarray(y) * mmw / np.asarray(self._rec.species_mw)

    def ideal_gas_density(self, p, T, y):
        return p * self.mixture_molecular_weight(y) / (T * self._rec.gas_constant)

    def ideal_gas_pressure(self, rho, T, y):
        return rho * T * self._rec.gas_constant / self.mixture_molecular_weight(y)

    def cp_mix(self, T, y):
        return float(self.thermo_batch(0, [T], np.asarray(y)[None, :])[0])

    def cv_mix(self, T, y):
        return float(self.thermo_batch(1, [T], np.asarray(y)[None, :])[0])

    def enthalpy_mix(self, T, y):
        return float(self.thermo_batch(2, [T], np.asarray(y)[None, :])[0])

    def energy_mix(self, T, y):
        return float(self.thermo_batch(3, [T], np.asarray(y)[None, :])[0])

    def _species(self, what, T, out):
        out[:] = self._np1(self.thermo_batch(what, [T], np.ones((1, self.n_species)))[0])

    def species_cp(self, T, out):
        self._species(4, T, out)

    def species_cv(self, T, out):
        self._species(5, T, out)

    def species_enthalpies(self, T, out):
        self._species(6, T, out)

    def species_energies(self, T, out):
        self._species(7, T, out)

    def dcpdT_species(self, T, mass_fractions, out):
        out[:] = self._np1(self.thermo_batch(10, [T], np.asarray(mass_fractions)[None, :])[0])

    def production_rates(self, density, temperature, mass_fractions, prodrates):
        """griffon.pyx:763-768 forwards its first positional argument as the temperature."""
        w = self.production_rates_batch([density], [temperature], np.asarray(mass_fractions)[None, :])
        prodrates[:] = self._np1(w[0])

    def prod_rates_primitive_sensitivities(self, density, temperature, mass_fractions, rates_sensitivity_option,
                                           prod_rates_sens):
        w, S = self.rates_sens_batch([density], [temperature], np.asarray(mass_fractions)[None, :],
                                     rates_sensitivity_option)
        prod_rates_sens[:] = self._np1(S[0])

    def _params(self, configuration, p_or_rho, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_):
        yptr = None
        if open_:
            # the feed mass fractions live on the device for the call (kept until the next call replaces them;
            # the reference-shaped methods read their results back, which orders the two)
            self._feed_Y = self._dev(np.asarray(Yin, dtype=np.float64).reshape(-1))
            yptr = self._feed_Y.data_ptr()
        if configuration == 'isobaric':
            return reactor_params('isobaric', int(heat), bool(open_), pressure=p_or_rho, inflow_temperature=Tin,
                                  inflow_Y_ptr=yptr, tau=tau, fluid_temperature=Tc, surface_temperature=Tr,
                                  h_convection=hc, eps_radiation=eps, surface_area_to_volume=SoV)
        return reactor_params('isochoric', int(heat), bool(open_), inflow_density=p_or_rho, inflow_temperature=Tin,
                              inflow_Y_ptr=yptr, tau=tau, fluid_temperature=Tc, surface_temperature=Tr,
                              h_convection=hc, eps_radiation=eps, surface_area_to_volume=SoV)

    def reactor_rhs_isobaric(self, state, pressure, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_, out):
        P = self._params('isobaric', pressure, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_)
        out[:] = self._np1(self.reactor_rhs_batch(P, np.asarray(state)[None, :])[0])

    def reactor_jac_isobaric(self, state, pressure, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_, ropt, topt,
                             out_rhs, out_jac):
        P = self._params('isobaric', pressure, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_)
        r, J = self.reactor_jac_batch(P, np.asarray(state)[None, :], ropt)
        out_rhs[:] = self._np1(r[0])
        out_jac[:] = self._np1(J[0])

    def reactor_rhs_isochoric(self, state, rho_in, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_, out):
        P = self._params('isochoric', rho_in, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_)
        out[:] = self._np1(self.reactor_rhs_batch(P, np.asarray(state)[None, :])[0])

    def reactor_jac_isochoric(self, state, rho_in, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_, ropt, out_rhs,
                              out_jac):
        P = self._params('isochoric', rho_in, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_)
        r, J = self.reactor_jac_batch(P, np.asarray(state)[None, :], ropt)
        out_rhs[:] = self._np1(r[0])
        out_jac[:] = self._np1(J[0])
