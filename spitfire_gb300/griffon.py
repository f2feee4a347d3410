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
    def workspace(self, kind, n):
        """(device tensor, bytes) of the workspace sf_chem_workspace_size asks for a batched chemistry call of kind
        0 rates, 1 sensitivities, 2 right-hand sides, 3 Jacobians on n states: (None, 0) for the lane-group kernels.
        It comes from torch's caching allocator on the current stream, so calls on different streams get their own
        and a later call on the same stream reuses it."""
        nb = int(N.load().sf_chem_workspace_size(self.handle, int(kind), int(n)))
        if nb == 0:
            return None, 0
        torch = _torch()
        return torch.empty(nb // 8 + 1, dtype=torch.float64, device='cuda'), nb

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
        ws, nb = self.workspace(0, n)
        N.check(N.load().sf_production_rates_batch(self.handle, n, N.ptr(T), N.ptr(rho), N.ptr(Y), N.ptr(out),
                                                   N.ptr(ws), nb, N.stream_handle()))
        return out

    def rates_sens_batch(self, rho, T, Y, option=0):
        torch = _torch()
        T, rho, Y = self._dev(T), self._dev(rho), self._dev(Y)
        n, ns = T.numel(), self.n_species
        w = torch.empty((n, ns), dtype=torch.float64, device=T.device)
        S = torch.empty((n, (ns + 1) ** 2), dtype=torch.float64, device=T.device)
        ws, nb = self.workspace(1, n)
        N.check(N.load().sf_rates_sens_batch(self.handle, n, N.ptr(rho), N.ptr(T), N.ptr(Y), int(option), N.ptr(w),
                                             N.ptr(S), N.ptr(ws), nb, N.stream_handle()))
        return w, S

    def reactor_params(self, configuration, **kw):
        return reactor_params(configuration, **kw)

    def reactor_rhs_batch(self, params, q, pressures=None, out=None):
        torch = _torch()
        q = self._dev(q)
        pr = self._dev(pressures) if pressures is not None else None
        out = torch.empty_like(q) if out is None else out
        ws, nb = self.workspace(2, q.shape[0])
        N.check(N.load().sf_reactor_rhs_batch(self.handle, C.byref(params), q.shape[0], N.ptr(q), N.ptr(pr),
                                              N.ptr(out), N.ptr(ws), nb, N.stream_handle()))
        return out

    def reactor_jac_batch(self, params, q, rates_option=0, pressures=None, out_rhs=None, out_jac=None):
        torch = _torch()
        q = self._dev(q)
        n, neq = q.shape
        pr = self._dev(pressures) if pressures is not None else None
        out_rhs = torch.empty_like(q) if out_rhs is None else out_rhs
        out_jac = torch.empty((n, neq * neq), dtype=torch.float64, device=q.device) if out_jac is None else out_jac
        ws, nb = self.workspace(3, n)
        N.check(N.load().sf_reactor_jac_batch(self.handle, C.byref(params), int(rates_option), n, N.ptr(q),
                                              N.ptr(pr), N.ptr(out_rhs), N.ptr(out_jac), N.ptr(ws), nb,
                                              N.stream_handle()))
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
        """Sensitivity transform option 0 ('exact', the only one the reference defines) writes the transformed
        (T, Y) Jacobian; any other value leaves out_jac as it was, as isobaric_reactor_kernels.cpp:305-311 does."""
        P = self._params('isobaric', pressure, Tin, Yin, tau, Tc, Tr, hc, eps, SoV, heat, open_)
        r, J = self.reactor_jac_batch(P, np.asarray(state)[None, :], ropt)
        out_rhs[:] = self._np1(r[0])
        if int(topt) == 0:
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

    # ---------------------------------------------------------------- reference-named flamelet methods
    def flamelet_stencils(self, dz, nzi, dissipationRate, invLewisNumbers, out_cmajor, out_csub, out_csup,
                          out_mcoeff, out_ncoeff):
        """Diffusion stencils of one flamelet (griffon.pyx:556-566, flamelet_kernels.cpp:31-48), host arrays."""
        L = N.load()
        d = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        dz, chi, inv = d(dz), d(dissipationRate), d(invLewisNumbers)
        outs = [out_cmajor, out_csub, out_csup, out_mcoeff, out_ncoeff]
        for o in outs:
            _require_writable_f64(o)
        p = lambda v: v.ctypes.data_as(C.POINTER(C.c_double))
        N.check(L.sf_flamelet_stencils(self.handle, p(dz), int(nzi), p(chi), p(inv), *[p(o) for o in outs]))

    def flamelet_jac_indices(self, nzi, out_row_indices, out_col_indices):
        """COO row/column indices of the BTDDOD Jacobian values (griffon.pyx:571-575)."""
        for o in (out_row_indices, out_col_indices):
            if not (isinstance(o, np.ndarray) and o.dtype == np.int32 and o.flags.c_contiguous):
                raise TypeError('flamelet_jac_indices writes into contiguous int32 numpy arrays')
        ip = lambda v: v.ctypes.data_as(C.POINTER(C.c_int))
        N.check(N.load().sf_flamelet_jac_indices(self.handle, int(nzi), ip(out_row_indices), ip(out_col_indices)))

    def _one_flamelet(self, state, pressure, oxyState, fuelState, adiabatic, T_convection, T_radiation,
                      h_convection, h_radiation, nzi, cmajor, csub, csup, mcoeff, ncoeff, chi, include_enthalpy_flux,
                      include_variable_cp, use_scaled_heat_loss):
        """A one-flamelet sf_flamelet_batch over device copies of the reference-shaped arguments; returns it with
        the tensors it points into (kept alive by the caller) and the device state."""
        from ._desc import SfFlameletBatch
        torch = _torch()
        ns, nzi = self.n_species, int(nzi)
        dev = torch.device('cuda', torch.cuda.current_device())
        f64 = lambda a, n: torch.tensor(np.asarray(a, dtype=np.float64).reshape(-1)[:n], dtype=torch.float64,
                                        device=dev)
        keep = dict(state=f64(state, nzi * ns), oxy=f64(oxyState, ns), fuel=f64(fuelState, ns),
                    cmajor=f64(cmajor, nzi * ns), csub=f64(csub, nzi * ns), csup=f64(csup, nzi * ns),
                    mc=f64(mcoeff, nzi), nc=f64(ncoeff, nzi),
                    # the reference hands over the full-grid dissipation rate and reads it at the interior index
                    # (flamelet_kernels.cpp:1174, :1360), so interior point i uses chi[i]
                    chi=f64(chi, nzi))
        offz = np.array([0, nzi], dtype=np.int32)
        keep['offz_host'] = offz
        keep['offz'] = torch.tensor(offz, dtype=torch.int32, device=dev)
        keep['offv'] = torch.tensor([0, ns * (nzi * ns + 2 * (nzi - 1))], dtype=torch.int64, device=dev)
        fb = SfFlameletBatch()
        fb.n_flamelets = 1
        fb.offsets_z = C.cast(keep['offz'].data_ptr(), C.POINTER(C.c_int))
        fb.offsets_v = C.cast(keep['offv'].data_ptr(), C.POINTER(C.c_longlong))
        fb.offsets_z_host = offz.ctypes.data_as(C.POINTER(C.c_int))
        fb.pressure = float(pressure)
        for name, key in (('oxy_state', 'oxy'), ('fuel_state', 'fuel'), ('cmajor', 'cmajor'), ('csub', 'csub'),
                          ('csup', 'csup'), ('mcoeff', 'mc'), ('ncoeff', 'nc'), ('chi', 'chi')):
            setattr(fb, name, C.cast(keep[key].data_ptr(), C.POINTER(C.c_double)))
        fb.include_enthalpy_flux = int(bool(include_enthalpy_flux))
        fb.include_variable_cp = int(bool(include_variable_cp))
        if not adiabatic:
            # named as the reference forwards them (griffon.pyx:606-609): the Python order is (T_conv, T_rad,
            # h_conv, h_rad), the engine's (T_conv, h_conv, T_rad, h_rad), each array by its own name
            for name, a in (('T_convection', T_convection), ('h_convection', h_convection),
                            ('T_radiation', T_radiation), ('h_radiation', h_radiation)):
                keep[name] = f64(a, nzi)
                setattr(fb, name, C.cast(keep[name].data_ptr(), C.POINTER(C.c_double)))
            fb.use_scaled_heat_loss = int(bool(use_scaled_heat_loss))
        return fb, keep

    def flamelet_rhs(self, state, pressure, oxyState, fuelState, adiabatic, T_convection, T_radiation, h_convection,
                     h_radiation, nzi, cmajor, csub, csup, mcoeff, ncoeff, chi, include_enthalpy_flux,
                     include_variable_cp, use_scaled_heat_loss, out_rhs):
        """Residual of one flamelet (griffon.pyx:580-620, flamelet_kernels.cpp:1039-1218) into out_rhs."""
        torch = _torch()
        fb, keep = self._one_flamelet(state, pressure, oxyState, fuelState, adiabatic, T_convection, T_radiation,
                                      h_convection, h_radiation, nzi, cmajor, csub, csup, mcoeff, ncoeff, chi,
                                      include_enthalpy_flux, include_variable_cp, use_scaled_heat_loss)
        out = torch.empty_like(keep['state'])
        N.check(N.load().sf_flamelet_rhs_batch(self.handle, C.byref(fb), N.ptr(keep['state']), N.ptr(out),
                                               N.stream_handle()))
        out_rhs[:out.numel()] = self._np1(out)

    def flamelet_jacobian(self, state, pressure, oxyState, fuelState, adiabatic, T_convection, T_radiation,
                          h_convection, h_radiation, nzi, cmajor, csub, csup, mcoeff, ncoeff, chi, compute_eigenvalues,
                          diffterm, scale_and_offset, prefactor, rates_sensitivity_option,
                          sensitivity_transform_option, include_enthalpy_flux, include_variable_cp,
                          use_scaled_heat_loss, out_expeig, out_jac):
        """BTDDOD Jacobian values of one flamelet (griffon.pyx:625-679, flamelet_kernels.cpp:1220-1409) into out_jac
        (written, not accumulated: the reference adds the off-diagonal coefficients to the zeroed array its
        callers pass). With compute_eigenvalues, out_expeig receives max(max Re(lambda) - diffterm, 0) of each
        point's chemistry block for every row of the point, taken before the scaling when scale_and_offset is
        also set, as the reference orders them."""
        if int(sensitivity_transform_option) != 0:
            raise ValueError("sensitivity_transform_option must be 0 ('exact', the only transform the reference "
                             "defines)")
        torch = _torch()
        ns, nzi = self.n_species, int(nzi)
        fb, keep = self._one_flamelet(state, pressure, oxyState, fuelState, adiabatic, T_convection, T_radiation,
                                      h_convection, h_radiation, nzi, cmajor, csub, csup, mcoeff, ncoeff, chi,
                                      include_enthalpy_flux, include_variable_cp, use_scaled_heat_loss)
        dev = keep['state'].device
        vals = torch.empty(ns * (nzi * ns + 2 * (nzi - 1)), dtype=torch.float64, device=dev)
        eig = torch.empty(nzi * ns, dtype=torch.float64, device=dev) if compute_eigenvalues else None
        L = N.load()
        fused = bool(scale_and_offset) and not compute_eigenvalues
        wsb = int(L.sf_flamelet_jac_workspace_size(self.handle, int(bool(compute_eigenvalues))))
        ws = torch.empty(max(wsb, 8) // 8, dtype=torch.float64, device=dev)
        N.check(L.sf_flamelet_jac_batch(self.handle, C.byref(fb), N.ptr(keep['state']), int(rates_sensitivity_option),
                                        int(fused), float(prefactor), float(diffterm), N.ptr(eig), N.ptr(vals),
                                        N.ptr(ws), wsb, N.stream_handle()))
        if scale_and_offset and compute_eigenvalues:
            ones = torch.ones(nzi * ns, dtype=torch.float64, device=dev)
            N.check(L.sf_btddod_scale_and_add_diagonal_batch(1, ns, N.ptr(keep['offz']), N.ptr(keep['offv']),
                                                             N.ptr(keep['offz_host']), N.ptr(vals), float(prefactor),
                                                             N.ptr(ones), -1., None, N.stream_handle()))
        out_jac[:vals.numel()] = self._np1(vals)
        if compute_eigenvalues:
            out_expeig[:eig.numel()] = self._np1(eig)


def _require_writable_f64(a):
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous and a.flags.writeable):
        raise TypeError('output arguments are writable contiguous float64 numpy arrays, as the reference requires')


# ------------------------------------------------------------------------------------------------------------------
# Block-tridiagonal, diagonal off-diagonal (BTDDOD) algebra with the reference's module-level names
# (griffon.pyx:1009-1113). Arguments and in-place outputs are numpy arrays, as the reference's callers pass them
# (flamelet.py:758, :913, :1424-1436, :1606-1618), or torch CUDA float64/int32 tensors, which are used in place
# without host copies. Every function runs on the GPU.
#
# Factor representation: py_btddod_full_factorize leaves in out_d_factors the inverses of the eliminated diagonal
# blocks (a twisted block-Thomas elimination from both ends), in out_l_values the multiplier blocks, and in
# out_d_pivots each block's pivot order; py_btddod_blockdiag_factorize writes the blocks' inverses. Only the matching
# solve functions read these, and the pairs reproduce the reference's solutions.
# ------------------------------------------------------------------------------------------------------------------
class _Dev:
    """Device views of the arguments of one call; numpy arrays are copied in, and back out if written."""

    def __init__(self):
        self._back = []

    def f64(self, a, n=None, out=False):
        return self._view(a, n, out, 'float64')

    def i32(self, a, n=None, out=False):
        return self._view(a, n, out, 'int32')

    def _view(self, a, n, out, dt):
        torch = _torch()
        tdt = getattr(torch, dt)
        if isinstance(a, torch.Tensor):
            if not a.is_cuda or a.dtype != tdt or not a.is_contiguous():
                raise TypeError(f'tensor arguments are contiguous CUDA {dt} tensors')
            return a.view(-1)[:n] if n is not None else a.view(-1)
        arr = np.asarray(a)
        if out and not (isinstance(a, np.ndarray) and a.dtype == np.dtype(dt) and a.flags.c_contiguous and
                        a.flags.writeable):
            raise TypeError(f'output arguments are writable contiguous {dt} numpy arrays, as the reference requires')
        flat = np.ascontiguousarray(arr, dtype=dt).reshape(-1)
        flat = flat[:n] if n is not None else flat
        t = torch.tensor(flat, device=torch.device('cuda', torch.cuda.current_device()))
        if out:
            self._back.append((a, t))
        return t

    def finish(self):
        for a, t in self._back:
            a.reshape(-1)[:t.numel()] = t.cpu().numpy()


def _single(num_blocks, block_size):
    """Offsets of one BTDDOD matrix of num_blocks blocks (device tensors and the host copy)."""
    torch = _torch()
    nb, ns = int(num_blocks), int(block_size)
    if nb < 1 or ns < 1:
        raise ValueError('num_blocks and block_size must be positive')
    dev = torch.device('cuda', torch.cuda.current_device())
    offz = np.array([0, nb], dtype=np.int32)
    return (torch.tensor(offz, device=dev), torch.tensor([0, ns * (nb * ns + 2 * (nb - 1))], dtype=torch.int64,
                                                         device=dev), offz, nb, ns)


def _nvals(nb, ns):
    return ns * (nb * ns + 2 * (nb - 1))


def py_btddod_full_matvec(matrix_values, vec, num_blocks, block_size, out_matvec):
    """out = A vec (griffon.pyx:1009-1014, btddod_matrix_kernels.cpp:121-165)."""
    oz, ov, oh, nb, ns = _single(num_blocks, block_size)
    d = _Dev()
    A, x, y = d.f64(matrix_values, _nvals(nb, ns)), d.f64(vec, nb * ns), d.f64(out_matvec, nb * ns, out=True)
    N.check(N.load().sf_btddod_matvec_batch(1, ns, N.ptr(oz), N.ptr(ov), N.ptr(oh), N.ptr(A), N.ptr(x), N.ptr(y),
                                            None, N.stream_handle()))
    d.finish()


def py_btddod_blockdiag_matvec(matrix_values, vec, num_blocks, block_size, out_matvec):
    """out_i = D_i vec_i with the diagonal blocks only (griffon.pyx:1019-1024, btddod_matrix_kernels.cpp:167-177)."""
    nb, ns = int(num_blocks), int(block_size)
    d = _Dev()
    A, x, y = d.f64(matrix_values, nb * ns * ns), d.f64(vec, nb * ns), d.f64(out_matvec, nb * ns, out=True)
    N.check(N.load().sf_btddod_blockdiag_matvec_batch(nb, ns, N.ptr(A), N.ptr(x), N.ptr(y), N.stream_handle()))
    d.finish()


def py_btddod_blockdiag_factorize(matrix_values, num_blocks, block_size, out_pivots, out_factors):
    """Factor every diagonal block (griffon.pyx:1029-1034, btddod_matrix_kernels.cpp:364-373): out_factors
    receives the blocks' inverses, out_pivots their pivot order."""
    nb, ns = int(num_blocks), int(block_size)
    d = _Dev()
    A = d.f64(matrix_values, nb * ns * ns)
    F, P = d.f64(out_factors, nb * ns * ns, out=True), d.i32(out_pivots, nb * ns, out=True)
    N.check(N.load().sf_btddod_blockdiag_factor_batch(nb, ns, N.ptr(A), N.ptr(F), N.ptr(P), N.stream_handle()))
    d.finish()


def py_btddod_blockdiag_solve(pivots, factors, rhs, num_blocks, block_size, out_solution):
    """x_i = D_i^-1 b_i with the factors of py_btddod_blockdiag_factorize (griffon.pyx:1039-1045,
    btddod_matrix_kernels.cpp:375-384)."""
    nb, ns = int(num_blocks), int(block_size)
    d = _Dev()
    F, b, x = d.f64(factors, nb * ns * ns), d.f64(rhs, nb * ns), d.f64(out_solution, nb * ns, out=True)
    N.check(N.load().sf_btddod_blockdiag_matvec_batch(nb, ns, N.ptr(F), N.ptr(b), N.ptr(x), N.stream_handle()))
    d.finish()


def _triangle(pivots, factors, matrix_values, rhs, num_blocks, block_size, out_solution, upper):
    oz, ov, oh, nb, ns = _single(num_blocks, block_size)
    d = _Dev()
    F, A = d.f64(factors, nb * ns * ns), d.f64(matrix_values, _nvals(nb, ns))
    b, x = d.f64(rhs, nb * ns), d.f64(out_solution, nb * ns, out=True)
    N.check(N.load().sf_btddod_triangle_solve_batch(1, ns, N.ptr(oz), N.ptr(ov), N.ptr(oh), N.ptr(F), N.ptr(A),
                                                    N.ptr(b), N.ptr(x), int(upper), None, N.stream_handle()))
    d.finish()


def py_btddod_lowerfulltriangle_solve(pivots, factors, matrix_values, rhs, num_blocks, block_size, out_solution):
    """Block lower-triangular solve with the block-diagonal factors (griffon.pyx:1050-1057,
    btddod_matrix_kernels.cpp:386-404)."""
    _triangle(pivots, factors, matrix_values, rhs, num_blocks, block_size, out_solution, 0)


def py_btddod_upperfulltriangle_solve(pivots, factors, matrix_values, rhs, num_blocks, block_size, out_solution):
    """Block upper-triangular solve with the block-diagonal factors (griffon.pyx:1062-1069,
    btddod_matrix_kernels.cpp:406-428)."""
    _triangle(pivots, factors, matrix_values, rhs, num_blocks, block_size, out_solution, 1)


def py_btddod_full_factorize(out_d_factors, num_blocks, block_size, out_l_values, out_d_pivots):
    """Block-Thomas factorization in place (griffon.pyx:1074-1079, btddod_matrix_kernels.cpp:19-80); the factors
    are read only by py_btddod_full_solve."""
    oz, ov, oh, nb, ns = _single(num_blocks, block_size)
    d = _Dev()
    A = d.f64(out_d_factors, _nvals(nb, ns), out=True)
    Lv, P = d.f64(out_l_values, nb * ns * ns, out=True), d.i32(out_d_pivots, nb * ns, out=True)
    N.check(N.load().sf_btddod_factor_batch(1, ns, N.ptr(oz), N.ptr(ov), N.ptr(oh), N.ptr(A), N.ptr(Lv), N.ptr(P),
                                            None, N.stream_handle()))
    d.finish()


def py_btddod_full_solve(d_factors, l_values, d_pivots, rhs, num_blocks, block_size, out_solution):
    """Solve with the factors of py_btddod_full_factorize (griffon.pyx:1084-1091, btddod_matrix_kernels.cpp:82-119)."""
    oz, ov, oh, nb, ns = _single(num_blocks, block_size)
    d = _Dev()
    A, Lv, P = d.f64(d_factors, _nvals(nb, ns)), d.f64(l_values, nb * ns * ns), d.i32(d_pivots, nb * ns)
    b, x = d.f64(rhs, nb * ns), d.f64(out_solution, nb * ns, out=True)
    N.check(N.load().sf_btddod_solve_batch(1, ns, N.ptr(oz), N.ptr(ov), N.ptr(oh), N.ptr(A), N.ptr(Lv), N.ptr(P),
                                           N.ptr(b), N.ptr(x), None, N.stream_handle()))
    d.finish()


def py_btddod_scale_and_add_scaled_block_diagonal(in_out_matrix_values, matrix_scale, block_diag, diag_scale,
                                                  num_blocks, block_size):
    """A <- matrix_scale A + diag_scale B on the diagonal blocks (griffon.pyx:1096-1102,
    btddod_matrix_kernels.cpp:430-446)."""
    oz, ov, oh, nb, ns = _single(num_blocks, block_size)
    d = _Dev()
    A, B = d.f64(in_out_matrix_values, _nvals(nb, ns), out=True), d.f64(block_diag, nb * ns * ns)
    N.check(N.load().sf_btddod_scale_and_add_block_diagonal_batch(1, ns, N.ptr(oz), N.ptr(ov), N.ptr(oh), N.ptr(A),
                                                                  float(matrix_scale), N.ptr(B), float(diag_scale),
                                                                  None, N.stream_handle()))
    d.finish()


def py_btddod_scale_and_add_diagonal(in_out_matrix_values, matrix_scale, diagonal, diag_scale, num_blocks,
                                     block_size):
    """A <- matrix_scale A + diag_scale diag(d) (griffon.pyx:1107-1113, btddod_matrix_kernels.cpp:448-465)."""
    oz, ov, oh, nb, ns = _single(num_blocks, block_size)
    d = _Dev()
    A, v = d.f64(in_out_matrix_values, _nvals(nb, ns), out=True), d.f64(diagonal, nb * ns)
    N.check(N.load().sf_btddod_scale_and_add_diagonal_batch(1, ns, N.ptr(oz), N.ptr(ov), N.ptr(oh), N.ptr(A),
                                                            float(matrix_scale), N.ptr(v), float(diag_scale), None,
                                                            N.stream_handle()))
    d.finish()
