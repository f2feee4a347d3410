"""Steady flamelets on the GPU: Spitfire's ``FlameletSpec``/``Flamelet``, adiabatic or with heat loss, batched.

``FlameletBatch`` holds any number of flamelets of one mechanism, each with its own mixture-fraction grid,
dissipation-rate profile and heat-loss parameters, and evaluates all of them with one launch per operation: the flamelet residual
(``sf_flamelet_rhs_batch``), the block-tridiagonal Jacobian (``sf_flamelet_jac_batch``), the block-Thomas
factorization and solve (``sf_btddod_*``). The steady solvers restate the reference's control flow per flamelet
(spitfire/chemistry/flamelet.py): ``steady_solve_newton`` (:1352-1485; chord Newton on -J with a refresh after
line-search cuts, max 38 iterations in compute_steady_state), ``steady_solve_psitc`` (:1487-1703; pseudo-transient
continuation with ds = min(0.1/(lambda+ + 1e-16), 1.1 ds, 1e4), a global ds on the first iteration, Jacobian
refresh every 8 iterations or while the residual exceeds 1e-2, restart with ds_init/4 on failure) and
``compute_steady_state`` (:1705-1778, Newton then psitc). All flamelets advance together; each has its own
iteration counters, Jacobian-refresh flags, line-search state and convergence status.
"""

import ctypes as C

import numpy as np
from scipy.special import erfinv

from . import _native as N
from ._desc import SfFlameletBatch


def _torch():
    import torch
    return torch


def clustered_grid(grid_points, grid_cluster_point, grid_cluster_intensity=6.):
    """Anderson's stretched grid clustered around grid_cluster_point (flamelet.py:300-341)."""
    if grid_cluster_intensity < 1.e-16:
        raise ValueError('cluster_coeff must be strictly positive')
    if grid_cluster_point < 0. or grid_cluster_point > 1.:
        raise ValueError('z_cluster must be between 0 and 1')
    z = np.linspace(0., 1., grid_points)
    a_ = grid_cluster_intensity
    zo = 1.0 / (2.0 * a_) * np.log((1. + (np.exp(a_) - 1.) * grid_cluster_point) /
                                  (1. + (np.exp(-a_) - 1.) * grid_cluster_point))
    a = np.sinh(a_ * zo)
    for i in range(grid_points):
        z[i] = grid_cluster_point / a * (np.sinh(a_ * (z[i] - zo)) + a)
    z[-1] = 1.
    return z, z[1:] - z[:-1]


def uniform_grid(grid_points):
    z = np.linspace(0., 1., grid_points)
    return z, z[1:] - z[:-1]


def compute_dissipation_rate(mixture_fraction, max_dissipation_rate, form='Peters'):
    """Peters' form chi = chi_max exp(-2 erfinv(2Z-1)^2), else constant (flamelet.py:240-266)."""
    if form in ('Peters', 'peters'):
        return max_dissipation_rate * np.exp(-2. * (erfinv(2. * mixture_fraction - 1.)) ** 2)
    return np.full_like(mixture_fraction, max_dissipation_rate)


class FlameletSpec:
    """The specification arguments of spitfire's FlameletSpec (flamelet.py:35-237): grid, dissipation rate,
    streams, initial condition and, for heat_transfer='nonadiabatic', the convection / radiation parameters
    (numbers or arrays over the interior points) and the heat-loss scaling options."""

    def __init__(self, mech_spec=None, initial_condition=None, oxy_stream=None, fuel_stream=None, grid=None,
                 grid_points=None, grid_type='clustered', grid_cluster_intensity=4.,
                 grid_cluster_point='stoichiometric', max_dissipation_rate=None, stoich_dissipation_rate=None,
                 dissipation_rate=None, dissipation_rate_form='Peters', heat_transfer='adiabatic',
                 convection_temperature=None, radiation_temperature=None, convection_coefficient=None,
                 radiative_emissivity=None, scale_heat_loss_by_temp_range=False,
                 scale_convection_by_dissipation=False, use_linear_ref_temp_profile=False,
                 rates_sensitivity_type='dense', sensitivity_transform_type='exact', include_enthalpy_flux=True,
                 include_variable_cp=True, **ignored):
        if heat_transfer not in ('adiabatic', 'nonadiabatic'):
            raise ValueError(f'bad heat_transfer {heat_transfer!r}; use adiabatic or nonadiabatic')
        self.convection_temperature = convection_temperature
        self.radiation_temperature = radiation_temperature
        self.convection_coefficient = convection_coefficient
        self.radiative_emissivity = radiative_emissivity
        self.scale_heat_loss_by_temp_range = scale_heat_loss_by_temp_range
        self.scale_convection_by_dissipation = scale_convection_by_dissipation
        self.use_linear_ref_temp_profile = use_linear_ref_temp_profile
        self.mech_spec = mech_spec
        self.initial_condition = initial_condition
        self.oxy_stream = oxy_stream
        self.fuel_stream = fuel_stream
        self.grid = grid
        self.grid_points = grid_points
        self.grid_type = grid_type
        self.grid_cluster_intensity = grid_cluster_intensity
        self.grid_cluster_point = grid_cluster_point
        self.max_dissipation_rate = max_dissipation_rate
        self.stoich_dissipation_rate = stoich_dissipation_rate
        self.dissipation_rate = dissipation_rate
        self.dissipation_rate_form = dissipation_rate_form
        self.heat_transfer = heat_transfer
        self.rates_sensitivity_type = rates_sensitivity_type
        self.sensitivity_transform_type = sensitivity_transform_type
        self.include_enthalpy_flux = include_enthalpy_flux
        self.include_variable_cp = include_variable_cp


class FlameletSetup:
    """Grid, dissipation rate, boundary states and initial state of one flamelet (flamelet.py:366-637)."""

    def __init__(self, fs: FlameletSpec):
        m = fs.mech_spec
        self.mech = m
        self.pressure = float(fs.oxy_stream.P)
        if abs(fs.fuel_stream.P - fs.oxy_stream.P) / fs.oxy_stream.P > 1.e-6:
            raise ValueError('fuel and oxidizer streams must have the same pressure')
        self.state_fuel = np.hstack([fs.fuel_stream.T, fs.fuel_stream.Y[:-1]])
        self.state_oxy = np.hstack([fs.oxy_stream.T, fs.oxy_stream.Y[:-1]])
        self.z_st = m.stoich_mixture_fraction(fs.fuel_stream, fs.oxy_stream)
        if fs.grid is not None:
            self.z = np.array(fs.grid, dtype=np.float64)
            self.dz = self.z[1:] - self.z[:-1]
        elif fs.grid_type == 'uniform':
            self.z, self.dz = uniform_grid(fs.grid_points)
        else:
            cp = self.z_st if fs.grid_cluster_point == 'stoichiometric' else fs.grid_cluster_point
            self.z, self.dz = clustered_grid(fs.grid_points, cp, fs.grid_cluster_intensity)
        self.nzi = self.z.size - 2
        ns = m.n_species
        if fs.dissipation_rate is not None:
            self.x = np.array(fs.dissipation_rate, dtype=np.float64)
            self.max_dissipation_rate = float(np.max(self.x))
            self.form = 'custom'
        elif fs.max_dissipation_rate is not None:
            self.max_dissipation_rate = fs.max_dissipation_rate
            self.form = fs.dissipation_rate_form
            self.x = compute_dissipation_rate(self.z, self.max_dissipation_rate, self.form)
        elif fs.stoich_dissipation_rate is not None:
            if fs.dissipation_rate_form in ('peters', 'Peters'):
                self.max_dissipation_rate = fs.stoich_dissipation_rate / np.exp(-2. * erfinv(2. * self.z_st - 1.) ** 2)
            else:
                self.max_dissipation_rate = fs.stoich_dissipation_rate
            self.form = fs.dissipation_rate_form
            self.x = compute_dissipation_rate(self.z, self.max_dissipation_rate, self.form)
        else:
            self.x = np.zeros_like(self.z)
            self.max_dissipation_rate = 0.
            self.form = 'unspecified-set-to-0'
        self.include_enthalpy_flux = fs.include_enthalpy_flux
        self.include_variable_cp = fs.include_variable_cp
        self.rates_option = {'dense': 0, 'no-TBAF': 1, 'sparse': 2}[fs.rates_sensitivity_type]
        # heat loss (flamelet.py:479-519): per interior point convection / radiation temperature and coefficient
        self.heat_transfer = fs.heat_transfer
        self.scale_heat_loss_by_temp_range = bool(fs.scale_heat_loss_by_temp_range)
        self.T_conv = self.T_rad = self.h_conv = self.h_rad = None
        if self.heat_transfer == 'nonadiabatic':
            def per_point(v, name):
                if v is None:
                    raise ValueError(f'Flamelet specifications: Nonadiabatic heat transfer was selected but no {name} '
                                     f'argument was given.')
                a = np.asarray(v, dtype=np.float64)
                if a.ndim == 0:
                    return float(a) + np.zeros(self.nzi)
                if a.shape != (self.nzi,):
                    raise ValueError(f'{name} needs one value per interior grid point ({self.nzi})')
                return a.copy()
            self.h_conv = per_point(fs.convection_coefficient, 'convection_coefficient')
            self.h_rad = per_point(fs.radiative_emissivity, 'radiative_emissivity')
            if fs.use_linear_ref_temp_profile:
                self.T_conv = fs.oxy_stream.T + self.z[1:-1] * (fs.fuel_stream.T - fs.oxy_stream.T)
                self.T_rad = self.T_conv.copy()
            else:
                self.T_rad = per_point(fs.radiation_temperature, 'radiation_temperature')
                self.T_conv = per_point(fs.convection_temperature, 'convection_temperature')
            if fs.scale_convection_by_dissipation:
                factor = np.max(self.x) / (1. - self.z_st) / self.z_st
                self.h_conv = self.h_conv * factor
                self.h_rad = self.h_rad * factor
        ic = fs.initial_condition
        if isinstance(ic, np.ndarray):
            if ic.size != self.nzi * ns:
                raise ValueError('size of initial condition is incorrect!')
            self.initial_state = ic.astype(np.float64).copy()
        elif ic == 'linear-TY':
            zz = self.z[1:-1]
            st = np.empty((self.nzi, ns))
            for i in range(ns):
                st[:, i] = self.state_oxy[i] + (self.state_fuel[i] - self.state_oxy[i]) * zz
            self.initial_state = st.ravel()
        elif ic == 'unreacted':
            st = np.empty((self.nzi, ns))
            for i in range(self.nzi):
                zi = self.z[1 + i]
                mix = m.mix_streams([(m.copy_stream(fs.oxy_stream), 1 - zi), (m.copy_stream(fs.fuel_stream), zi)],
                                    basis='mass', constant='HP')
                st[i] = np.hstack([mix.T, mix.Y[:-1]])
            self.initial_state = st.ravel()
        elif ic == 'Burke-Schumann':
            self.initial_state = burke_schumann_state(m, fs.oxy_stream, fs.fuel_stream, self.z, self.pressure)
        else:
            raise ValueError(f'initial_condition {ic!r} is not available on the GPU path (Cantera equilibrium is '
                             f'not available); use linear-TY, unreacted, Burke-Schumann or an array')

    @property
    def linear_temperature(self):
        return self.state_oxy[0] + self.z[1:-1] * (self.state_fuel[0] - self.state_oxy[0])


def burke_schumann_state(m, oxy, fuel, z, pressure):
    """Burke-Schumann (infinitely fast, complete combustion) interior state (flamelet.py:554-586), with HP mixing on
    the project's own NASA7 thermodynamics: the stoichiometric products N2, H2O (and CO2) at the stoichiometric
    mixture's atoms, mass fractions piecewise linear in Z through them, temperature from the mixed enthalpy."""
    zst = m.stoich_mixture_fraction(fuel, oxy)
    stmix = m.mix_streams([(m.copy_stream(oxy), 1 - zst), (m.copy_stream(fuel), zst)], 'mass', 'HP')
    atoms = m._get_atoms_in_stream(stmix, ['H', 'C', 'O', 'N'])
    X = np.zeros(m.n_species)
    X[m.species_index('N2')] = atoms['N'] / 2
    X[m.species_index('H2O')] = 0.5 * atoms['H']
    if 'CO2' in m.species_names:
        X[m.species_index('CO2')] = atoms['C']
    Yst = X * m.molecular_weights
    Yst /= Yst.sum()
    Yo, Yf = oxy.Y, fuel.Y
    zi = z[1:-1]
    # adiabatic mass-basis mixing: the mixture enthalpy is linear in Z between the stream enthalpies
    h = (1. - zi) * oxy.enthalpy_mass + zi * fuel.enthalpy_mass
    lean = (zi <= zst)[:, None]
    Y = np.where(lean, Yo[None, :] + (zi / zst)[:, None] * (Yst - Yo)[None, :],
                 Yst[None, :] + ((zi - zst) / (1. - zst))[:, None] * (Yf - Yst)[None, :])
    T = m.temperature_from_enthalpy_vec(h, Y, 1500.)
    out = np.hstack([T[:, None], Y[:, :-1]])
    return out.ravel()


class FlameletBatch:
    """GPU evaluation of a batch of flamelets (one mechanism, common pressure), adiabatic or with heat loss."""

    def __init__(self, setups):
        torch = _torch()
        self.setups = list(setups)
        m = self.setups[0].mech
        self.mech = m
        self.g = m.griffon
        ns = m.n_species
        self.ns = ns
        self.pressure = self.setups[0].pressure
        for s in self.setups:
            if abs(s.pressure - self.pressure) > 1e-9 * self.pressure:
                raise ValueError('all flamelets of a batch share one pressure')
            if s.include_enthalpy_flux != self.setups[0].include_enthalpy_flux or \
                    s.include_variable_cp != self.setups[0].include_variable_cp:
                raise ValueError('all flamelets of a batch share the enthalpy-flux / variable-cp options')
        nz = [s.nzi for s in self.setups]
        self.nf = len(nz)
        offz = np.zeros(self.nf + 1, dtype=np.int32)
        offz[1:] = np.cumsum(nz)
        offv = np.zeros(self.nf + 1, dtype=np.int64)
        offv[1:] = np.cumsum([ns * (n * ns + 2 * (n - 1)) for n in nz])
        self.offz_host = offz
        self.offv_host = offv
        self.npts = int(offz[-1])
        L = N.load()
        h = self.g.handle
        cma, csb, csp, mc, nc, chi = [], [], [], [], [], []
        invle = np.ones(ns)
        for s in self.setups:
            a = np.zeros(s.nzi * ns)
            b = np.zeros(s.nzi * ns)
            c = np.zeros(s.nzi * ns)
            mm = np.zeros(s.nzi)
            nn = np.zeros(s.nzi)
            p = lambda v: v.ctypes.data_as(C.POINTER(C.c_double))
            N.check(L.sf_flamelet_stencils(h, p(np.ascontiguousarray(s.dz)), s.nzi, p(np.ascontiguousarray(s.x)),
                                           p(invle), p(a), p(b), p(c), p(mm), p(nn)))
            cma.append(a)
            csb.append(b)
            csp.append(c)
            mc.append(mm)
            nc.append(nn)
            # the reference passes the full-grid dissipation rate to flamelet_rhs/flamelet_jacobian and indexes it
            # with the interior index (flamelet.py:654, flamelet_kernels.cpp:1174,1360), so interior point i reads
            # the value at grid index i
            chi.append(s.x[:-2])
        dev = torch.device('cuda', torch.cuda.current_device())
        T = lambda v, dt=torch.float64: torch.tensor(np.concatenate(v) if isinstance(v, list) else v, dtype=dt,
                                                     device=dev)
        self.t_offz = T(offz, torch.int32)
        self.t_offv = T(offv, torch.int64)
        self.t_cmajor, self.t_csub, self.t_csup = T(cma), T(csb), T(csp)
        self.t_mc, self.t_nc, self.t_chi = T(mc), T(nc), T(chi)
        self.t_oxy = T(np.stack([s.state_oxy for s in self.setups]).ravel())
        self.t_fuel = T(np.stack([s.state_fuel for s in self.setups]).ravel())
        fb = SfFlameletBatch()
        fb.n_flamelets = self.nf
        fb.offsets_z = C.cast(self.t_offz.data_ptr(), C.POINTER(C.c_int))
        fb.offsets_v = C.cast(self.t_offv.data_ptr(), C.POINTER(C.c_longlong))
        fb.offsets_z_host = self.offz_host.ctypes.data_as(C.POINTER(C.c_int))
        fb.pressure = self.pressure
        for name, t in (('oxy_state', self.t_oxy), ('fuel_state', self.t_fuel), ('cmajor', self.t_cmajor),
                        ('csub', self.t_csub), ('csup', self.t_csup), ('mcoeff', self.t_mc), ('ncoeff', self.t_nc),
                        ('chi', self.t_chi)):
            setattr(fb, name, C.cast(t.data_ptr(), C.POINTER(C.c_double)))
        fb.include_enthalpy_flux = int(self.setups[0].include_enthalpy_flux)
        fb.include_variable_cp = int(self.setups[0].include_variable_cp)
        # heat loss: per-point arrays when any flamelet is nonadiabatic (adiabatic members get zero coefficients,
        # which add exact zeros)
        nonad = [s for s in self.setups if s.heat_transfer == 'nonadiabatic']
        self.t_heat = None
        if nonad:
            scaled = {s.scale_heat_loss_by_temp_range for s in nonad}
            if len(scaled) > 1:
                raise ValueError('the nonadiabatic flamelets of a batch share scale_heat_loss_by_temp_range')
            arrs = {k: [] for k in ('T_convection', 'h_convection', 'T_radiation', 'h_radiation')}
            for s in self.setups:
                if s.heat_transfer == 'nonadiabatic':
                    vals = (s.T_conv, s.h_conv, s.T_rad, s.h_rad)
                else:
                    vals = (np.zeros(s.nzi), np.zeros(s.nzi), np.zeros(s.nzi), np.zeros(s.nzi))
                for k, v in zip(arrs, vals):
                    arrs[k].append(v)
            self.t_heat = {k: T(v) for k, v in arrs.items()}
            for k, t in self.t_heat.items():
                setattr(fb, k, C.cast(t.data_ptr(), C.POINTER(C.c_double)))
            fb.use_scaled_heat_loss = int(scaled.pop())
        self.fb = fb
        self.nvals = int(offv[-1])
        self.values = torch.empty(self.nvals, dtype=torch.float64, device=dev)
        self.lvalues = torch.empty(self.npts * ns * ns, dtype=torch.float64, device=dev)
        self.pivots = torch.empty(self.npts * ns, dtype=torch.int32, device=dev)
        self.point_flamelet = torch.repeat_interleave(torch.arange(self.nf, device=dev),
                                                      torch.tensor(nz, device=dev))
        self.dof_flamelet = self.point_flamelet.repeat_interleave(ns)
        scales = torch.ones(self.npts * ns, dtype=torch.float64, device=dev)
        scales[::ns] = 1.e3
        self.inv_scales = 1. / scales
        self.rates_option = self.setups[0].rates_option
        self.diffterm = 4. * np.array([s.max_dissipation_rate for s in self.setups])
        self.zeros_dof = torch.zeros(self.npts * ns, dtype=torch.float64, device=dev)
        # the Jacobian call's workspace (the eigenvalue kernel's work counter); a batch runs on one stream
        self.jac_ws = torch.zeros(max(int(L.sf_flamelet_jac_workspace_size(h, 1)), 8) // 8, dtype=torch.float64,
                                  device=dev)

    # ------------------------------------------------------------------------------------------ operations
    # Every operation takes `active`: None (all flamelets) or a bool tensor [nf]; flamelets outside it are left
    # untouched (their values, factors and outputs keep what they held).
    def _mask(self, active):
        if active is None:
            return None
        self._mask_keep = active.to(dtype=_torch().int32).contiguous()
        return self._mask_keep

    def initial_state(self):
        torch = _torch()
        return torch.tensor(np.concatenate([s.initial_state for s in self.setups]), dtype=torch.float64,
                            device=self.values.device)

    def rhs(self, state, out=None, active=None):
        torch = _torch()
        out = torch.empty_like(state) if out is None else out
        m = self._mask(active)
        self.fb.active = C.cast(m.data_ptr(), C.POINTER(C.c_int)) if m is not None else None
        try:
            N.check(N.load().sf_flamelet_rhs_batch(self.g.handle, C.byref(self.fb), N.ptr(state), N.ptr(out),
                                                   N.stream_handle()))
        finally:
            self.fb.active = None
        return out

    def jacobian(self, state, scale_and_offset=False, prefactor=0., eig=False, diffterm=0., diffterm_per_flamelet=None,
                 active=None):
        """BTDDOD Jacobian values into self.values; with eig also the eigenvalue bound per row, using
        diffterm_per_flamelet (CUDA FP64 [nf]) when given, else the scalar diffterm. prefactor: a number, or a CUDA
        FP64 tensor [nf] with each flamelet's own prefactor of the scale_and_offset form."""
        torch = _torch()
        expeig = torch.empty(self.npts * self.ns, dtype=torch.float64, device=state.device) if eig else None
        m = self._mask(active)
        self.fb.active = C.cast(m.data_ptr(), C.POINTER(C.c_int)) if m is not None else None
        self.fb.diffterm = C.cast(diffterm_per_flamelet.data_ptr(), C.POINTER(C.c_double)) \
            if diffterm_per_flamelet is not None else None
        per = torch.is_tensor(prefactor)
        if per:
            self._pref_keep = prefactor.to(dtype=torch.float64).contiguous()
            self.fb.prefactor = C.cast(self._pref_keep.data_ptr(), C.POINTER(C.c_double))
            prefactor = 0.
        try:
            N.check(N.load().sf_flamelet_jac_batch(self.g.handle, C.byref(self.fb), N.ptr(state), self.rates_option,
                                                   int(scale_and_offset), float(prefactor), float(diffterm),
                                                   N.ptr(expeig), N.ptr(self.values), N.ptr(self.jac_ws),
                                                   self.jac_ws.numel() * 8, N.stream_handle()))
        finally:
            self.fb.active = None
            self.fb.diffterm = None
            self.fb.prefactor = None
        return (self.values, expeig) if eig else self.values

    def diffterm_tensor(self, diffusion_factor=4.):
        """Per-flamelet diffusion term diffusion_factor * max(chi) of steady_solve_psitc (flamelet.py:1587)."""
        torch = _torch()
        return torch.tensor(diffusion_factor / 4. * self.diffterm, dtype=torch.float64, device=self.values.device)

    def expeig_per_flamelet_diffterm(self, state):
        """Eigenvalue bounds with each flamelet's own diffterm = 4 max(chi)."""
        return self.jacobian(state, eig=True, diffterm_per_flamelet=self.diffterm_tensor())[1]

    def factor(self, active=None):
        N.check(N.load().sf_btddod_factor_batch(self.nf, self.ns, N.ptr(self.t_offz), N.ptr(self.t_offv),
                                                N.ptr(self.offz_host), N.ptr(self.values), N.ptr(self.lvalues),
                                                N.ptr(self.pivots), N.ptr(self._mask(active)), N.stream_handle()))

    def solve(self, rhs, out=None, active=None):
        torch = _torch()
        out = torch.empty_like(rhs) if out is None else out
        N.check(N.load().sf_btddod_solve_batch(self.nf, self.ns, N.ptr(self.t_offz), N.ptr(self.t_offv),
                                               N.ptr(self.offz_host), N.ptr(self.values), N.ptr(self.lvalues),
                                               N.ptr(self.pivots), N.ptr(rhs), N.ptr(out), N.ptr(self._mask(active)),
                                               N.stream_handle()))
        return out

    def matvec(self, x, out=None, active=None):
        torch = _torch()
        out = torch.empty_like(x) if out is None else out
        N.check(N.load().sf_btddod_matvec_batch(self.nf, self.ns, N.ptr(self.t_offz), N.ptr(self.t_offv),
                                                N.ptr(self.offz_host), N.ptr(self.values), N.ptr(x), N.ptr(out),
                                                N.ptr(self._mask(active)), N.stream_handle()))
        return out

    def scale_and_add_diagonal(self, matrix_scale, diagonal, diag_scale, active=None):
        N.check(N.load().sf_btddod_scale_and_add_diagonal_batch(self.nf, self.ns, N.ptr(self.t_offz),
                                                                N.ptr(self.t_offv), N.ptr(self.offz_host),
                                                                N.ptr(self.values), float(matrix_scale),
                                                                N.ptr(diagonal), float(diag_scale),
                                                                N.ptr(self._mask(active)), N.stream_handle()))

    def norms(self, v):
        """Weighted inf-norm per flamelet (scales 1e3 on T)."""
        torch = _torch()
        out = torch.zeros(self.nf, dtype=torch.float64, device=v.device)
        return out.scatter_reduce(0, self.dof_flamelet, (v * self.inv_scales).abs(), reduce='amax',
                                  include_self=True)

    def mins(self, v):
        torch = _torch()
        out = torch.full((self.nf,), float('inf'), dtype=torch.float64, device=v.device)
        return out.scatter_reduce(0, self.dof_flamelet, v, reduce='amin', include_self=True)

    def finite(self, v):
        torch = _torch()
        bad = torch.zeros(self.nf, dtype=torch.float64, device=v.device)
        bad = bad.scatter_reduce(0, self.dof_flamelet, (~torch.isfinite(v)).double(), reduce='amax',
                                 include_self=True)
        return bad == 0

    def expand(self, per_flamelet):
        return per_flamelet[self.dof_flamelet]

    # ------------------------------------------------------------------------------------------ solvers
    def _steady_ws(self):
        torch = _torch()
        if getattr(self, '_steady_wsb', None) is None:
            nb = int(N.load().sf_flamelet_steady_workspace_size(self.g.handle, C.byref(self.fb)))
            self._steady_wsb = torch.empty((nb + 7) // 8, dtype=torch.float64, device=self.values.device)
        return self._steady_wsb

    def _steady_common(self, state, active):
        torch = _torch()
        dev = state.device
        state = state.clone().contiguous()
        m = None if active is None else active.to(dtype=torch.int32).contiguous()
        conv = torch.empty(self.nf, dtype=torch.int32, device=dev)
        it = torch.empty(self.nf, dtype=torch.int32, device=dev)
        return state, m, conv, it, self._steady_ws()

    def steady_solve_newton(self, state, active=None, tolerance=1.e-6, max_iterations=10,
                            max_factor_line_search=1.5, max_allowed_residual=1.e6, min_allowable_state_var=-1.e-6):
        """Flamelet.steady_solve_newton (flamelet.py:1352-1485) for every flamelet of the batch at once, on the
        native batched solver (sf_flamelet_steady_newton_batch). Returns (state, converged[nf] bool,
        iterations[nf])."""
        state, m, conv, it, ws = self._steady_common(state, active)
        N.check(N.load().sf_flamelet_steady_newton_batch(
            self.g.handle, C.byref(self.fb), N.ptr(state), N.ptr(m), float(tolerance), int(max_iterations),
            float(max_factor_line_search), float(max_allowed_residual), float(min_allowable_state_var),
            int(self.rates_option), N.ptr(conv), N.ptr(it), N.ptr(ws), ws.numel() * 8, N.stream_handle()))
        return state, conv.bool(), it.long()

    def steady_solve_psitc(self, initial, active=None, tolerance=1.e-6, max_iterations=400,
                           min_allowable_state_var=-1.e-6, ds_init=1., ds_init_decrease=4., diffusion_factor=4.,
                           global_ds=False, ds_safety=0.1, ds_ramp=1.1, ds_max=1.e4, max_factor_line_search=1.5,
                           max_allowed_residual=1.e6, max_recursion_depth=20, adaptive_restart=True):
        """Flamelet.steady_solve_psitc (flamelet.py:1487-1703) for every flamelet of the batch at once, with its
        restart from the initial guess after a failure, on the native batched solver
        (sf_flamelet_steady_psitc_batch). Returns (state, converged[nf] bool, iterations[nf]) and leaves each
        flamelet's smallest pseudo-time step where it stopped in last_psitc_min_ds."""
        torch = _torch()
        state, m, conv, it, ws = self._steady_common(initial, active)
        dterm = self.diffterm_tensor(diffusion_factor)
        mds = torch.empty(self.nf, dtype=torch.float64, device=state.device)
        N.check(N.load().sf_flamelet_steady_psitc_batch(
            self.g.handle, C.byref(self.fb), N.ptr(state), N.ptr(m), N.ptr(dterm), float(tolerance),
            int(max_iterations), float(min_allowable_state_var), float(ds_init), float(ds_init_decrease),
            int(bool(global_ds)), float(ds_safety), float(ds_ramp), float(ds_max), float(max_factor_line_search),
            float(max_allowed_residual), int(max_recursion_depth), int(bool(adaptive_restart)),
            int(self.rates_option), N.ptr(conv), N.ptr(it), N.ptr(mds), N.ptr(ws), ws.numel() * 8,
            N.stream_handle()))
        self.last_psitc_min_ds = mds
        return state, conv.bool(), it.long()

    def steady_solve_newton_host(self, state, active=None, tolerance=1.e-6, max_iterations=10,
                                 max_factor_line_search=1.5, max_allowed_residual=1.e6, min_allowable_state_var=-1.e-6):
        """The same solver as steady_solve_newton with its control loop on the host, over the batch's own
        operations (rhs, jacobian, factor, solve, norms): the native solver's arithmetic step by step, kept to check
        it against. Returns (state, converged[nf] bool, iterations[nf])."""
        torch = _torch()
        dev = state.device
        nf = self.nf
        state = state.clone()
        run = torch.ones(nf, dtype=torch.bool, device=dev) if active is None else active.clone()
        failed = torch.zeros(nf, dtype=torch.bool, device=dev)
        it = torch.zeros(nf, dtype=torch.int64, device=dev)
        res = torch.full((nf,), tolerance + 1., dtype=torch.float64, device=dev)
        rhs = self.rhs(state, active=run)
        eval_j = torch.ones(nf, dtype=torch.bool, device=dev)
        dstate = torch.zeros_like(state)
        for _ in range(max_iterations + 1):
            go = run & ~failed & (res > tolerance) & (it < max_iterations)
            if not bool(go.any()):
                break
            it = it + go.long()
            need = go & eval_j
            if bool(need.any()):
                self.jacobian(state, active=need)
                self.scale_and_add_diagonal(-1., self.zeros_dof, 0., active=need)  # J <- -J
                self.factor(active=need)
                eval_j = eval_j & ~need
            self.solve(rhs, out=dstate, active=go)
            ok = self.finite(dstate)
            failed = failed | (go & ~ok)
            go = go & ok
            dstate = torch.where(self.expand(go), dstate, torch.zeros_like(dstate))
            norm_old = self.norms(rhs)
            rhs_new = self.rhs(state + dstate, active=go)
            ok = self.finite(rhs_new)
            failed = failed | (go & ~ok)
            go = go & ok
            alpha = torch.ones(nf, dtype=torch.float64, device=dev)
            for _ls in range(12):
                n_new = self.norms(rhs_new)
                cut = go & (n_new > max_factor_line_search * norm_old) & (alpha > 0.001)
                if not bool(cut.any()):
                    break
                alpha = torch.where(cut, alpha * 0.5, alpha)
                dstate = torch.where(self.expand(cut), dstate * self.expand(alpha), dstate)
                trial = self.rhs(state + dstate, active=cut)
                rhs_new = torch.where(self.expand(cut), trial, rhs_new)
                eval_j = eval_j | cut
            state = torch.where(self.expand(go), state + dstate, state)
            rhs = torch.where(self.expand(go), rhs_new, rhs)
            res = torch.where(go, self.norms(rhs), res)
            failed = failed | (go & (res > max_allowed_residual))
            failed = failed | (go & (self.mins(state) < min_allowable_state_var))
        state = torch.clamp(state, min=0.)
        conv = run & ~failed & (res <= tolerance) & (it <= max_iterations)
        return state, conv, it

    def steady_solve_psitc_host(self, initial, active=None, tolerance=1.e-6, max_iterations=400,
                                min_allowable_state_var=-1.e-6, ds_init=1., ds_init_decrease=4., diffusion_factor=4.,
                                global_ds=False, ds_safety=0.1, ds_ramp=1.1, ds_max=1.e4, max_factor_line_search=1.5,
                                max_allowed_residual=1.e6, max_recursion_depth=20, adaptive_restart=True):
        """The same solver as steady_solve_psitc with its control loop on the host, including the restart from the
        initial guess with ds_init / ds_init_decrease after a failure (a flamelet gives up once a failure happens
        at restart depth > max_recursion_depth, or at once without adaptive_restart); kept to check the native
        solver against."""
        torch = _torch()
        dev = initial.device
        nf, ns = self.nf, self.ns
        run = torch.ones(nf, dtype=torch.bool, device=dev) if active is None else active.clone()
        dterm = self.diffterm_tensor(diffusion_factor)
        state = initial.clone()
        depth = torch.zeros(nf, dtype=torch.int64, device=dev)
        dsi = torch.full((nf,), float(ds_init), dtype=torch.float64, device=dev)
        ds = self.expand(dsi).clone()
        it = torch.zeros(nf, dtype=torch.int64, device=dev)
        jac_age = torch.zeros(nf, dtype=torch.int64, device=dev)
        res = torch.full((nf,), tolerance + 1., dtype=torch.float64, device=dev)
        dead = torch.zeros(nf, dtype=torch.bool, device=dev)
        rhs = self.rhs(state, active=run)
        eval_j = torch.ones(nf, dtype=torch.bool, device=dev)
        dstate = torch.zeros_like(state)
        total_cap = (max_iterations + 1) * (max_recursion_depth + 3)
        for _ in range(total_cap):
            go = run & ~dead & (res > tolerance) & (it < max_iterations)
            if not bool(go.any()):
                break
            it = it + go.long()
            need = go & eval_j
            if bool(need.any()):
                _, expeig = self.jacobian(state, eig=True, diffterm_per_flamelet=dterm, active=need)
                # a true division, as numpy's ds_safety / (expeig + 1e-16) in the reference (torch evaluates
                # scalar / tensor as scalar * reciprocal(tensor), two roundings)
                safe = torch.div(torch.full_like(expeig, float(ds_safety)), expeig + 1.e-16)
                new_ds = torch.minimum(torch.minimum(safe, ds_ramp * ds),
                                       torch.full_like(ds, ds_max))
                first = need & ((it == 1) | global_ds)
                mn = torch.full((nf,), float('inf'), dtype=torch.float64, device=dev).scatter_reduce(
                    0, self.dof_flamelet, new_ds, reduce='amin', include_self=True)
                new_ds = torch.where(self.expand(first), self.expand(mn), new_ds)
                ds = torch.where(self.expand(need), new_ds, ds)
                self.scale_and_add_diagonal(-1., 1. / ds, 1., active=need)
                self.factor(active=need)
                jac_age = torch.where(need, torch.zeros_like(jac_age), jac_age)
            jac_age = torch.where(go & ~need, jac_age + 1, jac_age)
            eval_j = torch.where(go, (jac_age == 8) | (res > 1.e-2), eval_j)
            self.solve(rhs, out=dstate, active=go)
            bad = go & ~self.finite(dstate)
            dstate = torch.where(self.expand(go), torch.nan_to_num(dstate), torch.zeros_like(dstate))
            norm_old = self.norms(rhs)
            rhs_new = self.rhs(state + dstate, active=go)
            bad = bad | (go & ~self.finite(rhs_new))
            rhs_new = torch.nan_to_num(rhs_new, nan=1e300, posinf=1e300, neginf=-1e300)
            alpha = torch.ones(nf, dtype=torch.float64, device=dev)
            ok_go = go & ~bad
            for _ls in range(12):
                cut = ok_go & (self.norms(rhs_new) > max_factor_line_search * norm_old) & (alpha > 0.001)
                if not bool(cut.any()):
                    break
                alpha = torch.where(cut, alpha * 0.5, alpha)
                dstate = torch.where(self.expand(cut), dstate * self.expand(alpha), dstate)
                trial = self.rhs(state + dstate, active=cut)
                rhs_new = torch.where(self.expand(cut), trial, rhs_new)
                eval_j = eval_j | cut
            state = torch.where(self.expand(ok_go), state + dstate, state)
            rhs = torch.where(self.expand(ok_go), rhs_new, rhs)
            res = torch.where(ok_go, self.norms(rhs), res)
            bad = bad | (ok_go & (res > max_allowed_residual)) | (ok_go & (self.mins(state) < min_allowable_state_var))
            # restart failed flamelets from the initial guess with a smaller initial pseudo-time step
            if bool(bad.any()):
                give_up = bad & ((depth > max_recursion_depth) | (not adaptive_restart))
                dead = dead | give_up
                rst = bad & ~give_up
                if bool(rst.any()):
                    depth = torch.where(rst, depth + 1, depth)
                    dsi = torch.where(rst, dsi / ds_init_decrease, dsi)
                    e = self.expand(rst)
                    state = torch.where(e, initial, state)
                    ds = torch.where(e, self.expand(dsi), ds)
                    it = torch.where(rst, torch.zeros_like(it), it)
                    jac_age = torch.where(rst, torch.zeros_like(jac_age), jac_age)
                    res = torch.where(rst, torch.full_like(res, tolerance + 1.), res)
                    eval_j = eval_j | rst
                    rhs = torch.where(e, self.rhs(state, active=rst), rhs)
        state = torch.clamp(state, min=0.)
        conv = run & ~dead & (res <= tolerance)
        # smallest pseudo-time step of each flamelet where it stopped (the reference's psitc returns it, and
        # compute_steady_state starts its ESDIRK fallback from 1e-2 of it)
        self.last_psitc_min_ds = torch.full((nf,), float('inf'), dtype=torch.float64, device=dev).scatter_reduce(
            0, self.dof_flamelet, ds, reduce='amin', include_self=True)
        return state, conv, it

    def integrate(self, state=None, **kwargs):
        """Transient integration of every flamelet of the batch (Flamelet.integrate, flamelet.py:1046-1213, for all
        of them at once); see _integrate_batch for the arguments and results."""
        return _integrate_batch(self, state, **kwargs)

    def compute_steady_state(self, state=None, tolerance=1.e-6, newton_iterations=38, psitc_iterations=400,
                             transient_args=None):
        """compute_steady_state of flamelet.py:1705-1778 for the whole batch: Newton (38 iterations); psitc (400) for
        the flamelets Newton did not converge; ESDIRK64 time integration to a steady state from the initial guess
        for those psitc did not converge either (steady tolerance `tolerance`, transient tolerance 1e-8, steps of at
        most 1e4 starting at 1e-2 of psitc's smallest pseudo-time step, the Jacobian reused for up to 10 steps;
        transient_args override these). Returns (state, converged [nf], {'newton', 'psitc', 'esdirk'} masks)."""
        torch = _torch()
        init = self.initial_state() if state is None else state
        s1, c1, i1 = self.steady_solve_newton(init, tolerance=tolerance, max_iterations=newton_iterations)
        none = torch.zeros_like(c1)
        if bool(c1.all()):
            return s1, c1, {'newton': c1, 'psitc': none, 'esdirk': none}
        s2, c2, i2 = self.steady_solve_psitc(init, active=~c1, tolerance=tolerance, max_iterations=psitc_iterations)
        out = torch.where(self.expand(c1), s1, s2)
        conv = c1 | c2
        esdirk = none.clone()
        if not bool(conv.all()):
            fail = (~conv).cpu().numpy()
            mds = self.last_psitc_min_ds.cpu().numpy()
            args = dict(stop_at_steady=tolerance, transient_tolerance=1.e-8, max_time_step=1.e4,
                        first_time_step=np.where(np.isfinite(mds), 1.e-2 * mds, 1.e-8),
                        maximum_steps_per_jacobian=10, save_each_step=False)
            args.update(transient_args or {})
            traj, stats = self.integrate(init, active=fail, **args)
            for f in np.flatnonzero(fail & (stats['status'] == 3)):
                lo, hi = int(self.offz_host[f]) * self.ns, int(self.offz_host[f + 1]) * self.ns
                out[lo:hi] = torch.from_numpy(traj[f][1][-1]).to(out.device)
                esdirk[f] = True
            conv = conv | esdirk
        return out, conv, {'newton': c1, 'psitc': c2 & ~c1, 'esdirk': esdirk}


# ESDIRK64 (Kennedy & Carpenter's six-stage, fourth-order ESDIRK with a third-order embedded estimate), the
# published tableau that spitfire/time/methods.py:464-500 and the batched reactor integrator use
_ESDIRK_GAMMA = 0.25
_ESDIRK_A = np.array([[0., 0., 0., 0., 0., 0.],
                      [0.25, 0.25, 0., 0., 0., 0.],
                      [8611. / 62500., -1743. / 31250., 0.25, 0., 0., 0.],
                      [5012029. / 34652500., -654441. / 2922500., 174375. / 388108., 0.25, 0., 0.],
                      [15267082809. / 155376265600., -71443401. / 120774400., 730878875. / 902184768.,
                       2285395. / 8070912., 0.25, 0.],
                      [82889. / 524892., 0., 15625. / 83664., 69875. / 102672., -2260. / 8211., 0.25]])
_ESDIRK_B = _ESDIRK_A[5].copy()
_ESDIRK_BH = np.array([4586570599. / 29645900160., 0., 178811875. / 945068544., 814220225. / 1159782912.,
                       -3700637. / 11593932., 61727. / 225920.])


def _integrate_batch(b, state=None, stop_criteria=None, stop_at_time=None, stop_at_steady=None,
                     first_time_step=1.e-6, max_time_step=1.e-3, minimum_time_step_count=40,
                     maximum_time_step_count=None, transient_tolerance=1.e-10, maximum_steps_per_jacobian=10,
                     nonlinear_solve_tolerance=1.e-12, max_nonlinear_iter=20, save_each_step=True, active=None,
                     max_attempts=1000000, host_attempts=False):
    """Transient integration of every flamelet of the batch b, each with its own time, step size and Jacobian.

    Batched restatement of Flamelet.integrate (flamelet.py:1046-1213) with its defaults: odesolve
    (time/integrator.py:229-713) driving ESDIRK64 (time/methods.py:441-612), SimpleNewtonSolver (time/nonlinear.py:
    185-268; frozen Jacobian, weighted inf-norm below nonlinear_solve_tolerance, max_nonlinear_iter iterations) and
    PIController (time/stepcontrol.py:84-101). The linear setup is prefactor * J - I with prefactor = gamma * dt,
    factorized by the block-Thomas kernels (flamelet.py:756-761, 881-886). It is reused for up to
    maximum_steps_per_jacobian steps and redone after a slow Newton solve or a step-size change beyond
    [0.9, 1.05] (integrator.py:100-130). Negative entries are clipped after every accepted step
    (flamelet.py:1119-1121). Each round of the loop is one step attempt of every running flamelet: every Newton
    iteration is one batched solve and one batched right-hand side over the flamelets still iterating.

    first_time_step: a number or one per flamelet. stop_criteria: None or a callable (f, t, state_f, residual,
    steps) -> bool for flamelet f (host arrays), checked after every attempt and overridden below
    minimum_time_step_count steps, as odesolve does (integrator.py:629-641). Returns (trajectories, stats):
    trajectories[f] = (times [nt], states [nt, nzi*ns]) with every accepted step (first and last only without
    save_each_step); stats: per-flamelet steps, failed_steps, newton_iters,
    jac_setups and status (1 stop_at_time, 3 steady, 4 step limit, 7 stop criteria).

    Each step attempt of the running flamelets (iteration matrices where needed, the five implicit stages with
    their Newton iterations, the error and step norms, the acceptance) is one native call,
    sf_flamelet_esdirk_attempt_batch; the step-size control, the stop rules and the recorded trajectory stay here.
    host_attempts=True runs the same attempt as torch operations over the batch's primitives instead: the same
    arithmetic in the same order, kept to check the native attempt against."""
    torch = _torch()
    dev = b.values.device
    nf, ns = b.nf, b.ns
    state = (b.initial_state() if state is None else state).clone()
    run = np.ones(nf, dtype=bool) if active is None else \
        np.asarray(active.cpu().numpy() if torch.is_tensor(active) else active, dtype=bool).copy()
    seg = [(int(b.offz_host[f]) * ns, int(b.offz_host[f + 1]) * ns) for f in range(nf)]
    t = np.zeros(nf)
    dt = np.broadcast_to(np.asarray(first_time_step, dtype=np.float64), (nf,)).copy()  # a number or one per flamelet
    eval_setup = np.ones(nf, dtype=bool)
    setup_count = np.zeros(nf, dtype=np.int64)
    steps = np.zeros(nf, dtype=np.int64)
    failed = np.zeros(nf, dtype=np.int64)
    newton = np.zeros(nf, dtype=np.int64)
    jac_setups = np.zeros(nf, dtype=np.int64)
    attempts = np.zeros(nf, dtype=np.int64)
    status = np.zeros(nf, dtype=np.int64)
    host = state.cpu().numpy()
    times = [[0.] for _ in range(nf)]
    states = [[host[a:e].copy()] for (a, e) in seg]
    G, A, B, BH = _ESDIRK_GAMMA, _ESDIRK_A, _ESDIRK_B, _ESDIRK_BH
    k = [torch.zeros_like(state) for _ in range(6)]
    coerce = stop_at_time is not None
    mask = lambda m: torch.from_numpy(np.ascontiguousarray(m)).to(dev)

    def host_attempt(state, dt, run, need):
        """One step attempt of the running flamelets as torch operations (the native attempt's check)."""
        if need.any():
            # one launch for every flamelet that needs a setup, each with its own prefactor gamma * dt
            b.jacobian(state, scale_and_offset=True, prefactor=torch.from_numpy(dt * G).to(dev), active=mask(need))
            b.factor(active=mask(need))
        runm = mask(run)
        dtd = b.expand(torch.from_numpy(dt).to(dev))
        k[0] = b.rhs(state, out=k[0], active=runm)
        Y = state.clone()
        nl_ok = np.ones(nf, dtype=bool)
        for st in range(1, 6):
            prior = A[st, 0] * k[0]
            for j in range(1, st):
                prior = prior + A[st, j] * k[j]
            fs = k[st - 1].clone()
            resid = dtd * (G * fs + prior) - (Y - state)
            go = runm.clone()
            conv = torch.zeros(nf, dtype=torch.bool, device=dev)
            for _ in range(max_nonlinear_iter):
                newton[:] += go.cpu().numpy()
                god = b.expand(go)
                dx = b.solve(resid, active=go)
                Y = torch.where(god, Y - dx, Y)
                fs = torch.where(god, b.rhs(Y, active=go), fs)
                resid = torch.where(god, dtd * (G * fs + prior) - (Y - state), resid)
                c = go & (b.norms(resid) < nonlinear_solve_tolerance)
                conv |= c
                go &= ~c
                if not bool(go.any()):
                    break
            k[st] = fs
            nl_ok &= conv.cpu().numpy() | ~run
        dstate = B[0] * k[0]
        derr = (B[0] - BH[0]) * k[0]
        for j in range(1, 6):
            dstate = dstate + B[j] * k[j]
            derr = derr + (B[j] - BH[j]) * k[j]
        dstate = dtd * dstate
        err = b.norms(dtd * derr).cpu().numpy()
        residual = b.norms(dstate).cpu().numpy() / dt
        fin = b.finite(dstate).cpu().numpy()
        acc = run & fin
        if acc.any():
            new = state + dstate
            new = torch.where(new < 0., torch.zeros_like(new), new)
            state = torch.where(b.expand(mask(acc)), new, state)
        return state, err, residual, fin, nl_ok

    if not host_attempts:
        L = N.load()
        nb = int(L.sf_flamelet_esdirk_workspace_size(b.g.handle, C.byref(b.fb)))
        att_ws = torch.empty(nb // 8 + 1, dtype=torch.float64, device=dev)
        dtt = torch.empty(nf, dtype=torch.float64, device=dev)
        runi = torch.empty(nf, dtype=torch.int32, device=dev)
        needi = torch.empty(nf, dtype=torch.int32, device=dev)
        att_err, att_norm, att_bad = (torch.empty(nf, dtype=torch.float64, device=dev) for _ in range(3))
        att_nlok = torch.empty(nf, dtype=torch.int32, device=dev)
        att_newton = torch.zeros(nf, dtype=torch.int32, device=dev)
        state = state.contiguous()
    while run.any():
        attempts[run] += 1
        over = run & (attempts > max_attempts)
        status[over] = 4
        run &= ~over
        if not run.any():
            break
        if coerce:
            dt = np.where(run & (t + dt > stop_at_time), stop_at_time - t, dt)
        need = run & eval_setup
        setup_count[run] += 1
        jac_setups[need] += 1
        if host_attempts:
            state, err, residual, fin, nl_ok = host_attempt(state, dt, run, need)
        else:
            dtt.copy_(torch.from_numpy(dt))
            runi.copy_(torch.from_numpy(run.astype(np.int32)))
            needi.copy_(torch.from_numpy(need.astype(np.int32)))
            N.check(L.sf_flamelet_esdirk_attempt_batch(
                b.g.handle, C.byref(b.fb), N.ptr(state), N.ptr(dtt), N.ptr(runi), N.ptr(needi), int(need.any()),
                float(nonlinear_solve_tolerance), int(max_nonlinear_iter), int(b.rates_option), N.ptr(att_err),
                N.ptr(att_norm), N.ptr(att_bad), N.ptr(att_nlok), N.ptr(att_newton), N.ptr(att_ws),
                att_ws.numel() * 8, N.stream_handle()))
            outs = torch.cat([att_err, att_norm, att_bad, att_nlok.double(), att_newton.double()]).cpu().numpy()
            err, residual = outs[:nf], outs[nf:2 * nf] / dt
            fin = outs[2 * nf:3 * nf] == 0.
            nl_ok = outs[3 * nf:4 * nf] != 0.
            newton[:] = outs[4 * nf:5 * nf].astype(np.int64)
        # the states reach the host only for the recorded trajectory or a stop criterion
        host = state.cpu().numpy() if (save_each_step or stop_criteria is not None) else None
        for f in np.flatnonzero(run):
            recent = dt[f]
            if fin[f]:
                t[f] += dt[f]
                steps[f] += 1
                if save_each_step:
                    times[f].append(t[f])
                    states[f].append(host[seg[f][0]:seg[f][1]].copy())
                e = err[f]
                dt[f] = min(dt[f] * 1.1, max_time_step) if e < 1.e-16 else \
                    min(dt[f] * min(1.1, (transient_tolerance / e) ** 0.1333333333), max_time_step)
                if setup_count[f] == maximum_steps_per_jacobian:
                    setup_count[f] = 0
                    eval_setup[f] = True
                elif not nl_ok[f]:
                    dt[f] *= 0.8
                    eval_setup[f] = True
                elif dt[f] > recent * 1.05 or dt[f] < recent * 0.9:
                    eval_setup[f] = True
                else:
                    eval_setup[f] = False
            else:
                dt[f] *= 0.8
                eval_setup[f] = True
                failed[f] += 1
            cont = True
            if stop_criteria is not None:
                cont = not stop_criteria(f, t[f], host[seg[f][0]:seg[f][1]], residual[f], steps[f])
                if not cont:
                    status[f] = 7
            if steps[f] < minimum_time_step_count:
                cont = True
                status[f] = 0
            if maximum_time_step_count is not None and steps[f] > maximum_time_step_count:
                cont = False
                status[f] = 4
            elif coerce and t[f] >= stop_at_time:
                cont = False
                status[f] = 1
            elif stop_at_steady is not None and residual[f] < stop_at_steady:
                cont = False
                status[f] = 3
            if not cont:
                run[f] = False
    host = state.cpu().numpy()
    out = []
    for f in range(nf):
        if save_each_step:
            out.append((np.array(times[f]), np.array(states[f])))
        else:
            out.append((np.array([0., t[f]]), np.array([states[f][0], host[seg[f][0]:seg[f][1]].copy()])))
    return out, dict(steps=steps, failed_steps=failed, newton_iters=newton, jac_setups=jac_setups, status=status)



class Flamelet:
    """Drop-in for spitfire.chemistry.flamelet.Flamelet's steady path (one flamelet, GPU kernels)."""

    def __init__(self, flamelet_specs=None, **kwargs):
        fs = FlameletSpec(**flamelet_specs) if isinstance(flamelet_specs, dict) else \
            (flamelet_specs if flamelet_specs is not None else FlameletSpec(**kwargs))
        self._fs = fs
        self._setup = FlameletSetup(fs)
        self._batch = None
        self._current_state = self._setup.initial_state.copy()

    def _b(self):
        if self._batch is None:
            self._batch = FlameletBatch([self._setup])
        return self._batch

    @property
    def mechanism(self):
        return self._setup.mech

    @property
    def oxy_stream(self):
        return self._fs.oxy_stream

    @property
    def fuel_stream(self):
        return self._fs.fuel_stream

    @property
    def mixfrac_grid(self):
        return self._setup.z

    @property
    def dissipation_rate(self):
        return self._setup.x

    @property
    def initial_interior_state(self):
        return self._setup.initial_state.copy()

    @property
    def current_interior_state(self):
        return self._current_state.copy()

    @property
    def current_temperature(self):
        return self._current_state[::self._setup.mech.n_species]

    @property
    def linear_temperature(self):
        return self._setup.linear_temperature

    def _run(self, fn, **kw):
        torch = _torch()
        b = self._b()
        st = torch.tensor(self._current_state, dtype=torch.float64, device='cuda')
        out, conv, it = fn(st, **kw)
        return out, bool(conv[0]), int(it[0])

    def steady_solve_newton(self, initial_guess=None, tolerance=1.e-6, max_iterations=10, **kw):
        if initial_guess is not None:
            self._current_state = np.array(initial_guess, dtype=np.float64)
        out, conv, it = self._run(self._b().steady_solve_newton, tolerance=tolerance, max_iterations=max_iterations)
        if not conv:
            return None, None, False
        self._current_state = out.cpu().numpy()
        return self.make_library_from_interior_state(self._current_state), it, True

    def steady_solve_psitc(self, initial_guess=None, tolerance=1.e-6, max_iterations=400, **kw):
        if initial_guess is not None:
            self._current_state = np.array(initial_guess, dtype=np.float64)
        out, conv, it = self._run(self._b().steady_solve_psitc, tolerance=tolerance, max_iterations=max_iterations,
                                  **kw)
        if not conv:
            return None, None, False, None
        self._current_state = out.cpu().numpy()
        return self.make_library_from_interior_state(self._current_state), it, True, None

    def compute_steady_state(self, tolerance=1.e-6, verbose=False, use_psitc=True, **kw):
        torch = _torch()
        b = self._b()
        st = torch.tensor(self._current_state, dtype=torch.float64, device='cuda')
        out, conv, _ = b.compute_steady_state(st, tolerance=tolerance)
        if not bool(conv[0]):
            raise RuntimeError('steady flamelet solve failed (Newton, psitc and ESDIRK time integration)')
        self._current_state = out.cpu().numpy()
        return self.make_library_from_interior_state(self._current_state)

    def integrate(self, stop_at_time=None, stop_at_steady=None, stop_criteria=None, first_time_step=1.e-6,
                  max_time_step=1.e-3, minimum_time_step_count=40, transient_tolerance=1.e-10, write_log=False,
                  log_rate=100, maximum_steps_per_jacobian=10, nonlinear_solve_tolerance=1.e-12,
                  linear_solver='block thomas', save_first_and_last_only=False, print_exception_on_failure=False,
                  **kw):
        """Transient integration from the current state (flamelet.py:1046-1213), on the GPU kernels: ESDIRK64,
        simple Newton and PI control with the block-Thomas linear solver. stop_criteria(t, state, residual, steps)
        as in the reference. Returns a Library over (time, mixture_fraction) with temperature, pressure and mass
        fractions; the current state and time move to the last step."""
        torch = _torch()
        if linear_solver.lower() != 'block thomas':
            raise ValueError('only the block-Thomas linear solver is on the GPU path')
        custom = [k for k in ('stepper_type', 'nlsolver_type', 'stepcontrol_type') if kw.get(k) is not None] + \
            [k for k in ('extra_integrator_args', 'extra_stepper_args', 'extra_nlsolver_args',
                         'extra_stepcontrol_args') if kw.get(k)]
        if custom:
            raise NotImplementedError('the GPU path integrates with the defaults of Flamelet.integrate (ESDIRK64, '
                                      'simple Newton, PI control); not supported: ' + ', '.join(custom))
        unknown = set(kw) - {'stepper_type', 'nlsolver_type', 'stepcontrol_type', 'extra_integrator_args',
                             'extra_stepper_args', 'extra_nlsolver_args', 'extra_stepcontrol_args'}
        if unknown:
            raise TypeError('integrate() got unexpected arguments: ' + ', '.join(sorted(unknown)))
        if stop_at_time is None and stop_at_steady is None and stop_criteria is None:
            raise ValueError('integrate needs stop_at_time, stop_at_steady or stop_criteria')
        crit = None if stop_criteria is None else (lambda f, t, st, res, n: stop_criteria(t, st, res, n))
        st = torch.tensor(self._current_state, dtype=torch.float64, device='cuda')
        t0 = getattr(self, '_current_time', 0.)
        traj, _ = self._b().integrate(st, stop_criteria=crit,
                                      stop_at_time=None if stop_at_time is None else stop_at_time - t0,
                                      stop_at_steady=stop_at_steady, first_time_step=first_time_step,
                                      max_time_step=max_time_step, minimum_time_step_count=minimum_time_step_count,
                                      transient_tolerance=transient_tolerance,
                                      maximum_steps_per_jacobian=maximum_steps_per_jacobian,
                                      nonlinear_solve_tolerance=nonlinear_solve_tolerance,
                                      save_each_step=not save_first_and_last_only)
        times, states = traj[0]
        times = times + t0
        self._current_state = states[-1].copy()
        self._current_time = float(times[-1])
        if save_first_and_last_only:
            times, states = times[-1:], states[-1:]
        return self._library_over_time(times, states)

    def integrate_to_steady(self, steady_tolerance=1.e-4, **kwargs):
        """flamelet.py:1215-1225."""
        return self.integrate(stop_at_steady=steady_tolerance, **kwargs)

    def integrate_to_time(self, final_time, **kwargs):
        """flamelet.py:1227-1237."""
        return self.integrate(stop_at_time=final_time, **kwargs)

    def integrate_for_heat_loss(self, temperature_tolerance=0.05, steady_tolerance=1.e-4, **kwargs):
        """flamelet.py:1263-1286: integrate until max(state) < (1 + temperature_tolerance) max(T_oxy, T_fuel) or
        the step residual falls below steady_tolerance."""
        T_bc_max = max(self.oxy_stream.T, self.fuel_stream.T)

        def stop(t, state, residual, *args):
            return np.max(state) < (1. + temperature_tolerance) * T_bc_max or residual < steady_tolerance

        return self.integrate(stop_criteria=stop, **kwargs)

    def _library_over_time(self, times, states):
        from .library import Dimension, Library
        s = self._setup
        ns = s.mech.n_species
        lib = Library(Dimension('time', np.asarray(times)), Dimension('mixture_fraction', s.z))
        lib.extra_attributes['mech_spec'] = s.mech
        nt = len(times)
        st = np.asarray(states).reshape(nt, s.nzi, ns)
        full = np.concatenate([np.broadcast_to(s.state_oxy, (nt, 1, ns)), st,
                               np.broadcast_to(s.state_fuel, (nt, 1, ns))], axis=1)
        lib['temperature'] = full[:, :, 0].copy()
        lib['pressure'] = np.full((nt, s.z.size), s.pressure)
        names = s.mech.species_names
        last = np.ones((nt, s.z.size))
        for i, sp in enumerate(names[:-1]):
            lib['mass fraction ' + sp] = full[:, :, 1 + i].copy()
            last -= full[:, :, 1 + i]
        lib['mass fraction ' + names[-1]] = last
        return lib

    def make_library_from_interior_state(self, state):
        from .library import Dimension, Library
        s = self._setup
        ns = s.mech.n_species
        st = np.array(state).reshape(s.nzi, ns)
        full = np.vstack([s.state_oxy, st, s.state_fuel])
        lib = Library(Dimension('mixture_fraction', s.z))
        lib['temperature'] = full[:, 0]
        lib['pressure'] = np.full(s.z.size, s.pressure)
        names = s.mech.species_names
        last = np.ones(s.z.size)
        for i, sp in enumerate(names[:-1]):
            lib['mass fraction ' + sp] = full[:, 1 + i]
            last -= full[:, 1 + i]
        lib['mass fraction ' + names[-1]] = last
        return lib
