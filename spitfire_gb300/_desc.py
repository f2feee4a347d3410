"""Flat mechanism description and ctypes mirrors of the C-ABI structs in include/spitfire_gb300.h.

``MechanismRecorder`` keeps the calls Spitfire makes on Griffon's 16 ``mechanism_*`` setters
(``griffon.pyx:234-551``; argument meanings as in ``combustion_kernels.h:293-379``) and turns them into the arrays
of ``sf_mech_desc``. Reactant, product, efficiency and order maps are emitted in ascending species-name order,
which is the ``std::map<std::string, ...>`` order Griffon iterates in (``chemistry_setup.cpp:361-392``), so index
lists, order classes and summation orders derived from them match Griffon's.
"""

import ctypes as C

import numpy as np

SF_THERMO_CONST, SF_THERMO_NASA7, SF_THERMO_NASA9 = 1, 2, 3
SF_RXN_SIMPLE, SF_RXN_THIRD_BODY, SF_RXN_LINDEMANN, SF_RXN_TROE = 1, 2, 3, 4

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_longlong)


class SfMechDesc(C.Structure):
    _fields_ = [('n_species', C.c_int), ('n_reactions', C.c_int), ('n_elements', C.c_int),
                ('gas_constant', C.c_double), ('ref_pressure', C.c_double), ('ref_temperature', C.c_double),
                ('molecular_weights', _dp), ('thermo_kind', _ip), ('thermo_coefs', _dp),
                ('nasa9_offsets', _ip), ('nasa9_coefs', _dp),
                ('rxn_kind', _ip), ('rxn_reversible', _ip), ('rxn_kfwd', _dp), ('rxn_kflf', _dp),
                ('rxn_troe', _dp), ('rxn_default_eff', _dp),
                ('reac_offsets', _ip), ('reac_species', _ip), ('reac_stoich', _ip),
                ('prod_offsets', _ip), ('prod_species', _ip), ('prod_stoich', _ip),
                ('eff_offsets', _ip), ('eff_species', _ip), ('eff_values', _dp),
                ('order_offsets', _ip), ('order_species', _ip), ('order_values', _dp)]


class SfReactorParams(C.Structure):
    _fields_ = [('configuration', C.c_int), ('heat_transfer', C.c_int), ('open', C.c_int),
                ('pressure', C.c_double), ('inflow_density', C.c_double), ('inflow_temperature', C.c_double),
                ('inflow_Y', _dp), ('tau', C.c_double), ('fluid_temperature', C.c_double),
                ('surface_temperature', C.c_double), ('h_convection', C.c_double), ('eps_radiation', C.c_double),
                ('surface_area_to_volume', C.c_double)]


class SfIntegrateParams(C.Structure):
    _fields_ = [('first_time_step', C.c_double), ('max_time_step', C.c_double),
                ('transient_tolerance', C.c_double), ('nonlinear_tolerance', C.c_double),
                ('minimum_time_step_count', C.c_int), ('maximum_time_step_count', C.c_int),
                ('max_nonlinear_iter', C.c_int), ('maximum_steps_per_jacobian', C.c_int),
                ('stop_at_time', C.c_double), ('delta_temperature_ignition', C.c_double),
                ('minimum_allowable_residual', C.c_double), ('stop_at_steady', C.c_double),
                ('linear_precision', C.c_int), ('refine_sweeps', C.c_int), ('rates_option', C.c_int),
                ('max_attempts', C.c_int), ('time_table', _dp), ('time_points', C.c_int),
                ('time_width', C.c_int), ('time_columns', C.c_int), ('time_t0', C.c_double),
                ('time_dt', C.c_double), ('time_jac_t0', C.c_double), ('ignition_time_interp', _dp)]

# bits of SfIntegrateParams.time_columns (enum sf_time_param), in column order
TIME_PARAMS = [('feed_temperature', 1), ('mixing_tau', 2), ('convection_temperature', 4),
               ('convection_coefficient', 8), ('radiation_temperature', 16), ('radiative_emissivity', 32),
               ('feed_mass_fractions', 64)]


class SfFlameletBatch(C.Structure):
    _fields_ = [('n_flamelets', C.c_int), ('offsets_z', _ip), ('offsets_v', _lp), ('offsets_z_host', _ip),
                ('pressure', C.c_double), ('oxy_state', _dp), ('fuel_state', _dp),
                ('cmajor', _dp), ('csub', _dp), ('csup', _dp), ('mcoeff', _dp), ('ncoeff', _dp), ('chi', _dp),
                ('include_enthalpy_flux', C.c_int), ('include_variable_cp', C.c_int), ('diffterm', _dp),
                ('active', _ip), ('T_convection', _dp), ('h_convection', _dp), ('T_radiation', _dp),
                ('h_radiation', _dp), ('use_scaled_heat_loss', C.c_int), ('prefactor', _dp)]


def reactor_params(configuration='isobaric', heat_transfer='adiabatic', open_=False, pressure=101325.,
                   inflow_density=0., inflow_temperature=300., inflow_Y_ptr=None, tau=1., fluid_temperature=300.,
                   surface_temperature=300., h_convection=0., eps_radiation=0., surface_area_to_volume=1.):
    p = SfReactorParams()
    p.configuration = {'isobaric': 0, 'isochoric': 1}[configuration] if isinstance(configuration, str) else \
        int(configuration)
    p.heat_transfer = {'adiabatic': 0, 'isothermal': 1, 'diathermal': 2}[heat_transfer] \
        if isinstance(heat_transfer, str) else int(heat_transfer)
    p.open = int(bool(open_))
    p.pressure = pressure
    p.inflow_density = inflow_density
    p.inflow_temperature = inflow_temperature
    p.inflow_Y = C.cast(C.c_void_p(inflow_Y_ptr), _dp) if inflow_Y_ptr else None
    p.tau = tau
    p.fluid_temperature = fluid_temperature
    p.surface_temperature = surface_temperature
    p.h_convection = h_convection
    p.eps_radiation = eps_radiation
    p.surface_area_to_volume = surface_area_to_volume
    return p


class MechanismRecorder:
    """Records Griffon setter calls; ``desc()`` returns an SfMechDesc whose arrays this object keeps alive."""

    def __init__(self):
        self.ref_pressure = 101325.
        self.ref_temperature = 298.15
        self.gas_constant = 8314.46261815324
        self.element_mw = {}
        self.elements = []
        self.species = []
        self.species_mw = []
        self.thermo = {}
        self.reactions = []
        self._desc = None

    # ---- setters with the argument meanings of griffon.pyx:234-551 ----
    def set_element_mw_map(self, m):
        self.element_mw = {str(k): float(v) for k, v in m.items()}

    def add_element(self, name):
        if name not in self.elements:
            self.elements.append(name)

    def add_species(self, name, atom_map):
        if name in self.species:
            raise ValueError(f'species {name} cannot be added twice')
        for a in atom_map:
            if a not in self.elements:
                raise ValueError(f'cannot find atom {a}')
        mw = 0.
        for a in sorted(atom_map):
            mw += self.element_mw[a] * atom_map[a]
        self.species.append(name)
        self.species_mw.append(mw)

    def add_thermo(self, name, kind, coefs, nasa9=None):
        self.thermo[name] = (kind, np.asarray(coefs, dtype=np.float64), nasa9)

    def add_reaction(self, kind, reactants, products, reversible, kfwd, kflf=None, troe=None, efficiencies=None,
                     default_eff=1.0, orders=None):
        self.reactions.append(dict(kind=kind, reactants=dict(reactants), products=dict(products),
                                   reversible=bool(reversible), kfwd=[float(v) for v in kfwd],
                                   kflf=[float(v) for v in (kflf or [0., 0., 0.])],
                                   troe=[float(v) for v in (list(troe) if troe is not None else [0., 0., 0., 0.])],
                                   efficiencies=dict(efficiencies or {}), default_eff=float(default_eff),
                                   orders=dict(orders or {})))
        self._desc = None

    # ---- flattening ----
    def arrays(self):
        ns = len(self.species)
        nr = len(self.reactions)
        sidx = {s: i for i, s in enumerate(self.species)}
        a = {}
        a['mw'] = np.array(self.species_mw, dtype=np.float64)
        a['thermo_kind'] = np.zeros(ns, dtype=np.int32)
        a['thermo_coefs'] = np.zeros(ns * 20, dtype=np.float64)
        n9off = [0]
        n9 = []
        for i, s in enumerate(self.species):
            if s not in self.thermo:
                raise ValueError(f'species {s} has no heat-capacity data')
            kind, coefs, nasa9 = self.thermo[s]
            a['thermo_kind'][i] = kind
            a['thermo_coefs'][20 * i:20 * i + coefs.size] = coefs
            if kind == SF_THERMO_NASA9:
                n9 += list(nasa9)
            n9off.append(len(n9))
        a['nasa9_offsets'] = np.array(n9off, dtype=np.int32)
        a['nasa9_coefs'] = np.array(n9 if n9 else [0.], dtype=np.float64)
        a['rxn_kind'] = np.array([r['kind'] for r in self.reactions] or [0], dtype=np.int32)
        a['rxn_reversible'] = np.array([int(r['reversible']) for r in self.reactions] or [0], dtype=np.int32)
        a['rxn_kfwd'] = np.array([v for r in self.reactions for v in r['kfwd']] or [0.], dtype=np.float64)
        a['rxn_kflf'] = np.array([v for r in self.reactions for v in r['kflf']] or [0.], dtype=np.float64)
        a['rxn_troe'] = np.array([v for r in self.reactions for v in r['troe']] or [0.], dtype=np.float64)
        a['rxn_default_eff'] = np.array([r['default_eff'] for r in self.reactions] or [0.], dtype=np.float64)

        def csr(key, cast, dtype):
            off = [0]
            idx = []
            val = []
            for r in self.reactions:
                for name in sorted(r[key]):
                    if name not in sidx:
                        if key == 'efficiencies':
                            continue
                        raise ValueError(f'unknown species {name}')
                    idx.append(sidx[name])
                    val.append(cast(r[key][name]))
                off.append(len(idx))
            return (np.array(off, dtype=np.int32), np.array(idx or [0], dtype=np.int32),
                    np.array(val or [0], dtype=dtype))

        a['reac_offsets'], a['reac_species'], a['reac_stoich'] = csr('reactants', lambda v: int(round(v)), np.int32)
        a['prod_offsets'], a['prod_species'], a['prod_stoich'] = csr('products', lambda v: int(round(v)), np.int32)
        a['eff_offsets'], a['eff_species'], a['eff_values'] = csr('efficiencies', float, np.float64)
        a['order_offsets'], a['order_species'], a['order_values'] = csr('orders', float, np.float64)
        return a

    def desc(self):
        if self._desc is not None:
            return self._desc
        a = self.arrays()
        self._arrays = a
        d = SfMechDesc()
        d.n_species = len(self.species)
        d.n_reactions = len(self.reactions)
        d.n_elements = len(self.elements)
        d.gas_constant = self.gas_constant
        d.ref_pressure = self.ref_pressure
        d.ref_temperature = self.ref_temperature

        def p(name, ctype):
            arr = a[name]
            return arr.ctypes.data_as(C.POINTER(ctype))
        d.molecular_weights = p('mw', C.c_double)
        d.thermo_kind = p('thermo_kind', C.c_int)
        d.thermo_coefs = p('thermo_coefs', C.c_double)
        d.nasa9_offsets = p('nasa9_offsets', C.c_int)
        d.nasa9_coefs = p('nasa9_coefs', C.c_double)
        for k in ('rxn_kind', 'rxn_reversible'):
            setattr(d, k, p(k, C.c_int))
        for k in ('rxn_kfwd', 'rxn_kflf', 'rxn_troe', 'rxn_default_eff'):
            setattr(d, k, p(k, C.c_double))
        for k in ('reac_offsets', 'reac_species', 'reac_stoich', 'prod_offsets', 'prod_species', 'prod_stoich',
                  'eff_offsets', 'eff_species', 'order_offsets', 'order_species'):
            setattr(d, k, p(k, C.c_int))
        d.eff_values = p('eff_values', C.c_double)
        d.order_values = p('order_values', C.c_double)
        self._desc = d
        return d


class GriffonSetters:
    """The 16 mechanism setters of ``PyCombustionKernels`` (griffon.pyx:234-551), recording into
    ``self._rec`` (a MechanismRecorder). Activation energies arrive already divided by R, as Spitfire passes
    them (mechanism.py:191)."""

    def _recorder(self):
        if not hasattr(self, '_rec') or self._rec is None:
            self._rec = MechanismRecorder()
        return self._rec

    def _mechanism_changed(self):
        pass

    def mechanism_set_element_mw_map(self, element_mw_map):
        self._recorder().set_element_mw_map(element_mw_map)

    def mechanism_add_element(self, element_name):
        self._recorder().add_element(element_name)

    def mechanism_add_species(self, species_name, atom_map):
        self._recorder().add_species(species_name, atom_map)

    def mechanism_set_ref_pressure(self, p):
        self._recorder().ref_pressure = float(p)

    def mechanism_set_ref_temperature(self, T):
        self._recorder().ref_temperature = float(T)

    def mechanism_set_gas_constant(self, Ru):
        self._recorder().gas_constant = float(Ru)

    def mechanism_resize_heat_capacity_data(self):
        pass

    def mechanism_add_const_cp(self, spec_name, Tmin, Tmax, T0, h0, s0, cp):
        self._recorder().add_thermo(spec_name, SF_THERMO_CONST, [Tmin, Tmax, T0, h0, s0, cp])
        self._mechanism_changed()

    def mechanism_add_nasa7_cp(self, spec_name, Tmin, Tmid, Tmax, low_coeffs, high_coeffs):
        self._recorder().add_thermo(spec_name, SF_THERMO_NASA7,
                                    [Tmin, Tmid, Tmax] + list(low_coeffs) + list(high_coeffs))
        self._mechanism_changed()

    def mechanism_add_nasa9_cp(self, spec_name, Tmin, Tmax, coeffs):
        self._recorder().add_thermo(spec_name, SF_THERMO_NASA9, [Tmin, Tmax], nasa9=list(coeffs))
        self._mechanism_changed()

    def mechanism_add_reaction_simple(self, reactants_stoich, products_stoich, reversible, fwd_pre_exp_value,
                                      fwd_temp_exponent, fwd_act_energy):
        self._recorder().add_reaction(SF_RXN_SIMPLE, reactants_stoich, products_stoich, reversible,
                                      [fwd_pre_exp_value, fwd_temp_exponent, fwd_act_energy])
        self._mechanism_changed()

    def mechanism_add_reaction_three_body(self, reactants_stoich, products_stoich, reversible, fwd_pre_exp_value,
                                          fwd_temp_exponent, fwd_act_energy, three_body_efficiencies,
                                          default_efficiency):
        self._recorder().add_reaction(SF_RXN_THIRD_BODY, reactants_stoich, products_stoich, reversible,
                                      [fwd_pre_exp_value, fwd_temp_exponent, fwd_act_energy],
                                      efficiencies=three_body_efficiencies, default_eff=default_efficiency)
        self._mechanism_changed()

    def mechanism_add_reaction_Lindemann(self, reactants_stoich, products_stoich, reversible, fwd_pre_exp_value,
                                         fwd_temp_exponent, fwd_act_energy, three_body_efficiencies,
                                         default_efficiency, flf_pre_exp_value, flf_temp_exponent, flf_act_energy):
        self._recorder().add_reaction(SF_RXN_LINDEMANN, reactants_stoich, products_stoich, reversible,
                                      [fwd_pre_exp_value, fwd_temp_exponent, fwd_act_energy],
                                      kflf=[flf_pre_exp_value, flf_temp_exponent, flf_act_energy],
                                      efficiencies=three_body_efficiencies, default_eff=default_efficiency)
        self._mechanism_changed()

    def mechanism_add_reaction_Troe(self, reactants_stoich, products_stoich, reversible, fwd_pre_exp_value,
                                    fwd_temp_exponent, fwd_act_energy, three_body_efficiencies, default_efficiency,
                                    flf_pre_exp_value, flf_temp_exponent, flf_act_energy, troe_parameters):
        self._recorder().add_reaction(SF_RXN_TROE, reactants_stoich, products_stoich, reversible,
                                      [fwd_pre_exp_value, fwd_temp_exponent, fwd_act_energy],
                                      kflf=[flf_pre_exp_value, flf_temp_exponent, flf_act_energy],
                                      troe=troe_parameters, efficiencies=three_body_efficiencies,
                                      default_eff=default_efficiency)
        self._mechanism_changed()

    def mechanism_add_reaction_simple_with_special_orders(self, reactants_stoich, products_stoich, reversible,
                                                          fwd_pre_exp_value, fwd_temp_exponent, fwd_act_energy,
                                                          special_orders):
        self._recorder().add_reaction(SF_RXN_SIMPLE, reactants_stoich, products_stoich, reversible,
                                      [fwd_pre_exp_value, fwd_temp_exponent, fwd_act_energy],
                                      orders=special_orders)
        self._mechanism_changed()

    def mechanism_add_reaction_three_body_with_special_orders(self, reactants_stoich, products_stoich, reversible,
                                                              fwd_pre_exp_value, fwd_temp_exponent, fwd_act_energy,
                                                              three_body_efficiencies, default_efficiency,
                                                              special_orders):
        self._recorder().add_reaction(SF_RXN_THIRD_BODY, reactants_stoich, products_stoich, reversible,
                                      [fwd_pre_exp_value, fwd_temp_exponent, fwd_act_energy],
                                      efficiencies=three_body_efficiencies, default_eff=default_efficiency,
                                      orders=special_orders)
        self._mechanism_changed()

    def mechanism_add_reaction_Lindemann_with_special_orders(self, reactants_stoich, products_stoich, reversible,
                                                             fwd_pre_exp_value, fwd_temp_exponent, fwd_act_energy,
                                                             three_body_efficiencies, default_efficiency,
                                                             flf_pre_exp_value, flf_temp_exponent, flf_act_energy,
                                                             special_orders):
        self._recorder().add_reaction(SF_RXN_LINDEMANN, reactants_stoich, products_stoich, reversible,
                                      [fwd_pre_exp_value, fwd_temp_exponent, fwd_act_energy],
                                      kflf=[flf_pre_exp_value, flf_temp_exponent, flf_act_energy],
                                      efficiencies=three_body_efficiencies, default_eff=default_efficiency,
                                      orders=special_orders)
        self._mechanism_changed()

    def mechanism_add_reaction_Troe_with_special_orders(self, reactants_stoich, products_stoich, reversible,
                                                        fwd_pre_exp_value, fwd_temp_exponent, fwd_act_energy,
                                                        three_body_efficiencies, default_efficiency,
                                                        flf_pre_exp_value, flf_temp_exponent, flf_act_energy,
                                                        troe_parameters, special_orders):
        self._recorder().add_reaction(SF_RXN_TROE, reactants_stoich, products_stoich, reversible,
                                      [fwd_pre_exp_value, fwd_temp_exponent, fwd_act_energy],
                                      kflf=[flf_pre_exp_value, flf_temp_exponent, flf_act_energy],
                                      troe=troe_parameters, efficiencies=three_body_efficiencies,
                                      default_eff=default_efficiency, orders=special_orders)
        self._mechanism_changed()
