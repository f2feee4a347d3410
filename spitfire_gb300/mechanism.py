"""Mechanism loading and stream utilities: the GB300 build's ``ChemicalMechanismSpec``.

Spitfire's ``ChemicalMechanismSpec`` (``spitfire/chemistry/mechanism.py:53``) loads a Cantera input file through
Cantera, extracts species, NASA7 thermodynamics and reactions (``_extract_cantera_mechanism_data``,
``mechanism.py:388-541``) and feeds them to Griffon (``_populate_griffon_mechanism_data``, ``mechanism.py:122-258``).
Cantera is not available here, so this module reads the Cantera YAML files directly and produces the same
extracted data:

* element weights are Cantera's (H 1.008, O 15.999, N 14.007, Ar 39.95, He 4.002602, C 12.011), species
  molecular weights are their atom-weighted sums;
* species keep the order of the chosen phase;
* pre-exponential factors are taken as written (the files carry no ``units:`` block, so they are in Cantera's
  default kmol-m-s units); activation energies are converted to J/kmol (``cal/mol`` x 4184, ``kcal/mol`` x 4.184e6,
  ``J/mol`` x 1e3, ``K`` x R) and later divided by R, exactly as ``mechanism.py:191`` does;
* reactions are stably sorted simple -> three-body -> Lindemann -> Troe (``mechanism.py:540``); a reaction with
  an explicit collider (``H2 + AR <=> 2 H + AR``) stays *simple*;
* Troe parameters are ``[A, T3, T1, T2]`` with ``T2 = 0`` when absent, and T3, T1 pass through Cantera's
  reciprocal storage (``1/(1/T)``), which is what the Cantera-built gold files contain.

The loaded data are identical to the ``mech_data`` embedded in the reference's gold pickles for h2-burke
(checked by the tests).
"""

import re
import numpy as np

from . import yaml_subset

GAS_CONSTANT = 8314.46261815324  # J/kmol/K, Cantera's value (mechanism.py:135)
ONE_ATM = 101325.
REF_TEMPERATURE = 298.15  # mechanism.py:391

ELEMENT_WEIGHTS = {'H': 1.008, 'O': 15.999, 'N': 14.007, 'Ar': 39.95, 'He': 4.002602, 'C': 12.011,
                   'AR': 39.95, 'HE': 4.002602, 'S': 32.06, 'E': 5.485799090441e-4}

_EA_UNITS = {'J/kmol': 1.0, 'cal/mol': 4184.0, 'kcal/mol': 4184000.0, 'J/mol': 1000.0, 'kJ/mol': 1.0e6,
             'eV': 96485332.12331001}

RXN_TYPE_ORDER = {'simple': 0, 'three-body': 1, 'Lindemann': 2, 'Troe': 3}


def _activation_energy(value):
    """Convert a YAML activation energy (number or 'number unit') to J/kmol."""
    if isinstance(value, (int, float)):
        return float(value)
    tok = str(value).split()
    v = float(tok[0])
    unit = tok[1] if len(tok) > 1 else 'J/kmol'
    if unit == 'K':
        return v * GAS_CONSTANT
    if unit not in _EA_UNITS:
        raise ValueError(f'unsupported activation-energy unit "{unit}"')
    return v * _EA_UNITS[unit]


def _quantity(value):
    if isinstance(value, (int, float)):
        return float(value)
    return float(str(value).split()[0])


def _parse_side(text):
    """'2 H + O2 (+ M)' -> ({'H': 2, 'O2': 1}, collider) where collider is 'M', a species name, or None."""
    collider = None
    m = re.search(r'\(\s*\+\s*([^)\s]+)\s*\)', text)
    if m:
        collider = m.group(1)
        text = text[:m.start()] + text[m.end():]
    out = {}
    for term in text.split(' + '):
        term = term.strip()
        if not term:
            continue
        parts = term.split()
        if len(parts) == 2:
            coef, name = float(parts[0]), parts[1]
        else:
            coef, name = 1.0, parts[0]
        if name == 'M':
            collider = 'M'
            continue
        out[name] = out.get(name, 0.0) + coef
    return out, collider


def parse_equation(eq):
    if '<=>' in eq:
        lhs, rhs = eq.split('<=>')
        reversible = True
    elif '=>' in eq:
        lhs, rhs = eq.split('=>')
        reversible = False
    elif '=' in eq:
        lhs, rhs = eq.split('=')
        reversible = True
    else:
        raise ValueError(f'cannot parse reaction equation "{eq}"')
    reac, c1 = _parse_side(lhs)
    prod, c2 = _parse_side(rhs)
    return reac, prod, reversible, c1 or c2


def _troe_params(troe):
    """Troe parameters as Cantera reports them: [A, 1/(1/T3), 1/(1/T1), T2 or 0]."""
    a = float(troe['A'])
    t3 = float(troe['T3'])
    t1 = float(troe['T1'])
    t2 = float(troe.get('T2', 0.0))
    rt3 = float('inf') if abs(t3) < 1e-300 else 1.0 / t3
    rt1 = float('inf') if abs(t1) < 1e-300 else 1.0 / t1
    return [a, 1.0 / rt3 if rt3 != float('inf') else 0.0, 1.0 / rt1 if rt1 != float('inf') else 0.0, t2]


def load_cantera_yaml(path, group_name=None):
    """Read a Cantera YAML mechanism and return the data Spitfire extracts from Cantera.

    Returns a dict with keys element_mw_map, elements, ref_temperature, ref_pressure, species (ordered list of
    names), species_data ({name: {'atoms', 'heat-capacity'}}), reactions (type-sorted list of dicts in the
    format of ``_extract_cantera_mechanism_data``).
    """
    doc = yaml_subset.load(path)
    phases = doc['phases']
    if group_name is None:
        phase = phases[0]
    else:
        cands = [p for p in phases if p['name'] == group_name]
        if not cands:
            raise ValueError(f'phase "{group_name}" not found in {path}; available: {[p["name"] for p in phases]}')
        phase = cands[0]
    if 'units' in doc or 'units' in phase:
        raise ValueError('mechanisms with a units: block are not supported (Spitfire test files have none)')
    elements = list(phase['elements'])
    species_names = list(phase['species'])
    species_defs = {s['name']: s for s in doc['species']}
    species_data = {}
    for name in species_names:
        s = species_defs[name]
        th = s['thermo']
        model = th['model']
        if model == 'NASA7':
            tr = [float(t) for t in th['temperature-ranges']]
            data = th['data']
            if len(tr) == 2:  # single range: same polynomial both sides
                tr = [tr[0], tr[1], tr[1]]
                data = [data[0], data[0]]
            hc = {'type': 'NASA7', 'Tmin': tr[0], 'Tmid': tr[1], 'Tmax': tr[2],
                  'low-coeffs': np.array(data[0], dtype=np.float64),
                  'high-coeffs': np.array(data[1], dtype=np.float64)}
        elif model == 'constant-cp':
            hc = {'type': 'constant', 'Tmin': _quantity(th.get('T-min', 0.1)), 'Tmax': _quantity(th.get('T-max', 5000.)),
                  'T0': _quantity(th.get('T0', REF_TEMPERATURE)), 'h0': _quantity(th.get('h0', 0.)),
                  's0': _quantity(th.get('s0', 0.)), 'cp': _quantity(th.get('cp0', 0.))}
        elif model == 'NASA9':
            tr = [float(t) for t in th['temperature-ranges']]
            nreg = len(th['data'])
            coeffs = [float(nreg)]
            for k in range(nreg):
                coeffs += [tr[k], tr[k + 1]] + [float(c) for c in th['data'][k]]
            hc = {'type': 'NASA9', 'Tmin': tr[0], 'Tmax': tr[-1], 'coeffs': np.array(coeffs)}
        else:
            raise ValueError(f'unsupported thermo model {model} for species {name}')
        species_data[name] = {'atoms': {k: float(v) for k, v in s['composition'].items()}, 'heat-capacity': hc}

    rxn_entries = doc.get(phase.get('reactions', 'reactions') if isinstance(phase.get('reactions'), str)
                          and phase.get('reactions') not in ('all', 'none') else 'reactions') or []
    if phase.get('reactions') == 'none':
        rxn_entries = []
    sset = set(species_names)
    temp = []
    for rx in rxn_entries:
        reac, prod, reversible, collider = parse_equation(rx['equation'])
        if not (set(reac) <= sset and set(prod) <= sset):
            continue
        rtype = rx.get('type', 'elementary')
        eff = {k: float(v) for k, v in (rx.get('efficiencies') or {}).items() if k in sset}
        default_eff = float(rx.get('default-efficiency', 1.0))
        orders = {k: float(v) for k, v in (rx.get('orders') or {}).items()}
        if rtype == 'falloff':
            hi = rx['high-P-rate-constant']
            lo = rx['low-P-rate-constant']
            if collider not in (None, 'M'):
                eff = {collider: 1.0}
                default_eff = 0.0
            d = {'reversible': reversible, 'reactants': reac, 'products': prod, 'default-eff': default_eff,
                 'efficiencies': eff,
                 'fwd-A': _quantity(hi['A']), 'fwd-b': _quantity(hi['b']), 'fwd-Ea': _activation_energy(hi['Ea']),
                 'flf-A': _quantity(lo['A']), 'flf-b': _quantity(lo['b']), 'flf-Ea': _activation_energy(lo['Ea'])}
            if 'Troe' in rx:
                d['type'] = 'Troe'
                d['Troe-params'] = np.array(_troe_params(rx['Troe']))
                key = 3
            elif 'SRI' in rx:
                raise ValueError('SRI falloff is not supported by Griffon')
            else:
                d['type'] = 'Lindemann'
                key = 2
        elif rtype == 'three-body':
            rc = rx['rate-constant']
            d = {'type': 'three-body', 'reversible': reversible, 'reactants': reac, 'products': prod,
                 'default-eff': default_eff, 'efficiencies': eff,
                 'A': _quantity(rc['A']), 'b': _quantity(rc['b']), 'Ea': _activation_energy(rc['Ea'])}
            key = 1
        elif rtype in ('elementary', 'reaction'):
            rc = rx['rate-constant']
            d = {'type': 'simple', 'reversible': reversible, 'reactants': reac, 'products': prod,
                 'A': _quantity(rc['A']), 'b': _quantity(rc['b']), 'Ea': _activation_energy(rc['Ea'])}
            key = 0
        else:
            raise ValueError(f'unsupported reaction type "{rtype}" in: {rx["equation"]}')
        if orders:
            d['orders'] = orders
        d['yaml_index'] = len(temp)
        temp.append((key, d))
    reactions = [d for _, d in sorted(temp, key=lambda x: x[0])]
    element_mw_map = {e: ELEMENT_WEIGHTS[e] for e in elements}
    return dict(element_mw_map=element_mw_map, elements=elements, ref_temperature=REF_TEMPERATURE,
                ref_pressure=ONE_ATM, species=species_names, species_data=species_data, reactions=reactions)


def species_molecular_weight(atoms, element_mw_map):
    """Sum over atoms in std::map (sorted name) order, as Griffon's mechanism_add_species does
    (``chemistry_setup.cpp:52-56``)."""
    mw = 0.
    for a in sorted(atoms):
        mw += element_mw_map[a] * atoms[a]
    return mw


class Stream:
    """The part of a Cantera ``Quantity`` that Spitfire's reactor and flamelet front ends use.

    A stream holds T, p and composition (mass fractions) for one mechanism, plus an amount (mass) for mixing.
    Mass- and mole-fraction setters follow Cantera's conventions (compositions normalised, names case-sensitive
    except that ``stream(stp_air=True)`` uses 'o2:1 n2:3.74' as Spitfire does).
    """

    def __init__(self, mech, T=300., P=ONE_ATM, Y=None):
        self._mech = mech
        self._T = float(T)
        self._P = float(P)
        ns = mech.n_species
        self._Y = np.zeros(ns) if Y is None else np.array(Y, dtype=np.float64)
        if Y is None:
            self._Y[0] = 1.
        self.mass = 1.
        self.constant = 'HP'

    # --- composition parsing ---
    def _parse_comp(self, comp):
        ns = self._mech.n_species
        if isinstance(comp, str):
            v = np.zeros(ns)
            for item in re.split(r'[,\s]+', comp.strip()):
                if not item:
                    continue
                name, val = item.split(':')
                idx = self._mech._species_index_ci(name)
                v[idx] += float(val)
            return v
        if isinstance(comp, dict):
            v = np.zeros(ns)
            for name, val in comp.items():
                v[self._mech._species_index_ci(name)] += float(val)
            return v
        return np.array(comp, dtype=np.float64)

    @property
    def species_names(self):
        return self._mech.species_names

    def n_atoms(self, species, element):
        return self._mech._species_atoms[species].get(element, 0.)

    @property
    def T(self):
        return self._T

    @T.setter
    def T(self, v):
        self._T = float(v)

    @property
    def P(self):
        return self._P

    @P.setter
    def P(self, v):
        self._P = float(v)

    @property
    def Y(self):
        return self._Y.copy()

    @Y.setter
    def Y(self, comp):
        y = np.maximum(self._parse_comp(comp), 0.)
        self._Y = y / np.sum(y)

    @property
    def X(self):
        mw = self._mech.molecular_weights
        x = self._Y / mw
        return x / np.sum(x)

    @X.setter
    def X(self, comp):
        x = np.maximum(self._parse_comp(comp), 0.)
        x = x / np.sum(x)
        y = x * self._mech.molecular_weights
        self._Y = y / np.sum(y)

    @property
    def TP(self):
        return self._T, self._P

    @TP.setter
    def TP(self, v):
        self._T, self._P = float(v[0]), float(v[1])

    @property
    def TPX(self):
        return self._T, self._P, self.X

    @TPX.setter
    def TPX(self, v):
        self.TP = v[:2]
        self.X = v[2]

    @property
    def TPY(self):
        return self._T, self._P, self.Y

    @TPY.setter
    def TPY(self, v):
        self.TP = v[:2]
        self.Y = v[2]

    @property
    def mean_molecular_weight(self):
        return 1. / np.sum(self._Y / self._mech.molecular_weights)

    @property
    def density(self):
        return self._P * self.mean_molecular_weight / (GAS_CONSTANT * self._T)

    @property
    def enthalpy_mass(self):
        return float(np.dot(self._mech.species_enthalpies_host(self._T), self._Y))

    @property
    def cp_mass(self):
        return float(np.dot(self._mech.species_cp_host(self._T), self._Y))

    @property
    def HP(self):
        return self.enthalpy_mass, self._P

    @HP.setter
    def HP(self, v):
        h, p = float(v[0]), float(v[1])
        self._P = p
        self._T = self._mech.temperature_from_enthalpy(h, self._Y, self._T)

    def __add__(self, other):
        """Adiabatic, isobaric mass-weighted mixing (Cantera Quantity addition with constant='HP')."""
        m1, m2 = self.mass, other.mass
        y = (m1 * self._Y + m2 * other._Y) / (m1 + m2)
        h = (m1 * self.enthalpy_mass + m2 * other.enthalpy_mass) / (m1 + m2)
        out = Stream(self._mech, self._T, self._P, y)
        out.mass = m1 + m2
        out.HP = h, self._P
        return out

    def __radd__(self, other):
        if other == 0:
            return self
        return self.__add__(other)


class ChemicalMechanismSpec:
    """Drop-in for ``spitfire.chemistry.mechanism.ChemicalMechanismSpec`` (``mechanism.py:53-757``).

    ``ChemicalMechanismSpec(cantera_input='h2-burke.yaml', group_name='h2-burke')`` loads the mechanism with the
    project loader and builds a GPU-backed Griffon object (``.griffon``) whose methods keep the names and argument
    order of ``spitfire.griffon.griffon.PyCombustionKernels``.
    """

    def __init__(self, cantera_input=None, group_name='gas', cantera_solution=None, cantera_xml=None,
                 mech_data=None):
        from .griffon import PyCombustionKernels
        if cantera_xml is not None and cantera_input is None:
            cantera_input = cantera_xml
        self._element_stoichiometry = {'O': -1.0, 'H': 0.5, 'C': 2.0, 'Al': 1.5, 'U': 1.0, 'Ar': 0.0, 'N': 0.0,
                                       'He': 0.0}
        if mech_data is not None:
            self._init_from_mech_data(mech_data)
        else:
            if cantera_input is None:
                raise ValueError('ChemicalMechanismSpec needs cantera_input (a Cantera YAML file)')
            gname = group_name
            doc_phases = None
            try:
                ext = load_cantera_yaml(cantera_input, gname)
            except ValueError:
                if gname == 'gas':
                    ext = load_cantera_yaml(cantera_input, None)
                else:
                    raise
            self._file = cantera_input
            self._group = gname
            self._ext = ext
            self._build_mech_data()
        self._griffon = PyCombustionKernels()
        self._populate_griffon(self._griffon)

    # ---------------------------------------------------------------------------------------------------------
    def _build_mech_data(self):
        ext = self._ext
        md = dict(ref_pressure=ext['ref_pressure'], ref_temperature=ext['ref_temperature'],
                  gas_constant=GAS_CONSTANT, element_mw_map=dict(ext['element_mw_map']),
                  elements=list(ext['elements']), species=dict(), reactions=list(), **{'transport-model': None})
        for s in ext['species']:
            sd = ext['species_data'][s]
            cp = sd['heat-capacity']
            md['species'][s] = {'atom_map': dict(sd['atoms'])}
            if cp['type'] == 'NASA7':
                md['species'][s]['cp'] = ('NASA7', cp['Tmin'], cp['Tmid'], cp['Tmax'], cp['low-coeffs'].tolist(),
                                          cp['high-coeffs'].tolist())
            elif cp['type'] == 'constant':
                md['species'][s]['cp'] = ('constant', cp['Tmin'], cp['Tmax'], cp['T0'], cp['h0'], cp['s0'], cp['cp'])
            elif cp['type'] == 'NASA9':
                md['species'][s]['cp'] = ('NASA9', cp['Tmin'], cp['Tmax'], cp['coeffs'].tolist())
        for rx in ext['reactions']:
            t = rx['type']
            sp = '-special' if 'orders' in rx else ''
            if t == 'simple':
                tup = ('simple' + sp, rx['reactants'], rx['products'], rx['reversible'], rx['A'], rx['b'], rx['Ea'])
            elif t == 'three-body':
                tup = ('three-body' + sp, rx['reactants'], rx['products'], rx['reversible'], rx['A'], rx['b'],
                       rx['Ea'], rx['efficiencies'], rx['default-eff'])
            elif t == 'Lindemann':
                tup = ('Lindemann' + sp, rx['reactants'], rx['products'], rx['reversible'], rx['fwd-A'],
                       rx['fwd-b'], rx['fwd-Ea'], rx['efficiencies'], rx['default-eff'], rx['flf-A'], rx['flf-b'],
                       rx['flf-Ea'])
            else:
                tup = ('Troe' + sp, rx['reactants'], rx['products'], rx['reversible'], rx['fwd-A'], rx['fwd-b'],
                       rx['fwd-Ea'], rx['efficiencies'], rx['default-eff'], rx['flf-A'], rx['flf-b'], rx['flf-Ea'],
                       rx['Troe-params'].tolist())
            if sp:
                tup = tup + (rx['orders'],)
            md['reactions'].append(tup)
        self._reaction_yaml_index = [rx['yaml_index'] for rx in ext['reactions']]
        self._mech_data = md
        self._species_names = list(ext['species'])
        self._finish_species()

    def _init_from_mech_data(self, md):
        """Rebuild from a ``mech_data`` dict (the pickled form, ``mechanism.py:108-115``)."""
        self._mech_data = md
        self._species_names = list(md['species'].keys())
        self._file = None
        self._group = None
        self._finish_species()

    def _finish_species(self):
        md = self._mech_data
        emw = md['element_mw_map']
        self._species_atoms = {s: dict(md['species'][s]['atom_map']) for s in self._species_names}
        self._mw = np.array([species_molecular_weight(self._species_atoms[s], emw) for s in self._species_names])
        self._sidx = {s: i for i, s in enumerate(self._species_names)}
        self._sidx_ci = {s.lower(): i for i, s in enumerate(self._species_names)}
        # host-side NASA7 arrays for stream utilities (not the hot path)
        ns = len(self._species_names)
        self._nasa = np.zeros((ns, 3 + 14))
        self._thermo_kind = []
        for i, s in enumerate(self._species_names):
            cp = md['species'][s]['cp']
            self._thermo_kind.append(cp[0])
            if cp[0] == 'NASA7':
                self._nasa[i, 0:3] = [cp[1], cp[2], cp[3]]
                self._nasa[i, 3:10] = cp[4]
                self._nasa[i, 10:17] = cp[5]

    def _populate_griffon(self, g):
        """Same sequence of setter calls as ``_populate_griffon_mechanism_data`` (mechanism.py:122-258)."""
        md = self._mech_data
        g.mechanism_set_ref_pressure(md['ref_pressure'])
        g.mechanism_set_ref_temperature(md['ref_temperature'])
        g.mechanism_set_gas_constant(md['gas_constant'])
        g.mechanism_set_element_mw_map(md['element_mw_map'])
        for e in md['elements']:
            g.mechanism_add_element(e)
        for s in self._species_names:
            g.mechanism_add_species(s, md['species'][s]['atom_map'])
        g.mechanism_resize_heat_capacity_data()
        for s in self._species_names:
            cp = md['species'][s]['cp']
            if cp[0] == 'NASA7':
                g.mechanism_add_nasa7_cp(s, cp[1], cp[2], cp[3], list(cp[4]), list(cp[5]))
            elif cp[0] == 'constant':
                g.mechanism_add_const_cp(s, *cp[1:])
            elif cp[0] == 'NASA9':
                g.mechanism_add_nasa9_cp(s, cp[1], cp[2], list(cp[3]))
        R = md['gas_constant']
        for rx in md['reactions']:
            kind = rx[0]
            if kind == 'simple':
                g.mechanism_add_reaction_simple(rx[1], rx[2], rx[3], rx[4], rx[5], rx[6] / R)
            elif kind == 'simple-special':
                g.mechanism_add_reaction_simple_with_special_orders(rx[1], rx[2], rx[3], rx[4], rx[5], rx[6] / R,
                                                                    rx[7])
            elif kind == 'three-body':
                g.mechanism_add_reaction_three_body(rx[1], rx[2], rx[3], rx[4], rx[5], rx[6] / R, rx[7], rx[8])
            elif kind == 'three-body-special':
                g.mechanism_add_reaction_three_body_with_special_orders(rx[1], rx[2], rx[3], rx[4], rx[5],
                                                                        rx[6] / R, rx[7], rx[8], rx[9])
            elif kind == 'Lindemann':
                g.mechanism_add_reaction_Lindemann(rx[1], rx[2], rx[3], rx[4], rx[5], rx[6] / R, rx[7], rx[8],
                                                   rx[9], rx[10], rx[11] / R)
            elif kind == 'Lindemann-special':
                g.mechanism_add_reaction_Lindemann_with_special_orders(rx[1], rx[2], rx[3], rx[4], rx[5], rx[6] / R,
                                                                       rx[7], rx[8], rx[9], rx[10], rx[11] / R,
                                                                       rx[12])
            elif kind == 'Troe':
                g.mechanism_add_reaction_Troe(rx[1], rx[2], rx[3], rx[4], rx[5], rx[6] / R, rx[7], rx[8], rx[9],
                                              rx[10], rx[11] / R, list(rx[12]))
            elif kind == 'Troe-special':
                g.mechanism_add_reaction_Troe_with_special_orders(rx[1], rx[2], rx[3], rx[4], rx[5], rx[6] / R,
                                                                  rx[7], rx[8], rx[9], rx[10], rx[11] / R,
                                                                  list(rx[12]), rx[13])
            else:
                raise ValueError(f'unknown reaction kind {kind}')

    # --- JSON form of mech_data (bundled mechanisms, spitfire_gb300/data) ---
    def mech_data_json(self):
        md = dict(self._mech_data)
        md['species_order'] = list(self._species_names)
        md['reaction_yaml_index'] = [int(i) for i in self.reaction_yaml_index]
        md['element_mw_map'] = {k: float(v) for k, v in md['element_mw_map'].items()}
        md['species'] = {s: {'atom_map': v['atom_map'], 'cp': [float(c) if not isinstance(c, (str, list)) else c
                                                                 for c in v['cp']]}
                         for s, v in md['species'].items()}
        md['reactions'] = [list(r) for r in md['reactions']]
        return md

    @classmethod
    def from_json(cls, path):
        import json
        with open(path) as f:
            md = json.load(f)
        order = md.pop('species_order')
        yaml_index = md.pop('reaction_yaml_index', None)
        md['species'] = {s: {'atom_map': md['species'][s]['atom_map'], 'cp': tuple(md['species'][s]['cp'])}
                         for s in order}
        md['reactions'] = [tuple(r) for r in md['reactions']]
        spec = cls(mech_data=md)
        if yaml_index is not None:
            spec._reaction_yaml_index = list(yaml_index)
        return spec

    @classmethod
    def bundled(cls, name):
        """A mechanism shipped in spitfire_gb300/data (h2-burke, methane-gri30, reaction-test, unit-*)."""
        import os
        return cls.from_json(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'data', name + '.json'))

    # --- pickling as in mechanism.py:108-115 ---
    def __getstate__(self):
        return dict({'mech_data': self._mech_data, 'element_stoichiometry': self._element_stoichiometry})

    def __setstate__(self, state):
        self.__init__(mech_data=state['mech_data'])
        if 'element_stoichiometry' in state:
            self._element_stoichiometry = state['element_stoichiometry']

    # --- properties ---
    @property
    def mech_data(self):
        return self._mech_data

    @property
    def element_stoichiometry(self):
        return self._element_stoichiometry

    @element_stoichiometry.setter
    def element_stoichiometry(self, v):
        if v is not None:
            self._element_stoichiometry = v

    @property
    def griffon(self):
        return self._griffon

    @property
    def reaction_yaml_index(self):
        """Position in the mechanism file of each reaction, in the internal order (reactions are stably sorted
        simple, three-body, Lindemann, Troe as the reference does, mechanism.py:540); identity when the mechanism
        was built from a mech_data dict without file order."""
        idx = getattr(self, '_reaction_yaml_index', None)
        return np.array(idx if idx is not None else range(len(self._mech_data['reactions'])), dtype=np.int64)

    @property
    def mech_file_path(self):
        return self._file

    @property
    def group_name(self):
        return self._group

    @property
    def n_species(self):
        return len(self._species_names)

    @property
    def n_reactions(self):
        return len(self._mech_data['reactions'])

    @property
    def species_names(self):
        return list(self._species_names)

    @property
    def element_names(self):
        return list(self._mech_data['elements'])

    def species_index(self, name):
        return self._sidx[name]

    def _species_index_ci(self, name):
        if name in self._sidx:
            return self._sidx[name]
        return self._sidx_ci[name.lower()]

    @property
    def molecular_weights(self):
        return self._mw.copy()

    def molecular_weight(self, ni):
        if isinstance(ni, str):
            return self._mw[self._sidx[ni]]
        if isinstance(ni, (int, np.integer)):
            return self._mw[ni]
        raise TypeError('ChemicalMechanismSpec.molecular_weight(ni) takes a string or integer, given ' + str(ni))

    # --- host-side thermo for stream utilities (NASA7) ---
    def species_cp_host(self, T):
        cp = np.zeros(self.n_species)
        for i in range(self.n_species):
            tmin, tmid, tmax = self._nasa[i, 0:3]
            t = min(max(T, tmin), tmax)
            a = self._nasa[i, 3:10] if t <= tmid else self._nasa[i, 10:17]
            cp[i] = GAS_CONSTANT * (a[0] + t * (a[1] + t * (a[2] + t * (a[3] + t * a[4])))) / self._mw[i]
        return cp

    def species_enthalpies_host(self, T):
        h = np.zeros(self.n_species)
        for i in range(self.n_species):
            tmin, tmid, tmax = self._nasa[i, 0:3]
            t = min(max(T, tmin), tmax)
            a = self._nasa[i, 3:10] if t <= tmid else self._nasa[i, 10:17]
            hh = GAS_CONSTANT * t * (a[0] + t * (a[1] / 2 + t * (a[2] / 3 + t * (a[3] / 4 + t * a[4] / 5))) + a[5] / t)
            if T != t:
                hh += GAS_CONSTANT * (a[0] + t * (a[1] + t * (a[2] + t * (a[3] + t * a[4])))) * (T - t)
            h[i] = hh / self._mw[i]
        return h

    def species_h_cp_host_vec(self, T):
        """Species enthalpies and heat capacities (J/kg, J/kg/K) at an array of temperatures: [n, ns] each, the
        same clipped-range NASA7 evaluation as species_enthalpies_host / species_cp_host."""
        T = np.asarray(T, dtype=np.float64)[:, None]
        tmin, tmid, tmax = self._nasa[:, 0], self._nasa[:, 1], self._nasa[:, 2]
        t = np.minimum(np.maximum(T, tmin[None, :]), tmax[None, :])
        a = np.where((t <= tmid[None, :])[:, :, None], self._nasa[None, :, 3:10], self._nasa[None, :, 10:17])
        cpr = a[..., 0] + t * (a[..., 1] + t * (a[..., 2] + t * (a[..., 3] + t * a[..., 4])))
        hh = GAS_CONSTANT * t * (a[..., 0] + t * (a[..., 1] / 2 + t * (a[..., 2] / 3 + t * (a[..., 3] / 4 + t *
                                                                                            a[..., 4] / 5))) +
                                 a[..., 5] / t)
        hh = hh + np.where(T != t, GAS_CONSTANT * cpr * (T - t), 0.)
        return hh / self._mw[None, :], GAS_CONSTANT * cpr / self._mw[None, :]

    def temperature_from_enthalpy_vec(self, h, Y, T_guess=1000.):
        """temperature_from_enthalpy for arrays of enthalpies h[n] and mass fractions Y[n, ns]."""
        h = np.asarray(h, dtype=np.float64)
        T = np.full(h.shape, float(T_guess))
        done = np.zeros(h.shape, dtype=bool)
        for _ in range(100):
            hs, cps = self.species_h_cp_host_vec(T)
            dT = -((hs * Y).sum(1) - h) / (cps * Y).sum(1)
            T = np.where(done, T, T + dT)
            done |= np.abs(dT) < 1e-10 * T
            if done.all():
                break
        return T

    def temperature_from_enthalpy(self, h, Y, T_guess=1000.):
        T = float(T_guess)
        for _ in range(100):
            f = np.dot(self.species_enthalpies_host(T), Y) - h
            cp = np.dot(self.species_cp_host(T), Y)
            dT = -f / cp
            T += dT
            if abs(dT) < 1e-10 * T:
                break
        return T

    # --- streams (mechanism.py:562-757) ---
    def stream(self, properties=None, values=None, stp_air=False):
        q = Stream(self)
        if stp_air:
            q.TPX = 300., ONE_ATM, 'o2:1 n2:3.74'
        else:
            if properties is None:
                raise ValueError('ChemicalMechanismSpec.stream() was called improperly: use stream(stp_air=True) '
                                 'or stream(properties, values)')
            if values is None:
                raise ValueError('ChemicalMechanismSpec.stream() expects two arguments if properties are set')
            setattr(q, properties, values)
        return q

    def copy_stream(self, stream):
        q = Stream(self)
        q.TPX = stream.TPX
        return q

    @staticmethod
    def mix_streams(streams, basis, constant='HP'):
        if constant != 'HP':
            raise ValueError('only constant="HP" mixing is supported')
        q_list = []
        for stream, amount in streams:
            if basis == 'mass':
                stream.mass = amount
            elif basis == 'mole':
                stream.mass = amount * stream.mean_molecular_weight
            q_list.append(stream)
        mix = q_list[0]
        for q in q_list[1:]:
            mix = mix + q
        return mix

    def _o2_required(self, X):
        """Moles of O2 needed to burn the mixture X (C->CO2, H->H2O, S->SO2) minus the O2 it carries."""
        req = 0.
        coef = {'C': 1.0, 'H': 0.25, 'S': 1.0, 'O': -0.5}
        for i, s in enumerate(self._species_names):
            for e, n in self._species_atoms[s].items():
                req += X[i] * n * coef.get(e, 0.)
        return req

    def mix_for_equivalence_ratio(self, phi, fuel, oxy):
        """Mixture at equivalence ratio phi on a mole basis (Cantera's set_equivalence_ratio)."""
        xf = fuel.X
        xo = oxy.X
        of = self._o2_required(xf)
        oo = self._o2_required(xo)
        if of <= 0 or oo > 0:
            raise ValueError('fuel/oxidizer streams cannot be combusted to the requested equivalence ratio')
        ratio = phi * (-oo / of)
        x = ratio * xf + xo
        q = Stream(self, fuel.T, fuel.P)
        q.X = x / np.sum(x)
        return q

    def mix_for_normalized_equivalence_ratio(self, normalized_phi, fuel, oxy):
        return self.mix_for_equivalence_ratio(normalized_phi / (1. - normalized_phi), fuel, oxy)

    def _get_atoms_in_stream(self, stream, atom_names):
        atoms = {a: 0. for a in atom_names}
        X = stream.X
        for i, s in enumerate(self._species_names):
            for a in atom_names:
                atoms[a] += X[i] * self._species_atoms[s].get(a, 0.)
        return atoms

    def stoich_molar_fuel_to_oxy_ratio(self, fuel_stream, oxy_stream):
        present = self.element_names
        for atom in present:
            if atom not in self._element_stoichiometry:
                raise KeyError(f'atom "{atom}" is not present in the element stoichiometry map')
        atom_names = [a for a in self._element_stoichiometry if a in present]
        fa = self._get_atoms_in_stream(fuel_stream, atom_names)
        oa = self._get_atoms_in_stream(oxy_stream, atom_names)
        return -sum([self._element_stoichiometry[a] * oa[a] for a in atom_names]) / \
            sum([self._element_stoichiometry[a] * fa[a] for a in atom_names])

    def stoich_mass_fuel_to_oxy_ratio(self, fuel_stream, oxy_stream):
        return fuel_stream.mean_molecular_weight / oxy_stream.mean_molecular_weight * \
            self.stoich_molar_fuel_to_oxy_ratio(fuel_stream, oxy_stream)

    def stoich_mixture_fraction(self, fuel_stream, oxy_stream):
        eta = self.stoich_mass_fuel_to_oxy_ratio(fuel_stream, oxy_stream)
        return eta / (1. + eta)

    def mix_fuels_for_stoich_mixture_fraction(self, fuel1, fuel2, zstoich, oxy):
        """Mole-basis mix of two fuel streams whose stoichiometric mixture fraction with `oxy` is zstoich
        (mechanism.py:724-757), e.g. a fuel diluted with nitrogen; hydrocarbon oxidation (C -> CO2, H -> H2O).

        With k moles of fuel1 and 1 - k of fuel2, the oxygen atoms the fuel needs per mole are k n1 + (1 - k) n2
        (n = 2 C + H/2 - O), the oxidizer brings e = O - H/2 - 2 C per mole, and the stoichiometric fuel-to-oxidizer
        mass ratio zstoich / (1 - zstoich) equals (k M1 + (1 - k) M2) e / (M_oxy (k n1 + (1 - k) n2)); that is
        linear in k. Raises ValueError when no k in [0, 1] reaches zstoich."""
        names = ['H', 'O', 'C']
        a = self._get_atoms_in_stream(fuel1, names)
        b = self._get_atoms_in_stream(fuel2, names)
        x = self._get_atoms_in_stream(oxy, names)
        need = lambda c: 2. * c['C'] + 0.5 * c['H'] - c['O']
        n1, n2, e = need(a), need(b), -need(x)
        m1, m2, mx = fuel1.mean_molecular_weight, fuel2.mean_molecular_weight, oxy.mean_molecular_weight
        lhs = mx / e * zstoich / (1. - zstoich)  # fuel molar mass per unit oxygen demand at stoichiometry
        k = (m2 - lhs * n2) / (lhs * (n1 - n2) - (m1 - m2))
        if not 0. <= k <= 1.:
            raise ValueError('The provided fuel combination cannot reach the desired stoichiometric mixture fraction!')
        return self.mix_streams([(fuel1, k), (fuel2, 1. - k)], 'mole')
