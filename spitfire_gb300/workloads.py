"""Seeded synthetic inputs of the benchmark workloads (numpy.random.default_rng, one seed per workload).

There is no public benchmark for this path; states are drawn as follows.
* H2 states: h2-burke, T ~ U(800, 2500) K, p = 1 atm, Y = 0.5 Dir(0.5) over the nine named species
  (H2, O2, H2O, H, O, OH, HO2, H2O2, N2) + 0.5 e_N2, AR = HE = 0; isochoric state [rho, T, Y_0..Y_{ns-2}].
* GRI states (the batched RHS + Jacobian workload): methane-gri30, T ~ U(600, 2800) K,
  p = 101325 exp(U(0, ln 40)) Pa, Y = 0.7 Dir(1 over 53) + 0.3 Y_maj(phi), phi ~ U(0.5, 2), where Y_maj is the
  complete-combustion product of CH4/air at phi (lean: CO2, H2O, N2, O2 excess; rich: CO2, CO, H2O, H2, N2 with the carbon and hydrogen deficit
  split 1:1 between CO and H2); Newton factor gamma*h = exp(U(ln 1e-9, ln 1e-5)) s.
* Ignition batch: isobaric CH4/air, T0 ~ U(900, 1500) K, phi ~ U(0.5, 2), p = 101325 exp(U(0, ln 20)).
* Adjoint batch: isobaric CH4/air, T0 ~ U(1000, 1400) K, phi ~ U(0.7, 1.5), p = 10 atm, t_end = 5e-3 s.
* Steady flamelets: GRI-3.0, oxidizer air 300 K (O2:N2 = 1:3.76 molar), fuel CH4 300 K, 1 atm;
  64 stoichiometric dissipation rates log-spaced 1e-2 - 1e3 1/s (Peters profile); flamelet k has a grid of
  nz_k = 64 + floor(192 k / 63) points clustered at the stoichiometric mixture fraction (intensity 4), the grid
  sizes assigned to the dissipation rates by a seeded permutation; Burke-Schumann initial profiles.
"""

import numpy as np

from .mechanism import GAS_CONSTANT, ChemicalMechanismSpec

H2_NAMED = ['H2', 'O2', 'H2O', 'H', 'O', 'OH', 'HO2', 'H2O2', 'N2']


def h2_states(mech: ChemicalMechanismSpec, n, seed=1001):
    rng = np.random.default_rng(seed)
    ns = mech.n_species
    T = rng.uniform(800., 2500., n)
    idx = [mech.species_index(s) for s in H2_NAMED]
    Y = np.zeros((n, ns))
    Y[:, idx] = 0.5 * rng.dirichlet(0.5 * np.ones(len(idx)), n)
    Y[:, mech.species_index('N2')] += 0.5
    Y /= Y.sum(1, keepdims=True)
    p = np.full(n, 101325.)
    mmw = 1. / (Y / mech.molecular_weights).sum(1)
    rho = p * mmw / (GAS_CONSTANT * T)
    return dict(T=T, p=p, Y=Y, rho=rho)


def _major_products(mech, phi):
    """Complete-combustion mass fractions of CH4/air (O2:N2 = 1:3.76) at equivalence ratio phi."""
    mw = {s: mech.molecular_weight(s) for s in ('CH4', 'O2', 'N2', 'CO2', 'H2O', 'CO', 'H2')}
    n_o2 = 2. / phi
    n_n2 = 3.76 * n_o2
    moles = {'N2': n_n2}
    if phi <= 1.:
        moles.update(CO2=1., H2O=2., O2=n_o2 - 2.)
    else:
        # oxygen deficit d (O atoms) shared by CO (one O less than CO2) and H2 (one O less than H2O), 1:1
        d = 2. * (2. - n_o2)  # O atoms missing relative to complete combustion
        co = min(d / 2., 1.)
        h2 = min(d - co, 2.)
        moles.update(CO2=1. - co, CO=co, H2O=2. - h2, H2=h2)
    Y = np.zeros(mech.n_species)
    for s, v in moles.items():
        Y[mech.species_index(s)] = max(v, 0.) * mw[s]
    return Y / Y.sum()


def gri_states(mech: ChemicalMechanismSpec, n, seed=1002):
    rng = np.random.default_rng(seed)
    ns = mech.n_species
    T = rng.uniform(600., 2800., n)
    p = 101325. * np.exp(rng.uniform(0., np.log(40.), n))
    phi = rng.uniform(0.5, 2.0, n)
    D = rng.dirichlet(np.ones(ns), n)
    Ymaj = np.array([_major_products(mech, f) for f in phi])
    Y = 0.7 * D + 0.3 * Ymaj
    Y /= Y.sum(1, keepdims=True)
    mmw = 1. / (Y / mech.molecular_weights).sum(1)
    rho = p * mmw / (GAS_CONSTANT * T)
    gh = np.exp(rng.uniform(np.log(1e-9), np.log(1e-5), n))
    return dict(T=T, p=p, Y=Y, rho=rho, phi=phi, gamma_h=gh)


def isochoric_state(d):
    """[rho, T, Y_0..Y_{ns-2}] rows."""
    return np.hstack([d['rho'][:, None], d['T'][:, None], d['Y'][:, :-1]])


def isobaric_state(d):
    """[T, Y_0..Y_{ns-2}] rows."""
    return np.hstack([d['T'][:, None], d['Y'][:, :-1]])


def ch4_air_mixture(mech: ChemicalMechanismSpec, phi):
    """Mass fractions of CH4/air (O2:N2 = 1:3.76 molar) at equivalence ratio phi."""
    X = np.zeros(mech.n_species)
    X[mech.species_index('CH4')] = phi
    X[mech.species_index('O2')] = 2.
    X[mech.species_index('N2')] = 2. * 3.76
    Y = X * mech.molecular_weights
    return Y / Y.sum()


def ignition_batch(mech: ChemicalMechanismSpec, n, seed=1003, T_range=(900., 1500.), phi_range=(0.5, 2.0),
                   p_log_range=(1., 20.)):
    rng = np.random.default_rng(seed)
    T0 = rng.uniform(*T_range, n)
    phi = rng.uniform(*phi_range, n)
    p = 101325. * np.exp(rng.uniform(np.log(p_log_range[0]), np.log(p_log_range[1]), n))
    Y = np.array([ch4_air_mixture(mech, f) for f in phi])
    q0 = np.hstack([T0[:, None], Y[:, :-1]])
    return dict(T0=T0, phi=phi, p=p, Y=Y, q0=q0)


def slfm_flamelet_setups(mech: ChemicalMechanismSpec, n=64, seed=1004, chi_range=(1e-2, 1e3), nz_range=(64, 256)):
    """FlameletSetup objects of the steady-flamelet workload (see the module docstring)."""
    from .flamelet import FlameletSetup, FlameletSpec
    rng = np.random.default_rng(seed)
    air = mech.stream('TPX', (300., 101325., 'O2:1 N2:3.76'))
    fuel = mech.stream('TPX', (300., 101325., 'CH4:1'))
    chis = np.logspace(np.log10(chi_range[0]), np.log10(chi_range[1]), n)
    span = nz_range[1] - nz_range[0]
    nz = np.array([nz_range[0] + (span * k) // max(n - 1, 1) for k in range(n)])
    nz = nz[rng.permutation(n)]
    out = []
    for k in range(n):
        fs = FlameletSpec(mech_spec=mech, oxy_stream=air, fuel_stream=fuel, grid_points=int(nz[k]),
                          grid_type='clustered', grid_cluster_intensity=4., grid_cluster_point='stoichiometric',
                          stoich_dissipation_rate=float(chis[k]), initial_condition='Burke-Schumann')
        out.append(FlameletSetup(fs))
    return out


def adjoint_batch(mech: ChemicalMechanismSpec, n, seed=1005):
    """Reactors of the adjoint workload: isobaric CH4/air, T0 ~ U(1000, 1400) K, phi ~ U(0.7, 1.5), p = 10 atm."""
    return ignition_batch(mech, n, seed=seed, T_range=(1000., 1400.), phi_range=(0.7, 1.5), p_log_range=(10., 10.))
