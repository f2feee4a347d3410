"""Library post-processing used with the flamelet libraries (spitfire/chemistry/analysis.py:77-217, which computes
these with Cantera): the mass-specific mixture enthalpy, isobaric and isochoric heat capacities, ideal-gas density
and pressure of every state of a library, from the mechanism's own NASA7 polynomials and molecular weights (the
same functions Cantera evaluates). Viscosity needs transport data and Cantera, and is not provided."""

import numpy as np

_R = 8314.46261815324  # J/(kmol K), the universal gas constant in the units of the mechanism data


def _T_Y(mechanism, output_library):
    names = mechanism.species_names
    T = np.asarray(output_library['temperature'], dtype=np.float64)
    Y = np.stack([np.asarray(output_library['mass fraction ' + n], dtype=np.float64) for n in names], axis=-1)
    return T, Y.reshape(-1, len(names))


def _inverse_molar_mass(mechanism, Y):
    return (Y / np.asarray(mechanism.molecular_weights, dtype=np.float64)[None, :]).sum(1)


def compute_specific_enthalpy(mechanism, output_library):
    """Adds 'enthalpy' (J/kg) from the library's temperature and mass fractions; returns the library."""
    names = mechanism.species_names
    T = np.asarray(output_library['temperature'], dtype=np.float64)
    Y = np.stack([np.asarray(output_library['mass fraction ' + n], dtype=np.float64) for n in names], axis=-1)
    hs, _ = mechanism.species_h_cp_host_vec(T.ravel())
    output_library['enthalpy'] = (hs * Y.reshape(-1, len(names))).sum(1).reshape(T.shape)
    return output_library


def compute_isobaric_specific_heat(mechanism, output_library):
    """Adds 'heat capacity cp' (J/(kg K)), sum_i Y_i cp_i(T) (analysis.py:173-194); returns the library."""
    T, Y = _T_Y(mechanism, output_library)
    _, cps = mechanism.species_h_cp_host_vec(T.ravel())
    output_library['heat capacity cp'] = (cps * Y).sum(1).reshape(T.shape)
    return output_library


def compute_isochoric_specific_heat(mechanism, output_library):
    """Adds 'heat capacity cv' (J/(kg K)), cp - R / M of the mixture (analysis.py:197-218); returns the library."""
    T, Y = _T_Y(mechanism, output_library)
    _, cps = mechanism.species_h_cp_host_vec(T.ravel())
    output_library['heat capacity cv'] = ((cps * Y).sum(1) - _R * _inverse_molar_mass(mechanism, Y)).reshape(T.shape)
    return output_library


def compute_density(mechanism, output_library):
    """Adds 'density' (kg/m^3), the ideal-gas density at the library's pressure (analysis.py:101-122)."""
    T, Y = _T_Y(mechanism, output_library)
    p = np.asarray(output_library['pressure'], dtype=np.float64).ravel()
    output_library['density'] = (p / (_R * T.ravel() * _inverse_molar_mass(mechanism, Y))).reshape(T.shape)
    return output_library


def compute_pressure(mechanism, output_library):
    """Adds 'pressure' (Pa), the ideal-gas pressure at the library's density (analysis.py:125-146)."""
    T, Y = _T_Y(mechanism, output_library)
    rho = np.asarray(output_library['density'], dtype=np.float64).ravel()
    output_library['pressure'] = (rho * _R * T.ravel() * _inverse_molar_mass(mechanism, Y)).reshape(T.shape)
    return output_library
