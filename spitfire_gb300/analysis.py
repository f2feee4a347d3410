"""Library post-processing used with the flamelet libraries: the mass-specific mixture enthalpy of every state of a
library (spitfire/chemistry/analysis.py:77-98 computes it with Cantera's enthalpy_mass; here from the mechanism's
own NASA7 polynomials, the same functions)."""

import numpy as np


def compute_specific_enthalpy(mechanism, output_library):
    """Adds 'enthalpy' (J/kg) from the library's temperature and mass fractions; returns the library."""
    names = mechanism.species_names
    T = np.asarray(output_library['temperature'], dtype=np.float64)
    Y = np.stack([np.asarray(output_library['mass fraction ' + n], dtype=np.float64) for n in names], axis=-1)
    hs, _ = mechanism.species_h_cp_host_vec(T.ravel())
    output_library['enthalpy'] = (hs * Y.reshape(-1, len(names))).sum(1).reshape(T.shape)
    return output_library
