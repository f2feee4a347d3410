"""Flamelet golden cases shared by tests/golden/make_golden.py (which ran them through the reference Flamelet) and
the tests: streams, grid and dissipation-rate arguments, and loaders of tests/golden/flamelet_ref.npz."""
import os

import numpy as np

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')

FLAMELET_CASES = [
    # name, mechanism file, phase, oxidizer (T, X), fuel (T, basis, composition), grid points, chi_st, seed
    ('h2', 'h2-burke.yaml', 'h2-burke', (1200., 'O2:1 N2:3.74'), (300., 'Y', 'H2:1'), 34, 1., 11),
    ('gri', 'methane-gri30.yaml', 'methane-gri30', (300., 'O2:1 N2:3.76'), (300., 'X', 'CH4:1'), 16, 1., 12),
]
BUNDLED = {'h2': 'h2-burke', 'gri': 'methane-gri30'}


def case(name):
    return [c for c in FLAMELET_CASES if c[0] == name][0]


def flamelet_case_setup(spec, c):
    """(oxidizer stream, fuel stream, FlameletSpec keyword arguments) of a case."""
    name, _, _, (To, Xo), (Tf, basis, comp), npts, chi_st, seed = c
    oxy = spec.stream('TPX', (To, 101325., Xo))
    fuel = spec.stream('TP' + basis, (Tf, 101325., comp))
    return oxy, fuel, dict(oxy_stream=oxy, fuel_stream=fuel, grid_points=npts, grid_type='clustered',
                           grid_cluster_intensity=4., grid_cluster_point='stoichiometric',
                           stoich_dissipation_rate=chi_st, dissipation_rate_form='Peters')


def golden():
    return np.load(os.path.join(GOLD, 'flamelet_ref.npz'))


def btddod_row_err(a, b, nzi, ns):
    """Row-normwise relative error of two BTDDOD value arrays (blocks and off-diagonals of each matrix row)."""
    bs = nzi * ns * ns
    Ba = np.swapaxes(a[:bs].reshape(nzi, ns, ns), 1, 2).reshape(nzi * ns, ns)
    Bb = np.swapaxes(b[:bs].reshape(nzi, ns, ns), 1, 2).reshape(nzi * ns, ns)
    m = (nzi - 1) * ns
    sub_a, sup_a = a[bs:bs + m], a[bs + m:]
    sub_b, sup_b = b[bs:bs + m], b[bs + m:]
    num = np.abs(Ba - Bb).max(1)
    den = np.abs(Bb).max(1)
    num[ns:] = np.maximum(num[ns:], np.abs(sub_a - sub_b))
    den[ns:] = np.maximum(den[ns:], np.abs(sub_b))
    num[:m] = np.maximum(num[:m], np.abs(sup_a - sup_b))
    den[:m] = np.maximum(den[:m], np.abs(sup_b))
    return float((num / np.maximum(den, 1e-300)).max())


def vec_err(a, b, ns, floor=1e-300):
    """Per-variable relative error of point-major vectors: |a - b| over the largest |b| of that variable (at least
    `floor`)."""
    a = np.asarray(a).reshape(-1, ns)
    b = np.asarray(b).reshape(-1, ns)
    return float((np.abs(a - b).max(0) / np.maximum(np.abs(b).max(0), floor)).max())


def eig_err(e, ref, op, state):
    """Largest |e - ref| over the tolerance two backward-stable eigenvalue solvers can be held to:
    1e-13 ||A||_F of the point's chemistry block plus 1e-8 max(|ref|, 1)."""
    B = op.blocks(op.jac(state, eflux=False))
    ns = op.ns
    scale = np.zeros(op.nzi * ns)
    for i in range(op.nzi):
        A = B[i] - np.diag(op.cmajor[i * ns:(i + 1) * ns])
        scale[i * ns:(i + 1) * ns] = 1e-13 * np.linalg.norm(A)
    tol = scale + 1e-8 * np.maximum(np.abs(ref), 1.)
    return float(np.max(np.abs(np.asarray(e) - ref) / tol))
