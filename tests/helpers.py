"""Shared test helpers: row-normwise relative error and mechanism/oracle pairs."""
import numpy as np


def rownorm_err(A, B, floor=1e-300):
    """max over rows of max_j |A_ij - B_ij| / max(max_j |B_ij|, floor); A, B shaped [..., rows, cols]."""
    A = np.asarray(A)
    B = np.asarray(B)
    num = np.abs(A - B).max(axis=-1)
    den = np.maximum(np.abs(B).max(axis=-1), floor)
    return float((num / den).max())


def colmajor(J, n):
    """Column-major flat block(s) -> [..., row, col] arrays."""
    J = np.asarray(J)
    return np.swapaxes(J.reshape(J.shape[:-1] + (n, n)), -1, -2)


def pair(name):
    """(ChemicalMechanismSpec from the bundled data, OracleGriffon filled with the same setters)."""
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    import oracle as orc
    spec = ChemicalMechanismSpec.bundled(name)
    og = orc.OracleGriffon()
    spec._populate_griffon(og)
    return spec, og
