"""Oracle jobs run in a pool of spawned processes (test infrastructure): steady flamelet solves, the SLFM
continuation and finite-difference gradients, each on one host core. Spawned, not forked, so that no child inherits
the parent's CUDA context."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def init():
    for p in (ROOT, os.path.join(ROOT, 'oracle'), os.path.join(ROOT, 'tests')):
        if p not in sys.path:
            sys.path.insert(0, p)
    import oracle as orc
    orc.set_threads(1)


def pool(n):
    import multiprocessing as mp
    return mp.get_context('spawn').Pool(max(1, min(n, os.cpu_count() or 1)), initializer=init)


_MECH = {}


def _mech(name):
    if name not in _MECH:
        import oracle as orc
        from spitfire_gb300.mechanism import ChemicalMechanismSpec
        spec = ChemicalMechanismSpec.bundled(name)
        og = orc.OracleGriffon()
        spec._populate_griffon(og)
        _MECH[name] = (spec, og)
    return _MECH[name]


def steady_flamelet(args):
    """compute_steady_state of the oracle (flamelet.py:1705-1778 restated) -> (key, state, method, iterations)."""
    key, mech, z, chi, oxy, fuel, ic = args
    import flamelet_steady as FS
    _, og = _mech(mech)
    op = FS.FlameletOperator(og, z, chi, oxy, fuel)
    st, how, it = FS.compute_steady_state(op, ic)
    return key, st, how, it


def slfm_continuation(args):
    """The adiabatic SLFM library loop of tabulation.py:229-336 on the oracle: one flamelet per dissipation rate,
    each started from the previous solution (the first from the Burke-Schumann profile), stopping at the first
    extinguished one (max(T - T_linear) < 10 K). Returns the list of (chi_st, state, method, iterations)."""
    mech, spec_kw, chis = args
    import flamelet_steady as FS
    from spitfire_gb300.flamelet import FlameletSetup, FlameletSpec
    spec, og = _mech(mech)
    out = []
    ic = 'Burke-Schumann'
    for chi in chis:
        s = FlameletSetup(FlameletSpec(mech_spec=spec, initial_condition=ic, stoich_dissipation_rate=float(chi),
                                       **spec_kw))
        op = FS.FlameletOperator(og, s.z, s.x, s.state_oxy, s.state_fuel)
        st, how, it = FS.compute_steady_state(op, s.initial_state)
        if st is None:
            out.append((chi, None, how, it))
            break
        if np.max(st[::spec.n_species] - s.linear_temperature) < 10.:
            out.append((chi, 'extinguished', how, it))
            break
        out.append((chi, st, how, it))
        ic = st.copy()
    return out


def fd_chunk(args):
    """Central differences of (T_end, tau_s) on the frozen step sequence for a chunk of parameters."""
    key, mech, configuration, pressure, q0, dts, params = args
    import sensitivity as SE
    spec, _ = _mech(mech)
    return key, params, SE.fd_gradient(spec, configuration, pressure, q0, dts, params)
