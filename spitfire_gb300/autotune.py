"""Autotuner of the launch shapes of the batched kernels (warp-per-state and per-block shapes).

For one mechanism on the current device it times the candidate shapes on a sample of the caller's workload with
CUDA events and applies the fastest through ``sf_mech_set_tuning``:
  * lanes per state (8, 16, 32, or 1: the thread-per-state kernels, with their resident blocks per SM) of the
    production-rate, right-hand-side and Jacobian kernels;
  * for the persistent ESDIRK64 integrator: where each warp keeps its Griffon scratch and iteration matrix (shared
    memory, or L2-resident global slots, which leave room for more warps per SM) and how many warps (reactors)
    share a block.
The knobs change launch shapes only. The integrator's candidates produce bit-identical results; the lane-group
width changes the order of the per-species sums, so those candidates agree to rounding (the tuner checks both).
Choices are cached per (mechanism, device) in spitfire_gb300/_tuning (created on first use).
"""

import ctypes as C
import hashlib
import json
import os

import numpy as np

from . import _native as N

KNOBS = {'group_rates': 0, 'group_sens': 1, 'group_rhs': 2, 'group_jac': 3, 'integrate_warps': 4,
         'integrate_scratch': 5, 'tps_ctas': 6}
CACHE_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), '_tuning')


def _torch():
    import torch
    return torch


def set_tuning(mech, name, value):
    N.check(N.load().sf_mech_set_tuning(mech.griffon.handle, KNOBS[name], int(value)))


def get_tuning(mech, name):
    v = C.c_int()
    N.check(N.load().sf_mech_get_tuning(mech.griffon.handle, KNOBS[name], C.byref(v)))
    return v.value


def _time(fn, reps=3):
    torch = _torch()
    fn()
    torch.cuda.synchronize()
    best = float('inf')
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def _key(mech):
    torch = _torch()
    h = hashlib.sha1(json.dumps(mech.mech_data_json(), sort_keys=True).encode()).hexdigest()[:16]
    dev = torch.cuda.get_device_name().replace(' ', '_')
    return f'{h}_{dev}'


def tune_chemistry(mech, states, pressures=None, configuration='isochoric', kinds=('rates', 'rhs', 'jac'), reps=3,
                   thread_per_state=True):
    """Choose lanes per state for each kernel family on `states` (a batch of reactor states of the given
    configuration): 8, 16 or 32, or (with thread_per_state) 1 at a few resident-block counts of the thread-per-state
    kernels. Returns {knob: (best value, {candidate: ms})}, candidates labelled G or '1/<blocks per SM>', and, when
    a family chose 1, 'tps_ctas': (blocks per SM, None)."""
    torch = _torch()
    from ._desc import reactor_params
    g = mech.griffon
    q = g._dev(states)
    pr = g._dev(pressures) if pressures is not None else None
    P = reactor_params(configuration)
    tix = 1 if configuration == 'isochoric' else 0
    T = q[:, tix].contiguous()
    Y = torch.cat([q[:, tix + 1:], 1. - q[:, tix + 1:].sum(1, keepdim=True)], dim=1).contiguous()
    if configuration == 'isochoric':
        rho = q[:, 0].contiguous()
    else:
        mw = torch.tensor(mech.molecular_weights, device=q.device)
        rho = (pr if pr is not None else torch.full_like(T, 101325.)) / (8314.46261815324 * T * (Y / mw).sum(1))
    calls = {'rates': lambda: g.production_rates_batch(T, rho, Y),
             'rhs': lambda: g.reactor_rhs_batch(P, q, pressures=pr),
             'jac': lambda: g.reactor_jac_batch(P, q, 0, pressures=pr)}
    out = {}
    tps_choice = {}
    for kind in kinds:
        knob = 'group_' + kind
        times = {}
        ref = None
        cands = {8: 8, 16: 16, 32: 32}
        if thread_per_state:
            cands.update({f'1/{c}': (1, c) for c in (0, 2, 1)})  # label '1/<blocks per SM>' (0: all that fit)
        for label, cand in cands.items():
            if isinstance(cand, tuple):
                set_tuning(mech, 'tps_ctas', cand[1])
                set_tuning(mech, knob, 1)
            else:
                set_tuning(mech, knob, cand)
            res = calls[kind]()
            res = res if isinstance(res, tuple) else (res,)
            if ref is None:
                ref = [r.clone() for r in res]
            else:
                for a, b in zip(ref, res):
                    scale = a.abs().amax(dim=-1, keepdim=True).clamp_min(1e-300)
                    if float(((a - b).abs() / scale).max()) > 1e-12:
                        set_tuning(mech, knob, 0)
                        raise RuntimeError(f'{knob}={label} changed the results beyond rounding')
            times[label] = _time(calls[kind], reps)
            del res
        best = cands[min(times, key=times.get)]
        if isinstance(best, tuple):
            tps_choice[kind] = best[1]
            best = 1
        set_tuning(mech, knob, best)
        out[knob] = (best, times)
    # one resident-block count serves every thread-per-state family: that of the heaviest family that chose it
    for kind in ('jac', 'rhs', 'rates'):
        if kind in tps_choice:
            set_tuning(mech, 'tps_ctas', tps_choice[kind])
            out['tps_ctas'] = (tps_choice[kind], None)
            break
    else:
        set_tuning(mech, 'tps_ctas', 0)
    return out


def tune_integrator(integrator, q0, pressures=None, reps=1, **controls):
    """Choose the integrator's memory placement and warps per block on a sample batch (q0 rows): scratch 3 (all in
    shared memory), 1 (Griffon scratch in an L2-resident global slot per warp) or 2 (the iteration matrix there
    too). The sample should fill the largest candidate's resident warps (16 per SM at 8 warps per block), or the
    smaller shapes win on it. Returns (best (scratch, warps), {(scratch, warps): ms})."""
    torch = _torch()
    mech = integrator.mech
    times = {}
    ref = None
    saved = (get_tuning(mech, 'integrate_scratch'), get_tuning(mech, 'integrate_warps'))
    for scratch in (3, 1, 2):  # all in shared memory, Griffon scratch global, matrix global too
        set_tuning(mech, 'integrate_scratch', scratch)
        set_tuning(mech, 'integrate_warps', 0)
        fit = _fitting_warps(integrator)
        for warps in sorted({fit, max(1, fit // 2), max(1, (3 * fit) // 4)}):
            set_tuning(mech, 'integrate_warps', warps)
            res = integrator.run(q0, pressures=pressures, **controls)
            torch.cuda.synchronize()
            if ref is None:
                ref = res
            elif not (torch.equal(ref['t'], res['t']) and torch.equal(ref['q'], res['q'])):
                set_tuning(mech, 'integrate_scratch', saved[0])
                set_tuning(mech, 'integrate_warps', saved[1])
                raise RuntimeError(f'integrator shape {(scratch, warps)} changed the results')
            times[(scratch, warps)] = _time(lambda: integrator.run(q0, pressures=pressures, **controls), reps)
    best = pick_integrator_shape(times)
    set_tuning(mech, 'integrate_scratch', best[0])
    set_tuning(mech, 'integrate_warps', best[1])
    return best, times


def pick_integrator_shape(times, within=0.02):
    """The integrator shape to keep from {(scratch, warps): ms} of a tuning sample. The sample is smaller than the
    batches the tuning serves, and the larger shapes gain on larger batches (8192 GRI ignitions: 8 warps per block
    3-4 % faster than 6, which tie on 4096 reactors), so among the shapes within `within` of the fastest the one
    with the most warps per block wins, the faster one on equal warps."""
    fastest = min(times.values())
    return max((k for k in times if times[k] <= (1. + within) * fastest), key=lambda k: (k[1], -times[k]))


def _fitting_warps(integrator):
    """Warps per block that fit the shared memory with the current scratch placement (1..8)."""
    torch = _torch()
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    smem = getattr(props, 'shared_memory_per_block_optin', 232448)
    h = integrator.mech.griffon
    # per-warp doubles as the integrator lays them out (integrate_kernels.cu per_warp_doubles)
    lay = h.scratch_layout()
    neq = integrator.mech.n_species + (1 if integrator.configuration == 'isochoric' else 0)
    v = get_tuning(integrator.mech, 'integrate_scratch')
    place = 2 if v == 0 else (0 if v == 3 else v)  # knob value -> placement (0: the built-in choice, 2)
    gs, gm = place >= 1, place == 2
    n2 = neq * neq
    per = (0 if gm else n2) + 12 * neq + (0 if gs else lay['total']) + \
        (((0 if gm else (n2 + 1) // 2) + neq) if integrator.linear_precision == 1 else 0) + (neq + 1) // 2 + 2 + neq
    return int(max(1, min(8, (smem - lay['blob_bytes'] - 64) // (per * 8))))


def save(mech, results):
    os.makedirs(CACHE_DIR, exist_ok=True)
    knobs = {name: get_tuning(mech, name) for name in KNOBS}
    with open(os.path.join(CACHE_DIR, _key(mech) + '.json'), 'w') as f:
        json.dump({'knobs': knobs, 'results': results}, f, indent=1, default=str)


def load(mech):
    """Apply cached choices for this mechanism and device, if any. Returns the knob dict or None."""
    path = os.path.join(CACHE_DIR, _key(mech) + '.json')
    if not os.path.exists(path):
        return None
    with open(path) as f:
        knobs = json.load(f)['knobs']
    for name, v in knobs.items():
        set_tuning(mech, name, v)
    return knobs
