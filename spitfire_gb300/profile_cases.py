"""Small, self-contained runs of each kernel family for profiling (``ncu``) and quick checks.

    python -m spitfire_gb300.profile_cases <case>

Cases (GRI-3.0 unless stated; each ends by checking the device error word):
  jac        isochoric RHS + Jacobian of 8192 states (chem_kernel MODE_JAC), 3 launches
  jac_tps    the same with the thread-per-state kernel (chem_kernel_tps MODE_JAC) at 2 resident 4-warp blocks per
             SM, on 38912 states (one warp batch per resident warp), 2 launches
  rates_rhs  production rates (chem_kernel_tps MODE_RATES) and the isochoric right-hand side (MODE_RHS) of 38912
             states, thread per state at 2 resident 4-warp blocks per SM, 2 launches each
  integrate_2048  2048 isobaric reactors of the batched-ignition distribution to ignition or 0.1 s with the
             autotuner's shape (Griffon scratch in global slots, 6 warps per block)
  integrate  256 isobaric reactors of the batched-ignition distribution to ignition or 0.1 s (integrate_kernel)
  flamelet   8 steady-flamelet profiles of 64-120 points: one RHS sweep, Jacobian with eigenvalue bounds,
             block-Thomas factorization, solve and matvec
  adjoint    64 reactors of the adjoint distribution recorded to 1 ms, then the batched adjoint
  fp64issue  warp-level FP64 FMA instructions per second with 1, 2, 4, 8, 16 and 32 active lanes per warp
"""

import sys

import numpy as np


def _spec():
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    return ChemicalMechanismSpec.bundled('methane-gri30')


def case_jac():
    import torch
    from spitfire_gb300 import workloads as W
    from spitfire_gb300._desc import reactor_params
    spec = _spec()
    q = torch.tensor(W.isochoric_state(W.gri_states(spec, 8192)), device='cuda')
    P = reactor_params('isochoric')
    for _ in range(3):
        spec.griffon.reactor_jac_batch(P, q, 0)
    torch.cuda.synchronize()
    return spec


def case_jac_tps():
    import torch
    from spitfire_gb300 import autotune as AT
    from spitfire_gb300 import workloads as W
    from spitfire_gb300._desc import reactor_params
    spec = _spec()
    AT.set_tuning(spec, 'tps_ctas', 2)
    AT.set_tuning(spec, 'group_jac', 1)
    n = torch.cuda.get_device_properties(0).multi_processor_count * 2 * 4 * 32
    q = torch.tensor(W.isochoric_state(W.gri_states(spec, n)), device='cuda')
    P = reactor_params('isochoric')
    for _ in range(2):
        spec.griffon.reactor_jac_batch(P, q, 0)
    torch.cuda.synchronize()
    return spec


def case_rates_rhs():
    import torch
    from spitfire_gb300 import autotune as AT
    from spitfire_gb300 import workloads as W
    from spitfire_gb300._desc import reactor_params
    spec = _spec()
    AT.set_tuning(spec, 'tps_ctas', 2)
    AT.set_tuning(spec, 'group_rates', 1)
    AT.set_tuning(spec, 'group_rhs', 1)
    n = torch.cuda.get_device_properties(0).multi_processor_count * 2 * 4 * 32
    d = W.gri_states(spec, n)
    g = spec.griffon
    q = torch.tensor(W.isochoric_state(d), device='cuda')
    T = torch.tensor(d['T'], device='cuda')
    rho = torch.tensor(d['rho'], device='cuda')
    Y = torch.tensor(d['Y'], device='cuda')
    P = reactor_params('isochoric')
    for _ in range(2):
        g.production_rates_batch(T, rho, Y)
    for _ in range(2):
        g.reactor_rhs_batch(P, q)
    torch.cuda.synchronize()
    return spec


def case_integrate():
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.reactors import BatchIntegrator
    spec = _spec()
    d = W.ignition_batch(spec, 256, seed=1003)
    BatchIntegrator(spec, 'isobaric').run(d['q0'], pressures=d['p'], delta_temperature_ignition=400.,
                                          stop_at_time=0.1)
    return spec


def case_integrate_2048():
    from spitfire_gb300 import autotune as AT
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.reactors import BatchIntegrator
    spec = _spec()
    AT.set_tuning(spec, 'integrate_scratch', 1)
    AT.set_tuning(spec, 'integrate_warps', 6)
    d = W.ignition_batch(spec, 2048, seed=1003)
    BatchIntegrator(spec, 'isobaric').run(d['q0'], pressures=d['p'], delta_temperature_ignition=400.,
                                          stop_at_time=0.1)
    return spec


def case_flamelet():
    import torch
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.flamelet import FlameletBatch
    spec = _spec()
    setups = W.slfm_flamelet_setups(spec, 8, seed=1004, nz_range=(64, 120))
    b = FlameletBatch(setups)
    x = b.initial_state()
    y = b.rhs(x)
    b.jacobian(x, eig=True, diffterm_per_flamelet=b.diffterm_tensor())
    b.factor()
    b.solve(y)
    b.matvec(x)
    torch.cuda.synchronize()
    return spec


def case_adjoint():
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.adjoint import ReactorAdjoint
    spec = _spec()
    d = W.adjoint_batch(spec, 64, seed=1005)
    adj = ReactorAdjoint(spec, 'isobaric')
    tr = adj.forward(d['q0'], pressures=d['p'], t_end=1.e-3)
    g = adj.backward(tr)
    assert bool(np.isfinite(g['theta'].cpu().numpy()).all())
    return spec


def case_fp64issue():
    import ctypes as C
    import torch
    from spitfire_gb300 import _native as N
    sink = torch.zeros(1, dtype=torch.float64, device='cuda')
    out = C.c_double()
    for lanes in (1, 2, 4, 8, 16, 32):
        N.check(N.load().sf_fp64_issue_probe(4000, lanes, C.byref(out), N.ptr(sink), N.stream_handle()))
        print(f'active lanes {lanes:2d}: {out.value:.4e} warp FP64 FMA instructions/s, '
              f'{out.value * lanes * 2 / 1e12:.3f} TFLOP/s of useful lanes')
    return None


CASES = {'jac': case_jac, 'jac_tps': case_jac_tps, 'rates_rhs': case_rates_rhs, 'integrate_2048': case_integrate_2048,
         'integrate': case_integrate, 'flamelet': case_flamelet, 'adjoint': case_adjoint,
         'fp64issue': case_fp64issue}


def main(argv):
    if len(argv) != 1 or argv[0] not in CASES:
        print(__doc__)
        return 2
    from spitfire_gb300 import build
    build.build()
    spec = CASES[argv[0]]()
    status = spec.griffon.device_status() if spec is not None else 0
    print(f'{argv[0]}: done, device status {status}')
    return 0 if status == 0 else 1


if __name__ == '__main__':
    sys.exit(main(sys.argv[1:]))
