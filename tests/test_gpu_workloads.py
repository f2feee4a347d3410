"""GPU parity at the benchmark workloads' own sizes and ranges, against the oracle.

* Batched ignition, low-temperature band: GRI-3.0 isobaric reactors with T0 in 900-1050 K, where many reach
  t = 0.1 s without igniting. Status, accepted-step count, ignition delay (1e-6) and final state (1e-6) per reactor.
* Steady SLFM flamelets at the flamelet workload's sizes: GRI-3.0 CH4/air flamelets of 64, 128 and 256 points at
  chi_st = 1e-2, 1 and 1e3 1/s (the last extinguishes), solved in one batch from Burke-Schumann profiles. Same
  method (Newton or psitc) and iteration count as the oracle's compute_steady_state, temperatures within 1e-6,
  mass fractions within 1e-6 of each species' maximum (at least 1e-12: an extinguished flamelet holds radicals at
  1e-30 and below, where the two solvers' clipping of negative round-off differs), extinction agreeing.
* The GRI-3.0 adiabatic SLFM library on a short chi_st sweep through build_adiabatic_slfm_library, against the
  oracle's restatement of the reference's continuation loop: the same dissipation rates kept before extinction and
  the same profiles.
* Adjoint gradients against central finite differences for 3 reactors x 64 parameters each.

The oracle runs in a pool of spawned processes (tests/oracle_pool.py), one job per host core.
"""
import numpy as np
import pytest

import flamelet_cases as FC
import oracle_pool as OP
from helpers import pair

pytestmark = pytest.mark.gpu


def test_low_temperature_ignition_band_matches_oracle(cuda):
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.reactors import BatchIntegrator
    import integrate as I
    import oracle as orc
    orc.set_threads(1)
    spec, og = pair('methane-gri30')
    n = 24
    d = W.ignition_batch(spec, n, seed=91, T_range=(900., 1050.))
    out = BatchIntegrator(spec, 'isobaric').run(d['q0'], pressures=d['p'], delta_temperature_ignition=400.,
                                                stop_at_time=0.1)
    tau, st = out['t'].cpu().numpy(), out['status'].cpu().numpy()
    cnt, qf = out['counts'].cpu().numpy(), out['q'].cpu().numpy()
    ti = out['t_interp'].cpu().numpy()
    statuses = []
    for i in range(n):
        r = I.integrate(I.ReactorProblem(og, 'isobaric', pressure=d['p'][i]), d['q0'][i],
                        delta_temperature_ignition=400., stop_at_time=0.1)
        statuses.append(r['status'])
        assert st[i] == r['status'], (i, st[i], r['status'])
        assert cnt[i, 0] == r['steps'], (i, cnt[i], r['steps'])
        assert abs(tau[i] - r['t']) / r['t'] <= 1e-6, (i, tau[i], r['t'])
        if r['t_interp'] is None:
            assert np.isnan(ti[i]), i
        else:
            assert abs(ti[i] - r['t_interp']) / r['t_interp'] <= 1e-6, i
        ref = r['state']
        assert abs(qf[i, 0] - ref[0]) / ref[0] < 1e-6, i
        assert np.max(np.abs(qf[i, 1:] - ref[1:])) / np.max(np.abs(ref[1:])) < 1e-6, i
    # both outcomes are in the band: reactors that ignite and reactors that reach 0.1 s without igniting
    assert 1 in statuses and 2 in statuses, statuses
    assert spec.griffon.device_status() == 0


def _gri_streams(spec):
    air = spec.stream('TPX', (300., 101325., 'O2:1 N2:3.76'))
    fuel = spec.stream('TPX', (300., 101325., 'CH4:1'))
    return air, fuel


GRID = dict(grid_type='clustered', grid_cluster_intensity=4., grid_cluster_point='stoichiometric')


def test_workload_sized_flamelets_match_oracle(cuda):
    from spitfire_gb300.flamelet import FlameletBatch, FlameletSetup, FlameletSpec
    spec, _ = pair('methane-gri30')
    air, fuel = _gri_streams(spec)
    cases = ((64, 1.e-2), (128, 1.), (256, 1.e3))
    setups = [FlameletSetup(FlameletSpec(mech_spec=spec, oxy_stream=air, fuel_stream=fuel, grid_points=nz,
                                         stoich_dissipation_rate=chi, initial_condition='Burke-Schumann', **GRID))
              for nz, chi in cases]
    with OP.pool(len(cases)) as pool:
        jobs = pool.map_async(OP.steady_flamelet, [(k, 'methane-gri30', s.z, s.x, s.state_oxy, s.state_fuel,
                                                     s.initial_state) for k, s in enumerate(setups)])
        b = FlameletBatch(setups)
        ns = b.ns
        init = b.initial_state()
        s1, c1, i1 = b.steady_solve_newton(init, tolerance=1.e-6, max_iterations=38)
        s2, c2, i2 = b.steady_solve_psitc(init, active=~c1, tolerance=1.e-6, max_iterations=400)
        ref = {k: (st, how, it) for k, st, how, it in jobs.get(timeout=900)}
    c1, i1, c2, i2 = (t.cpu().numpy() for t in (c1, i1, c2, i2))
    s1, s2 = s1.cpu().numpy(), s2.cpu().numpy()
    extinct = []
    for f, s in enumerate(setups):
        st, how, it = ref[f]
        assert st is not None, f
        lo, hi = b.offz_host[f] * ns, b.offz_host[f + 1] * ns
        if c1[f]:
            got, gh, gi = s1[lo:hi], 'newton', int(i1[f])
        else:
            assert c2[f], f
            got, gh, gi = s2[lo:hi], 'psitc', int(i2[f])
        assert (gh, gi) == (how, it), (f, gh, gi, how, it)
        assert np.max(np.abs(got[::ns] - st[::ns]) / st[::ns]) < 1e-6, f
        assert FC.vec_err(got, st, ns, floor=1e-12) < 1e-6, f
        ext_gpu = np.max(got[::ns] - s.linear_temperature) < 10.
        ext_cpu = np.max(st[::ns] - s.linear_temperature) < 10.
        assert ext_gpu == ext_cpu, f
        extinct.append(ext_gpu)
    assert extinct == [False, False, True], extinct
    assert spec.griffon.device_status() == 0


def test_gri_slfm_library_matches_oracle_continuation(cuda):
    from spitfire_gb300.tabulation import build_adiabatic_slfm_library
    spec, _ = pair('methane-gri30')
    air, fuel = _gri_streams(spec)
    chis = np.logspace(-1., 2., 4)
    kw = dict(oxy_stream=air, fuel_stream=fuel, grid_points=64, **GRID)
    with OP.pool(1) as pool:
        job = pool.apply_async(OP.slfm_continuation, (('methane-gri30', kw, chis),))
        lib = build_adiabatic_slfm_library(dict(mech_spec=spec, **kw), diss_rate_values=chis, verbose=False)
        ref = job.get(timeout=900)
    kept = [r for r in ref if isinstance(r[1], np.ndarray)]
    assert len(kept) >= 2 and len(kept) < len(chis), [r[2:] for r in ref]  # burning entries, then extinction
    assert lib.dissipation_rate_stoich_npts == len(kept)
    ns = spec.n_species
    for ix, (chi, st, how, it) in enumerate(kept):
        T = lib['temperature'][1:-1, ix]
        assert np.max(np.abs(T - st[::ns]) / st[::ns]) < 1e-6, ix
        for k, name in enumerate(spec.species_names[:-1]):
            y = lib['mass fraction ' + name][1:-1, ix]
            assert np.max(np.abs(y - st[k + 1::ns])) <= 1e-6 * max(np.max(np.abs(st[k + 1::ns])), 1e-12), \
                (ix, name)
    assert spec.griffon.device_status() == 0


def test_adjoint_matches_finite_differences_widely(cuda):
    """Three GRI-3.0 reactors of the adjoint workload, each integrated into its ignition (t_end = its smoothed
    ignition delay), 64 parameters each (the 44 largest ln A and 20 largest E_a gradients of either output):
    both outputs' GPU gradients against central differences of the oracle on the frozen step sequence, normwise
    over each parameter kind relative to the largest gradient of that kind, 1e-5."""
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.adjoint import ReactorAdjoint
    spec, _ = pair('methane-gri30')
    d = W.adjoint_batch(spec, 16, seed=31)
    adj = ReactorAdjoint(spec, 'isobaric')
    tau = adj.forward(d['q0'], pressures=d['p'], t_end=5.e-3).tau_s.cpu().numpy()
    picks = [int(i) for i in np.argsort(tau)[:3]]
    assert np.all(tau[picks] < 4.e-3)
    yi = spec.reaction_yaml_index
    inv = np.argsort(yi)  # file position -> internal index
    jobs, grads = [], {}
    for i in picks:
        q0, p = d['q0'][i:i + 1], d['p'][i:i + 1]
        tr = adj.forward(q0, pressures=p, t_end=float(tau[i]))
        th = adj.backward(tr)['theta'].cpu().numpy()[0]  # [2 outputs, nr (file order), 2 kinds]
        dts = tr.rec[0, :tr.steps[0].item(), 1].cpu().numpy()
        score = [np.abs(th[:, :, c]).max(0) / np.abs(th[:, :, c]).max() for c in (0, 1)]
        sel = [(int(r), 0) for r in np.argsort(-score[0])[:44]] + [(int(r), 1) for r in np.argsort(-score[1])[:20]]
        grads[i] = (th, sel)
        params = [2 * int(inv[r]) + c for r, c in sel]
        for k in range(0, len(params), 8):
            jobs.append(((i, k), 'methane-gri30', 'isobaric', float(p[0]), q0[0], dts, params[k:k + 8]))
    with OP.pool(len(jobs)) as pool:
        res = pool.map(OP.fd_chunk, jobs)
    fd = {}
    for (i, k), params, g in res:
        fd.setdefault(i, {})[k] = g
    for i in picks:
        th, sel = grads[i]
        f = np.concatenate([fd[i][k] for k in sorted(fd[i])], axis=1)  # [2, 64]
        got = np.array([[th[o, r, c] for r, c in sel] for o in range(2)])
        for o in range(2):
            for c in (0, 1):
                m = [k for k, (_, cc) in enumerate(sel) if cc == c]
                scale = np.max(np.abs(th[o, :, c]))
                err = np.max(np.abs(got[o, m] - f[o, m])) / scale
                assert err < 1e-5, (i, o, c, err)
    assert spec.griffon.device_status() == 0
