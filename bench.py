"""Benchmark of the GB300 Griffon hot path; prints one JSON line.

Headline workload (one "step"): the analytical isochoric reactor right-hand side + Jacobian of GRI-3.0 (53 species,
325 reactions) on 65536 seeded states (T ~ U(600, 2800) K, p log-uniform 1-40 atm, Y = 0.7 Dir + 0.3
complete-combustion profile; spitfire_gb300.workloads.gri_states). One step = one batched evaluation of all states.

  value      states/s of the batched kernel, inputs resident in HBM (L2 flushed between steps by writing a
             256 MB buffer outside the timed events)
  e2e        states/s through the public API with host buffers: every step copies the states host->device (pinned)
             and the RHS + Jacobian device->host, inside the timed region
  roofline   the kernel is FP64-pipe bound: achieved = executed FP64 flops per state (counted by ncu, see
             profiles/) x states / kernel time, peak = FP64 FMA throughput measured live by bench_probes.cu
  cpu_baseline / --impl reference: the oracle (C++ restatement of Griffon, OpenMP over all host cores) on the
             same states

Further blocks of the same line (each measured once after warm-up, inputs resident):
  newton     batched factor + solve of gamma*h*J - I (54 x 54) for the 65536 states: FP64 LU vs FP32 LU + 2 FP64
             refinement sweeps, with the FP32 variant's error against the FP64 solution
  ignition   8192 isobaric adiabatic GRI-3.0 reactors (T0 ~ U(900, 1500) K, phi ~ U(0.5, 2), p log-uniform 1-20
             atm) integrated to T0 + 400 K or t = 0.1 s in one persistent launch replayed from a CUDA graph;
             ignitions/s, ignition-delay error against the oracle integrator on a sample, the oracle's rate on the
             host cores
  adjoint    gradients of the final temperature and a smoothed ignition delay with respect to ln A and E_a of all
             325 reactions for 2048 isobaric GRI-3.0 reactors (T0 ~ U(1000, 1400) K, phi ~ U(0.7, 1.5), 10 atm,
             t_end = 5 ms): recorded forward integration plus batched discrete adjoint; gradients/s and peak
             memory, the oracle's CPU forward sensitivity on a sample
  flamelet   64 steady GRI-3.0 CH4/air flamelets (chi_st log-spaced 1e-2 - 1e3 1/s, grids of 64 - 256 points)
             solved together from Burke-Schumann profiles (batched Newton, then pseudo-transient continuation);
             flamelets/s, per-kernel times and rooflines of one batched launch, the oracle solver on a sample

Multi-GPU: states, reactors and flamelets are independent, so each rank runs its own batch (weak scaling, no
collective; the time is the max over ranks).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'oracle'))

from spitfire_gb300.sharding import dist_env, max_over_ranks, sum_over_ranks  # noqa: E402

METRIC = 'batched ignitions/s at 1e-6 rel τ_ign err; RHS+Jac states/s vs plain & CPU'
N_STATES = 65536
N_REACTORS = 8192
N_FLAMELETS = 64
N_ADJOINT = 2048
TUNE_REACTORS = 4096
# Per GRI state of each Jacobian kernel the autotuner can choose, from ncu on the profiling cases
# (python bench.py --profile-case jac | jac_tps): executed FP64 flops (thread-level DADD + DMUL + 2*DFMA),
# warp-level FP64 instructions (smsp__inst_executed_pipe_fp64.sum / states) and DRAM bytes
# (dram__bytes_read.sum + dram__bytes_write.sum / states; the 8192-state case of the lane-group kernel keeps part of
# its Jacobians in L2 at the end, so its figure is a lower bound; it was captured before the table-driven exponential,
# which took the thread-per-state kernel from 79,842 to 76,159 flops and from 1,733 to 1,727 instructions).
FP64_PER_STATE = {
    32: {'kernel': 'chem_kernel<32, MODE_JAC>', 'flops': 86953., 'warp_instr': 2816., 'dram_bytes': 18725.},
    1: {'kernel': 'chem_kernel_tps<MODE_JAC>', 'flops': 76159., 'warp_instr': 1727., 'dram_bytes': 124181.},
}


def griffon_dense_flops(spec):
    """FP64 flops per state of Griffon's own dense exact-Jacobian algorithm (rates_sensitivities_exact.cpp
    accumulation 2*n_net*(ns-1) per reaction, third-body/falloff dCtbaf/dY 4*(ns-1), assembly 2*(ns+1)^2*2)."""
    rec = spec.griffon._rec
    ns = spec.n_species
    flops = 0
    for r in rec.reactions:
        net = {}
        for s, v in r['reactants'].items():
            net[s] = net.get(s, 0) + v
        for s, v in r['products'].items():
            net[s] = net.get(s, 0) - v
        n_net = sum(1 for v in net.values() if abs(v) > 1e-14)
        flops += 2 * n_net * (ns - 1)
        if r['kind'] != 1:
            flops += 4 * (ns - 1)
    return flops + 4 * (ns + 1) ** 2


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = 'clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,' \
             'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,' \
             'clocks_event_reasons.sw_power_cap'

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(['nvidia-smi', '-i', str(self.index), f'--query-gpu={self.FIELDS}',
                                      '--format=csv,noheader,nounits'], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([v.strip() for v in out.stdout.strip().split(',')])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['unavailable']}
        sm = [float(s[0]) for s in self.samples if s[0].replace('.', '').isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[j] for s in self.samples for j in range(4) if len(s) > 4 + j and
                          s[4 + j].lower() == 'active'})
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': max(mx) if mx else None,
                'reasons': reasons, 'samples': len(self.samples)}


def cpu_baseline(spec, q, seconds=10.0, threads=None):
    """Oracle RHS+Jacobian on the host cores over repeated passes of a sample of the states."""
    import numpy as np
    import oracle as orc
    from spitfire_gb300._desc import reactor_params
    og = orc.OracleGriffon()
    spec._populate_griffon(og)
    cores = threads or os.cpu_count()
    orc.set_threads(cores)
    P = reactor_params('isochoric')
    yin = np.zeros(spec.n_species)
    P.inflow_Y = orc._p(yin)
    sample = q[:4096]
    og.reactor_jac_batch(P, sample[:256], 0)
    t0 = time.perf_counter()
    done = 0
    while time.perf_counter() - t0 < seconds:
        og.reactor_jac_batch(P, sample, 0)
        done += sample.shape[0]
    dt = time.perf_counter() - t0
    return {'value': done / dt, 'unit': 'states/s', 'cores': cores, 'kind': 'port',
            'sample': f'{done} GRI-3.0 isochoric RHS+Jacobian evaluations ({sample.shape[0]}-state passes of the '
                      f'benchmark states) in {dt:.1f} s'}


def _ignite_one(args):
    """Oracle integration of one isobaric GRI-3.0 reactor (runs in a spawned worker)."""
    q0, p = args
    import oracle as orc
    import integrate as I
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    g = _ignite_one.__dict__.get('og')
    if g is None:
        orc.set_threads(1)
        spec = ChemicalMechanismSpec.bundled('methane-gri30')
        g = orc.OracleGriffon()
        spec._populate_griffon(g)
        _ignite_one.og = g
    r = I.integrate(I.ReactorProblem(g, 'isobaric', pressure=p), q0, delta_temperature_ignition=400.,
                    stop_at_time=0.1)
    return r['t'], r['status'], r['steps'], r['t_interp']


def _worker_init(root):
    sys.path[:0] = [root, os.path.join(root, 'oracle')]


def cpu_ignitions(q0, p, n_sample, seconds=30.0):
    """Oracle ignitions of the first n_sample reactors on all host cores (spawned pool). Returns (ignitions/s,
    cores, tau[list], status[list], wall seconds)."""
    import multiprocessing as mp
    cores = os.cpu_count()
    ctx = mp.get_context('spawn')
    with ctx.Pool(cores, initializer=_worker_init, initargs=(ROOT,)) as pool:
        pool.map(_ignite_one, [(q0[0], p[0])] * cores)  # worker start-up outside the timing
        t0 = time.perf_counter()
        res = []
        it = pool.imap(_ignite_one, [(q0[i], p[i]) for i in range(n_sample)])
        for r in it:
            res.append(r)
            if time.perf_counter() - t0 > seconds:
                break
        dt = time.perf_counter() - t0
        pool.terminate()
    return len(res) / dt, cores, [r[0] for r in res], [r[1] for r in res], dt, [r[3] for r in res]


def _flamelet_one(args):
    z, x, oxy, fuel, ic = args
    import oracle as orc
    import flamelet_steady as FS
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    g = _flamelet_one.__dict__.get('og')
    if g is None:
        orc.set_threads(1)
        spec = ChemicalMechanismSpec.bundled('methane-gri30')
        g = orc.OracleGriffon()
        spec._populate_griffon(g)
        _flamelet_one.og = g
    t0 = time.perf_counter()
    op = FS.FlameletOperator(g, z, x, oxy, fuel)
    st, how, it = FS.compute_steady_state(op, ic)
    return st, how, it, time.perf_counter() - t0


def cpu_flamelets(setups, idx, seconds=60.0):
    """Oracle compute_steady_state of the flamelets `idx` on all host cores (spawned pool), stopped after `seconds`.
    Returns (list of (index, state, method, cpu seconds)), cores, wall seconds."""
    import multiprocessing as mp
    cores = os.cpu_count()
    ctx = mp.get_context('spawn')
    out = []
    with ctx.Pool(min(cores, len(idx)), initializer=_worker_init, initargs=(ROOT,)) as pool:
        t0 = time.perf_counter()
        args = [(setups[k].z, setups[k].x, setups[k].state_oxy, setups[k].state_fuel, setups[k].initial_state)
                for k in idx]
        it = pool.imap_unordered(_flamelet_job, list(zip(idx, args)))
        try:
            while True:
                left = seconds - (time.perf_counter() - t0)
                if left <= 0:
                    break
                out.append(it.next(timeout=left))
        except (StopIteration, mp.TimeoutError):
            pass
        dt = time.perf_counter() - t0
        pool.terminate()
    return out, min(cores, len(idx)), dt


def _flamelet_job(a):
    k, args = a
    st, how, it, sec = _flamelet_one(args)
    return k, st, how, sec


def _timed(fn, stream, reps=1):
    """Average milliseconds of fn() on `stream` with CUDA events (one untimed call first)."""
    import torch
    fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def measured_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'MEASURED_PEAKS.json hbm_gbs (of measured)'
    except Exception:
        return 6800., 'fallback 6.8 TB/s (of fallback)'


def bench_newton(q, rhs, J, gamma_h, stream):
    """Batched Newton algebra on the benchmark states: FP64 LU vs FP32 LU + 2 FP64 refinement sweeps."""
    import numpy as np
    import torch
    from spitfire_gb300.linalg import NewtonSystems, backward_error
    n, m = q.shape
    out = {'systems': n, 'm': m, 'gamma_h': 'log-uniform 1e-9 - 1e-5 s'}
    xs = {}
    for prec, name in ((0, 'fp64'), (1, 'fp32_lu_fp64_refine2')):
        ns = NewtonSystems(n, m, prec, refine=2)
        f_ms = _timed(lambda: ns.factor(J, gamma_h), stream)
        x = torch.empty_like(rhs)
        s_ms = _timed(lambda: ns.solve(rhs, out=x), stream)
        xs[name] = x
        A = ns.A[:512].cpu().numpy().reshape(-1, m, m).transpose(0, 2, 1)
        be = backward_error(A, x[:512].cpu().numpy(), rhs[:512].cpu().numpy())
        out[name] = {'factor_ms': f_ms, 'solve_ms': s_ms, 'systems_per_s': n / ((f_ms + s_ms) * 1e-3),
                     'lu_tflops': (2. / 3. * m ** 3) * n / (f_ms * 1e-3) / 1e12,
                     'max_backward_error_sample512': float(be.max()),
                     'info_nonzero': int((ns.info != 0).sum().item())}
        del ns
    d = (xs['fp32_lu_fp64_refine2'] - xs['fp64']).abs().amax(1) / xs['fp64'].abs().amax(1)
    q = torch.quantile(d, torch.tensor([0.5, 0.99, 0.999], dtype=torch.float64, device=d.device))
    out['fp32_variant_rel_err_vs_fp64'] = {
        'median': float(q[0]), 'p99': float(q[1]), 'p999': float(q[2]), 'max': float(d.max()),
        'note': 'normwise forward difference of the two solutions per system; gamma*h*J - I reaches condition '
                'numbers near 1/eps for the largest gamma*h, where any FP64 solver has O(1) forward error, so the '
                'backward errors above are the accuracy statement'}
    return out


# integrator memory placement knob: Griffon scratch and iteration matrix in shared memory or L2-resident global slots
PLACEMENT = {3: 'shared', 1: 'global scratch', 2: 'global scratch + matrix'}


def bench_ignition(spec, rank, stream, cpu):
    import numpy as np
    import torch
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.reactors import BatchIntegrator
    d = W.ignition_batch(spec, N_REACTORS, seed=1003 + rank)
    from spitfire_gb300 import autotune as AT
    bi = BatchIntegrator(spec, 'isobaric')
    kw = dict(delta_temperature_ignition=400., stop_at_time=0.1)
    # launch shape from the autotuner, on a 4096-reactor sample of the batch (not timed): the sample must fill the
    # largest candidate's resident warps (16 per SM at 8 warps per block), or it favours the smaller shapes
    best, cand = AT.tune_integrator(bi, d['q0'][:TUNE_REACTORS], pressures=d['p'][:TUNE_REACTORS], **kw)
    out = bi.run(d['q0'], pressures=d['p'], graph=True, **kw)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    bi.replay()
    e1.record(stream)
    e1.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1))
    tau = out['t'].cpu().numpy()
    tau_i = out['t_interp'].cpu().numpy()
    status = out['status'].cpu().numpy()
    steps = out['counts'][:, 0].cpu().numpy()
    world = int(os.environ.get('WORLD_SIZE', '1'))
    res = {'reactors': N_REACTORS, 'value': world * N_REACTORS / (ms * 1e-3), 'unit': 'ignitions/s',
           'ms': ms, 'graph': 'one persistent launch captured in a CUDA graph, replay timed',
           'status_counts': {str(k): int(v) for k, v in zip(*np.unique(status, return_counts=True))},
           'steps': {'min': int(steps.min()), 'median': float(np.median(steps)), 'max': int(steps.max())},
           'device_status': spec.griffon.device_status(),
           'tau_interpolated': _tau_interp_summary(tau, tau_i, status),
           'autotune': {'chosen': {'placement': PLACEMENT[best[0]], 'warps_per_block': best[1]},
                        f'candidates_ms_{TUNE_REACTORS}_reactors': {f'{PLACEMENT[k[0]]}/{k[1]}w': v
                                                                     for k, v in cand.items()}}}
    # comparison point: the plain single-state GPU form (one thread per reactor, same step logic) on the same batch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    outp = bi.run_plain(d['q0'], pressures=d['p'], **kw)
    e1.record(stream)
    e1.synchronize()
    plain_ms = e0.elapsed_time(e1)
    tp = outp['t'].cpu().numpy()
    same = outp['counts'][:, 0].cpu().numpy() == steps
    res['plain_gpu_form'] = {'value': world * N_REACTORS / (plain_ms * 1e-3), 'unit': 'ignitions/s', 'ms': plain_ms,
                             'speedup_batched_over_plain': plain_ms / ms,
                             'tau_rel_diff_vs_batched_max': float(np.max(np.abs(tp - tau) / tau)),
                             'steps_equal_fraction': float(same.mean())}
    del outp
    # FP32-LU + FP64-refinement integrator on the first 512 reactors against the FP64 run
    o32 = BatchIntegrator(spec, 'isobaric', linear_precision=1, refine_sweeps=2).run(
        d['q0'][:512], pressures=d['p'][:512], **kw)
    t32 = o32['t'].cpu().numpy()
    s32 = o32['status'].cpu().numpy()
    ok = (s32 == status[:512])
    rel32 = np.abs(t32[ok] - tau[:512][ok]) / tau[:512][ok]
    res['fp32_lu_variant'] = {'reactors': 512, 'status_mismatches': int((~ok).sum()),
                              'tau_rel_err_vs_fp64_max': float(rel32.max()),
                              'tau_rel_err_vs_fp64_median': float(np.median(rel32))}
    if cpu:
        n_s = 256
        rate, cores, t_cpu, st_cpu, dt, ti_cpu = cpu_ignitions(d['q0'], d['p'], n_s, seconds=30.)
        k = len(t_cpu)
        both = [i for i in range(k) if st_cpu[i] == 2 and status[i] == 2]
        rel = [abs(tau[i] - t_cpu[i]) / t_cpu[i] for i in both]
        rel_i = [abs(tau_i[i] - ti_cpu[i]) / ti_cpu[i] for i in both if ti_cpu[i] is not None]
        res['tau_interpolated']['rel_err_vs_oracle_max'] = max(rel_i) if rel_i else None
        res['cpu_baseline'] = {'value': rate, 'unit': 'ignitions/s', 'cores': cores, 'kind': 'port',
                               'sample': f'oracle integrator (ESDIRK64 + Newton + PI restated, C++ kernels) on the '
                                         f'first {k} reactors, spawned pool, {dt:.1f} s'}
        res['tau_rel_err_vs_oracle'] = {'reactors_compared': len(both), 'max': max(rel) if rel else None,
                                        'status_mismatches': int(sum(st_cpu[i] != status[i] for i in range(k)))}
    return res


N_H2 = 4096


def bench_h2(rank, stream, cpu):
    """The small-mechanism workload: h2-burke isochoric RHS + analytical Jacobian on 4096 seeded states (T ~ U(800,
    2500) K, 1 atm, Y = 0.5 Dir(0.5) over the nine named species + 0.5 N2), L2 flushed between steps; and one ESDIRK64
    ignition of stoichiometric H2/air (H2:O2:N2 = 2:1:3.76) from 1200 K at 1 atm to t = 1e-3 s, isochoric and
    isobaric, against the oracle integrator."""
    import numpy as np
    import torch
    import integrate as I
    import oracle as orc
    from spitfire_gb300 import autotune as AT
    from spitfire_gb300 import workloads as W
    from spitfire_gb300._desc import reactor_params
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    from spitfire_gb300.reactors import BatchIntegrator
    spec = ChemicalMechanismSpec.bundled('h2-burke')
    g = spec.griffon
    dev = torch.device('cuda', torch.cuda.current_device())
    d = W.h2_states(spec, N_H2, seed=1001 + rank)
    qh = W.isochoric_state(d)
    q = torch.tensor(qh, device=dev)
    neq = q.shape[1]
    P = reactor_params('isochoric')
    tuned = AT.tune_chemistry(spec, qh, kinds=('jac',))
    rhs = torch.empty_like(q)
    J = torch.empty((N_H2, neq * neq), dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        g.reactor_jac_batch(P, q, 0, out_rhs=rhs, out_jac=J)
    for _ in range(5):
        step()
    torch.cuda.synchronize()
    times = []
    for _ in range(20):
        flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = max_over_ranks(statistics.mean(times))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    hbm, hbm_src = measured_peaks()
    per_state = (neq + neq + neq * neq) * 8
    ach = per_state * N_H2 / (ms * 1e-3) / 1e9
    res = {'workload': f'h2-burke (11 species, 27 reactions) isochoric RHS + analytical Jacobian, {N_H2} states',
           'value': world * N_H2 / (ms * 1e-3), 'unit': 'states/s', 'ms': ms,
           'l2': 'flushed between steps (256 MB write outside the timed events)',
           'autotune': {'group_jac': tuned['group_jac'][0]},
           'roofline': {'bound': 'hbm', 'algorithmic_bytes_per_state': per_state, 'achieved': ach, 'peak': hbm,
                        'unit': 'GB/s', 'frac': ach / hbm, 'peak_source': hbm_src,
                        'note': '4096 states are 5.5 MB of output: one launch of a few microseconds, so the time '
                                'is launch and ramp-up latency, not bandwidth'}}
    # the plain single-state GPU form on the same states
    from spitfire_gb300 import _native as N
    wsp = torch.empty(N.load().sf_reactor_jac_plain_workspace_size(g.handle, N_H2) // 8 + 1, dtype=torch.float64,
                      device=dev)
    plain_ms = sorted(_timed(lambda: g.reactor_jac_plain_batch(P, q, workspace=wsp), stream) for _ in range(3))[1]
    res['plain_gpu_form'] = {'value': world * N_H2 / (plain_ms * 1e-3), 'unit': 'states/s', 'ms': plain_ms,
                             'speedup_batched_over_plain': plain_ms / ms}
    # one stoichiometric H2/air ignition from 1200 K at 1 atm to t = 1e-3 s
    X = np.zeros(spec.n_species)
    X[spec.species_index('H2')], X[spec.species_index('O2')], X[spec.species_index('N2')] = 2., 1., 3.76
    Y = X * spec.molecular_weights
    Y /= Y.sum()
    og = orc.OracleGriffon()
    spec._populate_griffon(og)
    orc.set_threads(1)
    ign = {}
    for conf in ('isochoric', 'isobaric'):
        if conf == 'isobaric':
            q0 = np.hstack([[1200.], Y[:-1]])[None, :]
        else:
            rho = 101325. / (Y / spec.molecular_weights).sum() / (8314.46261815324 * 1200.)
            q0 = np.hstack([[rho, 1200.], Y[:-1]])[None, :]
        bi = BatchIntegrator(spec, conf, pressure=101325.)
        bi.run(q0, stop_at_time=1.e-3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = bi.run(q0, stop_at_time=1.e-3)
        torch.cuda.synchronize()
        gpu_s = time.perf_counter() - t0
        qf = out['q'].cpu().numpy()[0]
        steps = int(out['counts'][0, 0].item())
        prob = I.ReactorProblem(og, conf, pressure=101325.)
        t0 = time.perf_counter()
        r = I.integrate(prob, q0[0], stop_at_time=1.e-3)
        cpu_s = time.perf_counter() - t0
        Ti = 1 if conf == 'isochoric' else 0
        ign[conf] = {'gpu_seconds': gpu_s, 'steps': steps, 'T_end': float(qf[Ti]),
                     'oracle_steps': int(r['steps']), 'oracle_seconds_1core': cpu_s,
                     'T_end_rel_err_vs_oracle': float(abs(qf[Ti] - r['state'][Ti]) / r['state'][Ti]),
                     'note': 'one reactor is one warp on one SM: a latency figure, not a throughput one'}
    res['ignition_1200K_to_1ms'] = ign
    if cpu:
        og2 = orc.OracleGriffon()
        spec._populate_griffon(og2)
        cores = os.cpu_count()
        orc.set_threads(cores)
        P2 = reactor_params('isochoric')
        yin = np.zeros(spec.n_species)
        P2.inflow_Y = orc._p(yin)
        og2.reactor_jac_batch(P2, qh[:256], 0)
        t0 = time.perf_counter()
        done = 0
        while time.perf_counter() - t0 < 5.:
            og2.reactor_jac_batch(P2, qh, 0)
            done += N_H2
        dt = time.perf_counter() - t0
        res['cpu_baseline'] = {'value': done / dt, 'unit': 'states/s', 'cores': cores, 'kind': 'port',
                               'sample': f'{done} h2-burke isochoric RHS+Jacobian evaluations (passes over the '
                                         f'{N_H2} benchmark states) in {dt:.1f} s'}
    del flush, J, wsp
    torch.cuda.empty_cache()
    return res


def _flamelet_time_split(setups, native_wall):
    """Where the steady solve's time goes. The native solvers run every operation inside the library, so a second
    solve of the same batch runs the same solvers with their control loop on the host
    (FlameletBatch.steady_solve_*_host: the same device operations in the same order, bit-identical results) with
    CUDA events around every batched operation. Its operation times against the native wall time give the native
    solvers' own control cost (their masks, norms, flag reads and synchronizations)."""
    import torch
    from spitfire_gb300.flamelet import FlameletBatch
    b = FlameletBatch(setups)
    b.steady_solve_newton = b.steady_solve_newton_host
    b.steady_solve_psitc = b.steady_solve_psitc_host
    rec = {}
    for name in ('rhs', 'jacobian', 'factor', 'solve', 'scale_and_add_diagonal'):
        f = getattr(b, name)

        def wrap(*a, _f=f, _n=name, **kw):
            key = _n + ('_eig' if kw.get('eig') else '')
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            r = _f(*a, **kw)
            e1.record()
            rec.setdefault(key, []).append((e0, e1))
            return r
        setattr(b, name, wrap)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.compute_steady_state()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ops = {k: {'calls': len(v), 'seconds': sum(a.elapsed_time(e) for a, e in v) * 1e-3} for k, v in rec.items()}
    gpu = sum(o['seconds'] for o in ops.values())
    return {'native_wall_s': native_wall, 'batched_ops_s': gpu, 'native_control_s': native_wall - gpu,
            'host_loop_wall_s': wall, 'host_loop_control_s': wall - gpu, 'ops': ops,
            'note': 'batched operations timed with CUDA events in a host-loop solve of the same batch (same '
                    'operations, same order); control = wall - operations: the masks, norms, flag reads and '
                    'synchronizations of the native solvers (native_control_s) and of the host loop'}


def _tau_interp_summary(tau, tau_i, status):
    """How far the step-end ignition delays (the reference's measure) sit from the Hermite-interpolated crossing."""
    import numpy as np
    ign = (status == 2) & np.isfinite(tau_i)
    rel = (tau[ign] - tau_i[ign]) / tau_i[ign]
    return {'reactors': int(ign.sum()),
            'step_end_minus_interpolated_rel': {'median': float(np.median(rel)) if rel.size else None,
                                                'max': float(rel.max()) if rel.size else None},
            'note': 'the delay as the end of the accepted step that first has T > T0 + 400 K (the reference\'s '
                    'measure, reactors.py:774-790) against the time the cubic Hermite interpolant over that step '
                    'crosses T0 + 400 K'}


def bench_flamelet(spec, rank, stream, cpu):
    import numpy as np
    import torch
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.flamelet import FlameletBatch
    setups = W.slfm_flamelet_setups(spec, N_FLAMELETS, seed=1004 + rank)
    FlameletBatch(setups[:2]).compute_steady_state()
    b = FlameletBatch(setups)
    ns = b.ns
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out, conv, how = b.compute_steady_state()
    torch.cuda.synchronize()
    wall = max_over_ranks(time.perf_counter() - t0)
    world = int(os.environ.get('WORLD_SIZE', '1'))
    st = out.cpu().numpy()
    conv_h = conv.cpu().numpy()
    ext = []
    for f, s in enumerate(setups):
        T = st[b.offz_host[f] * ns:b.offz_host[f + 1] * ns:ns]
        ext.append(bool(np.max(T - s.linear_temperature) < 10.))
    pts = b.npts
    res = {'flamelets': N_FLAMELETS, 'points': pts, 'value': world * N_FLAMELETS / wall, 'unit': 'flamelets/s',
           'seconds': wall, 'points_per_s': world * pts / wall,
           'converged': int(conv_h.sum()), 'by_newton': int(how['newton'].sum().item()),
           'by_psitc': int(how['psitc'].sum().item()), 'by_esdirk': int(how['esdirk'].sum().item()),
           'extinguished': int(sum(ext)),
           'device_status': spec.griffon.device_status()}
    # one batched launch of each operation on the converged profiles
    x = out.clone()
    y = torch.empty_like(x)
    k = {}
    k['rhs_ms'] = _timed(lambda: b.rhs(x, out=y), stream, 3)
    k['jacobian_ms'] = _timed(lambda: b.jacobian(x), stream, 3)
    dterm = b.diffterm_tensor()
    k['jacobian_eig_ms'] = _timed(lambda: b.jacobian(x, eig=True, diffterm_per_flamelet=dterm), stream, 3)
    b.jacobian(x)
    vals = b.values.clone()
    k['matvec_ms'] = _timed(lambda: b.matvec(x, out=y), stream, 3)

    def fac():
        b.values.copy_(vals)
        b.factor()
    copy_ms = _timed(lambda: b.values.copy_(vals), stream, 3)
    k['factor_ms'] = _timed(fac, stream, 3) - copy_ms
    k['solve_ms'] = _timed(lambda: b.solve(x, out=y), stream, 3)
    hbm, hbm_src = measured_peaks()
    nvals = b.nvals
    mv_bytes = (nvals + 2 * pts * ns) * 8
    rhs_bytes = pts * 4 * ns * 8
    # per point: LU 2/3 ns^3 flops, the inverse from the LU factors 4/3 ns^3 (identity right-hand sides)
    fac_flops = pts * 2. * ns ** 3
    mv_fmas = float(nvals)  # one FMA per matrix value (diagonal blocks and the sub/super-diagonal values)
    _, issue_peak = fp64_fma_probe(20000, 32)
    k['roofline'] = {
        'matvec': {'bound': 'hbm', 'algorithmic_bytes': mv_bytes, 'achieved': mv_bytes / (k['matvec_ms'] * 1e-3)
                   / 1e9, 'peak': hbm, 'unit': 'GB/s', 'frac': mv_bytes / (k['matvec_ms'] * 1e-3) / 1e9 / hbm,
                   'peak_source': hbm_src,
                   # one FMA per 8-byte value is 0.25 flop/byte, above GB300's FP64 balance: FP64 issue binds first
                   'fp64_issue': {'warp_instr': mv_fmas / 32., 'achieved_per_s': mv_fmas / 32. / (k['matvec_ms'] * 1e-3),
                                  'peak_per_s': issue_peak,
                                  'frac': mv_fmas / 32. / (k['matvec_ms'] * 1e-3) / issue_peak,
                                  'peak_source': 'bench_fp64_fma (bench_probes.cu), measured live'}},
        'rhs_sweep': {'bound': 'fp64 (rates per point); HBM bytes reported', 'algorithmic_bytes': rhs_bytes,
                      'achieved_gbs': rhs_bytes / (k['rhs_ms'] * 1e-3) / 1e9,
                      'points_per_s': pts / (k['rhs_ms'] * 1e-3)},
        'jacobian': {'points_per_s': pts / (k['jacobian_ms'] * 1e-3),
                     'fp64_tflops_executed_est': FP64_PER_STATE[32]['flops'] * pts / (k['jacobian_ms'] * 1e-3)
                     / 1e12},
        'factor': {'bound': 'fp64 (critical path: the longest flamelet)', 'flops_per_point': 2. * ns ** 3,
                   'achieved_tflops': fac_flops / (k['factor_ms'] * 1e-3) / 1e12}}
    res['kernels'] = k
    res['time_split'] = _flamelet_time_split(setups, wall)
    if cpu:
        idx = list(range(0, N_FLAMELETS, 4))
        done, cores, dt = cpu_flamelets(setups, idx, seconds=60.)
        errs, mism = [], 0
        for kf, s_cpu, how_cpu, sec in done:
            g = st[b.offz_host[kf] * ns:b.offz_host[kf + 1] * ns]
            if s_cpu is None or not conv_h[kf]:
                mism += int((s_cpu is None) != (not conv_h[kf]))
                continue
            errs.append(float(np.max(np.abs(g[::ns] - s_cpu[::ns]) / s_cpu[::ns])))
        npts_done = sum(setups[kf].nzi for kf, *_ in done)
        res['cpu_baseline'] = {'value': len(done) / dt, 'unit': 'flamelets/s', 'cores': cores, 'kind': 'port',
                               'points_per_s': npts_done / dt,
                               'sample': f'oracle compute_steady_state (restated Newton + psitc, C++ kernels, numpy '
                                         f'eigvals) of {len(done)} of the {len(idx)} flamelets k = 0, 4, 8, ... '
                                         f'finished in {dt:.1f} s, one per core'}
        res['T_rel_err_vs_oracle'] = {'flamelets_compared': len(errs), 'max': max(errs) if errs else None,
                                      'convergence_mismatches': mism}
    return res


def _fwd_sens_sample(args):
    """CPU forward sensitivity (oracle) over the first `nsteps` recorded steps of one reactor; returns seconds."""
    q0, p, dts, nsteps = args
    import oracle as orc
    import integrate as I
    import sensitivity as SE
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    orc.set_threads(1)
    spec = ChemicalMechanismSpec.bundled('methane-gri30')
    og = orc.OracleGriffon()
    spec._populate_griffon(og)
    prob = I.ReactorProblem(og, 'isobaric', pressure=p)
    dts = dts[:nsteps]
    fs, st = SE.frozen_integrate(prob, q0, dts)
    pj = SE.ParamJacobian(spec, og, 'isobaric', p)
    t0 = time.perf_counter()
    SE.forward_sensitivity(prob, pj, q0, dts, st)
    return time.perf_counter() - t0


def bench_adjoint(spec, rank, stream, cpu):
    import numpy as np
    import torch
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.adjoint import ReactorAdjoint
    d = W.adjoint_batch(spec, N_ADJOINT, seed=1005 + rank)
    adj = ReactorAdjoint(spec, 'isobaric')
    tr = adj.forward(d['q0'][:32], d['p'][:32], 5.e-3)
    adj.backward(tr)
    del tr
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats()
    t0 = time.perf_counter()
    tr = adj.forward(d['q0'], d['p'], 5.e-3)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    g = adj.backward(tr)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    peak = torch.cuda.max_memory_allocated()
    world = int(os.environ.get('WORLD_SIZE', '1'))
    total = max_over_ranks(t2 - t0)
    steps = tr.steps.cpu().numpy()
    theta = g['theta']
    res = {'reactors': N_ADJOINT, 'parameters': int(theta.shape[2] * 2), 'outputs': ['T_end', 'tau_s'],
           'value': world * N_ADJOINT / total, 'unit': 'reactor gradients/s (650 parameters x 2 outputs)',
           'forward_s': t1 - t0, 'backward_s': t2 - t1, 'peak_memory_gb': peak / 1e9,
           'steps': {'min': int(steps.min()), 'median': float(np.median(steps)), 'max': int(steps.max())},
           'finite': bool(torch.isfinite(theta).all().item()), 'device_status': spec.griffon.device_status(),
           'central_fd_equivalent': '1300 integrations per reactor gradient'}
    if cpu:
        import multiprocessing as mp
        nsample, nst = min(16, os.cpu_count()), 12
        rec = tr.rec.cpu().numpy()
        jobs = [(d['q0'][i], d['p'][i], rec[i, :steps[i], 1], nst) for i in range(nsample)]
        ctx = mp.get_context('spawn')
        with ctx.Pool(nsample, initializer=_worker_init, initargs=(ROOT,)) as pool:
            t0 = time.perf_counter()
            secs = pool.map(_fwd_sens_sample, jobs)
            wall = time.perf_counter() - t0
        per_reactor = [secs[i] / min(nst, steps[i]) * steps[i] for i in range(nsample)]
        res['cpu_baseline'] = {'value': nsample / sum(per_reactor) * nsample, 'unit': 'reactor gradients/s',
                               'cores': nsample, 'kind': 'port',
                               'sample': f'oracle forward sensitivity (650 parameters, both outputs) over the first '
                                         f'{nst} recorded steps of {nsample} reactors, one per core ({wall:.1f} s), '
                                         f'scaled to each reactor\'s step count'}
    return res


# ---------------------------------------------------------------------------------------------- FP64 probes
# bench_probes.cu (beside this file) holds the FP64 throughput probes, compiled on their own into _build/: they are
# measurement code, not part of the library.
_PROBES = None


def build_probes():
    """Compile bench_probes.cu for sm_103a into _build/libbench_probes.so (skipped when up to date)."""
    import hashlib
    from spitfire_gb300 import build as B
    src = os.path.join(ROOT, 'bench_probes.cu')
    out_dir = os.path.join(ROOT, '_build')
    lib = os.path.join(out_dir, 'libbench_probes.so')
    stamp = lib + '.stamp'
    deps = [src] + [os.path.join(B.CSRC, f) for f in ('chem_device.cuh', 'exp_table.h', 'sf_mech.h')]
    h = hashlib.sha256(b''.join(open(f, 'rb').read() for f in deps) + ' '.join(B.ARCH).encode() +
                       os.uname().machine.encode()).hexdigest()
    if os.path.exists(lib) and os.path.exists(stamp) and open(stamp).read() == h:
        return lib
    os.makedirs(out_dir, exist_ok=True)
    subprocess.check_call([B.nvcc(), '-shared', '-Xcompiler', '-fPIC', '-O3', '-lineinfo', *B.ARCH, src,
                           '-o', lib + '.tmp'])
    os.replace(lib + '.tmp', lib)
    with open(stamp, 'w') as f:
        f.write(h)
    return lib


def _probes():
    global _PROBES
    if _PROBES is None:
        import ctypes as C
        L = C.CDLL(build_probes())
        L.bench_fp64_fma.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p,
                                     C.c_void_p]
        L.bench_fp64_dmma.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.c_void_p, C.c_void_p]
        L.bench_fp64_mixed.argtypes = [C.c_int, C.POINTER(C.c_double), C.c_void_p, C.c_void_p]
        L.bench_store.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.POINTER(C.c_double), C.c_void_p]
        L.bench_exp.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.c_void_p, C.c_void_p]
        L.bench_exp_values.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p]
        _PROBES = L
    return _PROBES


def fp64_fma_probe(iters, active_lanes=32):
    """(TFLOP/s of the active lanes, warp FP64 instructions/s) of register FMA chains on every SM."""
    import ctypes as C
    import torch
    sink = torch.zeros(1, dtype=torch.float64, device='cuda')
    tf, wi = C.c_double(), C.c_double()
    rc = _probes().bench_fp64_fma(int(iters), int(active_lanes), C.byref(tf), C.byref(wi), sink.data_ptr(),
                                  torch.cuda.current_stream().cuda_stream)
    if rc:
        raise RuntimeError(f'bench_fp64_fma failed ({rc})')
    return tf.value, wi.value


def fp64_dmma_probe(iters, which=0):
    """TFLOP/s of FP64 mma.sync (which 0: m8n8k4, 1: m16n8k16) with independent accumulators on every SM."""
    import ctypes as C
    import torch
    sink = torch.zeros(1, dtype=torch.float64, device='cuda')
    tf = C.c_double()
    rc = _probes().bench_fp64_dmma(int(iters), int(which), C.byref(tf), sink.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream)
    if rc:
        raise RuntimeError(f'bench_fp64_dmma failed ({rc})')
    return tf.value


def fp64_mixed_probe(iters):
    """TFLOP/s of a launch whose even warps run DFMA chains and odd warps FP64 m8n8k4 MMAs (equal flops)."""
    import ctypes as C
    import torch
    sink = torch.zeros(1, dtype=torch.float64, device='cuda')
    tf = C.c_double()
    rc = _probes().bench_fp64_mixed(int(iters), C.byref(tf), sink.data_ptr(), torch.cuda.current_stream().cuda_stream)
    if rc:
        raise RuntimeError(f'bench_fp64_mixed failed ({rc})')
    return tf.value


def store_probe(t, pattern):
    """GB/s of kernel stores into the tensor t (CUDA, or pinned CPU memory written over the host link)."""
    import ctypes as C
    import torch
    gbs = C.c_double()
    rc = _probes().bench_store(C.c_void_p(t.data_ptr()), t.numel() * t.element_size(), int(pattern), C.byref(gbs),
                               torch.cuda.current_stream().cuda_stream)
    if rc:
        raise RuntimeError(f'bench_store failed ({rc})')
    return gbs.value


# ---------------------------------------------------------------------------------------------- profiling cases
# Small, self-contained runs of each kernel family for ncu and quick checks:  python bench.py --profile-case <case>
#   jac        isochoric RHS + Jacobian of 8192 GRI-3.0 states (chem_kernel MODE_JAC), 3 launches
#   jac_tps    the same with the thread-per-state kernel (chem_kernel_tps MODE_JAC) at 2 resident 4-warp blocks
#              per SM, on 38912 states (one warp batch per resident warp), 2 launches
#   rates_rhs  production rates (chem_kernel_tps MODE_RATES) and the isochoric right-hand side (MODE_RHS) of 38912
#              states, thread per state at 2 resident 4-warp blocks per SM, 2 launches each
#   integrate_2048  2048 isobaric reactors of the batched-ignition distribution to ignition or 0.1 s with the
#              autotuner's shape (Griffon scratch in global slots, 6 warps per block)
#   integrate  256 isobaric reactors of the batched-ignition distribution to ignition or 0.1 s (integrate_kernel)
#   flamelet   8 steady-flamelet profiles of 64-120 points: one RHS sweep, Jacobian with eigenvalue bounds,
#              block-Thomas factorization, solve and matvec
#   adjoint    64 reactors of the adjoint distribution recorded to 1 ms, then the batched adjoint
#   adjoint_sweep  the benchmark's adjoint workload (2048 reactors to 5 ms, the thread-per-state Jacobian shape the
#              headline tunes): forward record, then one backward sweep (sf_adjoint_batch), its time printed
#   fp64issue  warp-level FP64 FMA instructions per second with 1, 2, 4, 8, 16 and 32 active lanes per warp
#   dmma       FP64 mma.sync (m8n8k4, m16n8k16) throughput beside the DFMA pipe's
#   sysmem     kernel stores into device memory and into pinned host memory (coalesced, and the thread-per-state
#              Jacobian pattern), beside cudaMemcpy device-to-host of the same 1.5 GB, on one stream and split over
#              2 and 4 streams at once
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


def case_integrate_2048():
    from spitfire_gb300 import autotune as AT
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.reactors import BatchIntegrator
    spec = _spec()
    AT.set_tuning(spec, 'integrate_scratch', 2)
    AT.set_tuning(spec, 'integrate_warps', 8)
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


def case_adjoint_sweep():
    import torch
    from spitfire_gb300 import autotune as AT
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.adjoint import ReactorAdjoint
    spec = _spec()
    AT.set_tuning(spec, 'group_jac', 1)
    AT.set_tuning(spec, 'tps_ctas', 2)
    d = W.adjoint_batch(spec, N_ADJOINT, seed=1005)
    adj = ReactorAdjoint(spec, 'isobaric')
    tr = adj.forward(d['q0'], d['p'], 5.e-3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g = adj.backward(tr)
    torch.cuda.synchronize()
    print(f'backward sweep of {N_ADJOINT} reactors: {time.perf_counter() - t0:.3f} s')
    assert bool(torch.isfinite(g['theta']).all().item())
    return spec


def case_fp64issue():
    for lanes in (1, 2, 4, 8, 16, 32):
        tf, wi = fp64_fma_probe(4000, lanes)
        print(f'active lanes {lanes:2d}: {wi:.4e} warp FP64 FMA instructions/s, {tf:.3f} TFLOP/s of useful lanes')
    return None


def case_dmma():
    tf, _ = fp64_fma_probe(20000, 32)
    print(f'FP64 FMA (DFMA pipe), all lanes: {tf:.3f} TFLOP/s')
    for which, name in ((0, 'm8n8k4'), (1, 'm16n8k16')):
        print(f'FP64 mma.sync {name}: {fp64_dmma_probe(2000 if which == 0 else 500, which):.3f} TFLOP/s')
    print(f'half the warps DFMA, half m8n8k4 (equal flops): {fp64_mixed_probe(16000):.3f} TFLOP/s')
    return None


def case_exp():
    """CUDA's exp against the library's table-driven tab_exp: FP64 instructions per call in throughput loops, and
    accuracy in ulps against numpy's long double exponential (113-bit on the Arm host, 64-bit on x86)."""
    import ctypes as C
    import numpy as np
    import torch
    L = _probes()
    sink = torch.zeros(1, dtype=torch.float64, device='cuda')
    st = torch.cuda.current_stream().cuda_stream
    _, wi = fp64_fma_probe(4000, 32)
    iters = 1024
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    calls = 4. * iters * nsm * 8 * 256
    ms = []
    for which in (0, 1, 2):
        v = C.c_double()
        if L.bench_exp(which, iters, C.byref(v), sink.data_ptr(), st):
            raise RuntimeError('bench_exp failed')
        ms.append(v.value)
    per = [(m - ms[0]) * 1e-3 * wi / (calls / 32.) for m in ms]
    print(f'warp FP64 instructions/s (bench_fp64_fma): {wi:.4e}')
    print(f'loop alone {ms[0]:.3f} ms; CUDA exp {ms[1]:.3f} ms, {per[1]:.2f} warp FP64 instructions per call beyond '
          f'the loop; tab_exp {ms[2]:.3f} ms, {per[2]:.2f}')
    rng = np.random.default_rng(7)
    n = 1 << 21
    x = np.concatenate([rng.uniform(-745.1, 709.7, n), rng.uniform(-80., 5., n), rng.uniform(-0.02, 0.02, n)])
    xd = torch.from_numpy(x).cuda()
    oc, ot = torch.empty_like(xd), torch.empty_like(xd)
    if L.bench_exp_values(xd.data_ptr(), oc.data_ptr(), ot.data_ptr(), xd.numel(), st):
        raise RuntimeError('bench_exp_values failed')
    c, t = oc.cpu().numpy(), ot.cpu().numpy()
    sel = np.arange(0, x.size, 3)
    ref = np.exp(x[sel].astype(np.longdouble))
    ok = np.isfinite(ref) & (ref >= np.longdouble(np.finfo(np.float64).tiny)) & \
        (ref < np.longdouble(np.finfo(np.float64).max))
    ulp = np.spacing(ref[ok].astype(np.float64)).astype(np.longdouble)
    print(f'accuracy on {int(ok.sum())} normal results (reference: numpy long double, '
          f'{np.finfo(np.longdouble).nmant + 1}-bit):')
    for name, v in (('CUDA exp', c), ('tab_exp', t)):
        e = np.abs((v[sel][ok].astype(np.longdouble) - ref[ok]) / ulp).astype(np.float64)
        cr = float(np.mean(v[sel][ok] == ref[ok].astype(np.float64)))
        print(f'  {name}: max {e.max():.3f} ulp, mean {e.mean():.4f} ulp, correctly rounded {cr:.4f}')
    print(f'tab_exp equal to CUDA exp bit for bit: {float(np.mean(c == t)):.4f} of {x.size}')
    special = np.array([0., -0., np.inf, -np.inf, np.nan, 709.78, -745.2, -708.5, 1e-300])
    sd = torch.from_numpy(special).cuda()
    sc, stt = torch.empty_like(sd), torch.empty_like(sd)
    L.bench_exp_values(sd.data_ptr(), sc.data_ptr(), stt.data_ptr(), sd.numel(), st)
    print('special arguments (x, CUDA exp, tab_exp):')
    for a, b, d in zip(special, sc.cpu().numpy(), stt.cpu().numpy()):
        print(f'  {a!r}: {b!r} {d!r}')
    return None


def case_sysmem():
    import torch
    n = 1536 * 1024 * 1024 // 8
    dev = torch.empty(n, dtype=torch.float64, device='cuda')
    host = torch.empty(n, dtype=torch.float64).pin_memory()
    for pattern, name in ((0, 'coalesced'), (1, 'thread-per-state blocks')):
        print(f'stores, {name}: device memory {store_probe(dev, pattern):.1f} GB/s, pinned host memory '
              f'{store_probe(host, pattern):.1f} GB/s')
    host.copy_(dev, non_blocking=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    host.copy_(dev, non_blocking=True)
    e1.record()
    e1.synchronize()
    print(f'cudaMemcpy device-to-host (pinned): {n * 8 / (e0.elapsed_time(e1) * 1e-3) / 1e9:.1f} GB/s')
    # the same bytes split over k streams at once: whether more copy engines raise the link's rate
    for k in (2, 4):
        streams = [torch.cuda.Stream() for _ in range(k)]
        part = n // k
        for rep in range(2):
            torch.cuda.synchronize()
            e0.record()
            for i, s in enumerate(streams):
                s.wait_event(e0)
                with torch.cuda.stream(s):
                    host[i * part:(i + 1) * part].copy_(dev[i * part:(i + 1) * part], non_blocking=True)
            for s in streams:
                torch.cuda.current_stream().wait_stream(s)
            e1.record()
            e1.synchronize()
        print(f'device-to-host over {k} streams at once: {part * k * 8 / (e0.elapsed_time(e1) * 1e-3) / 1e9:.1f} GB/s')
    import glob
    nodes = sorted(glob.glob('/sys/devices/system/node/node[0-9]*'))
    print(f'host: {len(os.sched_getaffinity(0))} cores in this process\'s affinity, {len(nodes)} NUMA nodes')
    return None


PROFILE_CASES = {'jac': case_jac, 'jac_tps': case_jac_tps, 'rates_rhs': case_rates_rhs,
                 'integrate_2048': case_integrate_2048, 'exp': case_exp, 'flamelet': case_flamelet,
                 'adjoint': case_adjoint, 'adjoint_sweep': case_adjoint_sweep, 'fp64issue': case_fp64issue, 'dmma': case_dmma, 'sysmem': case_sysmem}


def run_profile_case(name):
    import numpy as np  # noqa: F401  (the cases use it)
    from spitfire_gb300 import build
    build.build()
    spec = PROFILE_CASES[name]()
    status = spec.griffon.device_status() if spec is not None else 0
    print(f'{name}: done, device status {status}')
    return 0 if status == 0 else 1


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU path for this workload on the host cores, as the oracle port (its C++
    restatement of Griffon, measured here at the reference's own speed; the reference's sources are not on the GPU
    box). Every step evaluates all 65536 states' RHS + Jacobian with OpenMP over all host cores."""
    if rank != 0:
        return
    import numpy as np
    import oracle as orc
    from spitfire_gb300 import workloads as W
    from spitfire_gb300._desc import reactor_params
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    spec = ChemicalMechanismSpec.bundled('methane-gri30')
    d = W.gri_states(spec, N_STATES)
    q = W.isochoric_state(d)
    og = orc.OracleGriffon()
    spec._populate_griffon(og)
    cores = os.cpu_count()
    orc.set_threads(cores)
    P = reactor_params('isochoric')
    yin = np.zeros(spec.n_species)
    P.inflow_Y = orc._p(yin)
    per = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        og.reactor_jac_batch(P, q, 0)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            per.append(dt)
    ms = 1e3 * statistics.mean(per)
    v = N_STATES / (ms * 1e-3)
    line = {'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': 'states/s', 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic (seeded GRI-3.0 states)',
            'config': {'workload': f'GRI-3.0 isochoric RHS + analytical Jacobian, {N_STATES} states',
                       'l2': 'n/a (CPU)'},
            'cpu_baseline': {'value': v, 'unit': 'states/s', 'cores': cores, 'kind': 'port',
                             'sample': f'every step: all {N_STATES} states, OpenMP over {cores} host threads; the '
                                       f'port runs at 0.99x the unmodified reference Griffon single-threaded on the '
                                       f'same GRI states'},
            'e2e': {'value': v, 'unit': 'states/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--no-cpu', action='store_true', help='skip the CPU baseline leg')
    ap.add_argument('--profile-case', choices=sorted(PROFILE_CASES), help='run one profiling case and exit')
    ap.add_argument('--headline-only', action='store_true',
                    help='measure the headline workload (value, e2e, roofline) and skip the further blocks')
    args = ap.parse_args()
    if args.profile_case:
        sys.exit(run_profile_case(args.profile_case))
    rank, world, local = dist_env()
    if args.impl == 'reference':
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group('gloo')
        run_reference(args, rank, world)
        return

    import numpy as np
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl', device_id=torch.device('cuda', local))
    from spitfire_gb300 import _native as N
    from spitfire_gb300 import build
    from spitfire_gb300 import workloads as W
    from spitfire_gb300._desc import reactor_params
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    build.build()
    dev = torch.device('cuda', local)
    spec = ChemicalMechanismSpec.bundled('methane-gri30')
    g = spec.griffon
    d = W.gri_states(spec, N_STATES, seed=1002 + rank)
    qh = W.isochoric_state(d)
    q = torch.tensor(qh, device=dev)
    neq = q.shape[1]
    P = reactor_params('isochoric')
    rhs = torch.empty_like(q)
    J = torch.empty((N_STATES, neq * neq), dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # lanes per state of the Jacobian kernel from the autotuner, on the whole batch (not timed): a sample smaller than
    # the resident lanes would leave the thread-per-state kernel's grid mostly idle
    from spitfire_gb300 import autotune as AT
    tuned = AT.tune_chemistry(spec, qh, kinds=('jac',))
    group = tuned['group_jac'][0]
    kern = FP64_PER_STATE.get(group, {'kernel': f'chem_kernel<{group}, MODE_JAC>', 'flops': None,
                                      'warp_instr': None, 'dram_bytes': None})

    def step():
        g.reactor_jac_batch(P, q, 0, out_rhs=rhs, out_jac=J)

    for _ in range(max(args.warmup, 3)):
        step()
    barrier()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    barrier()
    ms = max_over_ranks(statistics.mean(times), dev)
    value = world * N_STATES / (ms * 1e-3)

    # ---------------- end to end through the public API (host buffers)
    qpin = torch.from_numpy(qh).pin_memory()
    rhs_h = torch.empty((N_STATES, neq), dtype=torch.float64).pin_memory()
    J_h = torch.empty((N_STATES, neq * neq), dtype=torch.float64).pin_memory()

    def e2e_step():
        # the host-buffer entry point (sf_reactor_jac_host_batch): states in, results out, the copies back of one
        # chunk overlapping the next chunk's kernel
        g.reactor_jac_host_batch(P, qpin, rhs_h, J_h)

    for _ in range(max(args.warmup, 3)):
        e2e_step()
    torch.cuda.synchronize()
    barrier()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    ev[0].record(stream)
    for k in range(args.steps):
        e2e_step()
        ev[k + 1].record(stream)
    ev[-1].synchronize()
    e2e_steps = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    e2e_ms = max_over_ranks(ev[0].elapsed_time(ev[-1]) / args.steps, dev)
    e2e = {'value': world * N_STATES / (e2e_ms * 1e-3), 'unit': 'states/s', 'ms_per_step': e2e_ms,
           'ms_per_step_min_median_max': [min(e2e_steps), statistics.median(e2e_steps), max(e2e_steps)],
           'ms_each_step': [round(x, 3) for x in e2e_steps],
           'h2d_bytes_per_step': qpin.numel() * 8, 'd2h_bytes_per_step': (rhs_h.numel() + J_h.numel()) * 8,
           'api': 'PyCombustionKernels.reactor_jac_host_batch -> sf_reactor_jac_host_batch (pinned host buffers; '
                  'chunks of one resident wave, device-to-host copies overlapping the next chunk)'}

    # ---------------- comparison point: the plain single-state GPU form on the same states
    ws = torch.empty(N.load().sf_reactor_jac_plain_workspace_size(g.handle, N_STATES) // 8 + 1,
                     dtype=torch.float64, device=dev)
    g.reactor_jac_plain_batch(P, q, workspace=ws)
    torch.cuda.synchronize()
    plain_runs = []
    for _ in range(3):  # median of three launches
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        g.reactor_jac_plain_batch(P, q, workspace=ws)
        e1.record(stream)
        e1.synchronize()
        plain_runs.append(e0.elapsed_time(e1))
    plain_ms = sorted(plain_runs)[1]
    del ws

    # ---------------- roofline (FP64 pipe)
    peak_tflops, issue_peak = fp64_fma_probe(20000, 32)
    dense = griffon_dense_flops(spec)
    algo = kern['flops']
    roof = {'bound': 'fp64', 'unit': 'TFLOP/s', 'peak': peak_tflops,
            'peak_source': 'measured live by bench_probes.cu bench_fp64_fma (FP64 FMA chains on every SM); the '
                           'measured-peaks file has no FP64 figure',
            'kernel': kern['kernel']}
    if algo:
        roof['achieved'] = algo * N_STATES / (ms * 1e-3) / 1e12
        roof['frac'] = roof['achieved'] / peak_tflops
        roof['flops_per_state'] = algo
    else:
        roof['achieved'] = None
        roof['frac'] = None
    # DRAM bytes of one launch: the ncu figure per state times the states of a launch
    roof['traffic'] = kern['dram_bytes'] * N_STATES if kern.get('dram_bytes') else None
    roof['traffic_source'] = 'ncu dram__bytes_read.sum + dram__bytes_write.sum per state on the profiling case ' \
                             '(python bench.py --profile-case jac_tps | jac), scaled to the launch'
    if kern['warp_instr']:
        ach_issue = kern['warp_instr'] * N_STATES / (ms * 1e-3)
        roof['fp64_issue'] = {'unit': 'warp FP64 instructions/s', 'per_state': kern['warp_instr'],
                              'achieved': ach_issue, 'peak': issue_peak, 'frac': ach_issue / issue_peak,
                              'note': 'GB300 charges FP64 per warp instruction whatever the active lanes; this is '
                                      'the pipe-occupancy roofline, the TFLOP/s one above counts useful lanes'}
    roof['griffon_dense_flops_per_state'] = dense
    roof['griffon_dense_equiv_tflops'] = dense * N_STATES / (ms * 1e-3) / 1e12
    hbm_bytes = N_STATES * (neq + neq + neq * neq) * 8
    roof['hbm'] = {'algorithmic_bytes': hbm_bytes, 'achieved_gbs': hbm_bytes / (ms * 1e-3) / 1e9}

    # ---------------- further workloads
    cpu = rank == 0 and world == 1 and not args.no_cpu
    extra = {}
    if not args.headline_only:
        gh = torch.tensor(d['gamma_h'], dtype=torch.float64, device=dev)
        extra['newton'] = bench_newton(q, rhs, J, gh, stream)
        del J, J_h
        torch.cuda.empty_cache()
        extra['h2_small'] = bench_h2(rank, stream, cpu)
        extra['ignition'] = bench_ignition(spec, rank, stream, cpu)
        extra['flamelet'] = bench_flamelet(spec, rank, stream, cpu)
        extra['adjoint'] = bench_adjoint(spec, rank, stream, cpu)

    line = {'metric': METRIC, 'value': value, 'unit': 'states/s', 'n_gpus': world, 'steps': args.steps,
            'warmup': max(args.warmup, 3), 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic (seeded GRI-3.0 states of the workloads.gri_states distribution)',
            'config': {'workload': f'GRI-3.0 isochoric RHS + analytical Jacobian (rates option 0), {N_STATES} '
                                   f'states per GPU', 'mechanism': 'methane-gri30 (53 species, 325 reactions)',
                       'states_per_gpu': N_STATES, 'parallelism': f'replicas x{world}',
                       'l2': 'flushed between steps (256 MB write outside the timed events)'},
            'e2e': e2e, 'roofline': roof, 'clocks': clk.summary(), 'gpu_launches': args.steps,
            'autotune': {'group_jac': group, 'tps_ctas': tuned.get('tps_ctas', (None,))[0],
                         'candidates_ms': {str(k): v for k, v in tuned['group_jac'][1].items()}},
            'plain_gpu_form': {'value': N_STATES / (plain_ms * 1e-3), 'unit': 'states/s', 'ms': plain_ms,
                               'speedup_batched_over_plain': plain_ms / ms},
            **extra}
    if rank == 0 and world == 1 and not args.no_cpu:
        line['cpu_baseline'] = cpu_baseline(spec, qh)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == '__main__':
    main()
