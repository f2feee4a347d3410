"""Benchmark of the GB300 Griffon hot path; prints one JSON line.

Workload (one "step"): the analytical isochoric reactor right-hand side + Jacobian of GRI-3.0 (53 species,
325 reactions) on 65536 seeded states (T ~ U(600, 2800) K, p log-uniform 1-40 atm, Y = 0.7 Dir + 0.3
complete-combustion profile; spitfire_gb300.workloads.gri_states). One step = one batched evaluation of all states.

  value      states/s of the batched kernel, inputs resident in HBM (L2 flushed between steps by writing a
             256 MB buffer outside the timed events)
  e2e        states/s through the public API with host buffers: every step copies the states host->device (pinned)
             and the RHS + Jacobian device->host, inside the timed region
  roofline   the kernel is FP64-pipe bound: achieved = executed FP64 flops per state (counted by ncu, see
             profiles/) x states / kernel time, peak = FP64 FMA throughput measured live by sf_fp64_peak_probe
  cpu_baseline / --impl reference: the oracle (C++ restatement of Griffon, OpenMP over all host cores) on the
             same states

Multi-GPU: states are independent, so each rank evaluates its own 65536-state batch (weak scaling, no collective).
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

METRIC = 'batched ignitions/s at 1e-6 rel τ_ign err; RHS+Jac states/s vs plain & CPU'
N_STATES = 65536
# executed FP64 flops per GRI state of the batched Jacobian kernel (thread-level DADD + DMUL + 2*DFMA counted by
# ncu, profiles/chem_kernel_jac_gri30_8192.md)
FP64_FLOPS_PER_STATE = float(os.environ.get('SF_FP64_FLOPS_PER_STATE', '104960'))


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


def dist_env():
    rank = int(os.environ.get('RANK', '0'))
    world = int(os.environ.get('WORLD_SIZE', '1'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return rank, world, local


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


def run_reference(args, rank, world):
    """--impl reference: the oracle C++ restatement of Griffon on the host cores (the reference's own code path
    cannot run on the GPU machine: it is not present there)."""
    if rank != 0:
        return
    import numpy as np
    from spitfire_gb300 import workloads as W
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    spec = ChemicalMechanismSpec.bundled('methane-gri30')
    d = W.gri_states(spec, N_STATES)
    q = W.isochoric_state(d)
    per = []
    base = None
    for k in range(args.warmup + args.steps):
        b = cpu_baseline(spec, q, seconds=max(1.0, 20.0 / max(args.steps, 1)))
        if k >= args.warmup:
            per.append(b['value'])
            base = b
    v = statistics.mean(per)
    line = {'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': 'states/s', 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': 1e3 * N_STATES / v,
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic (seeded GRI-3.0 states)',
            'config': {'workload': f'GRI-3.0 isochoric RHS + analytical Jacobian, {N_STATES} states',
                       'l2': 'n/a (CPU)'},
            'cpu_baseline': {**base, 'value': v},
            'e2e': {'value': v, 'unit': 'states/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--no-cpu', action='store_true', help='skip the CPU baseline leg')
    args = ap.parse_args()
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
    ms = statistics.mean(times)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * N_STATES / (ms * 1e-3)

    # ---------------- end to end through the public API (host buffers)
    qpin = torch.from_numpy(qh).pin_memory()
    rhs_h = torch.empty((N_STATES, neq), dtype=torch.float64).pin_memory()
    J_h = torch.empty((N_STATES, neq * neq), dtype=torch.float64).pin_memory()

    def e2e_step():
        q.copy_(qpin, non_blocking=True)
        g.reactor_jac_batch(P, q, 0, out_rhs=rhs, out_jac=J)
        rhs_h.copy_(rhs, non_blocking=True)
        J_h.copy_(J, non_blocking=True)

    for _ in range(2):
        e2e_step()
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    e1.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e = {'value': world * N_STATES / (e2e_ms * 1e-3), 'unit': 'states/s', 'ms_per_step': e2e_ms,
           'h2d_bytes_per_step': qpin.numel() * 8, 'd2h_bytes_per_step': (rhs_h.numel() + J_h.numel()) * 8}

    # ---------------- comparison point: the plain single-state GPU form on the same states
    ws = torch.empty(N.load().sf_reactor_jac_plain_workspace_size(g.handle, N_STATES) // 8 + 1,
                     dtype=torch.float64, device=dev)
    g.reactor_jac_plain_batch(P, q, workspace=ws)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    g.reactor_jac_plain_batch(P, q, workspace=ws)
    e1.record(stream)
    e1.synchronize()
    plain_ms = e0.elapsed_time(e1)
    del ws

    # ---------------- roofline (FP64 pipe)
    sink = torch.zeros(1, dtype=torch.float64, device=dev)
    import ctypes as C
    peak = C.c_double()
    N.check(N.load().sf_fp64_peak_probe(20000, C.byref(peak), N.ptr(sink), N.stream_handle()))
    dense = griffon_dense_flops(spec)
    algo = FP64_FLOPS_PER_STATE
    roof = {'bound': 'fp64', 'unit': 'TFLOP/s', 'peak': peak.value,
            'peak_source': 'measured live by sf_fp64_peak_probe (FP64 FMA chains on every SM); the measured-peaks '
                           'file has no FP64 figure',
            'kernel': 'chem_kernel<32, MODE_JAC>'}
    if algo:
        roof['achieved'] = algo * N_STATES / (ms * 1e-3) / 1e12
        roof['frac'] = roof['achieved'] / peak.value
        roof['flops_per_state'] = algo
    else:
        roof['achieved'] = None
        roof['frac'] = None
    roof['traffic'] = None
    roof['griffon_dense_flops_per_state'] = dense
    roof['griffon_dense_equiv_tflops'] = dense * N_STATES / (ms * 1e-3) / 1e12
    hbm_bytes = N_STATES * (neq + neq + neq * neq) * 8
    roof['hbm'] = {'algorithmic_bytes': hbm_bytes, 'achieved_gbs': hbm_bytes / (ms * 1e-3) / 1e9}

    line = {'metric': METRIC, 'value': value, 'unit': 'states/s', 'n_gpus': world, 'steps': args.steps,
            'warmup': max(args.warmup, 3), 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic (seeded GRI-3.0 states, config 2 distribution)',
            'config': {'workload': f'GRI-3.0 isochoric RHS + analytical Jacobian (rates option 0), {N_STATES} '
                                   f'states per GPU', 'mechanism': 'methane-gri30 (53 species, 325 reactions)',
                       'states_per_gpu': N_STATES, 'parallelism': f'replicas x{world}',
                       'l2': 'flushed between steps (256 MB write outside the timed events)'},
            'e2e': e2e, 'roofline': roof, 'clocks': clk.summary(), 'gpu_launches': args.steps,
            'plain_gpu_form': {'value': N_STATES / (plain_ms * 1e-3), 'unit': 'states/s', 'ms': plain_ms,
                               'speedup_batched_over_plain': plain_ms / ms}}
    if rank == 0 and world == 1 and not args.no_cpu:
        line['cpu_baseline'] = cpu_baseline(spec, qh)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == '__main__':
    main()
