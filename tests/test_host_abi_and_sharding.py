"""CPU: the C-ABI library loads and exports every function include/spitfire_gb300.h declares (no compute calls),
the host-side batching logic, and the multi-rank sharding path as world_size-2 gloo process groups."""
import os
import re
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, 'include', 'spitfire_gb300.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'^\s*(?:const\s+)?\w+\s*\**\s*(sf_\w+)\s*\(', src, flags=re.M)))


def test_library_exports_every_declared_symbol():
    import ctypes as C
    from spitfire_gb300 import _native as N
    from spitfire_gb300 import build
    build.build()
    names = _declared()
    assert len(names) >= 25, names
    lib = C.CDLL(N.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the binding declares every one of them too
    assert set(names) <= set(N.EXPORTED) | {'sf_last_error', 'sf_version'}, set(names) - set(N.EXPORTED)
    L = N.load()
    assert L.sf_version().decode()
    assert L.sf_last_error() is not None


def test_argument_errors_are_reported_without_a_device():
    """Entry points validate arguments before touching the device: null pointers come back as
    SF_ERR_INVALID_ARGUMENT with a message, no CUDA call made."""
    import ctypes as C
    from spitfire_gb300 import _native as N
    L = N.load()
    assert L.sf_flamelet_stencils(None, None, 0, None, None, None, None, None, None, None) == 1
    assert 'bad argument' in L.sf_last_error().decode()
    assert L.sf_btddod_matvec_batch(0, 0, None, None, None, None, None, None, None, None) == 1
    assert L.sf_btddod_solve_batch(0, 0, None, None, None, None, None, None, None, None, None, None) == 1


def test_c_caller_compiles_links_and_gets_status_codes(tmp_path):
    """tests/c_abi/abi_smoke.c, plain C99 against include/spitfire_gb300.h, linked to the library by name: the
    header is valid C and a C caller gets the status codes and messages without a GPU."""
    import shutil
    import subprocess
    from spitfire_gb300 import _native as N
    from spitfire_gb300 import build
    build.build()
    gcc = shutil.which('gcc')
    if gcc is None:
        pytest.skip('no C compiler')
    exe = str(tmp_path / 'abi_smoke')
    libdir = os.path.dirname(N.LIB_PATH)
    subprocess.run([gcc, '-std=c99', '-Wall', '-Werror', '-I', os.path.join(ROOT, 'include'),
                    os.path.join(ROOT, 'tests', 'c_abi', 'abi_smoke.c'), '-L', libdir, '-lspitfire_gb300',
                    '-Wl,-rpath,' + libdir, '-o', exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith('OK'), r.stdout


def test_shard_ranges_cover_contiguously():
    from spitfire_gb300.sharding import shard_range
    for n in (0, 1, 7, 8192, 65537):
        for world in (1, 2, 3, 8):
            spans = [shard_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [hi - lo for lo, hi in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q, ret):
    import sys
    sys.path[:0] = [ROOT, os.path.join(ROOT, 'oracle')]
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import oracle as orc
    from spitfire_gb300._desc import reactor_params
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    from spitfire_gb300.sharding import dist_env, gather_rows, max_over_ranks, shard_range, sum_over_ranks
    dist.init_process_group('gloo')
    r, w, _ = dist_env()
    spec = ChemicalMechanismSpec.bundled('h2-burke')
    og = orc.OracleGriffon()
    spec._populate_griffon(og)
    orc.set_threads(1)
    lo, hi = shard_range(q.shape[0], r, w)
    P = reactor_params('isochoric')
    yin = np.zeros(spec.n_species)
    P.inflow_Y = orc._p(yin)
    rhs, J = og.reactor_jac_batch(P, q[lo:hi], 0)
    full = gather_rows(np.hstack([rhs, J]), q.shape[0])
    t = max_over_ranks(0.5 + r)
    n = sum_over_ranks(hi - lo)
    if r == 0:
        ret.put((full, t, n))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_sharding_matches_single_process():
    """Each of 2 gloo ranks evaluates its contiguous slice of 37 states (uneven split); the host-side gather gives
    exactly the single-process result, the max-over-ranks time is the slower rank's, the unit count adds up."""
    import multiprocessing as mp
    import oracle as orc
    from spitfire_gb300 import workloads as W
    from spitfire_gb300._desc import reactor_params
    from spitfire_gb300.mechanism import ChemicalMechanismSpec
    spec = ChemicalMechanismSpec.bundled('h2-burke')
    q = W.isochoric_state(W.h2_states(spec, 37, seed=3))
    ctx = mp.get_context('spawn')
    ret = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q, ret)) for r in range(2)]
    for p in procs:
        p.start()
    full, t, n = ret.get(timeout=240)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    og = orc.OracleGriffon()
    spec._populate_griffon(og)
    P = reactor_params('isochoric')
    yin = np.zeros(spec.n_species)
    P.inflow_Y = orc._p(yin)
    rhs, J = og.reactor_jac_batch(P, q, 0)
    assert np.array_equal(full, np.hstack([rhs, J]))
    assert t == 1.5 and n == 37


def test_integrator_shape_choice_prefers_more_warps_among_near_ties():
    """The tuner keeps the shape with the most warps per block among those within 2 % of the fastest on its sample
    (larger shapes gain on batches larger than the sample), and the fastest shape otherwise."""
    from spitfire_gb300.autotune import pick_integrator_shape
    times = {(3, 1): 7982.8, (3, 2): 4204.8, (1, 3): 2994.2, (1, 5): 2447.3, (2, 4): 2214.2, (2, 6): 1971.6,
             (2, 8): 1984.3}
    assert pick_integrator_shape(times) == (2, 8)
    times[(2, 8)] = 2030.
    assert pick_integrator_shape(times) == (2, 6)
    assert pick_integrator_shape({(1, 5): 10., (2, 5): 10.1, (2, 4): 9.9}) == (1, 5)
    assert pick_integrator_shape({(2, 6): 5.}) == (2, 6)
