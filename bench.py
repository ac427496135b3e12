#!/usr/bin/env python
'''
Benchmark of the block-sparse contraction path: the two-site DMRG effective-Hamiltonian matvec
`einsum('EPaqj,JRSFb,AQsb->EPrf', head, tail, theta)` of a U(1) spin-1/2 Heisenberg chain at bond
chi = 256 (17 Sz sectors q = -8..8 with multiplets ~ exp(-q^2/8) summing to 256, MPO bond w = 5,
physical d = 2, theta in the Sz = 0 sector), inputs N(0, 1) float64 from a seed.

A step is one matvec through the public API, with the operator (head, tail) prepared once as a
Lanczos window uses it and a different resident vector every step.  L2 (129 MB) is flushed between
timed steps by writing a 256 MB buffer, and each step is timed alone with CUDA events on the
launching stream.  The headline form is split precision (6 bf16 slices by default); the same loop
times the grouped FP64 form and the per-block FP64 form (one cuBLAS call per block pair) on the same
inputs.  The DMRG section times one sweep of the L = 64, chi = 256, n_iter = 10 Heisenberg chain in
each form from one FP64 state, with the energy differences.  Prints ONE JSON line (rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision P] [--impl reference]
                    [--dmrg-length L] [--chi X] [--workload matvec|svd|recoupling|windows|dmrg]

Other workloads print a line of their own: recoupling (the SU(2) and Fibonacci recoupling einsums
at their named sizes), windows (64 batched windows of drawn bonds), svd (the split of a two-site
tensor), dmrg (the DMRG sweeps of every form at --dmrg-length sites and bond --chi).

--impl reference times the reference's CPU path for the same workload on the host cores: the
oracle port of tentorch's einsum (oracle/engine.py), a bounded sample of matvecs.  With N > 1 (one
process per GPU under torchrun) every rank runs an independent replica; the path has no exchange
between windows, so there is no collective on the data path.
'''
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = 'DMRG s/sweep & matvecs/s (U(1) χ=256) vs plain FP64 on same GPU at ΔE≤1e-10'
WORKLOAD = 'u1_heisenberg_twosite_matvec_chi256'
CHI = 256
SEED = 0
MATVEC = 'EPaqj,JRSFb,AQsb->EPrf'  # the two-site matvec (tentorch/algorithms/dmrg.py:118)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type = int, default = 1)
    p.add_argument('--steps', type = int, default = 1000)
    p.add_argument('--warmup', type = int, default = 10)
    p.add_argument('--impl', default = 'gb300', choices = ['gb300', 'reference'])
    p.add_argument('--precision', type = int, default = 6,
                   help = 'the headline form: k bf16 slices (1..8) or 0 for FP64 block products; 6 slices give '
                          '1.4e-12 relative on the matvec and |dE| ~ 7e-12 over a sweep')
    p.add_argument('--chi', type = int, default = CHI)
    p.add_argument('--cpu-sample', type = int, default = 20, help = 'matvecs in the CPU baseline sample')
    p.add_argument('--dmrg-length', type = int, default = 64, help = 'chain of the DMRG sweep timing (0: skip)')
    p.add_argument('--dmrg-iter', type = int, default = 10, help = 'Lanczos steps per window in the DMRG timing')
    p.add_argument('--dmrg-warm', type = int, default = 4,
                   help = 'FP64 sweeps before the timed sweeps (four bring every bond of the L = 64 chain to chi = 256)')
    p.add_argument('--workload', default = 'matvec', choices = ['matvec', 'svd', 'recoupling', 'windows', 'dmrg'],
                   help = 'matvec: the headline line; svd: the truncating split of a two-site tensor; recoupling: '
                          'the SU(2) / Fibonacci einsum; windows: 64 batched matvecs in a CUDA graph')
    return p.parse_args()


def config(args, precision):
    return {'workload': WORKLOAD, 'chi': args.chi, 'sectors': 17, 'mpo_bond': 5, 'physical': 2,
            'equation': 'EPaqj,JRSFb,AQsb->EPrf', 'block_products': 'fp64' if precision == 0 else f'bf16x{precision} split',
            'l2': 'flushed between timed steps (256 MB write)', 'inputs': f'N(0,1) float64, seed {SEED}',
            'parallelism': f'replicas x{args.gpus}'}


def job_rate(total_ms, steps, world, device = 'cpu'):
    """The whole job's rate over `world` replicas that each ran `steps` steps: the slowest rank's
    time (max over ranks, so every rank returns the same numbers) and the units all ranks processed
    per second of it."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([total_ms], dtype = torch.float64, device = device)
        dist.all_reduce(t, op = dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return total_ms, world * steps / (total_ms / 1e3)


def bond_multiplicities(chi, qmax = 8):
    """The bond of the matvec workload: U(1) charges 2q for q = -qmax..qmax, one multiplet each and
    the rest apportioned proportional to exp(-q^2/8): floors first, the leftover in +-q pairs by
    descending fractional part (ties to the smaller |q|), an odd leftover to q = 0.  Symmetric in q."""
    qs = list(range(-qmax, qmax + 1))
    weight = {q: math.exp(-q * q / 8) for q in qs}
    share = {q: (chi - len(qs)) * weight[q] / sum(weight.values()) for q in qs}
    mult = {q: 1 + int(share[q]) for q in qs}
    left = chi - sum(mult.values())
    for q in sorted(range(1, qmax + 1), key = lambda q: (int(share[q]) - share[q], q)):
        if left >= 2:
            mult[q] += 1
            mult[-q] += 1
            left -= 2
    mult[0] += left
    return [(2 * q,) for q in qs], [mult[q] for q in qs]


def matvec_operands(tg, torch, device, chi, seed):
    """One two-site window of the matvec workload on the device: environments L, R = (bond, w | bond)
    and theta = (bond, phys | phys, bond) at the trivial charge, entries N(0, 1) float64 drawn in
    block-key order from `torch.Generator().manual_seed(seed)` (L, then R, then theta), the bulk
    site W of the Heisenberg MPO, and head = einsum('EIa,IPqj->EPaqj', L, W), tail =
    einsum('JRsk,Fkb->JRSFb', W, R) as tentorch/algorithms/dmrg.py:113-114 builds them."""
    cat = tg.u1
    site = tg.heisenberg(cat, 4, dtype = torch.float64, device = device).tensors[1]
    w, phys = site.codomain[0], site.codomain[1]
    bond = tg.Leg(cat, *bond_multiplicities(chi))
    gen = torch.Generator().manual_seed(seed)

    def filled(cod, dom):
        t = tg.Tensor(cat, cod, dom, (0,), dtype = torch.float64, device = device)
        for block in t.to_tuple()[3].values():
            block.copy_(torch.randn(block.shape, dtype = torch.float64, generator = gen))
        return t
    left, right = filled([bond, w], [bond]), filled([bond, w], [bond])
    theta = filled([bond, phys], [phys, bond])
    head = tg.einsum('EIa,IPqj->EPaqj', left, site)
    tail = tg.einsum('JRsk,Fkb->JRSFb', site, right)
    return head, tail, theta


def to_oracle(orc, t):
    """The oracle's copy of a device tensor (same legs, same blocks), for checking a result."""
    import numpy as np
    legs = lambda ls: [orc.Leg(orc.u1, list(l.sectors), list(l.multiplicities)) for l in ls]
    out = orc.Tensor(orc.u1, legs(t.codomain), legs(t.domain), tuple(t.qtotal), np.float64)
    for key in out.blocks:
        out.blocks[key][...] = t.block(*key).cpu().numpy()
    return out


# ---------------------------------------------------------------------------------------------
# the CPU baseline (oracle port of the reference's einsum)
# ---------------------------------------------------------------------------------------------


def cpu_matvecs(chi, count, warmup = 1):
    '''Time `count` matvecs of the oracle on the host after `warmup` untimed ones (the first builds
    its plans); returns (matvecs/s, seconds, count).'''
    from oracle import engine as orc
    head, tail, theta = orc.matvec_inputs(chi, seed = SEED)
    for _ in range(max(1, warmup)):
        orc.einsum(orc.MATVEC, head, tail, theta)
    start = time.perf_counter()
    for _ in range(count):
        orc.einsum(orc.MATVEC, head, tail, theta)
    elapsed = time.perf_counter() - start
    return count / elapsed, elapsed, count


def cpu_matvecs_one_thread(chi, count):
    '''The same sample with one BLAS thread, in a child process (the thread count of numpy's BLAS is
    fixed when it loads); (matvecs/s, seconds, count), or None when the child fails.'''
    env = dict(os.environ, OMP_NUM_THREADS = '1', OPENBLAS_NUM_THREADS = '1', MKL_NUM_THREADS = '1')
    code = f'import sys, json; sys.path.insert(0, {HERE!r}); import bench; print(json.dumps(bench.cpu_matvecs({chi}, {count})))'
    try:
        done = subprocess.run([sys.executable, '-c', code], env = env, capture_output = True, text = True, timeout = 600)
        return tuple(json.loads(done.stdout.strip().splitlines()[-1]))
    except Exception:
        return None


def run_reference(args, rank, world):
    if rank != 0:
        return
    # the arm's own steps and warm-up, a step one matvec (~0.15 s on the 16 Grace cores: the default
    # 1000 steps take ~2.5 minutes)
    count, warm = max(1, args.steps), max(1, args.warmup)
    value, elapsed, n = cpu_matvecs(args.chi, count, warm)
    cores = os.cpu_count()
    line = {'metric': METRIC, 'value': value, 'unit': 'matvecs/s', 'n_gpus': args.gpus, 'steps': n,
            'warmup': warm, 'ms_per_step': 1e3 * elapsed / n, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic', 'impl': 'reference',
            'config': config(args, 0),
            'cpu_baseline': {'value': value, 'unit': 'matvecs/s', 'cores': cores, 'kind': 'port',
                             'sample': f'{n} matvecs of the oracle port of tentorch einsum (numpy; scatter '
                                       f'single-threaded, block products on {cores} BLAS threads)'},
            'e2e': {'value': value, 'unit': 'matvecs/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush = True)


# ---------------------------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------------------------


class Clocks:
    FIELDS = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,'
              'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
              'clocks_event_reasons.sw_power_cap')

    def __init__(self, index):
        self.proc = None
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(index), f'--query-gpu={self.FIELDS}',
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout = subprocess.PIPE, stderr = subprocess.DEVNULL, text = True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        time.sleep(0.25)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout = 10)
        sm, sm_max, reasons = [], [], set()
        names = ('hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap')
        for row in out.strip().splitlines():
            parts = [x.strip() for x in row.split(',')]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                sm_max.append(float(parts[1]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[3:7]):
                if flag.lower().startswith('active'):
                    reasons.add(name)
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': max(sm_max) if sm_max else None,
                'reasons': sorted(reasons), 'samples': len(sm)}


# ---------------------------------------------------------------------------------------------
# the GPU arm
# ---------------------------------------------------------------------------------------------


def fp64_peak_tflops(torch, device):
    '''cuBLAS DGEMM 4096^3, best of 3: the FP64 roofline denominator (not in MEASURED_PEAKS.json).'''
    a = torch.randn(4096, 4096, dtype = torch.float64, device = device)
    b = torch.randn(4096, 4096, dtype = torch.float64, device = device)
    torch.matmul(a, b)
    torch.cuda.synchronize(device)
    best = float('inf')
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing = True), torch.cuda.Event(enable_timing = True)
        s.record()
        torch.matmul(a, b)
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    return 2 * 4096 ** 3 / best / 1e12


def measured_peaks():
    path = os.path.join(HERE, 'MEASURED_PEAKS.json')
    if os.path.exists(path):
        with open(path) as handle:
            return json.load(handle), 'measured'
    return {'hbm_gbs': 6800.0, 'bf16_tflops': 1900.0}, 'fallback'


def ncu_traffic(kernel):
    '''DRAM bytes of a kernel per matvec (its two launches) from the committed ncu summary, or None.'''
    path = os.path.join(HERE, 'profiles', 'traffic.json')
    if not os.path.exists(path):
        return None
    with open(path) as handle:
        return json.load(handle).get(kernel)


KIND_NAMES = {0: 'memset', 1: 'gather_kernel', 2: 'runs_kernel', 3: None, 4: 'add_f64_kernel', 5: 'memcpy',
              6: 'tiles_kernel', 7: 'chain_fp64_kernel'}


def gemm_kernel_name(precision):
    return {0: 'gemm_dmma_kernel', -1: 'cublas_dgemm'}.get(precision, 'gemm_split_kernel')


def launches_of(kind, precision):
    """Our kernel launches one op of this kind makes (a GEMM: the grouped kernel, plus the slicing
    kernel in split precision; the per-block form's cuBLAS calls are not ours)."""
    if kind == 3:
        return {0: 1, -1: 0}.get(precision, 2)
    return 1 if kind in (1, 2, 4, 6, 7) else 0


def dmrg_sweeps(tg, torch, device, precision, length, chi, n_iter, warm, forms = None):
    """The two-site DMRG of the U(1) Heisenberg chain (tentorch/algorithms/dmrg.py) timed per sweep
    in each form from one FP64 state: `warm` FP64 sweeps grow the bond to chi, then each form
    runs one sweep from a copy of that state, with the plan caches cleared first so that every
    form compiles its plans inside its sweep, and then the next sweep of its run with the plans
    kept (`s_per_sweep_continued`: the steady state of a long run, where the shapes recur).  Forms: split (grouped kernels, the Lanczos matvec in
    split precision), split_all_products_s7 (every block product of the sweep in seven slices),
    bf16x3_fp64_ritz (three slices, the window's energy the FP64 Rayleigh
    quotient of the Ritz vector), fp64_grouped (the grouped kernels in FP64) and fp64_per_block (one
    cuBLAS call per block pair and one SVD per block, as the reference runs on a CUDA device).  Wall time
    around the sweep, the device synchronised on both sides.  (At six slices every block product in
    split precision moves the sweep energy by ~2e-10, outside the bar; seven slices carry 2^-7 of
    that error.)"""
    from tentorch_gb300 import networks as nw
    from tentorch_gb300 import linalg as la
    from tentorch_gb300.linalg import PER_BLOCK, cached_plans, clear_plans
    # the reference's own float64 run of this chain and seed (sweep energies, per sweep)
    golden_path = os.path.join(HERE, 'tests', 'golden', 'dmrg_chi256.json')
    golden = None
    if length == 64 and chi == 256 and n_iter == 10 and os.path.exists(golden_path):
        golden = [s['energy'] for s in json.load(open(golden_path))['sweeps']]
    tg.set_precision(0)
    driver = nw.DMRG(nw.Model(length, cat = tg.u1), max_bond_dim = chi, n_iter = n_iter, dtype = torch.float64,
                     device = device, generator = torch.Generator().manual_seed(SEED), precision = 0)
    start = time.perf_counter()
    for _ in range(warm):
        driver.sweep()
    warm_s = time.perf_counter() - start
    snapshot = ([t.clone() for t in driver.state.tensors], driver.state.center)
    out = {}
    if forms is None:
        forms = (('fp64_grouped', 0, 'gesvd', False), ('split', precision, 'gesvd', False),
                 ('split_all_products_s7', 7, 'gesvd', False, True),
                 ('bf16x3_fp64_ritz', 3, 'gesvd', True), ('fp64_per_block', PER_BLOCK, 'gesvd', False),
                 ('fp64_per_block_default_svd', PER_BLOCK, None, False))
    for name, form, svd_driver, refine, *options in forms:
        driver.state.tensors = [t.clone() for t in snapshot[0]]
        driver.state.center = snapshot[1]
        driver.precision = form
        driver.refine_energy = refine
        # every block product of the sweep in split precision (environments, head, tail, the
        # two-site contraction), not only the Lanczos matvec
        driver.all_products = bool(options and options[0])
        la.PER_BLOCK_SVD_DRIVER = svd_driver
        tg.set_precision(PER_BLOCK if form == PER_BLOCK else 0)
        clear_plans()
        mv0 = driver.matvecs
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        energy, lost = driver.sweep()
        torch.cuda.synchronize(device)
        elapsed = time.perf_counter() - t0
        tg.set_precision(0)
        # the energy of the state the sweep left, evaluated in FP64
        check = driver.energy().real
        out[name] = {'s_per_sweep': elapsed, 'energy': energy, 'energy_fp64_check': check,
                     'discarded': lost, 'matvecs': driver.matvecs - mv0, 'max_bond': max(driver.state.bond_dims),
                     'svd': 'engine Jacobi (batched)' if form != PER_BLOCK else f'torch.linalg.svd per block, driver {svd_driver}',
                     'refined_energy': refine, 'all_products': driver.all_products}
        if golden is not None:
            out[name]['delta_e_vs_reference'] = abs(energy - golden[warm])
        if svd_driver is None:
            # the per-block form as the reference runs on a CUDA device (torch's default cuSOLVER
            # method): one sweep, for the record
            la.PER_BLOCK_SVD_DRIVER = 'gesvd'
            tg.set_precision(0)
            continue
        # the next sweep of the same run, its plans cached by the first where the shapes recur
        # (as in a long run); it compiles only the shapes that the truncations changed
        tg.set_precision(PER_BLOCK if form == PER_BLOCK else 0)
        plans0 = cached_plans()
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        energy2, _ = driver.sweep()
        torch.cuda.synchronize(device)
        out[name]['s_per_sweep_continued'] = time.perf_counter() - t0
        out[name]['continued_energy'] = energy2
        out[name]['continued_plans_compiled'] = cached_plans() - plans0
        if golden is not None and warm + 1 < len(golden):
            out[name]['continued_delta_e_vs_reference'] = abs(energy2 - golden[warm + 1])
        la.PER_BLOCK_SVD_DRIVER = 'gesvd'
        tg.set_precision(0)
    driver.refine_energy = False
    driver.all_products = False
    tg.set_precision(0)
    clear_plans()
    ref = out['fp64_grouped']['energy']
    for name in out:
        out[name]['delta_e_vs_fp64_grouped'] = abs(out[name]['energy'] - ref)
        out[name]['delta_e_vs_own_fp64_check'] = abs(out[name]['energy'] - out[name]['energy_fp64_check'])
    return {'length': length, 'chi': chi, 'n_iter': n_iter, 'warm_fp64_sweeps': warm, 'warm_s': warm_s,
            'forms': out,
            'svd_per_block_redos': la.svd_fallbacks,
            'reference_energy': golden[warm] if golden is not None else None,
            'reference': 'the reference run in float64 from the same seed (tests/golden/dmrg_chi256.json), sweep '
                         f'{warm + 1} and the next',
            **({'speedup_split_vs_per_block': out['fp64_per_block']['s_per_sweep'] / out['split']['s_per_sweep'],
                'speedup_split_vs_per_block_continued': out['fp64_per_block']['s_per_sweep_continued'] /
                                                        out['split']['s_per_sweep_continued'],
                'speedup_bf16x3_fp64_ritz_vs_per_block': out['fp64_per_block']['s_per_sweep'] /
                                                         out['bf16x3_fp64_ritz']['s_per_sweep']}
               if 'fp64_per_block' in out else {}),
            **({'speedup_split_vs_per_block_default_svd': out['fp64_per_block_default_svd']['s_per_sweep'] /
                                                          out['split']['s_per_sweep']}
               if 'fp64_per_block_default_svd' in out else {}),
            'speedup_split_vs_fp64_grouped': out['fp64_grouped']['s_per_sweep'] / out['split']['s_per_sweep'],
            'start': f'{warm} FP64 sweeps from the seeded random MPS (N(0,1) float64 blocks in key order, seed {SEED})'}


def run_gpu(args, rank, world):
    import torch
    import torch.distributed as dist

    import tentorch_gb300 as tg
    from oracle import engine as orc
    from tentorch_gb300 import _lib
    from tentorch_gb300.linalg import PER_BLOCK
    from torch.autograd.graph import increment_version

    local = int(os.environ.get('LOCAL_RANK', 0))
    torch.cuda.set_device(local)
    device = torch.device('cuda', local)

    head, tail, theta = matvec_operands(tg, torch, device, args.chi, SEED + rank)
    gen = torch.Generator(device = device).manual_seed(SEED + 17 + rank)
    vectors = [theta]
    for _ in range(3):
        v = theta.clone()
        v.data.copy_(torch.randn(v.data.shape, dtype = torch.float64, device = device, generator = gen))
        vectors.append(v)
    plan = tg.linalg.plan_of(MATVEC, head, tail, vectors[0])
    flush = torch.empty(64 * 1024 * 1024, dtype = torch.float32, device = device)  # 256 MB > L2
    stream = torch.cuda.current_stream(device)

    def timed_loop(steps, precision, fn):
        tg.set_precision(precision)
        starts = [torch.cuda.Event(enable_timing = True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing = True) for _ in range(steps)]
        for i in range(steps):
            flush.zero_()
            starts[i].record(stream)
            fn(i)
            ends[i].record(stream)
        torch.cuda.synchronize(device)
        return [s.elapsed_time(e) for s, e in zip(starts, ends)]

    def matvec(i):
        # a Lanczos vector is new at every step: mark it written (host-side version counter, no
        # device work) so that the engine runs its phase rather than reusing a prepared copy
        increment_version(vectors[i % 4].data)
        return tg.einsum(MATVEC, head, tail, vectors[i % 4])

    # correctness of this very workload before timing it, in every form, against the oracle
    want = orc.einsum(orc.MATVEC, to_oracle(orc, head), to_oracle(orc, tail), to_oracle(orc, theta))
    scale = max(np.abs(b).max() for b in want.blocks.values())
    parity = {}
    for name, form in (('split', args.precision), ('fp64_grouped', 0), ('fp64_per_block', PER_BLOCK)):
        with tg.precision(form):
            got = tg.einsum(MATVEC, head, tail, theta)
        parity[name] = max(float(np.abs(got.block(*k).cpu().numpy() - b).max()) for k, b in want.blocks.items()) / scale

    # the autotuner picks each grouped form's launch forms for this histogram (cached; the timed
    # steps run the choice)
    tuned = {}
    for name, form in (('split', args.precision), ('fp64_grouped', 0)):
        with tg.precision(form):
            forms, tune_ms = tg.linalg.autotune(MATVEC, head, tail, vectors[0])
        tuned[name] = {'forms': forms, 'ms': tune_ms}
    tuned['histogram_key'] = f'{tg.linalg.histogram_key(plan):016x}'

    for form in (args.precision, 0, PER_BLOCK):
        tg.set_precision(form)
        for i in range(args.warmup):
            matvec(i)
    torch.cuda.synchronize(device)

    # --- the timed region ------------------------------------------------------------------
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize(device)
    clocks = Clocks(local)
    wall0 = time.perf_counter()
    times = timed_loop(args.steps, args.precision, matvec)
    wall = time.perf_counter() - wall0
    clock_record = clocks.stop()
    torch.cuda.synchronize(device)
    if world > 1:
        dist.barrier()
    total_ms, value = job_rate(sum(times), args.steps, world, device)
    ms_per_step = total_ms / args.steps

    # the other forms on the same GPU and the same inputs
    form_ms = {'split': ms_per_step}
    form_ms['fp64_grouped'] = ms_per_step if args.precision == 0 else sum(timed_loop(args.steps, 0, matvec)) / args.steps
    form_ms['fp64_per_block'] = sum(timed_loop(args.steps, PER_BLOCK, matvec)) / args.steps

    # --- per-kernel durations inside the step (CUDA events on the launching stream) ----------
    def op_profile(precision):
        n_ops = plan.n_ops
        op_ms = np.zeros(n_ops)
        kinds = None
        samples = min(args.steps, 200)
        ws = torch.zeros(max(plan.workspace, 1), dtype = torch.float64, device = device)  # a fresh workspace is zero
        prepared = [tg.linalg._prepared_arena(plan, i, t, ws, stream.cuda_stream) for i, t in enumerate([head, tail, vectors[0]])]
        for i in range(samples):
            flush.zero_()
            out = torch.empty(plan.out_space.size, dtype = torch.float64, device = device)
            ms_arr, kind_arr = (_lib.ctypes.c_float * n_ops)(), (_lib.i32 * n_ops)()
            _lib.check(_lib.lib.tt_plan_execute_timed(
                plan.handle, 0, precision,
                _lib.pointers([head.data.data_ptr(), tail.data.data_ptr(), vectors[i % 4].data.data_ptr()]),
                _lib.pointers([p.data_ptr() if p is not None else None for p in prepared]), out.data_ptr(),
                ws.data_ptr(), stream.cuda_stream, n_ops, ms_arr, kind_arr))
            op_ms += np.maximum(np.array(ms_arr[:n_ops]), 0.0)
            kinds = list(kind_arr[:n_ops])
        op_ms /= samples
        by_kind, launches = {}, 0
        for ms, k in zip(op_ms, kinds):
            if ms <= 0:
                continue
            name = KIND_NAMES[k] or gemm_kernel_name(precision)
            by_kind[name] = by_kind.get(name, 0.0) + ms
            launches += launches_of(k, precision)
        return by_kind, launches

    peaks, peak_kind = measured_peaks()
    by_kind, launches_per_step = op_profile(args.precision)
    gemm_ms = by_kind.get(gemm_kernel_name(args.precision), 0.0)
    fp64_kinds, _ = op_profile(0)
    # the FP64 products of the matvec: one launch with the leg move between them (chain_fp64_kernel),
    # or the two grouped launches when the chain does not run as one
    fp64_kernel = 'chain_fp64_kernel' if 'chain_fp64_kernel' in fp64_kinds else 'gemm_dmma_kernel'
    dmma_ms = fp64_kinds.get(fp64_kernel, 0.0)
    fp64_peak = fp64_peak_tflops(torch, device)
    fp64_achieved = plan.flops / (dmma_ms / 1e3) / 1e12 if dmma_ms > 0 else 0.0
    roofline_fp64 = {'bound': 'fp64', 'achieved': fp64_achieved, 'peak': fp64_peak, 'unit': 'TFLOP/s',
                     'frac': fp64_achieved / fp64_peak, 'traffic': ncu_traffic(fp64_kernel),
                     'kernel': fp64_kernel, 'kernel_ms': dmma_ms,
                     'peak_source': 'cuBLAS DGEMM 4096^3 best of 3 measured in this run (MEASURED_PEAKS.json has no FP64)',
                     'algorithmic': f'{plan.flops:.4g} FLOP per launch (sum of 2mkn over the block pairs of both stages)',
                     'op_ms': {k: round(v, 6) for k, v in fp64_kinds.items()}}
    if args.precision == 0:
        roofline = dict(roofline_fp64)
    else:
        slices = args.precision
        bf16_flops = plan.flops * slices * (slices + 1) / 2
        achieved = bf16_flops / (gemm_ms / 1e3) / 1e12 if gemm_ms > 0 else 0.0
        peak = peaks['bf16_tflops']
        roofline = {'bound': 'tensor', 'achieved': achieved, 'peak': peak, 'unit': 'TFLOP/s', 'frac': achieved / peak,
                    'traffic': ncu_traffic('gemm_split_kernel'), 'kernel': 'gemm_split_kernel',
                    'peak_source': f'{peak_kind} bf16_tflops', 'kernel_ms': gemm_ms,
                    'algorithmic': f'{bf16_flops:.4g} bf16 FLOP per step ({slices}({slices}+1)/2 slice products)'}
    roofline['op_ms'] = {k: round(v, 6) for k, v in by_kind.items()}
    roofline['dominant'] = max(by_kind, key = by_kind.get)

    # --- end to end through the public API with host buffers ---------------------------------
    host_in = [torch.empty(v.data.shape, dtype = torch.float64, pin_memory = True) for v in vectors]
    for h, v in zip(host_in, vectors):
        h.copy_(v.data.cpu())
    host_out = torch.empty(plan.out_space.size, dtype = torch.float64, pin_memory = True)
    staging = theta.clone()

    def e2e_step(i):
        staging.data.copy_(host_in[i % 4], non_blocking = True)
        out = tg.einsum(MATVEC, head, tail, staging)
        host_out.copy_(out.data, non_blocking = True)

    def e2e_link_step(i):
        # the same transfers by kernels over the CPU-GPU link (tt_link_copy), no copy-engine call
        tg.linalg.link_copy(staging.data, host_in[i % 4])
        out = tg.einsum(MATVEC, head, tail, staging)
        tg.linalg.link_copy(host_out, out.data)

    tg.set_precision(args.precision)
    for i in range(3):
        e2e_step(i)
    e2e_times = timed_loop(args.steps, args.precision, e2e_step)
    copy_engine_ms = sum(e2e_times) / args.steps
    e2e_path = 'pinned host theta -> H2D (copy engine) -> tentorch_gb300.einsum (C ABI) -> D2H (copy engine) of the image'
    e2e_ms = copy_engine_ms
    link_ms = None
    try:
        for i in range(3):
            e2e_link_step(i)
        torch.cuda.synchronize(device)
        # the link path checked once against the copy-engine path on the same vector
        e2e_step(0)
        torch.cuda.synchronize(device)
        engine_image = host_out.clone()
        e2e_link_step(0)
        torch.cuda.synchronize(device)
        if not torch.equal(engine_image, host_out):
            raise RuntimeError('the link transfer gave another image')
        link_times = timed_loop(args.steps, args.precision, e2e_link_step)
        link_ms = sum(link_times) / args.steps
        e2e_ms = link_ms
        e2e_path = ('pinned host theta -> kernel read over NVLink-C2C (tt_link_copy) -> tentorch_gb300.einsum (C ABI) '
                    '-> kernel write of the image to pinned host memory (tt_link_copy)')
    except (ValueError, RuntimeError) as error:
        print(f'link transfers unavailable: {error}', file = sys.stderr)
    h2d = host_in[0].numel() * 8
    d2h = host_out.numel() * 8

    dmrg = None
    if args.dmrg_length > 0 and rank == 0:
        dmrg = dmrg_sweeps(tg, torch, device, args.precision, args.dmrg_length, args.chi, args.dmrg_iter,
                           args.dmrg_warm)

    if rank == 0:
        cpu_value, cpu_elapsed, cpu_n = cpu_matvecs(args.chi, args.cpu_sample)
        one = cpu_matvecs_one_thread(args.chi, max(1, args.cpu_sample // 2))
        line = {'metric': METRIC, 'value': value, 'unit': 'matvecs/s', 'n_gpus': world, 'steps': args.steps,
                'warmup': args.warmup, 'ms_per_step': ms_per_step, 'higher_is_better': True, 'scaling': 'weak',
                'vs_baseline': None, 'dtype': 'f64' if args.precision == 0 else f'bf16x{args.precision}-split/f64',
                'data': 'synthetic', 'config': config(args, args.precision),
                'gflops': plan.flops / (ms_per_step / 1e3) / 1e9,
                'matvecs_per_s': {name: 1e3 / ms for name, ms in form_ms.items()},
                'speedup_vs_fp64_per_block': form_ms['fp64_per_block'] / ms_per_step,
                'speedup_vs_fp64_grouped': form_ms['fp64_grouped'] / ms_per_step,
                'wall_s_timed_region': wall,
                'parity_vs_oracle': parity,
                'roofline': roofline,
                'roofline_fp64_grouped': roofline_fp64,
                'autotune': dict(tuned, meaning = 'forms bits: 1 product chain as separate launches, '
                                                  '2 split products off the tensor cores; ms: median of the choice'),
                'dmrg': dmrg,
                'cpu_baseline': {'value': cpu_value, 'unit': 'matvecs/s', 'cores': os.cpu_count(), 'kind': 'port',
                                 'sample': f'{cpu_n} matvecs at chi={args.chi} of the oracle port of tentorch einsum '
                                           f'(numpy; {cpu_elapsed:.1f} s)'},
                'cpu_baseline_one_thread': ({'value': one[0], 'unit': 'matvecs/s', 'cores': 1, 'kind': 'port',
                                             'sample': f'{one[2]} matvecs, one BLAS thread ({one[1]:.1f} s)'}
                                            if one else None),
                'e2e_vs_cpu': 'the e2e rate against cpu_baseline compares with the numpy port of the reference '
                              "(oracle/engine.py), not with the reference's compiled engine",
                'e2e': {'value': world * 1e3 / e2e_ms, 'unit': 'matvecs/s', 'h2d_bytes_per_step': h2d,
                        'd2h_bytes_per_step': d2h, 'path': e2e_path,
                        'copy_engine_value': world * 1e3 / copy_engine_ms,
                        'link_value': world * 1e3 / link_ms if link_ms else None},
                'clocks': clock_record,
                'gpu_launches': launches_per_step * args.steps}
        print(json.dumps(line), flush = True)


def run_splittings(args):
    """Time the truncating split of a chi-sized two-site tensor (the SVD of every window of a DMRG
    sweep): [bond, phys] -> [phys, bond] with the bond of the matvec workload, seeded N(0, 1) blocks,
    `tg.svd(t, chi, 1e-14, 2)` per step (all blocks in one launch, the kept factors in a second).
    Prints one line of its own (not the headline); also a driver for profiling the SVD kernels."""
    import torch
    import tentorch_gb300 as tg
    device = torch.device('cuda', int(os.environ.get('LOCAL_RANK', 0)))
    torch.cuda.set_device(device)
    cat = tg.u1
    bond = tg.Leg(cat, *bond_multiplicities(args.chi))
    phys = tg.Leg(cat, [(1,), (-1,)], [1, 1])
    t = tg.Tensor(cat, [bond, phys], [phys, bond], (0,), dtype = torch.float64, device = device)
    gen = torch.Generator().manual_seed(SEED)
    for block in t.to_tuple()[3].values():
        block.copy_(torch.randn(block.shape, dtype = torch.float64, generator = gen))
    for _ in range(args.warmup):
        tg.svd(t, args.chi, 1e-14, 2)
    torch.cuda.synchronize(device)
    start = time.perf_counter()
    for _ in range(args.steps):
        tg.svd(t, args.chi, 1e-14, 2)
    torch.cuda.synchronize(device)
    elapsed = time.perf_counter() - start
    shapes = sorted((r, c) for r, c in t._space.shapes)
    print(json.dumps({'workload': f'u1_two_site_svd_chi{args.chi}', 'ms_per_split': 1e3 * elapsed / args.steps,
                      'blocks': len(shapes), 'largest': shapes[-1], 'steps': args.steps}), flush = True)


def run_recoupling(args):
    """The SU(2) and Fibonacci recoupling einsum 'ABcd,DCef->ABef' (B's codomain order forces an
    exchange F.R.F-dagger before the block products): SU(2) legs of spins j = 0..4 with 8 multiplets
    each, float64; Fibonacci legs (vacuum 16, tau 16), complex128; seeded N(0, 1) blocks.  Times each
    form the engine has for it (grouped FP64, split (float64 only), per-block cuBLAS) and the
    largest relative difference between the forms.  Prints one line of its own."""
    import numpy as np
    import torch
    import tentorch_gb300 as tg
    from tentorch_gb300.linalg import PER_BLOCK
    from oracle import engine as orc
    device = torch.device('cuda', int(os.environ.get('LOCAL_RANK', 0)))
    torch.cuda.set_device(device)
    out = {'workload': 'recoupling_einsum_ABcd_DCef', 'equation': 'ABcd,DCef->ABef'}

    def orc_einsum_of(tensors):
        ocat = {id(tg.su2): orc.su2, id(tg.fibonacci): orc.fibonacci}[id(tensors[0].cat)]
        cast = np.complex128 if tensors[0].dtype == torch.complex128 else np.float64
        legs = lambda ls: [orc.Leg(ocat, l.sectors, l.multiplicities) for l in ls]
        ops = []
        for t in tensors:
            o = orc.Tensor(ocat, legs(t.codomain), legs(t.domain), tuple(t.qtotal), cast)
            for key in o.blocks:
                o.blocks[key][...] = t.block(*key).cpu().numpy()
            ops.append(o)
        return orc.einsum('ABcd,DCef->ABef', *ops).blocks
    for name, cat, leg, dtype in (('su2', tg.su2, tg.Leg(tg.su2, [(j,) for j in range(9)], [8] * 9), torch.float64),
                                  ('fibonacci', tg.fibonacci, tg.Leg(tg.fibonacci, [(0,), (1,)], [16, 16]),
                                   torch.complex128)):
        gen = torch.Generator().manual_seed(SEED)
        tensors = []
        for _ in range(2):
            t = tg.Tensor(cat, [leg, leg], [leg, leg], (0,), dtype = dtype, device = device)
            for block in t.to_tuple()[3].values():
                block.copy_(torch.randn(block.shape, dtype = torch.float64, generator = gen).to(dtype))
            tensors.append(t)
        plan = tg.linalg.plan_of('ABcd,DCef->ABef', *tensors)
        forms = {'fp64_grouped': 0, 'fp64_per_block': PER_BLOCK}
        if dtype == torch.float64:
            forms['split'] = args.precision
        results, images = {}, {}
        tuned = {}
        for form_name, form in forms.items():
            with tg.precision(form):
                if form >= 0:
                    # the autotuner times the forms that apply (tcgen05 or mma.sync split products)
                    # and the timed calls run its choice
                    chosen, tune_ms = tg.linalg.autotune('ABcd,DCef->ABef', *tensors)
                    tuned[form_name] = {'forms': chosen, 'ms': tune_ms}
                for _ in range(max(1, args.warmup)):
                    images[form_name] = tg.einsum('ABcd,DCef->ABef', *tensors)
                torch.cuda.synchronize(device)
                start = time.perf_counter()
                steps = max(1, min(args.steps, 5))
                for _ in range(steps):
                    tg.einsum('ABcd,DCef->ABef', *tensors)
                torch.cuda.synchronize(device)
            ms = 1e3 * (time.perf_counter() - start) / steps
            flops = plan.flops * (4 if dtype == torch.complex128 else 1)
            results[form_name] = {'ms': ms, 'tflops': flops / (ms / 1e3) / 1e12}
        # every form against the oracle (the CPU restatement of the reference's einsum) on the same
        # inputs, relative to the largest entry
        want = orc_einsum_of(tensors)
        scale = max(float(np.abs(b).max()) for b in want.values())
        for form_name in results:
            got = images[form_name]
            worst = max(float(np.abs(got.block(*k).cpu().numpy() - b).max()) for k, b in want.items())
            results[form_name]['max_rel_err_vs_oracle'] = worst / scale
        out[name] = {'dtype': str(dtype).replace('torch.', ''), 'blocks': tensors[0].nblocks(),
                     'entries_per_tensor': tensors[0].data.numel(), 'gemm_flop': plan.flops, 'forms': results,
                     'autotune': tuned}
    print(json.dumps(out), flush = True)


def run_windows(args):
    """Batched windows: 64 independent U(1) two-site matvecs whose bond is drawn from a seed over
    {32, 64, 128, 256, 512} (the sector layout, MPO and dtype of the matvec workload), one matvec per
    window per step.  Timed issued one after another (the environments of each window prepared
    once, as a Lanczos loop reuses them) and as one captured CUDA graph of all 64 (plans compiled and
    tables uploaded before the capture; the graph reads every operand from its own buffer), in the
    split form and the grouped FP64 form.  Prints one line of its own."""
    import numpy as np
    import torch
    import tentorch_gb300 as tg
    from torch.autograd.graph import increment_version
    device = torch.device('cuda', int(os.environ.get('LOCAL_RANK', 0)))
    torch.cuda.set_device(device)
    rng = np.random.default_rng(SEED)
    chis = [int(c) for c in rng.choice([32, 64, 128, 256, 512], size = 64)]
    windows = [matvec_operands(tg, torch, device, chi, SEED + i) for i, chi in enumerate(chis)]
    flops = sum(tg.linalg.plan_of(MATVEC, *win).flops for win in windows)
    out = {'workload': 'batched_windows_u1_matvec', 'windows': len(windows), 'chis': chis, 'gemm_flop_per_step': flops}
    # a few windows (bonds 512, 64, 32, 128) checked against the oracle in every form
    from oracle import engine as orc
    checked = (0, 3, 5, 12)
    wanted = {i: orc.einsum(MATVEC, *(to_oracle(orc, t) for t in windows[i])).blocks for i in checked}
    stream = torch.cuda.current_stream(device)
    for name, form in (('split', args.precision), ('fp64_grouped', 0)):
        with tg.precision(form):
            def step():
                # every window's vector is new at every step (see matvec in run_gpu)
                for win in windows:
                    increment_version(win[2].data)
                return [tg.einsum(MATVEC, *win) for win in windows]
            for _ in range(3):
                step()
            torch.cuda.synchronize(device)
            steps = max(1, min(args.steps, 50))
            start = time.perf_counter()
            for _ in range(steps):
                step()
            torch.cuda.synchronize(device)
            eager_ms = 1e3 * (time.perf_counter() - start) / steps
            # the same windows dealt round robin to four streams, so small windows' kernels overlap
            # (each stream keeps its own workspace; every stream waits for the default one first)
            streams = [torch.cuda.Stream(device) for _ in range(4)]

            def spread():
                for win in windows:
                    increment_version(win[2].data)
                main = torch.cuda.current_stream(device)
                for s in streams:
                    s.wait_stream(main)
                images = []
                for i, win in enumerate(windows):
                    with torch.cuda.stream(streams[i % len(streams)]):
                        images.append(tg.einsum(MATVEC, *win))
                for s in streams:
                    main.wait_stream(s)
                return images
            for _ in range(3):
                spread()
            torch.cuda.synchronize(device)
            start = time.perf_counter()
            for _ in range(steps):
                spread()
            torch.cuda.synchronize(device)
            streams_ms = 1e3 * (time.perf_counter() - start) / steps
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph):
                step()
            graph.replay()
            torch.cuda.synchronize(device)
            start = time.perf_counter()
            for _ in range(steps):
                graph.replay()
            torch.cuda.synchronize(device)
            graph_ms = 1e3 * (time.perf_counter() - start) / steps
            # all windows through one call: in FP64 one persistent launch for every window's products
            def batched():
                for win in windows:
                    increment_version(win[2].data)
                return tg.linalg.einsum_batch(MATVEC, windows)
            for _ in range(3):
                batched()
            torch.cuda.synchronize(device)
            start = time.perf_counter()
            for _ in range(steps):
                batched()
            torch.cuda.synchronize(device)
            batch_ms = 1e3 * (time.perf_counter() - start) / steps
            batch_launches = tg.linalg.last_batch_launches
            # the one call captured in a CUDA graph (config 4 as named: one persistent launch in a
            # captured graph; the graph reads every operand from its buffer, so the environments'
            # phases run in every replay)
            batch_graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(batch_graph):
                batched_images = tg.linalg.einsum_batch(MATVEC, windows)
            batch_graph.replay()
            torch.cuda.synchronize(device)
            start = time.perf_counter()
            for _ in range(steps):
                batch_graph.replay()
            torch.cuda.synchronize(device)
            batch_graph_ms = 1e3 * (time.perf_counter() - start) / steps
            worst = 0.0
            images = batched()
            for i in checked:
                scale = max(float(np.abs(b).max()) for b in wanted[i].values())
                for got in (tg.einsum(MATVEC, *windows[i]), images[i], batched_images[i]):
                    worst = max(worst, max(float(np.abs(got.block(*k).cpu().numpy() - b).max()) for k, b in wanted[i].items()) / scale)
        out[name] = {'eager_ms_per_step': eager_ms, 'four_streams_ms_per_step': streams_ms, 'graph_ms_per_step': graph_ms,
                     'one_call_ms_per_step': batch_ms, 'one_call_launches': batch_launches,
                     'one_call_graph_ms_per_step': batch_graph_ms,
                     'matvecs_per_s_graph': len(windows) / (graph_ms / 1e3),
                     'matvecs_per_s_one_call': len(windows) / (batch_ms / 1e3),
                     'gflops_graph': flops / (graph_ms / 1e3) / 1e9,
                     'max_rel_err_vs_oracle': {'windows': list(checked), 'value': worst}}
    print(json.dumps(out), flush = True)


def run_dmrg(args):
    """Config 5's other sizes: the U(1) Heisenberg DMRG at `--dmrg-length` sites and bond `--chi`
    (n_iter `--dmrg-iter`), `--dmrg-warm` FP64 sweeps from the seeded MPS, then each form's sweeps
    from that state (dmrg_sweeps; the per-block form only up to bond 512).  Every form's energy is
    reported against the grouped FP64 run from the same state.  Prints one line of its own."""
    import torch
    import tentorch_gb300 as tg
    from tentorch_gb300.linalg import PER_BLOCK
    device = torch.device('cuda', int(os.environ.get('LOCAL_RANK', 0)))
    torch.cuda.set_device(device)
    forms = [('fp64_grouped', 0, 'gesvd', False), ('split', args.precision, 'gesvd', False),
             ('bf16x3_fp64_ritz', 3, 'gesvd', True)]
    if args.chi <= 512:
        forms.append(('fp64_per_block', PER_BLOCK, 'gesvd', False))
    result = dmrg_sweeps(tg, torch, device, args.precision, args.dmrg_length, args.chi, args.dmrg_iter,
                         args.dmrg_warm, forms = tuple(forms))
    print(json.dumps({'workload': 'dmrg_u1_heisenberg', **result}), flush = True)


def main():
    args = parse()
    if args.workload == 'dmrg':
        run_dmrg(args)
        return
    if args.workload == 'svd':
        run_splittings(args)
        return
    if args.workload == 'recoupling':
        run_recoupling(args)
        return
    if args.workload == 'windows':
        run_windows(args)
        return
    rank, world = int(os.environ.get('RANK', 0)), int(os.environ.get('WORLD_SIZE', 1))
    if world > 1:
        import torch.distributed as dist
        if args.impl == 'reference':
            if rank != 0:
                return
        else:
            dist.init_process_group('nccl' if args.impl == 'gb300' else 'gloo')
    if args.impl == 'reference':
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == '__main__':
    main()
