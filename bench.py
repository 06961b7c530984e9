#!/usr/bin/env python
"""Benchmark of COMMIT's operator pair A*x + A'*y on one GB300 (or N replicas).

Workload (default ``hcp_1m``): seeded synthetic full-brain dictionary -- 145x174x145 grid,
600k-voxel mask, 1M streamlines (~1.2e8 segments), stick-zeppelin-ball model with 1 IC,
1 EC and 2 ISO responses, 18 b0 + 3 shells x 90 directions (nS = 288), 500 LUT
directions, FP32 LUT and lengths, FP64 vectors.  A step is one operator pair
y = A x, g = A' y over the whole workload; ``value`` is pairs/s with the inputs resident
in HBM (y is 1.38 GB, far larger than the 129 MB L2, so no L2 flush is needed).
``e2e`` is the same metric through LinearOperator.dot on pinned host buffers, host
copies included.  ``--impl reference`` times the reference's own compiled CPU operator
(oracle/_ref, or the C restatement when the reference was not compiled) on a bounded
voxel-slab sample of the same workload, scaled to the full workload by segment count.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'A·x+Aᵀx operator pairs/s (1M-streamline workload)'

# DRAM bytes (read + write) per product, recorded from one ncu capture of this workload
# (`ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum
# --clock-control none -k regex:"k_(forward_p|adjoint_p|fibre_sum)" --csv python bench.py
# --steps 1 --warmup 1 --no-e2e --no-cpu`, one pass, full workload).  A constant: the bench
# line labels it as such.  Keyed by (workload, streamlines, arith); the A' entry is the slab
# voxel passes plus the slab fibre passes of one product.
MEASURED_TRAFFIC = {('hcp_1m', 1000000, 'ff'): {'forward': 2679165952, 'adjoint': 11855011840}}


# relative-error bounds of the reduced-precision LUT formats (the FP64 path's bar is 1e-10)
REDUCED_BOUNDS = {'bf16': 1.5e-2, 'fp16': 4e-3, 'f32': 2e-5}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=10)
    p.add_argument('--warmup', type=int, default=3)
    p.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    p.add_argument('--workload', default='hcp_1m')
    p.add_argument('--fibers', type=int, default=0, help='override the number of streamlines (smaller runs)')
    p.add_argument('--arith', default='ff', choices=['ff', 'f64', 'bf16', 'fp16', 'f32'])
    p.add_argument('--slabs', type=int, default=-1,
                   help='adjoint slab count (0 automatic, 1 off; default: the handle\'s own choice)')
    p.add_argument('--fista', action='store_true', help='FISTA time-to-tolerance, plain vs mixed + refinement')
    p.add_argument('--fista-iters', type=int, default=8000, help='iterations of each plain arm')
    p.add_argument('--mixed-iters', type=int, default=4000, help='reduced-precision iterations of a mixed arm')
    p.add_argument('--refine-iters', type=int, default=6000, help='FP64 refinement iterations of a mixed arm')
    p.add_argument('--xstar-iters', type=int, default=20000, help='cap on the iterations computing x*')
    p.add_argument('--xstar-chunk', type=int, default=1000, help='iterations run from x* to measure its drift')
    p.add_argument('--demo', action='store_true',
                   help='demo-scale case (5k streamlines, nS=66): A*x, A\'y and 200 FISTA nnls iterations, '
                        'host-driven loop vs graph-captured loop, next to the reference CPU operator')
    p.add_argument('--trk2dict', action='store_true',
                   help='streamline voxelisation (trk2dictionary) on the device vs the CPU restatement')
    p.add_argument('--t2d-fibers', type=int, default=200000)
    p.add_argument('--batch', action='store_true',
                   help='regularisation paths: 8 tractograms x 16 lambdas, batched BF16 vs sequential plain solves')
    p.add_argument('--batch-tracts', type=int, default=8, help='number of tractograms of the batched workload')
    p.add_argument('--batch-scale', type=float, default=1.0, help='scale of the tractogram sizes (smaller runs)')
    p.add_argument('--batch-iters', type=int, default=20, help='FISTA iterations per solve (tolerances off)')
    p.add_argument('--batch-tol', type=float, default=0.0,
                   help='solve to tolerance instead (tol_fun; tol_x = tol_fun / 100, at most --batch-max '
                        'iterations): batched BF16 solves polished by a per-problem FP64 solve, against '
                        'sequential plain solves to the same tolerance')
    p.add_argument('--batch-max', type=int, default=1000, help='iteration cap per solve with --batch-tol')
    p.add_argument('--batch-streams', type=int, default=4, help='tractograms solved concurrently (streams)')
    p.add_argument('--sample-frac', type=float, default=0.25, help='CPU sample: fraction of the segments')
    p.add_argument('--no-e2e', action='store_true')
    p.add_argument('--no-cpu', action='store_true')
    p.add_argument('--no-f64', action='store_true', help='skip the native-FP64 arithmetic pairs')
    p.add_argument('--tensor-cores', type=int, default=-1,
                   help='reduced-precision BF16 path: 0 tensor cores when the shape allows, 1 CUDA cores, '
                        '2 tensor cores required (default: the handle\'s own setting)')
    return p.parse_args()


# ------------------------------------------------------------------ environment helpers
def dist_env():
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return ws, rank, local


def max_over_ranks(value: float, device=None) -> float:
    """The largest of the ranks' values (the job's time is its slowest replica's); the
    value itself with one rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank: float, seconds_max: float, world: int) -> float:
    """Whole-job throughput of N independent replicas: all ranks' units over the slowest
    rank's time (weak scaling)."""
    return units_per_rank * world / seconds_max


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""
    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix='.csv')
            os.close(fd)
            self.f = open(self.path, 'w')
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.gpu), f'--query-gpu={self.FIELDS}',
                                          '--format=csv,noheader,nounits', '-lms', '200'], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = [r.split(',') for r in open(self.path).read().strip().splitlines() if r.strip()]
        os.unlink(self.path)
        sm, mx, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for r in rows:
            r = [c.strip() for c in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for nm, val in zip(names, r[5:9]):
                if val.lower().startswith('active'):
                    reasons.add(nm)
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': max(mx) if mx else None,
                'reasons': sorted(reasons), 'samples': len(sm)}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        d = json.load(open(p))
        return {'hbm_gbs': d.get('hbm_gbs', 6800.0), 'src': 'measured'}
    return {'hbm_gbs': 6800.0, 'src': 'fallback'}


def algorithmic(D, K, reduced=False) -> tuple:
    """Compulsory bytes and FMAs of one product (A or A'), LUT bytes excluded (on-chip).
    Reduced precision: FP16 lengths and FP32 rows (columns stay FP64)."""
    n, nE, nI = D['IC']['n'], D['EC']['n'], D['ISO']['n']
    nIC, nEC, nISO = K['wmr'].shape[0], K['wmh'].shape[0], K['iso'].shape[0]
    nS = K['wmr'].shape[2]
    nrows = D['IC']['nVOX'] * nS
    ncols = D['IC']['nSTR'] * nIC + nE * nEC + nI * nISO
    sl, sy = (2, 4) if reduced else (4, 8)
    b = n * (4 + 4 + 2 + sl) + (nE * (4 + 2) if nEC else 0) + (nI * 4 if nISO else 0) + ncols * 8 + nrows * sy
    f = n * nS * nIC + nE * nS * nEC + nI * nS * nISO
    return b, f, nrows, ncols


def sample_slab(D, K, frac: float):
    """Central slab of voxels holding about `frac` of the IC segments (synth.voxel_slab)."""
    from commit_gb300 import synth
    S = synth.voxel_slab(D, K, frac)
    return S['D'], S['share'], S['voxels']


def cpu_reference_fista(D, K, frac, iters):
    """Per-iteration time of the reference's FISTA (numpy restatement of solvers.py driving
    the reference's compiled operator, all host cores) on the central voxel slab of the
    workload, scaled to the whole workload by segment share; nnls on all compartments."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    import build_ref
    Ds, share, (lo, hi) = sample_slab(D, K, frac)
    threads = min(os.cpu_count() or 1, 255)
    kind = 'port'
    try:
        if build_ref.generate() and build_ref.compile_operator() and O.ref_available():
            kind = 'reference'
    except Exception:
        kind = 'port'
    A = O.RefOperator(Ds, K, O.set_threads(Ds, threads)) if kind == 'reference' else \
        O.PortOperator(Ds, K, None, nthreads=threads)
    y = A.dot(np.random.default_rng(3).uniform(0.0, 1.0, A.nCOLS))
    rp = O.reg_params(Ds, K)
    t0 = time.perf_counter()
    O.solve(y, A, A.T, tol_fun=0.0, tol_x=0.0, max_iter=iters, verbose=0, regularisation=O.init_regularisation(rp))
    dt = (time.perf_counter() - t0) / iters
    return {'value': 1000.0 * dt / share, 'unit': 'ms/iteration', 'cores': threads, 'kind': kind,
            'sample': f'central voxel slab [{lo},{hi}) = {share * 100:.2f}% of the IC segments, {iters} iterations '
                      f'in {dt * iters:.2f} s (initialisation included), time scaled by segment share'}


def cpu_reference(D, K, frac, steps, warmup, x_full=None):
    """Time the reference CPU operator (oracle/_ref if compiled for this host, else the
    C restatement) on a voxel-slab sample; returns a cpu_baseline dict (pairs/s scaled
    to the full workload by segment count).  With x_full (the benchmark's own column
    vector) the sample's x is its slab columns, and the last pair's outputs are returned
    under 'outputs' for checking the GPU's results on the slab."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import oracle as O
    import build_ref
    from commit_gb300 import synth
    cores = os.cpu_count() or 1
    S = synth.voxel_slab(D, K, frac)
    Ds, share, (lo, hi) = S['D'], S['share'], S['voxels']
    kind = 'port'
    try:
        if build_ref.generate() and build_ref.compile_operator() and O.ref_available():
            kind = 'reference'
    except Exception:
        kind = 'port'
    threads = min(cores, 255)
    if kind == 'reference':
        A = O.RefOperator(Ds, K, O.set_threads(Ds, threads))
    else:
        A = O.PortOperator(Ds, K, None, nthreads=threads)
    if x_full is None:
        x = np.random.default_rng(11).uniform(0.0, 1.0, size=A.nCOLS)
    else:
        x = np.ascontiguousarray(x_full[S['cols']])
    for _ in range(max(1, warmup)):
        y = A.dot(x)
        g = A.T.dot(y)
    t0 = time.perf_counter()
    for _ in range(steps):
        y = A.dot(x)
        g = A.T.dot(y)
    dt = time.perf_counter() - t0
    rate_sample = steps / dt
    out = {'value': rate_sample * share, 'unit': 'pairs/s', 'cores': threads, 'kind': kind,
           'sample': (f'central voxel slab [{lo},{hi}) = {share * 100:.2f}% of the IC segments '
                      f'({Ds["IC"]["n"]} segments, {Ds["EC"]["n"]} EC, {Ds["ISO"]["n"]} ISO); {steps} pairs in '
                      f'{dt:.2f} s on {threads} threads, rate scaled by segment share'),
           'sample_pairs_per_s': rate_sample}
    if x_full is not None:
        out['outputs'] = {'y': y, 'g': g, 'cols': S['cols'], 'voxels': (lo, hi)}
    return out


def check_against_reference(A, y_gpu, cb, nS, arith='ff') -> dict:
    """Relative 2-norm errors of the GPU's timed A x on the reference sample's rows, and of
    the GPU's A' (of the reference's y placed in those rows, zero elsewhere) on its columns."""
    import torch
    o = cb.pop('outputs')
    lo, hi = o['voxels']
    r0, r1 = lo * nS, hi * nS
    yg = y_gpu[r0:r1].double().cpu().numpy()
    fwd = float(np.linalg.norm(yg - o['y']) / np.linalg.norm(o['y']))
    ym = torch.zeros(A.nROWS, dtype=torch.float64, device=y_gpu.device)
    ym[r0:r1] = torch.from_numpy(o['y']).to(y_gpu.device)
    if arith in REDUCED_BOUNDS:
        g = A.T.dot(ym.float(), arith=arith).double().cpu().numpy()
    else:
        g = A.T.dot(ym).cpu().numpy()
    gm = np.zeros(A.nCOLS)
    gm[o['cols']] = o['g']
    adj = float(np.linalg.norm(g - gm) / np.linalg.norm(gm))
    return {'forward_rel': fwd, 'adjoint_rel': adj, 'bar': REDUCED_BOUNDS.get(arith, 1e-10),
            'what': 'timed A x on the reference sample rows; A\' of the reference y on the sample columns',
            'rows': [int(r0), int(r1)]}


def build_workload(args, device):
    from commit_gb300 import synth
    spec = synth.SPECS[args.workload]
    if args.fibers:
        spec = synth.scaled_spec(args.workload, n_fibers=args.fibers)
    t0 = time.perf_counter()
    D, K = synth.make_dictionary(spec, device=device)
    D['IC']['eval'] = np.ones(D['IC']['nSTR'] * K['wmr'].shape[0], np.uint32)
    return spec, D, K, time.perf_counter() - t0


def workload_config(spec, D, K, args):
    nS = K['wmr'].shape[2]
    return {'workload': f'{args.workload}: {spec.n_fibers} synthetic streamlines, grid {"x".join(map(str, spec.dim))}, '
                        f'{spec.n_mask} mask voxels, SZB 1 IC / {K["wmh"].shape[0]} EC / {K["iso"].shape[0]} ISO, '
                        f'nS={nS}, ndirs={spec.ndirs}',
            'n_segments': int(D['IC']['n']), 'n_voxels': int(D['IC']['nVOX']), 'n_ec': int(D['EC']['n']),
            'n_iso': int(D['ISO']['n']), 'nS': int(nS), 'vectors': 'f64', 'lut': 'f32',
            'arith': args.arith, 'l2': 'inputs larger than L2 (y is nV*nS f64), no flush'}


def launches_per_pair(A, reduced: bool, tc: bool = False) -> int:
    """Kernels of one A + A' pair.  FP64 path: the max-|x| pass of the range guard and the
    forward, then per adjoint slab a voxel pass and a fibre pass.  Reduced precision: the
    FP32 -> FP64 column conversion and the forward, the adjoint (slab passes, or the
    tensor-core voxel pass and its fibre pass) and the FP64 -> FP32 conversion; the
    tensor-core forward adds its x*eval pass."""
    ns = max(1, A.set_slabs(None))
    if tc:
        return 3 + 3
    if reduced:
        return 2 + 2 * ns + 1
    return 2 + 2 * ns


def traffic_for(args, spec, dom: str):
    t = MEASURED_TRAFFIC.get((args.workload, spec.n_fibers, args.arith))
    if not t:
        return None
    return t['adjoint'] if dom.startswith('adjoint') else t['forward']


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    import torch
    dev = 'cuda' if torch.cuda.is_available() else 'cpu'
    spec, D, K, _ = build_workload(args, dev)
    cb = cpu_reference(D, K, args.sample_frac, args.steps, args.warmup)
    out = {'metric': METRIC, 'value': cb['value'], 'unit': 'pairs/s', 'impl': 'reference', 'n_gpus': args.gpus,
           'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': 1000.0 / cb['value'],
           'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
           'config': workload_config(spec, D, K, args), 'cpu_baseline': cb,
           'e2e': {'value': cb['value'], 'unit': 'pairs/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(out))
    return 0


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group('nccl')
    dev = torch.device('cuda', torch.cuda.current_device())
    from commit_gb300 import synth
    from commit_gb300.operator import LinearOperator
    spec, D, K, tgen = build_workload(args, 'cuda')
    if args.fista:
        return run_fista(args, spec, D, K, dev)
    reduced = args.arith in ('bf16', 'fp16', 'f32')
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    A = LinearOperator(D, K, None, arith='ff' if reduced else args.arith, device=dev.index)
    torch.cuda.synchronize()
    tcreate = time.perf_counter() - t0  # host arrays -> device re-layout (sorts, CSR, slabs)
    if args.slabs >= 0:
        A.set_slabs(args.slabs)
    if args.tensor_cores >= 0:
        A.tensor_cores(args.tensor_cores)
    At = A.T
    nbytes, nfma, nrows, ncols = algorithmic(D, K, reduced)
    vdt = torch.float32 if reduced else torch.float64
    x = torch.from_numpy(synth.make_x(ncols, spec.seed + 1)).to(dev).to(vdt)
    y = torch.empty(nrows, dtype=vdt, device=dev)
    g = torch.empty(ncols, dtype=vdt, device=dev)
    st = torch.cuda.current_stream(dev)
    kw = {'arith': args.arith} if reduced else {}
    for _ in range(args.warmup):
        A.dot(x, out=y, **kw)
        At.dot(y, out=g, **kw)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
        torch.cuda.synchronize()
    clocks = ClockSampler(dev.index)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_start.record(st)
    for k in range(args.steps):
        ev[k][0].record(st)
        A.dot(x, out=y, **kw)
        ev[k][1].record(st)
        At.dot(y, out=g, **kw)
        ev[k][2].record(st)
    e_end.record(st)
    torch.cuda.synchronize()
    ms = e_start.elapsed_time(e_end)
    if ws > 1:
        ms = max_over_ranks(ms, dev)
        torch.distributed.barrier()
    clk = clocks.stop()
    fwd_ms = statistics.mean(a.elapsed_time(b) for a, b, _ in ev)
    adj_ms = statistics.mean(b.elapsed_time(c) for _, b, c in ev)
    value = replica_value(args.steps, ms / 1000.0, ws)
    peaks = measured_peaks()
    dom, dom_ms = ('adjoint (voxel pass + fibre sum)', adj_ms) if adj_ms >= fwd_ms else ('forward k_forward', fwd_ms)
    achieved = nbytes / (dom_ms / 1000.0) / 1e9
    out = {'metric': METRIC, 'value': value, 'unit': 'pairs/s', 'n_gpus': ws, 'steps': args.steps,
           'warmup': args.warmup, 'ms_per_step': ms / args.steps, 'higher_is_better': True, 'scaling': 'weak',
           'vs_baseline': None, 'dtype': 'f32 rows / ' + args.arith + ' LUT' if reduced else 'f64',
           'data': 'synthetic', 'config': workload_config(spec, D, K, args),
           'roofline': {'bound': 'hbm', 'kernel': dom, 'achieved': achieved, 'peak': peaks['hbm_gbs'],
                        'unit': 'GB/s', 'frac': achieved / peaks['hbm_gbs'], 'peak_src': peaks['src'],
                        'traffic': traffic_for(args, spec, dom),
                        'traffic_src': 'recorded constant: dram__bytes_read.sum + dram__bytes_write.sum of one ncu '
                                       'capture of this workload and arithmetic, per product',
                        'algorithmic_bytes_per_launch': nbytes,
                        'forward_ms': fwd_ms, 'adjoint_ms': adj_ms,
                        'fma_per_product': nfma, 'achieved_gfma_s': nfma / (dom_ms / 1000.0) / 1e9},
           'clocks': clk,
           'gpu_launches': args.steps * launches_per_pair(A, reduced, reduced and args.arith == 'bf16' and A.tensor_cores()),
           'setup_s': {'generate': tgen, 'create_operator': tcreate},
           'occupancy_tuning': A.occupancy(), 'adjoint_slabs': A.set_slabs(None),
           'tensor_cores': bool(reduced and args.arith == 'bf16' and A.tensor_cores())}
    # the reference's own FP64 arithmetic (native FP64 FMAs) on the same vectors, a few pairs
    if args.arith == 'ff' and not args.no_f64:
        nf = 3
        for _ in range(2):
            A.dot(x, out=y, arith='f64')
            At.dot(y, out=g, arith='f64')
        torch.cuda.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        f_ms, a_ms = 0.0, 0.0
        for _ in range(nf):
            e[0].record(st)
            A.dot(x, out=y, arith='f64')
            e[1].record(st)
            At.dot(y, out=g, arith='f64')
            e[2].record(st)
            torch.cuda.synchronize()
            f_ms += e[0].elapsed_time(e[1]) / nf
            a_ms += e[1].elapsed_time(e[2]) / nf
        out['f64_arith'] = {'pairs_per_s': 1000.0 / (f_ms + a_ms), 'forward_ms': f_ms, 'adjoint_ms': a_ms,
                            'pairs': nf, 'note': 'native FP64 FMAs (the reference arithmetic), same workload'}
        # leave y as the float-float A x of the timed steps for the parity check below
        A.dot(x, out=y)
    # end to end through the public API on pinned host buffers
    if not args.no_e2e and not reduced:
        xh = torch.empty(ncols, dtype=torch.float64, pin_memory=True).numpy()
        xh[:] = x.cpu().numpy()
        yh = torch.empty(nrows, dtype=torch.float64, pin_memory=True).numpy()
        gh = torch.empty(ncols, dtype=torch.float64, pin_memory=True).numpy()
        for _ in range(max(1, args.warmup)):
            A.dot(xh, out=yh)
            At.dot(yh, out=gh)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            A.dot(xh, out=yh)
            At.dot(yh, out=gh)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if ws > 1:
            dt = max_over_ranks(dt, dev)
        out['e2e'] = {'value': replica_value(args.steps, dt, ws), 'unit': 'pairs/s', 'h2d_bytes_per_step': (ncols + nrows) * 8,
                      'd2h_bytes_per_step': (nrows + ncols) * 8,
                      'host_path': ('page-locked host vectors through LinearOperator.dot (cgb_op_apply_host): '
                                    'x copied to and from the device, the row vector read / written in place '
                                    'by the kernels over NVLink-C2C' if A.host_mode(None) != 1 else
                                    'staged copies pipelined against the kernels')}
        # the shape of COMMIT's own call site (operator.pyx:114-184): pageable numpy vectors in,
        # a fresh numpy output per call
        xp = x.cpu().numpy().copy()
        for _ in range(max(1, args.warmup)):
            At.dot(A.dot(xp))
        t0 = time.perf_counter()
        for _ in range(args.steps):
            yp = A.dot(xp)
            At.dot(yp)
        dt = time.perf_counter() - t0
        if ws > 1:
            dt = max_over_ranks(dt, dev)
        out['e2e_pageable'] = {'value': replica_value(args.steps, dt, ws), 'unit': 'pairs/s',
                               'h2d_bytes_per_step': (ncols + nrows) * 8, 'd2h_bytes_per_step': (nrows + ncols) * 8,
                               'host_path': 'pageable numpy vectors through LinearOperator.dot, fresh output '
                                            'arrays per call (the reference call site)'}
    if rank == 0 and ws == 1 and not args.no_cpu:
        cb = cpu_reference(D, K, args.sample_frac, 5, 1, x_full=x.double().cpu().numpy())
        out['parity_vs_reference'] = check_against_reference(A, y, cb, K['wmr'].shape[2], args.arith)
        out['cpu_baseline'] = cb
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_fista(args, spec, D, K, dev):
    """FISTA time-to-tolerance at the 1M-streamline workload (nnls on all compartments).

    x*: the FP64-accurate (float-float) solver with function-value momentum restart, run to
    tol_fun 1e-12 or --xstar-iters iterations; --xstar-chunk more iterations from it measure
    how far x* itself still moves (the better of the two points is kept).  Arms, each traced
    per accepted iteration (seconds since its start, |x_k - x*| / |x*|, cost): the plain
    FP64-accurate solver as the reference runs it (no restart), the same with restart, and
    reduced precision + FP64 refinement with restart: BF16 LUT on the tensor cores and FP32
    LUT on the CUDA cores.  Times to 1e-2 / 1e-3 / 1e-4 in x and to a relative cost gap of
    1e-6 / 1e-8 / 1e-10, and the errors of the reduced-precision phase's y = A x*, x and
    cost against FP64.  Prints one JSON line."""
    import torch
    from commit_gb300 import solvers, synth
    from commit_gb300.operator import LinearOperator
    A = LinearOperator(D, K, None, arith='ff', device=dev.index)
    x_true = synth.make_x(A.nCOLS, spec.seed + 1)
    y = A.dot(torch.from_numpy(x_true).to(dev))
    y = torch.from_numpy(synth.make_signal(y.cpu().numpy(), spec.seed + 2)).to(dev)
    rp = {'startIC': 0, 'sizeIC': A.ICnSTR * A.ICnRF, 'startEC': A.ICnSTR * A.ICnRF, 'sizeEC': A.ECn * A.ECnRF,
          'startISO': A.ICnSTR * A.ICnRF + A.ECn * A.ECnRF, 'sizeISO': A.ISOn * A.ISOnRF,
          'regIC': None, 'regEC': None, 'regISO': None, 'nnIC': True, 'nnEC': True, 'nnISO': True,
          'dictIC_params': None, 'dictEC_params': None, 'dictISO_params': None}
    reg = lambda: solvers.init_regularisation(dict(rp))  # noqa: E731
    rel = lambda a, b: float(torch.linalg.norm(a - b) / torch.linalg.norm(b))  # noqa: E731
    # ---- x*: one restarted FP64-accurate solve to tol_fun 1e-12 (or --xstar-iters), then
    # --xstar-chunk more iterations from it to measure how far x* itself still moves
    x0 = torch.zeros(A.nCOLS, dtype=torch.float64, device=dev)
    t0 = time.perf_counter()
    x_star, d = solvers.solve(y, A, A.T, tol_fun=1e-12, tol_x=0.0, max_iter=args.xstar_iters, verbose=0, x0=x0,
                              regularisation=reg(), restart=True)
    torch.cuda.synchronize()
    xs_info = {'method': 'float-float FISTA with function-value restart, tol_fun 1e-12',
               'iterations': d['iterations'], 'seconds': time.perf_counter() - t0, 'criterion': d['stopping_criterion'],
               'cost': d['cost_function'], 'backtracks': d['backtracks'], 'anchors': d['anchors']}
    cost_star = d['cost_function']
    print(json.dumps({'x_star': xs_info}), file=sys.stderr, flush=True)
    xn, d = solvers.solve(y, A, A.T, tol_fun=0.0, tol_x=0.0, max_iter=args.xstar_chunk, verbose=0, x0=x_star,
                          regularisation=reg(), restart=True)
    xs_info['drift'] = {'iterations': d['iterations'], 'rel_change': rel(xn, x_star),
                        'cost_change': (d['cost_function'] - cost_star) / cost_star}
    if d['cost_function'] < cost_star:  # the later point is the better minimiser
        x_star, cost_star = xn, d['cost_function']
    del xn
    x_tols, c_tols = (1e-2, 1e-3, 1e-4), (1e-6, 1e-8, 1e-10)

    def first_below(t, v, tol):
        idx = np.flatnonzero(v <= tol)
        return {'seconds': float(t[idx[0]]), 'iteration': int(idx[0]) + 1} if idx.size else None

    def summary(det, extra=None):
        tr = det['trace']
        t, xd, cost = tr[:, 0], tr[:, 1], tr[:, 2]
        gap = (cost - cost_star) / cost_star
        out = {'iterations': int(len(t)), 'seconds': float(t[-1]), 'final_rel': float(xd[-1]),
               'final_cost_gap': float(gap[-1]), 'backtracks': det.get('backtracks'), 'anchors': det.get('anchors'),
               'stopping_criterion': det.get('stopping_criterion'),
               'time_to_x': {f'{tol:g}': first_below(t, xd, tol) for tol in x_tols},
               'time_to_cost_gap': {f'{tol:g}': first_below(t, gap, tol) for tol in c_tols}}
        out['ms_per_iteration'] = 1000.0 * out['seconds'] / len(t)
        if extra:
            out.update(extra)
        return out

    arms = {}
    n = args.fista_iters
    _, d = solvers.solve(y, A, A.T, tol_fun=0.0, tol_x=0.0, max_iter=n, verbose=0, regularisation=reg(), x_ref=x_star,
                         restart=True)
    arms['plain_restart'] = summary(d)
    _, d = solvers.solve(y, A, A.T, tol_fun=0.0, tol_x=0.0, max_iter=n, verbose=0, regularisation=reg(), x_ref=x_star)
    arms['plain'] = summary(d)
    n1, n2 = args.mixed_iters, args.refine_iters
    errors = {}
    yf = A.dot(x_star)
    for name, ar, tcm in (('bf16_tensor_cores', 'bf16', 2), ('f32_lut', 'f32', 1)):
        if tcm == 2 and not A.tensor_cores(0):
            continue
        A.tensor_cores(tcm)
        xm, dm = solvers.solve_mixed(y, A, tol_fun=0.0, tol_x=0.0, max_iter=n1, verbose=0, regularisation=reg(),
                                     arith=ar, refine_max_iter=n2, x_ref=x_star, restart=True)
        mix = dm['mixed']['trace']
        errors[name] = {'y': rel(A.dot(x_star.float(), arith=ar).double(), yf),
                        'x_after_reduced_phase': float(mix[-1, 1]),
                        'cost_after_reduced_phase': float((mix[-1, 2] - cost_star) / cost_star)}
        arms[name + '_refined'] = summary(dm, {
            'reduced_iterations': int(len(mix)), 'refine_iterations': int(dm['refine']['iterations']),
            'refine_stopping_criterion': dm['refine']['stopping_criterion'],
            'ms_per_reduced_iteration': 1000.0 * float(mix[-1, 0]) / len(mix)})
    A.tensor_cores(1)
    for v in arms.values():
        v['speedup_vs_plain'] = {}
        for key in ('time_to_x', 'time_to_cost_gap'):
            for tol, hit in v[key].items():
                ref = arms['plain'][key][tol]
                v['speedup_vs_plain'][key[8:] + ':' + tol] = (ref['seconds'] / hit['seconds']
                                                             if ref and hit else None)
    out = {'metric': 'FISTA time-to-tolerance |x_k - x*|/|x*| (1M-streamline workload, nnls)',
           'unit': 's', 'higher_is_better': False, 'data': 'synthetic',
           'config': workload_config(spec, D, K, args) | {'regulariser': 'nnls (all compartments)'},
           'x_star': xs_info,
           'arms': arms, 'reduced_precision_errors_vs_fp64': errors}
    if not args.no_cpu:
        out['cpu_baseline'] = cpu_reference_fista(D, K, args.sample_frac, 5)
    print(json.dumps(out))
    return 0


def run_batch(args):
    """Regularisation paths on several tractograms: for each of the 8 tractograms (50k-400k
    streamlines, full-brain grid, nS = 288) 16 nonnegative group-lasso problems (64 random
    bundles, lambda = 1e-4..1e-1 of lambda_max), each run for the same number of FISTA
    iterations (tolerances off, so both arms do identical iteration counts).  Arm 1: the
    batched solver (BF16 LUT, multi-right-hand-side passes, one call per tractogram).  Arm 2:
    the 128 problems solved one after another by the plain FP64-accurate solver.  Prints one
    JSON line with both times, solves/s and the distance between the two arms' solutions."""
    import torch
    from commit_gb300 import evaluation, solvers, synth
    from commit_gb300.operator import LinearOperator
    dev = torch.device('cuda', torch.cuda.current_device())
    M = args.batch_iters
    tracts = []
    tgen = 0.0
    for k in range(args.batch_tracts):
        spec = synth.batch_spec(k, int(synth.BATCH_FIBERS[k] * args.batch_scale))
        t0 = time.perf_counter()
        D, K = synth.make_dictionary(spec, device='cuda')
        tgen += time.perf_counter() - t0
        A = LinearOperator(D, K, None, arith='ff', device=dev.index)
        y = A.dot(torch.from_numpy(synth.make_x(A.nCOLS, spec.seed + 1)).to(dev))
        y = torch.from_numpy(synth.make_signal(y.cpu().numpy(), spec.seed + 2)).to(dev)
        groups = synth.bundle_groups(D['IC']['nSTR'], 64, seed=spec.seed)
        regs = [evaluation.set_regularisation(
            A, y, D, K, regularisers=('group_lasso', None, None), lambdas=(lam, None, None),
            is_nonnegative=(True, True, True),
            params=({'group_idx': groups, 'group_weights_cardinality': True, 'group_weights_adaptive': False},
                    None, None)) for lam in synth.BATCH_LAMBDAS]
        tracts.append({'spec': spec, 'A': A, 'y': y, 'regs': regs, 'n_segments': int(D['IC']['n'])})
        del D, K
    # warm-up: reduced LUT copies, width tuning, plain kernels
    for t in tracts:
        solvers.solve_batch(t['y'], t['A'], t['regs'][:4], tol_fun=0.0, tol_x=0.0, max_iter=2)
        solvers.solve(t['y'], t['A'], t['A'].T, tol_fun=0.0, tol_x=0.0, max_iter=2, verbose=0,
                      regularisation=t['regs'][0])
    torch.cuda.synchronize()
    if args.batch_tol > 0:
        return run_batch_to_tolerance(args, tracts, tgen)
    clocks = ClockSampler(dev.index)
    clocks.start()
    t0 = time.perf_counter()
    xb = solvers.solve_batches([(t['y'], t['A'], t['regs']) for t in tracts], n_streams=args.batch_streams,
                               tol_fun=0.0, tol_x=0.0, max_iter=M)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    t0 = time.perf_counter()
    xs = [[solvers.solve(t['y'], t['A'], t['A'].T, tol_fun=0.0, tol_x=0.0, max_iter=M, verbose=0,
                         regularisation=rp) for rp in t['regs']] for t in tracts]
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    clk = clocks.stop()
    dist = []
    for b, s_ in zip(xb, xs):
        for (x1, d1), (x2, d2) in zip(b, s_):
            dist.append(float(torch.linalg.norm(x1 - x2) / torch.linalg.norm(x2)))
    nsolves = sum(len(t['regs']) for t in tracts)
    out = {'metric': 'regularisation paths: FISTA solves/s, batched BF16-LUT vs sequential plain',
           'value': nsolves / t_batch, 'unit': 'solves/s', 'higher_is_better': True, 'n_gpus': 1,
           'data': 'synthetic', 'dtype': 'bf16 LUT / f32 rows / f64 columns (batched); f64 (plain)',
           'config': {'workload': f'{len(tracts)} tractograms x {len(synth.BATCH_LAMBDAS)} lambdas '
                                  f'(1e-4..1e-1 of lambda_max), nonnegative group lasso over 64 random bundles, '
                                  f'grid 145x174x145, 600k mask voxels, nS=288',
                      'fibers': [t['spec'].n_fibers for t in tracts],
                      'segments': [t['n_segments'] for t in tracts],
                      'iterations_per_solve': M, 'tolerances': 'off (fixed iteration count)'},
           'batched': {'seconds': t_batch, 'solves_per_s': nsolves / t_batch,
                       'ms_per_solve_iteration': 1000.0 * t_batch / (nsolves * M),
                       'widths': [t['A'].batch_width() for t in tracts],
                       'voxel_shapes': [t['A'].batch_shape() for t in tracts], 'streams': args.batch_streams},
           'sequential_plain': {'seconds': t_seq, 'solves_per_s': nsolves / t_seq,
                                'ms_per_solve_iteration': 1000.0 * t_seq / (nsolves * M)},
           'speedup': t_seq / t_batch,
           'x_rel_batched_vs_plain': {'max': max(dist), 'median': statistics.median(dist)},
           'clocks': clk, 'setup_s': {'generate': tgen}}
    print(json.dumps(out))
    return 0


def run_batch_to_tolerance(args, tracts, tgen):
    """The 128 regularisation-path solves to COMMIT's stopping rule (tol_fun, tol_x =
    tol_fun / 100, commit/solvers.py:335-357): batched BF16-LUT solves, each polished by an
    FP64-accurate solve warm-started from it (the refinement removes the BF16 operator's
    bias), against the plain FP64-accurate solver run from zero for every problem."""
    import torch
    from commit_gb300 import solvers
    tol, tolx, cap = args.batch_tol, args.batch_tol / 100.0, args.batch_max
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    t0 = time.perf_counter()
    xb = solvers.solve_batches([(t['y'], t['A'], t['regs']) for t in tracts], n_streams=args.batch_streams,
                               tol_fun=tol, tol_x=tolx, max_iter=cap)
    torch.cuda.synchronize()
    t_b = time.perf_counter() - t0
    ref, it_b, it_r = [], [], []
    for t, b in zip(tracts, xb):
        row = []
        for rp, (x0, d0) in zip(t['regs'], b):
            it_b.append(int(d0['iterations']))
            x1, d1 = solvers.solve(t['y'], t['A'], t['A'].T, tol_fun=tol, tol_x=tolx, max_iter=cap, verbose=0, x0=x0,
                                   regularisation=rp)
            it_r.append(int(d1['iterations']))
            row.append((x1, d1))
        ref.append(row)
    torch.cuda.synchronize()
    t_r = time.perf_counter() - t0
    t0 = time.perf_counter()
    seq, it_s = [], []
    for t in tracts:
        row = []
        for rp in t['regs']:
            x2, d2 = solvers.solve(t['y'], t['A'], t['A'].T, tol_fun=tol, tol_x=tolx, max_iter=cap, verbose=0,
                                   regularisation=rp)
            it_s.append(int(d2['iterations']))
            row.append((x2, d2))
        seq.append(row)
    torch.cuda.synchronize()
    t_s = time.perf_counter() - t0
    clk = clocks.stop()
    dist, cost = [], []
    for r, q in zip(ref, seq):
        for (x1, d1), (x2, d2) in zip(r, q):
            dist.append(float(torch.linalg.norm(x1 - x2) / torch.linalg.norm(x2)))
            cost.append((d1['cost_function'] - d2['cost_function']) / d2['cost_function'])
    n = len(dist)
    out = {'metric': 'regularisation paths to tolerance: batched BF16-LUT + FP64 polish vs sequential plain',
           'value': n / t_r, 'unit': 'solves/s', 'higher_is_better': True, 'n_gpus': 1, 'data': 'synthetic',
           'config': {'workload': f'{len(tracts)} tractograms x {len(tracts[0]["regs"])} lambdas, nonnegative group '
                                  f'lasso over 64 random bundles, grid 145x174x145, nS=288',
                      'fibers': [t['spec'].n_fibers for t in tracts], 'tol_fun': tol, 'tol_x': tolx, 'max_iter': cap},
           'batched_then_polished': {'seconds': t_r, 'batched_seconds': t_b, 'batched_iterations_median':
                                     statistics.median(it_b), 'polish_iterations_median': statistics.median(it_r)},
           'sequential_plain': {'seconds': t_s, 'iterations_median': statistics.median(it_s)},
           'speedup': t_s / t_r,
           'x_rel_polished_vs_plain': {'max': max(dist), 'median': statistics.median(dist)},
           'cost_rel_polished_minus_plain': {'max': max(cost), 'min': min(cost)},
           'clocks': clk, 'setup_s': {'generate': tgen}}
    print(json.dumps(out))
    return 0


def run_demo(args):
    """The 5k-streamline demo case (grid 32x32x16, nS = 66): operator pair time, and 200 FISTA
    nnls iterations with the host-driven loop (momentum reuse off and on) and with the loop
    captured as one CUDA graph.  Prints one JSON line."""
    import torch
    from commit_gb300 import solvers, synth
    from commit_gb300.operator import LinearOperator
    dev = torch.device('cuda', torch.cuda.current_device())
    spec = synth.SPECS['demo_5k']
    D, K = synth.make_dictionary(spec, device='cuda')
    A = LinearOperator(D, K, None, device=dev.index)
    x = torch.from_numpy(synth.make_x(A.nCOLS, 1)).to(dev)
    y = torch.from_numpy(synth.make_signal(A.dot(x).cpu().numpy(), 2)).to(dev)
    yy = torch.empty(A.nROWS, dtype=torch.float64, device=dev)
    g = torch.empty(A.nCOLS, dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream(dev)
    for _ in range(max(3, args.warmup)):
        A.dot(x, out=yy)
        A.T.dot(yy, out=g)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    n = 200
    for _ in range(n):
        A.dot(x, out=yy)
        A.T.dot(yy, out=g)
    e1.record(st)
    torch.cuda.synchronize()
    pair_ms = e0.elapsed_time(e1) / n
    rp = {'startIC': 0, 'sizeIC': A.ICnSTR * A.ICnRF, 'startEC': A.ICnSTR * A.ICnRF, 'sizeEC': A.ECn * A.ECnRF,
          'startISO': A.ICnSTR * A.ICnRF + A.ECn * A.ECnRF, 'sizeISO': A.ISOn * A.ISOnRF,
          'regIC': None, 'regEC': None, 'regISO': None, 'nnIC': True, 'nnEC': True, 'nnISO': True,
          'dictIC_params': None, 'dictEC_params': None, 'dictISO_params': None}
    out = {}
    for name, kw in (('host_loop_reuse', dict(momentum_reuse=True)), ('host_loop', dict(momentum_reuse=False)),
                     ('graph', dict(graph=True))):
        solvers.solve(y, A, A.T, tol_fun=0.0, tol_x=0.0, max_iter=5, verbose=0,
                      regularisation=solvers.init_regularisation(dict(rp)), **kw)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        xs, d = solvers.solve(y, A, A.T, tol_fun=0.0, tol_x=0.0, max_iter=n, verbose=0,
                              regularisation=solvers.init_regularisation(dict(rp)), **kw)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out[name] = {'seconds': dt, 'ms_per_iteration': 1000.0 * dt / n, 'iterations': d['iterations'],
                     'cost_function': d['cost_function']}
    # reduced-precision operator: errors of y = A x, of the FISTA solution x and of its cost
    # against the float-float FP64 path (same 200 iterations)
    xf, df = solvers.solve(y, A, A.T, tol_fun=0.0, tol_x=0.0, max_iter=n, verbose=0,
                           regularisation=solvers.init_regularisation(dict(rp)))
    yf = A.dot(x)
    errs = {}
    for ar in ('bf16', 'fp16', 'f32'):
        yr = A.dot(x.float(), arith=ar).double()
        xr, dr = solvers.solve(y, A, A.T, tol_fun=0.0, tol_x=0.0, max_iter=n, verbose=0,
                               regularisation=solvers.init_regularisation(dict(rp)), arith=ar)
        errs[ar] = {'y_rel': float(torch.linalg.norm(yr - yf) / torch.linalg.norm(yf)),
                    'x_rel': float(torch.linalg.norm(xr - xf) / torch.linalg.norm(xf)),
                    'cost_rel': abs(dr['cost_function'] - df['cost_function']) / df['cost_function']}
    cpu = None
    if not args.no_cpu:
        cpu = cpu_reference(D, K, 1.0, 20, 2)
    res = {'metric': 'demo case: A*x+A\'y pair time and FISTA ms/iteration (host loop vs CUDA graph)',
           'unit': 'ms', 'higher_is_better': False, 'data': 'synthetic',
           'config': {'workload': f'demo_5k: {spec.n_fibers} streamlines, grid 32x32x16, '
                                  f'{int(D["IC"]["nVOX"])} voxels, {int(D["IC"]["n"])} segments, nS=66',
                      'fista': '200 nnls iterations, tolerances off'},
           'pair_ms': pair_ms, 'pairs_per_s': 1000.0 / pair_ms, 'fista': out,
           'graph_speedup_vs_host_loop': out['host_loop']['seconds'] / out['graph']['seconds'],
           'reduced_precision_errors_vs_fp64': errs}
    if cpu is not None:
        res['cpu_baseline'] = cpu
    print(json.dumps(res))
    return 0


def run_trk2dict(args):
    """Voxelisation of synthetic streamlines (random smooth curves of 1-300 points, 0.7 mm
    steps) on the 145x174x145 grid at 1.25 mm with the 500-direction hash table: streamlines
    per second through commit_gb300.trk2dictionary.voxelise (host arrays in and out) against
    the CPU restatement of the reference's voxeliser (one thread) on a sample."""
    import torch
    from commit_gb300 import trk2dictionary as V
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import trk2dict as T
    rng = np.random.default_rng(20)
    dim, pix = (145, 174, 145), (1.25, 1.25, 1.25)
    nf = args.t2d_fibers
    n_pts = rng.integers(1, 300, size=nf)
    off = np.concatenate([[0], np.cumsum(n_pts)]).astype(np.int64)
    ext = np.array(dim) * np.array(pix)
    start = rng.uniform(0.2, 0.8, (nf, 3)) * ext
    steps = rng.normal(size=(int(off[-1]), 3))
    d = np.cumsum(0.3 * steps, axis=0)                       # smooth random directions
    d -= np.repeat(d[off[:-1]], n_pts, axis=0)
    d += np.repeat(rng.normal(size=(nf, 3)), n_pts, axis=0)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    seg = 0.7 * d
    pos = np.cumsum(seg, axis=0)
    pos -= np.repeat(pos[off[:-1]], n_pts, axis=0)
    pts = (pos + np.repeat(start, n_pts, axis=0)).astype(np.float32)
    dirs = synth_dirs(500)
    H = V.hash_table(dirs)
    for _ in range(max(1, args.warmup)):
        V.voxelise(pts[:off[min(nf, 1000)]], off[:min(nf, 1000) + 1], dim, pix, H)
    torch.cuda.synchronize()
    times = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        r = V.voxelise(pts, off, dim, pix, H)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    gpu_s = statistics.median(times)
    ns = min(nf, 5000)
    t0 = time.perf_counter()
    rc = T.voxelise(pts[:off[ns]], off[:ns + 1], dim, pix, H)
    cpu_s = time.perf_counter() - t0
    rg = V.voxelise(pts[:off[ns]], off[:ns + 1], dim, pix, H)
    same = all(np.array_equal(rg[c][k], rc[c][k]) for c in ('IC', 'TRK') for k in rc[c])
    out = {'metric': 'streamline voxelisation (trk2dictionary IC/EC/ISO) streamlines/s', 'value': nf / gpu_s,
           'unit': 'streamlines/s', 'higher_is_better': True, 'n_gpus': 1, 'data': 'synthetic',
           'config': {'workload': f'{nf} random smooth streamlines, 1-300 points of 0.7 mm, grid 145x174x145 '
                                  f'at 1.25 mm, 500 directions, intersections on',
                      'points': int(off[-1]), 'segments': int(r['IC']['f'].size), 'kept': int(r['TRK']['kept'].sum())},
           'seconds': gpu_s, 'e2e': {'value': nf / gpu_s, 'unit': 'streamlines/s',
                                     'note': 'host arrays in and out, all copies inside the timed call'},
           'cpu_baseline': {'value': ns / cpu_s, 'unit': 'streamlines/s', 'cores': 1, 'kind': 'port',
                            'sample': f'first {ns} streamlines, {cpu_s:.2f} s'},
           'sample_bitwise_equal_to_cpu': bool(same)}
    print(json.dumps(out))
    return 0


def synth_dirs(n: int) -> np.ndarray:
    from commit_gb300 import synth
    return synth.fibonacci_sphere(n, hemisphere=True)


def main():
    args = parse()
    if args.impl == 'reference':
        return run_reference(args)
    if args.demo:
        return run_demo(args)
    if args.trk2dict:
        return run_trk2dict(args)
    if args.batch:
        return run_batch(args)
    return run_ours(args)


if __name__ == '__main__':
    sys.exit(main())
