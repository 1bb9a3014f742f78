#!/usr/bin/env python
"""Throughput benchmark of the iso-acoustic FDTD hot path (forward + adjoint vp gradient).

Workload (one "step"): the 2D adjoint-state vp gradient of a batch of shots, i.e. the forward
modelling of every shot with the undersampled wavefield saved, the L2 residual against
observed traces, and the reverse-time adjoint with the vp imaging condition, summed over the
shots:

    512 x 512 inner grid at 0.25 mm + 20 absorbing cells per side (552 x 552 extended),
    seeded vp/rho/alpha ellipse phantom ('true' model, observed data) and a 1500 m/s starting
    vp, 1 MHz 3-cycle tone burst, 256 jittered transducers on a 55 mm circle, 64 shots (every
    4th transducer fires, all 256 receive), 4000 steps at CFL 0.6 (OT4), undersampling 4.

The inputs are synthetic (seeded phantoms) with the shapes of the reference's breast-imaging
examples; no dataset is involved. Throughput follows Devito's convention: extended grid points
x time steps executed (forward and adjoint) / seconds.

Arms: ``--impl gb300`` (default) runs libstrideacc.so; ``--impl reference`` times the
reference algorithm's CPU implementation on this machine's host cores (the C restatement in
oracle/, because the reference's Devito operator cannot be installed here).
"""

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0
L2_BYTES = 129 * 10**6  # GB300 L2
# dram__bytes_read.sum + dram__bytes_write.sum of one time step of this workload's batch (64 shots
# of 552^2: one launch each of the two step passes, a forward step), from an ncu capture of those
# launches: a fixed figure of the kernels, not measured by this run.
NCU_TRAFFIC_PER_STEP = (101.428224e6 + 37.445120e6) + (263.725312e6 + 52.639232e6)


WORKLOADS = {
    # name: (generator, shots per GPU, mode)
    'fwdadj64': ('batched', 64, 'fwdadj'),  # default: the fwd+adj vp gradient of the headline metric
    'fwd256': ('batched', 256, 'fwd'),      # batched forward, one shot per transducer
    'single': ('single', 1, 'fwd'),         # single-shot forward, 256^2 at 0.5 mm, vp only
    'single256': ('single', 1, 'fwd'),      # the same with 256^2 as the whole grid, sponge included
    '3d': ('3d', 8, 'fwd'),                 # 3D forward, 296^3, 8 shots per launch
    '3dgrad': ('3d', 1, 'fwdadj'),          # 3D fwd+adj vp gradient of one shot (snapshots in HBM)
    'exact64': ('batched', 64, 'fwdadj'),   # exact gradient (autograd backward), checkpoints every 50 steps
    '3dgrad8': ('3d', 8, 'fwdadj'),         # 3D gradient of 8 shots, checkpoints under a 150 GB budget
    'fwi': ('single', 32, 'fwi'),           # plain vs learned-preconditioned FWI, wall time to a vp error
    'unet': ('single', 0, 'unet'),          # the learned preconditioner's network: forward at batch 4, 256^2
    'rho64': ('batched', 64, 'fwdadj'),     # vp and rho gradients from the raw saved wavefield
    'pml64': ('batched', 64, 'fwdadj'),     # vp gradient with the CFS-PML boundary (OT2)
    'ckpt64': ('batched', 64, 'fwdadj'),    # the default gradient from checkpoints every 50 steps with recompute
}
# gradient method per workload: the reference imaging condition from snapshots (default), the
# same from checkpoints with recompute, or the exact discrete adjoint from checkpoints
# (plan arguments: undersampling, checkpoint interval, checkpoint byte budget)
GRADIENT = {
    'exact64': ('exact', dict(undersampling=1, checkpoint_interval=50)),
    '3dgrad8': ('checkpoints', dict(undersampling=4, checkpoint_budget=150e9)),
    'rho64': ('raw', dict(undersampling=4)),
    'pml64': ('snapshots', dict(undersampling=4, kernel='OT2', boundary='pml', f_centre=1.0e6)),
    'ckpt64': ('checkpoints', dict(undersampling=4, checkpoint_interval=50)),
}
# time step of the workload's grid as a CFL number (OT2 needs one below its stability limit)
CFL = {'pml64': 0.4}
# inner grid of a workload smaller than its generator's
INNER = {'single256': 216}
WORKLOAD_NAMES = {
    'fwdadj64': '2D fwd+adj vp gradient: 552^2 extended (512^2 at 0.25 mm + 20 sponge), vp/rho/alpha phantom, '
                '64 shots x 256 receivers, 4000 steps, OT4, f=4',
    'fwd256': '2D batched forward: 552^2 extended, vp/rho/alpha phantom, 256 shots x 256 receivers, 4000 steps, OT4',
    'single': '2D single-shot forward: 296^2 extended (256^2 at 0.5 mm + 20 sponge), vp phantom, 128 receivers, '
              '2000 steps, OT4',
    'single256': '2D single-shot forward: 256^2 extended (216^2 at 0.5 mm + 20 sponge), vp phantom, 128 receivers, '
                 '2000 steps, OT4',
    '3d': '3D forward: 296^3 extended (256^3 at 0.5 mm + 20 sponge), vp/rho/alpha phantom, 8 shots x 512 receivers, '
          '3000 steps, OT4',
    '3dgrad': '3D fwd+adj vp gradient: 296^3 extended, vp/rho/alpha phantom, 1 shot x 512 receivers, 3000 steps, '
              'OT4, f=4',
    'exact64': '2D exact vp gradient (torch.autograd backward of the discrete forward map): 552^2 extended, '
               'vp/rho/alpha phantom, 64 shots x 256 receivers, 4000 steps, OT4, checkpoints every 50 steps with '
               'recompute',
    '3dgrad8': '3D fwd+adj vp gradient: 296^3 extended, vp/rho/alpha phantom, 8 shots per launch x 512 receivers, '
               '3000 steps, OT4, f=4, checkpoints under a 150 GB budget with recompute',
    'rho64': '2D fwd+adj vp and rho gradients (raw saved wavefield, held imaging terms every step): 552^2 extended, '
             'vp/rho/alpha phantom, 64 shots x 256 receivers, 4000 steps, OT4, f=4',
    'pml64': '2D fwd+adj vp gradient with the CFS-PML boundary: 552^2 extended (20-cell PML), vp/rho/alpha phantom, '
             '64 shots x 256 receivers, 4000 steps, OT2 at CFL 0.4, f=4',
    'ckpt64': '2D fwd+adj vp gradient: 552^2 extended, vp/rho/alpha phantom, 64 shots x 256 receivers, 4000 steps, '
              'OT4, f=4, forward wavefield checkpointed every 50 steps and recomputed for the imaging condition',
    'fwi': 'FWI of seeded 256^2 ellipse phantoms at 0.5 mm (296^2 extended), 32 shots x 128 receivers, 2000 steps, '
           '500 kHz, f_max 0.5 MHz: plain (reference loop, GPU pipelines) vs U-Net-preconditioned (BF16 tcgen05, '
           'trained on plain-FWI paths of held-out seeds), wall time to the target relative vp error',
}


WORKLOAD_NAMES['unet'] = ('learned preconditioner U-Net (4 levels, 32-64-128-256 channels, BF16 tcgen05, implicit-GEMM '
                          '3x3 convolutions) forward on a batch of 4 inputs of 256^2 x 2 channels')


def workload_name(name, nt):
    """The workload's description with its actual number of time steps."""
    return re.sub(r'\d+ steps', '%d steps' % nt, WORKLOAD_NAMES[name])


def workload_config(name='fwdadj64', nt=None, n_shots=None, rank=0):
    from stride_gb300 import phantoms
    gen, default_shots, _ = WORKLOADS[name]
    n_shots = default_shots if n_shots is None else n_shots
    if gen == '3d':
        w = phantoms.workload3d(seed=0, nt=nt, n_shots=n_shots)
    else:
        w = phantoms.workload(gen, seed=0, nt=nt, cfl=CFL.get(name, 0.6), inner=INNER.get(name))
    ntr = len(w['geometry'])
    stride = max(1, ntr // n_shots)
    first = rank % stride
    shots = list(range(first, ntr, stride))[:n_shots]
    w['shots'] = shots
    w['src'] = [w['geometry'][[s]] for s in shots]
    w['rec'] = [w['geometry'] for _ in shots]
    return w


def sponge_fraction(w):
    n = np.prod(w['shape'])
    inner = np.prod([s - 2 * a for s, a in zip(w['shape'], w['absorbing'])])
    return 1.0 - inner / n


def alg_bytes_per_point(w):
    """Compulsory FP32 traffic per grid point and time step with no temporal reuse:
    p[t], p[t-1] read, p[t+1] written, one read per medium field (vp, rho, alpha), the damping
    profile in the sponge; +4/f forward (snapshot write), +20/f adjoint (snapshot read,
    grad/prec read-modify-write)."""
    n_mat = 1 + (w['rho'] is not None) + (w['alpha'] is not None)
    base = 4.0 * (3 + n_mat) + 4.0 * sponge_fraction(w)
    f = 4
    return base + 4.0 / f, base + 20.0 / f


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix='.csv')
        os.close(fd)
        q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), '--query-gpu=' + q,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        out = {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': []}
        try:
            rows = [l.split(',') for l in open(self.path).read().strip().splitlines() if l.strip()]
            os.unlink(self.path)
        except Exception:
            return out
        sm, mx, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == 'active':
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if sm:
            out['sm_mhz'] = statistics.median(sm)
            out['sm_max_mhz'] = max(mx)
            out['samples'] = len(sm)
        out['reasons'] = sorted(reasons)
        return out


def measured_hbm():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            return float(json.load(f)['hbm_gbs']), 'measured'
    except Exception:
        return HBM_FALLBACK_GBS, 'fallback'


def cpu_arm(w, target_s=15.0, threads=None, calib=True, mode='fwdadj', full=False):
    """Times the oracle's C restatement of the reference operator (one shot: forward, plus
    the adjoint for mode 'fwdadj') on the host cores; returns GPts/s and the sample description.
    full: every time step of the shot, no calibration run."""
    from oracle import c_oracle
    threads = threads or os.cpu_count()
    origin = tuple(-e * h for e, h in zip(w['extra'], w['spacing']))
    N = int(np.prod(w['shape']))
    grad = mode == 'fwdadj'

    def run(nt):
        wav = w['wavelet'][:nt][None]
        t0 = time.perf_counter()
        tr, snaps = c_oracle.forward(w['vp'], w['spacing'], w['dt'], nt, w['absorbing'], w['src'][0], w['rec'][0],
                                     wav, origin, rho=w['rho'], alpha=w['alpha'], kernel='OT4', save=grad,
                                     nthreads=threads)
        pts = N * (nt - 2)
        if grad:
            c_oracle.adjoint(w['vp'], w['spacing'], w['dt'], nt, w['absorbing'], w['rec'][0], tr, origin, snaps,
                             rho=w['rho'], alpha=w['alpha'], kernel='OT4', nthreads=threads)
            pts += N * (nt - 1 - 4)
        dt = time.perf_counter() - t0
        return pts / dt / 1e9, dt

    if full:
        nt = w['nt']
        rate, dt = run(nt)
        return rate, threads, '1 shot of the workload, %s, %d of %d steps, %.1f s' % (
            'forward (save) + adjoint' if grad else 'forward', nt, w['nt'], dt), dt
    nt = min(24, w['nt'])
    rate, dt = run(nt)
    if calib:
        nt = int(min(w['nt'], max(nt, nt * target_s / max(dt, 1e-3))))
        rate, dt = run(nt)
    sample = '1 shot of the workload, %s, %d of %d steps, %.1f s' % (
        'forward (save) + adjoint' if grad else 'forward', nt, w['nt'], dt)
    return rate, threads, sample, dt


def _density(w):
    from stride_gb300 import _lib
    if w['rho'] is None:
        return _lib.SA_DENSITY_NONE
    r = w['rho']
    return _lib.SA_DENSITY_CONSTANT if np.isclose(np.min(r), np.max(r)) else _lib.SA_DENSITY_VARIABLE


def _points(w, workload):
    mode = WORKLOADS[workload][2]
    N = int(np.prod(w['shape']))
    nt = w['nt']
    pts = N * len(w['shots']) * (nt - 2)
    if mode == 'fwdadj':
        pts += N * len(w['shots']) * (nt - 1 - 4)
    return pts


METRIC = {'fwdadj': 'GPts/s (forward+adjoint vp gradient)', 'fwd': 'GPts/s (forward)',
          'unet': 'TFLOP/s (U-Net forward, tensor-core GEMM FLOPs of every convolution)',
          'fwi': 'seconds to the target relative vp error (learned-preconditioned FWI, median over test phantoms)'}


def _fwi_workload(seed):
    from stride_gb300 import phantoms
    w = phantoms.workload('single', seed=seed)
    shots = list(range(0, 128, 4))
    w['shots'] = shots
    w['src'] = [w['geometry'][[s]] for s in shots]
    w['rec'] = [w['geometry'] for _ in shots]
    return w


def unet_arm(args):
    """The U-Net's forward pass (the learned FWI's inference) on a batch of 4 seeded 256^2 inputs:
    tensor-core GEMM FLOPs of every convolution over the CUDA-event time of the pass."""
    import torch
    from stride_gb300.unet import UNet
    torch.cuda.set_device(0)
    g = torch.Generator(device='cpu').manual_seed(0)
    x = torch.randn((4, 256, 256, 2), generator=g).cuda()
    net = UNet(seed=0)
    for _ in range(args.warmup):
        net.forward(x)
    torch.cuda.synchronize()
    flush = torch.empty(64 * 2**20, dtype=torch.float32, device='cuda')  # the activations fit in L2
    times = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            net.forward(x)
            e1.record()
            times.append((e0, e1))
        torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in times) / len(times)
    flops = sum(2.0 * layer.saved[3] * layer.saved[4] * layer.saved[5] * layer.coutp * layer.kp
                for layer in net.layers())
    tflops = flops / (ms * 1e-3) / 1e12
    peak = 1883.3
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as f:
            peak, src = float(json.load(f)['bf16_tflops']), 'measured'
    except Exception:
        src = 'fallback'
    line = {
        'metric': METRIC['unet'], 'value': tflops, 'unit': 'TFLOP/s', 'n_gpus': 1, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'bf16 operands, fp32 accumulation', 'data': 'synthetic (seeded normal inputs, He-initialised weights)',
        'config': {'workload': WORKLOAD_NAMES['unet'], 'batch': 4, 'image': [256, 256],
                   'l2_flush': 'L2 flushed between timed passes (256 MB write, outside the passes\' events)'},
        'roofline': {'bound': 'tensor', 'achieved': tflops, 'peak': peak, 'unit': 'TFLOP/s', 'frac': tflops / peak,
                     'peak_source': src, 'traffic': None, 'kernel': 'k_umma_gemm (every convolution of the pass)'},
        'cpu_baseline': None, 'e2e': None, 'gpu_launches': None, 'clocks': clk.summary(),
        'gemm_timeouts': net.errors(),
    }
    print(json.dumps(line))
    return 0


def fwi_arm(args):
    """Plain vs learned FWI on one GPU: training pairs from plain-FWI paths of training seeds, U-Net
    training, then wall time to the target error on test seeds (both methods, same GPU)."""
    import torch
    from stride_gb300.fwi import LearnedFWI, PlainFWI, generate_pairs, run_to_error, train_unet
    from stride_gb300.unet import UNet
    torch.cuda.set_device(0)
    target, fmax = args.fwi_target, 0.5e6
    w0 = _fwi_workload(1000)
    plain = PlainFWI(w0, step_size=1.0)
    # the plain step size: the fastest to the target on two validation seeds (outside the training
    # and test seeds), ties broken by the final error; both methods then use it
    sweep = {}
    for st in [float(v) for v in args.fwi_steps.split(',')]:
        plain.set_step_size(st)
        res = [run_to_error(plain, _fwi_workload(2000 + i)['vp'], target, max_iter=args.fwi_iters, f_max=fmax)
               for i in range(2)]
        sweep[st] = (statistics.median([r[0] if r[0] is not None else float('inf') for r in res]),
                     float(np.mean([r[2][-1] for r in res])))
    step = min(sweep, key=lambda st: sweep[st])
    plain.set_step_size(step)
    t0 = time.perf_counter()
    X, T = generate_pairs(plain, [_fwi_workload(1000 + i)['vp'] for i in range(args.fwi_train)], iterations=5,
                          f_max=fmax)
    torch.cuda.synchronize()
    t_pairs = time.perf_counter() - t0
    net = UNet(seed=0)
    t0 = time.perf_counter()
    losses = train_unet(net, X, T, epochs=args.fwi_epochs, batch=4, lr=1e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    # tensor-core rate of the network's forward pass (batch 4, the training shape): GEMM FLOPs of
    # every convolution over the CUDA-event time of the whole forward
    xb = X[:4].contiguous()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    net.forward(xb)
    ev0.record()
    for _ in range(5):
        net.forward(xb)
    ev1.record()
    torch.cuda.synchronize()
    fwd_ms = ev0.elapsed_time(ev1) / 5
    flops = sum(2.0 * layer.saved[3] * layer.saved[4] * layer.saved[5] * layer.coutp * layer.kp
                for layer in net.layers())
    learned = LearnedFWI(w0, net, step_size=step)
    # one untimed iteration of each solver on a seed outside the test set, so that first-use costs
    # (graph capture, allocations, filter design) fall in neither method's timing
    for solver in (plain, learned):
        solver.reset(_fwi_workload(999)['vp'])
        solver.iterate(fmax)
    torch.cuda.synchronize()
    rows = []
    for seed in range(args.fwi_test):
        vt = _fwi_workload(seed)['vp']
        tp, ip, ep = run_to_error(plain, vt, target, max_iter=args.fwi_iters, f_max=fmax)
        tl, il, el = run_to_error(learned, vt, target, max_iter=args.fwi_iters, f_max=fmax)
        rows.append({'seed': seed, 'initial_error': ep[0], 'plain_s': tp, 'plain_iters': ip, 'plain_final': ep[-1],
                     'learned_s': tl, 'learned_iters': il, 'learned_final': el[-1],
                     'learned_steps_accepted': sum(h.get('learned', False) for h in learned.history)})

    def med(key):
        v = [r[key] if r[key] is not None else float('inf') for r in rows]
        return float(statistics.median(v)) if v else None

    line = {
        'metric': METRIC['fwi'], 'value': med('learned_s'), 'unit': 's', 'n_gpus': 1, 'steps': len(rows),
        'warmup': 0, 'ms_per_step': None, 'higher_is_better': False, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f32 solver, bf16 network', 'data': 'synthetic (seeded ellipse phantoms)',
        'config': {'workload': WORKLOAD_NAMES['fwi'], 'target_error': target, 'step_size': step,
                   'step_sweep': {str(k): {'median_s_to_target': v[0], 'mean_final_error': v[1]}
                                  for k, v in sweep.items()},
                   'train_phantoms': args.fwi_train, 'pairs': int(X.shape[0]), 'epochs': args.fwi_epochs,
                   'test_phantoms': args.fwi_test, 'max_iterations': args.fwi_iters},
        'plain_median_s': med('plain_s'), 'learned_median_s': med('learned_s'),
        'plain_reached': sum(r['plain_s'] is not None for r in rows),
        'learned_reached': sum(r['learned_s'] is not None for r in rows),
        'pair_generation_s': t_pairs, 'training_s': t_train, 'training_loss': [losses[0], losses[-1]],
        'gemm_timeouts': net.errors(), 'unet_forward_ms_batch4': fwd_ms,
        'unet_forward_tflops': flops / (fwd_ms * 1e-3) / 1e12, 'per_phantom': rows,
    }
    print(json.dumps(line))
    plain.close()
    learned.close()
    return 0


def reference_arm(args):
    """The reference algorithm's CPU implementation on all host cores. One step is one whole shot
    of the workload (every time step of the forward with save and, for gradient workloads, of the
    adjoint), the unit the reference's own worker processes at a time; `value` is that shot's
    points over its measured time, and `ms_per_step` the measured time of one such step."""
    rank = int(os.environ.get('RANK', '0'))
    if rank != 0:
        return 0
    w = workload_config(args.workload, nt=args.nt, n_shots=args.shots)
    mode = WORKLOADS[args.workload][2]
    threads = os.cpu_count()
    for _ in range(args.warmup):
        cpu_arm(w, threads=threads, calib=False, mode=mode, full=True)
    rates, times, sample = [], [], ''
    for _ in range(args.steps):
        r, _, sample, dt = cpu_arm(w, threads=threads, calib=False, mode=mode, full=True)
        rates.append(r)
        times.append(dt)
    ms_step = 1e3 * sum(times) / len(times)
    N = int(np.prod(w['shape']))
    shot_pts = N * (w['nt'] - 2) + (N * (w['nt'] - 1 - 4) if mode == 'fwdadj' else 0)
    value = shot_pts / (ms_step * 1e-3) / 1e9
    line = {
        'impl': 'reference', 'metric': METRIC[mode], 'value': value, 'unit': 'GPts/s',
        'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': ms_step, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic (seeded phantoms)',
        'config': {'workload': workload_name(args.workload, w['nt']), 'grid': list(w['shape']), 'shots': len(w['shots']),
                   'nt': w['nt'], 'kernel': 'OT4', 'l2_flush': 'inputs larger than L2',
                   'step': 'one whole shot of the workload per step (%s); the %d-shot batch is %d such steps'
                           % (sample, len(w['shots']), len(w['shots']))},
        'cpu_baseline': {'value': value, 'unit': 'GPts/s', 'cores': threads, 'kind': 'port',
                         'sample': sample + ' per step, %d steps (the reference Devito operator cannot be installed '
                                            'here; this is the oracle C/OpenMP restatement of it)' % args.steps},
        'e2e': {'value': value, 'unit': 'GPts/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line))
    return 0


def gb300_arm(args):
    import torch
    import torch.distributed as dist
    import scipy.signal
    from stride_gb300 import _lib, shards

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if world != args.gpus:
        raise SystemExit('bench.py: %d rank(s) running for --gpus %d' % (world, args.gpus))
    if world > 1:
        dist.init_process_group('nccl')
    torch.cuda.set_device(local)
    dev = torch.device('cuda', local)
    stream = torch.cuda.current_stream()
    mode = WORKLOADS[args.workload][2]
    grad_mode = mode == 'fwdadj'

    w = workload_config(args.workload, nt=args.nt, n_shots=args.shots, rank=rank)
    nt = w['nt']
    dim = len(w['shape'])
    n_shots = len(w['shots'])
    N = int(np.prod(w['shape']))
    eps = 1e-3 * np.asarray(w['spacing'])
    so = np.cumsum([0] + [len(x) for x in w['src']])
    ro = np.cumsum([0] + [len(x) for x in w['rec']])
    sx = (np.concatenate(w['src']) + eps).astype(np.float32)
    rx = (np.concatenate(w['rec']) + eps).astype(np.float32)
    win = scipy.signal.get_window(('tukey', 0.001), nt, False).astype(np.float32)

    method, plan_kw = GRADIENT.get(args.workload, ('snapshots', dict(undersampling=4)))
    save = {'snapshots': True, 'checkpoints': 'checkpoints', 'exact': 'checkpoints', 'raw': 'raw'}[method] \
        if grad_mode else False
    exact = method == 'exact'
    rho_grad = method == 'raw'
    plan_kw = dict(plan_kw)
    kernel = plan_kw.pop('kernel', 'OT4')
    plan = _lib.Plan(dim, w['shape'], w['spacing'], w['extra'], w['absorbing'], w['dt'], nt, kernel=kernel,
                     density=_density(w), attenuation=w['alpha'] is not None, max_shots=n_shots, **plan_kw)
    plan.set_geometry(so, sx, ro, rx)
    wav = torch.from_numpy(np.tile((w['wavelet'] * win)[None].astype(np.float32), (plan.n_src, 1))).to(dev)
    win_d = torch.from_numpy(win).to(dev)
    observed = torch.zeros((plan.n_rec, nt), device=dev)
    if grad_mode:  # observed data from the true phantom; the gradient is taken at 1500 m/s
        plan.set_medium(w['vp'], w['rho'], w['alpha'])
        plan.forward(wav, observed, stream=stream)
        plan.set_medium(np.full(w['shape'], 1500., np.float32), w['rho'], w['alpha'])
    else:
        plan.set_medium(w['vp'], w['rho'], w['alpha'])
    plan.autotune(stream=stream)
    traces = torch.zeros((plan.n_rec, nt), device=dev)
    grad = torch.zeros(w['shape'], device=dev)
    prec = torch.zeros(w['shape'], device=dev)
    rho_out = dict(grad_rho=torch.zeros(w['shape'], device=dev), prec_rho=torch.zeros(w['shape'], device=dev)) \
        if rho_grad else {}

    ev = lambda: torch.cuda.Event(enable_timing=True)
    fwd_ms, adj_ms = [], []
    launches = {'n': 0}

    def step(timed=False):
        e0, e1, e2 = ev(), ev(), ev()
        e0.record(stream)
        plan.forward(wav, traces, save=save, stream=stream)
        launches['n'] += plan.launches
        launches['persistent'] = dim == 2 and plan.launches <= 3  # transposes and the one launch
        e1.record(stream)
        if grad_mode:
            res = (traces - observed) * win_d[None, :]  # L2 residual, adjoint-source window
            plan.adjoint(res, grad, prec, stream=stream, exact=exact, **rho_out)
            launches['n'] += plan.launches
        e2.record(stream)
        if world > 1 and grad_mode:
            shards.allreduce_sum(grad, prec)  # the one exchange step: per-rank sums over every shot
        if timed:
            fwd_ms.append((e0, e1))
            adj_ms.append((e1, e2))

    # between timed steps, L2 is flushed (a 256 MB write) when a step's wavefields fit in it; the
    # step time is then the sum of the steps' own events, the flush outside them
    ws_bytes = 2 * N * n_shots * 4
    flush = torch.empty(64 * 2**20, dtype=torch.float32, device=dev) if ws_bytes < 2 * L2_BYTES else None

    torch.cuda.nvtx.range_push('warmup')
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches['n'] = 0
    with ClockSampler(local) as clk:
        t0, t1 = ev(), ev()
        torch.cuda.nvtx.range_push('timed')  # a profiler can restrict its capture to this range
        t0.record(stream)
        for _ in range(args.steps):
            if flush is not None:
                with torch.cuda.stream(stream):
                    flush.zero_()
            step(timed=True)
        t1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    if world > 1:
        dist.barrier()
    ms = t0.elapsed_time(t1)
    if flush is not None:
        ms = sum(a.elapsed_time(b) + c.elapsed_time(d) for (a, b), (c, d) in zip(fwd_ms, adj_ms))
    if world > 1:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    persistent = bool(launches.get('persistent'))
    pts_step = _points(w, args.workload)
    value = pts_step * world / (ms_step * 1e-3) / 1e9
    assert torch.isfinite(traces).all(), 'traces are not finite'
    if grad_mode:
        assert torch.isfinite(grad).all(), 'gradient is not finite'
        if nt >= 1000:  # by then the waves have reached the receivers
            assert float(grad.abs().max()) > 0, 'gradient is empty'

    # roofline of the step kernel(s): algorithmic bytes of a time step / average step time
    t_fwd = sum(a.elapsed_time(b) for a, b in fwd_ms) / len(fwd_ms)
    t_adj = sum(a.elapsed_time(b) for a, b in adj_ms) / len(adj_ms)
    b_fwd, b_adj = alg_bytes_per_point(w)
    if not grad_mode:
        b_fwd -= 4.0 / 4  # no snapshot write
    steps_f, steps_a = nt - 2, (nt - 1 - 4) if grad_mode else 0
    alg_bytes = N * n_shots * (steps_f * b_fwd + steps_a * b_adj)
    per_step_s = (t_fwd + t_adj) * 1e-3 / (steps_f + steps_a)
    achieved = alg_bytes / (steps_f + steps_a) / per_step_s / 1e9
    peak, peak_kind = measured_hbm()

    # end to end through the C ABI with host buffers (pinned), residual formed on the host
    e2e = None
    if not args.no_e2e:
        wav_h = wav.cpu().pin_memory()
        obs_h = observed.cpu()
        tr_h = torch.zeros((plan.n_rec, nt)).pin_memory()
        res_h = torch.zeros((plan.n_rec, nt)).pin_memory()
        g_h = torch.zeros(w['shape']).pin_memory()
        p_h = torch.zeros(w['shape']).pin_memory()
        rho_h = dict(grad_rho=torch.zeros(w['shape']).pin_memory(), prec_rho=torch.zeros(w['shape']).pin_memory()) \
            if rho_grad else {}
        win_h = torch.from_numpy(win)[None, :]

        def e2e_step():
            plan.forward(wav_h, tr_h, save=save, stream=stream)
            if grad_mode:
                # the residual on the host, with PyTorch's multithreaded CPU kernels
                torch.mul(torch.sub(tr_h, obs_h, out=res_h), win_h, out=res_h)
                plan.adjoint(res_h, g_h, p_h, stream=stream, exact=exact, **rho_h)

        e2e_step()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        s0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        es = (time.perf_counter() - s0) / args.steps
        if world > 1:
            t = torch.tensor([es], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            es = float(t.item())
        h2d = wav_h.numel() * 4 + (res_h.numel() * 4 if grad_mode else 0)
        d2h = tr_h.numel() * 4 + ((2 + 2 * rho_grad) * g_h.numel() * 4 if grad_mode else 0)
        e2e = {'value': pts_step * world / es / 1e9, 'unit': 'GPts/s', 'h2d_bytes_per_step': int(h2d),
               'd2h_bytes_per_step': int(d2h)}

    cpu = None
    # the C port restates the sponge / p.dt2 path only: no CPU line for the raw-save and CFS-PML workloads
    if rank == 0 and world == 1 and not args.no_cpu and args.workload not in ('rho64', 'pml64'):
        # 2D: one whole shot, as the reference arm times it; 3D: a calibrated sample of one shot
        rate, cores, sample, _ = cpu_arm(w, target_s=args.cpu_seconds, mode=mode, full=dim == 2)
        cpu = {'value': rate, 'unit': 'GPts/s', 'cores': cores, 'kind': 'port', 'sample': sample}

    if rank == 0:
        snap_gb = N * n_shots * (nt // 4) * 4 / 1e9 if grad_mode and method == 'snapshots' else 0.0
        line = {
            'metric': METRIC[mode], 'value': value, 'unit': 'GPts/s', 'n_gpus': world,
            'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms_step, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic (seeded phantoms)',
            'config': {'workload': workload_name(args.workload, nt), 'grid': list(w['shape']),
                       'shots_per_gpu': n_shots, 'nt': nt, 'kernel': 'OT4',
                       'layout': dict(zip(('threads', 'strips' if dim == 2 else 'tiles', 'chunks'), plan.layout)),
                       'gradient': (method + (' (adjoint time includes the forward recompute from checkpoints)'
                                              if method != 'snapshots' else '')) if grad_mode else None,
                       'parallelism': 'shots sharded over %d GPU(s)%s' % (world, ', gradient all-reduce' if grad_mode else ''),
                       'path': 'persistent (every time step in one launch)' if persistent
                               else 'streaming passes (one launch per time step)',
                       'l2_flush': ('L2 flushed between timed steps (256 MB write, outside the steps\' events): '
                                    '%.1f MB of wavefields per step' % (ws_bytes / 1e6)) if flush is not None
                                   else 'inputs larger than L2 (%.1f GB of wavefields per step)'
                                   % (ws_bytes / 1e9 + snap_gb)},
            'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                         'frac': achieved / peak, 'peak_source': peak_kind,
                         'traffic': NCU_TRAFFIC_PER_STEP if args.workload == 'fwdadj64' else None,
                         'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum of one forward time '
                                           'step (passes L and U) of this workload (a profile figure, not measured '
                                           'in this run)' if args.workload == 'fwdadj64' else None,
                         'alg_bytes_per_point': {'forward': b_fwd, 'adjoint': b_adj if grad_mode else None},
                         'kernel': 'fdtd3d_pass (A + B per time step)' if dim == 3 else
                                   ('fdtd2d_persist (every time step of a forward)' if persistent
                                    else 'fdtd2d_pass (L + U per time step)'),
                         'step_ms': per_step_s * 1e3},
            'cpu_baseline': cpu, 'e2e': e2e, 'gpu_launches': launches['n'], 'clocks': clk.summary(),
            'forward_ms': t_fwd, 'adjoint_ms': t_adj if grad_mode else None,
        }
        print(json.dumps(line))
    plan.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


def _free_port():
    import socket
    with socket.socket() as so:
        so.bind(('127.0.0.1', 0))
        return so.getsockname()[1]


def launch_ranks(n, argv, port=None, capture=False):
    """Runs the script argv[0] (with argv[1:]) as n ranks of one node under torch.distributed.run,
    rendezvous on 127.0.0.1; returns the exit status (and the ranks' stdout when capture)."""
    cmd = [sys.executable, '-m', 'torch.distributed.run', '--nnodes=1', '--nproc-per-node', str(n),
           '--master-addr', '127.0.0.1', '--master-port', str(port or _free_port())] + list(argv)
    env = dict(os.environ, OMP_NUM_THREADS=os.environ.get('OMP_NUM_THREADS', '1'))
    if capture:
        r = subprocess.run(cmd, env=env, stdout=subprocess.PIPE, text=True)
        return r.returncode, r.stdout
    return subprocess.call(cmd, env=env)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split('\n')[0])
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=3)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--nt', type=int, default=None, help='time steps (default: the workload\'s 4000)')
    ap.add_argument('--workload', default='fwdadj64', choices=sorted(WORKLOADS))
    ap.add_argument('--shots', type=int, default=None, help='shots per GPU (default: the workload\'s)')
    ap.add_argument('--cpu-seconds', type=float, default=15.0)
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--fwi-train', type=int, default=48, help='training phantoms (fwi workload)')
    ap.add_argument('--fwi-epochs', type=int, default=15)
    ap.add_argument('--fwi-test', type=int, default=16, help='test phantoms (fwi workload)')
    ap.add_argument('--fwi-steps', default='1,2,4', help='plain step sizes swept on validation seeds (fwi workload)')
    ap.add_argument('--fwi-target', type=float, default=0.01)
    ap.add_argument('--fwi-iters', type=int, default=25)
    args = ap.parse_args()
    if args.gpus > 1 and 'WORLD_SIZE' not in os.environ:
        # one process per GPU: this script again as --gpus ranks under torch.distributed.run
        return launch_ranks(args.gpus, [os.path.abspath(__file__)] + sys.argv[1:])
    if args.workload == 'unet':
        if args.impl == 'reference':
            print(json.dumps({'impl': 'reference', 'unavailable': 'the U-Net is the learned part, which has no '
                              'counterpart in the reference'}))
            return 0
        return unet_arm(args)
    if args.workload == 'fwi':
        if args.impl == 'reference':
            print(json.dumps({'impl': 'reference', 'unavailable': 'the fwi workload compares two GPU methods; its '
                              'solver throughput against the CPU port is the fwdadj/single workloads\' line'}))
            return 0
        return fwi_arm(args)
    if args.impl == 'reference':
        return reference_arm(args)
    return gb300_arm(args)


if __name__ == '__main__':
    sys.exit(main())
