"""Host-side pieces of bench.py (no GPU): workload shapes and names, the algorithmic bytes per point,
the point count of a step, the clock sampler's parsing and the reference arm's JSON line."""

import json
import subprocess
import sys

import numpy as np

import bench


def test_workload_configs_have_the_stated_shapes():
    w = bench.workload_config('fwdadj64', nt=40)
    assert w['shape'] == (552, 552) and len(w['shots']) == 64 and w['nt'] == 40
    assert w['rho'] is not None and w['alpha'] is not None
    w = bench.workload_config('single', nt=30)
    assert w['shape'] == (296, 296) and len(w['shots']) == 1 and w['rho'] is None
    w = bench.workload_config('pml64', nt=30)
    assert np.isclose(w['dt'], 0.4 * w['spacing'][0] / 1650.)  # OT2 within its stability limit
    assert '30 steps' in bench.workload_name('fwdadj64', 30)


def test_algorithmic_bytes_and_points():
    w = bench.workload_config('fwdadj64', nt=40)
    fwd, adj = bench.alg_bytes_per_point(w)
    phi = bench.sponge_fraction(w)
    assert np.isclose(fwd, 4 * (3 + 3) + 4 * phi + 1) and np.isclose(adj, fwd + 4)
    N = 552 * 552 * 64
    assert bench._points(w, 'fwdadj64') == N * (40 - 2) + N * (40 - 1 - 4)


def test_clock_sampler_summary(tmp_path):
    c = bench.ClockSampler()
    c.path = str(tmp_path / 'clk.csv')
    with open(c.path, 'w') as f:
        f.write('0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active\n')
        f.write('0, 2070, 2070, 1300.0, 0x4, Not Active, Not Active, Not Active, Active\n')
    s = c.summary()
    assert s['sm_mhz'] == 2070.0 and s['sm_max_mhz'] == 2070.0 and s['reasons'] == ['sw_power_cap']


def test_reference_arm_prints_one_json_line():
    """`bench.py --impl reference` on a short time axis: the contract's keys, the reference tag and a
    zero-copy e2e (the CPU port has no host-device transfers)."""
    out = subprocess.run([sys.executable, 'bench.py', '--impl', 'reference', '--nt', '12', '--steps', '1',
                          '--warmup', '0', '--cpu-seconds', '0.5'], capture_output=True, text=True, timeout=600,
                         cwd=bench.ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ('metric', 'value', 'unit', 'n_gpus', 'steps', 'warmup', 'ms_per_step', 'higher_is_better', 'scaling',
              'vs_baseline', 'dtype', 'data', 'config', 'cpu_baseline', 'e2e'):
        assert k in d
    assert d['impl'] == 'reference' and d['value'] > 0 and d['e2e']['h2d_bytes_per_step'] == 0
    assert d['cpu_baseline']['kind'] == 'port' and d['cpu_baseline']['cores'] >= 1
