"""Generates tests/golden/imaging_tutorial.npz (run: python tests/golden/make_imaging_golden.py).

The reference's imaging tutorial (stride_examples/tutorials/06_imaging.ipynb) runs full-waveform
inversion on the breast2D true model with Devito and keeps its printed log in the notebook. The
first iteration's per-shot functional values in that log are outputs of the reference itself: each
is the L2 loss, after the default trace pipelines, between the Devito forward of the true model
(the "observed" data) and the Devito forward of the homogeneous 1500 m/s starting model, for one of
15 randomly selected shots. This script

  * checks the tutorial's setup in its own code cells (grid, time axis, geometry, wavelet,
    frequency band, filter relaxation), so the fixture records the configuration those values
    belong to;
  * extracts the 15 values of block 1, iteration 1 from the log, and those of iteration 2, which the
    tutorial computes after one gradient-descent step (step size 10, clip 1400-1700 m/s) from the
    first iteration's summed gradient;
  * decodes the true model (stride_examples/examples/breast2D/data/anastasio2D-TrueModel.h5) with
    stride_gb300.h5 and checks it against the SHA-256 that tests/golden/anastasio2d_truemodel.json
    pins;

and writes them to one fixture.
"""

import hashlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from stride_gb300 import h5  # noqa: E402
from tests.golden import make_h5_golden  # noqa: E402

NOTEBOOK = os.path.join(make_h5_golden.REFERENCE_ROOT, 'stride_examples', 'tutorials', '06_imaging.ipynb')
OUT = os.path.join(HERE, 'imaging_tutorial.npz')

# the tutorial's setup, as its code cells state it
SETUP = [
    'Space(shape=(356, 385), extra=(50, 50), absorbing=(40, 40), spacing=0.5e-3)',
    'Time(start=0.0e-6, step=0.08e-6, num=2500)',
    'num_locations = 120',
    "problem.geometry.default('elliptical', num_locations)",
    'problem.acquisitions.default()',
    'f_centre = 0.50e6',
    'n_cycles = 3',
    'wavelets.tone_burst(f_centre, n_cycles, time.num, time.step)',
    'vp.fill(1500.)',
    'step_size = 10',
    'ProcessModelIteration(min=1400., max=1700.)',
    'GradientDescent(vp, step_size=step_size,',
    'max_freqs = [0.3e6, 0.4e6]',
    'process_wavelets(wavelets, f_max=f_max, filter_relaxation=0.75',
    'process_observed(observed, f_max=f_max, filter_relaxation=0.75',
    'process_traces(modelled, observed, f_max=f_max, filter_relaxation=0.75',
]


def iteration_losses(nb, iteration):
    """{shot id: functional value} of block 1, the given iteration (1 or 2) of the tutorial's log."""
    log = ''
    for cell in nb['cells']:
        for out in cell.get('outputs', []):
            if 'text' in out:
                log += ''.join(out['text'])
    start = log.index('Starting iteration %d (out of 4), block 1 (out of 2)' % iteration)
    end = log.index('Starting iteration %d (out of 4), block 1 (out of 2)' % (iteration + 1))
    found = re.findall(r'Functional value for shot (\d+): loss ([0-9.eE+-]+) for shot (\d+)', log[start:end])
    assert all(a == c for a, _, c in found)
    return {int(a): float(b) for a, b, _ in found}


def main():
    with open(NOTEBOOK) as fh:
        nb = json.load(fh)
    code = '\n'.join(''.join(c['source']) for c in nb['cells'] if c['cell_type'] == 'code')
    for line in SETUP:
        assert line in code, line
    losses = iteration_losses(nb, 1)
    losses2 = iteration_losses(nb, 2)
    assert len(losses) == 15 and len(losses2) == 15
    desc = h5.HDF5(make_h5_golden.FIXTURE, mode='r').load(lazy=False)
    vp = np.ascontiguousarray(desc['data'], np.float32)
    with open(os.path.join(HERE, 'anastasio2d_truemodel.json')) as fh:
        assert hashlib.sha256(vp.tobytes()).hexdigest() == json.load(fh)['data']['sha256']
    ids = np.array(sorted(losses), np.int64)
    ids2 = np.array(sorted(losses2), np.int64)
    np.savez_compressed(OUT, vp_true=vp, shot_ids=ids, losses=np.array([losses[i] for i in ids]),
                        shot_ids2=ids2, losses2=np.array([losses2[i] for i in ids2]), step_size=10.,
                        clip=np.array([1400., 1700.]),
                        shape=np.array([356, 385]), extra=np.array([50, 50]), absorbing=np.array([40, 40]),
                        spacing=0.5e-3, dt=0.08e-6, nt=2500, num_locations=120, f_centre=0.5e6, n_cycles=3,
                        f_max=0.3e6, relaxation=0.75)
    print('wrote', OUT, dict(zip(ids.tolist(), [losses[i] for i in ids])))


if __name__ == '__main__':
    main()
