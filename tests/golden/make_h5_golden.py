"""Generates tests/golden/anastasio2d_truemodel.json (run: python tests/golden/make_h5_golden.py).

The reference ships one HDF5 file written by libhdf5 through mosaic's h5py layer: the breast2D
true model (stride_examples/examples/breast2D/data/anastasio2D-TrueModel.h5). This script reads it
with stride_gb300.h5 and first checks what it decodes against values stated independently of the
file: the grid of the reference's own breast2D script (01_script_forward.py:7-24: shape (356, 385),
extra (50, 50), absorbing (40, 40), spacing 0.5 mm, 2500 steps of 0.08 us) and the inner slices
that grid implies. It then records the decoded description with a SHA-256 of the float32 model so
that tests/test_h5.py can check the reader against the file whenever it is available.
"""

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from stride_gb300 import h5  # noqa: E402

# the reference checkout's root: STRIDE_REFERENCE_ROOT, else a `reference` folder beside this repository
REFERENCE_ROOT = os.environ.get('STRIDE_REFERENCE_ROOT',
                                os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))), 'reference'))
FIXTURE = os.path.join(REFERENCE_ROOT, 'stride_examples', 'examples', 'breast2D', 'data', 'anastasio2D-TrueModel.h5')
OUT = os.path.join(HERE, 'anastasio2d_truemodel.json')


def summary(path):
    """The decoded description: metadata as plain values, the model as shape, dtype, SHA-256 and
    range."""
    d = h5.HDF5(path, mode='r').load(lazy=False)
    data = np.ascontiguousarray(d['data'])
    return {
        'keys': sorted(d.keys()),
        'space': {k: [float(v) for v in d['space'][k]] for k in sorted(d['space'])},
        'time': {k: float(d['time'][k]) for k in sorted(d['time'])},
        'shape': [int(v) for v in d['shape']],
        'extended_shape': [int(v) for v in d['extended_shape']],
        'inner': d['inner'],
        'dtype': d['dtype'],
        'time_dependent': bool(d['time_dependent']),
        'data': {'shape': list(data.shape), 'dtype': str(data.dtype),
                 'sha256': hashlib.sha256(data.tobytes()).hexdigest(),
                 'min': float(data.min()), 'max': float(data.max()), 'mean': float(data.astype(np.float64).mean())},
    }


def main():
    s = summary(FIXTURE)
    # the breast2D script's grid (01_script_forward.py:7-24)
    assert s['space']['shape'] == [356, 385] and s['shape'] == [356, 385]
    assert s['space']['extra'] == [50, 50] and s['space']['absorbing'] == [40, 40]
    assert s['space']['spacing'] == [0.5e-3, 0.5e-3]
    assert s['extended_shape'] == [456, 485]
    assert s['inner'] == [['50', '406', 'None'], ['50', '435', 'None']]
    assert s['time']['num'] == 2500 and abs(s['time']['step'] - 0.08e-6) < 1e-18
    assert s['data']['shape'] == [356, 385] and s['data']['dtype'] == 'float32'
    with open(OUT, 'w') as fh:
        json.dump(s, fh, indent=1, sort_keys=True)
    print('wrote', OUT)


if __name__ == '__main__':
    main()
