"""Host-side problem model used by the drop-in operator when Stride itself is not importable.

These classes mirror the attributes of Stride's problem model that the iso-acoustic problem
type reads (stride/problem/domain.py:9-414, stride/problem/data.py:98-1645,
stride/problem/acquisitions.py:57-290, stride/problem/problem.py:252-294). When Stride is
installed, its own objects are passed to the operator instead and these are not used.
"""

import numpy as np

from . import h5

__all__ = ['Space', 'Time', 'Grid', 'ScalarField', 'Traces', 'Shot', 'SubProblem', 'inv_transform']


def _grid_description(space, time):
    """GriddedSaved.grid_description (stride/problem/base.py:268-314)."""
    d = {}
    if space is not None:
        d['space'] = {'shape': space.shape, 'spacing': space.spacing, 'extra': space.extra,
                      'absorbing': space.absorbing}
    if time is not None:
        d['time'] = {'start': time.start, 'stop': time.stop, 'step': time.step, 'num': time.num}
    return d


def _pad_edge(data, extended_shape):
    """StructuredData.pad_data without smoothing (stride/problem/data.py:513-536): edge padding
    of half the size difference on each side."""
    widths = [(e - s) // 2 for e, s in zip(extended_shape, data.shape)]
    if sum(widths) > 0:
        data = np.pad(data, [(w, w) for w in widths], mode='edge')
    return data


class _Saved:
    """dump / append / load through the mosaic HDF5 layer (stride/problem/base.py:102-249):
    the file name is given (``filename``, ``path``) or formed from ``project_name``, the object's
    name as ``parameter`` and ``version``."""

    def dump(self, *args, **kwargs):
        kwargs['parameter'] = kwargs.get('parameter', self.name)
        desc = _grid_description(*self._grid_parts())
        desc.update(self.__get_desc__())
        with h5.HDF5(*args, **kwargs, mode='w') as f:
            f.dump(desc)

    def append(self, *args, **kwargs):
        kwargs['parameter'] = kwargs.get('parameter', self.name)
        desc = _grid_description(*self._grid_parts())
        desc.update(self.__get_desc__())
        with h5.HDF5(*args, **kwargs, mode='a') as f:
            f.append(desc)

    def load(self, *args, **kwargs):
        kwargs['parameter'] = self.name
        with h5.HDF5(*args, **kwargs, mode='r') as f:
            self.__set_desc__(f.load(lazy=False))


class Space:
    """Spatial grid: inner ``shape`` plus ``extra`` cells per side, of which ``absorbing``
    are sponge (domain.py:9-74)."""

    def __init__(self, shape, spacing, extra=None, absorbing=None):
        if isinstance(spacing, float):
            spacing = (spacing,) * len(shape)
        self.dim = len(shape)
        self.shape = tuple(int(s) for s in shape)
        self.spacing = tuple(float(h) for h in spacing)
        self.extra = tuple(extra or (0,) * self.dim)
        self.absorbing = tuple(absorbing or (0,) * self.dim)
        self.origin = (0.,) * self.dim
        self.pml_origin = tuple(-h * e for h, e in zip(self.spacing, self.extra))
        self.extended_shape = tuple(s + 2 * e for s, e in zip(self.shape, self.extra))
        self.limit = tuple(h * (s - 1) for h, s in zip(self.spacing, self.shape))

    @property
    def inner(self):
        return tuple(slice(e, e + s) for e, s in zip(self.extra, self.shape))


class Time:
    """Time grid (domain.py:264-330)."""

    def __init__(self, start=0., step=None, num=None, stop=None):
        if stop is None:
            stop = start + step * (num - 1)
        elif num is None:
            num = int(np.ceil((stop - start) / step + 1))
            stop = step * (num - 1) + start
        self.start, self.step, self.num, self.stop = start, step, int(num), stop
        self.extended_num = self.num

    @property
    def grid(self):
        return np.linspace(self.start, self.stop, self.num, endpoint=True)


class Grid:
    def __init__(self, space=None, time=None):
        self.space = space
        self.time = time


def inv_transform(x):
    """Slowness transform that Stride attaches to any field named ``vp`` (data.py:32-33)."""
    return 1 / x


class ScalarField(_Saved):
    """Scalar field on the extended grid; ``data`` is the inner view (data.py:98-446).
    ``dump``/``load`` write and read the reference's description (StructuredData and
    ScalarField, data.py:725-780,1163-1187) as HDF5; loading pads the stored inner data to
    the extended grid with edge values."""

    def __init__(self, name, grid, data=None, needs_grad=False, transform=None):
        self.name = name
        self.grid = grid
        space = grid.space
        self.extended_data = np.zeros(space.extended_shape, dtype=np.float32) if data is None \
            else np.asarray(data, dtype=np.float32)
        self.needs_grad = needs_grad
        if transform is None and 'vp' in name.split('_'):
            transform = inv_transform
        self.transform = transform
        self.grad = None
        self.prec = None

    @property
    def data(self):
        return self.extended_data[self.grid.space.inner]

    def fill(self, value):
        self.extended_data.fill(value)

    def _grid_parts(self):
        return self.grid.space, getattr(self.grid, 'time', None)

    def __get_desc__(self):
        space = self.grid.space
        return {'shape': space.shape, 'extended_shape': space.extended_shape,
                'inner': [[str(s.start), str(s.stop), str(s.step)] for s in space.inner],
                'dtype': 'float32', 'data': np.ascontiguousarray(self.data), 'compression': False,
                'step_size': None, 'time_dependent': False, 'slow_time_dependent': False}

    def __set_desc__(self, desc):
        if getattr(desc, 'compression', False):
            raise NotImplementedError('compressed field data')
        data = np.asarray(desc.data, dtype=np.float32)
        if tuple(data.shape) != tuple(self.grid.space.shape):
            raise ValueError('stored field of shape %s on a grid of shape %s' % (data.shape, self.grid.space.shape))
        self.extended_data = np.ascontiguousarray(_pad_edge(data, self.grid.space.extended_shape))

    def alike(self, name=None, data=None, **kwargs):
        out = ScalarField.__new__(ScalarField)
        out.name = name or self.name
        out.grid = self.grid
        out.extended_data = np.asarray(data, dtype=np.float32)
        out.needs_grad = False
        out.transform = self.transform
        out.grad = out.prec = None
        return out


class Traces(_Saved):
    """Time traces [n_points, nt] (data.py:1100-1645). ``dump``/``load`` write and read the
    reference's description (data.py:1631-1641: the structured data plus ``num_transducers``
    and ``transducer_ids``) as HDF5."""

    def __init__(self, name, data, grid=None):
        self.name = name
        self.data = np.asarray(data, dtype=np.float32)
        self.grid = grid
        self.needs_grad = False

    def alike(self, name=None, data=None, **kwargs):
        t = Traces(name or self.name, self.data if data is None else data, self.grid)
        return t

    def _grid_parts(self):
        return None, getattr(self.grid, 'time', None) if self.grid is not None else None

    def __get_desc__(self):
        shape = tuple(self.data.shape)
        return {'shape': shape, 'extended_shape': shape, 'inner': [['None', 'None', 'None']] * len(shape),
                'dtype': 'float32', 'data': np.ascontiguousarray(self.data), 'compression': False,
                'step_size': None, 'time_dependent': True, 'slow_time_dependent': False,
                'num_transducers': shape[0], 'transducer_ids': list(range(shape[0]))}

    def __set_desc__(self, desc):
        if getattr(desc, 'compression', False):
            raise NotImplementedError('compressed trace data')
        self.data = np.ascontiguousarray(np.asarray(desc.data, dtype=np.float32))


class Shot:
    """One shot: source and receiver coordinates in the inner-domain frame, wavelets and
    observed traces (acquisitions.py:57-290)."""

    def __init__(self, id, source_coordinates, receiver_coordinates, wavelets, observed=None, grid=None):
        self.id = id
        self.source_coordinates = np.asarray(source_coordinates, dtype=np.float32).reshape(-1, len(source_coordinates[0]))
        self.receiver_coordinates = np.asarray(receiver_coordinates, dtype=np.float32).reshape(
            -1, len(receiver_coordinates[0]))
        nt = np.asarray(wavelets).shape[-1]
        self.wavelets = wavelets if isinstance(wavelets, Traces) else Traces('wavelets', np.atleast_2d(wavelets), grid)
        self.observed = observed if observed is not None else Traces(
            'observed', np.zeros((len(self.receiver_coordinates), nt), np.float32), grid)

    @property
    def num_points_sources(self):
        return len(self.source_coordinates)

    @property
    def num_points_receivers(self):
        return len(self.receiver_coordinates)


class SubProblem:
    """The per-shot problem handed to the operator (problem.py:252-294)."""

    def __init__(self, shot, space, time, name='problem'):
        self.shot = shot
        self.shot_id = shot.id
        self.space = space
        self.time = time
        self.grid = Grid(space, time)
        self.name = name
