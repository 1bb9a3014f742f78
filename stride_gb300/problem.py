"""Host-side problem model used by the drop-in operator when Stride itself is not importable.

These classes mirror the attributes of Stride's problem model that the iso-acoustic problem
type reads (stride/problem/domain.py:9-414, stride/problem/data.py:98-1645,
stride/problem/acquisitions.py:57-290, stride/problem/problem.py:252-294). When Stride is
installed, its own objects are passed to the operator instead and these are not used.
"""

import numpy as np

__all__ = ['Space', 'Time', 'Grid', 'ScalarField', 'Traces', 'Shot', 'SubProblem', 'inv_transform']


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


class ScalarField:
    """Scalar field on the extended grid; ``data`` is the inner view (data.py:98-446)."""

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

    def alike(self, name=None, data=None, **kwargs):
        out = ScalarField.__new__(ScalarField)
        out.name = name or self.name
        out.grid = self.grid
        out.extended_data = np.asarray(data, dtype=np.float32)
        out.needs_grad = False
        out.transform = self.transform
        out.grad = out.prec = None
        return out


class Traces:
    """Time traces [n_points, nt] (data.py:1100-1645)."""

    def __init__(self, name, data, grid=None):
        self.name = name
        self.data = np.asarray(data, dtype=np.float32)
        self.grid = grid
        self.needs_grad = False

    def alike(self, name=None, data=None, **kwargs):
        t = Traces(name or self.name, self.data if data is None else data, self.grid)
        return t


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
