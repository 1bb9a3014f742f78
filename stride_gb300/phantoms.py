"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The reference quotes no public dataset for this path. Its examples build water tanks with
ellipse-shaped inclusions and transducers on a circle (stride/utils/geometries.py:115-214,
stride/problem/geometry.py:239-288), driven by a Gaussian tone burst
(stride/utils/wavelets.py:6-53). These helpers generate the same kind of inputs from a
numpy seed, so every run and test sees identical data:

* ``ellipse_phantom``: water (vp 1500 m/s, rho 1000 kg/m^3, alpha 0) with ellipses (2D)
  or ellipsoids (3D) whose centres are uniform in a 40 mm disk/ball about the grid centre,
  semi-axes U[5, 20] mm, random orientation; later inclusions overwrite earlier ones.
* ``circle_geometry`` / ``hemisphere_geometry``: transducer positions on a 55 mm circle or
  hemisphere about the centre, optionally jittered by U[-j, j] grid cells per coordinate.
* ``workload``: the 2D configurations (single shot 256^2 at 0.5 mm, batched 512^2 at
  0.25 mm), extended by 20 absorbing cells per side, dt at CFL 0.6 of 1650 m/s.
"""

import numpy as np

from . import wavelets as _wavelets


def ellipse_phantom(shape, spacing, n, rng, vp_range=(1400., 1650.), rho_range=None, alpha_range=None,
                    disk_radius=40e-3, axes=(5e-3, 20e-3)):
    """Returns inner-grid (vp, rho, alpha) float32 arrays (rho/alpha None when no range)."""
    dim = len(shape)
    coords = np.meshgrid(*[np.arange(s) * h for s, h in zip(shape, spacing)], indexing='ij')
    centre = np.array([(s - 1) * h / 2 for s, h in zip(shape, spacing)])
    vp = np.full(shape, 1500., dtype=np.float64)
    rho = np.full(shape, 1000., dtype=np.float64) if rho_range is not None else None
    alpha = np.zeros(shape, dtype=np.float64) if alpha_range is not None else None
    for _ in range(n):
        # centre uniform in the disk/ball
        while True:
            off = rng.uniform(-disk_radius, disk_radius, size=dim)
            if np.linalg.norm(off) <= disk_radius:
                break
        c = centre + off
        semi = rng.uniform(axes[0], axes[1], size=dim)
        if dim == 2:
            th = rng.uniform(0, np.pi)
            rot = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
        else:
            q = rng.standard_normal((3, 3))
            rot, _ = np.linalg.qr(q)
        rel = np.stack([x - ci for x, ci in zip(coords, c)], axis=-1) @ rot
        mask = np.sum((rel / semi) ** 2, axis=-1) <= 1.0
        vp[mask] = rng.uniform(*vp_range)
        if rho is not None:
            rho[mask] = rng.uniform(*rho_range)
        if alpha is not None:
            alpha[mask] = rng.uniform(*alpha_range)
    f32 = lambda a: None if a is None else a.astype(np.float32)
    return f32(vp), f32(rho), f32(alpha)


def extend(inner, extra):
    """Pads an inner-grid array to the extended grid with edge values."""
    return np.pad(inner, [(e, e) for e in extra], mode='edge').astype(np.float32)


def circle_geometry(num, radius, centre, jitter=0.0, spacing=None, rng=None):
    """Points on a circle, angles linspace(0, 2 pi, num, endpoint=False)
    (stride/utils/geometries.py:115-142), plus an optional uniform jitter in cells."""
    ang = np.linspace(0, 2 * np.pi, num, endpoint=False)
    g = np.stack([radius * np.cos(ang) + centre[0], radius * np.sin(ang) + centre[1]], axis=1)
    if jitter:
        g = g + rng.uniform(-jitter, jitter, size=g.shape) * np.asarray(spacing)[None, :]
    return g


def hemisphere_geometry(num, radius, centre):
    """Fibonacci points on a hemisphere (stride/utils/geometries.py:145-214 with
    threshold 0.5, no rotation)."""
    increment = np.pi * (3. - np.sqrt(5.))
    threshold = 0.5
    total = int(np.round(num / (1 - threshold)))
    offset = 2. / total
    pts = []
    for sample in range(total):
        z = ((sample * offset) - 1) + offset / 2
        r = np.sqrt(1 - z ** 2)
        phi = ((sample + 1) % total) * increment
        if z + 1 < threshold * 2:
            continue
        pts.append([np.sin(phi) * r * radius + centre[0], np.cos(phi) * r * radius + centre[1],
                    z * radius + centre[2]])
    return np.asarray(pts[:num])


def workload(name, seed=0, nt=None, n_shots=None, inner=None, cfl=0.6):
    """Synthetic 2D workload.

    name: 'single' (256^2 at 0.5 mm, vp only, 128 transducers, 500 kHz, shot 0, 2000 steps)
          or 'batched' (512^2 at 0.25 mm, vp/rho/alpha, 256 jittered transducers, 1 MHz,
          one shot per transducer, 4000 steps).
    ``nt``, ``n_shots`` and ``inner`` override the size for reduced test cases; ``cfl`` sets
    dt = cfl h / 1650 m/s (0.6 for OT4, 0.4 within the OT2 limit).
    Returns a dict with extended-grid materials, geometry per shot and wavelets.
    """
    rng = np.random.default_rng(seed)
    extra = 20
    if name == 'single':
        n, h, f0, ntr, steps, ne = 256, 0.5e-3, 0.5e6, 128, 2000, 6
        vpi, rhoi, ali = None, None, None
    elif name == 'batched':
        n, h, f0, ntr, steps, ne = 512, 0.25e-3, 1.0e6, 256, 4000, 6
    else:
        raise ValueError(name)
    if inner is not None:
        n = inner
    shape = (n, n)
    spacing = (h, h)
    if name == 'single':
        vpi, _, _ = ellipse_phantom(shape, spacing, ne, rng)
    else:
        vpi, rhoi, ali = ellipse_phantom(shape, spacing, ne, rng, rho_range=(950., 1100.), alpha_range=(0., 1.))
    centre = ((n - 1) * h / 2, (n - 1) * h / 2)
    radius = min(55e-3, 0.45 * (n - 1) * h)  # 55 mm, or less on reduced test grids
    geo = circle_geometry(ntr, radius, centre, jitter=0.5 if name == 'batched' else 0.0, spacing=spacing, rng=rng)
    dt = cfl * h / 1650.
    nt = steps if nt is None else nt
    n_tone = int((3 / f0) // dt + 1)
    wav = _wavelets.tone_burst(f0, 3, max(nt, n_tone), dt)[:nt]
    if name == 'single':
        shots = [0] if n_shots is None else list(range(n_shots))
    else:
        shots = list(range(ntr)) if n_shots is None else list(range(0, ntr, max(1, ntr // n_shots)))[:n_shots]
    ext = (extra, extra)
    return dict(
        name=name, shape=tuple(s + 2 * extra for s in shape), inner_shape=shape, spacing=spacing,
        extra=ext, absorbing=ext, dt=dt, nt=nt, f0=f0,
        vp=extend(vpi, ext), rho=None if rhoi is None else extend(rhoi, ext),
        alpha=None if ali is None else extend(ali, ext),
        vp_inner=vpi, geometry=geo.astype(np.float32), shots=shots,
        src=[geo[[s]] for s in shots], rec=[geo for _ in shots], wavelet=wav,
    )


def workload3d(seed=0, nt=None, n_shots=8, inner=None):
    """Synthetic 3D workload: 256^3 inner grid at 0.5 mm + 20 absorbing cells per side
    (296^3 extended), seeded vp/rho/alpha ellipsoid phantom in water, 512 transducers on a
    55 mm hemisphere, 500 kHz 3-cycle burst, 3000 steps at CFL 0.6; ``n_shots`` shots fire
    from evenly spaced transducers."""
    rng = np.random.default_rng(seed)
    extra = 20
    n = 256 if inner is None else inner
    h = 0.5e-3
    shape = (n, n, n)
    spacing = (h, h, h)
    vpi, rhoi, ali = ellipse_phantom(shape, spacing, 6, rng, rho_range=(950., 1100.), alpha_range=(0., 1.),
                                     disk_radius=min(40e-3, 0.3 * (n - 1) * h), axes=(min(5e-3, 0.05 * n * h),
                                                                                      min(20e-3, 0.15 * n * h)))
    centre = tuple((n - 1) * h / 2 for _ in range(3))
    radius = min(55e-3, 0.42 * (n - 1) * h)
    geo = hemisphere_geometry(512, radius, centre)
    dt = 0.6 * h / 1650.
    nt = 3000 if nt is None else nt
    n_tone = int((3 / 0.5e6) // dt + 1)
    wav = _wavelets.tone_burst(0.5e6, 3, max(nt, n_tone), dt)[:nt]
    shots = list(range(0, len(geo), max(1, len(geo) // n_shots)))[:n_shots]
    ext = (extra,) * 3
    return dict(
        name='3d', shape=tuple(s + 2 * extra for s in shape), inner_shape=shape, spacing=spacing, extra=ext,
        absorbing=ext, dt=dt, nt=nt, f0=0.5e6, vp=extend(vpi, ext), rho=extend(rhoi, ext), alpha=extend(ali, ext),
        vp_inner=vpi, geometry=geo.astype(np.float32), shots=shots, src=[geo[[s]] for s in shots],
        rec=[geo for _ in shots], wavelet=wav,
    )
