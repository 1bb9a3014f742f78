"""The drop-in problem type (IsoAcousticGB300) end to end on the GPU: the reference's
pde(wavelets, vp, rho=, alpha=, problem=) call through forward/adjoint hooks, checked against
the oracle (traces relative L2 <= 1e-4, gradient cosine >= 0.999)."""

import numpy as np
import pytest

from oracle import c_oracle
from oracle import numpy_oracle as O
from stride_gb300 import iso_acoustic, phantoms, problem, wavelets
from tests import _cases as C

pytestmark = pytest.mark.gpu


def _setup(density=True, alpha=True, nt=300, n=60, cfl=0.6):
    rng = np.random.default_rng(5)
    h = 0.5e-3
    space = problem.Space((n, n + 4), h, extra=(12, 12), absorbing=(12, 12))
    time = problem.Time(0., cfl * h / 1650, nt)
    grid = problem.Grid(space, time)
    vpi, rhoi, ali = phantoms.ellipse_phantom(space.shape, space.spacing, 3, rng, rho_range=(950., 1100.),
                                              alpha_range=(0., 1.), disk_radius=8e-3, axes=(2e-3, 6e-3))
    vp = problem.ScalarField('vp', grid, data=phantoms.extend(vpi, space.extra), needs_grad=True)
    rho = problem.ScalarField('rho', grid, data=phantoms.extend(rhoi, space.extra)) if density else None
    al = problem.ScalarField('alpha', grid, data=phantoms.extend(ali, space.extra)) if alpha else None
    c = ((n - 1) * h / 2, (n + 3) * h / 2)
    geo = phantoms.circle_geometry(16, 11e-3, c)
    w = wavelets.tone_burst(1e6, 3, nt, time.step)
    shot = problem.Shot(0, geo[:1], geo, w[None], grid=grid)
    sub = problem.SubProblem(shot, space, time)
    return space, time, vp, rho, al, shot, sub, geo, w


@pytest.mark.parametrize('density,alpha', [(False, False), (True, True)])
def test_pde_forward_and_gradient(density, alpha):
    space, time, vp, rho, al, shot, sub, geo, w = _setup(density, alpha)
    pde = iso_acoustic.IsoAcousticGB300(space=space, time=time)
    traces = pde(shot.wavelets, vp, rho=rho, alpha=al, problem=sub)
    assert traces.name == 'modelled'
    origin = space.pml_origin
    kw = dict(rho=None if rho is None else rho.extended_data, alpha=None if al is None else al.extended_data)
    ref, snaps = c_oracle.forward(vp.extended_data, space.spacing, time.step, time.num, space.absorbing, geo[:1],
                                  geo, w[None], origin, kernel='OT4', save=True, **kw)
    assert C.rel_l2(traces.data, ref) <= 1e-4
    residual = shot.observed.alike(name='residual', data=traces.data * np.float32(0.7))
    grads = pde.adjoint(residual, shot.wavelets, vp, rho, al, problem=sub)
    g_vp = grads[1]
    g_ref, p_ref = c_oracle.adjoint(vp.extended_data, space.spacing, time.step, time.num, space.absorbing, geo,
                                    traces.data * np.float32(0.7), origin, snaps, kernel='OT4', **kw)
    g_ref, p_ref = O.grad_vp_chain(g_ref[space.inner], p_ref[space.inner], vp.data, slowness=True)
    assert g_vp.extended_data.shape == space.shape
    assert C.cosine(g_vp.extended_data, g_ref) >= 0.999
    assert C.rel_l2(g_vp.prec.extended_data, p_ref) <= 1e-4


def test_batched_forward_matches_per_shot():
    space, time, vp, rho, al, shot, sub, geo, w = _setup(True, True)
    pde = iso_acoustic.IsoAcousticGB300(space=space, time=time)
    shots = [problem.Shot(k, geo[[k, (k + 5) % 16]][: 1 + k % 2], geo[: 16 - k], w[None].repeat(1 + k % 2, 0), grid=shot.wavelets.grid)
             for k in range(5)]
    out = pde.forward_batch(shots, vp, rho=rho, alpha=al)
    for k, s in enumerate(shots):
        ref, _ = c_oracle.forward(vp.extended_data, space.spacing, time.step, time.num, space.absorbing,
                                  s.source_coordinates, s.receiver_coordinates, s.wavelets.data, space.pml_origin,
                                  rho=rho.extended_data, alpha=al.extended_data, kernel='OT4')
        assert C.rel_l2(out[k], ref) <= 1e-4, k


def test_empty_wavelets_skip_the_run():
    space, time, vp, rho, al, shot, sub, geo, w = _setup(False, False)
    pde = iso_acoustic.IsoAcousticGB300(space=space, time=time)
    shot.wavelets.data[:] = 0
    traces = pde(shot.wavelets, vp, problem=sub)
    assert not np.any(traces.data)


def test_pde_wavelet_gradient():
    """wavelets.needs_grad: the adjoint returns (wavelets_grad, vp_grad, None, None) with the
    reference's -interp(p_a) at the sources."""
    space, time, vp, rho, al, shot, sub, geo, w = _setup(True, True)
    pde = iso_acoustic.IsoAcousticGB300(space=space, time=time)
    shot.wavelets.needs_grad = True
    traces = pde(shot.wavelets, vp, rho=rho, alpha=al, problem=sub)
    residual = shot.observed.alike(name='residual', data=traces.data * np.float32(0.7))
    grads = pde.adjoint(residual, shot.wavelets, vp, rho, al, problem=sub)
    assert grads[0] is not None and grads[0].name == 'wavelets_grad' and grads[1] is not None
    kw = dict(rho=rho.extended_data, alpha=al.extended_data)
    _, snaps = c_oracle.forward(vp.extended_data, space.spacing, time.step, time.num, space.absorbing, geo[:1], geo,
                                w[None], space.pml_origin, kernel='OT4', save=True, **kw)
    _, _, gw = O.adjoint(vp.extended_data, space.spacing, time.step, time.num, space.absorbing, geo,
                         traces.data * np.float32(0.7), space.pml_origin, snaps, kernel='OT4', src_coords=geo[:1], **kw)
    assert C.rel_l2(grads[0].data, gw) <= 1e-4
    # with the wavelets needing a gradient the reference saves the raw wavefield, and so does the
    # drop-in: its vp gradient follows the raw-wavefield path
    _, raw = O.forward(vp.extended_data, space.spacing, time.step, time.num, space.absorbing, geo[:1], geo, w[None],
                       space.pml_origin, kernel='OT4', save='raw', **kw)
    g_ref, _ = O.adjoint(vp.extended_data, space.spacing, time.step, time.num, space.absorbing, geo,
                         traces.data * np.float32(0.7), space.pml_origin, raw, kernel='OT4', raw=True, **kw)
    g_ref, _ = O.grad_vp_chain(g_ref[space.inner], g_ref[space.inner], vp.data, slowness=True)
    assert C.cosine(grads[1].extended_data, g_ref) >= 0.999


def test_pde_rho_gradient():
    """rho.needs_grad (positional rho, as the reference's adjoint graph needs): the adjoint returns
    (None, vp_grad, rho_grad, None); rho_grad is the raw imaging term on the inner grid."""
    space, time, vp, rho, al, shot, sub, geo, w = _setup(True, True)
    rho.needs_grad = True
    pde = iso_acoustic.IsoAcousticGB300(space=space, time=time)
    traces = pde(shot.wavelets, vp, rho, al, problem=sub)
    residual = shot.observed.alike(name='residual', data=traces.data * np.float32(0.7))
    grads = pde.adjoint(residual, shot.wavelets, vp, rho, al, problem=sub)
    assert grads[0] is None and grads[3] is None
    assert grads[2].name == 'rho_grad' and grads[2].prec.name == 'rho_prec'
    kw = dict(rho=rho.extended_data, alpha=al.extended_data)
    _, raw = O.forward(vp.extended_data, space.spacing, time.step, time.num, space.absorbing, geo[:1], geo, w[None],
                       space.pml_origin, kernel='OT4', save='raw', **kw)
    g, _, g_rho, p_rho = O.adjoint(vp.extended_data, space.spacing, time.step, time.num, space.absorbing, geo,
                                   traces.data * np.float32(0.7), space.pml_origin, raw, kernel='OT4', raw=True,
                                   rho_grad=True, **kw)
    assert C.cosine(grads[2].extended_data, g_rho[space.inner]) >= 0.999
    assert C.rel_l2(grads[2].prec.extended_data, p_rho[space.inner]) <= 1e-3
    g_ref, _ = O.grad_vp_chain(g[space.inner], g[space.inner], vp.data, slowness=True)
    assert C.cosine(grads[1].extended_data, g_ref) >= 0.999


def test_pde_alpha_gradient_is_not_implemented():
    """The reference has no alpha gradient: its prepare_grad raises ValueError."""
    space, time, vp, rho, al, shot, sub, geo, w = _setup(True, True)
    al.needs_grad = True
    pde = iso_acoustic.IsoAcousticGB300(space=space, time=time)
    traces = pde(shot.wavelets, vp, rho, al, problem=sub)
    residual = shot.observed.alike(name='residual', data=traces.data)
    with pytest.raises(ValueError, match='alpha not implemented'):
        pde.adjoint(residual, shot.wavelets, vp, rho, al, problem=sub)


def test_pde_cfs_pml():
    """boundary_type='complex_frequency_shift_PML_2' with kernel OT2: traces against the oracle's
    CFS-PML with the band centre the drop-in estimated (IsoAcousticDevito._bandwidth[1])."""
    space, time, vp, rho, al, shot, sub, geo, w = _setup(True, True, cfl=0.4)
    pde = iso_acoustic.IsoAcousticGB300(space=space, time=time)
    traces = pde(shot.wavelets, vp, rho=rho, alpha=al, problem=sub, boundary_type='complex_frequency_shift_PML_2',
                 kernel='OT2')
    ref, _ = O.forward(vp.extended_data, space.spacing, time.step, time.num, space.absorbing, geo[:1], geo, w[None],
                       space.pml_origin, rho=rho.extended_data, alpha=al.extended_data, kernel='OT2',
                       boundary='pml', f_centre=pde._bandwidth[1])
    assert np.abs(ref).max() > 0
    assert C.rel_l2(traces.data, ref) <= 1e-4


def test_pde_checkpointed_gradient_is_bitwise_equal():
    """checkpoint_interval / checkpoint_budget: the adjoint recomputes segments from checkpoints
    and returns the snapshot path's vp gradient bit for bit."""
    space, time, vp, rho, al, shot, sub, geo, w = _setup(True, True)
    out = []
    for kw in (dict(), dict(checkpoint_interval=24), dict(checkpoint_budget=2e9)):
        pde = iso_acoustic.IsoAcousticGB300(space=space, time=time)
        traces = pde(shot.wavelets, vp, rho=rho, alpha=al, problem=sub, **kw)
        assert pde._saved == ('checkpoints' if kw else 'snapshots')
        residual = shot.observed.alike(name='residual', data=traces.data * np.float32(0.7))
        g = pde.adjoint(residual, shot.wavelets, vp, rho, al, problem=sub, **kw)[1]
        out.append((traces.data.copy(), g.extended_data.copy(), g.prec.extended_data.copy()))
    assert np.abs(out[0][1]).max() > 0
    for o in out[1:]:
        for a, b in zip(out[0], o):
            assert np.array_equal(a, b)


def test_pde_3d_forward_and_gradient():
    """The drop-in on a 3D problem: pde(...) traces and the adjoint's vp gradient against the C
    oracle (3D extended grid, variable density and attenuation)."""
    rng = np.random.default_rng(9)
    h = 0.5e-3
    n = 24
    space = problem.Space((n, n + 2, n + 4), h, extra=(8, 8, 8), absorbing=(8, 8, 8))
    time = problem.Time(0., 0.6 * h / 1650, 140)
    grid = problem.Grid(space, time)
    vpi, rhoi, ali = phantoms.ellipse_phantom(space.shape, space.spacing, 3, rng, rho_range=(950., 1100.),
                                              alpha_range=(0., 1.), disk_radius=3e-3, axes=(1.5e-3, 4e-3))
    vp = problem.ScalarField('vp', grid, data=phantoms.extend(vpi, space.extra), needs_grad=True)
    rho = problem.ScalarField('rho', grid, data=phantoms.extend(rhoi, space.extra))
    al = problem.ScalarField('alpha', grid, data=phantoms.extend(ali, space.extra))
    c = np.array([(s - 1) * h / 2 for s in space.shape])
    geo = c + 4e-3 * np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [-1, 0, 0], [0, -1, 0.3], [0.5, 0.5, -0.6]])
    w = wavelets.tone_burst(1e6, 3, time.num, time.step)
    shot = problem.Shot(0, geo[:1], geo, w[None], grid=grid)
    sub = problem.SubProblem(shot, space, time)
    pde = iso_acoustic.IsoAcousticGB300(space=space, time=time)
    traces = pde(shot.wavelets, vp, rho=rho, alpha=al, problem=sub)
    kw = dict(rho=rho.extended_data, alpha=al.extended_data)
    ref, snaps = c_oracle.forward(vp.extended_data, space.spacing, time.step, time.num, space.absorbing, geo[:1], geo,
                                  w[None], space.pml_origin, kernel=pde.kernel, save=True,
                                  undersampling=pde.undersampling_factor, **kw)
    assert np.abs(ref).max() > 0
    assert C.rel_l2(traces.data, ref) <= 1e-4
    residual = shot.observed.alike(name='residual', data=traces.data * np.float32(0.7))
    grads = pde.adjoint(residual, shot.wavelets, vp, rho, al, problem=sub)
    g_ref, _ = c_oracle.adjoint(vp.extended_data, space.spacing, time.step, time.num, space.absorbing, geo,
                                traces.data * np.float32(0.7), space.pml_origin, snaps, kernel=pde.kernel,
                                undersampling=pde.undersampling_factor, **kw)
    g_ref, _ = O.grad_vp_chain(g_ref[space.inner], g_ref[space.inner], vp.data, slowness=True)
    assert grads[1].extended_data.shape == space.shape
    assert C.cosine(grads[1].extended_data, g_ref) >= 0.999
