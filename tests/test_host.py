"""Host-side logic of the drop-in operator (no GPU): option validation with the reference's
error types, scheme selection, source preparation, the L2 loss and the synthetic workloads."""

import numpy as np
import pytest

from oracle import numpy_oracle as O
from stride_gb300 import fft, iso_acoustic, loss, phantoms, problem, wavelets


def _setup(nt=400, n=64):
    space = problem.Space((n, n), 0.5e-3, extra=(20, 20), absorbing=(20, 20))
    time = problem.Time(0., 0.6 * 0.5e-3 / 1650, nt)
    grid = problem.Grid(space, time)
    vp = problem.ScalarField('vp', grid)
    vp.fill(1500.)
    w = wavelets.tone_burst(0.5e6, 3, nt, time.step)
    shot = problem.Shot(0, [[10e-3, 10e-3]], [[20e-3, 20e-3], [25e-3, 5e-3]], w[None], grid=grid)
    sub = problem.SubProblem(shot, space, time)
    pde = iso_acoustic.IsoAcousticGB300(space=space, time=time)
    return pde, shot, sub, vp, grid


def test_kernel_selection_matches_reference_rule():
    pde, shot, sub, vp, grid = _setup()
    pde._check_problem(shot.wavelets, vp, problem=sub)
    assert pde.kernel == 'OT4' and pde.undersampling_factor == 4
    pde._check_problem(shot.wavelets, vp, problem=sub, kernel='OT2', save_undersampling=6)
    assert pde.kernel == 'OT2' and pde.undersampling_factor == 6


@pytest.mark.parametrize('kw,exc', [
    (dict(boundary_type='nonsense'), ValueError),
    (dict(boundary_type='complex_frequency_shift_PML_2'), NotImplementedError),
    (dict(interpolation_type='cubic'), ValueError),
    (dict(kernel='OT6'), ValueError),
    (dict(checkpoint_interval=-4), ValueError),
    (dict(checkpoint_interval=2.5), ValueError),
    (dict(checkpoint_budget=-1.0), ValueError),
])
def test_option_errors(kw, exc):
    pde, shot, sub, vp, grid = _setup()
    with pytest.raises(exc):
        pde._check_problem(shot.wavelets, vp, problem=sub, **kw)


def test_sinc_interpolation_is_accepted():
    """interpolation_type='sinc' (common/devito.py:634-638) is accepted and kept."""
    pde, shot, sub, vp, grid = _setup()
    pde._check_problem(shot.wavelets, vp, problem=sub, interpolation_type='sinc')
    assert pde.interpolation_type == 'sinc'


def test_cfs_pml_runs_with_ot2_in_2d():
    """The CFS-PML is accepted with OT2 (the reference example's combination) and refused with OT4."""
    pde, shot, sub, vp, grid = _setup()
    pde._check_problem(shot.wavelets, vp, problem=sub, boundary_type='complex_frequency_shift_PML_2', kernel='OT2')
    assert pde.boundary_type == 'complex_frequency_shift_PML_2' and pde.kernel == 'OT2'
    with pytest.raises(NotImplementedError):
        pde._check_problem(shot.wavelets, vp, problem=sub, boundary_type='complex_frequency_shift_PML_2',
                           kernel='OT4')


def test_saved_wavefield_choice():
    """Snapshots for the vp gradient, checkpoints when an interval or budget is given, the raw
    wavefield whenever rho or the wavelets need a gradient (devito.py:319,410-413)."""
    pde, shot, sub, vp, grid = _setup()
    rho = problem.ScalarField('rho', grid, needs_grad=True)
    pde._check_problem(shot.wavelets, vp, problem=sub)
    assert pde._save_wavefield(vp, None, None, {}) is False
    vp.needs_grad = True
    assert pde._save_wavefield(vp, None, None, {}) == 'snapshots'
    assert pde._save_wavefield(vp, rho, None, {}) == 'raw'
    pde._check_problem(shot.wavelets, vp, problem=sub, checkpoint_interval=40)
    assert pde.checkpoint_interval == 40
    assert pde._save_wavefield(vp, None, None, {}) == 'checkpoints'
    assert pde._save_wavefield(vp, rho, None, {}) == 'raw'
    pde._check_problem(shot.wavelets, vp, problem=sub, checkpoint_budget=1e9)
    assert pde.checkpoint_interval == 0 and pde._save_wavefield(vp, None, None, {}) == 'checkpoints'
    pde._check_problem(shot.wavelets, vp, problem=sub)
    assert pde._save_wavefield(vp, None, None, {}) == 'snapshots'


def test_perf_lines(caplog):
    """The reference's per-shot 'perf' lines (devito.py:406,1289,1347,1382,1458) and the run times,
    with the forward and adjoint driven through a stub plan (no GPU)."""
    pde, shot, sub, vp, grid = _setup()
    vp.needs_grad = True

    class StubPlan:
        n_src = 1
        save = adj = None

        def forward(self, src, traces, save=False):
            self.save = save

        def adjoint(self, res, grad, prec, **kw):
            self.adj = True

    with caplog.at_level(iso_acoustic.PERF, logger='stride_gb300'):
        pde._check_problem(shot.wavelets, vp, problem=sub)
        pde._plan = StubPlan()
        pde._src = np.zeros((1, 400), np.float32)
        pde._traces = np.zeros((2, 400), np.float32)
        pde.run_forward(shot.wavelets, vp, problem=sub)
        pde._res = np.zeros((2, 400), np.float32)
        pde.run_adjoint(shot.observed.alike(name='residual', data=np.ones((2, 400), np.float32)), shot.wavelets, vp,
                        problem=sub)
    for m in ('(ShotID 0) Selected boundary type sponge_boundary_2', 'Estimated bandwidth for the propagated wavelet',
              'Selected time stepping scheme OT4', 'Selected undersampling level 4', 'Expected wavefield size',
              'Forward ran in', 'Adjoint ran in'):
        assert m in caplog.text
    assert pde._plan.save == 'snapshots' and pde._plan.adj


def test_attenuation_power_errors():
    pde, shot, sub, vp, grid = _setup()
    alpha = problem.ScalarField('alpha', grid)
    with pytest.raises(ValueError):
        pde._check_problem(shot.wavelets, vp, alpha=alpha, problem=sub, attenuation_power=3)
    with pytest.raises(NotImplementedError):
        pde._check_problem(shot.wavelets, vp, alpha=alpha, problem=sub, attenuation_power=2)


def test_drp_warns_and_is_ignored(caplog):
    pde, shot, sub, vp, grid = _setup()
    pde._check_problem(shot.wavelets, vp, problem=sub, drp=True)
    assert pde.drp is False


def test_host_helpers_match_oracle():
    dt = 1e-7
    np.testing.assert_array_equal(wavelets.tone_burst(1e6, 3, 500, dt), O.tone_burst(1e6, 3, 500, dt))
    w = O.tone_burst(1e6, 3, 500, dt)
    assert fft.bandwidth(w, dt) == O.bandwidth(w, dt)


def test_source_window_and_diff_source():
    pde, shot, sub, vp, grid = _setup()
    src = pde._source_data(shot.wavelets, diff_source=False)
    np.testing.assert_allclose(src[0], (shot.wavelets.data[0] * O.tukey(pde.time.num)).astype(np.float32))
    d = pde._source_data(shot.wavelets, diff_source=True)
    ref = np.gradient(shot.wavelets.data[0].astype(np.float64), pde.time.step) * pde.time.step * O.tukey(pde.time.num)
    np.testing.assert_allclose(d[0], ref.astype(np.float32), rtol=1e-6, atol=1e-9)


def test_grad_chain_rule_slowness_and_vp():
    pde, shot, sub, vp, grid = _setup()
    ext = pde.space.extended_shape
    pde._grad = np.ones(ext, np.float32)
    pde._prec = np.ones(ext, np.float32)
    g = pde.get_grad_vp(vp)
    np.testing.assert_allclose(g.extended_data, 1 / 1500., rtol=1e-6)
    np.testing.assert_allclose(g.prec.extended_data, (1 / 1500.) ** 2, rtol=1e-6)
    vp.transform = None
    g = pde.get_grad_vp(vp)
    np.testing.assert_allclose(g.extended_data, -2 / 1500. ** 3, rtol=1e-6)


def test_l2_loss():
    L = loss.L2DistanceLoss()
    m = np.array([[1., 2.], [3., 4.]], np.float32)
    o = np.array([[0., 2.], [1., 4.]], np.float32)
    assert L(m, o) == pytest.approx(0.5 * (1 + 4))
    gm, go = L.adjoint(1.0)
    np.testing.assert_array_equal(gm, m - o)
    np.testing.assert_array_equal(go, o - m)


def test_workloads_are_seeded_and_shaped():
    a = phantoms.workload('batched', seed=3, nt=100, n_shots=8)
    b = phantoms.workload('batched', seed=3, nt=100, n_shots=8)
    np.testing.assert_array_equal(a['vp'], b['vp'])
    np.testing.assert_array_equal(a['rho'], b['rho'])
    assert a['shape'] == (552, 552) and len(a['src']) == 8
    assert 1400 <= a['vp'].min() and a['vp'].max() <= 1650
    assert 950 <= a['rho'].min() and a['rho'].max() <= 1100
    assert 0 <= a['alpha'].min() and a['alpha'].max() <= 1
    s = phantoms.workload('single', nt=100)
    assert s['shape'] == (296, 296) and s['rho'] is None
    r = np.linalg.norm(s['geometry'] - np.array([(255 * 0.5e-3) / 2] * 2), axis=1)
    np.testing.assert_allclose(r, 55e-3, rtol=1e-5)
