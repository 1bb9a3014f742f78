"""The oracle (CPU restatements) against known answers, golden fixtures and each other.

No GPU. Devito is not vendored and cannot be installed here; besides the losses the reference's
imaging tutorial recorded from Devito (tests/test_pin_tutorial.py), these checks pin the
restatement to the reference's own analytic check, to fixtures, to the independent C
restatement and to properties of the scheme (self-convergence, the FP32 noise floor, adjoint
identities).
"""

import os

import numpy as np
import pytest

from oracle import c_oracle
from oracle import numpy_oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def _corr(a, b):
    return float(np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b)))


@pytest.fixture(scope='module')
def homogeneous_2d():
    g = np.load(os.path.join(GOLD, 'analytic_2d.npz'))
    n, extra, h, dt, nt = int(g['n']), int(g['extra']), float(g['h']), float(g['dt']), int(g['nt'])
    shape = (n + 2 * extra,) * 2
    vp = np.full(shape, 1500., np.float32)
    tr, _ = c_oracle.forward(vp, (h, h), dt, nt, (extra, extra), g['geometry'][:1], g['geometry'],
                             g['wavelet'][None], (-extra * h, -extra * h), kernel='OT4', diff_source=True)
    return g, tr


def test_analytic_2d_reference_formula(homogeneous_2d):
    """The reference example's metric (forward_2D.py:92-124): normalised traces against its
    analytic formula; the reference prints this error without a threshold."""
    g, tr = homogeneous_2d
    an = g['reference_formula'] / np.max(np.abs(g['reference_formula']))
    t = tr / np.max(np.abs(tr))
    err = np.sqrt(np.sum((t - an) ** 2) / an.shape[0])
    assert err < 0.3


def test_analytic_2d_exact_integral(homogeneous_2d):
    """Against the Green's function integrated exactly per sample, away from the source."""
    g, tr = homogeneous_2d
    ex = g['exact_integral']
    for i in (3, 4, 5, 6, 8, 10, 12):
        assert _corr(tr[i], ex[i]) > 0.98, i


def test_analytic_3d():
    g = np.load(os.path.join(GOLD, 'analytic_3d.npz'))
    n, e, h, dt, nt = int(g['n']), int(g['extra']), float(g['h']), float(g['dt']), int(g['nt'])
    vp = np.full((n + 2 * e,) * 3, 1500., np.float32)
    tr, _ = c_oracle.forward(vp, (h, h, h), dt, nt, (e, e, e), g['src'][None], g['recs'], g['wavelet'][None],
                             (-e * h,) * 3, kernel='OT4', diff_source=True)
    for i in range(len(g['recs'])):
        # the analytic delay is rounded to a whole sample (utils.py:48), hence the 0.95 floor
        assert _corr(tr[i], g['analytic'][i]) > 0.95, i


def test_numpy_matches_golden():
    g = np.load(os.path.join(GOLD, 'oracle_small.npz'))
    e = int(g['extra'])
    h = tuple(g['h'])
    origin = (-e * h[0], -e * h[1])
    tr, snaps = O.forward(g['vp'], h, float(g['dt']), int(g['nt']), (e, e), g['src'], g['rec'], g['wavelet'], origin,
                          rho=g['rho'], alpha=g['alpha'], save=True)
    np.testing.assert_array_equal(tr, g['traces'])
    assert np.sum(snaps, dtype=np.float64) == float(g['snap_sum'])
    gg, pp = O.adjoint(g['vp'], h, float(g['dt']), int(g['nt']), (e, e), g['rec'], tr * 0.5, origin, snaps,
                       rho=g['rho'], alpha=g['alpha'])
    np.testing.assert_array_equal(gg, g['grad'])
    np.testing.assert_array_equal(pp, g['prec'])


def _refined_traces(level, kernel):
    """A homogeneous 2D shot (vp 1500) at h = 2 mm / 2^level and dt = 0.4 h / 1500 (fixed CFL),
    over the same physical domain (110 mm inner, a 20 mm sponge) and time window (51 us), in the
    FP64 oracle. The source (a Gaussian derivative, sigma 3 us) and the receivers (20-30 mm away,
    so that nothing returns from the sponge within the window) sit on nodes of the coarsest
    grid; the coordinates are given 1e-3 h below the nodes so that the reference's eps shift
    (iso_acoustic/devito.py:307-309) puts them on the nodes at every level. The injection
    amplitude 2 dt vp / h (:357-363) makes the same continuous source at every level."""
    h = 2e-3 / 2 ** level
    n, ab = 55 * 2 ** level + 1, 10 * 2 ** level
    dt = 0.4 * h / 1500.
    nt = 96 * 2 ** level + 1
    t = np.arange(nt) * dt
    sig = 3e-6
    wav = -(t - 5 * sig) / sig * np.exp(-0.5 * ((t - 5 * sig) / sig) ** 2)
    c = 54e-3
    offs = [(20, 0), (0, 24), (-14, 14), (30, -6), (-22, -18)]
    src = np.array([[c, c]]) - 1e-3 * h
    rec = np.array([[c + a * 1e-3, c + b * 1e-3] for a, b in offs]) - 1e-3 * h
    vp = np.full((n + 2 * ab,) * 2, 1500., np.float32)
    tr, _ = O.forward(vp, (h, h), dt, nt, (ab, ab), src.astype(np.float32), rec.astype(np.float32), wav[None],
                      (-ab * h, -ab * h), kernel=kernel, dtype=np.float64)
    # rec[k] of a level is p at time (k + 1) dt: the coarse samples 1 .. nt - 2 on every level
    k = np.arange(1, 96)
    return tr[:, (k + 1) * 2 ** level - 1].astype(np.float64)


def test_self_convergence_under_refinement():
    """The oracle converges under h/2, dt/2 refinement at fixed CFL: the trace differences between
    successive levels fall by 4 per level (second order; measured 2.00 for OT2 and 2.03 for OT4,
    whose update is fourth order in time but whose point source enters without the dt^2/12
    correction, so that the source term is second order). OT4's differences are the smaller."""
    err = {}
    for kernel in ('OT2', 'OT4'):
        s = [_refined_traces(level, kernel) for level in range(3)]
        e = [np.linalg.norm(s[i] - s[i + 1]) / np.linalg.norm(s[2]) for i in range(2)]
        order = np.log2(e[0] / e[1])
        assert 1.8 <= order <= 2.3, (kernel, e, order)
        err[kernel] = e
    assert err['OT4'][1] < 0.6 * err['OT2'][1] and err['OT2'][1] < 5e-3


@pytest.mark.parametrize('kernel,rho_mode,alpha', [('OT4', 'variable', True), ('OT2', 'constant', False)])
def test_fp32_noise_floor(kernel, rho_mode, alpha):
    """The FP32 oracle against the same oracle in FP64: the FP32 rounding of a 300-step shot
    (measured 0.9-4.0e-6 relative) lies well below the 1e-4 trace tolerance of the parity tests."""
    from tests import _cases as C
    c = C.small_case(kernel=kernel, density=rho_mode, alpha=alpha, nt=300)
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    tr = [O.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][0], c['recs'][0], c['wav'][None],
                    origin, rho=c['rho'], alpha=c['alpha'], kernel=kernel, dtype=d)[0].astype(np.float64)
          for d in (np.float32, np.float64)]
    assert np.linalg.norm(tr[0] - tr[1]) <= 1e-5 * np.linalg.norm(tr[1])


@pytest.mark.parametrize('dim,n', [(2, 40), (3, 22)])
@pytest.mark.parametrize('kernel', ['OT2', 'OT4'])
@pytest.mark.parametrize('rho_mode', ['none', 'variable', 'constant'])
def test_c_matches_numpy(dim, n, kernel, rho_mode):
    """The two restatements are written independently but perform the same FP32 operations
    in the same order, so traces and snapshots agree bit for bit."""
    rng = np.random.default_rng(3)
    shape = (n,) * dim
    h = (0.5e-3,) * dim
    vp = (1500 + 100 * rng.random(shape)).astype(np.float32)
    rho = None if rho_mode == 'none' else (
        np.full(shape, 1000., np.float32) if rho_mode == 'constant' else (1000 + 90 * rng.random(shape)).astype(np.float32))
    al = (rng.random(shape)).astype(np.float32)
    dt = (0.6 if kernel == 'OT4' else 0.4) * h[0] / 1650
    nt, e = 90, 6
    origin = tuple(-e * x for x in h)
    lim = (n - 2 * e - 1) * h[0]
    src = np.array([[lim * 0.3] * dim])
    rec = np.array([[lim * 0.7] + [lim * 0.5] * (dim - 1), [lim * 0.2] * dim])
    w = O.tone_burst(0.5e6, 3, nt, dt)[None]
    kw = dict(rho=rho, alpha=al, kernel=kernel, save=True)
    a, sa = O.forward(vp, h, dt, nt, (e,) * dim, src, rec, w, origin, **kw)
    b, sb = c_oracle.forward(vp, h, dt, nt, (e,) * dim, src, rec, w, origin, **kw)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(sa, sb)
    ga, pa = O.adjoint(vp, h, dt, nt, (e,) * dim, rec, a, origin, sa, rho=rho, alpha=al, kernel=kernel)
    gb, pb = c_oracle.adjoint(vp, h, dt, nt, (e,) * dim, rec, a, origin, sa, rho=rho, alpha=al, kernel=kernel)
    nrm = np.linalg.norm(ga.astype(np.float64))
    assert np.linalg.norm((ga - gb).astype(np.float64)) <= 1e-5 * nrm


def test_kernel_and_undersampling_selection():
    """OT2 below (2/pi) h / (vmax sqrt(dim)), OT4 above (devito.py:1412-1431); CFL 0.6 of the
    benchmark configurations selects OT4 in 2D and 3D; f = 4 for their tone bursts."""
    h, v = 0.5e-3, 1650.
    assert O.select_kernel(0.44 * h / v, h, v, 2) == 'OT2'
    assert O.select_kernel(0.6 * h / v, h, v, 2) == 'OT4'
    assert O.select_kernel(0.6 * h / v, h, v, 3) == 'OT4'
    dt = 0.6 * h / v
    assert O.select_undersampling(O.tone_burst(0.5e6, 3, 2000, dt)[None], dt) == 4
    dt = 0.6 * 0.25e-3 / v
    assert O.select_undersampling(O.tone_burst(1.0e6, 3, 4000, dt)[None], dt) == 4


def test_damping_profile_rules():
    """SpongeBoundary2 damping (boundaries/devito.py:49-60, boundary.py:59-170): zero in the
    interior and on the innermost sponge layer, symmetric, corners take the outer slab."""
    shape, A, h = (60, 64), 20, (0.5e-3, 0.5e-3)
    vp = np.full(shape, 1500., np.float32)
    d = O.damping_profile(shape, h, (A, A), vp, 1e-7)
    assert np.all(d[A:-A, A:-A] == 0)
    assert np.all(d[A - 1, A - 1:-(A - 1)] == 0)
    np.testing.assert_array_equal(d, d[::-1, :])
    np.testing.assert_array_equal(d, d[:, ::-1])
    assert d[0, 5] == d[0, 30] and d[5, 0] == d[30, 0]   # corner point (0,5) takes the x slab's layer 0
    assert d[0, 0] > d[0, 30]                             # the diagonal takes both slabs


def test_linear_interpolation_weights():
    base, w = O.linear_stencil(np.array([[1.25e-3, 2.0e-3]], np.float32), (-1e-3, -1e-3), (0.5e-3, 0.5e-3))
    assert list(base[0]) == [4, 5] or list(base[0]) == [4, 6]
    np.testing.assert_allclose(w.sum(), 1.0, rtol=1e-12)


def _exact_case(kernel, rho_mode, alpha, seed=0, nt=110):
    rng = np.random.default_rng(seed)
    h, e, n = 0.5e-3, 8, 20
    shape = (n + 2 * e, n + 3 + 2 * e)
    vp = (1500 + 100 * rng.random(shape)).astype(np.float64)
    rho = None if rho_mode == 'none' else (
        np.full(shape, 1000.) if rho_mode == 'constant' else 950 + 150 * rng.random(shape))
    al = 20 * rng.random(shape) if alpha else None
    dt = (0.6 if kernel == 'OT4' else 0.4) * h / 1650
    src = np.array([[4.1e-3, 5.3e-3], [6.2e-3, 2.1e-3]])
    rec = np.array([[1.3e-3, 1.1e-3], [8.7e-3, 9.2e-3], [2.2e-3, 8.8e-3]])
    wav = np.stack([O.tone_burst(1.0e6, 3, nt, dt), O.tone_burst(0.8e6, 3, nt, dt)])
    return dict(vp=vp, rho=rho, alpha=al, spacing=(h, h), dt=dt, nt=nt, ab=(e, e), origin=(-e * h, -e * h), src=src,
                rec=rec, wav=wav, kernel=kernel, rng=rng)


def _exact_traces(c, vp, wav):
    return O.forward(vp, c['spacing'], c['dt'], c['nt'], c['ab'], c['src'], c['rec'], wav, c['origin'], rho=c['rho'],
                     alpha=c['alpha'], kernel=c['kernel'], dtype=np.float64)[0]


@pytest.mark.parametrize('kernel,rho_mode,alpha', [('OT4', 'variable', True), ('OT2', 'none', False),
                                                   ('OT4', 'constant', True)])
def test_exact_adjoint_dot_product(kernel, rho_mode, alpha):
    """<F w, r> = <w, F^T r> for the (linear) wavelets -> traces map of the FP64 oracle."""
    c = _exact_case(kernel, rho_mode, alpha)
    r = c['rng'].standard_normal((len(c['rec']), c['nt']))
    w = c['rng'].standard_normal(c['wav'].shape).astype(np.float32).astype(np.float64)
    _, gw = O.adjoint_exact(c['vp'], c['spacing'], c['dt'], c['nt'], c['ab'], c['src'], c['rec'], w, r, c['origin'],
                            rho=c['rho'], alpha=c['alpha'], kernel=kernel)
    lhs = float(np.sum(_exact_traces(c, c['vp'], w) * r))
    rhs = float(np.sum(gw * w))
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs)


@pytest.mark.parametrize('kernel,rho_mode,alpha', [('OT4', 'variable', True), ('OT2', 'constant', False)])
def test_exact_adjoint_central_differences(kernel, rho_mode, alpha):
    """dJ/dvp of the FP64 oracle against central differences, J = sum(r * traces), along random
    directions over the whole grid (sponge included)."""
    c = _exact_case(kernel, rho_mode, alpha, seed=1)
    r = c['rng'].standard_normal((len(c['rec']), c['nt']))
    g, _ = O.adjoint_exact(c['vp'], c['spacing'], c['dt'], c['nt'], c['ab'], c['src'], c['rec'], c['wav'], r,
                           c['origin'], rho=c['rho'], alpha=c['alpha'], kernel=kernel)
    for _ in range(3):
        d = c['rng'].standard_normal(c['vp'].shape)
        eps = 1.0  # vp is rounded to FP32 as the reference stores it; 1 m/s keeps that below 1e-4
        fd = (np.sum(r * _exact_traces(c, c['vp'] + eps * d, c['wav']))
              - np.sum(r * _exact_traces(c, c['vp'] - eps * d, c['wav']))) / (2 * eps)
        assert abs(fd - np.sum(g * d)) <= 2e-3 * abs(fd)


def test_rho_term_known_answers():
    """The rho imaging term -grad(b, -1/2) . grad(s, -1/2) - b laplace(s) on fields the 10th-order
    stencils differentiate exactly, away from the edges: s = x^2 + y^2 with constant b gives
    -4 b; s = x with b = b0 + c x gives -c (laplace(x) = 0, the staggered derivatives exact)."""
    h = (0.5e-3, 0.4e-3)
    n = (30, 34)
    x = np.arange(n[0])[:, None] * h[0] * np.ones(n)
    y = np.arange(n[1])[None, :] * h[1] * np.ones(n)
    inner = (slice(6, -6), slice(6, -6))
    t = O.rho_term(x ** 2 + y ** 2, np.full(n, 1e-3), h)
    assert np.allclose(t[inner], -4e-3, rtol=1e-9)
    c = 2.0
    t = O.rho_term(x, 1e-3 + c * x, h)
    assert np.allclose(t[inner], -c, rtol=1e-9)
    # b varying along y only, s along x only: the dot product vanishes, laplace(x) = 0
    t = O.rho_term(x, 1e-3 + c * y, h)
    assert np.allclose(t[inner], 0, atol=1e-9)


def test_raw_vp_gradient_matches_snapshot_path_at_f1():
    """At undersampling 1 the raw path's held p_dt is the p.dt2 snapshot of the same step, so its
    vp gradient equals the standard imaging condition (FP64 oracle)."""
    c = _exact_case('OT4', 'variable', True, nt=90)
    r = c['rng'].standard_normal((len(c['rec']), c['nt']))
    kw = dict(rho=c['rho'], alpha=c['alpha'], kernel='OT4', undersampling=1, dtype=np.float64)
    args = (c['vp'], c['spacing'], c['dt'], c['nt'], c['ab'], c['src'], c['rec'], c['wav'], c['origin'])
    _, snaps = O.forward(*args, save=True, **kw)
    _, raw = O.forward(*args, save='raw', **kw)
    g, _ = O.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['ab'], c['rec'], r, c['origin'], snaps, **kw)
    g_raw, _, g_rho, p_rho = O.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['ab'], c['rec'], r, c['origin'],
                                       raw, raw=True, rho_grad=True, **kw)
    assert np.abs(g).max() > 0 and np.abs(g_rho).max() > 0 and p_rho.min() >= 0
    assert np.linalg.norm(g_raw - g) <= 1e-6 * np.linalg.norm(g)  # FP32 snapshots and outputs


def test_cfs_pml_absorbs_better_than_the_sponge():
    """The CFS-PML restatement (OT2) against a domain large enough that nothing returns from its
    edges: its traces stay within 3 % where the 20-cell sponge is off by several per cent."""
    h, e, n, nt = 0.5e-3, 20, 40, 700
    dt = 0.4 * h / 1650
    src = np.array([[10 * h, 20 * h]])
    rec = np.array([[30 * h, 20 * h], [20 * h, 38 * h]])
    w = O.tone_burst(0.5e6, 3, nt, dt)[None]
    run = lambda E, **kw: O.forward(np.full((n + 2 * E,) * 2, 1500., np.float32), (h, h), dt, nt, (E, E), src, rec,
                                    w, (-E * h, -E * h), kernel='OT2', **kw)[0]
    big = run(120)
    pml = run(e, boundary='pml', f_centre=0.5e6)
    sponge = run(e)
    err = lambda tr: np.linalg.norm(tr - big) / np.linalg.norm(big)
    assert err(pml) < 0.03 and err(pml) < err(sponge) / 3


def test_cfs_pml_ot4_literal_reading_diverges():
    """With OT4 the reference hands the CFS-PML the `laplacian` Function as its boundary field
    (iso_acoustic/devito.py:1551), and that Function holds vp^2 laplace(p) (:1504-1524,
    _diff_op :1648-1659), where OT2 hands it p itself. The auxiliary fields then carry two more
    space derivatives and a factor vp^2, about 1e13 times the OT2 term on this grid, and the
    update diverges within a few hundred steps even at OT2's time step; OT2 on the same case stays
    finite and decays. This is why the build rejects the combination (SA_E_UNSUPPORTED)."""
    h, e, n, nt = 0.5e-3, 20, 40, 400
    dt = 0.4 * h / 1650
    src = np.array([[10 * h, 20 * h]])
    rec = np.array([[30 * h, 20 * h], [20 * h, 38 * h]])
    w = O.tone_burst(0.5e6, 3, nt, dt)[None]
    run = lambda kernel: O.forward(np.full((n + 2 * e,) * 2, 1500., np.float32), (h, h), dt, nt, (e, e), src, rec, w,
                                   (-e * h, -e * h), kernel=kernel, boundary='pml', f_centre=0.5e6)[0]
    ot2 = run('OT2')
    assert np.isfinite(ot2).all() and np.abs(ot2).max() < 1
    with np.errstate(all='ignore'):
        ot4 = run('OT4')
    bad = ~np.isfinite(ot4) | (np.abs(ot4) > 1e6)
    assert bad.any(axis=0)[:nt // 2].any()  # blown up within the first half of the run


def test_sinc_stencil_weights():
    """The sinc support (half-width 7, 14 points per axis): a point on a grid node is that node
    alone (sinc vanishes on the other nodes), the weights of any position sum to one within the
    windowed sinc's ripple, and they are symmetric about the cell centre."""
    rng = np.random.default_rng(0)
    base, w, offs = O.sinc_stencil(np.array([[3., 5.]]), (0., 0.), (1., 1.))
    assert offs.shape == (196, 2) and np.array_equal(base, [[3, 5]])
    k = int(np.argmax(np.abs(w[0])))
    assert tuple(offs[k]) == (0, 0) and abs(w[0, k] - 1) < 1e-12
    assert np.abs(np.delete(w[0], k)).max() < 1e-12
    pts = rng.uniform(1., 9., (50, 2))
    _, w, _ = O.sinc_stencil(pts, (0., 0.), (1., 1.))
    assert np.abs(w.sum(axis=1) - 1).max() < 1e-3
    _, wa, oa = O.sinc_stencil(np.array([[0.25]]), (0.,), (1.,))
    _, wb, ob = O.sinc_stencil(np.array([[0.75]]), (0.,), (1.,))
    assert np.allclose(wa[0], wb[0][::-1], atol=1e-12)  # x at +0.25 mirrors x at +0.75


@pytest.mark.parametrize('interp', ['hicks', 'sinc'])
def test_exact_adjoint_dot_product_hicks(interp):
    """The exact adjoint with wide-support sources and receivers (Hicks: the sources smoothed;
    sinc): <F w, r> = <w, F^T r>."""
    c = _exact_case('OT4', 'variable', True)
    r = c['rng'].standard_normal((len(c['rec']), c['nt']))
    w = c['rng'].standard_normal(c['wav'].shape).astype(np.float32).astype(np.float64)
    _, gw = O.adjoint_exact(c['vp'], c['spacing'], c['dt'], c['nt'], c['ab'], c['src'], c['rec'], w, r, c['origin'],
                            rho=c['rho'], alpha=c['alpha'], kernel='OT4', interpolation=interp)
    tr = O.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['ab'], c['src'], c['rec'], w, c['origin'], rho=c['rho'],
                   alpha=c['alpha'], kernel='OT4', dtype=np.float64, interpolation=interp)[0]
    lhs = float(np.sum(tr * r))
    rhs = float(np.sum(gw * w))
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs)


def test_older_adjoint_injection_is_the_current_one_two_samples_later():
    """The reference's non-fw3d adjoint injection (-res[t-1] dt^2 vp^2 into p_a[t] before the stencil,
    iso_acoustic/devito.py:750-751, 793-794), which the recorded imaging tutorial used, equals its
    fw3d branch (forced on at :725; the branch the plan implements) on the residual delayed by two
    samples, bit for bit when the residual is zero where only the older reading reads it (the first
    sample's window weight, and sample nt - 2 - f, which it injects into the first level)."""
    from tests import _cases as C
    c = C.small_case(kernel='OT2', density='variable', alpha=True, nt=200)
    origin = tuple(-e * h for e, h in zip(c['extra'], c['spacing']))
    kw = dict(rho=c['rho'], alpha=c['alpha'], kernel='OT2', undersampling=4)
    _, snaps = O.forward(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['srcs'][0], c['recs'][0],
                         c['wav'][None], origin, save=True, **kw)
    r = np.random.default_rng(5).standard_normal((len(c['recs'][0]), c['nt'])).astype(np.float32)
    r[:, 0] = 0
    r[:, c['nt'] - 2 - 4:] = 0
    late = np.zeros_like(r)
    late[:, 2:] = r[:, :-2]
    old = O.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][0], r, origin, snaps,
                    fw3d=False, **kw)
    new = O.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][0], late, origin, snaps, **kw)
    assert np.array_equal(old[0], new[0]) and np.array_equal(old[1], new[1])
    same = O.adjoint(c['vp'], c['spacing'], c['dt'], c['nt'], c['absorbing'], c['recs'][0], r, origin, snaps, **kw)
    assert C.cosine(same[0], old[0]) < 0.999  # the two readings differ on the same residual
