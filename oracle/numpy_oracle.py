"""NumPy oracle for the iso-acoustic FDTD hot path (test infrastructure only).

This module is the CPU restatement that the CUDA path is checked against. It is
imported only by ``tests/``, by ``__graft_entry__.smoke()`` and by the CPU legs of
``bench.py``; the product path never calls it.

Parity status: **unpinned against Devito.** The reference builds its time loop
with Devito (a third-party JIT compiler that is not vendored and cannot be
imported here), and the reference ships no tests or golden vectors for this
path. What pins this restatement instead: the analytic 2D/3D Green's-function
known-answer check of the reference's own example
(``stride_examples/examples/homogeneous_acoustic/utils.py:5-59``), exact
dot-product tests of the discrete adjoint, central finite differences, and
agreement with the independent C restatement in ``oracle/fdtd_oracle.c``.

Every function cites the reference lines whose behaviour it restates (paths
relative to the reference repository root).
"""

from fractions import Fraction

import numpy as np
import scipy.signal

__all__ = [
    'second_derivative_weights', 'staggered_weights', 'damping_profile',
    'linear_stencil', 'select_kernel', 'select_undersampling', 'bandwidth',
    'tone_burst', 'tukey', 'forward', 'adjoint', 'grad_vp_chain', 'adjoint_exact', 'rho_term',
    'DB_TO_NEPER',
]

# dB/cm -> Np/m for attenuation power 0 (stride/physics/iso_acoustic/devito.py:487-497)
DB_TO_NEPER = 100 * (1e-6 / (2 * np.pi)) ** 0 / (20 * np.log10(np.exp(1)))


def _fornberg(m, x0, xs):
    """Fornberg's recursion with exact rationals (published algorithm, 1988)."""
    n = len(xs)
    c = [[Fraction(0)] * (m + 1) for _ in range(n)]
    c1 = Fraction(1)
    c4 = xs[0] - x0
    c[0][0] = Fraction(1)
    for i in range(1, n):
        mn = min(i, m)
        c2 = Fraction(1)
        c5 = c4
        c4 = xs[i] - x0
        for j in range(i):
            c3 = xs[i] - xs[j]
            c2 *= c3
            if j == i - 1:
                for k in range(mn, 0, -1):
                    c[i][k] = c1 * (k * c[i - 1][k - 1] - c5 * c[i - 1][k]) / c2
                c[i][0] = -c1 * c5 * c[i - 1][0] / c2
            for k in range(mn, 0, -1):
                c[j][k] = (c4 * c[j][k] - k * c[j][k - 1]) / c3
            c[j][0] = c4 * c[j][0] / c3
        c1 = c2
    return [c[i][m] for i in range(n)]


def second_derivative_weights(order=10):
    """Centred 2nd-derivative weights c0..c_{order/2} (Devito ``laplace`` at space_order 10,
    stride/physics/iso_acoustic/devito.py:1652)."""
    r = order // 2
    w = _fornberg(2, Fraction(0), [Fraction(i) for i in range(-r, r + 1)])
    return [float(w[r + k]) for k in range(r + 1)]


def staggered_weights(order=10):
    """Staggered 1st-derivative weights at offsets 1/2..(order-1)/2, antisymmetric
    (Devito ``grad(shift=+.5)`` / ``div(shift=-.5)``, iso_acoustic/devito.py:1655-1663)."""
    r = order // 2
    xs = [Fraction(2 * i + 1, 2) for i in range(-r, r)]
    w = _fornberg(1, Fraction(0), xs)
    return [float(w[r + k]) for k in range(r)]  # weight of +(k+1/2); -(k+1/2) is its negative


def damping_profile(shape, spacing, absorbing, vp_ext, dt):
    """Sponge damping ``damp`` of SpongeBoundary2 (stride/physics/boundaries/devito.py:49-60)
    built with Boundary.damping (stride/physics/boundaries/boundary.py:59-170), sine profile,
    power_degree 2, reflection coefficient from the absorbing width. FP32 like the reference."""
    dim = len(shape)
    refl = 10 ** (-(np.log10(max(*absorbing)) - 1) / np.log10(2) - 3)
    damp = np.zeros(shape, dtype=np.float32)
    for d in range(dim):
        A = absorbing[d]
        coef = (2 + 1) / 2 * np.log(1.0 / refl)
        coef = coef / (A * spacing[d]) if A > 15 else 0.67 / spacing[d]
        for index in range(A):
            pos = np.abs((A - index - 1) / float(A - 1))
            pos = pos - np.sin(2 * np.pi * pos) / (2 * np.pi)
            val = coef * pos
            sl = [slice(index, s - index) for s in shape]
            sl[d] = slice(index, index + 1)
            damp[tuple(sl)] += val
            sl = [slice(index, s - index) for s in shape]
            sl[d] = slice(shape[d] - index - 1, shape[d] - index)
            damp[tuple(sl)] += val
    damp *= vp_ext.astype(np.float32)
    damp = 7 * damp * np.float32(dt)
    return damp.astype(np.float32)


def first_derivative_weights(order=10):
    """Centred 1st-derivative weights c_1..c_{order/2} (c_{-k} = -c_k) for Devito's
    Derivative(f, (d, 1)) at space order 10 (boundaries/devito.py:131)."""
    r = order // 2
    w = _fornberg(1, Fraction(0), [Fraction(i) for i in range(-r, r + 1)])
    return [float(w[r + k]) for k in range(1, r + 1)]


def pml_profiles(shape, spacing, absorbing, vp_max, f_centre):
    """CFS-PML profiles of ComplexFrequencyShiftPML2 (stride/physics/boundaries/devito.py:72-127),
    one 1D FP32 array per axis, built with Boundary.damping (boundaries/boundary.py:59-170):
    sigma 'power' degree 3 with the coefficient from the reflection coefficient, times max(vp)
    (the 1D profile does not match the velocity's shape); alpha 'power' degree 2 with
    coefficient 0.01 pi f_centre as a mask (interior = the coefficient, layer = -coefficient
    pos^2); their derivatives are 2nd-order centred differences over an edge-padded halo of 2.
    Returns [(sigma, alpha, dsigma, dalpha)] per axis."""
    refl = 10 ** (-(np.log10(max(*absorbing)) - 1) / np.log10(2) - 3)
    out = []
    for d, n in enumerate(shape):
        A, h = absorbing[d], spacing[d]
        cs = (3 + 1) / 2 * np.log(1.0 / refl)
        cs = cs / (A * h) if A > 15 else 0.67 / h
        ca = 0.01 * np.pi * f_centre
        sig = np.zeros(n, np.float32)
        alp = np.ones(n, np.float32)
        alp *= ca
        for index in range(A):
            pos = np.abs((A - index - 1) / float(A - 1))
            sig[index] = sig[n - index - 1] = cs * pos ** 3
            alp[index] = alp[n - index - 1] = ca * -(pos ** 2)
        sig *= np.float32(vp_max)
        sp = np.pad(sig, 2, mode='edge')
        ap = np.pad(alp, 2, mode='edge')
        dsig = ((sp[3:-1] - sp[1:-3]) / np.float32(2 * h)).astype(np.float32)
        dalp = ((ap[3:-1] - ap[1:-3]) / np.float32(2 * h)).astype(np.float32)
        out.append((sig, alp, dsig, dalp))
    return out


def _pml_aux(aux, f, prof, spacing, absorbing, dt, adjoint):
    """One update of the CFS-PML auxiliary fields u_3, u_2, u_1 of every axis d on its two
    slabs (PMLSide subdomains: the absorbing cells of axis d, every cell of the others), from
    the boundary field f (ComplexFrequencyShiftPML2.apply, boundaries/devito.py:129-160):
        u3' = u3 - dt ((a + s) u3 - s^2 (s' + a') f_d)
        u2' = u2 - dt ((a + s) u2 - s (2 s' f_d + a' f_d + s f_dd) + u3')
        u1' = u1 - dt ((a + s) u1 - (s' f_d + 2 s f_dd) + u2')
    f_d, f_dd the 10th-order centred derivatives along d (zero halo); the adjoint uses the
    transposed first derivative, -f_d. Returns sum_d u1' (zero outside the slabs)."""
    t = f.dtype.type
    c1 = first_derivative_weights()
    w2 = second_derivative_weights()
    dt_ = t(dt)
    B = np.zeros_like(f)
    for d in range(f.ndim):
        n = f.shape[d]
        h = t(spacing[d])
        bs = [1] * f.ndim
        bs[d] = n
        sg, al, dsg, dal = (x.astype(f.dtype).reshape(bs) for x in prof[d])
        fd = sum(t(c1[k - 1]) * (_shift(f, d, k) - _shift(f, d, -k)) for k in range(1, 6)) / h
        fdd = (t(w2[0]) * f + sum(t(w2[k]) * (_shift(f, d, k) + _shift(f, d, -k)) for k in range(1, 6))) / (h * h)
        if adjoint:
            fd = -fd
        i = np.arange(n)
        slab = ((i < absorbing[d]) | (i >= n - absorbing[d])).reshape(bs)
        u3, u2, u1 = aux[d]
        a_s = al + sg
        n3 = u3 - dt_ * (a_s * u3 - sg * sg * (dsg + dal) * fd)
        n2 = u2 - dt_ * (a_s * u2 - sg * (t(2) * dsg * fd + dal * fd + sg * fdd) + n3)
        n1 = u1 - dt_ * (a_s * u1 - (dsg * fd + t(2) * sg * fdd) + n2)
        aux[d] = [np.where(slab, n3, u3), np.where(slab, n2, u2), np.where(slab, n1, u1)]
        B = B + np.where(slab, n1, t(0))
    return B


def linear_stencil(coords, origin, spacing):
    """Bi/trilinear corner indices and weights of Devito's linear SparseTimeFunction
    (stride/physics/common/devito.py:580-653). ``coords`` are the float32 point
    coordinates already shifted by +1e-3*h (iso_acoustic/devito.py:307-309).
    Returns (base [n, dim] int64, weights [n, 2**dim] float64 in corner order
    (bit d of the corner id = +1 along axis d, axis 0 is the most significant bit))."""
    coords = np.asarray(coords, dtype=np.float32).astype(np.float64)
    origin = np.asarray(origin, dtype=np.float64)
    spacing = np.asarray(spacing, dtype=np.float64)
    rel = (coords - origin) / spacing
    base = np.floor(rel).astype(np.int64)
    frac = rel - base
    n, dim = coords.shape
    ncorner = 2 ** dim
    w = np.ones((n, ncorner), dtype=np.float64)
    for c in range(ncorner):
        for d in range(dim):
            bit = (c >> (dim - 1 - d)) & 1
            w[:, c] *= frac[:, d] if bit else (1.0 - frac[:, d])
    return base, w


def hicks_stencil(coords, origin, spacing, smooth=False):
    """Hicks (Kaiser-windowed sinc) coefficients of GridDevito._calculate_hicks
    (stride/physics/common/devito.py:843-885) on the support of Devito's
    PrecomputedSparseTimeFunction with r = 8 (common/devito.py:640-648): grid points
    floor(x) - 3 .. floor(x) + 4 along each axis (the last coefficient is zero). ``smooth``: the
    reference's smoothing of the central coefficients (sources are smooth, receivers are not).
    Returns (base [n, dim], weights [n, 8**dim], offsets [8**dim, dim])."""
    import itertools
    import scipy.special
    coords = np.asarray(coords, dtype=np.float32).astype(np.float64)
    grid = (coords - np.asarray(origin, np.float64)) / np.asarray(spacing, np.float64)
    base = np.floor(grid).astype(np.int64)
    frac = grid - base
    n, dim = coords.shape
    kaiser_b, half = 4.14, 3
    den = scipy.special.iv(0, kaiser_b)
    ext = half / 0.99
    coef = np.zeros((n, dim, 2 * half + 2))
    for gp in range(-half, half + 1):
        x = frac - gp
        wgt = (x / ext) ** 2
        wgt[wgt > 1] = 1
        coef[:, :, half + gp] = np.sinc(x) * scipy.special.iv(0, kaiser_b * np.sqrt(1 - wgt)) / den
    if smooth:
        m = half - 1
        a, b, c = coef[:, :, m].copy(), coef[:, :, m + 1].copy(), coef[:, :, m + 2].copy()
        coef[:, :, m - 1] = coef[:, :, m - 1] + a * 0.01
        coef[:, :, m] = a * 0.98 + b * 0.03
        coef[:, :, m + 1] = b * 0.94 + (a + c) * 0.01
        coef[:, :, m + 2] = c * 0.98 + b * 0.03
        coef[:, :, m + 3] = coef[:, :, m + 3] + c * 0.01
    offs = np.array(list(itertools.product(range(-half, half + 2), repeat=dim)), dtype=np.int64)
    w = np.ones((n, len(offs)))
    for k, off in enumerate(offs):
        for d in range(dim):
            w[:, k] *= coef[:, d, off[d] + half]
    return base, w, offs


# Kaiser window parameter b by half-width r (Hicks 2002, "Arbitrary source and receiver positioning
# in finite-difference schemes using Kaiser windowed sinc functions", Geophysics 67(1), table 1).
SINC_B = {1: 1.24, 2: 2.94, 3: 4.53, 4: 4.14, 5: 5.26, 6: 6.40, 7: 7.51, 8: 8.56, 9: 9.56, 10: 10.64}


def sinc_stencil(coords, origin, spacing, r=7):
    """Kaiser-windowed sinc of half-width r, the interpolation of Devito's
    SparseTimeFunction(interpolation='sinc', r=7) that stride/physics/common/devito.py:634-638
    builds: grid points floor(x) - r + 1 .. floor(x) + r along each axis, weight
    sinc(d) I0(b sqrt(1 - (d/r)^2)) / I0(b) at the distance d = point - x, product over axes.
    Devito is not installed here: this restates the published method, it is not checked
    against Devito's own weights. Returns (base [n, dim], weights [n, (2r)**dim],
    offsets [(2r)**dim, dim])."""
    import itertools
    import scipy.special
    coords = np.asarray(coords, dtype=np.float32).astype(np.float64)
    grid = (coords - np.asarray(origin, np.float64)) / np.asarray(spacing, np.float64)
    base = np.floor(grid).astype(np.int64)
    frac = grid - base
    n, dim = coords.shape
    b = SINC_B[r]
    rel = np.arange(-r + 1, r + 1)
    d = rel[None, None, :] - frac[:, :, None]                       # [n, dim, 2r]
    coef = np.sinc(d) * scipy.special.iv(0, b * np.sqrt(np.clip(1 - (d / r) ** 2, 0, None))) / scipy.special.iv(0, b)
    offs = np.array(list(itertools.product(rel, repeat=dim)), dtype=np.int64)
    w = np.ones((n, len(offs)))
    for k, off in enumerate(offs):
        for a in range(dim):
            w[:, k] *= coef[:, a, off[a] + r - 1]
    return base, w, offs


def sparse_stencil(interpolation, coords, origin, spacing, smooth):
    """(base, weights, offsets) of a SparseTimeFunction with the given interpolation (the Hicks
    sources smoothed when ``smooth``; sinc has no smoothing)."""
    if interpolation == 'hicks':
        return hicks_stencil(coords, origin, spacing, smooth)
    if interpolation == 'sinc':
        return sinc_stencil(coords, origin, spacing)
    base, w = linear_stencil(coords, origin, spacing)
    return base, w, _corner_offsets(base.shape[1])


def _corner_offsets(dim):
    return [tuple((c >> (dim - 1 - d)) & 1 for d in range(dim)) for c in range(2 ** dim)]


def select_kernel(dt, h, vp_max, dim):
    """OT2/OT4 auto-selection (stride/physics/iso_acoustic/devito.py:1412-1431,1688-1689)."""
    dt_ot2 = (2.0 / np.pi) * h / vp_max / np.sqrt(dim)
    return 'OT2' if dt <= dt_ot2 else 'OT4'


def bandwidth(signal, dt, cutoff=-10):
    """-10 dB bandwidth (stride/utils/fft.py:97-141 with magnitude_spectrum in dB)."""
    num = signal.shape[-1]
    freqs = np.fft.rfftfreq(num, dt)
    mag = np.abs(np.fft.rfft(signal, axis=-1, norm='forward'))
    mag = 20 * np.log10((mag + 1e-31) / (np.max(mag) + 1e-31))
    if mag.ndim > 1:
        mag = np.mean(mag, axis=0)
    above = np.nonzero(mag > cutoff)[0]
    f_min = freqs[above[0]] if len(above) else 0
    f_max = freqs[above[-1]] if len(above) else mag.shape[-1]
    return f_min, freqs[np.argmax(mag)], f_max


def select_undersampling(wavelets, dt):
    """f = min(max(4, int(1/(4 f_max dt))), 10) (iso_acoustic/devito.py:1360-1375,1447-1456)."""
    f_maxs = [bandwidth(w, dt)[2] for w in np.atleast_2d(wavelets) if np.any(w)]
    f_max = np.max(f_maxs) if f_maxs else 0.05 / dt
    return min(max(4, int((1 / (4 * f_max)) / dt)), 10)


def tone_burst(centre_freq, n_cycles, n_samples, dt, offset=0):
    """Gaussian tone burst (stride/utils/wavelets.py:6-53)."""
    tone_length = n_cycles / centre_freq
    t = np.linspace(0, tone_length, int(tone_length // dt + 1), endpoint=False)
    sig = np.sin(2 * np.pi * centre_freq * t)
    n_tone = sig.shape[0]
    win = np.exp(-np.linspace(-3, 3, n_tone) ** 2 / 2)
    sig = sig * win * scipy.signal.get_window(('tukey', 0.05), n_tone, False)
    return np.pad(sig, ((offset, n_samples - offset - n_tone),), mode='constant')


def tukey(nt, lo=0, hi=None, total=None):
    """Source/adjoint-source time window (iso_acoustic/devito.py:505-509, 865-869)."""
    hi = nt if hi is None else hi
    total = nt if total is None else total
    w = scipy.signal.get_window(('tukey', 0.001), hi - lo, False)
    return np.pad(w, ((lo, total - hi),), mode='constant')


# --------------------------------------------------------------------------------------
# spatial operators on the extended grid, zero halo for the field (common/devito.py:805-841)
# --------------------------------------------------------------------------------------

def _shift(u, d, k):
    """u[i+k] along axis d with zeros outside."""
    out = np.zeros_like(u)
    n = u.shape[d]
    src = [slice(None)] * u.ndim
    dst = [slice(None)] * u.ndim
    if k >= 0:
        src[d] = slice(k, n)
        dst[d] = slice(0, n - k)
    else:
        src[d] = slice(0, n + k)
        dst[d] = slice(-k, n)
    out[tuple(dst)] = u[tuple(src)]
    return out


def _laplace(u, spacing, w2):
    """10th-order Laplacian (Devito ``field.laplace``, iso_acoustic/devito.py:1652)."""
    out = np.zeros_like(u)
    for d in range(u.ndim):
        h2 = u.dtype.type(spacing[d] ** 2)
        acc = u.dtype.type(w2[0]) * u
        for k in range(1, len(w2)):
            acc = acc + u.dtype.type(w2[k]) * (_shift(u, d, k) + _shift(u, d, -k))
        out = out + acc / h2
    return out


def _half_buoy(buoy, d, R):
    """Buoyancy at half points j+1/2 along axis d for j = -R .. n+R-2: arithmetic mean of
    the two neighbouring nodes, the nodes beyond the grid taking the edge value (materials
    are padded with 'edge', common/devito.py:805-841; the averaging rule is unpinned)."""
    n = buoy.shape[d]
    j = np.arange(-R, n + R - 1)
    b0 = np.take(buoy, np.clip(j, 0, n - 1), axis=d)
    b1 = np.take(buoy, np.clip(j + 1, 0, n - 1), axis=d)
    return buoy.dtype.type(0.5) * (b0 + b1)


def _stagger_div_grad(u, spacing, ws, bhalf):
    """sum_d D-_d[ b(i+1/2) D+_d u ] with 10th-order staggered weights
    (iso_acoustic/devito.py:1655-1665). ``bhalf`` None means b == 1 (the rho-constant
    branch, :1654)."""
    R = len(ws)
    out = np.zeros_like(u)
    t = u.dtype.type
    for d in range(u.ndim):
        n = u.shape[d]
        h = t(spacing[d])
        pad = [(0, 0)] * u.ndim
        pad[d] = (2 * R, 2 * R)
        up = np.pad(u, pad)  # zero halo
        m = n + 2 * R - 1    # half points j+1/2, j = -R .. n+R-2 (F index j+R)
        F = None
        for k in range(R):
            a = [slice(None)] * u.ndim
            b = [slice(None)] * u.ndim
            a[d] = slice(R + 1 + k, R + 1 + k + m)
            b[d] = slice(R - k, R - k + m)
            term = t(ws[k]) * (up[tuple(a)] - up[tuple(b)])
            F = term if F is None else F + term
        F = F / h
        if bhalf is not None:
            F = F * bhalf[d]
        acc = None
        for k in range(R):
            a = [slice(None)] * u.ndim
            b = [slice(None)] * u.ndim
            a[d] = slice(R + k, R + k + n)
            b[d] = slice(R - k - 1, R - k - 1 + n)
            term = t(ws[k]) * (F[tuple(a)] - F[tuple(b)])
            acc = term if acc is None else acc + term
        out = out + acc / h
    return out


class _Medium:
    """Per-point material arrays on the extended grid in the reference's FP32 form
    (iso_acoustic/devito.py:476-497)."""

    def __init__(self, vp, rho, alpha_db, spacing, dtype):
        t = dtype
        self.vp = vp.astype(np.float32).astype(t)
        self.vp2 = self.vp * self.vp
        self.rho_mode = 0
        self.rho = None
        self.bhalf = None
        if rho is not None:
            rho32 = rho.astype(np.float32)
            if np.isclose(np.min(rho32), np.max(rho32)):
                self.rho_mode = 2  # staggered operator, no rho/buoyancy (:1472-1475,1654)
            else:
                self.rho_mode = 1
                self.rho = rho32.astype(t)
                buoy = (1 / rho32).astype(t)
                self.bhalf = [_half_buoy(buoy, d, 5) for d in range(vp.ndim)]
        self.alpha = None
        if alpha_db is not None:
            self.alpha = (alpha_db.astype(np.float32).astype(np.float64) * DB_TO_NEPER).astype(np.float32).astype(t)
        self.spacing = spacing

    def L(self, u, w2, ws):
        if self.rho_mode == 0:
            return self.vp2 * _laplace(u, self.spacing, w2)
        if self.rho_mode == 2:
            return self.vp2 * _stagger_div_grad(u, self.spacing, ws, None)
        return self.vp2 * self.rho * _stagger_div_grad(u, self.spacing, ws, self.bhalf)


def _Lt(med, u, kernel, dt, w2, ws):
    """Spatial term of the time update: L u (OT2) or L u + dt^2/12 L(L u) (OT4),
    iso_acoustic/devito.py:1503-1534,1632-1644; the intermediate has a zero halo."""
    lap = med.L(u, w2, ws)
    if kernel == 'OT2':
        return lap
    return lap + u.dtype.type(dt * dt / 12) * med.L(lap, w2, ws)


def _update(med, damp, Lt, u, um, dt):
    """Solve p.dt2 - Lt + 2 a vp p.dt + vp^2 (2 d p.dtc + d^2 p) = 0 for the new level
    (iso_acoustic/devito.py:1575-1581, boundaries/devito.py:62-67). Centred first
    derivatives; the backward direction uses the transposed (negated) ones, which is the
    same formula with the roles of p[t+1] and p[t-1] exchanged."""
    t = u.dtype.type
    dt_ = t(dt)
    beta = damp * med.vp2 / t(1)  # vp^2 d
    if med.alpha is not None:
        beta = beta + med.alpha * med.vp
    beta = dt_ * beta
    num = dt_ * dt_ * Lt + (t(2) - dt_ * dt_ * med.vp2 * damp * damp) * u - (t(1) - beta) * um
    return num / (t(1) + beta)


def _scatter(field, base, w, amp, dim, offs=None):
    offs = _corner_offsets(dim) if offs is None else offs
    for c, off in enumerate(offs):
        idx = tuple(base[:, d] + off[d] for d in range(dim))
        np.add.at(field, idx, (w[:, c] * amp).astype(field.dtype))


def _gather(field, base, w, dim, offs=None):
    offs = _corner_offsets(dim) if offs is None else offs
    out = np.zeros(base.shape[0], dtype=np.float64)
    for c, off in enumerate(offs):
        idx = tuple(base[:, d] + off[d] for d in range(dim))
        out += w[:, c] * field[idx]
    return out


def _pml_state(boundary, vp, spacing, absorbing, f_centre, dtype):
    """Profiles and zero auxiliary fields of the CFS-PML (None for the sponge)."""
    if boundary == 'sponge':
        return None
    if boundary != 'pml':
        raise ValueError('boundary %r' % boundary)
    prof = pml_profiles(vp.shape, spacing, absorbing, np.max(vp.astype(np.float32)), f_centre)
    aux = [[np.zeros(vp.shape, dtype) for _ in range(3)] for _ in range(vp.ndim)]
    return dict(prof=prof, aux=aux, lap=np.zeros(vp.shape, dtype))


def _pml_Lt(pml, med, u, kernel, dt, w2, ws, spacing, absorbing, adjoint):
    """Lt - vp^2 sum_d u_1,d for the CFS-PML update (iso_acoustic/devito.py:1552-1582): the
    auxiliary equations run before the step's first Laplacian, so under OT4 they see the
    boundary field `laplacian` of the previous step (zero on the first), under OT2 the field."""
    f = pml['lap'] if kernel != 'OT2' else u
    B = _pml_aux(pml['aux'], f, pml['prof'], spacing, absorbing, dt, adjoint)
    lap = med.L(u, w2, ws)
    if kernel == 'OT2':
        Lt = lap
    else:
        Lt = lap + u.dtype.type(dt * dt / 12) * med.L(lap, w2, ws)
        pml['lap'] = lap
    return Lt - med.vp2 * B


def forward(vp, spacing, dt, nt, absorbing, src_coords, rec_coords, wavelets, origin,
            rho=None, alpha=None, kernel=None, save=False, undersampling=4,
            dtype=np.float32, diff_source=False, interpolation='linear', boundary='sponge', f_centre=None):
    """Forward modelling of one shot (iso_acoustic/devito.py:220-581).

    Arrays are on the extended grid. ``wavelets`` [n_src, nt] raw (the Tukey window
    of :505-509 is applied here). Returns traces [n_rec, nt] (float32) and, when
    ``save``, the undersampled second time derivative snapshots [n_snap, *shape]
    (:398-418, common/devito.py:492-578); ``save='raw'`` stores p[t] itself instead, as the
    reference does when the rho or wavelet gradient is needed (:410-413). ``boundary='pml'``:
    ComplexFrequencyShiftPML2 with centre frequency ``f_centre`` instead of the sponge.
    """
    dim = vp.ndim
    shape = vp.shape
    h = max(spacing)
    if kernel is None:
        kernel = select_kernel(dt, h, float(np.max(vp)), dim)
    w2 = second_derivative_weights()
    ws = staggered_weights()
    med = _Medium(vp, rho, alpha, spacing, dtype)
    damp = damping_profile(shape, spacing, absorbing, vp, dt).astype(dtype)
    eps = 1e-3 * np.asarray(spacing)
    sb, sw, soffs = sparse_stencil(interpolation, np.asarray(src_coords, np.float32) + eps, origin, spacing, True)
    rb, rw, roffs = sparse_stencil(interpolation, np.asarray(rec_coords, np.float32) + eps, origin, spacing, False)
    wav = np.asarray(wavelets, np.float64)
    if diff_source:
        wav = np.gradient(wav, dt, axis=-1)
    src = (wav.T * tukey(nt)[:, None]).astype(np.float32)  # [nt, n_src]
    scale = 2 * dt * dt / h
    if not diff_source:
        scale /= dt
    rec = np.zeros((nt, rb.shape[0]), dtype=np.float64)
    f = undersampling
    n_snap = (nt + f) // f + 1
    snaps = np.zeros((n_snap,) + shape, dtype=np.float32) if save else None
    pm = np.zeros(shape, dtype=dtype)
    p = np.zeros(shape, dtype=dtype)
    pml = _pml_state(boundary, vp, spacing, absorbing, f_centre, dtype)
    if pml is not None:
        damp = np.zeros_like(damp)
    for t in range(1, nt - 1):
        if pml is None:
            Lt = _Lt(med, p, kernel, dt, w2, ws)
        else:
            Lt = _pml_Lt(pml, med, p, kernel, dt, w2, ws, spacing, absorbing, False)
        pn = _update(med, damp, Lt, p, pm, dt)
        # src.inject(p.forward, src * 2 dt^2 vp / h / dt): vp at each support point (H1 reading)
        for c, off in enumerate(soffs):
            idx = tuple(sb[:, d] + off[d] for d in range(dim))
            amp = src[t].astype(np.float64) * scale * med.vp[idx].astype(np.float64)
            np.add.at(pn, idx, (sw[:, c] * amp).astype(dtype))
        rec[t] = _gather(pn, rb, rw, dim, roffs)
        if save and t % f == 0:
            snaps[t // f] = p if save == 'raw' else (pn - 2 * p + pm) / dtype(dt * dt)
        pm, p = p, pn
    return rec.T.astype(np.float32 if dtype == np.float32 else np.float64), snaps


def _edge(a, d, idx):
    return np.take(a, np.clip(idx, 0, a.shape[d] - 1), axis=d)


def _zero(a, d, idx):
    n = a.shape[d]
    out = np.take(a, np.clip(idx, 0, n - 1), axis=d)
    bad = (idx < 0) | (idx >= n)
    shape = [1] * a.ndim
    shape[d] = n
    return np.where(bad.reshape(shape), 0, out)


def rho_term(s, buoy, spacing):
    """The rho imaging term of a raw snapshot s (iso_acoustic/devito.py:1137-1138):
    -grad(b, shift=-1/2) . grad(s, shift=-1/2) - b laplace(s), FP64. The shifted gradients are
    10th-order staggered first derivatives at i-1/2 from the nodes i+m, i-1-m (m = 0..4); b takes
    the edge value beyond the grid (edge-padded material halo), s is zero there."""
    ws = staggered_weights()
    w2 = second_derivative_weights()
    s = s.astype(np.float64)
    b = buoy.astype(np.float64)
    out = -b * _laplace(s, spacing, w2)
    for d in range(s.ndim):
        i = np.arange(s.shape[d])
        db = sum(ws[m] * (_edge(b, d, i + m) - _edge(b, d, i - 1 - m)) for m in range(len(ws))) / spacing[d]
        ds = sum(ws[m] * (_zero(s, d, i + m) - _zero(s, d, i - 1 - m)) for m in range(len(ws))) / spacing[d]
        out = out - db * ds
    return out


def adjoint(vp, spacing, dt, nt, absorbing, rec_coords, residual, origin, snaps,
            rho=None, alpha=None, kernel=None, undersampling=4, dtype=np.float32, src_coords=None,
            interpolation='linear', raw=False, rho_grad=False, boundary='sponge', f_centre=None, fw3d=True):
    """Reverse-time adjoint and vp imaging condition of the reference
    (iso_acoustic/devito.py:689-920, 985-1043): backward update of p_a[t-1],
    injection of -res[t] dt^2 vp^2 at the receivers (fw3d_mode, :725,748-753), and on
    t % f == 0 in the interior: grad += snap[t/f] p_a[t], prec += snap[t/f]^2.
    Returns raw (grad, prec) on the extended grid (zero outside the interior); with src_coords
    also the wavelet gradient [n_src, nt], src[t] = -interp(p_a[t]) (src.interpolate(expr=-p_a),
    :755-756).

    ``raw``: the snapshots hold p[n f] (forward ``save='raw'``) and the gradients follow the
    reference's raw-wavefield path (:1003-1024, 1133-1150): on t = n f the held terms
    p_dt = (s[n+1] - 2 s[n] + s[n-1]) / (f dt)^2 and, with ``rho_grad``, the rho term
    (``rho_term``) are recomputed (the Eqs under the undersampling condition), and on every step
    grad += held p_a[t], prec += held^2 (the Incs, which no conditional dimension guards). The
    time spacing f dt of the undersampled derivative is the physical one (unpinned: Devito
    is not available to confirm it). ``fw3d=False``: the reference's other injection branch, which
    its before_adjoint forces off (iso_acoustic/devito.py:725): -res[t-1] dt^2 vp^2 into p_a[t]
    before the stencil (:750-751, 793-794) instead of -res[t] dt^2 vp^2 into p_a[t-1] after it.
    Returns (grad, prec, grad_rho, prec_rho[, gsrc]) with
    ``rho_grad``. ``boundary='pml'``: the CFS-PML's adjoint as Devito forms it (time derivative
    and first space derivative transposed, boundaries/devito.py:135-149)."""
    dim = vp.ndim
    shape = vp.shape
    h = max(spacing)
    if kernel is None:
        kernel = select_kernel(dt, h, float(np.max(vp)), dim)
    w2 = second_derivative_weights()
    ws = staggered_weights()
    med = _Medium(vp, rho, alpha, spacing, dtype)
    damp = damping_profile(shape, spacing, absorbing, vp, dt).astype(dtype)
    eps = 1e-3 * np.asarray(spacing)
    rb, rw, roffs = sparse_stencil(interpolation, np.asarray(rec_coords, np.float32) + eps, origin, spacing, False)
    res = (np.asarray(residual, np.float64).T * tukey(nt)[:, None]).astype(np.float32)
    f = undersampling
    interior = tuple(slice(a, n - a) for a, n in zip(absorbing, shape))
    grad = np.zeros(shape, dtype=np.float64)
    prec = np.zeros(shape, dtype=np.float64)
    qp = np.zeros(shape, dtype=dtype)  # p_a[t+1]
    q = np.zeros(shape, dtype=dtype)   # p_a[t]
    offs = roffs
    gsrc = None
    if src_coords is not None:
        sb, sw, soffs = sparse_stencil(interpolation, np.asarray(src_coords, np.float32) + eps, origin, spacing,
                                       True)
        gsrc = np.zeros((nt, sb.shape[0]))
    if rho_grad:
        if rho is None:
            raise ValueError('the rho gradient needs rho')
        buoy = (1 / rho.astype(np.float32)).astype(np.float32)
        grad_rho = np.zeros(shape, dtype=np.float64)
        prec_rho = np.zeros(shape, dtype=np.float64)
    hold_vp = np.zeros(shape)
    hold_rho = np.zeros(shape)
    pml = _pml_state(boundary, vp, spacing, absorbing, f_centre, dtype)
    if pml is not None:
        damp = np.zeros_like(damp)
    def inject(field, row):
        for c, off in enumerate(offs):
            idx = tuple(rb[:, d] + off[d] for d in range(dim))
            amp = -res[row].astype(np.float64) * dt * dt * med.vp2[idx].astype(np.float64)
            np.add.at(field, idx, (rw[:, c] * amp).astype(dtype))

    for t in range(nt - 1 - f, 0, -1):
        if not fw3d:
            inject(q, t - 1)
        if gsrc is not None:
            gsrc[t] = -_gather(q, sb, sw, dim, soffs)
        if pml is None:
            Lt = _Lt(med, q, kernel, dt, w2, ws)
        else:
            Lt = _pml_Lt(pml, med, q, kernel, dt, w2, ws, spacing, absorbing, True)
        qn = _update(med, damp, Lt, q, qp, dt)
        if fw3d:
            inject(qn, t)
        if raw:
            if t % f == 0:
                n = t // f
                sn = [snaps[n + k].astype(np.float64) for k in (-1, 0, 1)]
                hold_vp = (sn[2] - 2 * sn[1] + sn[0]) / (f * dt) ** 2
                if rho_grad:
                    hold_rho = rho_term(snaps[n], buoy, spacing)
            qd = q.astype(np.float64)
            grad[interior] += (hold_vp * qd)[interior]
            prec[interior] += (hold_vp * hold_vp)[interior]
            if rho_grad:
                grad_rho[interior] += (hold_rho * qd)[interior]
                prec_rho[interior] += (hold_rho * hold_rho)[interior]
        elif t % f == 0:
            s = snaps[t // f].astype(np.float64)
            grad[interior] += (s * q.astype(np.float64))[interior]
            prec[interior] += (s * s)[interior]
        qp, q = q, qn
    out = (grad.astype(np.float32), prec.astype(np.float32))
    if rho_grad:
        out = out + (grad_rho.astype(np.float32), prec_rho.astype(np.float32))
    if gsrc is not None:
        out = out + (gsrc.T.astype(np.float32),)
    return out


def grad_vp_chain(grad, prec, vp_inner, slowness=True):
    """get_grad_vp chain rule on the inner grid (iso_acoustic/devito.py:1045-1081).
    The non-slowness preconditioner keeps the reference's ``(2/vp)**3**2`` precedence."""
    g = grad.astype(np.float32).copy()
    p = prec.astype(np.float32).copy()
    vp = vp_inner.astype(np.float32)
    if slowness:
        g *= +1 / vp
        p *= (1 / vp) ** 2
    else:
        g *= -2 / vp ** 3
        p *= (2 / vp) ** 3 ** 2
    return g, p


def _coefficient_derivatives(med, damp, dt):
    """Per-point update coefficients C1, C2, C3 of ``_update`` and their derivatives with respect
    to vp, with the damping's own vp factor (``damping_profile`` multiplies by vp) included:
    beta = dt (vp^2 d + a vp), C1 = dt^2/(1+beta), C2 = (2 - dt^2 vp^2 d^2)/(1+beta),
    C3 = (1-beta)/(1+beta)."""
    vp = med.vp.astype(np.float64)
    d = damp.astype(np.float64)
    a = np.zeros_like(vp) if med.alpha is None else med.alpha.astype(np.float64)
    beta = dt * (vp * vp * d + a * vp)
    dbeta = dt * (3 * vp * d + a)                  # d(vp^2 d)/dvp = 3 vp d since d is proportional to vp
    q = 1 + beta
    C1 = dt * dt / q
    C2 = (2 - dt * dt * vp * vp * d * d) / q
    C3 = (1 - beta) / q
    dC1 = -dt * dt * dbeta / q ** 2
    dC2 = (-dt * dt * 4 * vp * d * d * q - (2 - dt * dt * vp * vp * d * d) * dbeta) / q ** 2
    dC3 = -2 * dbeta / q ** 2
    return C1, C2, C3, dC1, dC2, dC3


def adjoint_exact(vp, spacing, dt, nt, absorbing, src_coords, rec_coords, wavelets, rec_weights, origin,
                  rho=None, alpha=None, kernel=None, interpolation='linear'):
    """Exact discrete adjoint of ``forward`` (FP64): the gradient of L = sum(rec_weights * traces)
    with respect to vp at every grid point and to the raw wavelets, i.e. the transpose of the
    linearised forward map applied to ``rec_weights`` [n_rec, nt] (dL/dtraces).

    The forward is u[n+1] = C1 Lt(u[n]) + C2 u[n] - C3 u[n-1] + s[n] (n = 1..nt-2) with
    rec[n] = P u[n+1]. With mu[n] = dL/du[n], the recursion runs backwards from mu[nt] = 0:
    mu[n] = P^T r[n-1] + Lt^T(C1 mu[n+1]) + C2 mu[n+1] - C3 mu[n+2]. Because Lt = W G (OT2) or
    W G + dt^2/12 W G W G (OT4) with G symmetric, Lt^T x = Lt(W x) / W, so z = C1 W mu obeys the
    forward recursion itself. The vp gradient collects, per step, mu[n+1] times the vp
    derivative of the update: the coefficients (attenuation and damping included), W inside Lt
    (dW/dvp = 2 W / vp), the OT4 term's inner W (dt^2/12 dW (G u)(G z)) and the source
    injection's vp factor. This is the ``exact`` gradient mode (no counterpart in the
    reference, whose imaging condition is iso_acoustic/devito.py:985-1043). ``interpolation``:
    'linear', 'hicks' (sources smoothed, receivers not) or 'sinc' for both the forward and its transpose."""
    dim = vp.ndim
    shape = vp.shape
    h = max(spacing)
    if kernel is None:
        kernel = select_kernel(dt, h, float(np.max(vp)), dim)
    w2 = second_derivative_weights()
    ws = staggered_weights()
    t64 = np.float64
    med = _Medium(vp, rho, alpha, spacing, t64)
    damp = damping_profile(shape, spacing, absorbing, vp, dt).astype(t64)
    eps = 1e-3 * np.asarray(spacing)
    sb, sw, offs = sparse_stencil(interpolation, np.asarray(src_coords, np.float32) + eps, origin, spacing, True)
    rb, rw, roffs = sparse_stencil(interpolation, np.asarray(rec_coords, np.float32) + eps, origin, spacing, False)
    win = tukey(nt)
    src = np.asarray(wavelets, np.float64).T * win[:, None]
    scale = 2 * dt / h
    # forward levels u[0..nt-1]
    u = np.zeros((nt,) + shape)
    for n in range(1, nt - 1):
        pn = _update(med, damp, _Lt(med, u[n], kernel, dt, w2, ws), u[n], u[n - 1], dt)
        for c, off in enumerate(offs):
            idx = tuple(sb[:, d] + off[d] for d in range(dim))
            np.add.at(pn, idx, sw[:, c] * src[n] * scale * med.vp[idx])
        u[n + 1] = pn
    C1, C2, C3, dC1, dC2, dC3 = _coefficient_derivatives(med, damp, dt)
    W = med.L(np.ones(shape), w2, ws) * 0 + (med.vp2 if med.rho_mode != 1 else med.vp2 * med.rho)
    vpf = med.vp.astype(np.float64)
    r = np.asarray(rec_weights, np.float64).T  # [nt, n_rec]
    grad = np.zeros(shape)
    gsrc = np.zeros((nt, sb.shape[0]))
    z1 = np.zeros(shape)  # z[n+1]
    z2 = np.zeros(shape)  # z[n+2]
    for n in range(nt - 1, 1, -1):
        zn = _update(med, damp, _Lt(med, z1, kernel, dt, w2, ws), z1, z2, dt) if n < nt - 1 else np.zeros(shape)
        if 1 <= n - 1 <= nt - 2:
            for c, off in enumerate(roffs):
                idx = tuple(rb[:, d] + off[d] for d in range(dim))
                np.add.at(zn, idx, rw[:, c] * r[n - 1] * (C1 * W)[idx])
        # contributions of step m = n-1 (u[n] = RHS(u[n-1], u[n-2])) with mu[n] = z[n] / (C1 W)
        m = n - 1
        mu = zn / (C1 * W)
        Ltu = _Lt(med, u[m], kernel, dt, w2, ws)
        grad += mu * (dC1 * Ltu + C1 * (2 / vpf) * Ltu + dC2 * u[m] - dC3 * u[m - 1])
        if kernel == 'OT4':
            grad += dt * dt / 12 * (2 * W / vpf) * (med.L(u[m], w2, ws) / W) * (med.L(zn, w2, ws) / W)
        for c, off in enumerate(offs):
            idx = tuple(sb[:, d] + off[d] for d in range(dim))
            np.add.at(grad, idx, mu[idx] * sw[:, c] * src[m] * scale)
            gsrc[m] += mu[idx] * sw[:, c] * scale * med.vp[idx]
        z2, z1 = z1, zn
    return grad, (gsrc * win[:, None]).T
